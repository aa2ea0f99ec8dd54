#!/usr/bin/env python3
"""Benchmark of the GB300 multi-phase-field time step.

Default workload (the largest single-GPU configuration of the headline
metric, which names the learned-vs-plain solve): the wet multi-phase-field
monolayer on a periodic 1024x1024 box, 6400 cells of radius 8 on 41x41
patches, wetmodel (nematic activity, Brinkman viscous solve xi = eta = 1,
rtol 1e-8), FP64 fields, the viscous solve by the learned flexible CG (FP32
inner iterations with the U-Net preconditioner on the tensor cores, FP64
refinement and plain FP64 CG fallback).  Set-up, outside the timed region:
training samples harvested from the plain FP64 solve of the 256x256 /
400-cell monolayer of the same physics (160 steps), the network trained on
the GPU (30 epochs), its parameters moved to the 1024^2 engine; then the
solve stage timed with the plain FP64 CG and with the learned solver on the
same states, and the velocity difference of the two solves of one
right-hand side.  Seeded synthetic initial condition (jittered triangular
lattice, tanh interfaces) -- synthetic data with the workload's shapes, no
dataset exists.  A "step" is one FD_CPUBackend::sim_step (Heun predictor +
corrector, two force evaluations, four viscous solves).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload wet1024|wet512|wet256|dry140|ensemble64]
                  [--precision double|mixed|float] [--solver learned|plain]

Prints one JSON line (rank 0).  `value` is site-updates/s over all ranks with
the state resident on the device, timed with CUDA events per step on the
engine's stream, the L2 cache flushed (256 MiB write) before every timed
step.  `e2e` is the same metric through the C ABI with host buffers: each
step uploads phi from pinned memory, steps, and downloads phi.  Under
torchrun every rank runs an independent replica on its own GPU (a monolayer
does not shard; replicas only).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MPF steps/s + site-updates/s; wet-step CG time, learned-PCG vs plain @ rtol 1e-8"


def workload(name):
    from rheocell_gb300 import generator as g
    if name == "wet256":
        return dict(name="wet MPF 256x256, 400 cells, R=8, 41x41 patches, wetmodel xi=eta=1, CG rtol 1e-8",
                    L=256, n=400, params=g.WET_NEMATIC, seed=1)
    if name == "wet512":
        return dict(name="wet MPF 512x512, 1600 cells, R=8, 41x41 patches, wetmodel nematic zeta=0.05, xi=eta=1, "
                         "CG rtol 1e-8", L=512, n=1600, params=g.WET_NEMATIC, seed=1)
    if name == "wet1024":
        return dict(name="wet MPF 1024x1024, 6400 cells, R=8, 41x41 patches, wetmodel nematic zeta=0.05, xi=eta=1, "
                         "CG rtol 1e-8 (polar+nematic activity has no single reference model)",
                    L=1024, n=6400, params=g.WET_NEMATIC, seed=1)
    if name == "dry140":
        return dict(name="dry polar MPF 140x140, 100 cells, R=8, 41x41 patches, wetpolarmodel friction_cell=0",
                    L=140, n=100, params=g.DRY_POLAR, seed=1)
    if name == "ensemble64":
        return dict(name="ensemble of 64 dry polar monolayers, box side uniform in 96-256 (numpy seed 64), "
                         "N = round(0.75 L^2 / (pi 8^2)) cells each, R=8, 41x41 patches, seeds 1000-1063, FP64",
                    members=ensemble_members(), params=g.DRY_POLAR, seed=1000)
    if name == "ensemble64wet":
        return dict(name="ensemble of 64 wet monolayers (wetmodel, xi=eta=1, CG rtol 1e-8), box side uniform in "
                         "96-256 (numpy seed 64), N = round(0.75 L^2 / (pi 8^2)) cells each, R=8, 41x41 patches, "
                         "seeds 1000-1063; each member's viscous system solved on its own box",
                    members=ensemble_members(), params=g.WET_NEMATIC, seed=1000)
    raise SystemExit("unknown workload %s" % name)


def ensemble_members(count=64, seed=64, R=8.0):
    """(L, N, seed) of each ensemble member: L uniform in [96, 256], N at 75%
    area fraction of radius-R discs."""
    import math
    import numpy as np
    sides = np.random.default_rng(seed).integers(96, 257, size=count)
    return [(int(L), int(round(0.75 * L * L / (math.pi * R * R))), 1000 + i) for i, L in enumerate(sides)]


def make_case(w):
    """[(keys, monolayer)] of the workload's members (one for a single box)."""
    from rheocell_gb300 import generator as g
    if "members" in w:
        out = []
        for L, n, seed in w["members"]:
            m = g.make_monolayer(L, n, seed=seed)
            keys = {k: str(v) for k, v in w["params"].items()}
            keys.update(seed=str(seed), box="square")
            out.append((keys, m))
        return out
    m = g.make_monolayer(w["L"], w["n"], seed=w["seed"])
    keys, m2 = g.case_keys(m, w["params"], seed=w["seed"])
    return [(keys, m2)]


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.lines = []
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cg_bytes_per_launch(S, L2, iters_per_launch, setup_reads=68.0):
    """Algorithmic bytes of one viscous-solve launch (both components):
    setup S*68 B (b, x, r, map); per component-iteration the minimal fused
    Jacobi-PCG, 11 FP64 vector passes = S*88 B (SpMV: read p, write Ap;
    update: read x, r, p, Ap, write x, r; direction: read r, p, write p),
    plus the box sums of p written and read (16 B) and the box count n(k)
    (4 B) per box site = L2*20 B."""
    return S * setup_reads + iters_per_launch * (S * 88.0 + L2 * 20.0)


# BF16 activation bytes of one network application per finest-grid pixel and
# velocity component: every layer reads its input and writes its output once
# (the first layer's FP32 input, the pooled and upsampled inputs at their own
# resolution, the last layer's FP32 output), summed over the three levels
NET_BYTES_PER_PIXEL = 348.0


def learned_bytes_per_launch(S, L2, inner_per_launch, refinements_per_launch):
    """Algorithmic bytes of one learned-solve launch (both components):
    setup S*68 B; per inner iteration and component the flexible CG's
    minimal FP32 vector passes (11 x 4 B per unknown) and the network
    application (NET_BYTES_PER_PIXEL per box pixel); per refinement sweep
    and component the FP64 true residual (read b, x, e, write x, r: 40 B per
    unknown)."""
    return (S * 68.0 + inner_per_launch * (S * 44.0 + L2 * NET_BYTES_PER_PIXEL)
            + refinements_per_launch * 2 * S * 40.0)


def fused_bytes_per_site(model):
    """Algorithmic HBM bytes per site of the dry fused predictor+corrector pair:
    predictor reads phi^n, writes phi*, dphi^n (24 B); corrector reads phi*,
    phi^n, dphi^n, writes phi^{n+1} (32 B); two box gathers read phi (16 B)."""
    return 72.0


def solve_stage(eng, lib, steps, flush):
    """(solve ms per step, CG iterations per solve) over `steps` steps, from
    the stage timers (CUDA events around each solve launch)."""
    import torch
    from rheocell_gb300 import abi
    lib.rc_set_timing(eng.h, 1)
    lib.rc_timers(eng.h, None, None, 1)
    st = abi.RcStepStats()
    lib.rc_wait(eng.h, C.byref(st))
    for _ in range(steps):
        flush.zero_()
        lib.rc_step_async(eng.h, 1)
    torch.cuda.synchronize()
    lib.rc_wait(eng.h, C.byref(st))
    tms = (C.c_double * abi.NUM_TIMERS)()
    tn = (C.c_longlong * abi.NUM_TIMERS)()
    lib.rc_timers(eng.h, tms, tn, 1)
    lib.rc_set_timing(eng.h, 0)
    return tms[3] / steps, st.cg_iterations / max(st.cg_solves, 1), st.cg_max_rel_residual


def prepare_learned(args, eng, lib):
    """Harvest samples from the plain FP64 solve, train the network on the
    device, then time the solve stage with the plain FP64 CG and with the
    learned flexible CG on the same state; leaves the learned solver on."""
    import torch
    from rheocell_gb300 import abi
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    # samples come from this monolayer's own plain solve, or from a smaller
    # monolayer of the same physics (--train-workload): the network is
    # convolutional, so parameters trained there apply at any box side
    import numpy as np
    if args.load_params:
        # parameters of an earlier training (set-up shortcut for experiments)
        lp = args.load_params
        eng.set_params(np.load(lp).astype(np.float64) if lp.endswith(".npy") else np.loadtxt(lp))
        harvest_s, n, rep = 0.0, 0, {"loaded_from": os.path.basename(args.load_params)}
    else:
        own = not args.train_workload or args.train_workload == args.workload
        src = eng if own else make_engine(args.train_workload, abi.RC_PRECISION_DOUBLE, eng.device)
        src.set_solver(abi.RC_SOLVER_PLAIN_FP64)  # samples come from plain FP64 solves
        src.harvest(capacity=args.harvest_capacity, every=3, per_solve=6)
        t0 = time.perf_counter()
        src.step(args.harvest_steps)
        harvest_s = time.perf_counter() - t0
        n = src.harvested()
        src.harvest(args.harvest_capacity, 3, 0)  # stop collecting, keep the samples
        rep = src.train(epochs=args.train_epochs, batch=8, learning_rate=args.train_lr, seed=1,
                        learning_rate_final=args.train_lr * args.train_lr_final, max_samples=args.train_max_samples)
        if src is not eng:
            eng.set_params(src.get_params())
            src.close()
    if args.save_params:
        np.savetxt(args.save_params, eng.get_params(), fmt="%.17g")
    k = max(2, min(args.steps, 10))
    # the plain FP64 device CG on the same states (whatever the engine's precision)
    eng.set_solver(abi.RC_SOLVER_PLAIN_FP64)
    solve_stage(eng, lib, 1, flush)
    plain_ms, plain_it, plain_res = solve_stage(eng, lib, k, flush)
    eng.set_solver(abi.RC_SOLVER_LEARNED)
    solve_stage(eng, lib, 1, flush)
    learned_ms, learned_it, learned_res = solve_stage(eng, lib, k, flush)
    accuracy = velocity_error(eng)
    # per-phase breakdown of the learned solve (device clock, one block)
    phases = None
    if args.solver_phases:
        lib.rc_solver_profile(eng.h, 1, None, 0)
        for _ in range(k):
            lib.rc_step_async(eng.h, 1)
        torch.cuda.synchronize()
        nph = len(abi.SOLVER_PHASES)
        ms = (C.c_double * nph)()
        lib.rc_solver_profile(eng.h, 0, ms, nph)
        phases = {nm: round(ms[i] / k, 4) for i, nm in enumerate(abi.SOLVER_PHASES)}
    return {"harvest_steps": args.harvest_steps, "harvest_s": harvest_s, "samples": n,
            "trained_on": args.train_workload or args.workload,
            "training": {kk: (round(v, 6) if isinstance(v, float) else v) for kk, v in rep.items()},
            "solve_ms_per_step": {"plain_fp64_cg": plain_ms, "learned_fcg": learned_ms,
                                  "speedup": plain_ms / learned_ms if learned_ms > 0 else None},
            "iterations_per_solve": {"plain_fp64_cg": plain_it, "learned_fcg_inner": learned_it},
            "max_rel_residual": {"plain_fp64_cg": plain_res, "learned_fcg": learned_res},
            "steps_each": k, "phases_ms_per_step": phases,
            "velocity_rel_err_vs_fp64": accuracy}


def field_errors(args, eng_device=0, steps=20):
    """Error of every reported field against the FP64 engine: the training
    workload (256^2, same physics) run from the same start in FP64 and in
    the benchmarked precision for `steps` steps; max |a - b| / max |b|."""
    from rheocell_gb300 import abi
    name = args.train_workload or "wet256"
    prec = {"mixed": abi.RC_PRECISION_MIXED, "float": abi.RC_PRECISION_FLOAT}[args.precision]
    a = make_engine(name, abi.RC_PRECISION_DOUBLE, eng_device)
    b = make_engine(name, prec, eng_device)
    a.step(steps)
    b.step(steps)
    sa, sb = a.state(), b.state()
    a.close()
    b.close()
    out = {"workload": workload(name)["name"], "steps": steps,
           "how": "FP64 engine vs this precision from the same start, plain solves, max |a-b| / max |a|"}
    for k in ("phi", "vx", "vy", "mu", "area", "sum_f", "com_x", "com_y"):
        den = max(float(abs(sa[k]).max()), 1e-300)
        out[k] = float(abs(sb[k] - sa[k]).max()) / den
    return out


def velocity_error(eng, tol=1e-8, tight=1e-12):
    """The last evaluation's viscous system solved again from a cold start
    (rc_viscous_resolve, device arrays, engine state untouched): once with
    the FP64 CG at a tight tolerance -- the FP64 oracle solution -- and then
    at the bench tolerance by the plain FP64 CG and by the learned flexible
    CG; max |v - v_oracle| / max |v_oracle| per component for both, and the
    learned solve against the plain one."""
    import torch
    from rheocell_gb300 import abi
    S = eng.site_count()
    v = [torch.zeros(S, dtype=torch.float64, device="cuda") for _ in range(6)]
    torch.cuda.synchronize()
    eng.set_cg_tolerance(tight)
    so = eng.resolve(abi.RC_SOLVER_PLAIN_FP64, v[4].data_ptr(), v[5].data_ptr())
    eng.set_cg_tolerance(tol)
    sp = eng.resolve(abi.RC_SOLVER_PLAIN_FP64, v[0].data_ptr(), v[1].data_ptr())
    sl = eng.resolve(abi.RC_SOLVER_LEARNED, v[2].data_ptr(), v[3].data_ptr())

    def err(a, b):
        return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))
    def err2(a, b):
        return float((a - b).norm() / b.norm().clamp_min(1e-300))
    learned = [err(v[2 + c], v[4 + c]) for c in range(2)]
    plain = [err(v[c], v[4 + c]) for c in range(2)]
    return {"vx": learned[0], "vy": learned[1], "max": max(learned),
            "norm": "max |v - v_oracle| / max |v_oracle| per component",
            "l2_max": max(err2(v[2 + c], v[4 + c]) for c in range(2)),
            "plain_fp64_max": max(plain),
            "learned_vs_plain_max": max(err(v[2 + c], v[c]) for c in range(2)),
            "how": "same right-hand side (last evaluation of the timed run), cold-start solves of all %d unknowns; "
                   "oracle = FP64 CG to |r|/|b| < %g; learned flexible CG and plain FP64 CG at %g against it" % (S, tight, tol),
            "oracle_fp64": {"iterations": so.cg_iterations, "max_rel_residual": so.cg_max_rel_residual},
            "plain_fp64": {"iterations": sp.cg_iterations, "max_rel_residual": sp.cg_max_rel_residual},
            "learned": {"inner_iterations": sl.cg_iterations, "refinements": sl.refinements,
                        "fallbacks": sl.fallbacks, "max_rel_residual": sl.cg_max_rel_residual}}


def make_engine(name, prec, dev):
    """A single-monolayer engine of workload `name` on device `dev`, in phase 1."""
    from rheocell_gb300 import engine, host
    (keys, m), = make_case(workload(name))
    p, cells = host.engine_inputs(keys, m, precision=prec)
    e = engine.Engine(p, m.L, cells, device=dev)
    e.set_phase(1)
    return e


def run_gb300(args, rank, world):
    import torch
    from rheocell_gb300 import abi, engine, host

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    w = workload(args.workload)
    members = all_members = make_case(w)
    sharded = world > 1 and len(members) > 1
    if sharded:
        # an ensemble is split into contiguous blocks of members, one per
        # rank (no data-path collective); a single monolayer runs as replicas
        from rheocell_gb300 import replicas
        members = replicas.shard(members, rank, world)
        if not members:
            raise SystemExit("more ranks (%d) than ensemble members (%d)" % (world, len(all_members)))
    prec = {"double": abi.RC_PRECISION_DOUBLE, "mixed": abi.RC_PRECISION_MIXED,
            "float": abi.RC_PRECISION_FLOAT}[args.precision]
    built = [host.engine_inputs(keys, m, precision=prec) for keys, m in members]
    stream = torch.cuda.Stream(dev)  # a real stream: the engine's graphs cannot capture on the legacy one
    torch.cuda.set_stream(stream)
    if len(members) == 1:
        p, cells = built[0]
        eng = engine.Engine(p, members[0][1].L, cells, device=dev)
    else:
        eng = engine.Engine.batch(built[0][0], [(m.L, cells, p.rng_state) for (_, m), (p, cells)
                                                in zip(members, built)], device=dev)
    eng.set_stream(stream.cuda_stream)
    eng.set_phase(1)
    lib = eng._lib
    S = eng.site_count()
    L2 = sum(m.L * m.L for _, m in members)
    n_cells = sum(m.n for _, m in members)
    learned = None
    if args.solver == "learned":
        learned = prepare_learned(args, eng, lib)
    # tile shape of the FP32 cell kernel, timed on this workload (setup, untimed)
    tuned = None
    if args.precision == "float" and not args.no_autotune:
        tuned = eng.autotune(steps_per_candidate=4)
    # warm-up
    eng.step(max(args.warmup, 3) if args.warmup >= 0 else 3)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    evs = []
    for _ in range(args.steps):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        rc = lib.rc_step_async(eng.h, 1)
        if rc != 0:
            raise RuntimeError(lib.rc_last_error(eng.h).decode())
        b.record(stream)
        evs.append((a, b))
    torch.cuda.synchronize()
    st = abi.RcStepStats()
    rc = lib.rc_wait(eng.h, C.byref(st))
    if rc != 0:
        raise RuntimeError(lib.rc_last_error(eng.h).decode())
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    # per-stage kernel times (events around each stage launch, same stream,
    # direct launches) over a second run of timed steps, L2 flushed likewise
    lib.rc_set_timing(eng.h, 1)
    lib.rc_timers(eng.h, None, None, 1)
    st2 = abi.RcStepStats()
    prof_steps = max(1, min(args.steps, 10))
    for _ in range(prof_steps):
        flush.zero_()
        lib.rc_step_async(eng.h, 1)
    torch.cuda.synchronize()
    lib.rc_wait(eng.h, C.byref(st2))
    tms = (C.c_double * abi.NUM_TIMERS)()
    tn = (C.c_longlong * abi.NUM_TIMERS)()
    lib.rc_timers(eng.h, tms, tn, 1)
    lib.rc_set_timing(eng.h, 0)
    # max over ranks of the timed region, sum over ranks of the sites updated
    from rheocell_gb300 import replicas
    ms, total_sites = replicas.reduce_timing(ms, float(S * args.steps))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()

    # end-to-end through the C ABI with host buffers
    import numpy as np
    host = torch.empty(S, dtype=torch.float64, pin_memory=True)
    hp = C.cast(host.data_ptr(), abi.DP)
    lib.rc_download_phi(eng.h, hp, S)
    e2e_steps = max(1, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        if lib.rc_upload_phi(eng.h, hp, S) != 0 or lib.rc_step(eng.h, 1, None) != 0 or lib.rc_download_phi(eng.h, hp, S) != 0:
            raise RuntimeError(lib.rc_last_error(eng.h).decode())
    e2e_s = time.perf_counter() - t0
    S_after = eng.site_count()
    eng.close()
    e2e_ms, e2e_sites = replicas.reduce_timing(e2e_s * 1e3, float(S * e2e_steps))

    value = total_sites / (ms / 1e3)
    names = abi.TIMER_NAMES
    stage = {names[i]: {"ms": round(tms[i], 3), "launches": int(tn[i])} for i in range(abi.NUM_TIMERS) if tn[i]}
    peak, peak_kind = measured_peaks()
    dom = max(range(abi.NUM_TIMERS), key=lambda i: tms[i])
    dom_avg_s = tms[dom] / max(tn[dom], 1) / 1e3
    if names[dom] == "solve" and args.solver == "learned":
        it_per_launch = st2.cg_iterations / max(tn[dom], 1)
        ref_per_launch = st2.refinements / max(tn[dom], 1)
        bytes_launch = learned_bytes_per_launch(S, L2, it_per_launch, ref_per_launch)
        unit_desc = ("learned solve: %.1f inner component-iterations and %.1f refinement sweeps per launch "
                     "(FP32 flexible CG, BF16 network, FP64 residuals); binding limit: grid barriers and the "
                     "network's row pipeline, not DRAM or the tensor pipe (profiles/cg_kernel_learned_wet512.md)"
                     % (it_per_launch, ref_per_launch))
    elif names[dom] == "solve":
        it_per_launch = st2.cg_iterations / max(tn[dom], 1)
        bytes_launch = cg_bytes_per_launch(S, L2, it_per_launch)
        unit_desc = "viscous solve: %.1f component-iterations per launch" % it_per_launch
    else:
        bytes_launch = fused_bytes_per_site(w["params"]["interaction_type"]) / 2 * S
        unit_desc = "per-cell update kernel: 36 B/site per launch"
    achieved = bytes_launch / dom_avg_s / 1e9
    traffic = None
    # DRAM bytes per launch of the dominant kernel from an ncu capture of the
    # same workload, precision and solver (profiles/), when one was taken
    prof = os.path.join(ROOT, "profiles", "traffic_%s_%s%s.json" % (args.workload, args.precision,
                                                                 "_learned" if args.solver == "learned" else ""))
    if os.path.exists(prof):
        try:
            traffic = json.load(open(prof)).get(names[dom])
        except Exception:
            traffic = None
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "site-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "steps_per_s": args.steps / (ms / 1e3),
        "higher_is_better": True,
        "scaling": "strong" if sharded else "weak",
        "vs_baseline": None,
        "dtype": {"double": "f64", "mixed": "f64 fields, f32 solve inner iterations",
                  "float": "f32 site arithmetic, f64 field storage and cell-area integrals"}[args.precision],
        "data": "synthetic (seeded jittered lattice, tanh interfaces)",
        "config": dict(arm_config(args, w, all_members), parallelism=("ensemble sharded by member" if sharded else "replicas") if world > 1 else "single GPU",
                       l2="flushed (256 MiB write) before every timed step"),
        "cg": {"solves": st.cg_solves, "iterations": st.cg_iterations, "max_iterations": st.cg_max_iterations,
               "max_rel_residual": st.cg_max_rel_residual,
               "ms_per_step": tms[3] / prof_steps if tn[3] else 0.0},
        "stages_ms": stage,
        "stages_note": "per-stage CUDA-event totals over %d further steps (direct launches)" % prof_steps,
        "gpu_launches": int(st.kernel_launches),
        "clocks": clk,
        "e2e": {"value": e2e_sites / (e2e_ms / 1e3), "unit": "site-updates/s",
                "h2d_bytes_per_step": 8 * S, "d2h_bytes_per_step": 8 * S,
                "how": "rc_upload_phi (pinned) + rc_step(1) + rc_download_phi (pinned), wall clock, %d steps" % e2e_steps},
        "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes_per_launch": bytes_launch, "launch_ms": dom_avg_s * 1e3,
                     "units": unit_desc, "traffic": traffic},
    }
    if S_after != S:
        out["config"]["sites_after"] = S_after
    if tuned is not None:
        out["config"]["cell_tile_threads"] = tuned["chosen"]
        out["autotune"] = {"cell_kernels_ms_per_step": {str(t): round(ms, 4) for t, ms in tuned["candidates"]},
                           "chosen": tuned["chosen"]}
    # the phi update (the per-cell update kernel alone; its per-cell epilogue
    # is timed apart) against its roofline.  Algorithmic bytes per site =
    # the update's inputs and outputs as the engine stores them: phi and the
    # solve's velocities in FP64, the force evaluation's mu and gradient
    # (FP32 engines: FP32, 12 B; FP64 engines: 24 B), dphi^n (FP32 engines:
    # FP32).  Predictor: read phi, vx, vy, mu, d_x phi, d_y phi, write phi*,
    # dphi; corrector: read phi^n, dphi, vx, vy, mu, d_x phi, d_y phi, write
    # phi^{n+1}: 48 B each on FP32 engines (64 B on FP64 engines).  Beside it,
    # the analysis formula of the update (reads phi* in the corrector, leaves
    # out mu and the gradient): 36 + 44 B (FP32 dphi), 40 + 48 B (FP64).
    iu = names.index("update")
    if tn[iu] and args.workload.startswith("wet"):
        upd_s = tms[iu] / tn[iu] / 1e3
        alg = 48.0 if args.precision == "float" else 64.0
        formula = 40.0 if args.precision == "float" else 44.0
        ie = names.index("epilogue")
        out["phi_update"] = {
            "kernel": "cell_update_bulk" if args.precision == "float" else "cell_kernel",
            "launch_ms": upd_s * 1e3, "launches": int(tn[iu]),
            "achieved_gbs": alg * S / upd_s / 1e9, "frac": alg * S / upd_s / 1e9 / peak,
            "algorithmic_bytes_per_site": alg,
            "formula_bytes_per_site": formula, "formula_frac": formula * S / upd_s / 1e9 / peak,
            "epilogue_ms": tms[ie] / tn[ie] if tn[ie] else None,
            "peak": peak, "unit": "GB/s"}
    if learned is not None:
        out["learned_pcg"] = learned
        out["dtype"] = {"double": "f64 fields, f32 solve inner iterations, bf16 learned preconditioner",
                        "mixed": "f64 fields, f32 solve inner iterations, bf16 learned preconditioner",
                        "float": "f32 site arithmetic (f64 field storage and cell-area integrals), f32 solve "
                                 "inner iterations with f64 refinement, bf16 learned preconditioner"}[args.precision]
    if args.precision != "double" and args.workload.startswith("wet"):
        out["field_error_vs_fp64"] = field_errors(args, eng_device=dev)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, w, members)
        if out["cpu_baseline"]["kind"] == "reference" and len(members) == 1:
            # the restatement beside it: how far the port's speed is from the reference's
            out["cpu_baseline_port"] = cpu_baseline(args, w, members, kind="port")
    return out


# A 1024^2 or 512^2 main-loop step of the CPU codes takes minutes (the
# reference's alone about a quarter of an hour at 1024^2 on one core), so
# their bounded sample is the 256^2 / 400-cell monolayer of the same physics
# (area fraction, R, xi, eta, activity).  Its solves need fewer iterations
# (about 48 against 65 per solve on the device), so the CPU rate measured
# there is an upper bound on the CPU rate at the larger box.
SAMPLE_OF = {"wet1024": "wet256", "wet512": "wet256"}


def reference_driver():
    """The reference built out of tree with its own Release flags
    (oracle/_ref/<machine>/ref_driver_fast), or None."""
    import platform
    path = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "ref_driver_fast")
    return path if os.access(path, os.X_OK) else None


def _time_reference_case(exe, keys, m, steps):
    """Wall-clock seconds of `steps` main-loop steps of the reference on one
    monolayer (its driver's std::chrono around the loop; set-up untimed)."""
    import shutil
    import tempfile
    from rheocell_gb300 import generator as g
    d = tempfile.mkdtemp(prefix="rc_refcase_")
    try:
        g.write_case(d, m, keys, steps=steps, seed=int(keys.get("seed", 1)))
        res = subprocess.run([exe, "time", str(steps), "input"], cwd=d, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("reference driver failed: %s" % res.stderr[-1000:])
        line = [ln for ln in res.stdout.splitlines() if ln.startswith("{")][-1]
        return float(json.loads(line)["seconds"])
    finally:
        shutil.rmtree(d, ignore_errors=True)


def _reference_worker(group):
    """Reference steps of each (exe, keys, monolayer, seconds) of a group:
    one step to size the sample, then as many as fit the member's share.
    Returns (site-updates, stepping seconds, steps)."""
    work, el, n = 0.0, 0.0, 0
    for exe, keys, m, budget in group:
        t1 = _time_reference_case(exe, keys, m, 1)
        k = int(budget / t1) if t1 > 0 else 1
        if k >= 2:
            t = _time_reference_case(exe, keys, m, k)
        else:
            k, t = 1, t1
        work += m.sites * k
        el += t
        n += k
    return work, el, n


def _port_worker(group):
    """The CPU restatement (oracle/) on each (keys, monolayer, seconds) of a
    group; returns (site-updates, stepping seconds, steps)."""
    sys.path.insert(0, ROOT)
    from oracle import oracle as orc
    from rheocell_gb300 import host
    work, el, n = 0.0, 0.0, 0
    for keys, m, budget in group:
        p, cells = host.engine_inputs(keys, m)
        sim = orc.OracleSim(p, m.L, cells)
        sim.set_phase(1)
        t0 = time.perf_counter()
        k = 0
        while True:
            sim.step(1)
            k += 1
            t = time.perf_counter() - t0
            if t >= budget or t / k * (k + 1) > budget * 1.5:
                break
        sim.close()
        el += t
        work += m.sites * k
        n += k
    return work, el, n


def cpu_baseline(args, w, members, budget_s=25.0, kind=None):
    """A CPU implementation of the path timed on this host over a bounded
    sample of the workload: the reference's own build (kind "reference",
    oracle/_ref, the reference's Release flags) when it was built here, else
    the CPU restatement (kind "port", oracle/, the reference's algorithm in
    serial C).  One monolayer: main-loop steps on one core (the reference
    steps serially); the 512^2 and 1024^2 boxes are sampled on the 256^2 box
    of the same physics (SAMPLE_OF).  An ensemble: its independent members
    spread over the host cores, aggregate = sum over workers of work / time."""
    import multiprocessing as mp
    exe = reference_driver()
    if kind is None:
        kind = "reference" if exe else "port"
    if kind == "reference" and not exe:
        raise RuntimeError("the reference build (oracle/_ref) is missing")
    sample_name = SAMPLE_OF.get(args.workload)
    sample_members = make_case(workload(sample_name)) if sample_name else members
    what = ("the reference's own build (Release flags -O3 -ffast-math -march=native, Eigen CG through the "
            "documented-semantics shim)" if kind == "reference" else "the CPU restatement (serial C)")
    if len(sample_members) == 1:
        keys, m = sample_members[0]
        item = [(exe, keys, m, budget_s)] if kind == "reference" else [(keys, m, budget_s)]
        work, el, steps = (_reference_worker if kind == "reference" else _port_worker)(item)
        where = ("the %dx%d / %d-cell monolayer of the same physics (a %s step takes minutes on one core)"
                 % (m.L, m.L, m.n, args.workload) if sample_name else "the same workload")
        sample = "%s: %d main-loop step(s) of %s, %.1f s of stepping" % (what, steps, where, el)
        return {"value": work / el, "unit": "site-updates/s", "cores": 1, "kind": kind, "sample": sample}
    cores = max(1, min(os.cpu_count() or 1, len(sample_members)))
    per_member = budget_s * cores / len(sample_members)
    groups = [[] for _ in range(cores)]
    for i, (keys, m) in enumerate(sample_members):
        groups[i % cores].append((exe, keys, m, per_member) if kind == "reference" else (keys, m, per_member))
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_reference_worker if kind == "reference" else _port_worker, groups)
    value = sum(wk / t for wk, t, _ in res if t > 0)
    steps = sum(n for _, _, n in res)
    el = max(t for _, t, _ in res)
    sample = ("%s: %d main-loop steps over the %d members (>= 1 each, about %.1f s per member), %d worker "
              "processes, %.1f s of stepping per worker" % (what, steps, len(sample_members), per_member, cores, el))
    return {"value": value, "unit": "site-updates/s", "cores": cores, "kind": kind, "sample": sample}


def run_reference(args, rank, world):
    """Reference arm: the reference's own CPU build of the path (oracle/_ref,
    compiled on this host from the reference's sources with its Release
    flags) on all the host cores the path can use -- one for a monolayer,
    whose stepping is serial in the reference; the ensemble's members in
    parallel -- over a bounded sample of the workload (cpu_baseline).  Falls
    back to the CPU restatement where the reference could not be built."""
    if rank != 0:
        return None
    w = workload(args.workload)
    members = make_case(w)
    base = cpu_baseline(args, w, members, budget_s=90.0)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": base["value"],
        "unit": "site-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded jittered lattice, tanh interfaces)",
        "config": arm_config(args, w, members),
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def arm_config(args, w, members):
    """The `config` block both arms print for the workload."""
    cfg = {"workload": w["name"], "L": [m.L for _, m in members] if len(members) > 1 else members[0][1].L,
           "monolayers": len(members), "cells": sum(m.n for _, m in members),
           "sites": sum(m.sites for _, m in members), "precision": args.precision}
    if args.solver == "learned":
        cfg["solver"] = "learned flexible CG (FP32 inner, FP64 refinement)"
    return cfg


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="wet1024",
                    choices=["wet1024", "wet512", "wet256", "dry140", "ensemble64", "ensemble64wet"])
    ap.add_argument("--precision", default=None, choices=["double", "mixed", "float"],
                    help="default: float (FP32 site arithmetic) for the wet workloads, double otherwise")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--solver", default=None, choices=["plain", "learned"],
                    help="viscous solver (default: learned for the wet workloads)")
    ap.add_argument("--harvest-steps", type=int, default=320)
    ap.add_argument("--harvest-capacity", type=int, default=8000)
    ap.add_argument("--train-epochs", type=int, default=30)
    ap.add_argument("--solver-phases", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default cell tile (FP32 only)")
    ap.add_argument("--train-workload", default="wet256", choices=["wet256", "wet512", "wet1024"],
                    help="harvest and train on this monolayer (the network transfers to the timed one)")
    ap.add_argument("--train-max-samples", type=int, default=0, help="train on at most this many samples (0: all)")
    ap.add_argument("--save-params", default=None, help="write the trained network parameters to this file")
    ap.add_argument("--load-params", default=None, help="use these network parameters instead of training")
    ap.add_argument("--train-lr", type=float, default=2e-3)
    ap.add_argument("--train-lr-final", type=float, default=0.05, help="final step size as a fraction of --train-lr")
    args = ap.parse_args()
    if args.precision is None:
        args.precision = "float" if args.workload.startswith("wet") else "double"
    if args.solver is None:
        args.solver = "learned" if args.workload.startswith("wet") else "plain"
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        from rheocell_gb300 import build
        if rank == 0:
            build.build()  # in-tree; the other ranks wait for it
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        out = run_gb300(args, rank, world)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
