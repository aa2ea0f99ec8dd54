"""Helpers shared by the tests: fixtures from tests/golden, case set-up through
the host mirror, and runners for the engine (CUDA) and the oracle (CPU)."""
from __future__ import annotations

import os
import tempfile
from typing import Dict, List, Tuple

import numpy as np

from rheocell_gb300 import abi, generator as g, host

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name: str) -> Dict[str, np.ndarray]:
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def case_from_texts(input_text: str, conf_text: str, topo_text: str):
    """(keys, monolayer, params, cells) exactly as the reference reads them."""
    d = tempfile.mkdtemp(prefix="rc_case_")
    with open(os.path.join(d, "input"), "w") as f:
        f.write(input_text)
    with open(os.path.join(d, "conf"), "w") as f:
        f.write(conf_text)
    keys = host.read_input(os.path.join(d, "input"))
    m = g.read_conf(os.path.join(d, "conf"))
    types = [int(t) for t in topo_text.splitlines()[1].split()]
    m.types = types
    return keys, m


# case set-up shared with bench.py (rheocell_gb300.host / .generator)
build_inputs = host.engine_inputs
case_from_monolayer = g.case_keys


def run(sim_factory, keys, m, steps: List[int], eq: int = 0, precision=abi.RC_PRECISION_DOUBLE):
    """Run equilibration (phase 0), switch to phase 1, and return the states at
    the requested main-loop steps (0 = before the first main step)."""
    p, cells = build_inputs(keys, m, precision)
    walls = host.box_walls(keys, m.L)
    sim = sim_factory(p, m.L, cells) if walls is None else sim_factory(p, m.L, cells, walls=walls)
    for _ in range(eq):
        sim.step(1)
    sim.set_phase(1)
    out = {}
    cur = 0
    for s in sorted(steps):
        if s > cur:
            sim.step(s - cur)
            cur = s
        out[s] = sim.state()
    return sim, out


def rel_err(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    den = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / den


# dump key -> engine/oracle state key
CELL_KEYS = {"lx": "lsub_x", "ly": "lsub_y", "offx": "offset_x", "offy": "offset_y", "corner": "corner",
             "comx": "com_x", "comy": "com_y", "unrapx": "unrap_x", "unrapy": "unrap_y", "q00": "q00",
             "q01": "q01", "thetaq": "theta_q", "nemqx": "nemq_x", "nemqy": "nemq_y", "area": "area",
             "sumf": "sum_f", "perimeter": "perimeter", "s00": "s00", "s01": "s01",
             "frepx": "force_rep_x", "frepy": "force_rep_y"}
INT_KEYS = ("lx", "ly", "offx", "offy", "corner")


def compare_to_golden(gd, states: Dict[int, Dict[str, np.ndarray]], skip=(), absolute=()):
    """Max relative error of each compared quantity (0.0 means bit-identical);
    keys in `absolute` report the max absolute error instead."""
    errs = {}
    steps = [int(s) for s in gd["steps"]]
    for s in steps:
        st = states[s]
        for k, sk in CELL_KEYS.items():
            if k in skip:
                continue
            key = "s%d_%s" % (s, k)
            if key not in gd:
                continue
            if k in INT_KEYS:
                errs[(s, k)] = 0.0 if np.array_equal(gd[key], st[sk]) else float("inf")
            elif k in absolute:
                errs[(s, k)] = float(np.max(np.abs(np.asarray(st[sk], float) - gd[key]))) if len(gd[key]) else 0.0
            else:
                errs[(s, k)] = rel_err(st[sk], gd[key])
        if "s%d_phi" % s in gd:
            errs[(s, "phi")] = rel_err(st["phi"], gd["s%d_phi" % s])
    last = states[steps[-1]]
    for k, sk in (("vx", "vx"), ("vy", "vy"), ("mu", "mu")):
        if k not in skip:
            errs[("last", k)] = rel_err(last[sk], gd["last_" + k])
    errs[("last", "map")] = 0.0 if np.array_equal(last["box_index"], gd["last_map"]) else float("inf")
    return errs


def full_size_case(gd):
    """(keys, monolayer) of a full-size golden case whose configuration is not
    stored: it is regenerated from the recorded generator arguments and
    checked against the SHA-256 of the file the reference ran on."""
    import hashlib
    import json
    import shutil
    mkw = json.loads(str(gd["monolayer"]))
    m = g.make_monolayer(mkw.pop("L"), mkw.pop("n"), mkw.pop("seed"), **mkw)
    d = tempfile.mkdtemp(prefix="rc_case_")
    try:
        g.write_conf(os.path.join(d, "start_conf.dat"), m)
        conf = open(os.path.join(d, "start_conf.dat")).read()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    assert hashlib.sha256(conf.encode()).hexdigest() == str(gd["conf_sha256"])
    return case_from_texts(str(gd["input"]), conf, str(gd["topology"]))


def sampled_errors(gd, states):
    """Errors of a run against a full-size golden stored at sampled sites
    (tests/golden/make_golden.py SAMPLED): per-cell scalars in full, per-site
    arrays at the 8192 sites numpy seed 0 draws, and their sums of squares;
    the box map by digest.  Max relative error per quantity (inf: unequal
    integers)."""
    import hashlib

    def sample(a):
        a = np.asarray(a)
        return a[np.sort(np.random.default_rng(0).choice(a.size, size=min(8192, a.size), replace=False))]

    errs = {}
    steps = [int(s) for s in gd["steps"]]
    for s in steps:
        st = states[s]
        for k, sk in CELL_KEYS.items():
            if k in INT_KEYS:
                errs[(s, k)] = 0.0 if np.array_equal(st[sk], gd["s%d_%s" % (s, k)]) else float("inf")
            else:
                errs[(s, k)] = rel_err(st[sk], gd["s%d_%s" % (s, k)])
        if s > 0:
            errs[(s, "phi")] = rel_err(sample(st["phi"]), gd["s%d_phi_sample" % s])
            errs[(s, "phi_sumsq")] = rel_err(np.sum(np.asarray(st["phi"]) ** 2), gd["s%d_phi_sumsq" % s])
    last = states[steps[-1]]
    for k in ("vx", "vy", "mu"):
        errs[("last", k)] = rel_err(sample(last[k]), gd["last_%s_sample" % k])
        errs[("last", k + "_sumsq")] = rel_err(np.sum(np.asarray(last[k]) ** 2), gd["last_%s_sumsq" % k])
    digest = hashlib.sha256(np.ascontiguousarray(last["box_index"], dtype="<i8").tobytes()).hexdigest()
    errs[("last", "map")] = 0.0 if digest == str(gd["last_map_sha256"]) else float("inf")
    return errs
