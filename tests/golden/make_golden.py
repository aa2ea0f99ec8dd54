"""Generate the golden fixtures in this directory from the reference itself.

Runs the unmodified reference (compiled out of tree by oracle/Makefile into
oracle/_ref/ref_driver_exact; the wet models use the project's Eigen-API
shim) on small seeded cases written by rheocell_gb300.generator, and stores
its state dumps as compressed .npz files:

  * per recorded step: every per-cell scalar of the dump;
  * phi at the first and the last recorded step after step 0;
  * at the last recorded step also vx, vy, mu and the box map.

Run from the repository root:  python tests/golden/make_golden.py
(needs the reference built out of tree, `make -C oracle REF_SRC=<reference>/src`;
only a machine with the reference's sources can run it).
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from rheocell_gb300 import generator as g  # noqa: E402
from oracle import refdump  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

SMALL = dict(R=5, lam=1.5, patch=27)
DRY_POLAR_S = dict(g.DRY_POLAR, R=5)
NEMATIC_S = dict(interaction_type="activenematic", R=5, dt=0.1, gamma=0.06, mu=45, kappa=0.1,
                 **{"lambda": 1.5}, friction=1, zetaQ_self=0.1, zetaQ_inter=0.05, J_Q=0.5, omega=0.004)
WET_S = dict(g.WET_NEMATIC, R=5, **{"lambda": 1.5}, omega=0.004, zetaQ_inter=0.02)
WETPOLAR_S = dict(DRY_POLAR_S, friction_cell=1, CGtolerance=1e-8, J_Q=0.3, zetaQ_inter=0.1)
SIMPLE_S = dict(interaction_type="simplefield", R=5, dt=0.1, gamma=0.06, mu=45, kappa=0.1, omega=0)

# name: (monolayer kwargs, params, dump steps, seed, equilibration steps)
CASES = {
    "polar_dry": (dict(L=48, n=9, seed=3, **SMALL), DRY_POLAR_S, [0, 1, 2, 10], 11, 0),
    "polar_noise": (dict(L=36, n=4, seed=4, **SMALL), dict(DRY_POLAR_S, zetaQ_inter=0.2, J_Q=0.5), [0, 1, 5], 12, 0),
    "nematic": (dict(L=48, n=9, seed=5, types=[0, 1, 1, 0, 1, 1, 0, 1, 1], **SMALL), NEMATIC_S, [0, 1, 10], 13, 0),
    "simple": (dict(L=36, n=4, seed=6, **SMALL), SIMPLE_S, [0, 1, 5], 14, 0),
    "wet": (dict(L=48, n=9, seed=7, **SMALL), WET_S, [0, 1, 4], 15, 0),
    "wetpolar": (dict(L=36, n=4, seed=8, **SMALL), WETPOLAR_S, [0, 1, 4], 16, 0),
    "wet_equil": (dict(L=36, n=4, seed=9, **SMALL), WET_S, [0, 2], 17, 3),
    "polar41": (dict(L=64, n=4, seed=10), g.DRY_POLAR, [0, 1, 3], 18, 0),
    "resize": (dict(L=64, n=4, seed=11, R=5, lam=1.5, patch=27, aspect=2.2), DRY_POLAR_S, [0, 1, 2], 19, 0),
    # conserved dynamics (sim_type = FD_CH); the fourth-order update wants a smaller dt
    "ch_polar": (dict(L=48, n=9, seed=21, **SMALL), dict(DRY_POLAR_S, sim_type="FD_CH", dt=0.01), [0, 1, 5], 31, 0),
    "ch_nematic": (dict(L=48, n=9, seed=22, types=[0, 1, 1, 0, 1, 1, 0, 1, 1], **SMALL),
                   dict(NEMATIC_S, sim_type="FD_CH", dt=0.01), [0, 1, 5], 32, 0),
    "ch_wet": (dict(L=36, n=4, seed=23, **SMALL), dict(WET_S, sim_type="FD_CH", dt=0.01), [0, 1, 3], 33, 0),
    "ch_simple": (dict(L=36, n=4, seed=28, **SMALL), dict(SIMPLE_S, sim_type="FD_CH", dt=0.01), [0, 1, 5], 38, 0),
    "ch_wetpolar": (dict(L=36, n=4, seed=29, **SMALL), dict(WETPOLAR_S, sim_type="FD_CH", dt=0.01), [0, 1, 3], 39, 0),
    # the polar model's perimeter term (beta != 0) with adhesion, dry and wet
    "polar_beta": (dict(L=48, n=9, seed=24, **SMALL), dict(DRY_POLAR_S, beta=0.5, J_Q=0.5, zetaQ_inter=0.3, omega=0.004),
                   [0, 1, 5], 34, 0),
    "wetpolar_beta": (dict(L=36, n=4, seed=25, **SMALL), dict(WETPOLAR_S, beta=0.3, omega=0.004), [0, 1, 4], 35, 0),
    # past the viscous solve's cold restarts: one solve per force evaluation,
    # a cold start every 100 warm solves (wetmodel) or every 10 (wetpolarmodel)
    "wet_restart": (dict(L=36, n=4, seed=26, **SMALL), WET_S, [0, 1, 52], 36, 0),
    "wetpolar_restart": (dict(L=36, n=4, seed=27, **SMALL), WETPOLAR_S, [0, 1, 7], 37, 0),
    # wall boxes (box = square with type = square_walls / circle_walls /
    # triangle_walls): the wall branches of the stencils, adhesion and forces
    "walls_polar": (dict(L=48, n=9, seed=41, **SMALL),
                    dict(DRY_POLAR_S, type="square_walls", lambda_wall=4, beta=0.5, J_Q=0.5, zetaQ_inter=0.3,
                         omega=0.004), [0, 1, 5], 51, 0),
    "walls_simple": (dict(L=36, n=4, seed=42, **SMALL), dict(SIMPLE_S, type="circle_walls", lambda_wall=3),
                     [0, 1, 5], 52, 0),
    "walls_wetdry": (dict(L=48, n=9, seed=43, **SMALL), dict(WET_S, friction_cell=0, type="triangle_walls", lambda_wall=3),
                     [0, 1, 5], 53, 0),
    "walls_ch_polar": (dict(L=36, n=4, seed=44, **SMALL),
                       dict(DRY_POLAR_S, sim_type="FD_CH", dt=0.01, type="square_walls", lambda_wall=3, wall_slip=0.7),
                       [0, 1, 5], 54, 0),
}


# Full-size cases stored compactly: the project generator regenerates the
# configuration (its text is checked against the recorded SHA-256), per-cell
# scalars are stored as they are, and per-site arrays as SHA-256 digests of
# their bytes -- the dry oracle must reproduce them bit for bit -- with their
# sums of squares to size a mismatch.
# name: (monolayer kwargs, params, dump steps, seed)
HASHED = {
    # the 140x140 / 100-cell dry polar workload on 41x41 patches, over 100 steps
    "dry140_100": (dict(L=140, n=100, seed=1), g.DRY_POLAR, [0, 1, 10, 100], 1),
}


# Full-size wet cases: the viscous solve reduces in another order than the
# reference's (shim) CG, so per-site arrays are held to 1e-12 relative, not bit
# for bit; they are stored at SAMPLE_SITES fixed sites (numpy seed 0) with
# their sums of squares.  name: (monolayer kwargs, params, dump steps, seed)
SAMPLED = {
    # the 256x256 / 400-cell wet nematic workload on 41x41 patches
    "wet256": (dict(L=256, n=400, seed=1), g.WET_NEMATIC, [0, 1, 2], 1),
}
SAMPLE_SITES = 8192


def sample_index(n_sites: int) -> np.ndarray:
    return np.sort(np.random.default_rng(0).choice(n_sites, size=min(SAMPLE_SITES, n_sites), replace=False))


def record_sampled(name):
    mkw, params, steps, seed = SAMPLED[name]
    m = monolayer(mkw)
    d = tempfile.mkdtemp(prefix="rc_golden_")
    try:
        g.write_case(d, m, params, steps=max(steps), seed=seed)
        recs = refdump.run_reference(d, steps, flavour="exact")
        conf = open(os.path.join(d, "start_conf.dat")).read()
        topo = open(os.path.join(d, "topology.top")).read()
        inp = open(os.path.join(d, "input")).read()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    assert conf == conf_text(monolayer(mkw))
    out = {"monolayer": np.array(json.dumps(mkw)), "conf_sha256": np.array(hashlib.sha256(conf.encode()).hexdigest()),
           "topology": np.array(topo), "input": np.array(inp),
           "steps": np.array([r["step"] for r in recs], dtype=np.int64)}
    for r in recs:
        s = r["step"]
        for k in refdump.CELL_I32 + refdump.CELL_F64:
            out["s%d_%s" % (s, k)] = r[k]
        if s > 0:
            idx = sample_index(r["phi"].size)
            out["s%d_phi_sample" % s] = r["phi"][idx]
            out["s%d_phi_sumsq" % s] = np.array(float(np.sum(r["phi"] ** 2)))
    last = recs[-1]
    idx = sample_index(last["vx"].size)
    for k in ("vx", "vy", "mu"):
        out["last_%s_sample" % k] = last[k][idx]
        out["last_%s_sumsq" % k] = np.array(float(np.sum(last[k] ** 2)))
    out["last_map_sha256"] = np.array(sha256_of(last["map"], "<i8"))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return recs


def sha256_of(a, dtype) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()


def conf_text(m) -> str:
    d = tempfile.mkdtemp(prefix="rc_golden_")
    try:
        g.write_conf(os.path.join(d, "start_conf.dat"), m)
        return open(os.path.join(d, "start_conf.dat")).read()
    finally:
        shutil.rmtree(d, ignore_errors=True)


def record_hashed(name):
    mkw, params, steps, seed = HASHED[name]
    m = monolayer(mkw)
    d = tempfile.mkdtemp(prefix="rc_golden_")
    try:
        g.write_case(d, m, params, steps=max(steps), seed=seed)
        recs = refdump.run_reference(d, steps, flavour="exact")
        conf = open(os.path.join(d, "start_conf.dat")).read()
        topo = open(os.path.join(d, "topology.top")).read()
        inp = open(os.path.join(d, "input")).read()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    assert conf == conf_text(monolayer(mkw))
    out = {"monolayer": np.array(json.dumps(mkw)), "conf_sha256": np.array(hashlib.sha256(conf.encode()).hexdigest()),
           "topology": np.array(topo), "input": np.array(inp),
           "steps": np.array([r["step"] for r in recs], dtype=np.int64)}
    for r in recs:
        s = r["step"]
        for k in refdump.CELL_I32 + refdump.CELL_F64:
            out["s%d_%s" % (s, k)] = r[k]
        if s > 0:
            out["s%d_phi_sha256" % s] = np.array(sha256_of(r["phi"], "<f8"))
            out["s%d_phi_sumsq" % s] = np.array(float(np.sum(r["phi"] ** 2)))
    last = recs[-1]
    for k in ("vx", "vy", "mu"):
        out["last_%s_sha256" % k] = np.array(sha256_of(last[k], "<f8"))
        out["last_%s_sumsq" % k] = np.array(float(np.sum(last[k] ** 2)))
    out["last_map_sha256"] = np.array(sha256_of(last["map"], "<i8"))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return recs


def monolayer(kw):
    kw = dict(kw)
    return g.make_monolayer(kw.pop("L"), kw.pop("n"), kw.pop("seed"), **kw)


def record(name):
    mkw, params, steps, seed, eq = CASES[name]
    m = monolayer(mkw)
    d = tempfile.mkdtemp(prefix="rc_golden_")
    try:
        g.write_case(d, m, params, steps=max(steps), seed=seed, equilibration_steps=eq)
        recs = refdump.run_reference(d, steps, flavour="exact")
        conf = open(os.path.join(d, "start_conf.dat")).read()
        topo = open(os.path.join(d, "topology.top")).read()
        inp = open(os.path.join(d, "input")).read()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    out = {"conf": np.array(conf), "topology": np.array(topo), "input": np.array(inp),
           "steps": np.array([r["step"] for r in recs], dtype=np.int64)}
    for i, r in enumerate(recs):
        s = r["step"]
        for k in refdump.CELL_I32 + refdump.CELL_F64:
            out["s%d_%s" % (s, k)] = r[k]
        if s > 0 and (i == 1 or i == len(recs) - 1):
            out["s%d_phi" % s] = r["phi"]
    last = recs[-1]
    for k in ("vx", "vy", "mu", "map"):
        out["last_%s" % k] = last[k]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return recs


def record_overlap():
    """21 patches on one spot: the reference aborts (WetModel.cpp:475-480)."""
    pos = np.tile([[24.3, 24.7]], (21, 1))
    m = g.make_monolayer(48, 21, seed=1, R=5, lam=1.5, patch=27, positions=pos)
    d = tempfile.mkdtemp(prefix="rc_golden_")
    try:
        g.write_case(d, m, DRY_POLAR_S, steps=1, seed=1)
        res = subprocess.run([refdump.driver_path("exact"), "dump", os.path.join(d, "x.bin"), "1", "input"],
                             cwd=d, capture_output=True, text=True)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    info = {"returncode": res.returncode, "overlap_error": "Too many field patches overlap" in res.stderr}
    with open(os.path.join(HERE, "overlap.json"), "w") as f:
        json.dump(info, f, indent=1)
    return info


def record_cli():
    """The reference's own executable (rheoCell input) on a small dry polar
    case with equilibration and periodic printing: its output files are the
    goldens of the stand-alone driver (rheocell_gb300/_build/rheocell)."""
    m = g.make_monolayer(48, 9, seed=21, **SMALL)
    d = tempfile.mkdtemp(prefix="rc_golden_")
    try:
        g.write_case(d, m, dict(DRY_POLAR_S, J_Q=0.2, zetaQ_inter=0.1), steps=20, seed=23, equilibration_steps=3,
                     extra=dict(print_conf_interval=10))
        res = subprocess.run([os.path.join(refdump.REF_DIR, "rheoCell_exact"), "input"], cwd=d,
                             capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(res.stderr[-2000:])
        out = {}
        for f in ("input", "topology.top", "start_conf.dat", "trajectory.dat", "last_conf.dat",
                  "equilibrated_conf.dat"):
            out[f.replace(".", "_")] = np.array(open(os.path.join(d, f)).read())
    finally:
        shutil.rmtree(d, ignore_errors=True)
    np.savez_compressed(os.path.join(HERE, "cli_polar.npz"), **out)


def record_confgenerator():
    """The reference's confGenerator on three placement modes: byte-exact
    goldens for rheocell_gb300/_build/confgenerator."""
    out = {}
    for mode, inter in (("random", "wetmodel"), ("lattice", "wetpolarmodel"), ("cluster", "wetpolarmodel")):
        d = tempfile.mkdtemp(prefix="rc_golden_")
        try:
            with open(os.path.join(d, "topo.top"), "w") as f:
                f.write("6 1\n0 1 0 1 0 1\n")
            inp = ("interaction_type = %s\nR = 8\nseed = 77\ntopology = topo.top\nconf_file = ref.dat\n"
                   "trajectory_file = t.dat\ninitial_configuration_type = %s\nn_rows = 2\nn_columns = 3\n" % (inter, mode))
            with open(os.path.join(d, "input"), "w") as f:
                f.write(inp)
            subprocess.run([os.path.join(refdump.REF_DIR, "confGenerator_exact"), "input", "80"], cwd=d,
                           capture_output=True, check=True)
            out[mode + "_input"] = np.array(inp)
            out[mode + "_conf"] = np.array(open(os.path.join(d, "ref.dat")).read())
        finally:
            shutil.rmtree(d, ignore_errors=True)
    np.savez_compressed(os.path.join(HERE, "confgenerator.npz"), **out)


# field observables of the reference (ForceField, StressField) after `step`
# main-loop steps: name -> (monolayer kwargs, params, step, seed, size_grid)
OBS_CASES = {
    "obs_wet": (dict(L=36, n=4, seed=41, **SMALL), WET_S, 2, 51, 3),
    "obs_wetpolar": (dict(L=36, n=4, seed=42, **SMALL), WETPOLAR_S, 2, 52, 3),
    "obs_nematic": (dict(L=36, n=4, seed=43, types=[0, 1, 1, 0], **SMALL), NEMATIC_S, 2, 53, 4),
    "obs_polar": (dict(L=36, n=4, seed=44, **SMALL), dict(DRY_POLAR_S, J_Q=0.3), 2, 54, 3),
    "obs_simple": (dict(L=36, n=4, seed=45, **SMALL), SIMPLE_S, 2, 55, 3),
}


def record_observables(name):
    """The reference's own ForceField, StressField and ThermodynamicStressField output strings (its
    observable classes, driven by oracle/ref_driver.cpp's observe mode) as
    number arrays after the two header lines."""
    mkw, params, step, seed, sg = OBS_CASES[name]
    m = monolayer(mkw)
    d = tempfile.mkdtemp(prefix="rc_golden_")
    out = {}
    try:
        g.write_case(d, m, params, steps=step, seed=seed)
        for kind in ("force_field", "stress_field", "thermodynamic_stress_field"):
            res = subprocess.run([refdump.driver_path("exact"), "observe", kind + ".txt", "%d:%s:%d" % (step, kind, sg),
                                  "input"], cwd=d, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(res.stderr[-2000:])
            lines = open(os.path.join(d, kind + ".txt")).read().split("\n", 2)
            out[kind] = np.array(lines[2].split(), dtype=np.float64)
        for f, k in (("start_conf.dat", "conf"), ("topology.top", "topology"), ("input", "input")):
            out[k] = np.array(open(os.path.join(d, f)).read())
    finally:
        shutil.rmtree(d, ignore_errors=True)
    out["step"] = np.array(step)
    out["size_grid"] = np.array(sg)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def main():
    if not refdump.have_reference("exact"):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "-j8"])
    only = sys.argv[1:]  # optional: record only these cases
    for name in HASHED:
        if only and name not in only:
            continue
        recs = record_hashed(name)
        print("%-12s steps %s  cells %d  %.0f KB" % (name, [r["step"] for r in recs], recs[0]["N"],
                                                  os.path.getsize(os.path.join(HERE, name + ".npz")) / 1024))
    for name in SAMPLED:
        if only and name not in only:
            continue
        recs = record_sampled(name)
        print("%-12s steps %s  cells %d  %.0f KB" % (name, [r["step"] for r in recs], recs[0]["N"],
                                                  os.path.getsize(os.path.join(HERE, name + ".npz")) / 1024))
    for name in CASES:
        if only and name not in only:
            continue
        recs = record(name)
        sz = os.path.getsize(os.path.join(HERE, name + ".npz"))
        print("%-12s steps %s  cells %d  sizes %s  %.0f KB" % (name, [r["step"] for r in recs], recs[0]["N"],
                                                                sorted(set(zip(recs[-1]["lx"], recs[-1]["ly"]))), sz / 1024))
    for name in OBS_CASES:
        if only and name not in only:
            continue
        record_observables(name)
        print("%-12s %.0f KB" % (name, os.path.getsize(os.path.join(HERE, name + ".npz")) / 1024))
    if only:
        return
    print("overlap", record_overlap())
    record_cli()
    record_confgenerator()
    print("cli_polar %.0f KB" % (os.path.getsize(os.path.join(HERE, "cli_polar.npz")) / 1024))


if __name__ == "__main__":
    main()
