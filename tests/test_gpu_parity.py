"""Parity of the CUDA engine (through its C ABI) with the reference's golden
dumps and with the CPU restatement.

Tolerances: every operation is the reference's IEEE FP64 arithmetic in its
order, except that well-conditioned per-cell sums (area, sums of phi,
centre-of-mass sums) use a fixed tree instead of the reference's sequential
loop, GPU atan2/cos/sin may differ from glibc in the last bit, and the viscous
solve reduces in its own order.  The bar is 1e-10 relative over 100 steps
(checked on the 140x140 / 100-cell workload).  Two per-cell sums cancel
strongly -- the shape tensor S of nearly round cells and the polar repulsion
totals -- and the reference itself is not reproducible there: its own
-ffast-math build differs from its exact build by 3e-7 in S01 and 2e-5 in the
repulsion totals.  Where they drive the dynamics (S for activenematic and
wetmodel, the totals for wetpolarmodel with J_Q != 0) the engine forms them in
the reference's sequential order.  S itself is compared in absolute terms at
1e-12, far below its summands (~1e-2 each): relative to its own small value it
amplifies 1e-16 differences in phi by ~1e6; the quantities it drives (Q, v,
phi) are held to the 1e-10 relative bar.  The repulsion totals are not tracked when J_Q = 0 in
both phases: then they are unused and no observable reads them."""
import numpy as np
import pytest

from oracle import oracle as orc
from rheocell_gb300 import abi, engine, generator as g
from tests.common import (build_inputs, case_from_monolayer, case_from_texts, compare_to_golden, golden,
                          rel_err, run)

pytestmark = pytest.mark.gpu

ALL = ["polar_dry", "polar_noise", "nematic", "simple", "polar41", "resize", "wet", "wetpolar", "wet_equil", "ch_polar",
       "ch_nematic", "ch_wet", "polar_beta", "wetpolar_beta", "walls_polar", "walls_simple", "walls_wetdry",
       "walls_ch_polar"]
EQ = {"wet_equil": 3}
TOL = 1e-10


def tolerances(keys):
    """(skipped keys, keys compared in absolute terms) for a case's inputs."""
    model = keys["interaction_type"]
    skip, absolute = set(), {"s00", "s01"}
    if model != "wetpolarmodel" or float(keys.get("J_Q", 0)) == 0.0:
        skip |= {"frepx", "frepy"}
    return skip, absolute


@pytest.mark.parametrize("name", ALL)
def test_engine_matches_reference_golden(name):
    gd = golden(name)
    keys, m = case_from_texts(str(gd["input"]), str(gd["conf"]), str(gd["topology"]))
    _, states = run(engine.Engine, keys, m, [int(s) for s in gd["steps"]], eq=EQ.get(name, 0))
    skip, absolute = tolerances(keys)
    errs = compare_to_golden(gd, states, skip=skip, absolute=absolute)
    bad = {k: v for k, v in errs.items() if v > (1e-12 if k[1] in absolute else TOL)}
    assert not bad, bad


def _pair(keys, m, steps, eq=0):
    _, a = run(engine.Engine, keys, m, steps, eq=eq)
    _, b = run(orc.OracleSim, keys, m, steps, eq=eq)
    return a, b


FIELDS = ["phi", "vx", "vy", "mu", "area", "com_x", "com_y", "q00", "q01", "nemq_x", "s00", "s01"]


def _check(a, b, steps, tol=TOL, fields=FIELDS, absolute=()):
    worst = {}
    for s in steps:
        for f in fields:
            if f in absolute:
                worst[(s, f)] = float(np.max(np.abs(a[s][f] - b[s][f]))) * (tol / 1e-12)
            else:
                worst[(s, f)] = rel_err(a[s][f], b[s][f])
        for f in ("lsub_x", "lsub_y", "corner", "offset_x", "offset_y"):
            assert np.array_equal(a[s][f], b[s][f]), (s, f)
        assert np.array_equal(a[s]["box_index"], b[s]["box_index"]), s
    bad = {k: v for k, v in worst.items() if v > tol}
    assert not bad, bad
    return worst


def test_dry_polar_140_100cells_100_steps():
    """The CPU-runnable workload: 140x140, 100 cells, 41x41 patches, dry polar."""
    m = g.make_monolayer(140, 100, seed=1)
    keys, m2 = case_from_monolayer(m, g.DRY_POLAR, seed=1)
    a, b = _pair(keys, m2, [1, 10, 100])
    _check(a, b, [1, 10, 100], absolute=("s00", "s01"))


def test_many_cells_split_epilogue_vs_oracle():
    """400 cells: the per-cell epilogue runs as its own kernel (one thread per
    cell); results must still follow the reference's arithmetic."""
    m = g.make_monolayer(256, 400, seed=12)
    keys, m2 = case_from_monolayer(m, dict(g.DRY_POLAR, zetaQ_inter=0.1, J_Q=0.2, omega=0.004), seed=13)
    a, b = _pair(keys, m2, [1, 3])
    _check(a, b, [1, 3], absolute=("s00", "s01"))


@pytest.mark.parametrize("model", ["activenematic", "simplefield"])
def test_dry_models_vs_oracle(model):
    m = g.make_monolayer(96, 36, seed=2, types=[i % 2 for i in range(36)])
    params = dict(g.DRY_POLAR, interaction_type=model, zetaQ_self=0.1, zetaQ_inter=0.05, J_Q=0.2, omega=0.004)
    keys, m2 = case_from_monolayer(m, params, seed=3)
    a, b = _pair(keys, m2, [1, 30])
    _check(a, b, [1, 30], absolute=("s00", "s01") if model == "simplefield" else ())


def test_polar_noise_and_torque_vs_oracle():
    m = g.make_monolayer(96, 36, seed=4)
    params = dict(g.DRY_POLAR, zetaQ_inter=0.3, J_Q=0.5, beta=0.5, omega=0.004)
    keys, m2 = case_from_monolayer(m, params, seed=5)
    a, b = _pair(keys, m2, [1, 20], eq=2)
    _check(a, b, [1, 20], fields=FIELDS + ["theta_q", "force_rep_x", "perimeter"], absolute=("s00", "s01"))


@pytest.mark.parametrize("model", ["wetmodel", "wetpolarmodel"])
def test_wet_vs_oracle(model):
    m = g.make_monolayer(64, 9, seed=6)
    params = dict(g.WET_NEMATIC, interaction_type=model, beta=0, zetaQ_inter=0.02, omega=0.004)
    keys, m2 = case_from_monolayer(m, params, seed=7)
    a, b = _pair(keys, m2, [1, 12])
    _check(a, b, [1, 12], tol=1e-9, absolute=("s00", "s01") if model == "wetpolarmodel" else ())


def test_deterministic_bitwise():
    m = g.make_monolayer(96, 36, seed=8)
    keys, m2 = case_from_monolayer(m, dict(g.WET_NEMATIC, zetaQ_inter=0.02), seed=9)
    _, a = run(engine.Engine, keys, m2, [5])
    _, b = run(engine.Engine, keys, m2, [5])
    for k in ("phi", "vx", "vy", "area", "com_x"):
        assert np.array_equal(a[5][k], b[5][k]), k


def test_overlap_is_an_error():
    pos = np.tile([[24.3, 24.7]], (21, 1))
    m = g.make_monolayer(48, 21, seed=1, R=5, lam=1.5, patch=27, positions=pos)
    keys, m2 = case_from_monolayer(m, dict(g.DRY_POLAR, R=5))
    p, cells = build_inputs(keys, m2)
    with pytest.raises(engine.EngineError) as ei:
        engine.Engine(p, m2.L, cells)
    assert ei.value.code == abi.RC_ERR_OVERLAP


def test_cg_residual_and_stats():
    """Every solve stops at |r| < tol |b| (Eigen's criterion)."""
    m = g.make_monolayer(128, 64, seed=10)
    keys, m2 = case_from_monolayer(m, g.WET_NEMATIC, seed=11)
    p, cells = build_inputs(keys, m2)
    e = engine.Engine(p, m2.L, cells)
    e.set_phase(1)
    st = e.step(3)
    assert st.steps_done == 3 and st.cg_solves == 3 * 2 * 2
    assert 0 < st.cg_max_rel_residual < 1e-8
    assert st.cg_iterations > 0


@pytest.mark.parametrize("model", ["wetmodel", "wetpolarmodel"])
def test_mixed_precision_solve(model):
    """backend_precision = mixed: FP32 inner CG in FP64 refinement reaches the
    same true-residual criterion; velocities stay within 1e-7 of FP64."""
    m = g.make_monolayer(96, 36, seed=12)
    params = dict(g.WET_NEMATIC, interaction_type=model, beta=0, zetaQ_inter=0.02)
    keys, m2 = case_from_monolayer(m, params, seed=13)
    _, a = run(engine.Engine, keys, m2, [1, 3], precision=abi.RC_PRECISION_MIXED)
    _, b = run(engine.Engine, keys, m2, [1, 3])
    for s in (1, 3):
        for f in ("vx", "vy"):
            assert rel_err(a[s][f], b[s][f]) < 1e-7, (s, f, rel_err(a[s][f], b[s][f]))
        assert rel_err(a[s]["phi"], b[s]["phi"]) < 1e-9
    p, cells = build_inputs(keys, m2, precision=abi.RC_PRECISION_MIXED)
    e = engine.Engine(p, m2.L, cells)
    e.set_phase(1)
    st = e.step(2)
    assert st.refinements >= 4 and 0 < st.cg_max_rel_residual < 1e-8


@pytest.mark.parametrize("model", ["wetpolarmodel", "activenematic", "simplefield", "wetmodel"])
def test_first_evaluation_bitwise(model):
    """One force evaluation from identical inputs is bit-identical to the CPU
    restatement (itself bit-identical to the reference's exact build): box
    sums in the reference's order, IEEE FP64 in its order of operations, and
    correctly rounded divisions.  lambda = 2.5 and friction = 1.7 make the
    divisions inexact."""
    m = g.make_monolayer(96, 36, seed=14, types=[i % 2 for i in range(36)])
    params = dict(g.DRY_POLAR, interaction_type=model, **{"lambda": 2.5}, friction=1.7, omega=0.004,
                  zetaQ_self=0.1, zetaQ_inter=0.05, J_Q=0.2)
    keys, m2 = case_from_monolayer(m, params, seed=15)
    p, cells = build_inputs(keys, m2)
    a = engine.Engine(p, m2.L, cells).state()
    p, cells = build_inputs(keys, m2)
    b = orc.OracleSim(p, m2.L, cells).state()
    for k in ("mu", "vx", "vy", "box_index", "area", "sum_f"):
        assert np.array_equal(a[k], b[k]), (k, rel_err(a[k], b[k]))


WALL_BOXES = [dict(type="square_walls", lambda_wall=6), dict(type="circle_walls", lambda_wall=4),
              dict(type="triangle_walls", lambda_wall=5)]


@pytest.mark.parametrize("box", range(len(WALL_BOXES)))
@pytest.mark.parametrize("model", ["wetpolarmodel", "simplefield", "wetmodel"])
def test_walls_vs_oracle(model, box):
    """Wall boxes on 41x41 patches over 20 steps (the oracle itself is bit
    for bit the reference's exact build on the wall goldens)."""
    m = g.make_monolayer(96, 16, seed=5)
    params = dict(g.DRY_POLAR, interaction_type=model, zetaQ_inter=0.05, J_Q=0.2, omega=0.004, beta=0.2,
                  friction_cell=0, **WALL_BOXES[box])
    keys, m2 = case_from_monolayer(m, params, seed=5)
    _, a = run(engine.Engine, keys, m2, [1, 20])
    _, b = run(orc.OracleSim, keys, m2, [1, 20])
    for s_ in (1, 20):
        assert np.array_equal(a[s_]["box_index"], b[s_]["box_index"])
        for k in ("phi", "vx", "vy", "area", "com_x", "com_y", "dx", "dy", "mu"):
            err = rel_err(a[s_][k], b[s_][k])
            assert err <= TOL, (s_, k, err)
