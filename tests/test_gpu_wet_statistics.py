"""Ensemble statistics of long wet runs: the mixed-precision solve, the
learned solve and FP32 site arithmetic (with either solve) against the plain
FP64 path.

Active wet monolayers are chaotic, so trajectories from the same start
separate once rounding differences grow; the runs are compared by their
statistics instead -- mean cell speed (unwrapped centre-of-mass
displacement per unit time), the area distribution (mean and standard
deviation over cells) and the shape index (mean elongation |S| and mean
aspect ratio of the cells' shape tensors, rc_observe_cells) -- time-averaged
over 2000 steps of the 256^2 / 400-cell wetmodel monolayer, and over 1000
steps of the 1024^2 / 6400-cell one, after 100 steps of transient, each
within 1% of the plain FP64 run's."""
from __future__ import annotations

import numpy as np
import pytest

from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer

pytestmark = pytest.mark.gpu

STEPS, EVERY, WARM = 2000, 50, 100


def _engine(keys, m, precision=abi.RC_PRECISION_DOUBLE):
    p, cells = build_inputs(keys, m, precision=precision)
    e = engine.Engine(p, m.L, cells)
    e.set_phase(1)
    return e


def _positions(st, L):
    return np.stack([st["unrap_x"] + st["com_x"] - (st["corner"] % L),
                     st["unrap_y"] + st["com_y"] - (st["corner"] // L)], axis=1)


def statistics(e, L, steps=STEPS, every=EVERY, dt=0.1):
    """Time averages over `steps` steps sampled every `every` steps."""
    cell_obs = np.zeros(6 * e.n)
    layer_obs = np.zeros(4)
    pos = _positions(e.state(abi.RC_FIELD_SCALARS), L)
    speed, area_mean, area_std, elong, aspect = [], [], [], [], []
    for _ in range(steps // every):
        e.step(every)
        st = e.state(abi.RC_FIELD_SCALARS)
        p2 = _positions(st, L)
        speed.append(np.mean(np.linalg.norm(p2 - pos, axis=1)) / (every * dt))
        pos = p2
        area_mean.append(np.mean(st["area"]))
        area_std.append(np.std(st["area"]))
        assert e._lib.rc_observe_cells(e.h, cell_obs.ctypes.data_as(abi.DP), layer_obs.ctypes.data_as(abi.DP)) == 0
        c = cell_obs.reshape(-1, 6)
        elong.append(np.mean(c[:, 3]))
        aspect.append(np.mean(c[:, 4]))
    return {"speed": np.mean(speed), "area_mean": np.mean(area_mean), "area_std": np.mean(area_std),
            "elongation": np.mean(elong), "aspect": np.mean(aspect)}


@pytest.fixture(scope="module")
def wet256():
    m = g.make_monolayer(256, 400, seed=1)
    keys, m2 = case_from_monolayer(m, g.WET_NEMATIC, seed=1)
    ref = _engine(keys, m2)
    ref.harvest(capacity=2000, every=3, per_solve=6)
    ref.step(WARM)
    ref.harvest(2000, 3, 0)
    ref.train(epochs=15, batch=8, learning_rate=2e-3, learning_rate_final=1e-4, seed=1)
    params = ref.get_params()
    ref.harvest(0, 0, 0)
    base = statistics(ref, m2.L)
    ref.close()
    return keys, m2, params, base


def _check(got, base):
    print("statistics", {k: (round(base[k], 6), round(got[k], 6)) for k in base})
    bad = {k: (base[k], got[k]) for k in base if abs(got[k] - base[k]) > 0.01 * abs(base[k])}
    assert not bad, bad


def test_mixed_precision_statistics_within_one_percent(wet256):
    keys, m, _, base = wet256
    e = _engine(keys, m, abi.RC_PRECISION_MIXED)
    e.step(WARM)
    _check(statistics(e, m.L), base)


@pytest.mark.parametrize("solver", [abi.RC_SOLVER_LEARNED])
def test_learned_solver_statistics_within_one_percent(wet256, solver):
    keys, m, params, base = wet256
    e = _engine(keys, m)
    e.step(WARM)
    e.set_params(params)
    e.set_solver(solver)
    got = statistics(e, m.L)
    assert e.stats.cg_max_rel_residual < 1e-8
    _check(got, base)


@pytest.mark.parametrize("solver", [abi.RC_SOLVER_PLAIN, abi.RC_SOLVER_LEARNED])
def test_fp32_fields_statistics_within_one_percent(wet256, solver):
    """FP32 site arithmetic (RC_PRECISION_FLOAT) with the mixed-precision
    solve, plain (Jacobi inner iterations) or learned."""
    keys, m, params, base = wet256
    e = _engine(keys, m, abi.RC_PRECISION_FLOAT)
    e.step(WARM)
    if solver != abi.RC_SOLVER_PLAIN:
        e.set_params(params)
        e.set_solver(solver)
    got = statistics(e, m.L)
    assert e.stats.cg_max_rel_residual < 1e-8
    _check(got, base)


def test_learned_fp32_statistics_at_1024_within_one_percent():
    """The benchmark spec's configuration, judged the same way: the wet 1024^2 /
    6400-cell monolayer (the bench's default line) with FP32 site arithmetic
    and the learned solve (the network the bench trains at 256^2, committed
    as tests/golden/unet_wet256.npy) against the plain FP64 run from the same
    start, statistics over 1000 steps after 100 of transient."""
    import os
    import bench
    params = np.load(os.path.join(os.path.dirname(__file__), "golden", "unet_wet256.npy")).astype(np.float64)
    w = bench.workload("wet1024")
    (keys, m), = bench.make_case(w)
    ref = bench.make_engine("wet1024", abi.RC_PRECISION_DOUBLE, 0)
    ref.set_solver(abi.RC_SOLVER_PLAIN_FP64)
    ref.step(WARM)
    base = statistics(ref, m.L, steps=1000)
    ref.close()
    e = bench.make_engine("wet1024", abi.RC_PRECISION_FLOAT, 0)
    e.set_params(params)
    e.set_solver(abi.RC_SOLVER_LEARNED)
    e.step(WARM)
    got = statistics(e, m.L, steps=1000)
    assert e.stats.cg_max_rel_residual < 1e-8
    e.close()
    _check(got, base)
