"""Ensembles (rc_batch_create): independent monolayers of different sizes
advanced by the same launches must reproduce, bit for bit, the same
monolayers run one engine each, and one member must match the oracle --
dry members, and wet members whose viscous systems are solved member by
member (FP64 and mixed precision)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as orc
from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer, rel_err, run

pytestmark = pytest.mark.gpu

# uneven members: box side, cells, configuration seed
MEMBERS = [(96, 36, 21), (112, 49, 22), (80, 25, 23)]
PARAMS = dict(g.DRY_POLAR, zetaQ_inter=0.2, J_Q=0.5, omega=0.004)
STEPS = 12


def _member(L, n, seed):
    m = g.make_monolayer(L, n, seed=seed)
    keys, m2 = case_from_monolayer(m, PARAMS, seed=seed + 100)
    p, cells = build_inputs(keys, m2)
    return keys, m2, p, cells


def _batch():
    members = [_member(*mb) for mb in MEMBERS]
    p0 = members[0][2]
    layers = [(m2.L, cells, p.rng_state) for _, m2, p, cells in members]
    e = engine.Engine.batch(p0, layers)
    return members, e


def test_batch_matches_single_engines_bitwise():
    members, e = _batch()
    assert e.layer_count() == len(MEMBERS)
    e.set_phase(1)
    e.step(STEPS)
    parts = e.split(e.state())
    for (keys, m2, _, _), got in zip(members, parts):
        _, ref = run(engine.Engine, keys, m2, [STEPS])
        want = ref[STEPS]
        for k in ("phi", "vx", "vy", "mu", "box_index", "com_x", "com_y", "q00", "q01", "theta_q", "area",
                  "lsub_x", "corner", "force_rep_x"):
            assert np.array_equal(got[k], want[k]), k
    e.close()


def test_batch_member_vs_oracle():
    members, e = _batch()
    e.set_phase(1)
    e.step(STEPS)
    got = e.split(e.state())[1]
    keys, m2, _, _ = members[1]
    _, ref = run(orc.OracleSim, keys, m2, [STEPS])
    want = ref[STEPS]
    for k in ("phi", "vx", "vy", "mu", "com_x", "com_y", "theta_q", "area"):
        assert rel_err(got[k], want[k]) < 1e-10, k
    assert np.array_equal(got["box_index"], want["box_index"])
    e.close()


WET_MEMBERS = [(64, 9, 31), (80, 16, 32), (48, 4, 33)]
WET_PARAMS = dict(g.WET_NEMATIC, zetaQ_inter=0.02, omega=0.004)
WET_STEPS = 6


def _wet_batch(precision):
    members = []
    for L, n, seed in WET_MEMBERS:
        m = g.make_monolayer(L, n, seed=seed)
        keys, m2 = case_from_monolayer(m, WET_PARAMS, seed=seed + 100)
        p, cells = build_inputs(keys, m2, precision=precision)
        members.append((keys, m2, p, cells))
    layers = [(m2.L, cells, p.rng_state) for _, m2, p, cells in members]
    return members, engine.Engine.batch(members[0][2], layers)


@pytest.mark.parametrize("precision", [abi.RC_PRECISION_DOUBLE, abi.RC_PRECISION_MIXED])
def test_wet_batch_matches_single_engines_bitwise(precision):
    members, e = _wet_batch(precision)
    e.set_phase(1)
    e.step(WET_STEPS)
    assert e.stats.cg_solves > 0 and e.stats.cg_max_rel_residual < 1e-8
    parts = e.split(e.state())
    for (keys, m2, _, _), got in zip(members, parts):
        _, ref = run(engine.Engine, keys, m2, [WET_STEPS], precision=precision)
        want = ref[WET_STEPS]
        for k in ("phi", "vx", "vy", "mu", "box_index", "com_x", "com_y", "q00", "q01", "area", "lsub_x", "corner"):
            assert np.array_equal(got[k], want[k]), k
    e.close()


def test_wet_batch_member_vs_oracle():
    members, e = _wet_batch(abi.RC_PRECISION_DOUBLE)
    e.set_phase(1)
    e.step(WET_STEPS)
    got = e.split(e.state())[0]
    keys, m2, _, _ = members[0]
    _, ref = run(orc.OracleSim, keys, m2, [WET_STEPS])
    want = ref[WET_STEPS]
    for k in ("phi", "vx", "vy", "mu", "com_x", "com_y", "area"):
        assert rel_err(got[k], want[k]) < 1e-9, k
    e.close()


def test_learned_solver_not_provided_for_ensembles():
    members, e = _wet_batch(abi.RC_PRECISION_DOUBLE)
    with pytest.raises(engine.EngineError) as ei:
        e.set_solver(abi.RC_SOLVER_LEARNED)
    assert ei.value.code == abi.RC_ERR_UNSUPPORTED
    e.close()
