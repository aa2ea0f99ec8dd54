"""Diagnostic observables on the device (rc_observe_field, rc_observe_cells)
against a numpy restatement of the reference's observable loops
(VelocityField/ShapeField/NematicField::calc_field and the coarse-graining,
src/Observables/VelocityField.cpp:69-121; shape statistics of
scripts/calcAvgShape.py:274-336) applied to the engine's downloaded state."""
from __future__ import annotations

import numpy as np
import pytest

from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer, rel_err

pytestmark = pytest.mark.gpu


def _dp(a):
    return a.ctypes.data_as(abi.DP)


def _engine(L=96, n=36, seed=41, model="wetpolarmodel", **extra):
    m = g.make_monolayer(L, n, seed=seed, types=[i % 2 for i in range(n)])
    keys, m2 = case_from_monolayer(m, dict(g.DRY_POLAR, interaction_type=model, zetaQ_inter=0.1, J_Q=0.3,
                                          omega=0.004, **extra), seed=seed + 1)
    p, cells = build_inputs(keys, m2)
    e = engine.Engine(p, m2.L, cells)
    e.set_phase(1)
    return e, m2


def _ref_fields(st, L, kind, only_type, sg):
    """The reference's accumulation: cells in index order, f[k] += g * phi."""
    lx, ly = st["lsub_x"], st["lsub_y"]
    sizes = lx * ly
    f0 = np.zeros(L * L)
    f1 = np.zeros(L * L)
    s0 = 0
    types = st["type"]
    for i, ns in enumerate(sizes):
        sl = slice(s0, s0 + int(ns))
        s0 += int(ns)
        if only_type >= 0 and types[i] != only_type:
            continue
        k = st["box_index"][sl]
        phi = st["phi"][sl]
        if kind == abi.RC_OBS_VELOCITY:
            g0, g1 = st["vx"][sl], st["vy"][sl]
        elif kind == abi.RC_OBS_SHAPE:
            g0, g1 = st["s00"][i], st["s01"][i]
        else:
            g0, g1 = st["q00"][i], st["q01"][i]
        f0[k] += g0 * phi
        f1[k] += g1 * phi
    c0 = np.zeros(L * L)
    c1 = np.zeros(L * L)
    if sg > 0:
        ii, jj = np.divmod(np.arange(L * L), L)
        for kk in range(sg):
            for ll in range(sg):
                xx = (((jj - sg // 2 + L) % L) + ll) % L
                yy = (((ii - sg // 2 + L) % L) + kk) % L
                c0 += f0[xx + yy * L] / (sg * sg)
                c1 += f1[xx + yy * L] / (sg * sg)
    return f0, f1, c0, c1


@pytest.mark.parametrize("kind", [abi.RC_OBS_VELOCITY, abi.RC_OBS_SHAPE, abi.RC_OBS_NEMATIC])
@pytest.mark.parametrize("only_type", [-1, 1])
def test_fields_match_reference_loops(kind, only_type):
    e, m = _engine()
    e.step(7)
    L, sg = m.L, 3
    out = [np.zeros(L * L) for _ in range(4)]
    rc = e._lib.rc_observe_field(e.h, kind, 0, only_type, sg, *[_dp(o) for o in out])
    assert rc == 0, e._lib.rc_last_error(e.h).decode()
    st = e.state()
    ref = _ref_fields(st, L, kind, only_type, sg)
    for got, want in zip(out, ref):
        assert np.array_equal(got, want)
    assert np.any(out[0] != 0.0)


def test_wet_velocity_field():
    e, m = _engine(L=64, n=9, seed=43, model="wetmodel", friction_cell=1)
    e.step(3)
    L = m.L
    out = [np.zeros(L * L) for _ in range(4)]
    assert e._lib.rc_observe_field(e.h, abi.RC_OBS_VELOCITY, 0, -1, 0, *[_dp(o) for o in out]) == 0
    ref = _ref_fields(e.state(), L, abi.RC_OBS_VELOCITY, -1, 0)
    assert np.array_equal(out[0], ref[0]) and np.array_equal(out[1], ref[1])


def test_cell_statistics():
    e, m = _engine()
    e.step(5)
    n = e.n
    co = np.zeros(6 * n)
    lo = np.zeros(4)
    assert e._lib.rc_observe_cells(e.h, _dp(co), _dp(lo)) == 0
    co = co.reshape(n, 6)
    st = e.state()
    L = m.L
    sizes = st["lsub_x"] * st["lsub_y"]
    s0 = 0
    for i, ns in enumerate(sizes):
        dx, dy = st["dx"][s0:s0 + ns], st["dy"][s0:s0 + ns]
        s0 += ns
        a, b, c = np.sum(dx * dx), np.sum(dy * dy), np.sum(dx * dy)
        s00, s01 = -0.5 * (a - b), -c
        D = np.hypot(s00, s01)
        sv = np.linalg.svd(np.array([[a, c], [c, b]]), compute_uv=False)
        ox = (st["com_x"][i] - st["corner"][i] % L) % L
        oy = (st["com_y"][i] - st["corner"][i] // L) % L
        want = [st["unrap_x"][i] + ox, st["unrap_y"][i] + oy, st["area"][i], D, np.sqrt(sv[0] / sv[1]) - 1,
                0.5 * np.arctan2(s01, s00)]
        for j in range(6):
            assert abs(co[i, j] - want[j]) <= 1e-10 * max(1.0, abs(want[j])), (i, j, co[i, j], want[j])
    assert abs(lo[0] - co[:, 2].mean()) <= 1e-12 * lo[0]
    assert abs(lo[1] - co[:, 2].var()) <= 1e-9 * max(lo[1], 1.0)
    assert abs(lo[2] - co[:, 3].mean()) <= 1e-12 * lo[2]
    assert abs(lo[3] - co[:, 4].mean()) <= 1e-12 * lo[3]


def test_batch_member_fields_equal_single():
    members = [(96, 36, 51), (80, 25, 52)]
    singles, layers = [], []
    for L, n, seed in members:
        mm = g.make_monolayer(L, n, seed=seed)
        keys, m2 = case_from_monolayer(mm, dict(g.DRY_POLAR, zetaQ_inter=0.1, J_Q=0.3), seed=seed + 1)
        p, cells = build_inputs(keys, m2)
        singles.append((p, m2, cells))
        layers.append((m2.L, cells, p.rng_state))
    b = engine.Engine.batch(singles[0][0], layers)
    b.set_phase(1)
    b.step(4)
    for li, (p, m2, cells) in enumerate(singles):
        s = engine.Engine(p, m2.L, cells)
        s.set_phase(1)
        s.step(4)
        L = m2.L
        ob = [np.zeros(L * L) for _ in range(4)]
        os_ = [np.zeros(L * L) for _ in range(4)]
        assert b._lib.rc_observe_field(b.h, abi.RC_OBS_VELOCITY, li, -1, 2, *[_dp(o) for o in ob]) == 0
        assert s._lib.rc_observe_field(s.h, abi.RC_OBS_VELOCITY, 0, -1, 2, *[_dp(o) for o in os_]) == 0
        for x, y in zip(ob, os_):
            assert np.array_equal(x, y)
