"""FP32 site arithmetic for the dry polar model (RC_PRECISION_FLOAT): close
to the FP64 engine over short runs, and the same ensemble statistics (mean
cell speed, area, shape-tensor magnitude) within 1% over longer runs."""
from __future__ import annotations

import numpy as np
import pytest

from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer, rel_err

pytestmark = pytest.mark.gpu


def _engine(keys, m, precision):
    p, cells = build_inputs(keys, m, precision=precision)
    e = engine.Engine(p, m.L, cells)
    e.set_phase(1)
    return e


def _case(L=140, n=100, seed=1, **extra):
    m = g.make_monolayer(L, n, seed=seed)
    return case_from_monolayer(m, dict(g.DRY_POLAR, **extra), seed=seed)


def test_float_close_to_double_short_run():
    keys, m = _case()
    a = _engine(keys, m, abi.RC_PRECISION_DOUBLE)
    b = _engine(keys, m, abi.RC_PRECISION_FLOAT)
    a.step(20)
    b.step(20)
    sa, sb = a.state(), b.state()
    assert rel_err(sb["phi"], sa["phi"]) < 1e-4
    assert rel_err(sb["area"], sa["area"]) < 1e-5
    assert rel_err(sb["com_x"], sa["com_x"]) < 1e-5
    assert np.array_equal(sb["lsub_x"], sa["lsub_x"])


def _stats(e, L, steps, every):
    """Mean cell speed (unwrapped centre-of-mass displacement per unit time),
    mean area and mean shape-tensor magnitude, sampled every `every` steps."""
    dt = 0.1
    st = e.state()
    pos = np.stack([st["unrap_x"] + st["com_x"] - (st["corner"] % L),
                    st["unrap_y"] + st["com_y"] - (st["corner"] // L)], axis=1)
    speeds, areas, shapes = [], [], []
    for _ in range(steps // every):
        e.step(every)
        st = e.state()
        p2 = np.stack([st["unrap_x"] + st["com_x"] - (st["corner"] % L),
                       st["unrap_y"] + st["com_y"] - (st["corner"] // L)], axis=1)
        speeds.append(np.mean(np.linalg.norm(p2 - pos, axis=1)) / (every * dt))
        pos = p2
        areas.append(np.mean(st["area"]))
        shapes.append(np.mean(np.hypot(st["s00"], st["s01"])))
    return np.mean(speeds), np.mean(areas), np.mean(shapes)


def test_float_ensemble_statistics_within_one_percent():
    keys, m = _case(seed=3)
    a = _engine(keys, m, abi.RC_PRECISION_DOUBLE)
    b = _engine(keys, m, abi.RC_PRECISION_FLOAT)
    a.step(100)
    b.step(100)
    sa = _stats(a, m.L, 400, 20)
    sb = _stats(b, m.L, 400, 20)
    for x, y, name in zip(sa, sb, ("speed", "area", "shape")):
        assert abs(x - y) <= 0.01 * abs(x), (name, x, y)
