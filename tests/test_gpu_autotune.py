"""Tile-shape autotuning of the FP32 cell kernel (rc_autotune,
rc_set_cell_threads): every tile gives the FP32 results (close to the FP64
engine), with the fused and the split per-cell epilogue; the autotuner times
all candidates and keeps the fastest; FP64 engines keep their single tile."""
from __future__ import annotations

import numpy as np
import pytest

from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer, rel_err

pytestmark = pytest.mark.gpu

TILES = (128, 256, 512)


def _engine(keys, m, precision, threads=None):
    p, cells = build_inputs(keys, m, precision=precision)
    e = engine.Engine(p, m.L, cells)
    e.set_phase(1)
    if threads:
        e.set_cell_threads(threads)
    return e


def _case(L, n, seed=1):
    m = g.make_monolayer(L, n, seed=seed)
    return case_from_monolayer(m, dict(g.DRY_POLAR), seed=seed)


@pytest.mark.parametrize("L,n", [(140, 100), (256, 400)])  # fused epilogue; split epilogue (>= 256 cells)
def test_every_tile_close_to_double(L, n):
    keys, m = _case(L, n)
    ref = _engine(keys, m, abi.RC_PRECISION_DOUBLE)
    ref.step(20)
    sa = ref.state()
    for t in TILES:
        e = _engine(keys, m, abi.RC_PRECISION_FLOAT, threads=t)
        e.step(20)
        sb = e.state()
        assert rel_err(sb["phi"], sa["phi"]) < 1e-4, t
        assert rel_err(sb["area"], sa["area"]) < 1e-5, t
        assert rel_err(sb["com_x"], sa["com_x"]) < 1e-5, t
        assert np.array_equal(sb["lsub_x"], sa["lsub_x"]), t
        e.close()


def test_autotune_keeps_the_fastest_tile():
    keys, m = _case(140, 100)
    e = _engine(keys, m, abi.RC_PRECISION_FLOAT)
    rep = e.autotune(steps_per_candidate=3)
    threads = [t for t, _ in rep["candidates"]]
    times = [ms for _, ms in rep["candidates"]]
    assert sorted(threads) == list(TILES)
    assert all(ms > 0 for ms in times)
    assert rep["chosen"] == threads[int(np.argmin(times))]
    e.step(5)  # the engine keeps stepping with the chosen tile
    assert np.all(np.isfinite(e.state()["phi"]))


def test_double_engine_has_nothing_to_tune():
    keys, m = _case(140, 100)
    e = _engine(keys, m, abi.RC_PRECISION_DOUBLE)
    rep = e.autotune(steps_per_candidate=2)
    assert rep["candidates"] == [] and rep["chosen"] == 256


def test_invalid_tile_is_rejected():
    keys, m = _case(140, 100)
    e = _engine(keys, m, abi.RC_PRECISION_FLOAT)
    with pytest.raises(engine.EngineError):
        e.set_cell_threads(200)
