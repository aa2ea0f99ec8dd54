"""The C ABI rejects invalid input with the documented status and message
before it makes any CUDA call, and every entry point taking an engine handle
returns RC_ERR_INVALID for a NULL handle.  No case here reaches the device, so
the file runs without a GPU; the conventions follow the reference's, where a
bad configuration is an RCexception caught in main (src/rheoCell.cpp:40-43)
and reported, not a crash."""
from __future__ import annotations

import ctypes as C

import pytest

from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer


@pytest.fixture(scope="module")
def lib():
    return engine.lib()


def _inputs(params=g.WET_NEMATIC, L=64, n=9, seed=5):
    m = g.make_monolayer(L, n, seed=seed)
    keys, m2 = case_from_monolayer(m, params, seed=seed)
    p, cells = build_inputs(keys, m2)
    return p, m2.L, cells


def _create(lib, p, L, cells, n=None, Ly=None):
    h = C.c_void_p()
    box = abi.RcBox(L, L if Ly is None else Ly)
    rc = lib.rc_create(C.byref(p), C.byref(box), cells.n if n is None else n, cells.arr, 0, C.byref(h))
    # every rejection below happens before an engine exists
    assert not h
    return rc, lib.rc_last_error(None).decode()


def test_create_rejects_bad_parameters(lib):
    p, L, cells = _inputs()
    rc = lib.rc_create(C.byref(p), C.byref(abi.RcBox(L, L)), cells.n, cells.arr, 0, None)
    assert rc == abi.RC_ERR_INVALID and "out is NULL" in lib.rc_last_error(None).decode()

    bad = abi.RcParams.from_buffer_copy(p)
    bad.model = 7
    assert _create(lib, bad, L, cells) == (abi.RC_ERR_INVALID, "unknown interaction model 7")

    bad = abi.RcParams.from_buffer_copy(p)
    bad.precision = 9
    assert _create(lib, bad, L, cells) == (abi.RC_ERR_INVALID, "unknown precision 9")

    bad = abi.RcParams.from_buffer_copy(p)
    bad.anchoring = 1
    assert _create(lib, bad, L, cells)[0] == abi.RC_ERR_UNSUPPORTED

    # FP32 site arithmetic exists for wetpolarmodel and wetmodel; not for activenematic
    bad = abi.RcParams.from_buffer_copy(p)
    bad.precision = abi.RC_PRECISION_FLOAT
    bad.model = abi.RC_ACTIVENEMATIC
    rc, msg = _create(lib, bad, L, cells)
    assert rc == abi.RC_ERR_UNSUPPORTED and "wetpolarmodel and wetmodel only" in msg


def test_create_rejects_walls_it_does_not_provide(lib):
    # walls with a viscous solve, and walls on FP32 engines: rejected before any CUDA call
    import numpy as np
    p, L, cells = _inputs()  # the wet nematic model with friction_cell = 1
    walls = np.zeros(L * L)
    walls[:L] = 1.0
    h = C.c_void_p()
    rc = lib.rc_create(C.byref(p), C.byref(abi.make_box(L, walls)), cells.n, cells.arr, 0, C.byref(h))
    assert rc == abi.RC_ERR_UNSUPPORTED and not h
    assert "walls with a viscous solve" in lib.rc_last_error(None).decode()
    dry = abi.RcParams.from_buffer_copy(p)
    dry.friction_cell = abi.D2(0.0, 0.0)
    dry.precision = abi.RC_PRECISION_FLOAT
    rc = lib.rc_create(C.byref(dry), C.byref(abi.make_box(L, walls)), cells.n, cells.arr, 0, C.byref(h))
    assert rc == abi.RC_ERR_UNSUPPORTED and "FP64 cell kernels only" in lib.rc_last_error(None).decode()


def test_create_rejects_bad_box_and_cells(lib):
    p, L, cells = _inputs()
    rc, msg = _create(lib, p, L, cells, Ly=L + 1)
    assert rc == abi.RC_ERR_INVALID and "not a square" in msg
    rc, msg = _create(lib, p, L, cells, n=-1)
    assert rc == abi.RC_ERR_INVALID and "negative cell count" in msg

    h = C.c_void_p()
    rc = lib.rc_create(C.byref(p), C.byref(abi.RcBox(L, L)), 3, None, 0, C.byref(h))
    assert rc == abi.RC_ERR_INVALID and "cells is NULL" in lib.rc_last_error(None).decode()

    c0 = cells.arr[0]
    saved = (c0.lsub_x, c0.offset_x, c0.corner, c0.phi)
    try:
        c0.lsub_x = L + 1
        rc, msg = _create(lib, p, L, cells)
        assert rc == abi.RC_ERR_INVALID and "does not fit" in msg
        c0.lsub_x = saved[0]
        c0.offset_x = c0.lsub_x
        rc, msg = _create(lib, p, L, cells)
        assert rc == abi.RC_ERR_INVALID and "offset out of range" in msg
        c0.offset_x = saved[1]
        c0.corner = L * L
        rc, msg = _create(lib, p, L, cells)
        assert rc == abi.RC_ERR_INVALID and "corner out of box" in msg
        c0.corner = saved[2]
        c0.phi = None
        rc, msg = _create(lib, p, L, cells)
        assert rc == abi.RC_ERR_INVALID and "phi is NULL" in msg
    finally:
        c0.lsub_x, c0.offset_x, c0.corner, c0.phi = saved


def test_batches_of_wet_monolayers_with_walls_are_rejected(lib):
    import numpy as np
    p, L, cells = _inputs()
    walls = np.zeros(L * L)
    walls[:L] = 1.0
    boxes = (abi.RcBox * 2)(abi.make_box(L, walls), abi.RcBox(L, L))
    counts = (C.c_int * 2)(cells.n, 0)
    h = C.c_void_p()
    rc = lib.rc_batch_create(C.byref(p), 2, boxes, counts, cells.arr, None, 0, C.byref(h))
    assert rc == abi.RC_ERR_UNSUPPORTED and not h
    assert "walls with a viscous solve" in lib.rc_last_error(None).decode()


def test_null_handle_is_invalid(lib):
    null = None
    dp = C.cast(None, abi.DP)
    st = abi.RcStepStats()
    assert lib.rc_step(null, 1, C.byref(st)) == abi.RC_ERR_INVALID
    assert lib.rc_step_async(null, 1) == abi.RC_ERR_INVALID
    assert lib.rc_wait(null, None) == abi.RC_ERR_INVALID
    assert lib.rc_set_phase(null, 1) == abi.RC_ERR_INVALID
    assert lib.rc_download_phi(null, dp, 0) == abi.RC_ERR_INVALID
    assert lib.rc_upload_phi(null, dp, 0) == abi.RC_ERR_INVALID
    assert lib.rc_download(null, None, 0) == abi.RC_ERR_INVALID
    assert lib.rc_upload(null, None, 0) == abi.RC_ERR_INVALID
    assert lib.rc_get_sizes(null, None, None, None) == abi.RC_ERR_INVALID
    assert lib.rc_set_stream(null, None) == abi.RC_ERR_INVALID
    assert lib.rc_learned_harvest(null, 1, 1, 1) == abi.RC_ERR_INVALID
    assert lib.rc_set_solver(null, abi.RC_SOLVER_PLAIN) == abi.RC_ERR_INVALID
    assert lib.rc_viscous_resolve_noalloc(null, None, None, 0, None) == abi.RC_ERR_INVALID
    assert lib.rc_site_count(null) == 0
    assert lib.rc_layer_count(null) == 0
    lib.rc_destroy(null)  # a no-op
