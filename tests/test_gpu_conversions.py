"""The FP32 cell kernels convert between double and float on the integer
pipes (on GB300 the conversion instructions issue on the narrow FP64 pipe).
Both forms are checked here against CUDA's own round-to-nearest conversion
on the device (rc_selftest_conversions):

* d2f_int (exact form): equal to __double2float_rn wherever the result is an
  FP32 normal number; magnitudes below the FP32 normal range give a signed
  zero (the fields never need FP32 subnormals);
* d2f_fast (streaming form, the update kernel): equal to __double2float_rn
  except at exact ties, where it rounds away from zero instead of to even
  (one ulp apart), and beyond the FP32 range, where infinities and NaN give
  NaN;
* f2d_int widens exactly (the widened value equals the float)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from rheocell_gb300 import abi, engine

pytestmark = pytest.mark.gpu


def _inputs():
    rng = np.random.default_rng(5)
    parts = [
        rng.standard_normal(200000),                                # O(1) values of both signs
        rng.uniform(-1, 1, 100000) * 10.0 ** rng.uniform(-37, 37, 100000),  # the FP32 normal range
        np.array([0.0, -0.0, 1.0, -1.0, 0.5, 2.0 ** -126, -(2.0 ** -126), 3.4e38, -3.4e38]),
    ]
    # exact ties: a float plus half an ulp, with even and odd last bits
    f = rng.standard_normal(20000).astype(np.float32)
    ulp = np.spacing(np.abs(f)).astype(np.float64)
    parts.append(f.astype(np.float64) + 0.5 * ulp)
    parts.append(f.astype(np.float64) - 0.5 * ulp)
    # below the FP32 normal range, beyond its range, non-finite
    parts.append(np.array([1e-39, -1e-39, 1e-45, 1e-300, -1e-300, 1e39, -1e39, 1e300, np.inf, -np.inf, np.nan]))
    return np.ascontiguousarray(np.concatenate(parts))


def test_integer_pipe_conversions_against_cuda():
    lib = engine.lib()
    x = _inputs()
    n = x.size
    ex, fa, cu = (np.zeros(n, np.float32) for _ in range(3))
    wd = np.zeros(n)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    rc = lib.rc_selftest_conversions(x.ctypes.data_as(abi.DP), fp(ex), fp(fa), fp(cu), wd.ctypes.data_as(abi.DP), n, 0)
    assert rc == abi.RC_OK, lib.rc_last_error(None).decode()
    tiny = 2.0 ** -126
    normal = np.isfinite(x) & (np.abs(x) >= tiny) & (np.abs(cu) < np.inf) & (np.abs(cu) >= tiny)
    below = np.isfinite(x) & (np.abs(x) < tiny)
    # exact form
    assert np.array_equal(ex[normal].view(np.uint32), cu[normal].view(np.uint32))
    assert np.all(ex[below] == 0) and np.array_equal(np.signbit(ex[below]), np.signbit(x[below]))
    # streaming form: equal but at exact ties (one ulp, away from zero)
    same = fa[normal].view(np.uint32) == cu[normal].view(np.uint32)
    diff = ~same
    xf, cf, ff = x[normal][diff], cu[normal][diff], fa[normal][diff]
    assert np.all(np.abs(ff.astype(np.float64)) > np.abs(cf.astype(np.float64)))
    assert np.all(np.abs(ff.view(np.int32).astype(np.int64) - cf.view(np.int32).astype(np.int64)) == 1)
    assert np.all(np.abs(xf - cf.astype(np.float64)) == np.abs(xf - ff.astype(np.float64)))  # ties
    assert diff.sum() <= 40000
    assert np.all(fa[below] == 0)
    big = ~np.isfinite(x) | (np.abs(x) >= 2.0 ** 128)
    assert np.all(np.isnan(fa[big]))
    # widening is exact
    ok = np.isfinite(cu) & ((np.abs(cu) >= tiny) | (cu == 0))
    assert np.array_equal(wd[ok], cu[ok].astype(np.float64))
