"""Device training kernels of the learned preconditioner's network against
the CPU oracle (oracle/unet.py): forward output, loss and the gradient of
every layer, through the C ABI (rc_unet_loss_grad)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import unet as U
from rheocell_gb300 import abi, engine

pytestmark = pytest.mark.gpu


def _dp(a):
    return a.ctypes.data_as(abi.DP)


@pytest.mark.parametrize("L,batch", [(16, 2), (32, 3)])
def test_forward_loss_and_gradients_match_oracle(L, batch):
    lib = engine.lib()
    rng = np.random.default_rng(L)
    p = U.init_params(L)
    for name, ci, co, w, b in U.param_layout():
        p[b:b + co] = rng.normal(0.0, 0.05, size=co)
    x = np.ascontiguousarray(rng.normal(size=(batch, L, L, 2)))
    x[..., 1] = np.abs(x[..., 1]) * 0.25  # the coefficient channel is non-negative
    t = np.ascontiguousarray(rng.normal(size=(batch, L, L, 1)))
    loss = np.zeros(1)
    grad = np.zeros(U.n_params())
    out = np.zeros((batch, L, L))
    rc = lib.rc_unet_loss_grad(L, batch, _dp(p), _dp(x), _dp(t), _dp(loss), _dp(grad), _dp(out), 0)
    assert rc == 0
    y = U.forward(p, x)[..., 0]
    l_ref, g_ref = U.loss_and_grad(p, x, t)
    # FP32 device arithmetic against the FP64 oracle
    assert np.max(np.abs(out - y)) <= 1e-4 * np.max(np.abs(y))
    assert abs(loss[0] - l_ref) <= 1e-4 * abs(l_ref)
    for name, ci, co, w, b in U.param_layout():
        gw, gw_ref = grad[w:b + co], g_ref[w:b + co]
        assert np.max(np.abs(gw - gw_ref)) <= 1e-3 * np.max(np.abs(gw_ref)), name


@pytest.mark.parametrize("L,batch", [(16, 2), (64, 2), (128, 1), (256, 2), (384, 1), (512, 2), (1024, 1)])
def test_tensor_core_forward_matches_oracle(L, batch):
    """The solve's forward pass (BF16 activations, tcgen05 layers) against the
    FP64 oracle, within BF16 rounding over eleven layers.  Sides that are
    multiples of 128 take the strip path (one to four tiles per strip, one or
    more strips per row); the others, and the coarse levels below 128, the
    gathered path."""
    lib = engine.lib()
    rng = np.random.default_rng(100 + L)
    p = U.init_params(L + 1)
    for name, ci, co, w, b in U.param_layout():
        p[b:b + co] = rng.normal(0.0, 0.05, size=co)
    x = np.ascontiguousarray(rng.normal(size=(batch, L, L, 2)))
    x[..., 1] = np.abs(x[..., 1]) * 0.25
    out = np.zeros((batch, L, L))
    rc = lib.rc_unet_forward_tc(L, batch, _dp(p), _dp(x), _dp(out), 0)
    assert rc == 0
    y = U.forward(p, x)[..., 0]
    err = np.max(np.abs(out - y)) / np.max(np.abs(y))
    assert err < 3e-2, err
