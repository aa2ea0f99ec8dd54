"""The CPU oracle of the learned preconditioner's network: its analytic
gradient against central finite differences, and its layout against the C
header's parameter count."""
from __future__ import annotations

import numpy as np

from oracle import unet as U
from rheocell_gb300 import abi


def test_parameter_count_matches_header():
    assert U.n_params() == abi.RC_UNET_PARAMS


def test_gradient_matches_finite_differences():
    p = U.init_params(1)
    p[U.param_layout()[0][4]:U.param_layout()[0][4] + 16] = 0.05  # nonzero biases
    rng = np.random.default_rng(2)
    x = rng.normal(size=(2, 8, 8, 2))
    t = rng.normal(size=(2, 8, 8, 1))
    _, g = U.loss_and_grad(p, x, t)
    h = 1e-6
    for i in rng.choice(len(p), 40, replace=False):
        pp = p.copy()
        pp[i] += h
        pm = p.copy()
        pm[i] -= h
        fd = (U.loss_and_grad(pp, x, t)[0] - U.loss_and_grad(pm, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_periodic_shift_equivariance():
    """Convolutions wrap around the box: shifting the input shifts the output."""
    p = U.init_params(3)
    x = np.random.default_rng(4).normal(size=(1, 16, 16, 2))
    y = U.forward(p, x)
    ys = U.forward(p, np.roll(x, (4, 8), axis=(1, 2)))  # shifts by multiples of 4 commute with pooling
    assert np.allclose(np.roll(y, (4, 8), axis=(1, 2)), ys, rtol=1e-12, atol=1e-12)
