"""CPU oracle of the learned preconditioner's network (test infrastructure).

A 3-level U-Net on the periodic box grid, channel-last float64 arrays of shape
(batch, L, L, C).  It is the checker for the device training kernels
(forward, loss, every gradient) and for the inference convolutions; nothing
in the engine calls it.  The network has no counterpart in the reference (its
viscous solve is Eigen's ConjugateGradient, WetModel.cpp:279-376); the
architecture is the project's own:

  e0a 2->16, e0b 16->16 = s0          (L)      input: [R/s, W]
  e1a 16->16, e1b 16->16 = s1         (L/2)    input: avgpool2(s0)
  b0 16->16, b1 16->16 = t2           (L/4)    input: avgpool2(s1)
  d1a 32->16, d1b 16->16 = t1         (L/2)    input: [upsample2(t2), s1]
  d0a 32->16, d0b 16->16              (L)      input: [upsample2(t1), s0]
  out 16->1 (no activation)           (L)

Every layer is a 3x3 convolution with periodic wrap and a bias, followed by
ReLU except `out`.  Weights w[tap, ci, co] with tap = (dy + 1) * 3 + (dx + 1)
and y[i, j] += x[(i + dy) mod L, (j + dx) mod L] w[tap].  The loss of a batch
is the mean over samples of |f(x) - y|^2 / |y|^2.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

# (name, c_in, c_out, relu)
LAYERS: List[Tuple[str, int, int, bool]] = [
    ("e0a", 2, 16, True), ("e0b", 16, 16, True),
    ("e1a", 16, 16, True), ("e1b", 16, 16, True),
    ("b0", 16, 16, True), ("b1", 16, 16, True),
    ("d1a", 32, 16, True), ("d1b", 16, 16, True),
    ("d0a", 32, 16, True), ("d0b", 16, 16, True),
    ("out", 16, 1, False),
]


def param_layout() -> List[Tuple[str, int, int, int, int]]:
    """(name, c_in, c_out, weight offset, bias offset) in the flat parameter
    vector: per layer 9*c_in*c_out weights then c_out biases."""
    out, off = [], 0
    for name, ci, co, _ in LAYERS:
        out.append((name, ci, co, off, off + 9 * ci * co))
        off += 9 * ci * co + co
    return out


def n_params() -> int:
    name, ci, co, w, b = param_layout()[-1]
    return b + co


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation (normal, std sqrt(2 / (9 c_in))), zero biases."""
    rng = np.random.default_rng(seed)
    p = np.zeros(n_params())
    for name, ci, co, w, b in param_layout():
        p[w:w + 9 * ci * co] = rng.normal(0.0, np.sqrt(2.0 / (9 * ci)), size=9 * ci * co)
    return p


def unpack(p: np.ndarray) -> Dict[str, Tuple[np.ndarray, np.ndarray]]:
    d = {}
    for name, ci, co, w, b in param_layout():
        d[name] = (p[w:w + 9 * ci * co].reshape(9, ci, co), p[b:b + co])
    return d


TAPS = [(dy, dx) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def conv(x: np.ndarray, w: np.ndarray, b: np.ndarray) -> np.ndarray:
    y = np.zeros(x.shape[:3] + (w.shape[2],))
    for t, (dy, dx) in enumerate(TAPS):
        xs = np.roll(x, shift=(-dy, -dx), axis=(1, 2))  # xs[i, j] = x[i + dy, j + dx]
        y += xs @ w[t]
    return y + b


def conv_back(x: np.ndarray, w: np.ndarray, gy: np.ndarray):
    gx = np.zeros_like(x)
    gw = np.zeros_like(w)
    for t, (dy, dx) in enumerate(TAPS):
        xs = np.roll(x, shift=(-dy, -dx), axis=(1, 2))
        gw[t] = np.einsum("nijc,nijd->cd", xs, gy)
        gx += np.roll(gy @ w[t].T, shift=(dy, dx), axis=(1, 2))
    gb = gy.sum(axis=(0, 1, 2))
    return gx, gw, gb


def pool(x):
    n, L, _, c = x.shape
    return x.reshape(n, L // 2, 2, L // 2, 2, c).mean(axis=(2, 4))


def pool_back(g):
    return np.repeat(np.repeat(g, 2, axis=1), 2, axis=2) / 4.0


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_back(g):
    n, L, _, c = g.shape
    return g.reshape(n, L // 2, 2, L // 2, 2, c).sum(axis=(2, 4))


def forward(p: np.ndarray, x: np.ndarray, keep: bool = False):
    """x: (n, L, L, 2).  Returns the output (n, L, L, 1) [and the cache]."""
    P = unpack(p)
    cache = {}

    def layer(name, inp, relu):
        w, b = P[name]
        z = conv(inp, w, b)
        a = np.maximum(z, 0.0) if relu else z
        cache[name] = (inp, a)
        return a

    s0 = layer("e0b", layer("e0a", x, True), True)
    s1 = layer("e1b", layer("e1a", pool(s0), True), True)
    t2 = layer("b1", layer("b0", pool(s1), True), True)
    t1 = layer("d1b", layer("d1a", np.concatenate([up(t2), s1], axis=3), True), True)
    t0 = layer("d0b", layer("d0a", np.concatenate([up(t1), s0], axis=3), True), True)
    y = layer("out", t0, False)
    return (y, cache) if keep else y


def loss_and_grad(p: np.ndarray, x: np.ndarray, target: np.ndarray):
    """Mean over samples of |f - y|^2 / |y|^2, and its gradient w.r.t. p."""
    y, cache = forward(p, x, keep=True)
    n = x.shape[0]
    den = np.maximum((target ** 2).sum(axis=(1, 2, 3)), 1e-300)
    diff = y - target
    loss = float(np.mean((diff ** 2).sum(axis=(1, 2, 3)) / den))
    g = 2.0 * diff / (n * den[:, None, None, None])
    P = unpack(p)
    grads = {}

    def back(name, gout, relu):
        inp, a = cache[name]
        if relu:
            gout = gout * (a > 0)
        w, _ = P[name]
        gx, gw, gb = conv_back(inp, w, gout)
        grads[name] = (gw, gb)
        return gx

    g = back("out", g, False)
    g = back("d0a", back("d0b", g, True), True)
    g_up1, g_s0 = g[..., :16], g[..., 16:]
    g = back("d1a", back("d1b", up_back(g_up1), True), True)
    g_up2, g_s1 = g[..., :16], g[..., 16:]
    g = back("b0", back("b1", up_back(g_up2), True), True)
    g_s1 = g_s1 + pool_back(g)
    g = back("e1a", back("e1b", g_s1, True), True)
    g_s0 = g_s0 + pool_back(g)
    back("e0a", back("e0b", g_s0, True), True)
    flat = np.zeros_like(p)
    for name, ci, co, w, b in param_layout():
        gw, gb = grads[name]
        flat[w:w + 9 * ci * co] = gw.ravel()
        flat[b:b + co] = gb
    return loss, flat


def adam(p, g, m, v, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (t counts from 1); returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
