"""The box-grid reduction behind the learned preconditioner, checked on the
CPU with the operator of the wet models' viscous system.

The reference assembles, per velocity component, the SPD matrix over the
stacked patch sites (WetModel.cpp:279-347):

    (A v)_j = (xi + eta D_j) v_j - eta sum_{k' in N4(k_j)} sum_{i covers k'} v_i,
    D_j = sum_{k' in N4(k_j)} n(k'),

with k_j the box site of patch site j and n(k) the number of patches covering
box site k.  Every unknown at one box site k has the same diagonal T(k), so
A v = r reduces exactly to the box-grid system

    V - eta W (N4 V) = R,   R[k] = sum_{j at k} r_j / T(k),   W[k] = n(k) / T(k),

for the box sums V = S v, after which v_j = (r_j + eta (N4 V)[k_j]) / T(k_j).
The learned solve's network approximates R -> V; this file checks that the
reduction itself is exact, so the preconditioner's only error is the
network's."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as orc
from rheocell_gb300 import generator as g
from tests.common import case_from_monolayer, run

sp = pytest.importorskip("scipy.sparse")
spla = pytest.importorskip("scipy.sparse.linalg")


def _n4(F, L):
    G = F.reshape(L, L)
    return (np.roll(G, 1, 0) + np.roll(G, -1, 0) + np.roll(G, 1, 1) + np.roll(G, -1, 1)).ravel()


def _n4_matrix(L):
    idx = np.arange(L * L).reshape(L, L)
    rows, cols = [], []
    for sh, ax in ((1, 0), (-1, 0), (1, 1), (-1, 1)):
        rows.append(idx.ravel())
        cols.append(np.roll(idx, sh, ax).ravel())
    r, c = np.concatenate(rows), np.concatenate(cols)
    return sp.csr_matrix((np.ones(r.size), (r, c)), shape=(L * L, L * L))


@pytest.fixture(scope="module")
def system():
    m = g.make_monolayer(48, 9, seed=41, R=5, lam=1.5, patch=27)
    keys, m2 = case_from_monolayer(m, dict(g.WET_NEMATIC, R=5, **{"lambda": 1.5}), seed=42)
    sim, states = run(orc.OracleSim, keys, m2, [0])
    sim.close()
    k = np.asarray(states[0]["box_index"], dtype=np.int64)
    L = m2.L
    xi, eta = float(keys["friction"]), float(keys["friction_cell"])
    n = np.bincount(k, minlength=L * L).astype(float)
    T = xi + eta * _n4(n, L)

    def apply_a(v):
        return T[k] * v - eta * _n4(np.bincount(k, weights=v, minlength=L * L), L)[k]

    return dict(k=k, L=L, xi=xi, eta=eta, n=n, T=T, A=apply_a)


def test_operator_is_symmetric_positive_definite(system):
    rng = np.random.default_rng(1)
    A = system["A"]
    u, v = rng.normal(size=(2, system["k"].size))
    assert abs(u @ A(v) - v @ A(u)) <= 1e-12 * abs(u @ A(v))
    for _ in range(4):
        w = rng.normal(size=system["k"].size)
        assert w @ A(w) > 0


def test_box_reduction_solves_the_patch_system_exactly(system):
    k, L, eta, n, T, A = (system[x] for x in ("k", "L", "eta", "n", "T", "A"))
    rng = np.random.default_rng(2)
    r = rng.normal(size=k.size)
    R = np.bincount(k, weights=r / T[k], minlength=L * L)
    W = n / T
    M = sp.identity(L * L, format="csr") - eta * sp.diags(W) @ _n4_matrix(L)
    V = spla.spsolve(M.tocsc(), R)
    v = (r + eta * _n4(V, L)[k]) / T[k]
    assert np.max(np.abs(A(v) - r)) <= 1e-11 * np.max(np.abs(r))
    assert np.allclose(np.bincount(k, weights=v, minlength=L * L), V, rtol=0, atol=1e-11 * np.max(np.abs(V)))


def test_box_system_is_screened(system):
    """On a confluent monolayer the coupling eta W N4 of the box system has
    spectral radius below one: the system is a screened Poisson problem
    (Jacobi on it converges), whose inverse is short-ranged -- what a
    three-level network with 3x3 convolutions can represent."""
    L, eta, n, T = (system[x] for x in ("L", "eta", "n", "T"))
    W = n / T
    B = eta * sp.diags(W) @ _n4_matrix(L)
    rho = abs(spla.eigs(B, k=1, which="LM", return_eigenvectors=False)[0])
    assert rho < 1.0


def test_scaled_direction_cg_follows_jacobi_cg(system):
    """The plain FP64 device solve carries q = T p in place of the Jacobi-CG
    direction p (T is constant on a box site) and forms p.Ap from box sums:
    p.Ap = sum_k (1/T) sum q^2 - eta sum_k P(k) N4(P)(k) with P = S p, Ap =
    q - eta N4(P), x += (alpha / T) q, r.z = sum (1/T) r^2, q = r + beta q.
    Restated here next to Eigen's Jacobi-CG recurrence (the reference's
    solver, WetModel.cpp:361-376): the iterates agree to rounding."""
    k, L, eta, T, A = (system[x] for x in ("k", "L", "eta", "T", "A"))
    Tj = T[k]
    rng = np.random.default_rng(3)
    b = rng.normal(size=k.size)

    # Eigen's ConjugateGradient with the diagonal preconditioner, from x = 0
    x1 = np.zeros_like(b)
    r = b - A(x1)
    p = r / Tj
    rz = r @ p
    xs1 = []
    for _ in range(25):
        Ap = A(p)
        alpha = rz / (p @ Ap)
        x1 += alpha * p
        r -= alpha * Ap
        z = r / Tj
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        xs1.append(x1.copy())

    # the device's form: scaled direction, box sums, no Ap vector
    x2 = np.zeros_like(b)
    r = b.copy()
    q = np.zeros_like(b)
    rz = np.sum(r * r / Tj)
    beta = 0.0
    xs2 = []
    for it in range(25):
        q = r + beta * q if it else r.copy()                      # phase A
        P = np.bincount(k, weights=q, minlength=L * L) / T
        w = np.sum(q * q / Tj)
        G = P.reshape(L, L)                                       # phase B
        s = np.sum(G * (np.roll(G, -1, 0) + np.roll(G, -1, 1)))
        alpha = rz / (w - 2 * eta * s)
        Ap = q - eta * _n4(P, L)[k]                               # phase C
        x2 += (alpha / Tj) * q
        r -= alpha * Ap
        rz_new = np.sum(r * r / Tj)
        beta = rz_new / rz
        rz = rz_new
        xs2.append(x2.copy())

    for a, c in zip(xs1, xs2):
        assert np.max(np.abs(a - c)) <= 1e-12 * np.max(np.abs(a))
    # and it converges on this operator (a random right-hand side, from zero)
    assert np.linalg.norm(b - A(xs2[-1])) < 1e-4 * np.linalg.norm(b)


def _fcg(A, b, precond, iters):
    """Flexible CG (Notay's FCG(1)) as the learned solve's inner iterations
    run it: beta = -z.Ap_old / p_old.Ap_old, alpha = r.z / p.Ap."""
    x = np.zeros_like(b)
    r = b.copy()
    p = Ap = None
    xs, res = [], []
    for _ in range(iters):
        z = precond(r)
        rz = r @ z
        if p is None:
            p = z.copy()
        else:
            p = z + (-(z @ Ap) / pap) * p
        Ap = A(p)
        pap = p @ Ap
        alpha = rz / pap
        x += alpha * p
        r -= alpha * Ap
        xs.append(x.copy())
        res.append(np.linalg.norm(r) / np.linalg.norm(b))
    return xs, res


def test_flexible_cg_with_jacobi_is_jacobi_cg_and_exact_box_solve_converges_at_once(system):
    """With a fixed SPD preconditioner FCG(1) is preconditioned CG: with
    z = r / T its iterates are Jacobi CG's (the mixed-precision solve's inner
    iterations without a network).  With the exact box-grid solve as the
    preconditioner (what the network approximates) one iteration reaches
    rounding level."""
    k, L, eta, n, T, A = (system[x] for x in ("k", "L", "eta", "n", "T", "A"))
    Tj = T[k]
    b = np.random.default_rng(4).normal(size=k.size)

    xs_f, _ = _fcg(A, b, lambda r: r / Tj, 20)
    x = np.zeros_like(b)
    r = b.copy()
    p = r / Tj
    rz = r @ p
    for it in range(20):
        Ap = A(p)
        alpha = rz / (p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        z = r / Tj
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        assert np.max(np.abs(xs_f[it] - x)) <= 1e-9 * np.max(np.abs(x))

    M = (sp.identity(L * L, format="csr") - eta * sp.diags(n / T) @ _n4_matrix(L)).tocsc()
    lu = spla.splu(M)

    def box_solve(r):
        V = lu.solve(np.bincount(k, weights=r / Tj, minlength=L * L))
        return (r + eta * _n4(V, L)[k]) / Tj

    _, res = _fcg(A, b, box_solve, 1)
    assert res[0] < 1e-12


def test_fp32_inner_iterations_in_fp64_refinement_reach_the_fp64_tolerance(system):
    """The mixed-precision solve: FCG(1) in FP32 on the correction A e = r
    stopped at 1e-4 of |r|, then x += e and the true residual in FP64, until
    |r| < 1e-8 |b| (the reference's CGtolerance).  Restated in numpy with
    float32 inner arithmetic, it reaches the FP64 tolerance in a few sweeps
    although FP32 alone cannot resolve 1e-8."""
    k, L, eta, T, A = (system[x] for x in ("k", "L", "eta", "T", "A"))
    Tj = T[k]
    f32 = np.float32
    b = np.random.default_rng(5).normal(size=k.size)

    def a32(v):
        Tj32 = Tj.astype(f32)
        P = np.bincount(k, weights=v, minlength=L * L).astype(f32)
        return (Tj32 * v - f32(eta) * _n4(P, L)[k].astype(f32)).astype(f32)

    x = np.zeros_like(b)
    r = b - A(x)
    sweeps = 0
    while np.linalg.norm(r) >= 1e-8 * np.linalg.norm(b):
        sweeps += 1
        assert sweeps <= 6
        rf = r.astype(f32)
        goal = f32(1e-4) * np.linalg.norm(rf)
        e = np.zeros_like(rf)
        p = Ap = None
        for _ in range(500):
            z = (rf / Tj.astype(f32)).astype(f32)
            rz = rf @ z
            p = z.copy() if p is None else (z + (-(z @ Ap) / pap) * p).astype(f32)
            Ap = a32(p)
            pap = p @ Ap
            alpha = rz / pap
            e = (e + alpha * p).astype(f32)
            rf = (rf - alpha * Ap).astype(f32)
            if np.linalg.norm(rf) < goal:
                break
        x += e.astype(np.float64)
        r = b - A(x)
    assert 2 <= sweeps <= 4
