"""Learned preconditioner of the viscous solve: samples harvested from the
plain FP64 solve, device training, and the flexible-CG solve that uses the
network.  Its velocities must stay within 1e-7 (relative) of the FP64 oracle,
the solve must stop at the FP64 tolerance, and the trained network must cut
the inner iterations of the mixed solve compared with the same solve
without it."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as orc
from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer, rel_err

pytestmark = pytest.mark.gpu

WARM = 20  # plain FP64 steps that harvest the training samples


def _case(L=64, n=16, seed=31):
    m = g.make_monolayer(L, n, seed=seed)
    return case_from_monolayer(m, dict(g.WET_NEMATIC, zetaQ_inter=0.02), seed=seed + 1)


@pytest.fixture(scope="module")
def trained():
    keys, m = _case()
    p, cells = build_inputs(keys, m)
    e = engine.Engine(p, m.L, cells)
    e.set_phase(1)
    e.harvest(capacity=2000, every=3, per_solve=6)
    e.step(WARM)
    n = e.harvested()
    rep = e.train(epochs=40, batch=8, learning_rate=2e-3, seed=1)
    return keys, m, e, n, rep


def test_training_reduces_validation_loss(trained):
    _, _, _, n, rep = trained
    print("harvested", n, "report", rep)
    assert n >= 200
    assert rep["samples"] > 100 and rep["steps"] > 0
    assert rep["validation_loss"] < 0.3 * rep["validation_loss_init"], rep
    assert rep["loss_last_epoch"] < rep["loss_first_epoch"], rep


def test_learned_solve_matches_fp64_oracle(trained):
    keys, m, e, _, _ = trained
    steps = 4
    e.set_solver(abi.RC_SOLVER_LEARNED)
    st = e.step(steps)
    print("learned solve:", st.cg_iterations, st.refinements, st.cg_max_rel_residual)
    assert st.cg_max_rel_residual < 1e-8
    got = e.state()
    # the oracle from the same initial state, plain FP64 CG throughout
    p, cells = build_inputs(keys, m)
    o = orc.OracleSim(p, m.L, cells)
    o.set_phase(1)
    o.step(WARM + steps)
    want = o.state()
    for k in ("vx", "vy", "phi", "area", "com_x"):
        assert rel_err(got[k], want[k]) < 1e-7, k
    e.set_solver(abi.RC_SOLVER_PLAIN)


@pytest.mark.parametrize("solver", [abi.RC_SOLVER_LEARNED, abi.RC_SOLVER_LEARNED_FP32])
def test_network_cuts_inner_iterations(trained, solver):
    """Same state, same mixed-precision refinement: inner iterations with the
    network (flexible CG) against the Jacobi inner iterations without it."""
    keys, m, e, _, _ = trained
    params = e.get_params()

    def run(solver):
        p, cells = build_inputs(keys, m, precision=abi.RC_PRECISION_MIXED)
        f = engine.Engine(p, m.L, cells)
        f.set_phase(1)
        f.step(WARM)
        f.set_params(params)
        f.set_solver(solver)
        s = f.step(4)
        out = (s.cg_iterations, s.cg_max_rel_residual)
        f.close()
        return out

    it_plain, res_plain = run(abi.RC_SOLVER_PLAIN)
    it_learned, res_learned = run(solver)
    print("inner iterations: plain", it_plain, res_plain, "learned", it_learned, res_learned)
    assert res_plain < 1e-8 and res_learned < 1e-8
    assert it_learned < 0.5 * it_plain, (it_learned, it_plain)


def test_learned_solve_with_strip_layers_matches_fp64_oracle(trained):
    """A 128^2 monolayer with the network trained on the 64^2 one: its finest
    level runs the strip tensor-core layers (first layer fused into the
    second's staging, decoupled row pipeline), the coarser levels the gathered
    ones; velocities within 1e-7 of the FP64 oracle, FP64 stopping rule met."""
    _, _, e64, _, _ = trained
    params = e64.get_params()
    m = g.make_monolayer(128, 64, seed=41)
    keys, m2 = case_from_monolayer(m, dict(g.WET_NEMATIC, zetaQ_inter=0.02), seed=42)
    warm, steps = 6, 3
    p, cells = build_inputs(keys, m2)
    e = engine.Engine(p, m2.L, cells)
    e.set_phase(1)
    e.step(warm)
    e.set_params(params)
    e.set_solver(abi.RC_SOLVER_LEARNED)
    st = e.step(steps)
    print("learned solve at 128:", st.cg_iterations, st.refinements, st.cg_max_rel_residual)
    assert st.cg_max_rel_residual < 1e-8
    got = e.state()
    p, cells = build_inputs(keys, m2)
    o = orc.OracleSim(p, m2.L, cells)
    o.set_phase(1)
    o.step(warm + steps)
    want = o.state()
    for k in ("vx", "vy", "phi", "area", "com_x"):
        assert rel_err(got[k], want[k]) < 1e-7, k
    e.close()


def test_stalled_refinement_falls_back_to_fp64(trained):
    """A network that points the wrong way (negated parameters): the
    refinement sweeps stop reducing the residual, the plain FP64 CG takes
    over (counted in rc_step_stats.fallbacks), and the solve still meets the
    FP64 stopping rule with velocities within 1e-7 of the FP64 oracle."""
    keys, m, e64, _, _ = trained
    params = -e64.get_params()
    p, cells = build_inputs(keys, m)
    e = engine.Engine(p, m.L, cells)
    e.set_phase(1)
    e.step(WARM)
    e.set_params(params)
    e.set_solver(abi.RC_SOLVER_LEARNED)
    st = e.step(2)
    print("negated network:", st.cg_iterations, st.refinements, st.fallbacks, st.cg_max_rel_residual)
    assert st.fallbacks > 0
    assert st.cg_max_rel_residual < 1e-8
    got = e.state()
    p, cells = build_inputs(keys, m)
    o = orc.OracleSim(p, m.L, cells)
    o.set_phase(1)
    o.step(WARM + 2)
    want = o.state()
    for k in ("vx", "vy", "phi"):
        assert rel_err(got[k], want[k]) < 1e-7, k
    e.close()


@pytest.mark.parametrize("L", [512, 800])
def test_learned_solve_on_large_boxes(trained, L):
    """The learned solve on the benchmark box sides with few cells: 512^2
    runs every network level on the strip tensor-core layers (512, 256, 128),
    800^2 the gathered layers and the grid-stride split of the box sites.
    The same right-hand side solved by the learned flexible CG and by the
    plain FP64 CG (rc_viscous_resolve) agrees within 1e-7, and after steps
    with the learned solver the state is within 1e-7 of the FP64 oracle."""
    import torch
    from tests.test_gpu_large_box import cluster_case
    _, _, e64, _, _ = trained
    params = e64.get_params()
    keys, m = cluster_case(L, "wetmodel")
    warm, steps = 3, 2
    p, cells = build_inputs(keys, m)
    e = engine.Engine(p, m.L, cells)
    e.set_phase(1)
    e.step(warm)
    e.set_params(params)
    S = e.site_count()
    v = [torch.zeros(S, dtype=torch.float64, device="cuda") for _ in range(4)]
    torch.cuda.synchronize()
    sp = e.resolve(abi.RC_SOLVER_PLAIN, v[0].data_ptr(), v[1].data_ptr())
    sl = e.resolve(abi.RC_SOLVER_LEARNED, v[2].data_ptr(), v[3].data_ptr())
    print("L=%d plain %d it, learned %d inner it (%d refinements)" % (L, sp.cg_iterations, sl.cg_iterations,
                                                                         sl.refinements))
    assert sp.cg_max_rel_residual < 1e-8 and sl.cg_max_rel_residual < 1e-8
    for a, b in ((v[2], v[0]), (v[3], v[1])):
        assert rel_err(a.cpu().numpy(), b.cpu().numpy()) < 1e-7
    e.set_solver(abi.RC_SOLVER_LEARNED)
    st = e.step(steps)
    assert st.cg_max_rel_residual < 1e-8
    got = e.state()
    e.close()
    p, cells = build_inputs(keys, m)
    o = orc.OracleSim(p, m.L, cells)
    o.set_phase(1)
    o.step(warm + steps)
    want = o.state()
    for k in ("vx", "vy", "phi", "area", "com_x"):
        assert rel_err(got[k], want[k]) < 1e-7, k


def test_committed_network_on_the_training_monolayer():
    """tests/golden/unet_wet256.npy holds the network the default bench line
    trains (tests/golden/make_unet_params.py).  On the monolayer it was
    trained on (wet 256^2, 400 cells, FP32 site arithmetic) the learned solve
    of one right-hand side needs under a fifth of the Jacobi flexible CG's
    inner iterations, converges to the learned solve's residual margin (0.2 of
    the tolerance), and its velocities are within 1e-7 (max norm, relative to
    the largest velocity) of the FP64 CG solved to 1e-12."""
    import os
    import torch
    import bench
    params = np.load(os.path.join(os.path.dirname(__file__), "golden", "unet_wet256.npy")).astype(np.float64)
    e = bench.make_engine("wet256", abi.RC_PRECISION_FLOAT, 0)
    e.set_params(params)
    e.set_solver(abi.RC_SOLVER_LEARNED)
    e.step(5)
    S = e.site_count()
    v = [torch.zeros(S, dtype=torch.float64, device="cuda") for _ in range(6)]
    torch.cuda.synchronize()
    e.set_cg_tolerance(1e-12)
    e.resolve(abi.RC_SOLVER_PLAIN_FP64, v[4].data_ptr(), v[5].data_ptr())
    e.set_cg_tolerance(1e-8)
    sj = e.resolve(abi.RC_SOLVER_PLAIN, v[0].data_ptr(), v[1].data_ptr())
    sl = e.resolve(abi.RC_SOLVER_LEARNED, v[2].data_ptr(), v[3].data_ptr())
    print("Jacobi FCG %d it, learned %d inner it, residual %.2e" % (sj.cg_iterations, sl.cg_iterations,
                                                                    sl.cg_max_rel_residual))
    assert sl.fallbacks == 0
    assert sl.cg_iterations * 5 < sj.cg_iterations
    assert sl.cg_max_rel_residual < 0.2 * 1e-8
    for c in range(2):
        err = float((v[2 + c] - v[4 + c]).abs().max() / v[4 + c].abs().max())
        assert err < 1e-7, err
    e.close()
