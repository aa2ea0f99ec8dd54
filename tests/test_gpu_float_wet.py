"""FP32 site arithmetic for the wet models (RC_PRECISION_FLOAT with
wetmodel or a wet wetpolarmodel): the chemical potential, stresses, forces
and the Heun update in FP32 (rc_cells_f32.cu), fields stored in FP64, the
cell-area integrals in double-float, and the viscous solve in mixed
precision (FP32 inner iterations, FP64 dots and true residual, |r|/|b| below
the FP64 run's 1e-8).

Each reported field is compared with the FP64 engine on the same start:
after the first step (the forces are the right-hand side of the solve, so
the velocities carry the FP32 force error) and after 20 steps.  The error
bounds are stated per field below; they are the FP32 rounding of O(1)
quantities (phi, box sums of phi^2 and phi Q) through a few dozen
operations, grown over the steps by the dynamics.  The first-step check
runs the wetmodel without self-propulsion (zetaQ_self = 0): the tanh discs
of the start are nearly round, and the reference updates a cell's Q only
when |S| > 1e-8 (WetModel.cpp:697-747); for such cells |S| is ~1e-8, below
what FP32 gradients resolve (~1e-7, the same order as the reference's own
-ffast-math build differs from its exact build), so FP32 and FP64 can take
different branches for a cell in the first predictor, and the self-active
force of the next evaluation differs by O(dt zetaQ_self).  That shifts phi
once by ~2.5e-5 (~2e-4 on a dry monolayer, where v = f / xi); the 20-step
bound covers it."""
from __future__ import annotations

import numpy as np
import pytest

from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer, rel_err

pytestmark = pytest.mark.gpu

WET_POLAR = dict(g.DRY_POLAR, friction_cell=1)
MODELS = {"wetmodel": g.WET_NEMATIC, "wetpolarmodel": WET_POLAR}

# relative to the largest magnitude of the FP64 field
FIRST_STEP_TOL = {"phi": 1e-5, "vx": 2e-5, "vy": 2e-5, "mu": 1e-5, "dx": 1e-5, "dy": 1e-5}
AFTER_20_TOL = {"phi": 1e-4, "vx": 1e-3, "vy": 1e-3, "area": 1e-5, "com_x": 1e-5, "com_y": 1e-5}


def _pair(model, L=64, n=16, seed=4, **extra):
    m = g.make_monolayer(L, n, seed=seed)
    keys, m2 = case_from_monolayer(m, dict(MODELS[model], **extra), seed=seed)
    out = []
    for prec in (abi.RC_PRECISION_DOUBLE, abi.RC_PRECISION_FLOAT):
        p, cells = build_inputs(keys, m2, precision=prec)
        e = engine.Engine(p, m2.L, cells)
        e.set_phase(1)
        out.append(e)
    return out


@pytest.mark.parametrize("model", sorted(MODELS))
def test_first_step_close_to_fp64(model):
    a, b = _pair(model, J_Q=0, zetaQ_self=0) if model == "wetmodel" else _pair(model)
    a.step(1)
    b.step(1)
    sa, sb = a.state(), b.state()
    assert np.array_equal(sa["box_index"], sb["box_index"])
    errs = {k: rel_err(sb[k], sa[k]) for k in FIRST_STEP_TOL}
    print(model, errs)
    for k, tol in FIRST_STEP_TOL.items():
        assert errs[k] < tol, (k, errs[k])
    assert b.stats.cg_max_rel_residual < 1e-8


@pytest.mark.parametrize("model", sorted(MODELS))
def test_twenty_steps_close_to_fp64(model):
    a, b = _pair(model)
    a.step(20)
    b.step(20)
    sa, sb = a.state(), b.state()
    assert np.array_equal(sb["lsub_x"], sa["lsub_x"])
    errs = {k: rel_err(sb[k], sa[k]) for k in AFTER_20_TOL}
    print(model, errs)
    for k, tol in AFTER_20_TOL.items():
        assert errs[k] < tol, (k, errs[k])


@pytest.mark.parametrize("tile", [128, 256, 512])
def test_every_tile_close_to_fp64(tile):
    """The autotuner's candidate tiles sweep the patch in different orders:
    each stays within the same bounds."""
    a, b = _pair("wetmodel", seed=6)
    b.set_cell_threads(tile)
    a.step(5)
    b.step(5)
    sa, sb = a.state(), b.state()
    assert rel_err(sb["phi"], sa["phi"]) < 1e-4
    assert rel_err(sb["area"], sa["area"]) < 1e-5


def test_plain_fp64_solver_on_fp32_engine():
    """RC_SOLVER_PLAIN_FP64 runs Eigen's Jacobi CG in FP64 on an FP32 engine:
    on the same right-hand side it agrees with the engine's mixed solve
    within the solver tolerance."""
    import torch
    _, b = _pair("wetmodel", seed=9)
    b.step(2)
    S = b.site_count()
    v = [torch.zeros(S, dtype=torch.float64, device="cuda") for _ in range(4)]
    torch.cuda.synchronize()
    sp = b.resolve(abi.RC_SOLVER_PLAIN_FP64, v[0].data_ptr(), v[1].data_ptr())
    sm = b.resolve(abi.RC_SOLVER_PLAIN, v[2].data_ptr(), v[3].data_ptr())
    assert sp.refinements == 0 and sm.refinements > 0
    for c in range(2):
        err = float((v[2 + c] - v[c]).abs().max() / v[c].abs().max())
        assert err < 1e-6, err


def test_learned_solve_on_fp32_fields():
    """The production combination: FP32 site arithmetic with the learned
    preconditioner (trained on an FP64 engine's plain solves)."""
    a, b = _pair("wetmodel", L=128, n=36, seed=8)
    a.harvest(capacity=480, every=3, per_solve=6)
    a.step(30)
    a.harvest(480, 3, 0)
    a.train(epochs=10, batch=8, learning_rate=2e-3, learning_rate_final=1e-4, seed=1)
    b.set_params(a.get_params())
    b.set_solver(abi.RC_SOLVER_LEARNED)
    a.harvest(0, 0, 0)
    a.step(5)
    b.step(35)
    sa, sb = a.state(), b.state()
    assert b.stats.cg_max_rel_residual < 1e-8
    assert rel_err(sb["phi"], sa["phi"]) < 1e-4
    assert rel_err(sb["area"], sa["area"]) < 1e-5
