"""Failure detection of the engine, exercised without faulting the GPU.

Every failure is made on the host or by a bounded wait that a test hook makes
run out: a NaN written into phi through rc_upload_phi, an iteration cap the
solve cannot meet, and a grid barrier that waits for an arrival that never
comes (every block gives up after a short poll limit and the kernel
returns).  After each, the CUDA context must still serve a fresh engine."""
import numpy as np
import pytest

from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer, rel_err, run

pytestmark = pytest.mark.gpu


def _wet(L=64, n=9, seed=6, model="wetmodel", precision=abi.RC_PRECISION_DOUBLE):
    m = g.make_monolayer(L, n, seed=seed)
    keys, m2 = case_from_monolayer(m, dict(g.WET_NEMATIC, interaction_type=model, beta=0, zetaQ_inter=0.02),
                                   seed=seed + 1)
    p, cells = build_inputs(keys, m2, precision=precision)
    e = engine.Engine(p, m2.L, cells)
    e.set_phase(1)
    return e, keys, m2


def _context_still_usable():
    e, _, _ = _wet(seed=16)
    st = e.step(2)
    assert st.steps_done == 2 and 0 < st.cg_max_rel_residual < 1e-8
    e.close()


@pytest.mark.parametrize("model", ["wetmodel", "wetpolarmodel"])
def test_nan_in_phi_is_reported(model):
    e, _, _ = _wet(model=model)
    e.step(1)
    S = e.site_count()
    phi = np.zeros(S)
    assert e._lib.rc_download_phi(e.h, phi.ctypes.data_as(abi.DP), S) == 0
    phi[S // 3] = np.nan
    assert e._lib.rc_upload_phi(e.h, phi.ctypes.data_as(abi.DP), S) == 0
    with pytest.raises(engine.EngineError) as ei:
        e.step(1)
    assert ei.value.code == abi.RC_ERR_NONFINITE, str(ei.value)
    e.close()
    _context_still_usable()


def test_nan_in_phi_dry_model_is_reported():
    m = g.make_monolayer(96, 36, seed=4)
    keys, m2 = case_from_monolayer(m, g.DRY_POLAR, seed=5)
    p, cells = build_inputs(keys, m2)
    e = engine.Engine(p, m2.L, cells)
    e.set_phase(1)
    e.step(1)
    S = e.site_count()
    phi = np.zeros(S)
    e._lib.rc_download_phi(e.h, phi.ctypes.data_as(abi.DP), S)
    phi[5] = np.inf
    e._lib.rc_upload_phi(e.h, phi.ctypes.data_as(abi.DP), S)
    with pytest.raises(engine.EngineError) as ei:
        e.step(1)
    assert ei.value.code == abi.RC_ERR_NONFINITE, str(ei.value)
    e.close()


def test_iteration_cap_reports_no_convergence():
    """Eigen's behaviour by default (stop at the cap, carry on); with
    fail_on_no_convergence the step fails with RC_ERR_CG."""
    e, _, _ = _wet()
    e.step(1)
    e.set_cg_limits(3, False)
    st = e.step(1)
    assert st.cg_max_iterations == 3 and st.cg_max_rel_residual > 1e-8
    e.set_cg_limits(3, True)
    with pytest.raises(engine.EngineError) as ei:
        e.step(1)
    assert ei.value.code == abi.RC_ERR_CG and "iteration cap" in str(ei.value), str(ei.value)
    e.close()


@pytest.mark.parametrize("precision", [abi.RC_PRECISION_DOUBLE, abi.RC_PRECISION_MIXED])
def test_generous_cap_changes_nothing(precision):
    """A cap above what the solve needs leaves the run bitwise unchanged."""
    keys_m = _wet(precision=precision)
    e, keys, m = keys_m
    e.set_cg_limits(10000, True)
    e.step(3)
    a = e.state()
    e.close()
    _, b = run(engine.Engine, keys, m, [3], precision=precision)
    for k in ("phi", "vx", "vy"):
        assert np.array_equal(a[k], b[3][k]), k


def test_barrier_wait_runs_out_and_the_kernel_returns():
    e, _, _ = _wet()
    e.step(1)
    assert e._lib.rc_test_barrier_timeout(e.h, 20000, 1) == 0
    with pytest.raises(engine.EngineError) as ei:
        e.step(1)
    assert ei.value.code == abi.RC_ERR_CG and "barrier" in str(ei.value), str(ei.value)
    e.close()
    _context_still_usable()


def test_viscous_resolve_leaves_the_engine_unchanged():
    """rc_viscous_resolve: FP64 re-solve of the last evaluation from a cold
    start agrees with the engine's own (warm-started) velocities to the
    solve's tolerance, and the engine's next steps are bitwise those of an
    engine that never re-solved."""
    import torch
    e, keys, m = _wet()
    e.step(2)
    S = e.site_count()
    vx = torch.zeros(S, dtype=torch.float64, device="cuda")
    vy = torch.zeros(S, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = e.resolve(abi.RC_SOLVER_PLAIN, vx.data_ptr(), vy.data_ptr())
    assert st.cg_solves == 2 and 0 < st.cg_max_rel_residual < 1e-8
    own = e.state()
    assert rel_err(vx.cpu().numpy(), own["vx"]) < 1e-7
    assert rel_err(vy.cpu().numpy(), own["vy"]) < 1e-7
    e.step(3)
    a = e.state()
    e.close()
    _, b = run(engine.Engine, keys, m, [5])
    for k in ("phi", "vx", "vy"):
        assert np.array_equal(a[k], b[5][k]), k
