"""Force observables on the device (rc_observe_field with the force kinds,
rc_observe_stress) against the reference's own ForceField, StressField and
ThermodynamicStressField
output (tests/golden/obs_*.npz: its observable classes run by
oracle/ref_driver.cpp after two main-loop steps of the same case).

Layouts compared, per box site in row-major order:
  ForceField  (ForceField.cpp:131-168): x, y, F, F_passive, F_active (x and y
              each), then the same of the size_grid window means;
  StressField (StressField.cpp:165-199): x, y, then xx, yy, xy of the
              total, passive and active forces, and xx, yy of the pressure;
  ThermodynamicStressField (ThermodynamicStressField.cpp:115-153): x, y,
              xx, yy, xy, sum of mu, sum of mu^2, then the window means.
The passive, active and pressure fields follow from phi, which the engine
holds to the reference within 1e-10 after two steps (dry models: far
closer); the total force is the velocity times the friction, which for the
wet models comes out of the viscous solve (1e-9 relative).  The reference
prints 15 significant digits.  Tolerance per column: 1e-9 of the column's
largest magnitude for the wet models, 1e-11 for the dry ones."""
import numpy as np
import pytest

from rheocell_gb300 import abi, engine
from tests.common import case_from_texts, golden, run

pytestmark = pytest.mark.gpu

CASES = {"obs_wet": 1e-9, "obs_wetpolar": 1e-9, "obs_nematic": 1e-11, "obs_polar": 1e-11, "obs_simple": 1e-11}


def _dp(a):
    return a.ctypes.data_as(abi.DP)


def _observe(e, L, sg):
    lib = e._lib
    n = L * L
    box = {}
    for kind in (abi.RC_OBS_FORCE, abi.RC_OBS_FORCE_PASSIVE, abi.RC_OBS_FORCE_ACTIVE):
        f = [np.zeros(n) for _ in range(4)]
        assert lib.rc_observe_field(e.h, kind, 0, -1, sg, *(_dp(a) for a in f)) == 0, lib.rc_last_error(e.h)
        box[kind] = f
    stress = {}
    for kind in (abi.RC_OBS_FORCE, abi.RC_OBS_FORCE_PASSIVE, abi.RC_OBS_FORCE_ACTIVE, abi.RC_OBS_PRESSURE):
        s = [np.zeros(n) for _ in range(3)]
        assert lib.rc_observe_stress(e.h, kind, 0, -1, sg, *(_dp(a) for a in s)) == 0, lib.rc_last_error(e.h)
        stress[kind] = s
    th = {}
    for kind in (abi.RC_OBS_THERMO, abi.RC_OBS_THERMO_XY, abi.RC_OBS_CHEMPOT2):
        f = [np.zeros(n) for _ in range(4)]
        assert lib.rc_observe_field(e.h, kind, 0, -1, sg, *(_dp(a) for a in f)) == 0, lib.rc_last_error(e.h)
        th[kind] = f
    jj, ii = np.meshgrid(np.arange(L), np.arange(L))
    x, y = (jj.ravel() + 0.5), (ii.ravel() + 0.5)
    F, P, A = abi.RC_OBS_FORCE, abi.RC_OBS_FORCE_PASSIVE, abi.RC_OBS_FORCE_ACTIVE
    force = np.concatenate([
        np.stack([x, y, box[F][0], box[F][1], box[P][0], box[P][1], box[A][0], box[A][1]], 1).ravel(),
        np.stack([x, y, box[F][2], box[F][3], box[P][2], box[P][3], box[A][2], box[A][3]], 1).ravel()])
    R = abi.RC_OBS_PRESSURE
    st = np.stack([x, y, *stress[F], *stress[P], *stress[A], stress[R][0], stress[R][1]], 1).ravel()
    T, X, M = abi.RC_OBS_THERMO, abi.RC_OBS_THERMO_XY, abi.RC_OBS_CHEMPOT2
    thermo = np.concatenate([
        np.stack([x, y, th[T][0], th[T][1], th[X][0], th[X][1], th[M][0]], 1).ravel(),
        np.stack([x, y, th[T][2], th[T][3], th[X][2], th[X][3], th[M][2]], 1).ravel()])
    return force, st, thermo


def _compare(got, want, ncol, tol):
    got, want = got.reshape(-1, ncol), want.reshape(-1, ncol)
    assert got.shape == want.shape
    bad = {}
    for c in range(ncol):
        scale = max(float(np.max(np.abs(want[:, c]))), 1e-300)
        err = float(np.max(np.abs(got[:, c] - want[:, c]))) / scale
        if err > tol:
            bad[c] = err
    assert not bad, bad


@pytest.mark.parametrize("name", sorted(CASES))
def test_force_and_stress_fields_match_reference(name):
    gd = golden(name)
    keys, m = case_from_texts(str(gd["input"]), str(gd["conf"]), str(gd["topology"]))
    step, sg = int(gd["step"]), int(gd["size_grid"])
    e, _ = run(engine.Engine, keys, m, [step])
    before = e.state()
    force, stress, thermo = _observe(e, m.L, sg)
    _compare(force, gd["force_field"], 8, CASES[name])
    _compare(stress, gd["stress_field"], 13, CASES[name])
    _compare(thermo, gd["thermodynamic_stress_field"], 7, CASES[name])
    # observing leaves the run unchanged
    after = e.state()
    for k in ("phi", "vx", "vy", "mu", "area", "force_rep_x", "theta_q"):
        assert np.array_equal(before[k], after[k]), k
    e.step(2)
    e2, _ = run(engine.Engine, keys, m, [step + 2])
    a, b = e.state(), e2.state()
    for k in ("phi", "vx", "vy", "com_x", "theta_q"):
        assert np.array_equal(a[k], b[k]), k
