"""rc_viscous_resolve_noalloc: the viscous solve re-run with its work arrays
in the library's fixed device area.  Its velocities must agree with the
engine's own solve of the same evaluation (rc_step, read back through
rc_download) to within the solver tolerance, on two calls in a row.  This
file is collected last, so it runs both after the other GPU tests and, alone,
in a fresh process."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from rheocell_gb300 import abi, engine, generator as g
from tests.common import build_inputs, case_from_monolayer, rel_err

pytestmark = pytest.mark.gpu

# both solves stop at |r| < 1e-8 |b|; their difference is bounded by the
# condition number (a few tens here) times that
TOL = 1e-6


def _wet_engine(L=64, n=9, seed=6):
    m = g.make_monolayer(L, n, seed=seed)
    keys, m2 = case_from_monolayer(m, dict(g.WET_NEMATIC, zetaQ_inter=0.02), seed=seed + 1)
    p, cells = build_inputs(keys, m2)
    e = engine.Engine(p, m2.L, cells)
    e.set_phase(1)
    return e


def _resolve(e, vx, vy):
    it = C.c_int(0)
    rc = e._lib.rc_viscous_resolve_noalloc(e.h, C.c_void_p(vx.data_ptr()), C.c_void_p(vy.data_ptr()),
                                           e.site_count(), C.byref(it))
    return rc, it.value


def test_noalloc_resolve_matches_engine_twice():
    import torch
    e = _wet_engine()
    e.step(3)
    st = e.state()
    S = e.site_count()
    assert S <= abi.RC_NOALLOC_MAX_UNKNOWNS
    vx = torch.full((S,), 7.0, dtype=torch.float64, device="cuda")
    vy = torch.full((S,), -7.0, dtype=torch.float64, device="cuda")
    for _ in range(2):
        # the fills run on torch's stream and the solve on the engine's:
        # finish them first (the entry point does not wait for the caller's
        # pending work on its arrays)
        torch.cuda.synchronize()
        rc, it = _resolve(e, vx, vy)
        assert rc == 0, e._lib.rc_last_error(e.h).decode()
        assert it > 0
        assert rel_err(vx.cpu().numpy(), st["vx"]) < TOL
        assert rel_err(vy.cpu().numpy(), st["vy"]) < TOL
        vx.fill_(3.0)
        vy.fill_(3.0)
    # the engine's own state is untouched and it keeps stepping
    e.step(1)
    st2 = e.state()
    assert np.all(np.isfinite(st2["vx"]))
    e.close()


def test_noalloc_rejects_what_does_not_fit():
    import torch
    e = _wet_engine(L=128, n=36, seed=11)
    e.step(1)
    S = e.site_count()
    assert S > abi.RC_NOALLOC_MAX_UNKNOWNS
    v = torch.zeros(8, dtype=torch.float64, device="cuda")
    it = C.c_int(0)
    rc = e._lib.rc_viscous_resolve_noalloc(e.h, C.c_void_p(v.data_ptr()), C.c_void_p(v.data_ptr()), S, C.byref(it))
    assert rc == abi.RC_ERR_CAPACITY
    assert "fixed area" in e._lib.rc_last_error(e.h).decode()
    e.close()

    m = g.make_monolayer(64, 9, seed=3)
    keys, m2 = case_from_monolayer(m, g.DRY_POLAR, seed=4)
    p, cells = build_inputs(keys, m2)
    d = engine.Engine(p, m2.L, cells)
    d.set_phase(1)
    d.step(1)
    rc = d._lib.rc_viscous_resolve_noalloc(d.h, C.c_void_p(v.data_ptr()), C.c_void_p(v.data_ptr()),
                                           d.site_count(), C.byref(it))
    assert rc == abi.RC_ERR_UNSUPPORTED
    d.close()
