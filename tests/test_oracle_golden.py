"""The CPU restatement (oracle/rc_oracle.c) against the unmodified reference's
own outputs (tests/golden, produced by tests/golden/make_golden.py).

Dry models must match bit for bit; the wet models' viscous solve sums its dot
products and operator rows in a different order than the reference's Eigen
(shim) CG, so they are held to 1e-12 relative."""
import json
import os
import shutil
import tempfile

import numpy as np
import pytest

from oracle import oracle as orc
from tests.common import GOLDEN, build_inputs, case_from_texts, compare_to_golden, golden, run

DRY = ["polar_dry", "polar_noise", "nematic", "simple", "polar41", "resize", "ch_polar", "ch_nematic", "polar_beta", "ch_simple",
       "walls_polar", "walls_simple", "walls_wetdry", "walls_ch_polar"]
WET = ["wet", "wetpolar", "wet_equil", "ch_wet", "wetpolar_beta", "wet_restart", "wetpolar_restart",
       "ch_wetpolar"]
EQ = {"wet_equil": 3}


def _run_oracle(name):
    gd = golden(name)
    keys, m = case_from_texts(str(gd["input"]), str(gd["conf"]), str(gd["topology"]))
    _, states = run(orc.OracleSim, keys, m, [int(s) for s in gd["steps"]], eq=EQ.get(name, 0))
    return gd, states


@pytest.mark.parametrize("name", DRY)
def test_oracle_matches_reference_bitwise(name):
    gd, states = _run_oracle(name)
    errs = compare_to_golden(gd, states)
    bad = {k: v for k, v in errs.items() if v != 0.0}
    assert not bad, bad


@pytest.mark.parametrize("name", WET)
def test_oracle_matches_reference_wet(name):
    gd, states = _run_oracle(name)
    errs = compare_to_golden(gd, states)
    bad = {k: v for k, v in errs.items() if v > 1e-12}
    assert not bad, bad


def test_resize_case_resizes():
    gd = golden("resize")
    last = int(gd["steps"][-1])
    sizes = set(zip(gd["s%d_lx" % last].tolist(), gd["s%d_ly" % last].tolist()))
    assert sizes != {(27, 27)}, "fixture must exercise MultiPhaseField::set_positions' resize branch"
    _, states = _run_oracle("resize")
    assert set(zip(states[last]["lsub_x"].tolist(), states[last]["lsub_y"].tolist())) == sizes


def test_overlap_error_like_reference():
    info = json.load(open(os.path.join(GOLDEN, "overlap.json")))
    assert info["returncode"] != 0 and info["overlap_error"]
    from rheocell_gb300 import generator as g
    from tests.common import case_from_monolayer
    from tests.golden.make_golden import DRY_POLAR_S
    pos = np.tile([[24.3, 24.7]], (21, 1))
    m = g.make_monolayer(48, 21, seed=1, R=5, lam=1.5, patch=27, positions=pos)
    keys, m2 = case_from_monolayer(m, DRY_POLAR_S)
    p, cells = build_inputs(keys, m2)
    with pytest.raises(RuntimeError, match="overlap"):
        orc.OracleSim(p, m2.L, cells)


# full-size cases whose per-site arrays are stored as digests (make_golden.HASHED)
HASHED = ["dry140_100"]


@pytest.mark.parametrize("name", HASHED)
def test_oracle_matches_reference_bitwise_full_size(name):
    import hashlib

    from tests.common import CELL_KEYS, full_size_case
    gd = golden(name)
    # the generator still writes the configuration the reference ran on
    keys, m2 = full_size_case(gd)
    steps = [int(s) for s in gd["steps"]]
    _, states = run(orc.OracleSim, keys, m2, steps)

    def digest(a, dtype):
        return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()

    bad = {}
    for s in steps:
        st = states[s]
        for k, sk in CELL_KEYS.items():
            if not np.array_equal(np.asarray(st[sk]), gd["s%d_%s" % (s, k)]):
                bad[(s, k)] = float(np.max(np.abs(np.asarray(st[sk], float) - gd["s%d_%s" % (s, k)])))
        if s > 0 and digest(st["phi"], "<f8") != str(gd["s%d_phi_sha256" % s]):
            bad[(s, "phi")] = (float(np.sum(st["phi"] ** 2)), float(gd["s%d_phi_sumsq" % s]))
    last = states[steps[-1]]
    for k in ("vx", "vy", "mu"):
        if digest(last[k], "<f8") != str(gd["last_%s_sha256" % k]):
            bad[("last", k)] = (float(np.sum(last[k] ** 2)), float(gd["last_%s_sumsq" % k]))
    if digest(last["box_index"], "<i8") != str(gd["last_map_sha256"]):
        bad[("last", "map")] = "differs"
    assert not bad, bad


# full-size wet cases whose per-site arrays are stored at sampled sites (make_golden.SAMPLED)
SAMPLED = ["wet256"]


@pytest.mark.parametrize("name", SAMPLED)
def test_oracle_matches_reference_wet_full_size(name):
    from tests.common import full_size_case, sampled_errors
    gd = golden(name)
    keys, m2 = full_size_case(gd)
    _, states = run(orc.OracleSim, keys, m2, [int(s) for s in gd["steps"]])
    errs = sampled_errors(gd, states)
    bad = {k: v for k, v in errs.items() if v > 1e-12}
    assert not bad, bad


@pytest.mark.parametrize("name", ["walls_polar", "walls_simple", "walls_wetdry"])
def test_wall_cases_differ_from_the_periodic_box(name):
    """The wall goldens exercise the wall branches: the same start without
    the walls gives a different phi after the first step."""
    from rheocell_gb300 import host
    from tests.common import rel_err
    gd = golden(name)
    keys, m = case_from_texts(str(gd["input"]), str(gd["conf"]), str(gd["topology"]))
    assert host.box_walls(keys, m.L) is not None
    plain = {k: v for k, v in keys.items() if k not in ("type", "lambda_wall")}
    _, a = run(orc.OracleSim, plain, m, [1])
    assert rel_err(a[1]["phi"], gd["s1_phi"]) > 1e-6
