"""Device-side initial configurations (rc_create_generated): every patch's phi
generated by a kernel instead of parsed from a configuration file.

  * tanh discs (the benchmark workloads' profile): the same state as the
    numpy generator's patches handed to rc_create, to the last bit of tanh
    (1e-15 absolute), and the run from it within the FP64 parity bar;
  * the reference's sharp initial discs: bitwise the configuration that the
    reference's own confGenerator wrote (tests/golden/confgenerator.npz), and
    bitwise the same run."""
import re

import numpy as np
import pytest

from rheocell_gb300 import abi, engine, generator as g, host
from tests.common import case_from_texts, golden, rel_err

pytestmark = pytest.mark.gpu


def _cells(keys, m, drop_phi):
    p, cells = host.engine_inputs(keys, m)
    if drop_phi:
        for i in range(cells.n):
            cells.arr[i].phi = None
    return p, cells


@pytest.mark.parametrize("L,n", [(140, 100), (256, 400)])
def test_generated_tanh_discs_match_host_patches(L, n):
    m = g.make_monolayer(L, n, seed=1)  # numpy phi, no text round trip
    keys = {k: str(v) for k, v in g.WET_NEMATIC.items()}
    keys.update(seed="1", box="square")
    p, cells = _cells(keys, m, False)
    a = engine.Engine(p, L, cells)
    p2, cells2 = _cells(keys, m, True)
    b = engine.Engine.generated(p2, L, cells2, abi.RC_PROFILE_TANH, 8.0, 2.0)
    sa, sb = a.state(), b.state()
    assert np.max(np.abs(sa["phi"] - sb["phi"])) <= 1e-14  # CUDA tanh against glibc tanh: a few tens of ulps
    for k in ("area", "sum_f", "com_x", "com_y"):
        assert rel_err(sb[k], sa[k]) <= 1e-13, k
    a.set_phase(1)
    b.set_phase(1)
    a.step(5)
    b.step(5)
    sa, sb = a.state(), b.state()
    for k in ("phi", "vx", "vy", "area", "com_x"):
        assert rel_err(sb[k], sa[k]) <= 1e-10, k
    assert np.array_equal(sa["box_index"], sb["box_index"])


def test_generated_sharp_discs_are_confgenerators_configuration():
    gd = golden("confgenerator")
    inp = str(gd["lattice_input"])
    R = int(re.search(r"^\s*R\s*=\s*(\d+)", inp, re.M).group(1))
    conf = str(gd["lattice_conf"])
    params = dict(g.DRY_POLAR, R=R)
    n = sum(1 for ln in conf.splitlines()[2:] if ln.strip())
    keys, m = case_from_texts("\n".join("%s = %s" % kv for kv in params.items()) + "\nseed = 3\n", conf,
                              "%d 1\n%s\n" % (n, " ".join("0" for _ in range(n))))
    assert {c.lx for c in m.cells} == {30}
    p, cells = _cells(keys, m, False)
    a = engine.Engine(p, m.L, cells)
    p2, cells2 = _cells(keys, m, True)
    b = engine.Engine.generated(p2, m.L, cells2, abi.RC_PROFILE_DISC, float(R // 2))
    sa, sb = a.state(), b.state()
    assert np.array_equal(sa["phi"], sb["phi"])
    assert np.array_equal(sa["area"], sb["area"])
    a.set_phase(1)
    b.set_phase(1)
    a.step(4)
    b.step(4)
    sa, sb = a.state(), b.state()
    for k in ("phi", "vx", "vy", "area", "com_x", "box_index"):
        assert np.array_equal(sa[k], sb[k]), k


def test_generate_rejects_bad_specs():
    m = g.make_monolayer(64, 4, seed=2)
    keys = {k: str(v) for k, v in g.DRY_POLAR.items()}
    keys.update(seed="1", box="square")
    p, cells = _cells(keys, m, True)
    for prof, r, w in ((7, 8.0, 2.0), (abi.RC_PROFILE_TANH, 8.0, 0.0), (abi.RC_PROFILE_DISC, -1.0, 1.0)):
        with pytest.raises(engine.EngineError) as ei:
            engine.Engine.generated(p, 64, cells, prof, r, w)
        assert ei.value.code == abi.RC_ERR_INVALID
    # without the generator, a NULL phi is still an error
    with pytest.raises(engine.EngineError):
        engine.Engine(p, 64, cells)
