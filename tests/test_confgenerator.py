"""The confgenerator drop-in (rheocell_gb300/_build/confgenerator) writes the
reference confGenerator's files byte for byte (tests/golden/confgenerator.npz,
made by the reference's own executable), and its benchmark options give 41x41
tanh patches readable by the engine's host mirror."""
import os
import subprocess

import numpy as np
import pytest

from rheocell_gb300 import build, generator as g
from tests.common import golden


@pytest.mark.parametrize("mode", ["random", "lattice", "cluster"])
def test_confgenerator_matches_reference(tmp_path, mode):
    gd = golden("confgenerator")
    (tmp_path / "topo.top").write_text("6 1\n0 1 0 1 0 1\n")
    (tmp_path / "input").write_text(str(gd[mode + "_input"]))
    build.build()
    subprocess.run([build.GEN, "input", "80", "conf_file=mine.dat"], cwd=str(tmp_path), check=True,
                   capture_output=True)
    assert (tmp_path / "mine.dat").read_text() == str(gd[mode + "_conf"])


def test_confgenerator_tanh_patches(tmp_path):
    (tmp_path / "topo.top").write_text("4 1\n0 0 0 0\n")
    (tmp_path / "input").write_text("interaction_type = wetmodel\nR = 8\nseed = 3\ntopology = topo.top\n"
                                    "conf_file = c.dat\ntrajectory_file = t.dat\ninitial_configuration_type = lattice\n"
                                    "n_rows = 2\nn_columns = 2\npatch_size = 41\nprofile = tanh\n")
    build.build()
    subprocess.run([build.GEN, "input", "64"], cwd=str(tmp_path), check=True, capture_output=True)
    m = g.read_conf(str(tmp_path / "c.dat"))
    assert m.L == 64 and m.n == 4 and all(c.lx == 41 for c in m.cells)
    area = [float(np.sum(c.phi ** 2)) for c in m.cells]
    assert all(150 < a < 230 for a in area)
