"""The stand-alone driver (rheocell_gb300/_build/rheocell, C++ over the C ABI)
against the reference's own executable: same input file, topology and
configuration; the trajectory, last_conf.dat and equilibrated_conf.dat it
writes must match the reference's files (tests/golden/cli_polar.npz) to the
engine's parity tolerance."""
import os
import subprocess

import numpy as np
import pytest

from rheocell_gb300 import build
from tests.common import golden

pytestmark = pytest.mark.gpu


def parse_confs(text):
    """List of (step, L, [per-cell number arrays]) from a configuration/trajectory text."""
    out = []
    lines = text.splitlines()
    i = 0
    while i < len(lines):
        if not lines[i].startswith("t = "):
            i += 1
            continue
        step = int(lines[i].split("=")[1])
        L = int(float(lines[i + 1].split("=")[1].split()[0]))
        cells = []
        i += 2
        while i < len(lines) and not lines[i].startswith("t = "):
            if lines[i].strip():
                cells.append(np.array(lines[i].split(), dtype=np.float64))
            i += 1
        out.append((step, L, cells))
    return out


def compare(ref_text, got_text, tol=1e-10):
    ref, got = parse_confs(ref_text), parse_confs(got_text)
    assert [r[:2] for r in ref] == [g[:2] for g in got]
    for (_, _, rc), (_, _, gc) in zip(ref, got):
        assert len(rc) == len(gc)
        for a, b in zip(rc, gc):
            assert a.shape == b.shape
            np.testing.assert_array_equal(a[:2], b[:2])        # patch size
            np.testing.assert_array_equal(a[4:7], b[4:7])      # offsets, corner
            np.testing.assert_array_equal(a[11::2], b[11::2])  # box index of every site
            scale = np.maximum(np.abs(a), 1.0)
            assert np.max(np.abs(a - b) / scale) <= tol


def test_cli_matches_reference_executable(tmp_path):
    gd = golden("cli_polar")
    for k, f in (("input", "input"), ("topology_top", "topology.top"), ("start_conf_dat", "start_conf.dat")):
        (tmp_path / f).write_text(str(gd[k]))
    build.build()
    res = subprocess.run([build.CLI, "input"], cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    compare(str(gd["equilibrated_conf_dat"]), (tmp_path / "equilibrated_conf.dat").read_text())
    compare(str(gd["trajectory_dat"]), (tmp_path / "trajectory.dat").read_text())
    compare(str(gd["last_conf_dat"]), (tmp_path / "last_conf.dat").read_text())


def test_cli_reports_reference_errors(tmp_path):
    gd = golden("cli_polar")
    (tmp_path / "input").write_text(str(gd["input"]) + "\ninteraction_type = lebcwetmodel\n")
    (tmp_path / "topology.top").write_text(str(gd["topology_top"]))
    (tmp_path / "start_conf.dat").write_text(str(gd["start_conf_dat"]))
    build.build()
    res = subprocess.run([build.CLI, "input"], cwd=str(tmp_path), capture_output=True, text=True, timeout=120)
    assert res.returncode != 0 and "not provided" in res.stderr


def test_cli_learned_solver_trains_then_reuses_parameters(tmp_path):
    """cg_solver = learned: harvest during the first steps, train, switch,
    save the parameters; a second run loads them instead of training."""
    from rheocell_gb300 import generator as g
    m = g.make_monolayer(64, 16, seed=31)
    params = dict(g.WET_NEMATIC, zetaQ_inter=0.02)
    g.write_case(str(tmp_path), m, params, steps=30, seed=32,
                 extra=dict(cg_solver="learned", learned_harvest_steps=10, learned_train_epochs=5,
                            learned_params_file="unet.txt", max_io=1e9, print_conf_interval=10))
    build.build()
    res = subprocess.run([build.CLI, "input"], cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    assert "trained on" in res.stderr
    vals = (tmp_path / "unet.txt").read_text().split()
    assert len(vals) == 25937
    confs = parse_confs((tmp_path / "trajectory.dat").read_text())
    assert [c[0] for c in confs] == [10, 20, 30]
    res2 = subprocess.run([build.CLI, "input"], cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert res2.returncode == 0, res2.stderr[-2000:]
    assert "read from unet.txt" in res2.stderr
