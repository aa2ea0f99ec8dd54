"""The reference's own rheoCell driving the GB300 engine.

The reference is built out of tree (oracle/Makefile, target cuda_backend)
without -DNOCUDA: its unmodified SimManager, BackendFactory, observables and
configuration I/O, with the `backend = CUDA` slot that BackendFactory.cpp:5-10
and :37-65 reserve filled by rheocell_gb300/refbackend (FD_CUDABackend, and
CUDAMixedBackend for backend_precision = mixed) over librheocell_gb300.so.

  * the CUDA_DOUBLE_PRECISION build (FP64) must write the trajectory,
    last_conf.dat and equilibrated_conf.dat of the reference's CPU executable
    (tests/golden/cli_polar.npz) to the engine's parity tolerance;
  * the mixed build on a wet monolayer must follow the reference's CPU build,
    run here on the same input, to the mixed solve's tolerance.

The reference's sources come from oracle/_ref/src, a git-ignored copy made by
`make -C oracle stage REF_SRC=<reference>/src` where the reference is
present; without it the test is skipped."""
import os
import subprocess

import pytest

from rheocell_gb300 import build, generator as g
from tests.common import golden
from tests.test_gpu_cli import compare

pytestmark = pytest.mark.gpu

ORACLE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")
STAGED = os.path.join(ORACLE, "_ref", "src")


@pytest.fixture(scope="module")
def exes():
    if not os.path.isfile(os.path.join(STAGED, "Backends", "BackendFactory.cpp")):
        pytest.skip("the reference's sources are not staged in oracle/_ref/src")
    build.build()
    res = subprocess.run(["make", "-C", ORACLE, "-j%d" % max(2, os.cpu_count() or 2), "cuda_backend", "cpu_main",
                          "REF_SRC=" + STAGED], capture_output=True, text=True, timeout=1200)
    assert res.returncode == 0, res.stdout[-3000:] + res.stderr[-3000:]
    from oracle import refdump
    return {k: os.path.join(refdump.REF_DIR, k) for k in ("rheoCell_cuda_double", "rheoCell_cuda", "rheoCell_exact")}


def _run(exe, d):
    res = subprocess.run([exe, "input"], cwd=str(d), capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    return res


def test_reference_rheocell_with_cuda_backend_matches_cpu_files(exes, tmp_path):
    gd = golden("cli_polar")
    text = str(gd["input"]).replace("backend = CPU", "backend = CUDA")
    assert "backend = CUDA" in text
    (tmp_path / "input").write_text(text)
    (tmp_path / "topology.top").write_text(str(gd["topology_top"]))
    (tmp_path / "start_conf.dat").write_text(str(gd["start_conf_dat"]))
    res = _run(exes["rheoCell_cuda_double"], tmp_path)
    assert "CUDA backend precision: double" in res.stdout + res.stderr
    compare(str(gd["equilibrated_conf_dat"]), (tmp_path / "equilibrated_conf.dat").read_text())
    compare(str(gd["trajectory_dat"]), (tmp_path / "trajectory.dat").read_text())
    compare(str(gd["last_conf_dat"]), (tmp_path / "last_conf.dat").read_text())


def test_reference_rheocell_mixed_backend_on_a_wet_monolayer(exes, tmp_path):
    m = g.make_monolayer(64, 9, seed=6)
    params = dict(g.WET_NEMATIC, zetaQ_inter=0.02)
    cpu, gpu = tmp_path / "cpu", tmp_path / "gpu"
    g.write_case(str(cpu), m, params, steps=6, seed=7, equilibration_steps=2)
    g.write_case(str(gpu), m, params, steps=6, seed=7, equilibration_steps=2, extra={"backend": "CUDA"})
    _run(exes["rheoCell_exact"], cpu)
    res = _run(exes["rheoCell_cuda"], gpu)
    assert "CUDA backend precision: mixed" in res.stdout + res.stderr
    for f in ("equilibrated_conf.dat", "trajectory.dat", "last_conf.dat"):
        compare((cpu / f).read_text(), (gpu / f).read_text(), tol=1e-7)
