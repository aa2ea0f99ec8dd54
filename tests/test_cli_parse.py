"""CPU-side check of the CLI golden: the parser used by the GPU CLI test reads
the reference executable's own output consistently."""
from tests.common import golden
from tests.test_gpu_cli import compare, parse_confs


def test_golden_cli_files_parse():
    gd = golden("cli_polar")
    traj = parse_confs(str(gd["trajectory_dat"]))
    assert [t[0] for t in traj] == [10, 20]
    last = parse_confs(str(gd["last_conf_dat"]))
    assert last[0][0] == 20 and len(last[0][2]) == 9
    compare(str(gd["last_conf_dat"]), str(gd["last_conf_dat"]))


def test_cli_rejects_invalid_keys_before_touching_the_gpu(tmp_path):
    """Input validation of the stand-alone driver runs before the engine is
    created, so it is checked here without a GPU."""
    import os
    import subprocess
    from rheocell_gb300 import build
    exe = os.path.join(os.path.dirname(build.LIB), "rheocell")
    if not os.path.exists(exe):
        build.build()
    base = str(golden("cli_polar")["input"])
    for extra, msg in [("cell_tile = 200", "cell_tile must be 128, 256 or 512"),
                       ("sim_type = FD_GPU", "sim_type 'FD_GPU' is not provided"),
                       ("backend_precision = half", "Backend precision 'half' is not allowed")]:
        (tmp_path / "input").write_text(base + "\n" + extra + "\n")
        res = subprocess.run([exe, "input"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
        assert res.returncode != 0 and msg in (res.stdout + res.stderr), (extra, res.stdout, res.stderr)


def test_cli_rejects_truncated_or_corrupt_configuration(tmp_path):
    """A configuration cut short inside a patch, a corrupt header, or fewer
    patch lines than the topology's cells end the driver with the
    reference's messages (SimBackend.cpp:224-299) before the engine exists."""
    import os
    import subprocess
    from rheocell_gb300 import build
    exe = os.path.join(os.path.dirname(build.LIB), "rheocell")
    if not os.path.exists(exe):
        build.build()
    gd = golden("cli_polar")
    conf = str(gd["start_conf_dat"])
    lines = conf.splitlines()
    cases = [
        ("\n".join(lines[:3] + [lines[3][: len(lines[3]) // 2]] + lines[4:]), "configuration line too short"),
        ("\n".join(["t = x"] + lines[1:]), "Malformed headers"),
        ("\n".join(lines[:-2]), "doesn't match the parsed number of particles"),
    ]
    (tmp_path / "topology.top").write_text(str(gd["topology_top"]))
    (tmp_path / "input").write_text(str(gd["input"]))
    for text, msg in cases:
        (tmp_path / "start_conf.dat").write_text(text)
        res = subprocess.run([exe, "input"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
        assert res.returncode != 0 and msg in (res.stdout + res.stderr), (msg, res.stdout, res.stderr)


def test_python_reader_rejects_truncated_configuration(tmp_path):
    import pytest
    from rheocell_gb300 import generator as g
    conf = str(golden("cli_polar")["start_conf_dat"]).splitlines()
    (tmp_path / "c").write_text("\n".join(conf[:3] + [conf[3][: len(conf[3]) // 2]] + conf[4:]))
    with pytest.raises(ValueError, match="too short"):
        g.read_conf(str(tmp_path / "c"))
