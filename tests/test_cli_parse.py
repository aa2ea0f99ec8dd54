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
