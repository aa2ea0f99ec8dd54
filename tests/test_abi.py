"""The engine library builds for sm_103a, loads, and exports every symbol the
C header declares (no CUDA calls: this runs without a GPU)."""
import ctypes
import os
import re

from rheocell_gb300 import abi, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "rheocell_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rc_[a-z_]+)\s*\(", src)))


def test_header_matches_python_mirror():
    assert declared_symbols() == sorted(abi.EXPORTED)


def test_library_exports_every_symbol():
    lib = ctypes.CDLL(build.build())
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_struct_sizes_match_header():
    # layouts the C compiler gives the header's structs, vs the ctypes mirror
    import subprocess
    import tempfile
    d = tempfile.mkdtemp()
    c = os.path.join(d, "s.c")
    with open(c, "w") as f:
        f.write('#include "%s"\n#include <stdio.h>\n#include <stddef.h>\nint main(){printf("%%zu %%zu %%zu %%zu %%zu %%zu '
                '%%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu\\n",'
                'sizeof(rc_params),sizeof(rc_cell_host),sizeof(rc_step_stats),offsetof(rc_params,rng_state),'
                'offsetof(rc_cell_host,phi),offsetof(rc_cell_host,box_index),sizeof(rc_train_options),'
                'sizeof(rc_train_report),offsetof(rc_train_report,ms),offsetof(rc_train_options,learning_rate_final),'
                'sizeof(rc_autotune_report),offsetof(rc_autotune_report,ms_per_step),'
                'offsetof(rc_autotune_report,chosen),offsetof(rc_params,conserved),sizeof(rc_box),'
                'offsetof(rc_params,wall_slip));}\n' % HEADER)
    subprocess.check_call(["gcc", c, "-o", os.path.join(d, "s")])
    out = subprocess.check_output([os.path.join(d, "s")]).decode().split()
    want = [ctypes.sizeof(abi.RcParams), ctypes.sizeof(abi.RcCellHost), ctypes.sizeof(abi.RcStepStats),
            abi.RcParams.rng_state.offset, abi.RcCellHost.phi.offset, abi.RcCellHost.box_index.offset,
            ctypes.sizeof(abi.RcTrainOptions), ctypes.sizeof(abi.RcTrainReport), abi.RcTrainReport.ms.offset,
            abi.RcTrainOptions.learning_rate_final.offset, ctypes.sizeof(abi.RcAutotuneReport),
            abi.RcAutotuneReport.ms_per_step.offset, abi.RcAutotuneReport.chosen.offset, abi.RcParams.conserved.offset,
            ctypes.sizeof(abi.RcBox), abi.RcParams.wall_slip.offset]
    assert [int(x) for x in out] == want
