"""Readers for the reference driver's state dumps (oracle/ref_driver.cpp).

Test infrastructure only: used by tests/ and tests/golden/make_golden.py to
turn the unmodified reference's output into numpy arrays.
"""
from __future__ import annotations

import os
import platform
import subprocess
from typing import Dict, List

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# binaries of the out-of-tree reference build for this machine (oracle/Makefile)
REF_DIR = os.path.join(HERE, "_ref", platform.machine())

CELL_I32 = ["lx", "ly", "offx", "offy", "corner", "type"]
CELL_F64 = ["comx", "comy", "unrapx", "unrapy", "q00", "q01", "thetaq", "nemqx", "nemqy",
            "area", "sumf", "perimeter", "s00", "s01", "frepx", "frepy"]


def read_dump(path: str) -> List[Dict[str, object]]:
    """Parse every record of a dump file.

    Each record is a dict with ``step``, ``N``, ``L``, per-cell scalar arrays
    (names in CELL_I32 / CELL_F64) and flat per-site arrays concatenated in
    cell order (``phi``, ``map``, ``vx``, ``vy``, ``mu``, ``dx``, ``dy``).
    """
    raw = open(path, "rb").read()
    pos = 0
    out = []

    def take(dtype, count):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=pos)
        pos += a.nbytes
        return a

    while pos < len(raw):
        magic, step, n, L = take("<i4", 4)
        if magic != 0x50444352:
            raise ValueError("bad dump magic at offset %d" % pos)
        rec: Dict[str, object] = {"step": int(step), "N": int(n), "L": int(L)}
        cells_i = {k: [] for k in CELL_I32}
        cells_f = {k: [] for k in CELL_F64}
        sites = {k: [] for k in ("phi", "map", "vx", "vy", "mu", "dx", "dy")}
        for _ in range(n):
            iv = take("<i4", len(CELL_I32))
            fv = take("<f8", len(CELL_F64))
            for k, v in zip(CELL_I32, iv):
                cells_i[k].append(int(v))
            for k, v in zip(CELL_F64, fv):
                cells_f[k].append(float(v))
            m = int(iv[0]) * int(iv[1])
            sites["phi"].append(take("<f8", m).copy())
            sites["map"].append(take("<i4", m).copy())
            for k in ("vx", "vy", "mu", "dx", "dy"):
                sites[k].append(take("<f8", m).copy())
        for k, v in cells_i.items():
            rec[k] = np.array(v, dtype=np.int32)
        for k, v in cells_f.items():
            rec[k] = np.array(v, dtype=np.float64)
        for k, v in sites.items():
            rec[k] = np.concatenate(v) if v else np.zeros(0)
        out.append(rec)
    return out


def driver_path(flavour: str = "exact") -> str:
    return os.path.join(REF_DIR, "ref_driver_" + flavour)


def have_reference(flavour: str = "exact") -> bool:
    return os.access(driver_path(flavour), os.X_OK)


def run_reference(case_dir: str, steps: List[int], flavour: str = "exact",
                  overrides: Dict[str, object] = None) -> List[Dict[str, object]]:
    """Run the reference on the case in ``case_dir`` and return its dumps."""
    out = os.path.abspath(os.path.join(case_dir, "ref_dump_%s.bin" % flavour))
    args = [driver_path(flavour), "dump", out, ",".join(str(s) for s in steps), "input"]
    for k, v in (overrides or {}).items():
        args.append("%s=%s" % (k, v))
    res = subprocess.run(args, cwd=case_dir, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference failed (%d): %s %s" % (res.returncode, res.stdout[-2000:], res.stderr[-2000:]))
    return read_dump(out)


def time_reference(case_dir: str, n_steps: int, flavour: str = "fast") -> float:
    """Wall-clock seconds of n_steps reference sim_step calls on the case."""
    import json
    res = subprocess.run([driver_path(flavour), "time", str(n_steps), "input"], cwd=case_dir,
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference failed: %s" % res.stderr[-2000:])
    line = [l for l in res.stdout.splitlines() if l.startswith("{")][-1]
    return json.loads(line)["seconds"]
