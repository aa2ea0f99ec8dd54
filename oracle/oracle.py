"""Python handle on the CPU restatement (oracle/rc_oracle.c) -- TEST
INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline import this module, as the checker or the baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Dict, List

import numpy as np

from rheocell_gb300 import abi
from rheocell_gb300.host import HostCells

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liborc.so")


def build(force: bool = False) -> str:
    """Compile the restatement (no FMA contraction, so results are exact
    IEEE double operations in the reference's order)."""
    src = os.path.join(HERE, "rc_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src) \
            and os.path.getmtime(LIB) >= os.path.getmtime(os.path.join(HERE, "..", "include", "rheocell_gb300.h")):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c99",
                           "-Wall", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = abi.declare(C.CDLL(LIB), "orc")
    return _lib


class OracleSim:
    """Same surface as rheocell_gb300.engine.Engine, on the CPU restatement."""

    def __init__(self, params: abi.RcParams, L: int, cells: HostCells, walls=None):
        self._lib = lib()
        self.h = C.c_void_p()
        walls = None if walls is None else np.ascontiguousarray(walls, dtype=np.float64)
        box = abi.make_box(L, walls)
        rc = self._lib.orc_create(C.byref(params), C.byref(box), cells.n, cells.arr, C.byref(self.h))
        if rc != 0:
            msg = self._lib.orc_last_error(self.h).decode()
            self._lib.orc_destroy(self.h)
            self.h = None
            raise RuntimeError("orc_create failed (%d): %s" % (rc, msg))
        self.n = cells.n
        self.L = L
        self.stats = abi.RcStepStats()

    def step(self, n: int = 1) -> abi.RcStepStats:
        rc = self._lib.orc_step(self.h, n, C.byref(self.stats))
        if rc != 0:
            raise RuntimeError("orc_step failed (%d): %s" % (rc, self._lib.orc_last_error(self.h).decode()))
        return self.stats

    def set_phase(self, active: int) -> None:
        self._lib.orc_set_phase(self.h, active)

    def sizes(self):
        lx = (C.c_int * self.n)()
        ly = (C.c_int * self.n)()
        self._lib.orc_get_sizes(self.h, None, lx, ly)
        return list(lx), list(ly)

    def rng_state(self) -> int:
        return int(self._lib.orc_rng_state(self.h))

    def state(self) -> Dict[str, np.ndarray]:
        lx, ly = self.sizes()
        sizes = [a * b for a, b in zip(lx, ly)]
        hc = HostCells(self.n)
        for i in range(self.n):
            hc.attach(i, sizes[i])
        rc = self._lib.orc_download(self.h, hc.arr, abi.RC_FIELD_ALL)
        if rc != 0:
            raise RuntimeError("orc_download failed")
        return state_dict(hc, sizes)

    def close(self):
        if self.h:
            self._lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SCALARS = ["lsub_x", "lsub_y", "offset_x", "offset_y", "corner", "type", "com_x", "com_y",
           "unrap_x", "unrap_y", "q00", "q01", "theta_q", "nemq_x", "nemq_y", "area", "sum_f",
           "perimeter", "s00", "s01", "force_rep_x", "force_rep_y"]


def state_dict(hc: HostCells, sizes: List[int]) -> Dict[str, np.ndarray]:
    out = {k: hc.scalar(k) for k in SCALARS}
    for nm in ("phi", "vx", "vy", "mu", "dx", "dy", "box_index"):
        out[nm] = hc.site_array(nm, sizes)
    return out
