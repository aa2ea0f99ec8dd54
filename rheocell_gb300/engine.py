"""Python handle on the GB300 engine's C ABI (librheocell_gb300.so).

This is a thin caller: every step, force evaluation and solve runs in the
CUDA library.  There is no CPU fallback -- if the library cannot be loaded the
constructor raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, List, Optional

import numpy as np

from . import abi, build as _build
from .host import HostCells

_lib = None


def library_path() -> str:
    return _build.LIB


def lib() -> C.CDLL:
    """Load (building first if needed) the engine library."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB):
            _build.build()
        if not os.path.exists(_build.LIB):
            raise RuntimeError("GB300 engine library %s is missing" % _build.LIB)
        _lib = abi.declare(C.CDLL(_build.LIB), "rc")
    return _lib


class EngineError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("rc error %d: %s" % (code, msg))
        self.code = code


SCALARS = ["lsub_x", "lsub_y", "offset_x", "offset_y", "corner", "type", "com_x", "com_y",
           "unrap_x", "unrap_y", "q00", "q01", "theta_q", "nemq_x", "nemq_y", "area", "sum_f",
           "perimeter", "s00", "s01", "force_rep_x", "force_rep_y"]
SITE_FIELDS = ("phi", "vx", "vy", "mu", "dx", "dy", "box_index")


class Engine:
    """One monolayer on one GPU (rc_create / rc_step / rc_download ...)."""

    def __init__(self, params: abi.RcParams, L: int, cells: HostCells, device: int = 0, walls=None):
        self._lib = lib()
        self.h = C.c_void_p()
        walls = None if walls is None else np.ascontiguousarray(walls, dtype=np.float64)
        box = abi.make_box(L, walls)
        rc = self._lib.rc_create(C.byref(params), C.byref(box), cells.n, cells.arr, device, C.byref(self.h))
        if rc != 0:
            msg = self._lib.rc_last_error(self.h).decode()
            if self.h:
                self._lib.rc_destroy(self.h)
            self.h = None
            raise EngineError(rc, msg)
        self.n = cells.n
        self.L = L
        self.device = device
        self.layer_sizes = [cells.n]
        self.stats = abi.RcStepStats()

    @classmethod
    def generated(cls, params: abi.RcParams, L: int, cells: HostCells, profile: int, radius: float,
                  width: float = 1.0, device: int = 0) -> "Engine":
        """A monolayer whose patches' phi is generated on the device
        (rc_create_generated); `cells` gives the geometry, centres and Q
        (their phi pointers are not read)."""
        self = cls.__new__(cls)
        self._lib = lib()
        self.h = C.c_void_p()
        spec = abi.RcGenerateSpec(profile, radius, width)
        rc = self._lib.rc_create_generated(C.byref(params), C.byref(abi.RcBox(L, L)), cells.n, cells.arr,
                                           C.byref(spec), device, C.byref(self.h))
        if rc != 0:
            msg = self._lib.rc_last_error(self.h).decode()
            if self.h:
                self._lib.rc_destroy(self.h)
            self.h = None
            raise EngineError(rc, msg)
        self.n = cells.n
        self.L = L
        self.device = device
        self.layer_sizes = [cells.n]
        self.stats = abi.RcStepStats()
        return self

    @classmethod
    def batch(cls, params: abi.RcParams, layers, device: int = 0) -> "Engine":
        """An ensemble of independent monolayers advanced together
        (rc_batch_create).  `layers` is a list of (L, HostCells, rng_state);
        cells of all layers are addressed layer-major afterwards."""
        self = cls.__new__(cls)
        self._lib = lib()
        self.h = C.c_void_p()
        nl = len(layers)
        boxes = (abi.RcBox * nl)(*[abi.RcBox(L, L) for L, _, _ in layers])
        counts = (C.c_int * nl)(*[hc.n for _, hc, _ in layers])
        total = sum(hc.n for _, hc, _ in layers)
        arr = (abi.RcCellHost * max(total, 1))()
        j = 0
        for _, hc, _ in layers:
            for i in range(hc.n):
                arr[j] = hc.arr[i]
                j += 1
        states = (C.c_ulonglong * nl)(*[int(s) for _, _, s in layers])
        self._keep = [hc for _, hc, _ in layers]
        rc = self._lib.rc_batch_create(C.byref(params), nl, boxes, counts, arr, states, device, C.byref(self.h))
        if rc != 0:
            msg = self._lib.rc_last_error(self.h).decode()
            if self.h:
                self._lib.rc_destroy(self.h)
            self.h = None
            raise EngineError(rc, msg)
        self.n = total
        self.device = device
        self.L = [L for L, _, _ in layers]
        self.layer_sizes = [hc.n for _, hc, _ in layers]
        self.stats = abi.RcStepStats()
        return self

    def layer_count(self) -> int:
        return int(self._lib.rc_layer_count(self.h))

    def split(self, state: Dict[str, np.ndarray]) -> List[Dict[str, np.ndarray]]:
        """Split a state() of a batch into one dict per layer."""
        lx, ly = np.asarray(state["lsub_x"]), np.asarray(state["lsub_y"])
        sizes = lx * ly
        out, c0, s0 = [], 0, 0
        for n in self.layer_sizes:
            ns = int(sizes[c0:c0 + n].sum())
            d = {}
            for k, v in state.items():
                d[k] = v[s0:s0 + ns] if k in SITE_FIELDS else v[c0:c0 + n]
            out.append(d)
            c0 += n
            s0 += ns
        return out

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise EngineError(rc, "%s: %s" % (what, self._lib.rc_last_error(self.h).decode()))

    def step(self, n: int = 1) -> abi.RcStepStats:
        self._check(self._lib.rc_step(self.h, n, C.byref(self.stats)), "rc_step")
        return self.stats

    def set_phase(self, active: int) -> None:
        self._check(self._lib.rc_set_phase(self.h, active), "rc_set_phase")

    def set_stream(self, stream_ptr: int) -> None:
        self._check(self._lib.rc_set_stream(self.h, C.c_void_p(stream_ptr)), "rc_set_stream")

    def site_count(self) -> int:
        return int(self._lib.rc_site_count(self.h))

    def sizes(self):
        lx = (C.c_int * self.n)()
        ly = (C.c_int * self.n)()
        self._check(self._lib.rc_get_sizes(self.h, None, lx, ly), "rc_get_sizes")
        return list(lx), list(ly)

    def state(self, mask: int = abi.RC_FIELD_ALL) -> Dict[str, np.ndarray]:
        lx, ly = self.sizes()
        sizes = [a * b for a, b in zip(lx, ly)]
        hc = HostCells(self.n)
        for i in range(self.n):
            hc.attach(i, sizes[i])
        self._check(self._lib.rc_download(self.h, hc.arr, mask), "rc_download")
        out = {k: hc.scalar(k) for k in SCALARS}
        for nm in ("phi", "vx", "vy", "mu", "dx", "dy", "box_index"):
            out[nm] = hc.site_array(nm, sizes)
        return out

    def download(self, hc: HostCells, mask: int) -> None:
        self._check(self._lib.rc_download(self.h, hc.arr, mask), "rc_download")

    def upload(self, hc: HostCells, mask: int) -> None:
        self._check(self._lib.rc_upload(self.h, hc.arr, mask), "rc_upload")

    # --- learned preconditioner of the viscous solve ---------------------------

    def harvest(self, capacity: int, every: int = 4, per_solve: int = 4) -> None:
        """Collect training samples from the following plain FP64 solves."""
        self._check(self._lib.rc_learned_harvest(self.h, capacity, every, per_solve), "rc_learned_harvest")

    def harvested(self) -> int:
        return int(self._lib.rc_learned_harvested(self.h))

    def train(self, epochs: int = 8, batch: int = 8, learning_rate: float = 1e-3, validation: float = 0.1,
              seed: int = 0, init: bool = True, max_samples: int = 0,
              learning_rate_final: float = 0.0) -> Dict[str, float]:
        """Train the network on the harvested samples (device kernels)."""
        o = abi.RcTrainOptions(epochs, batch, learning_rate, validation, seed, int(init), max_samples,
                               learning_rate_final)
        r = abi.RcTrainReport()
        self._check(self._lib.rc_learned_train(self.h, C.byref(o), C.byref(r)), "rc_learned_train")
        return {name: getattr(r, name) for name, _ in abi.RcTrainReport._fields_}

    def set_solver(self, solver: int) -> None:
        self._check(self._lib.rc_set_solver(self.h, solver), "rc_set_solver")

    def resolve(self, solver: int, vx_ptr: int, vy_ptr: int) -> abi.RcStepStats:
        """Re-run the last evaluation's viscous solve from a cold start with
        `solver` into device arrays (pointers) of site_count() doubles; the
        engine's own state is unchanged (rc_viscous_resolve)."""
        st = abi.RcStepStats()
        self._check(self._lib.rc_viscous_resolve(self.h, solver, C.c_void_p(vx_ptr), C.c_void_p(vy_ptr),
                                                 self.site_count(), C.byref(st)), "rc_viscous_resolve")
        return st

    def set_cg_limits(self, max_iterations: int, fail_on_no_convergence: bool) -> None:
        self._check(self._lib.rc_set_cg_limits(self.h, max_iterations, int(fail_on_no_convergence)),
                    "rc_set_cg_limits")

    def set_cg_tolerance(self, tolerance: float) -> None:
        self._check(self._lib.rc_set_cg_tolerance(self.h, tolerance), "rc_set_cg_tolerance")

    def get_params(self) -> np.ndarray:
        p = np.zeros(abi.RC_UNET_PARAMS)
        self._check(self._lib.rc_learned_get_params(self.h, p.ctypes.data_as(abi.DP)), "rc_learned_get_params")
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float64)
        if p.size != abi.RC_UNET_PARAMS:
            raise ValueError("the network has %d parameters, got %d" % (abi.RC_UNET_PARAMS, p.size))
        self._check(self._lib.rc_learned_set_params(self.h, p.ctypes.data_as(abi.DP)), "rc_learned_set_params")

    # --- tile-shape autotuning of the FP32 cell kernel ----------------------------

    def autotune(self, steps_per_candidate: int = 4) -> Dict[str, object]:
        """Time every cell tile on this workload and keep the fastest
        (advances the simulation by 3 x (steps_per_candidate + 1) steps)."""
        r = abi.RcAutotuneReport()
        self._check(self._lib.rc_autotune(self.h, steps_per_candidate, C.byref(r)), "rc_autotune")
        return {"candidates": [(r.threads[i], r.ms_per_step[i]) for i in range(r.candidates)], "chosen": r.chosen}

    def set_cell_threads(self, threads: int) -> None:
        self._check(self._lib.rc_set_cell_threads(self.h, threads), "rc_set_cell_threads")

    def close(self):
        if self.h:
            self._lib.rc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
