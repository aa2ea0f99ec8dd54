"""Host-side set-up that mirrors the reference's backend and interaction
construction for the selected model, producing the C-ABI inputs.

What is mirrored (paths relative to the reference's src/):
  * interaction constructors and get_settings: default values and which keys
    each model reads (SimpleMultiField.cpp:4-27, ActiveNematic.cpp:4-37,
    WetPolarModel.cpp:123-166, WetModel.cpp:4-47);
  * apply_changes_after_equilibration: which values switch from the
    constructor default to the input value (WetPolarModel.cpp:203-212,
    WetModel.cpp:88-96, ActiveNematic.cpp:76-80);
  * the order of drand48 draws before the first step: srand48(seed)
    (Managers/SimManager.cpp:86), one draw per cell in
    WetPolarModel::read_topology (WetPolarModel.cpp:191), then one draw per
    cell in MultiPhaseField::init (Fields/MultiPhaseField.cpp:79) which seeds
    the nematic director nemQ;
  * the configuration reader's derived values: thetaQ = atan2(2Q01, 2Q00)/2,
    area = sum phi^2, sumF = sum phi (Backends/SimBackend.cpp:283-296).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import abi
from .generator import Monolayer

PI_F = float(np.float32(3.141592653589793238462643))


class Drand48:
    """POSIX drand48/srand48 (48-bit LCG) plus Utils::gaussian's cached pair
    (src/Utilities/Utils.h:210-236)."""

    A = 0x5DEECE66D
    C = 0xB
    M = (1 << 48) - 1

    def __init__(self, seed: int):
        self.state = (((seed & 0xFFFFFFFF) << 16) | 0x330E) & self.M
        self.has_cached = 0
        self.cached = 0.0

    def drand48(self) -> float:
        self.state = (self.A * self.state + self.C) & self.M
        return self.state / float(1 << 48)

    def gaussian(self) -> float:
        if self.has_cached:
            self.has_cached = 0
            return self.cached
        w = 2.0
        while w >= 1.0:
            u = 2.0 * self.drand48() - 1.0
            v = 2.0 * self.drand48() - 1.0
            w = u * u + v * v
        w = math.sqrt((-2.0 * math.log(w)) / w)
        self.cached = v * w
        self.has_cached = 1
        return u * w


# (constructor default, key read by get_settings or None) per model.
_COMMON_KEYS = ("gamma", "lambda", "omega", "mu", "kappa")
_DEFAULTS = {
    "simplefield": dict(gamma=0.01, **{"lambda": 2.5}, mu=3.0, kappa=0.1, omega=0.0),
    "activenematic": dict(gamma=0.01, **{"lambda": 2.5}, omega=0.004, mu=3.0, kappa=0.1),
    "wetpolarmodel": dict(gamma=0.06, **{"lambda": 2.5}, omega=0.004, mu=20.0, kappa=0.1),
    "wetmodel": dict(gamma=0.01, **{"lambda": 2.5}, omega=0.004, mu=3.0, kappa=0.1),
}
# keys each model's get_settings reads among the common ones (simplefield does
# not read lambda: SimpleMultiField.cpp:19-27)
_READS = {
    "simplefield": ("gamma", "mu", "kappa", "omega"),
    "activenematic": _COMMON_KEYS,
    "wetpolarmodel": _COMMON_KEYS,
    "wetmodel": _COMMON_KEYS,
}


def _num(keys: Dict[str, object], k: str, default=None, required=False) -> Optional[float]:
    if k in keys:
        return float(keys[k])
    if required:
        raise ValueError("input key '%s' is required" % k)
    return default


def make_params(keys: Dict[str, object], precision: int = abi.RC_PRECISION_DOUBLE) -> abi.RcParams:
    """rc_params for the interaction named by keys['interaction_type']."""
    name = str(keys["interaction_type"]).strip().lower()
    if name not in abi.MODEL_NAMES:
        raise ValueError("interaction_type '%s' is not provided by the GB300 engine" % name)
    if str(keys.get("box", "square")).strip() != "square":
        raise ValueError("only the square boxes are provided (box = square, with or without walls)")
    if int(float(keys.get("external_forces", 0))) != 0:
        raise ValueError("external forces are not provided")
    if int(float(keys.get("anchoring", 0))) != 0:
        raise ValueError("anchoring is not provided")
    p = abi.RcParams()
    p.model = abi.MODEL_NAMES[name]
    p.precision = precision
    p.R = int(float(keys["R"]))
    p.border = 4
    p.dt = float(keys["dt"])
    p.J0 = _num(keys, "J0", 1.0)
    sim_type = str(keys.get("sim_type", "FD_CPU")).strip()
    if sim_type not in ("FD_CPU", "FD_CH"):
        raise ValueError("sim_type '%s' is not provided by the GB300 engine" % sim_type)
    p.conserved = 1 if sim_type == "FD_CH" else 0
    d = dict(_DEFAULTS[name])
    for k in _READS[name]:
        if k in keys:
            d[k] = float(keys[k])
    p.gamma, p.lambda_, p.omega, p.mu, p.kappa = d["gamma"], d["lambda"], d["omega"], d["mu"], d["kappa"]
    p.passive_alpha = _num(keys, "passive_alpha", 1.0) if name in ("wetmodel", "wetpolarmodel") else 1.0
    p.cg_tolerance = _num(keys, "CGtolerance", 0.0001) if name in ("wetmodel", "wetpolarmodel") else 0.0
    p.cg_restart_every = 10 if name == "wetpolarmodel" else 100
    p.anchoring = 0
    p.wall_slip = _num(keys, "wall_slip", 0.5)  # BaseInteraction.cpp:10,23
    if name == "simplefield":
        p.friction = abi.D2(1.0, 1.0)
        p.friction_cell = abi.D2(0, 0)
        p.zetaQ_self = abi.D2(0, 0)
        p.zetaQ_inter = abi.D2(0, 0)
        p.J_Q = abi.D2(0, 0)
        p.beta = abi.D2(0, 0)
    elif name == "activenematic":
        fr = _num(keys, "friction", 2.0)
        p.friction = abi.D2(fr, fr)
        p.friction_cell = abi.D2(0, 0)
        p.zetaQ_self = abi.D2(0, _num(keys, "zetaQ_self", required=True))
        p.zetaQ_inter = abi.D2(0, _num(keys, "zetaQ_inter", required=True))
        p.J_Q = abi.D2(0, _num(keys, "J_Q", required=True))
        p.beta = abi.D2(0, 0)
    else:
        p.friction = abi.D2(1.0, _num(keys, "friction", required=True))
        p.friction_cell = abi.D2(0.0, _num(keys, "friction_cell", required=True))
        p.zetaQ_self = abi.D2(0, _num(keys, "zetaQ_self", required=True))
        p.zetaQ_inter = abi.D2(0, _num(keys, "zetaQ_inter", required=True))
        p.J_Q = abi.D2(0, _num(keys, "J_Q", required=True))
        if name == "wetpolarmodel":
            p.beta = abi.D2(0, _num(keys, "beta", required=True))
        else:
            p.beta = abi.D2(0, 0)
    return p


class HostCells:
    """rc_cell_host array plus the numpy buffers it points into."""

    def __init__(self, n: int):
        self.n = n
        self.arr = (abi.RcCellHost * max(n, 1))()
        self.buffers: List[Dict[str, np.ndarray]] = [dict() for _ in range(n)]

    def attach(self, i: int, capacity: int, names=("phi", "vx", "vy", "mu", "dx", "dy", "box_index")) -> None:
        h = self.arr[i]
        h.capacity = capacity
        for nm in names:
            if nm == "box_index":
                a = np.zeros(capacity, dtype=np.int32)
                setattr(h, nm, a.ctypes.data_as(abi.IP))
            else:
                a = np.zeros(capacity, dtype=np.float64)
                setattr(h, nm, a.ctypes.data_as(abi.DP))
            self.buffers[i][nm] = a

    def site_array(self, name: str, sizes: List[int]) -> np.ndarray:
        """Concatenate per-cell arrays (first sizes[i] values of each)."""
        return np.concatenate([self.buffers[i][name][:sizes[i]] for i in range(self.n)]) if self.n else np.zeros(0)

    def scalar(self, name: str) -> np.ndarray:
        return np.array([getattr(self.arr[i], name) for i in range(self.n)])


def make_cells(m: Monolayer, keys: Dict[str, object], seed: int) -> Tuple[HostCells, Drand48]:
    """rc_cell_host inputs for monolayer m, with the drand48 sequence the
    reference consumes while reading topology and configuration."""
    name = str(keys["interaction_type"]).strip().lower()
    rng = Drand48(seed)
    if name == "wetpolarmodel":
        for _ in range(m.n):
            rng.drand48()  # run_clock draw in read_topology
    hc = HostCells(m.n)
    for i, c in enumerate(m.cells):
        h = hc.arr[i]
        theta = float(np.float64(PI_F) * (1 - 2 * rng.drand48()))
        q00i, q01i = math.cos(2 * theta), math.sin(2 * theta)
        mod = math.sqrt(q00i * q00i + q01i * q01i)
        nx = math.sqrt((1 + q00i / mod) / 2)
        sgn = 1.0 if q01i > 0 else (-1.0 if q01i < 0 else 0.0)
        ny = sgn * math.sqrt((1 - q00i / mod) / 2)
        h.lsub_x, h.lsub_y = c.lx, c.ly
        h.offset_x, h.offset_y = c.offset
        h.corner = c.corner
        h.type = int(m.types[i]) if i < len(m.types) else 0
        h.com_x, h.com_y = c.com
        # SimBackend.cpp:276 passes the unwrapped corner through (int)
        h.unrap_x, h.unrap_y = float(int(c.unrap[0])), float(int(c.unrap[1]))
        h.q00, h.q01 = c.q00, c.q01
        h.theta_q = 0.5 * math.atan2(2 * c.q01, 2 * c.q00)
        h.theta_q_old = h.theta_q
        h.nemq_x, h.nemq_y = nx, ny
        h.nemq_old_x, h.nemq_old_y = nx, ny
        hc.attach(i, c.lx * c.ly, names=("phi",))
        hc.buffers[i]["phi"][:] = c.phi
    return hc, rng


def attach_rng(p: abi.RcParams, rng: Drand48) -> None:
    p.rng_state = rng.state
    p.rng_has_cached = rng.has_cached
    p.rng_cached = rng.cached


def read_input(path: str, overrides: Optional[Dict[str, object]] = None) -> Dict[str, str]:
    """Minimal reader of the reference's `key = value` input format
    (src/Utilities/parse_input/parse_input.cpp:117-160): `#` starts a comment,
    later keys override earlier ones, overrides apply last."""
    keys: Dict[str, str] = {}
    with open(path) as f:
        for line in f:
            line = line.split("#", 1)[0].strip()
            if not line or "=" not in line:
                continue
            k, v = line.split("=", 1)
            keys[k.strip()] = v.strip()
    for k, v in (overrides or {}).items():
        keys[k] = str(v)
    return keys


WALL_TYPES = ("square_walls", "circle_walls", "triangle_walls")


def box_walls(keys: Dict[str, object], L: int) -> Optional[np.ndarray]:
    """getWalls(k) of the box the reference's BoxFactory makes from `keys`
    (src/Boxes/BoxFactory.cpp:13-27), as L*L doubles, or None for the periodic
    SquareBox.  The masks restate SquareWalls::init (SquareWalls.cpp:23-55),
    CircleWalls::init (CircleWalls.cpp:23-45) and TriangleWalls::init
    (TriangleWalls.cpp:24-60) with their integer and double arithmetic.  A
    SquareBox with wall_slip <= 0 has every site closed (getWalls = 0 is not
    below it), which an all-zero mask reproduces."""
    import math
    kind = str(keys.get("type", "none")).strip()
    if kind not in WALL_TYPES:
        if "wall_slip" in keys and float(keys["wall_slip"]) <= 0:
            return np.zeros(L * L)
        return None
    if "lambda_wall" not in keys:
        raise ValueError("box type %s needs lambda_wall" % kind)
    lw = float(keys["lambda_wall"])
    w = np.zeros((L, L))  # [y][x]
    if kind == "square_walls":
        for y in range(L):
            for x in range(L):
                if x < lw - 1 or x > L - lw or y < lw or y > L - lw:
                    w[y, x] = 1.0
    elif kind == "circle_walls":
        h = L // 2
        for y in range(L):
            for x in range(L):
                dist = h - math.sqrt(float((h - x) * (h - x) + (h - y) * (h - y)))
                w[y, x] = 1.0 if (dist <= 0 or dist < lw) else 0.0
    else:
        w[:, :] = 1.0
        side = int(L - lw * 2)
        height = int(round(side * math.sqrt(3.0) / 2.0))
        center = L // 2
        top = L // 2 - height // 2
        for row in range(height):
            half = int((side / 2.0) * (1.0 - float(row) / height))
            y = top + row
            if 0 <= y < L:
                for x in range(center - half, min(center + half, L - 1) + 1):
                    if x >= 0:
                        w[y, x] = 0.0
    return w.reshape(-1)


def engine_inputs(keys: Dict[str, object], m: Monolayer,
                  precision: int = abi.RC_PRECISION_DOUBLE) -> Tuple[abi.RcParams, HostCells]:
    """rc_params and host cells of a monolayer as the reference's SimBackend
    would set them up from `keys` (srand48(seed), then the configuration's
    draws), with drand48's state handed to the device's noise stream."""
    p = make_params(keys, precision=precision)
    cells, rng = make_cells(m, keys, int(keys.get("seed", 1)))
    attach_rng(p, rng)
    return p, cells
