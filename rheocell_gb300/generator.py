"""Seeded synthetic monolayers in the reference's file formats.

The reference's own ``confGenerator`` (src/Managers/GeneratorManager.cpp:130-158)
writes sharp discs of radius R/2 on 30x30 patches (src/Fields/BaseField.cpp:5,
src/Fields/MultiPhaseField.cpp:149-156).  The benchmark workloads need 41x41
patches and tanh interfaces, so this module writes them directly, in the
configuration format the reference reads
(src/Backends/SimBackend.cpp:220-299) and writes
(src/Observables/Configuration.cpp:36-56):

    t = <step>
    b = <Lx> <Ly>
    LsubX LsubY CoMx CoMy offx offy corner unrapx unrapy Q00 Q01 (box_index phi)*

and the topology format ``N 1`` / ``type type ...`` (examples/topology.top).

Layout of a monolayer (all draws from ``numpy.random.default_rng(seed)``, in
this order):
  1. positions: ``rows x cols`` jittered triangular lattice,
     ``x = (c + (r % 2) / 2) * L / cols + U(-1.5, 1.5)``,
     ``y = r * L / rows + U(-1.5, 1.5)``  (one x then one y draw per cell,
     cells in row-major order), wrapped into ``[0, L)``;
  2. angles: ``theta ~ U(-pi, pi)`` per cell; polar inputs store
     ``Q00 = cos(theta), Q01 = sin(theta)``.
Each cell gets a ``patch x patch`` patch whose bottom-left corner is
``floor(CoM) - patch // 2`` with zero storage offset, and
``phi = (1 - tanh((d - R) / lam)) / 2`` with ``d`` the distance from the
centre (optionally an ellipse stretched by ``aspect`` along x).
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Dict, List, Optional

import numpy as np


@dataclasses.dataclass
class Cell:
    """One phase-field patch as stored in a configuration file."""

    lx: int
    ly: int
    com: tuple
    offset: tuple
    corner: int          # box site index of the patch's bottom-left corner
    unrap: tuple         # unwrapped corner coordinates
    q00: float
    q01: float
    box_index: np.ndarray  # int32[ly*lx], box site of each storage site
    phi: np.ndarray        # float64[ly*lx]


@dataclasses.dataclass
class Monolayer:
    L: int
    cells: List[Cell]
    types: List[int]
    step: int = 0

    @property
    def n(self) -> int:
        return len(self.cells)

    @property
    def sites(self) -> int:
        return sum(c.lx * c.ly for c in self.cells)


def lattice_shape(n: int) -> tuple:
    """Rows and columns of the lattice for n cells (square when n is)."""
    r = int(round(math.sqrt(n)))
    if r * r == n:
        return r, r
    r = max(1, int(math.floor(math.sqrt(n))))
    c = int(math.ceil(n / r))
    return r, c


def make_monolayer(L: int, n: int, seed: int, R: float = 8.0, lam: float = 2.0,
                   patch: int = 41, jitter: float = 1.5, aspect: float = 1.0,
                   types: Optional[List[int]] = None,
                   positions: Optional[np.ndarray] = None) -> Monolayer:
    """Build a seeded synthetic monolayer (see the module docstring)."""
    if patch > L:
        raise ValueError("patch side %d exceeds box side %d" % (patch, L))
    rng = np.random.default_rng(seed)
    rows, cols = lattice_shape(n)
    pos = np.zeros((n, 2))
    for i in range(n):
        r, c = divmod(i, cols)
        x = (c + 0.5 * (r % 2)) * L / cols + rng.uniform(-jitter, jitter)
        y = r * L / rows + rng.uniform(-jitter, jitter)
        pos[i] = (x % L, y % L)
    if positions is not None:
        pos = np.asarray(positions, dtype=np.float64) % L
    theta = rng.uniform(-math.pi, math.pi, size=n)
    cells = []
    half = patch // 2
    ly_idx, lx_idx = np.divmod(np.arange(patch * patch), patch)
    for i in range(n):
        cx, cy = pos[i]
        x0 = int(math.floor(cx)) - half
        y0 = int(math.floor(cy)) - half
        dx = (x0 + lx_idx) - cx
        dy = (y0 + ly_idx) - cy
        d = np.sqrt((dx / aspect) ** 2 + dy ** 2)
        phi = 0.5 * (1.0 - np.tanh((d - R) / lam))
        bx = (x0 + lx_idx) % L
        by = (y0 + ly_idx) % L
        box_index = (bx + by * L).astype(np.int32)
        corner = (x0 % L) + (y0 % L) * L
        cells.append(Cell(lx=patch, ly=patch, com=(float(cx), float(cy)), offset=(0, 0),
                          corner=int(corner), unrap=(float(x0 % L), float(y0 % L)),
                          q00=float(math.cos(theta[i])), q01=float(math.sin(theta[i])),
                          box_index=box_index, phi=phi.astype(np.float64)))
    if types is None:
        types = [0] * n
    return Monolayer(L=L, cells=cells, types=list(types))


def _fmt(v: float) -> str:
    # C++ iostream with precision(15) (default float format) == %.15g
    return "%.15g" % v


def write_conf(path: str, m: Monolayer) -> None:
    """Write the configuration file (reference text format, 15 digits)."""
    with open(path, "w") as f:
        f.write("t = %d\n" % m.step)
        f.write("b = %d %d\n" % (m.L, m.L))
        lines = []
        for c in m.cells:
            head = "%d %d %s %s %d %d %d %s %s %s %s " % (
                c.lx, c.ly, _fmt(c.com[0]), _fmt(c.com[1]), c.offset[0], c.offset[1],
                c.corner, _fmt(c.unrap[0]), _fmt(c.unrap[1]), _fmt(c.q00), _fmt(c.q01))
            body = " ".join("%d %s" % (int(k), _fmt(float(p))) for k, p in zip(c.box_index, c.phi))
            lines.append(head + body + " ")
        f.write("\n".join(lines))


def read_conf(path: str) -> Monolayer:
    """Read a configuration file in the reference text format."""
    with open(path) as f:
        t = int(f.readline().split("=")[1])
        b = f.readline().split("=")[1].split()
        L = int(float(b[0]))
        cells = []
        for line in f:
            tok = line.split()
            if not tok:
                continue
            if len(tok) < 11:
                raise ValueError("configuration line %d: %d values, a patch header needs 11" % (len(cells) + 3, len(tok)))
            lx, ly = int(tok[0]), int(tok[1])
            n = lx * ly
            if len(tok) < 11 + 2 * n:
                raise ValueError("configuration line %d too short: %d values for a %dx%d patch (%d needed)"
                                 % (len(cells) + 3, len(tok), lx, ly, 11 + 2 * n))
            vals = np.array(tok[11:11 + 2 * n], dtype=np.float64)
            cells.append(Cell(lx=lx, ly=ly, com=(float(tok[2]), float(tok[3])),
                              offset=(int(tok[4]), int(tok[5])), corner=int(tok[6]),
                              unrap=(float(tok[7]), float(tok[8])),
                              q00=float(tok[9]), q01=float(tok[10]),
                              box_index=vals[0::2].astype(np.int32), phi=vals[1::2].copy()))
    return Monolayer(L=L, cells=cells, types=[0] * len(cells), step=t)


def write_topology(path: str, m: Monolayer) -> None:
    with open(path, "w") as f:
        f.write("%d 1\n" % m.n)
        f.write(" ".join(str(t) for t in m.types) + " \n")


# Interaction parameters of the benchmark workloads.  Every key the reference
# leaves uninitialised unless set (friction, friction_cell, zetaQ_self,
# zetaQ_inter, J_Q; src/Interactions/WetModel.h:31,41 and WetModel.cpp:41-42)
# is set explicitly.
DRY_POLAR = dict(interaction_type="wetpolarmodel", friction=1, friction_cell=0,
                 zetaQ_self=0.1, zetaQ_inter=0, J_Q=0, omega=0, beta=0, gamma=0.06,
                 kappa=0.1, mu=45, **{"lambda": 2}, R=8, dt=0.1, passive_alpha=1,
                 CGtolerance=1e-8)
WET_NEMATIC = dict(interaction_type="wetmodel", friction=1, friction_cell=1,
                   zetaQ_self=0.05, zetaQ_inter=0, J_Q=0.1, omega=0, gamma=0.06,
                   kappa=0.1, mu=45, **{"lambda": 2}, R=8, dt=0.1, passive_alpha=1,
                   CGtolerance=1e-8)


def write_input(path: str, params: Dict[str, object], steps: int, seed: int = 1,
                equilibration_steps: int = 0, topology: str = "topology.top",
                conf_file: str = "start_conf.dat", extra: Optional[Dict[str, object]] = None) -> None:
    """Write an input file with the keys the reference's backend reads."""
    keys = dict(backend="CPU", sim_type="FD_CPU", seed=seed, omp_thread_num=1, box="square",
                equilibration_steps=equilibration_steps, steps=steps,
                print_conf_interval=max(1, steps), time_scale="linear",
                restart_step_counter=1, topology=topology, conf_file=conf_file,
                trajectory_file="trajectory.dat", T=0.1, max_io=1e9)
    keys.update(params)
    if extra:
        keys.update(extra)
    with open(path, "w") as f:
        for k, v in keys.items():
            f.write("%s = %s\n" % (k, v))


def write_case(directory: str, m: Monolayer, params: Dict[str, object], steps: int,
               seed: int = 1, equilibration_steps: int = 0,
               extra: Optional[Dict[str, object]] = None) -> str:
    """Write input, topology and conf for a case; returns the input path."""
    os.makedirs(directory, exist_ok=True)
    write_conf(os.path.join(directory, "start_conf.dat"), m)
    write_topology(os.path.join(directory, "topology.top"), m)
    inp = os.path.join(directory, "input")
    write_input(inp, params, steps, seed=seed, equilibration_steps=equilibration_steps, extra=extra)
    return inp


def case_keys(m: Monolayer, params: Dict[str, object], seed: int = 1,
              extra: Optional[Dict[str, object]] = None):
    """(input keys, monolayer) of a run of `m` with interaction `params`: the
    keys as strings with `seed` and the square box, and the monolayer as the
    reference reads it back from its configuration file (15-digit text)."""
    import shutil
    import tempfile
    keys = {k: str(v) for k, v in params.items()}
    keys["seed"] = str(seed)
    keys.setdefault("box", "square")
    if extra:
        keys.update({k: str(v) for k, v in extra.items()})
    d = tempfile.mkdtemp(prefix="rc_case_")
    try:
        write_conf(os.path.join(d, "conf"), m)
        m2 = read_conf(os.path.join(d, "conf"))
    finally:
        shutil.rmtree(d, ignore_errors=True)
    m2.types = list(m.types)
    return keys, m2
