"""Seeded synthetic trap workloads for the quorum-sensing field step.

The reference publishes no benchmark inputs, so every workload here is synthetic:
a rectangular trap meshed with the "right" triangulation, a set of point cells with
per-cell production rates, and the physical constants of the step.  The same arrays
feed the GPU path, the oracle and the CPU baseline.  All draws come from
``numpy.random.Generator(PCG64(seed))`` in a fixed order.

Named workloads (sizes in micrometres and seconds):

* ``single_small``   40x20 um, 160x80 squares (13,041 nodes), 300 cells, s=1,
                     D=490, g=0.01, dt=0.1, 100 steps.
* ``single_large``   100x40 um, 1024x512 squares (525,825 nodes), 20,000 cells,
                     s ~ LogNormal(0, 0.5), dt=0.05, 500 steps.
* ``two_species``    the single_large mesh with two coupled species, advection
                     v = (0, -0.5*y/40) um/s, 300 steps.
* ``batched_uneven`` 512 traps, nx ~ U{64..1024}, ny ~ U{32..512}, h=0.25 um,
                     round(0.02*nx*ny) cells each, 200 steps of dt=0.1.

Walls: the open long edge y=0 is Dirichlet c=0; the other three walls are zero
flux.  This is the reference's THREEWALLED trap with DIRICHLET_0 walls
(src/fHSL.h:461-466, src/fHSL.cpp:557-569).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# wall bits (one per rectangle edge); a set bit makes that edge Dirichlet c=0
WALL_BOTTOM = 1  # y = 0
WALL_TOP = 2     # y = H
WALL_LEFT = 4    # x = 0
WALL_RIGHT = 8   # x = W

# trapType -> Dirichlet walls, as decoded by fenicsInterface::createHSL
# (src/fHSL.cpp:557-569 with the SubDomains of src/fHSL.h:456-504)
TRAP_TYPE_WALLS = {
    "NOWALLED": WALL_BOTTOM | WALL_TOP | WALL_LEFT | WALL_RIGHT,
    "THREEWALLED": WALL_BOTTOM,
    "TWOWALLED": WALL_BOTTOM | WALL_TOP,
    "ONEWALLED": WALL_LEFT | WALL_RIGHT | WALL_BOTTOM,
}


@dataclass
class Trap:
    """One trap: mesh, physics and cells for one or two species."""
    W: float
    H: float
    nx: int
    ny: int
    D: List[float]
    g: List[float]
    dt: float
    steps: int
    walls: int = WALL_BOTTOM
    cell_xy: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))
    cell_s: np.ndarray = field(default_factory=lambda: np.zeros((0,)))
    # two-species coupling (None for single species)
    cell_kind: Optional[np.ndarray] = None  # 1 = sender, 0 = receiver
    adv_u: float = 0.0  # v = (0, -adv_u * y / adv_len)
    adv_len: float = 40.0

    @property
    def n_nodes(self) -> int:
        return (self.nx + 1) * (self.ny + 1)

    @property
    def n_species(self) -> int:
        return len(self.D)

    @property
    def n_cells(self) -> int:
        return int(self.cell_xy.shape[0])

    def dof_steps(self, steps: Optional[int] = None) -> int:
        return self.n_nodes * self.n_species * (self.steps if steps is None else steps)


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _uniform_cells(rng, n, W, H, inset=0.5):
    x = rng.uniform(inset, W - inset, size=n)
    y = rng.uniform(inset, H - inset, size=n)
    return np.stack([x, y], axis=1)


def single_small(seed: int = 0) -> Trap:
    rng = _rng(seed)
    xy = _uniform_cells(rng, 300, 40.0, 20.0)
    return Trap(W=40.0, H=20.0, nx=160, ny=80, D=[490.0], g=[0.01], dt=0.1, steps=100,
                cell_xy=xy, cell_s=np.ones(300))


def single_large(seed: int = 1) -> Trap:
    rng = _rng(seed)
    n = 20000
    xy = _uniform_cells(rng, n, 100.0, 40.0)
    s = rng.lognormal(0.0, 0.5, size=n)
    return Trap(W=100.0, H=40.0, nx=1024, ny=512, D=[490.0], g=[0.01], dt=0.05, steps=500,
                cell_xy=xy, cell_s=s)


def two_species(seed: int = 2) -> Trap:
    rng = _rng(seed)
    n = 20000
    xy = _uniform_cells(rng, n, 100.0, 40.0)
    kind = (rng.uniform(size=n) < 0.5).astype(np.int32)
    return Trap(W=100.0, H=40.0, nx=1024, ny=512, D=[490.0, 300.0], g=[0.01, 0.02],
                dt=0.05, steps=300, cell_xy=xy, cell_s=np.ones(n), cell_kind=kind,
                adv_u=0.5, adv_len=40.0)


def batched_uneven(seed: int = 3, n_traps: int = 512, h: float = 0.25,
                   steps: int = 200) -> List[Trap]:
    rng = _rng(seed)
    nxs = rng.integers(64, 1025, size=n_traps)
    nys = rng.integers(32, 513, size=n_traps)
    traps = []
    for nx, ny in zip(nxs, nys):
        W, H = float(nx) * h, float(ny) * h
        n = int(round(0.02 * nx * ny))
        xy = _uniform_cells(rng, n, W, H)
        s = rng.lognormal(0.0, 0.5, size=n)
        traps.append(Trap(W=W, H=H, nx=int(nx), ny=int(ny), D=[490.0], g=[0.01], dt=0.1,
                          steps=steps, cell_xy=xy, cell_s=s))
    return traps


def scaled(trap: Trap, nx: int, ny: int, n_cells: Optional[int] = None,
           seed: int = 7) -> Trap:
    """Same physics and domain as ``trap`` on a coarser mesh with fresh cells."""
    rng = _rng(seed)
    n = trap.n_cells if n_cells is None else n_cells
    xy = _uniform_cells(rng, n, trap.W, trap.H)
    s = rng.lognormal(0.0, 0.5, size=n)
    kind = None
    if trap.cell_kind is not None:
        kind = (rng.uniform(size=n) < 0.5).astype(np.int32)
        s = np.ones(n)
    return Trap(W=trap.W, H=trap.H, nx=nx, ny=ny, D=list(trap.D), g=list(trap.g),
                dt=trap.dt, steps=trap.steps, walls=trap.walls, cell_xy=xy, cell_s=s,
                cell_kind=kind, adv_u=trap.adv_u, adv_len=trap.adv_len)


WORKLOADS = {
    "single_small": single_small,
    "single_large": single_large,
    "two_species": two_species,
}
