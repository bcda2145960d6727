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
    # wall conditions / flow channels (eqf_set_boundaries): {"walls": {side: (kind,
    # value, rate)}, "channel": {...}}; None = the walls bitfield above
    bc: Optional[dict] = None
    # anisotropic tensor (eqf_set_tensor): (D11, D22, D12) per node in grid order
    tensor: Optional[tuple] = None

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


def stratified_sample(traps: List[Trap], k: int) -> List[int]:
    """Indices of k traps spread evenly over the batch sorted by node count (the
    smallest and the largest included); deterministic."""
    order = np.argsort([t.n_nodes for t in traps], kind="stable")
    if k >= len(traps):
        return [int(i) for i in order]
    pos = np.linspace(0, len(traps) - 1, k).round().astype(int)
    return [int(order[p]) for p in pos]


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


# --- rod cells of the agent-based model (eqf_set_rods) ----------------------------

ROD_HELD, ROD_CIRCUIT, ROD_INERT = 0, 1, 2


def rod_records(cx, cy, angle, length, W: float, H: float) -> np.ndarray:
    """eqf_rod records of freshly created cells: the first body half at the centre
    with the cell's angle, its box of half-length (L - 1)/2 and half-width 1/2 in its
    own frame (upper-left, upper-right, lower-right, lower-left), as
    cpmEcoli::cpmEcoli builds it (src/abm/cpmEcoli.cpp:100-180), and the pole centres
    of Ecoli::updatePoleCenters (src/abm/Ecoli.cpp:36-60): centre + (cos, sin) *
    (0.5 L - W/2) and centre + (cos, sin) * (-0.5 L - W/2), clamped to the trap."""
    from ._lib import rod_dtype
    cx, cy, angle, length = (np.asarray(v, dtype=np.float64).ravel() for v in
                             (cx, cy, angle, length))
    n = len(cx)
    rec = np.zeros(n, dtype=rod_dtype())
    c, s = np.cos(angle), np.sin(angle)
    rec["center"][:, 0], rec["center"][:, 1] = cx, cy
    width = 1.0
    for key, r in (("pole_a", 1.0), ("pole_b", -1.0)):
        k = r * 0.5 * length - width / 2.0
        px, py = cx + c * k, cy + s * k
        rec[key][:, 0] = np.clip(px, 0.0, W)
        rec[key][:, 1] = np.clip(py, 0.0, H)
    rec["body_pos"][:, 0], rec["body_pos"][:, 1] = cx, cy
    rec["body_rot"][:, 0], rec["body_rot"][:, 1] = c, s
    off = (length - width) * 0.5
    rad = width * 0.5
    rec["verts"] = np.stack([-off, np.full(n, rad), off, np.full(n, rad),
                             off, np.full(n, -rad), -off, np.full(n, -rad)], axis=1)
    rec["length"] = length
    return rec


@dataclass
class RodColony:
    """One trap with rod cells coupled through their footprints, one field layer per
    HSL species, each with its own D, decay and membrane rate."""
    W: float
    H: float
    npm: float
    D: List[float]
    g: List[float]
    km: List[float]
    dt: float
    steps: int
    rods: np.ndarray
    ihsl: np.ndarray  # (n_cells, n_layers) molecules
    prod: np.ndarray  # (n_cells, n_layers) nM per time unit
    mode: np.ndarray  # (n_cells, n_layers) ROD_*
    walls: int = WALL_BOTTOM

    @property
    def nx(self) -> int:
        return int(self.W * self.npm)

    @property
    def ny(self) -> int:
        return int(self.H * self.npm)

    @property
    def n_nodes(self) -> int:
        return (self.nx + 1) * (self.ny + 1)

    @property
    def n_layers(self) -> int:
        return len(self.D)

    @property
    def n_cells(self) -> int:
        return len(self.rods)

    def dof_steps(self, steps: Optional[int] = None) -> int:
        return self.n_nodes * self.n_layers * (self.steps if steps is None else steps)


def rod_colony(seed: int = 11, W: float = 100.0, H: float = 40.0, npm: float = 4.0,
               n_cells: int = 1000, steps: int = 200, dt: float = 0.05,
               len_lo: float = 1.5, len_hi: float = 4.2) -> RodColony:
    """Sender/receiver colony on two HSL layers (C4-like, C14-like): centres uniform
    2 um inside the walls, angles uniform, lengths U(len_lo, len_hi) (rods may
    overlap, as compressed cells do).  Half the cells are senders: layer 0 runs
    their circuit with production 100 nM/time; receivers run it with production 0
    (pure membrane exchange); layer 1 is held (the strain does not update it), as
    sendRecvStrain does with a second HSL.  Membrane rates 3.0 and 2.1 per time
    unit (the reference's C4/C14 values, src/eQinit.h:12-13)."""
    rng = _rng(seed)
    cx = rng.uniform(2.0, W - 2.0, size=n_cells)
    cy = rng.uniform(2.0, H - 2.0, size=n_cells)
    ang = rng.uniform(0.0, np.pi, size=n_cells)
    length = rng.uniform(len_lo, len_hi, size=n_cells)
    sender = rng.uniform(size=n_cells) < 0.5
    rods = rod_records(cx, cy, ang, length, W, H)
    nl = 2
    prod = np.zeros((n_cells, nl))
    prod[:, 0] = np.where(sender, 100.0, 0.0)
    mode = np.full((n_cells, nl), ROD_HELD, dtype=np.uint8)
    mode[:, 0] = ROD_CIRCUIT
    return RodColony(W=W, H=H, npm=npm, D=[490.0, 300.0], g=[0.01, 0.02], km=[3.0, 2.1],
                     dt=dt, steps=steps, rods=rods, ihsl=np.zeros((n_cells, nl)), prod=prod,
                     mode=mode)


# --- MICROFLUIDIC_TRAP walls (eqf_set_boundaries) -----------------------------------

BC_NEUMANN, BC_DIRICHLET, BC_ROBIN, BC_CHANNEL = 0, 1, 2, 3
SIDE_BOTTOM, SIDE_TOP, SIDE_LEFT, SIDE_RIGHT = 0, 1, 2, 3


def microfluidic_bc(trap: Trap, velocity: float = 100.0, side_channel: float = 20.0,
                    length_scaling: float = 1.0) -> dict:
    """The reference's MICROFLUIDIC_TRAP walls for a trap: flow channels on the bottom
    and top walls, Robin side walls.  Robin rates from the flow over side channels of
    length side_channel (setRobinBoundaryConditions, src/fHSL.cpp:338-356: v/(1 -
    exp(-Lv/D)) and v/(exp(Lv/D) - 1)); channel sub-steps ceil(D dt^2 / h^2) with
    h = length_scaling / npm (checkAdvectionDiffusionStability, src/main.cpp:415-430);
    wellScaling = 10 (25 / length_scaling) h (src/fHSL.cpp:45-47)."""
    D, v, dt = trap.D[0], velocity, trap.dt
    npm = trap.nx / trap.W
    h = 1.0 / npm
    if v > 1.0e-6:
        lv = side_channel * v / D
        r_left, r_right = v * (1.0 / (1.0 - np.exp(-lv))), v * (1.0 / (np.exp(lv) - 1.0))
    else:
        r_left = r_right = D / side_channel
    hs = length_scaling / npm
    substeps = int(np.ceil(dt / (hs * hs / (D * dt))))
    return {"walls": {SIDE_BOTTOM: (BC_CHANNEL, 0.0, 0.0), SIDE_TOP: (BC_CHANNEL, 0.0, 0.0),
                      SIDE_LEFT: (BC_ROBIN, 0.0, float(r_left)),
                      SIDE_RIGHT: (BC_ROBIN, 0.0, float(r_right))},
            "channel": {"velocity": v, "D": D, "rate": (float(r_left), float(r_right)),
                        "substeps": max(1, substeps),
                        "well_scaling": 10.0 * (25.0 / length_scaling) * h}}


def batched_microfluidic(seed: int = 3, n_traps: int = 512, h: float = 0.25,
                         steps: int = 200) -> List[Trap]:
    """The batched_uneven traps with the MICROFLUIDIC_TRAP walls (flow channels on
    the bottom and top walls, Robin side walls)."""
    traps = batched_uneven(seed=seed, n_traps=n_traps, h=h, steps=steps)
    for t in traps:
        t.walls = 0
        t.bc = microfluidic_bc(t)
    return traps


# --- anisotropic tensors (eqf_set_tensor) -------------------------------------------

def rotated_tensor(theta: np.ndarray, Dx: float, Dy: float):
    """D11, D22, D12 of diag(Dx, Dy) turned by theta, as eQabm's setDiffusionTensor
    forms them (src/abm/eQabm.cpp:306-325): Dx cos^2 + Dy sin^2, Dx sin^2 + Dy cos^2,
    (Dx - Dy) sin cos."""
    c, s = np.cos(theta), np.sin(theta)
    cos2t, sin2t, sincost = c * c, s * s, s * c
    return Dx * cos2t + Dy * sin2t, Dx * sin2t + Dy * cos2t, (Dx - Dy) * sincost


def batched_anisotropic(seed: int = 3, n_traps: int = 512, Dx: float = 2.0,
                        Dy: float = 0.5) -> List[Trap]:
    """The batched_uneven traps with a smoothly turning anisotropic tensor: diag(Dx, Dy)
    rotated by theta(x, y) = 0.7 sin(2 pi x / W) + 0.5 y / H."""
    traps = batched_uneven(seed=seed, n_traps=n_traps)
    for t in traps:
        y, x = np.meshgrid(np.linspace(0, t.H, t.ny + 1), np.linspace(0, t.W, t.nx + 1),
                           indexing="ij")
        theta = 0.7 * np.sin(2 * np.pi * x / t.W) + 0.5 * y / t.H
        t.tensor = tuple(v.ravel() for v in rotated_tensor(theta, Dx, Dy))
    return traps
