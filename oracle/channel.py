"""FP64 CPU restatement of the reference's MICROFLUIDIC_TRAP boundary mode (the oracle
for eqf_set_boundaries).

TEST INFRASTRUCTURE ONLY.  Nothing in the product path imports this module; only
tests, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use it.

* Flow channel (fenicsChannel, src/fHSL.h:240-330): the P1 form of
  fenics/AdvectionDiffusion.ufl on the interval [0, W] with nx cells,
      F = w (u - u0) dx + dt D w' (u0 + u)'/2 dx + dt v ((u0 + u)/2)' w dx
          + dt r1 ((u0 + u)/2 - s1) w ds(1) + dt r2 ((u0 + u)/2 - s2) w ds(2),
  ds(1) the end x = 0 and ds(2) the end x = W (src/fHSL.cpp:412-420), s1 = s2 = 0
  (setRobinBoundaryConditions, src/fHSL.cpp:331-364).  Element matrices as the
  generated kernels compute them (fenics/AdvectionDiffusion.h:2226-2680; pinned by
  ``oracle/ref_kernels.py``), solved with SuperLU.
* Trap walls (createHSL, src/fHSL.cpp:446-540): Dirichlet (a value, or the channel's
  values on the bottom and top walls: DirichletBC(V, channel u, wall)), Robin
  (hslD's ds(1)/ds(2) terms) or Neumann; the DirichletBCs are applied left, right,
  top, bottom, so the bottom and top walls win at the corners.
* The step (fenicsInterface::stepDiffusion, src/fHSL.cpp:98-152): the trap solve
  with the channels' current values, then computeBoundaryFlux (54-95) -- per
  column j, gradc = (u[1][j] - u[0][j])/h at the bottom and (u[ny-1][j] - u[ny][j])/h
  at the top, flux = h*(dt*D*gradc)/wellScaling -- and `substeps` channel solves of
  dt/substeps, each after adding flux/substeps to every channel node.
"""
from __future__ import annotations

from typing import Dict, Optional, Sequence

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import hsld

NEUMANN, DIRICHLET, ROBIN, CHANNEL, WELL = 0, 1, 2, 3, 4
BOTTOM, TOP, LEFT, RIGHT = 0, 1, 2, 3
SIDE_BITS = {BOTTOM: hsld.WALL_BOTTOM, TOP: hsld.WALL_TOP, LEFT: hsld.WALL_LEFT,
             RIGHT: hsld.WALL_RIGHT}


def element_a(h: float, dt: float, D: float, v: float) -> np.ndarray:
    """Bilinear cell tensor of AdvectionDiffusion (fenics/AdvectionDiffusion.h:2244-2290):
    h/3, h/6 mass; 0.5 dt D / h stiffness; 0.25 dt v advection."""
    sp5 = abs(h)
    sp6 = 0.5 * (1.0 / h) * (dt * D * (1.0 / h)) * sp5
    sp7 = 0.5 * (1.0 / h) * (dt * v) * sp5
    return np.array([[0.3333333333333334 * sp5 - 0.5 * sp7 + sp6,
                      0.1666666666666667 * sp5 + 0.5 * sp7 - sp6],
                     [0.1666666666666667 * sp5 - 0.5 * sp7 - sp6,
                      0.3333333333333334 * sp5 + 0.5 * sp7 + sp6]])


def element_b(h: float, dt: float, D: float, v: float) -> np.ndarray:
    """The u0 part of the linear cell tensor: L = element_b @ u0 (mass minus the
    explicit half of stiffness and advection)."""
    m = np.array([[h / 3.0, h / 6.0], [h / 6.0, h / 3.0]])
    k = np.array([[1.0, -1.0], [-1.0, 1.0]]) / h
    c = np.array([[-0.5, 0.5], [-0.5, 0.5]])
    return m - 0.5 * dt * (D * k + v * c)


class Channel:
    """One flow channel with nx cells on [0, W]."""

    def __init__(self, W: float, nx: int, D: float, v: float, dt: float, substeps: int,
                 r_left: float, r_right: float):
        self.n = nx + 1
        self.substeps = int(substeps)
        h = W / nx
        dtc = dt / self.substeps
        ae, be = element_a(h, dtc, D, v), element_b(h, dtc, D, v)
        rows, cols, va, vb = [], [], [], []
        for e in range(nx):
            for r in range(2):
                for q in range(2):
                    rows.append(e + r)
                    cols.append(e + q)
                    va.append(ae[r, q])
                    vb.append(be[r, q])
        A = sp.coo_matrix((va, (rows, cols)), shape=(self.n, self.n)).tolil()
        B = sp.coo_matrix((vb, (rows, cols)), shape=(self.n, self.n)).tolil()
        # Robin ends: dt r (0.5 (u0 + u) - 0) w at x = 0 (r_left) and x = W (r_right)
        A[0, 0] += 0.5 * dtc * r_left
        B[0, 0] -= 0.5 * dtc * r_left
        A[self.n - 1, self.n - 1] += 0.5 * dtc * r_right
        B[self.n - 1, self.n - 1] -= 0.5 * dtc * r_right
        self.A = A.tocsc()
        self.B = B.tocsr()
        self.lu = spla.splu(self.A)

    def step(self, c: np.ndarray, flux: np.ndarray) -> np.ndarray:
        c = np.array(c, dtype=np.float64, copy=True)
        for _ in range(self.substeps):
            c = c + flux / float(self.substeps)
            c = self.lu.solve(self.B @ c)
        return c


def robin_rates(v: float, D: float, len_left: float, len_right: float):
    """Robin rates of the trap's / channel's left and right ends from the flow
    (setRobinBoundaryConditions, src/fHSL.cpp:338-356)."""
    if v > 1.0e-6:
        lvdl, lvdr = len_left * v / D, len_right * v / D
        return v * (1.0 / (1.0 - np.exp(-lvdl))), v * (1.0 / (np.exp(lvdr) - 1.0))
    return D / len_left, D / len_right


class MicrofluidicTrap:
    """One trap with wall conditions and (optionally) flow channels on its bottom and
    top walls.  walls[side] = (kind, value, rate) by BOTTOM, TOP, LEFT, RIGHT."""

    def __init__(self, W, H, nx, ny, D, dt, g, walls: Dict[int, tuple],
                 channel: Optional[dict] = None, well: Optional[tuple] = None):
        self.W, self.H, self.nx, self.ny = W, H, nx, ny
        # boundary well (Simulation::computeBoundaryWell, src/simulation.cpp:581-604):
        # (well_scaling, decay_rate); its concentration drives WELL walls
        self.well = well
        self.well_c = 0.0
        self.well_under = 0
        self.D, self.dt = float(D), float(dt)
        self.walls = walls
        bits = 0
        robin = {}
        for side, (kind, value, rate) in walls.items():
            if kind in (DIRICHLET, CHANNEL, WELL):
                bits |= SIDE_BITS[side]
            elif kind == ROBIN:
                robin[SIDE_BITS[side]] = (rate, value)
        self.trap = hsld.HsldOracle(W, H, nx, ny, D, dt, g, bits, robin=robin or None)
        self.mesh = self.trap.mesh
        self.channels = {}
        self.channel = channel
        if channel is not None:
            for side in (BOTTOM, TOP):
                if walls.get(side, (NEUMANN, 0, 0))[0] == CHANNEL:
                    self.channels[side] = np.zeros(nx + 1)
            self.ch = Channel(W, nx, channel["D"], channel["velocity"], dt, channel["substeps"],
                              channel["rate"][0], channel["rate"][1])

    def dirichlet_values(self) -> np.ndarray:
        nx, ny = self.nx, self.ny
        dv = np.zeros((ny + 1, nx + 1))
        for side in (LEFT, RIGHT, TOP, BOTTOM):  # createHSL's order: the last wins
            kind, value, _ = self.walls.get(side, (NEUMANN, 0.0, 0.0))
            if kind == DIRICHLET:
                vals = value
            elif kind == CHANNEL:
                vals = self.channels[side]
            elif kind == WELL:
                vals = self.well_c
            else:
                continue
            if side == BOTTOM:
                dv[0, :] = vals
            elif side == TOP:
                dv[ny, :] = vals
            elif side == LEFT:
                dv[:, 0] = vals
            else:
                dv[:, nx] = vals
        return dv.ravel()

    def step(self, u: np.ndarray, F: Optional[np.ndarray] = None) -> np.ndarray:
        u = self.trap.step(u, F, self.dirichlet_values())
        if self.channels:
            U = u.reshape(self.ny + 1, self.nx + 1)
            h = self.H / self.ny
            ch = self.channel
            for side, c in self.channels.items():
                if side == BOTTOM:
                    gradc = (U[1, :] - U[0, :]) / h
                else:
                    gradc = (U[self.ny - 1, :] - U[self.ny, :]) / h
                flux = h * (self.dt * self.D * gradc) / ch["well_scaling"]
                self.channels[side] = self.ch.step(c, flux)
        if self.well is not None:
            scale, decay = self.well
            flux = self.D * self.dt * hsld.boundary_flux_integral(self.mesh, u)
            c = self.well_c + flux / scale
            c -= self.dt * decay * c
            if c < 0.0:
                c = 0.0
                self.well_under += 1
            self.well_c = c
        return u
