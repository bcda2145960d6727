"""CPU restatement of the reference's rod-cell coupling (the oracle for eqf_set_rods).

TEST INFRASTRUCTURE ONLY.  Nothing in the product path imports this module; only
tests, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use it, and only
as the checker / the timed CPU baseline.

It follows eQ's per-cell loop eQabm::updateCells (src/abm/eQabm.cpp:234-390)
operation by operation, in plain Python floats (IEEE double, every operation
rounded on its own, as the reference's C++ evaluates them without contraction):

* findInteriorPoints (eQabm.cpp:268-304): lattice indices of the two pole centres
  by eQ::data::ij_from_xy (src/eQ.h:118-129, C ``round``), the bounding rectangle
  widened by nodesToEdge = round(npm * W/2) (eQabm.cpp:75) and clamped to the
  lattice, every lattice point of it (rows i ascending, columns j within a row)
  tested with cpmEcoli::pointIsInCell (src/abm/cpmEcoli.cpp:313-328) at
  eQ::data::xy_from_ij (src/eQ.h:114-117); the centre node if none is inside.
* pointIsInCell transforms the point into the frame of the cell's first body half
  with chipmunk's cpBodyWorldToLocal -- chipmunk 7.0.1 (cloned by the reference's
  eQsetup1.sh:3-6, not vendored): the rigid inverse of the body transform
  [c -s px; s c py] (centre of gravity at the body position, as eQ's shapes carry
  no mass), point -> ((c*x + s*y) + (-s*py - px*c), (-s*x + c*y) + (px*s - c*py)) --
  and requires all four cross(edge_k, p - v_{k+1}) < 0 with the edges of
  cpmEcoli::computeCellBoudaryEdges (cpmEcoli.cpp:71-76).
* readHSL (eQabm.cpp:326-337): sum of the field over the footprint in footprint
  order, from 0.0, divided by the point count.
* the strain's membrane exchange: Strain::computeConcentrations (src/Strain.h:281-318)
  converts iHSL from molecules to nM and forms dHSL = dt*(k_m*(iHSL - eHSL));
  sendRecvStrain::computeProteins (src/Strain.cpp:10-73) sets deltaHSL = dt*alpha -
  dHSL for the sender's species, -dHSL for the receiver's, 0 for the others, and
  returns dHSL; pushConcentrations (src/Strain.h:319-345) adds deltaHSL, clamps at 0
  and converts back to molecules.  Strains without an HSL circuit return zeros
  (aspectRatioInvasionStrain::computeProteins, src/Strain.cpp:75-83).
* writeHSL (eQabm.cpp:338-359): dHSL -> molecules (eQ::Cell::nanoMolarToMoleculeNumber)
  -> / extracellular volume fraction -> * npm * npm -> / point count, added to
  every footprint node, with the eQ::Cell volume model (src/eQcell.h:42-97).

Cells are processed strictly one after the other, as the reference does, so a cell
sees the deposits of earlier cells on shared nodes.  Modes per cell and layer:
HELD (0), CIRCUIT (1), INERT (2), as EQF_ROD_* in include/eqfield.h.
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np

HELD, CIRCUIT, INERT = 0, 1, 2

# eQ::Cell (src/eQcell.h:42-59), the same expressions
CELL_WIDTH = 1.0
POLE_RADIUS = CELL_WIDTH / 2.0
CYL = math.pi * (POLE_RADIUS * POLE_RADIUS)
POLE = 4.0 / 3.0 * math.pi * (POLE_RADIUS * POLE_RADIUS * POLE_RADIUS)
NM_PER_MOLECULE = 1.0 / 0.602


def c_round(x: float) -> int:
    """C round() for x >= 0 (half away from zero)."""
    f = math.floor(x)
    return int(f) + (1 if x - f >= 0.5 else 0)


def cell_volume(L: float) -> float:
    """eQ::Cell::computeCellVolumeActual (src/eQcell.h:61-64)."""
    return (L - CELL_WIDTH) * CYL + POLE


def nm_per_molecule(L: float) -> float:
    """moleculeNumberToNanoMolar(1.0, L) (src/eQcell.h:73-76)."""
    return (1.0 / cell_volume(L)) * NM_PER_MOLECULE


def nm_to_molecules(nm: float, L: float) -> float:
    """nanoMolarToMoleculeNumber (src/eQcell.h:77-80)."""
    return nm / NM_PER_MOLECULE * cell_volume(L)


def extracellular_fraction(L: float) -> float:
    """computeExtraCellularVolumeFraction (src/eQcell.h:82-93)."""
    return 1.0 - cell_volume(L) / (L * 1.0 * 1.0)


def world_to_local(rod, x: float, y: float) -> Tuple[float, float]:
    """chipmunk 7.0.1 cpBodyWorldToLocal for the body at body_pos, rotation body_rot."""
    c, s = float(rod["body_rot"][0]), float(rod["body_rot"][1])
    px, py = float(rod["body_pos"][0]), float(rod["body_pos"][1])
    tx = (-s) * py - px * c
    ty = px * s - c * py
    return (c * x + s * y) + tx, ((-s) * x + c * y) + ty


def point_in_cell(rod, x: float, y: float) -> bool:
    """cpmEcoli::pointIsInCell (src/abm/cpmEcoli.cpp:313-328)."""
    lx, ly = world_to_local(rod, x, y)
    v = [float(t) for t in rod["verts"]]
    for k in range(4):
        n = (k + 1) % 4
        ex, ey = v[2 * n] - v[2 * k], v[2 * n + 1] - v[2 * k + 1]
        px, py = lx - v[2 * n], ly - v[2 * n + 1]
        if not (ex * py - ey * px < 0.0):
            return False
    return True


def footprint(rod, npm: float, nx: int, ny: int) -> List[Tuple[int, int]]:
    """findInteriorPoints (src/abm/eQabm.cpp:268-304): (i, j) pairs in search order."""
    nte = c_round(npm * CELL_WIDTH / 2.0)
    ai, aj = c_round(float(rod["pole_a"][1]) * npm), c_round(float(rod["pole_a"][0]) * npm)
    bi, bj = c_round(float(rod["pole_b"][1]) * npm), c_round(float(rod["pole_b"][0]) * npm)
    i1, i2 = (bi, ai) if ai > bi else (ai, bi)
    j1, j2 = (bj, aj) if aj > bj else (aj, bj)
    i1 = i1 - nte if i1 >= nte else 0
    j1 = j1 - nte if j1 >= nte else 0
    i2 = ny if i2 + nte >= ny else i2 + nte
    j2 = nx if j2 + nte >= nx else j2 + nte
    pts = []
    for i in range(i1, i2 + 1):
        for j in range(j1, j2 + 1):
            if point_in_cell(rod, j / npm, i / npm):
                pts.append((i, j))
    if not pts:
        pts.append((c_round(float(rod["center"][1]) * npm), c_round(float(rod["center"][0]) * npm)))
    return pts


def exchange(fields: Sequence[np.ndarray], rods, ihsl: np.ndarray, prod: np.ndarray,
             mode: np.ndarray, npm: float, dt: float, km: Sequence[float]):
    """One pass of the cell loop over all cells, in order.

    fields: per layer a (ny+1, nx+1) float64 grid, updated in place (the deposits).
    ihsl, prod, mode: (n_cells, n_layers).  Returns (ihsl_new, ehsl, points)."""
    ny, nx = fields[0].shape[0] - 1, fields[0].shape[1] - 1
    n, nl = ihsl.shape
    ihsl = np.array(ihsl, dtype=np.float64, copy=True)
    ehsl = np.zeros((n, nl))
    points = np.zeros(n, dtype=np.int32)
    for c in range(n):
        rod = rods[c]
        pts = footprint(rod, npm, nx, ny)
        K = len(pts)
        points[c] = K
        L = float(rod["length"])
        V = cell_volume(L)
        nmpm = (1.0 / V) * NM_PER_MOLECULE
        ecf = 1.0 - V / (L * 1.0 * 1.0)
        for l in range(nl):
            u = fields[l]
            acc = 0.0
            for (i, j) in pts:
                acc += float(u[i, j])
            e = acc / float(K)
            ehsl[c, l] = e
            md = int(mode[c, l])
            if md == INERT:
                continue
            inm = float(ihsl[c, l]) * nmpm
            dH = dt * (float(km[l]) * (inm - e))
            delta = dt * float(prod[c, l]) - dH if md == CIRCUIT else 0.0
            inew = inm + delta
            if inew < 0.0:
                inew = 0.0
            ihsl[c, l] = inew / nmpm
            number = dH / NM_PER_MOLECULE * V
            per_um2 = number / ecf
            d = per_um2 * npm * npm / float(K)
            for (i, j) in pts:
                u[i, j] = float(u[i, j]) + d
    return ihsl, ehsl, points
