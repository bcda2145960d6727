"""The reference's own rod-cell coupling code, compiled from its sources, for pinning
the rod oracle (oracle/rods.py).

TEST INFRASTRUCTURE ONLY.  eQ couples its rod cells to the HSL field in
eQabm::updateCells (src/abm/eQabm.cpp:234-390) through three lambdas and a few
helpers that need no FEniCS, MPI or JSON.  This recipe slices, where they lie,

  * the lambdas findInteriorPoints, readHSL and writeHSL (src/abm/eQabm.cpp:268-359),
  * cpmEcoli::computeCellBoudaryEdges and cpmEcoli::pointIsInCell
    (src/abm/cpmEcoli.cpp:71-81, 313-340),
  * eQ::data::xy_from_ij / ij_from_xy (src/eQ.h:114-129),
  * eQ::Cell's constants and volume / unit conversions (src/eQcell.h:40-97),
  * Strain::computeConcentrations and Strain::pushConcentrations (src/Strain.h:281-345),

into oracle/_ref/ (git-ignored; nothing of the reference is committed), and compiles
them with g++ (no contraction of multiply-adds) against stubs written here:

  * chipmunk 7.0.1's cpVect arithmetic, the body transform and cpBodyWorldToLocal,
    restated from chipmunk's published source (the reference clones chipmunk at
    setup, eQsetup1.sh:3-6; it is not vendored),
  * minimal holders for the cell, its chipmunk model, the strain and the grids,
  * a driver that runs the per-cell sequence of eQabm::updateCells
    (eQabm.cpp:255-390: footprint, readHSL for every layer, computeProteins,
    writeHSL for every layer) over the cells in order, where computeProteins
    restates the two HSL lines of sendRecvStrain::computeProteins
    (src/Strain.cpp:38-45 sender, 63 receiver) and the all-zero return of strains
    without an HSL circuit (src/Strain.cpp:75-83).
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
from typing import List, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_DIR, "librods_ref.so")
# the reference checkout: EQ_REFERENCE_ROOT, else a "reference" directory beside the
# repository
REFERENCE = os.environ.get("EQ_REFERENCE_ROOT",
                           os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

STUBS = r'''
// Stand-ins for what the sliced reference code needs (not reference code).
#pragma once
#include <cmath>
#include <cstddef>
#include <iostream>
#include <memory>
#include <queue>
#include <utility>
#include <vector>

// chipmunk 7.0.1 subset, restated from its published source
typedef double cpFloat;
struct cpVect { cpFloat x, y; };
static inline cpVect cpv(const cpFloat x, const cpFloat y) { cpVect v = {x, y}; return v; }
static inline cpVect operator-(const cpVect a, const cpVect b) { return cpv(a.x - b.x, a.y - b.y); }
static inline cpFloat cpvcross(const cpVect a, const cpVect b) { return a.x * b.y - a.y * b.x; }
struct cpTransform { cpFloat a, b, c, d, tx, ty; };
static inline cpTransform cpTransformNewTranspose(cpFloat a, cpFloat c, cpFloat tx, cpFloat b,
                                                  cpFloat d, cpFloat ty) {
  cpTransform t = {a, b, c, d, tx, ty};
  return t;
}
static inline cpTransform cpTransformRigidInverse(cpTransform t) {
  return cpTransformNewTranspose(t.d, -t.c, (t.c * t.ty - t.tx * t.d),
                                 -t.b, t.a, (t.tx * t.b - t.a * t.ty));
}
static inline cpVect cpTransformPoint(cpTransform t, cpVect p) {
  return cpv(t.a * p.x + t.c * p.y + t.tx, t.b * p.x + t.d * p.y + t.ty);
}
struct cpBody { cpVect cog; cpTransform transform; };
// body transform from position p and rotation rot = (cos a, sin a) (cpBody.c SetTransform)
static inline void stubSetTransform(cpBody* body, cpVect p, cpVect rot) {
  cpVect c = body->cog;
  body->transform = cpTransformNewTranspose(rot.x, -rot.y, p.x - (c.x * rot.x - c.y * rot.y),
                                            rot.y, rot.x, p.y - (c.x * rot.y + c.y * rot.x));
}
static inline cpVect cpBodyWorldToLocal(const cpBody* body, const cpVect point) {
  return cpTransformPoint(cpTransformRigidInverse(body->transform), point);
}

namespace eQ {
using nodeType = size_t;
using nodePoint = std::pair<nodeType, nodeType>;
template <class T>
struct gridFunction {  // (i, j) -> value; here the identity DOF map j + i*nodesWide
  size_t nodesHigh, nodesWide;
  std::vector<T> v;
  gridFunction(size_t h, size_t w) : nodesHigh(h), nodesWide(w), v(h * w) {}
  T& operator[](const nodePoint& p) { return v[p.second + p.first * nodesWide]; }
};
struct data {
#include "eq_data.inc"
};
struct Cell {
#include "eq_cell.inc"
};
}  // namespace eQ

class cpmEcoli {
 public:
  cpBody body;
  cpBody* bodyA = &body;
  cpVect vertsA[4];
  cpVect edges[4];
  void computeCellBoudaryEdges();
  bool pointIsInCell(std::pair<double, double> point);
};

struct CellStub {
  std::pair<double, double> polePositionA, polePositionB;
  double cx, cy, length;
  std::shared_ptr<cpmEcoli> cpmCell;
  double getCenter_x() { return cx; }
  double getCenter_y() { return cy; }
  double getLengthMicrons() { return length; }
};

struct StrainStub {
  static constexpr int NUM_CONCENTRATIONS = 1;
  struct { double dt; } params;
  double conc[NUM_CONCENTRATIONS] = {0.0}, delta[NUM_CONCENTRATIONS] = {0.0};
  std::vector<double> iHSL, tHSL, dHSL, deltaHSL, iPROTEIN, tPROTEIN, deltaPROTEIN;
  std::vector<std::queue<double>> HSL_tau, PROTEIN_tau;
  double nanoMolarPerMolecule = 0.0;
#include "strain.inc"
};
'''

HARNESS = r'''
#include "stubs.h"
#include "cpm.inc"

using HSLdata = std::vector<double>;
using HSLsolution = std::shared_ptr<HSLdata>;
using HSLgrid = std::shared_ptr<eQ::gridFunction<eQ::nodeType>>;

// rods: 20 doubles per cell, the layout of eqf_rod (include/eqfield.h)
extern "C" int ref_rod_exchange(int nx, int ny, double npm, double dt, const double* km, int nl,
                                int n, const double* rods, const double* ihsl, const double* prod,
                                const unsigned char* mode, double* fields, double* ihsl_out,
                                double* ehsl_out, int* points_out) {
  // eQabm's lattice and search widening (eQabm.cpp:27-31, 75)
  const double nodesPerMicron = npm;
  const size_t nodesHigh = (size_t)ny + 1, nodesWide = (size_t)nx + 1;
  const size_t nodesToEdge =
      size_t(round(nodesPerMicron * eQ::Cell::DEFAULT_CELL_WIDTH_MICRONS / 2.0));
  std::vector<HSLsolution> hslSolutionVector;
  std::vector<HSLgrid> dofLookupTable;
  for (int l = 0; l < nl; ++l) {
    hslSolutionVector.push_back(std::make_shared<HSLdata>(
        fields + (size_t)l * nodesHigh * nodesWide, fields + (size_t)(l + 1) * nodesHigh * nodesWide));
    auto g = std::make_shared<eQ::gridFunction<eQ::nodeType>>(nodesHigh, nodesWide);
    for (size_t k = 0; k < nodesHigh * nodesWide; ++k) g->v[k] = k;
    dofLookupTable.push_back(g);
  }
  std::vector<double> membraneDiffusionRates(km, km + nl);
  for (int c = 0; c < n; ++c) {
    const double* r = rods + 20 * (size_t)c;
    auto thisCell = std::make_shared<CellStub>();
    thisCell->cx = r[0];
    thisCell->cy = r[1];
    thisCell->polePositionA = std::make_pair(r[2], r[3]);
    thisCell->polePositionB = std::make_pair(r[4], r[5]);
    thisCell->cpmCell = std::make_shared<cpmEcoli>();
    thisCell->cpmCell->body.cog = cpv(0.0, 0.0);
    stubSetTransform(&thisCell->cpmCell->body, cpv(r[6], r[7]), cpv(r[8], r[9]));
    for (int v = 0; v < 4; ++v) thisCell->cpmCell->vertsA[v] = cpv(r[10 + 2 * v], r[11 + 2 * v]);
    thisCell->cpmCell->computeCellBoudaryEdges();
    thisCell->length = r[18];
    double cellLength = thisCell->getLengthMicrons();
    std::vector<eQ::nodePoint> cellPoints;
#include "lambdas.inc"
    findInteriorPoints(nodesPerMicron, cellPoints);
    std::vector<double> hslData;
    for (size_t i(0); i < hslSolutionVector.size(); i++)
      hslData.push_back(readHSL(hslSolutionVector[i], dofLookupTable[i], cellPoints));
    // computeProteins of the cell's strain
    std::vector<double> deltaHSL(nl, 0.0);
    bool inert = true;
    for (int l = 0; l < nl; ++l) inert = inert && mode[c * nl + l] == 2;
    StrainStub strain;
    strain.params.dt = dt;
    strain.iHSL.assign(ihsl + (size_t)c * nl, ihsl + (size_t)(c + 1) * nl);
    strain.tHSL.assign(nl, 0.0);
    strain.dHSL.assign(nl, 0.0);
    strain.deltaHSL.assign(nl, 0.0);
    std::queue<double> q;
    q.push(0.0);
    strain.HSL_tau.assign(nl, q);
    if (!inert) {
      strain.computeConcentrations(hslData, membraneDiffusionRates, cellLength);
      for (int l = 0; l < nl; ++l)
        if (mode[c * nl + l] == 1)
          strain.deltaHSL[l] = strain.params.dt * (prod[c * nl + l]) - strain.dHSL[l];
      strain.pushConcentrations();
      deltaHSL = strain.dHSL;
    }
    for (size_t i(0); i < hslSolutionVector.size(); i++)
      writeHSL(deltaHSL[i], hslSolutionVector[i], dofLookupTable[i], cellPoints);
    for (int l = 0; l < nl; ++l) {
      ihsl_out[c * nl + l] = strain.iHSL[l];
      ehsl_out[c * nl + l] = hslData[l];
    }
    points_out[c] = (int)cellPoints.size();
  }
  for (int l = 0; l < nl; ++l)
    std::copy(hslSolutionVector[l]->begin(), hslSolutionVector[l]->end(),
              fields + (size_t)l * nodesHigh * nodesWide);
  return 0;
}
'''


def _read(rel: str) -> List[str]:
    with open(os.path.join(REFERENCE, rel)) as f:
        return f.read().splitlines()


def _brace_block(lines: List[str], start: int) -> List[str]:
    """Lines from `start` to the line closing the first brace opened there (braces in
    // comments ignored)."""
    depth, opened = 0, False
    for k in range(start, len(lines)):
        code = lines[k].split("//")[0]
        depth += code.count("{") - code.count("}")
        opened = opened or "{" in code
        if opened and depth == 0:
            return lines[start:k + 1]
    raise ValueError("unbalanced block")


def _find(lines: List[str], pattern: str) -> int:
    return next(i for i, ln in enumerate(lines) if re.search(pattern, ln))


def slices() -> dict:
    """The reference text the harness compiles, by include file name."""
    eq = _read("src/eQ.h")
    a = _find(eq, r"static inline std::pair<double, double> xy_from_ij")
    b = _find(eq, r"static inline size_t index_from_ij")
    cell = _read("src/eQcell.h")
    c0 = _find(cell, r"static constexpr double\s+DEFAULT_CELL_MASS\b")
    c1 = next(i for i in range(c0, len(cell)) if cell[i].strip() == "protected:")
    cpm = _read("src/abm/cpmEcoli.cpp")
    e0 = _find(cpm, r"^void cpmEcoli::computeCellBoudaryEdges\(\)")
    p0 = _find(cpm, r"^bool cpmEcoli::pointIsInCell\(")
    strain = _read("src/Strain.h")
    s0 = _find(strain, r"void computeConcentrations\(const std::vector<double> &eHSL")
    s1 = _find(strain, r"void pushConcentrations\(\)")
    abm = _read("src/abm/eQabm.cpp")
    l0 = _find(abm, r"auto findInteriorPoints = \[&\]")
    l1 = _find(abm, r"auto readHSL = \[&\]")
    l2 = _find(abm, r"auto writeHSL = \[&\]")
    return {
        "eq_data.inc": "\n".join(eq[a:b]),
        "eq_cell.inc": "\n".join(cell[c0:c1]),
        "cpm.inc": "\n".join(_brace_block(cpm, e0) + [""] + _brace_block(cpm, p0)),
        "strain.inc": "\n".join(_brace_block(strain, s0) + [""] + _brace_block(strain, s1)),
        "lambdas.inc": "\n".join(_brace_block(abm, l0) + _brace_block(abm, l1) +
                                 _brace_block(abm, l2)),
    }


def available() -> bool:
    return os.path.exists(os.path.join(REFERENCE, "src", "abm", "eQabm.cpp"))


def build_if_available(force: bool = False) -> Optional[str]:
    """Compile oracle/_ref/librods_ref.so from the reference sources (if present)."""
    if not available():
        return None
    if os.path.exists(LIB) and not force:
        return LIB
    os.makedirs(REF_DIR, exist_ok=True)
    for name, text in slices().items():
        with open(os.path.join(REF_DIR, name), "w") as f:
            f.write(text + "\n")
    with open(os.path.join(REF_DIR, "stubs.h"), "w") as f:
        f.write(STUBS)
    src = os.path.join(REF_DIR, "rods_harness.cpp")
    with open(src, "w") as f:
        f.write(HARNESS)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
                    REF_DIR, "-o", LIB, src], check=True)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise FileNotFoundError(LIB)
        lib = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        lib.ref_rod_exchange.restype = C.c_int
        lib.ref_rod_exchange.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, dp, C.c_int,
                                         C.c_int, dp, dp, dp, C.POINTER(C.c_uint8), dp, dp, dp,
                                         C.POINTER(C.c_int)]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def exchange(fields: np.ndarray, rods: np.ndarray, ihsl: np.ndarray, prod: np.ndarray,
             mode: np.ndarray, npm: float, dt: float, km):
    """The reference's cell loop over all cells.  fields: (n_layers, ny+1, nx+1),
    returned updated; rods: eqf_rod records (20 doubles each)."""
    f = np.ascontiguousarray(fields, dtype=np.float64).copy()
    nl, ny1, nx1 = f.shape
    r = np.ascontiguousarray(rods).view(np.float64).reshape(-1, 20).copy()
    n = r.shape[0]
    ih = np.ascontiguousarray(ihsl, dtype=np.float64).reshape(n, nl)
    pr = np.ascontiguousarray(prod, dtype=np.float64).reshape(n, nl)
    md = np.ascontiguousarray(mode, dtype=np.uint8).reshape(n, nl)
    k = np.ascontiguousarray(km, dtype=np.float64)[:nl].copy()
    io = np.zeros((n, nl))
    eo = np.zeros((n, nl))
    po = np.zeros(n, dtype=np.int32)
    load().ref_rod_exchange(nx1 - 1, ny1 - 1, float(npm), float(dt), _p(k), nl, n, _p(r), _p(ih),
                            _p(pr), md.ctypes.data_as(C.POINTER(C.c_uint8)), _p(f), _p(io),
                            _p(eo), po.ctypes.data_as(C.POINTER(C.c_int)))
    return f, io, eo, po
