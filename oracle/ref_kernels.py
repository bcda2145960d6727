"""The reference's own element kernels, compiled from its sources, for pinning the oracle.

TEST INFRASTRUCTURE ONLY.  eQ's element arithmetic is the FFC-generated C++ in
fenics/hslD.h (bilinear cell kernel 3103-3262, Robin facet kernels 3264-3445,
linear cell kernel 3446-3533, linear facet kernels 3534-3693) and
fenics/boundary.h (flux functional, exterior facet kernel 2632-2744).  Those
classes need only two UFC base classes (ufc::cell_integral,
ufc::exterior_facet_integral) and two reference-triangle tables from UFC's
geometry header (UFC 2018.1.0, not vendored in the reference).  This recipe

  * slices the integral classes out of the reference headers, where they lie,
    into oracle/_ref/ (git-ignored; nothing of the reference is committed),
  * compiles them with g++ against a stub of the two base classes and the two
    tables written here (the tables are facts of the reference triangle
    (0,0),(1,0),(0,1): facet i is the edge opposite vertex i),
  * exposes extern "C" wrappers loaded with ctypes.

DOLFIN's assembly, boundary-condition application and PETSc's LU are not
compiled (they need DOLFIN/PETSc/MPI); the oracle restates them.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_DIR, "libhsld_ref2.so")
# the reference checkout: EQ_REFERENCE_ROOT, else a "reference" directory beside the
# repository
REFERENCE = os.environ.get("EQ_REFERENCE_ROOT",
                           os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

HSLD_CLASSES = ["hsld_cell_integral_0_otherwise", "hsld_exterior_facet_integral_0_1",
                "hsld_exterior_facet_integral_0_2", "hsld_cell_integral_1_otherwise",
                "hsld_exterior_facet_integral_1_1", "hsld_exterior_facet_integral_1_2"]
BOUNDARY_CLASSES = ["boundary_exterior_facet_integral_0_otherwise"]
ADV_CLASSES = ["advectiondiffusion_cell_integral_0_otherwise",
               "advectiondiffusion_exterior_facet_integral_0_1",
               "advectiondiffusion_exterior_facet_integral_0_2",
               "advectiondiffusion_cell_integral_1_otherwise",
               "advectiondiffusion_exterior_facet_integral_1_1",
               "advectiondiffusion_exterior_facet_integral_1_2"]

UFC_STUB = r'''
// Minimal stand-in for the two UFC integral interfaces the generated kernels
// derive from, plus the reference-triangle facet tables they read.
#pragma once
#include <cmath>
#include <cstddef>
#include <vector>
#include <algorithm>
#include <stdexcept>
namespace ufc {
struct cell_integral {
  virtual ~cell_integral() {}
  virtual const std::vector<bool>& enabled_coefficients() const = 0;
  virtual void tabulate_tensor(double* A, const double* const* w, const double* coordinate_dofs,
                               int cell_orientation) const = 0;
};
struct exterior_facet_integral {
  virtual ~exterior_facet_integral() {}
  virtual const std::vector<bool>& enabled_coefficients() const = 0;
  virtual void tabulate_tensor(double* A, const double* const* w, const double* coordinate_dofs,
                               std::size_t facet, int cell_orientation) const = 0;
};
}  // namespace ufc
// facet i of the reference triangle (0,0),(1,0),(0,1) is the edge opposite vertex i
static const double triangle_reference_facet_jacobian[3][2][1] = {
    {{-1.0}, {1.0}}, {{0.0}, {1.0}}, {{1.0}, {0.0}}};
static const double triangle_reference_facet_normals[3][2] = {
    {0.70710678118654752440, 0.70710678118654752440}, {-1.0, 0.0}, {0.0, -1.0}};
'''

HARNESS = r'''
#include "ufc_stub.h"
#include "hsld_integrals.inc"
#include "boundary_integrals.inc"
#include "adv_integrals.inc"
extern "C" {
// flow channel, bilinear form of AdvectionDiffusion: w = {dt, D, v, r1, r2}
void ref_adv_a_cell(double dt, double D, double v, const double* coords, double* A) {
  const double a[1] = {dt}, b[1] = {D}, c[1] = {v}, z[1] = {0.0};
  const double* w[5] = {a, b, c, z, z};
  advectiondiffusion_cell_integral_0_otherwise k;
  k.tabulate_tensor(A, w, coords, 0);
}
void ref_adv_a_facet(int marker, double dt, double r, const double* coords, int facet,
                     double* A) {
  const double a[1] = {dt}, rv[1] = {r}, z[1] = {0.0};
  const double* w[5] = {a, z, z, marker == 1 ? rv : z, marker == 2 ? rv : z};
  if (marker == 1) {
    advectiondiffusion_exterior_facet_integral_0_1 k;
    k.tabulate_tensor(A, w, coords, facet, 0);
  } else {
    advectiondiffusion_exterior_facet_integral_0_2 k;
    k.tabulate_tensor(A, w, coords, facet, 0);
  }
}
// linear form: w = {u0[2], dt, D, v, r1, s1, r2, s2}
void ref_adv_L_cell(const double* u0, double dt, double D, double v, const double* coords,
                    double* b) {
  const double a[1] = {dt}, d[1] = {D}, c[1] = {v}, z[1] = {0.0};
  const double* w[8] = {u0, a, d, c, z, z, z, z};
  advectiondiffusion_cell_integral_1_otherwise k;
  k.tabulate_tensor(b, w, coords, 0);
}
void ref_adv_L_facet(int marker, const double* u0, double dt, double r, double s,
                     const double* coords, int facet, double* b) {
  const double a[1] = {dt}, rv[1] = {r}, sv[1] = {s}, z[1] = {0.0};
  const double* w[8] = {u0, a, z, z, marker == 1 ? rv : z, marker == 1 ? sv : z,
                        marker == 2 ? rv : z, marker == 2 ? sv : z};
  if (marker == 1) {
    advectiondiffusion_exterior_facet_integral_1_1 k;
    k.tabulate_tensor(b, w, coords, facet, 0);
  } else {
    advectiondiffusion_exterior_facet_integral_1_2 k;
    k.tabulate_tensor(b, w, coords, facet, 0);
  }
}
// bilinear cell kernel of hslD: w = {D11[3], D22[3], D12[3], D, dt, r1, r2}
void ref_hsld_a_cell(const double* D11, const double* D22, const double* D12, double D,
                     double dt, const double* coords, double* A) {
  const double Dv[1] = {D}, dtv[1] = {dt}, z[1] = {0.0};
  const double* w[7] = {D11, D22, D12, Dv, dtv, z, z};
  hsld_cell_integral_0_otherwise k;
  k.tabulate_tensor(A, w, coords, 0);
}
// bilinear Robin facet kernels (marker 1 uses r1, marker 2 uses r2)
void ref_hsld_a_facet(int marker, double dt, double r, const double* coords, int facet,
                      double* A) {
  const double dtv[1] = {dt}, rv[1] = {r}, z[1] = {0.0};
  const double* w[7] = {z, z, z, z, dtv, marker == 1 ? rv : z, marker == 2 ? rv : z};
  if (marker == 1) {
    hsld_exterior_facet_integral_0_1 k;
    k.tabulate_tensor(A, w, coords, facet, 0);
  } else {
    hsld_exterior_facet_integral_0_2 k;
    k.tabulate_tensor(A, w, coords, facet, 0);
  }
}
// linear cell kernel of hslD: w = {u0[3], dt, f, r1, s1, r2, s2}
void ref_hsld_L_cell(const double* u0, double dt, double f, const double* coords, double* b) {
  const double dtv[1] = {dt}, fv[1] = {f}, z[1] = {0.0};
  const double* w[7] = {u0, dtv, fv, z, z, z, z};
  hsld_cell_integral_1_otherwise k;
  k.tabulate_tensor(b, w, coords, 0);
}
// linear Robin facet kernels
void ref_hsld_L_facet(int marker, double dt, double r, double s, const double* coords,
                      int facet, double* b) {
  const double dtv[1] = {dt}, rv[1] = {r}, sv[1] = {s}, z[1] = {0.0};
  const double* w[7] = {z, dtv, z, marker == 1 ? rv : z, marker == 1 ? sv : z,
                        marker == 2 ? rv : z, marker == 2 ? sv : z};
  if (marker == 1) {
    hsld_exterior_facet_integral_1_1 k;
    k.tabulate_tensor(b, w, coords, facet, 0);
  } else {
    hsld_exterior_facet_integral_1_2 k;
    k.tabulate_tensor(b, w, coords, facet, 0);
  }
}
// flux functional -grad(u).n over one exterior facet: w = {u[3]}
void ref_boundary_flux_facet(const double* u, const double* coords, int facet, double* out) {
  const double* w[1] = {u};
  boundary_exterior_facet_integral_0_otherwise k;
  k.tabulate_tensor(out, w, coords, facet, 0);
}
}
'''


def _slice_classes(path: str, names) -> str:
    """Text of the named top-level classes (from `class NAME` to the closing `};`)."""
    with open(path) as f:
        lines = f.read().splitlines()
    out = []
    for name in names:
        start = next(i for i, ln in enumerate(lines) if re.match(rf"^class {name}\b", ln))
        end = next(i for i in range(start + 1, len(lines)) if lines[i].rstrip() == "};")
        out.extend(lines[start:end + 1])
        out.append("")
    return "\n".join(out)


def available() -> bool:
    return os.path.exists(os.path.join(REFERENCE, "fenics", "hslD.h"))


def build_if_available(force: bool = False) -> Optional[str]:
    """Compile oracle/_ref/libhsld_ref.so from the reference sources (if present)."""
    if not available():
        return None
    if os.path.exists(LIB) and not force:
        return LIB
    os.makedirs(REF_DIR, exist_ok=True)
    with open(os.path.join(REF_DIR, "ufc_stub.h"), "w") as f:
        f.write(UFC_STUB)
    with open(os.path.join(REF_DIR, "hsld_integrals.inc"), "w") as f:
        f.write(_slice_classes(os.path.join(REFERENCE, "fenics", "hslD.h"), HSLD_CLASSES))
    with open(os.path.join(REF_DIR, "boundary_integrals.inc"), "w") as f:
        f.write(_slice_classes(os.path.join(REFERENCE, "fenics", "boundary.h"), BOUNDARY_CLASSES))
    with open(os.path.join(REF_DIR, "adv_integrals.inc"), "w") as f:
        f.write(_slice_classes(os.path.join(REFERENCE, "fenics", "AdvectionDiffusion.h"),
                               ADV_CLASSES))
    src = os.path.join(REF_DIR, "harness.cpp")
    with open(src, "w") as f:
        f.write(HARNESS)
    subprocess.run(["g++", "-O2", "-std=c++14", "-shared", "-fPIC", "-I", REF_DIR, "-o", LIB,
                    src], check=True)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise FileNotFoundError(LIB)
        _lib = C.CDLL(LIB)
    return _lib


def _p(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


def a_cell(coords, D11, D22, D12, D, dt) -> np.ndarray:
    A = np.zeros(9)
    c = np.ascontiguousarray(coords, dtype=np.float64).ravel()
    d11, d22, d12 = (np.ascontiguousarray(v, dtype=np.float64) for v in (D11, D22, D12))
    load().ref_hsld_a_cell(_p(d11), _p(d22), _p(d12), C.c_double(D), C.c_double(dt), _p(c),
                           A.ctypes.data_as(C.POINTER(C.c_double)))
    return A.reshape(3, 3)


def a_facet(marker, dt, r, coords, facet) -> np.ndarray:
    A = np.zeros(9)
    c = np.ascontiguousarray(coords, dtype=np.float64).ravel()
    load().ref_hsld_a_facet(marker, C.c_double(dt), C.c_double(r), _p(c), facet,
                            A.ctypes.data_as(C.POINTER(C.c_double)))
    return A.reshape(3, 3)


def L_cell(coords, u0, dt, f) -> np.ndarray:
    b = np.zeros(3)
    c = np.ascontiguousarray(coords, dtype=np.float64).ravel()
    u = np.ascontiguousarray(u0, dtype=np.float64)
    load().ref_hsld_L_cell(_p(u), C.c_double(dt), C.c_double(f), _p(c),
                           b.ctypes.data_as(C.POINTER(C.c_double)))
    return b


def L_facet(marker, dt, r, s, coords, facet) -> np.ndarray:
    b = np.zeros(3)
    c = np.ascontiguousarray(coords, dtype=np.float64).ravel()
    load().ref_hsld_L_facet(marker, C.c_double(dt), C.c_double(r), C.c_double(s), _p(c), facet,
                            b.ctypes.data_as(C.POINTER(C.c_double)))
    return b


def flux_facet(coords, u, facet) -> float:
    out = np.zeros(1)
    c = np.ascontiguousarray(coords, dtype=np.float64).ravel()
    uu = np.ascontiguousarray(u, dtype=np.float64)
    load().ref_boundary_flux_facet(_p(uu), _p(c), facet, out.ctypes.data_as(C.POINTER(C.c_double)))
    return float(out[0])


# ---- flow channel (fenics/AdvectionDiffusion.h) ----
def adv_a_cell(coords, dt, D, v) -> np.ndarray:
    A = np.zeros(4)
    c = np.ascontiguousarray(coords, dtype=np.float64).ravel()
    load().ref_adv_a_cell(C.c_double(dt), C.c_double(D), C.c_double(v), _p(c),
                          A.ctypes.data_as(C.POINTER(C.c_double)))
    return A.reshape(2, 2)


def adv_a_facet(marker, dt, r, coords, facet) -> np.ndarray:
    A = np.zeros(4)
    c = np.ascontiguousarray(coords, dtype=np.float64).ravel()
    load().ref_adv_a_facet(marker, C.c_double(dt), C.c_double(r), _p(c), facet,
                           A.ctypes.data_as(C.POINTER(C.c_double)))
    return A.reshape(2, 2)


def adv_L_cell(coords, u0, dt, D, v) -> np.ndarray:
    b = np.zeros(2)
    c = np.ascontiguousarray(coords, dtype=np.float64).ravel()
    u = np.ascontiguousarray(u0, dtype=np.float64)
    load().ref_adv_L_cell(_p(u), C.c_double(dt), C.c_double(D), C.c_double(v), _p(c),
                          b.ctypes.data_as(C.POINTER(C.c_double)))
    return b


def adv_L_facet(marker, coords, u0, dt, r, s, facet) -> np.ndarray:
    b = np.zeros(2)
    c = np.ascontiguousarray(coords, dtype=np.float64).ravel()
    u = np.ascontiguousarray(u0, dtype=np.float64)
    load().ref_adv_L_facet(marker, _p(u), C.c_double(dt), C.c_double(r), C.c_double(s), _p(c),
                           facet, b.ctypes.data_as(C.POINTER(C.c_double)))
    return b
