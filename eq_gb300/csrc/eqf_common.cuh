// Shared host/device definitions of the trap field solver: level geometry, the
// matrix-free P1 stencil and the tile work lists.
//
// Mesh: eQ builds each HSL layer on RectangleMesh(p0, p1, nx, ny, "right")
// (src/fHSL.cpp:164-172): vertex (i, j) at (j*hx, i*hy), natural index
// k = j + i*(nx+1), each square cut along (i, j)-(i+1, j+1).  The stencil below is
// the assembled hslD bilinear form (fenics/hslD.ufl:31-49, cell kernel
// fenics/hslD.h:3123-3262) for an isotropic tensor, written per node from the six
// incident right triangles, plus the reaction scaling of the mass block.
//
// Multigrid levels keep the same form on a coarser tensor grid whose spacing is
// uniform except for the last column/row of cells ("last-cell" size <= spacing),
// which is what nested coarsening of an odd cell count produces.  Every level
// therefore needs only (nx, ny, hx, hy, hx_last, hy_last, alpha, beta, walls).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define EQF_HD __host__ __device__ __forceinline__

namespace eqf {

enum : unsigned { WALL_BOTTOM = 1u, WALL_TOP = 2u, WALL_LEFT = 4u, WALL_RIGHT = 8u };

// One trap on one multigrid level.
struct LevelGeom {
  long long off;      // offset of node (0,0) in the level's arrays
  int nx, ny;         // cells along x / y (nodes: (nx+1)*(ny+1))
  int trap;           // trap index in the batch
  unsigned walls;     // Dirichlet walls (WALL_* bits)
  int cx, cy;         // 1 if this level halves x / y relative to the finer level
  int fine_nx, fine_ny;  // cell counts of the finer level (for transfers)
  long long fine_off;    // node offset of this trap on the finer level
  double hx, hy;         // regular spacing
  double hxl, hyl;       // size of the last column / row of cells
  double alpha, beta;    // mass scale (1 + dt*g) and dt*D
  double adv;            // advection: v_y(y) = -adv * y  (0: none)
  // Uniform-interior stencil (nodes with 2 <= i <= ny-2 and 2 <= j <= nx-2).
  double cC, cE, cN, cD;  // centre, east=west, north=south, NE=SW
  float fC, fE, fN, fD;
  float lam_max;          // upper bound of spectrum(D^-1 A)
  float lam_min;          // lower estimate (coarsest-level solve)
};

// A contiguous node range [k0, k1) of one trap on one level (one CTA each).
struct Tile {
  int geom;   // index into the level's LevelGeom array
  int k0, k1;
};

template <class T>
struct Sten {
  T c, e, w, n, s, ne, sw;
};

EQF_HD bool is_dirichlet(const LevelGeom& g, int i, int j) {
  return ((g.walls & WALL_BOTTOM) && i == 0) || ((g.walls & WALL_TOP) && i == g.ny) ||
         ((g.walls & WALL_LEFT) && j == 0) || ((g.walls & WALL_RIGHT) && j == g.nx);
}

EQF_HD bool is_uniform_interior(const LevelGeom& g, int i, int j) {
  return i >= 2 && i <= g.ny - 2 && j >= 2 && j <= g.nx - 2 && g.adv == 0.0;
}

// Full stencil of node (i, j) from the surrounding cell sizes, in arithmetic T.
// Mass (scaled by alpha): each triangle of area A adds A/6 on the diagonal and
// A/12 per edge.  Stiffness (scaled by beta): right triangles couple only along
// their legs, -cot/2 = -(other leg)/(2*this leg); hypotenuses carry no stiffness.
// Advection (c2): dt * int v_y d(phi_b)/dy phi_a over each triangle with a P1 v_y.
template <class T>
EQF_HD Sten<T> stencil_general(const LevelGeom& g, int i, int j) {
  const T hx = T(g.hx), hy = T(g.hy);
  const T hxl = j > 0 ? (j == g.nx ? T(g.hxl) : hx) : T(0);
  const T hxr = j < g.nx ? (j == g.nx - 1 ? T(g.hxl) : hx) : T(0);
  const T hyd = i > 0 ? (i == g.ny ? T(g.hyl) : hy) : T(0);
  const T hyu = i < g.ny ? (i == g.ny - 1 ? T(g.hyl) : hy) : T(0);
  const T a = T(g.alpha), b = T(g.beta);
  const T sy = hyd + hyu, sx = hxl + hxr;
  Sten<T> s;
  T ke = hxr > T(0) ? b * sy / (T(2) * hxr) : T(0);
  T kw = hxl > T(0) ? b * sy / (T(2) * hxl) : T(0);
  T kn = hyu > T(0) ? b * sx / (T(2) * hyu) : T(0);
  T ks = hyd > T(0) ? b * sx / (T(2) * hyd) : T(0);
  s.e = a * hxr * sy / T(24) - ke;
  s.w = a * hxl * sy / T(24) - kw;
  s.n = a * hyu * sx / T(24) - kn;
  s.s = a * hyd * sx / T(24) - ks;
  s.ne = a * hxr * hyu / T(12);
  s.sw = a * hxl * hyd / T(12);
  s.c = a * (T(2) * hxl * hyd + hxr * hyd + hxl * hyu + T(2) * hxr * hyu) / T(12) + ke + kw +
        kn + ks;
  if (g.adv != 0.0) {
    // v_y at the node rows: v(y) = -adv*y with y measured on this level's grid
    const T y0 = (i == g.ny) ? T(g.hy) * T(g.ny - 1) + T(g.hyl) : T(g.hy) * T(i);
    const T yd = y0 - hyd, yu = y0 + hyu;
    const T va = -T(g.adv) * y0, vd = -T(g.adv) * yd, vu = -T(g.adv) * yu;
    // C_ab = dt-scaled in adv; each triangle: (area/12) * dphi_b/dy * (v_a + sum v)
    // Cell UR (x in [0,hxr], y in [0,hyu]), both triangles contain the node.
    if (hxr > T(0) && hyu > T(0)) {
      const T A = hxr * hyu / T(2);
      // lower-right (v0 = node, v1 = E, v3 = NE): dphi/dy: v0 0, v1 -1/hyu, v3 1/hyu
      T vs = va + va + vu;  // v at (node, E, NE): E is on the node row, NE on the upper
      T f = A / T(12) * (va + vs);
      s.e += f * (-T(1) / hyu);
      s.ne += f * (T(1) / hyu);
      // upper-left (v0 = node, v2 = N, v3 = NE): dphi/dy: v0 -1/hyu, v2 1/hyu, v3 0
      vs = va + vu + vu;
      f = A / T(12) * (va + vs);
      s.c += f * (-T(1) / hyu);
      s.n += f * (T(1) / hyu);
    }
    // Cell LL (x in [-hxl,0], y in [-hyd,0]), node is its v3 corner, both triangles.
    if (hxl > T(0) && hyd > T(0)) {
      const T A = hxl * hyd / T(2);
      // lower-right (v0 = SW, v1 = S, v3 = node): dphi/dy: v0 0, v1 -1/hyd, v3 1/hyd
      T vs = vd + vd + va;
      T f = A / T(12) * (va + vs);
      s.s += f * (-T(1) / hyd);
      s.c += f * (T(1) / hyd);
      // upper-left (v0 = SW, v2 = W, v3 = node): dphi/dy: v0 -1/hyd, v2 1/hyd, v3 0
      vs = vd + va + va;
      f = A / T(12) * (va + vs);
      s.sw += f * (-T(1) / hyd);
      s.w += f * (T(1) / hyd);
    }
    // Cell LR (x in [0,hxr], y in [-hyd,0]): node is its v2 corner (upper-left tri).
    if (hxr > T(0) && hyd > T(0)) {
      const T A = hxr * hyd / T(2);
      // upper-left (v0 = S, v2 = node, v3 = E): dphi/dy: v0 -1/hyd, v2 1/hyd, v3 0
      const T vs = vd + va + va;
      const T f = A / T(12) * (va + vs);
      s.s += f * (-T(1) / hyd);
      s.c += f * (T(1) / hyd);
    }
    // Cell UL (x in [-hxl,0], y in [0,hyu]): node is its v1 corner (lower-right tri).
    if (hxl > T(0) && hyu > T(0)) {
      const T A = hxl * hyu / T(2);
      // lower-right (v0 = W, v1 = node, v3 = N): dphi/dy: v0 0, v1 -1/hyu, v3 1/hyu
      const T vs = va + va + vu;
      const T f = A / T(12) * (va + vs);
      s.c += f * (-T(1) / hyu);
      s.n += f * (T(1) / hyu);
    }
  }
  if (g.walls) {
    if (is_dirichlet(g, i, j)) {
      s.c = T(1);
      s.e = s.w = s.n = s.s = s.ne = s.sw = T(0);
      return s;
    }
    if (is_dirichlet(g, i, j + 1)) s.e = T(0);
    if (is_dirichlet(g, i, j - 1)) s.w = T(0);
    if (is_dirichlet(g, i + 1, j)) s.n = T(0);
    if (is_dirichlet(g, i - 1, j)) s.s = T(0);
    if (is_dirichlet(g, i + 1, j + 1)) s.ne = T(0);
    if (is_dirichlet(g, i - 1, j - 1)) s.sw = T(0);
  }
  return s;
}

template <class T>
EQF_HD Sten<T> stencil_at(const LevelGeom& g, int i, int j);

template <>
EQF_HD Sten<float> stencil_at<float>(const LevelGeom& g, int i, int j) {
  if (is_uniform_interior(g, i, j)) return Sten<float>{g.fC, g.fE, g.fE, g.fN, g.fN, g.fD, g.fD};
  return stencil_general<float>(g, i, j);
}
template <>
EQF_HD Sten<double> stencil_at<double>(const LevelGeom& g, int i, int j) {
  if (is_uniform_interior(g, i, j)) return Sten<double>{g.cC, g.cE, g.cE, g.cN, g.cN, g.cD, g.cD};
  return stencil_general<double>(g, i, j);
}

// Mass-matrix stencil (unscaled, alpha = 1, no stiffness): the u0*v part of L.
template <class T>
EQF_HD Sten<T> mass_stencil(const LevelGeom& g, int i, int j) {
  const T hx = T(g.hx), hy = T(g.hy);
  const T hxl = j > 0 ? (j == g.nx ? T(g.hxl) : hx) : T(0);
  const T hxr = j < g.nx ? (j == g.nx - 1 ? T(g.hxl) : hx) : T(0);
  const T hyd = i > 0 ? (i == g.ny ? T(g.hyl) : hy) : T(0);
  const T hyu = i < g.ny ? (i == g.ny - 1 ? T(g.hyl) : hy) : T(0);
  const T sy = hyd + hyu, sx = hxl + hxr;
  Sten<T> s;
  s.e = hxr * sy / T(24);
  s.w = hxl * sy / T(24);
  s.n = hyu * sx / T(24);
  s.s = hyd * sx / T(24);
  s.ne = hxr * hyu / T(12);
  s.sw = hxl * hyd / T(12);
  s.c = (T(2) * hxl * hyd + hxr * hyd + hxl * hyu + T(2) * hxr * hyu) / T(12);
  return s;
}

}  // namespace eqf
