// Shared host/device definitions of the trap field solver: level geometry, the
// matrix-free P1 stencil and the tile work lists.
//
// Mesh: eQ builds each HSL layer on RectangleMesh(p0, p1, nx, ny, "right")
// (src/fHSL.cpp:164-172): vertex (i, j) at (j*hx, i*hy), natural index
// j + i*(nx+1), each square cut along (i, j)-(i+1, j+1).  On the device a row is
// stored with pitch P = nx+1 rounded up to a multiple of 4 (k = j + i*P): every row
// starts 16-byte aligned, so rows, row segments and 4-node quads are aligned
// vectors.  The pad columns nx+1 .. P-1 hold zeros and carry all-zero stencils.  The stencil below is
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

// Lengths and physics of one level in one arithmetic type (kept in both FP32 and
// FP64 so kernels never convert or divide per node).
template <class T>
struct Lens {
  T hx, hy, hxl, hyl;      // regular spacing and last column/row cell sizes
  T ihx, ihy, ihxl, ihyl;  // their reciprocals
  T alpha, beta;           // mass scale (1 + dt*g) and dt*D
  T adv;                   // advection: dt * v_y(y) = -adv * y
  T rob[4];                // Robin walls: dt * rate (bottom, top, left, right; 0 = none)
};

// One trap on one multigrid level.
struct LevelGeom {
  long long off;      // offset of node (0,0) in the level's arrays
  int nx, ny;         // cells along x / y (nodes: (nx+1)*(ny+1))
  int P;              // row pitch: nx + 1 rounded up to a multiple of 4
  int trap;           // trap index in the batch
  unsigned walls;     // Dirichlet walls (WALL_* bits)
  int cx, cy;         // 1 if this level halves x / y relative to the finer level
  int fine_nx, fine_ny;  // cell counts of the finer level (for transfers)
  int fine_P;            // row pitch of the finer level
  long long fine_off;    // node offset of this trap on the finer level
  int adv_on;            // advection present (disables the uniform-interior path)
  double hx, hy;         // regular spacing (host-side construction)
  double hxl, hyl;       // size of the last column / row of cells
  double alpha, beta;    // mass scale (1 + dt*g) and dt*D
  double adv;            // advection: dt * v_y(y) = -adv * y  (0: none)
  double rob[4];         // Robin walls: dt * rate (bottom, top, left, right; 0 = none)
  int dvals;             // finest level: Dirichlet rows carry values (b = F there)
  // Anisotropic tensor (D11, D22, D12 per node, pitched like the field, tstride apart):
  // device copy for kernels, host copy for host-side setup; null = isotropic
  const double* tens;
  const double* htens;
  const float* tensf;  // FP32 copy for the FP32 operator path
  long long tstride;
  // the per-node stencils of an anisotropic level (c, e, w, n, s, ne, sw, 1/c per node,
  // pitched), built once per tensor update: the general path reads them
  const float* coef_f;
  const double* coef_d;
  // an advective level's stencils, which vary by row only (v_y depends on y): per row
  // i and column class edge_class(j) (c, e, w, n, s, ne, sw, 1/c), built once from
  // the FP64 rows (FP32: rounded); null = none
  const float* rowc_f;
  const double* rowc_d;
  Lens<double> ld;
  Lens<float> lf;
  // Uniform-interior stencil (nodes with 2 <= i <= ny-2 and 2 <= j <= nx-2).
  double cC, cE, cN, cD;  // centre, east=west, north=south, NE=SW
  double cCinv;           // 1 / cC
  double mC, mE, mN, mD;  // uniform-interior mass stencil (alpha = 1)
  float fC, fE, fN, fD, fCinv;
  float lam_max;          // upper bound of spectrum(D^-1 A)
  float lam_min;          // lower estimate (coarsest-level solve)
  float inv_pitch;        // 1 / P, for division-free row/column walks
  // Chebyshev-Jacobi step coefficients on this level's interval ([lam_max/ratio,
  // lam_max] for smoothing, [lam_min, lam_max] on the coarsest level), step s:
  // d_new = ch_old[s] d + ch_res[s] D^-1 r
  float ch_old[16], ch_res[16];
};
constexpr int kMaxChebSteps = 16;

template <class T>
EQF_HD const Lens<T>& lens(const LevelGeom& g);
template <>
EQF_HD const Lens<double>& lens<double>(const LevelGeom& g) { return g.ld; }
template <>
EQF_HD const Lens<float>& lens<float>(const LevelGeom& g) { return g.lf; }

// Rows [r0, r1) of one trap on one level (one CTA each); k0 = r0*P and k1 = r1*P
// are the node range.
struct Tile {
  int geom;  // index into the level's LevelGeom array (= trap index)
  int k0, k1;
  int r0, r1;
};

template <class T>
struct Sten {
  T c, e, w, n, s, ne, sw;
};

// Class of node index j on a grid of n cells along one axis: 0 and 1 (the first two
// nodes), 2 (interior, 2 <= j <= n - 2), 3 (n - 1) and 4 (n); edge_rep is the node a
// class's stencil is evaluated at (where edge_class(edge_rep(c)) == c).
EQF_HD int edge_class(int j, int n) { return j < 2 ? j : (j > n - 2 ? 4 - (n - j) : 2); }
EQF_HD int edge_rep(int c, int n) { return c < 2 ? c : (c == 2 ? 2 : (c == 3 ? n - 1 : n)); }

EQF_HD bool is_dirichlet(const LevelGeom& g, int i, int j) {
  return ((g.walls & WALL_BOTTOM) && i == 0) || ((g.walls & WALL_TOP) && i == g.ny) ||
         ((g.walls & WALL_LEFT) && j == 0) || ((g.walls & WALL_RIGHT) && j == g.nx);
}

// integer-only: 2 <= i <= ny-2 and 2 <= j <= nx-2, no advection
EQF_HD bool is_uniform_interior(const LevelGeom& g, int i, int j) {
  return i >= 2 && i <= g.ny - 2 && j >= 2 && j <= g.nx - 2 && !g.adv_on;
}

// Tensor (D11, D22, D12) of node (i, j) of this level, in the stencil's arithmetic
// (FP32 stencils read the FP32 copy; the host reads its own FP64 copy).
template <class T>
EQF_HD void tensor_at(const LevelGeom& g, int i, int j, T& d11, T& d22, T& d12) {
  const long long k = (long long)i * g.P + j;
#ifdef __CUDA_ARCH__
  if (sizeof(T) == sizeof(float)) {
    const float* t = g.tensf;
    d11 = (T)t[k];
    d22 = (T)t[k + g.tstride];
    d12 = (T)t[k + 2 * g.tstride];
    return;
  }
  const double* t = g.tens;
#else
  const double* t = g.htens;
#endif
  d11 = (T)t[k];
  d22 = (T)t[k + g.tstride];
  d12 = (T)t[k + 2 * g.tstride];
}

// One triangle's stiffness beta * area * grad(phi_a) . A grad(phi_b), A the mean of its
// vertex tensors, added to the node's row: gn the node's gradient, (gb[q], cb[q]) the
// other two vertices' gradients and the stencil entries they go to.
template <class T>
EQF_HD void aniso_tri(T beta_area, const T (&m)[3], T gnx, T gny, T gbx0, T gby0,
                      T& cb0, T gbx1, T gby1, T& cb1, T& cc) {
  const T a11 = m[0], a22 = m[1], a12 = m[2];
  auto form = [&](T ux, T uy, T vx, T vy) {
    return ux * (a11 * vx + a12 * vy) + uy * (a12 * vx + a22 * vy);
  };
  cc += beta_area * form(gnx, gny, gnx, gny);
  cb0 += beta_area * form(gnx, gny, gbx0, gby0);
  cb1 += beta_area * form(gnx, gny, gbx1, gby1);
}

// Stiffness of an anisotropic row from its (up to) six incident right triangles:
// square UR (the node is v0): (node, E, NE) and (node, N, NE); square LL (v3):
// (SW, S, node) and (SW, W, node); square LR (v2): (S, node, E); square UL (v1):
// (W, node, N).  The "right" cut couples no NW / SE pair, so the 7-point shape holds.
template <class T>
EQF_HD void aniso_stiffness(const LevelGeom& g, int i, int j, T hxl, T hxr, T hyd, T hyu,
                            Sten<T>& s) {
  const T beta = lens<T>(g).beta, half = T(0.5), third = T(1.0 / 3.0);
  T t0[3];
  tensor_at<T>(g, i, j, t0[0], t0[1], t0[2]);
  auto mean3 = [&](int i1, int j1, int i2, int j2, T (&m)[3]) {
    T u[3], v[3];
    tensor_at<T>(g, i1, j1, u[0], u[1], u[2]);
    tensor_at<T>(g, i2, j2, v[0], v[1], v[2]);
    for (int q = 0; q < 3; ++q) m[q] = third * (t0[q] + u[q] + v[q]);
  };
  T zero = T(0);
  T m[3];
  if (hxr > T(0) && hyu > T(0)) {
    const T ba = beta * half * hxr * hyu, ix = T(1) / hxr, iy = T(1) / hyu;
    mean3(i, j + 1, i + 1, j + 1, m);  // (node, E, NE)
    aniso_tri<T>(ba, m, -ix, zero, ix, -iy, s.e, zero, iy, s.ne, s.c);
    mean3(i + 1, j, i + 1, j + 1, m);  // (node, N, NE)
    aniso_tri<T>(ba, m, zero, -iy, -ix, iy, s.n, ix, zero, s.ne, s.c);
  }
  if (hxl > T(0) && hyd > T(0)) {
    const T ba = beta * half * hxl * hyd, ix = T(1) / hxl, iy = T(1) / hyd;
    mean3(i - 1, j - 1, i - 1, j, m);  // (SW, S, node)
    aniso_tri<T>(ba, m, zero, iy, -ix, zero, s.sw, ix, -iy, s.s, s.c);
    mean3(i - 1, j - 1, i, j - 1, m);  // (SW, W, node)
    aniso_tri<T>(ba, m, ix, zero, zero, -iy, s.sw, -ix, iy, s.w, s.c);
  }
  if (hxr > T(0) && hyd > T(0)) {
    const T ba = beta * half * hxr * hyd, ix = T(1) / hxr, iy = T(1) / hyd;
    mean3(i - 1, j, i, j + 1, m);  // (S, node, E)
    aniso_tri<T>(ba, m, -ix, iy, zero, -iy, s.s, ix, zero, s.e, s.c);
  }
  if (hxl > T(0) && hyu > T(0)) {
    const T ba = beta * half * hxl * hyu, ix = T(1) / hxl, iy = T(1) / hyu;
    mean3(i, j - 1, i + 1, j, m);  // (W, node, N)
    aniso_tri<T>(ba, m, ix, -iy, -ix, zero, s.w, zero, iy, s.n, s.c);
  }
}

// Full stencil of node (i, j) from the surrounding cell sizes, in arithmetic T.
// ANISO = false leaves out the anisotropic branch (for device callers that never see
// a tensor: anisotropic levels read their stencils built once by k_aniso_coefs).
// Mass (scaled by alpha): each triangle of area A adds A/6 on the diagonal and
// A/12 per edge.  Stiffness (scaled by beta): right triangles couple only along
// their legs, -cot/2 = -(other leg)/(2*this leg); hypotenuses carry no stiffness.
// Advection (c2): dt * int v_y d(phi_b)/dy phi_a over each triangle with a P1 v_y.
// WALLS = false gives the full operator's row, without the Dirichlet reduction.
template <class T, bool ANISO = true, bool WALLS = true>
EQF_HD Sten<T> stencil_general(const LevelGeom& g, int i, int j) {
  const Lens<T>& L = lens<T>(g);
  const T hxl = j > 0 ? (j == g.nx ? L.hxl : L.hx) : T(0);
  const T hxr = j < g.nx ? (j == g.nx - 1 ? L.hxl : L.hx) : T(0);
  const T hyd = i > 0 ? (i == g.ny ? L.hyl : L.hy) : T(0);
  const T hyu = i < g.ny ? (i == g.ny - 1 ? L.hyl : L.hy) : T(0);
  const T ihxl = j > 0 ? (j == g.nx ? L.ihxl : L.ihx) : T(0);
  const T ihxr = j < g.nx ? (j == g.nx - 1 ? L.ihxl : L.ihx) : T(0);
  const T ihyd = i > 0 ? (i == g.ny ? L.ihyl : L.ihy) : T(0);
  const T ihyu = i < g.ny ? (i == g.ny - 1 ? L.ihyl : L.ihy) : T(0);
  const T a = L.alpha, hb = T(0.5) * L.beta;
  const T sy = hyd + hyu, sx = hxl + hxr;
  const T a24 = a * T(1.0 / 24.0), a12 = a * T(1.0 / 12.0);
  Sten<T> s;
  if (ANISO && g.tens) {
    // mass as below; stiffness per incident triangle with the mean of the vertex
    // tensors (the P1 tensor integrates exactly to area x mean)
    s.e = a24 * hxr * sy;
    s.w = a24 * hxl * sy;
    s.n = a24 * hyu * sx;
    s.s = a24 * hyd * sx;
    s.ne = a12 * hxr * hyu;
    s.sw = a12 * hxl * hyd;
    s.c = a12 * (T(2) * hxl * hyd + hxr * hyd + hxl * hyu + T(2) * hxr * hyu);
    aniso_stiffness<T>(g, i, j, hxl, hxr, hyd, hyu, s);
  } else {
    const T ke = hb * sy * ihxr, kw = hb * sy * ihxl;  // zero where the cell is missing
    const T kn = hb * sx * ihyu, ks = hb * sx * ihyd;
    s.e = a24 * hxr * sy - ke;
    s.w = a24 * hxl * sy - kw;
    s.n = a24 * hyu * sx - kn;
    s.s = a24 * hyd * sx - ks;
    s.ne = a12 * hxr * hyu;
    s.sw = a12 * hxl * hyd;
    s.c = a12 * (T(2) * hxl * hyd + hxr * hyd + hxl * hyu + T(2) * hxr * hyu) + ke + kw + kn + ks;
  }
  if (g.adv_on) {
    // v_y at the node rows: dt*v(y) = -adv*y with y measured on this level's grid
    const T y0 = (i == g.ny) ? L.hy * T(g.ny - 1) + L.hyl : L.hy * T(i);
    const T yd = y0 - hyd, yu = y0 + hyu;
    const T va = -L.adv * y0, vd = -L.adv * yd, vu = -L.adv * yu;
    // each triangle adds (area/12) * dphi_b/dy * (v_a + sum of its vertex v)
    // Cell UR (x in [0,hxr], y in [0,hyu]), both triangles contain the node.
    if (hxr > T(0) && hyu > T(0)) {
      const T A12 = hxr * hyu * T(1.0 / 24.0);
      // lower-right (v0 = node, v1 = E, v3 = NE): dphi/dy: v0 0, v1 -1/hyu, v3 1/hyu
      T f = A12 * (va + (va + va + vu)) * ihyu;
      s.e -= f;
      s.ne += f;
      // upper-left (v0 = node, v2 = N, v3 = NE): dphi/dy: v0 -1/hyu, v2 1/hyu, v3 0
      f = A12 * (va + (va + vu + vu)) * ihyu;
      s.c -= f;
      s.n += f;
    }
    // Cell LL (x in [-hxl,0], y in [-hyd,0]), node is its v3 corner, both triangles.
    if (hxl > T(0) && hyd > T(0)) {
      const T A12 = hxl * hyd * T(1.0 / 24.0);
      // lower-right (v0 = SW, v1 = S, v3 = node): dphi/dy: v0 0, v1 -1/hyd, v3 1/hyd
      T f = A12 * (va + (vd + vd + va)) * ihyd;
      s.s -= f;
      s.c += f;
      // upper-left (v0 = SW, v2 = W, v3 = node): dphi/dy: v0 -1/hyd, v2 1/hyd, v3 0
      f = A12 * (va + (vd + va + va)) * ihyd;
      s.sw -= f;
      s.w += f;
    }
    // Cell LR (x in [0,hxr], y in [-hyd,0]): node is its v2 corner (upper-left tri).
    if (hxr > T(0) && hyd > T(0)) {
      const T A12 = hxr * hyd * T(1.0 / 24.0);
      // upper-left (v0 = S, v2 = node, v3 = E): dphi/dy: v0 -1/hyd, v2 1/hyd, v3 0
      const T f = A12 * (va + (vd + va + va)) * ihyd;
      s.s -= f;
      s.c += f;
    }
    // Cell UL (x in [-hxl,0], y in [0,hyu]): node is its v1 corner (lower-right tri).
    if (hxl > T(0) && hyu > T(0)) {
      const T A12 = hxl * hyu * T(1.0 / 24.0);
      // lower-right (v0 = W, v1 = node, v3 = N): dphi/dy: v0 0, v1 -1/hyu, v3 1/hyu
      const T f = A12 * (va + (va + va + vu)) * ihyu;
      s.c -= f;
      s.n += f;
    }
  }
  // Robin walls: dt*r*u*v on the wall's facets (fenics/hslD.ufl:36-42, facet
  // kernels fenics/hslD.h:3264-3445): facet mass |e|/3 on the diagonal, |e|/6 along it
  if (i == 0 && L.rob[0] != T(0)) {
    s.c += L.rob[0] * (hxl + hxr) * T(1.0 / 3.0);
    s.e += L.rob[0] * hxr * T(1.0 / 6.0);
    s.w += L.rob[0] * hxl * T(1.0 / 6.0);
  }
  if (i == g.ny && L.rob[1] != T(0)) {
    s.c += L.rob[1] * (hxl + hxr) * T(1.0 / 3.0);
    s.e += L.rob[1] * hxr * T(1.0 / 6.0);
    s.w += L.rob[1] * hxl * T(1.0 / 6.0);
  }
  if (j == 0 && L.rob[2] != T(0)) {
    s.c += L.rob[2] * (hyd + hyu) * T(1.0 / 3.0);
    s.n += L.rob[2] * hyu * T(1.0 / 6.0);
    s.s += L.rob[2] * hyd * T(1.0 / 6.0);
  }
  if (j == g.nx && L.rob[3] != T(0)) {
    s.c += L.rob[3] * (hyd + hyu) * T(1.0 / 3.0);
    s.n += L.rob[3] * hyu * T(1.0 / 6.0);
    s.s += L.rob[3] * hyd * T(1.0 / 6.0);
  }
  if (WALLS && g.walls) {
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

// 1 / diagonal of the operator row
template <class T>
EQF_HD T inv_diag(const LevelGeom& g, int i, int j, const Sten<T>& s);
template <>
EQF_HD float inv_diag<float>(const LevelGeom& g, int i, int j, const Sten<float>& s) {
  return is_uniform_interior(g, i, j) ? g.fCinv : 1.f / s.c;
}
template <>
EQF_HD double inv_diag<double>(const LevelGeom& g, int i, int j, const Sten<double>& s) {
  return is_uniform_interior(g, i, j) ? g.cCinv : 1.0 / s.c;
}

// Mass-matrix stencil (unscaled, alpha = 1, no stiffness): the u0*v part of L.
template <class T>
EQF_HD Sten<T> mass_stencil(const LevelGeom& g, int i, int j) {
  const Lens<T>& L = lens<T>(g);
  const T hxl = j > 0 ? (j == g.nx ? L.hxl : L.hx) : T(0);
  const T hxr = j < g.nx ? (j == g.nx - 1 ? L.hxl : L.hx) : T(0);
  const T hyd = i > 0 ? (i == g.ny ? L.hyl : L.hy) : T(0);
  const T hyu = i < g.ny ? (i == g.ny - 1 ? L.hyl : L.hy) : T(0);
  const T sy = hyd + hyu, sx = hxl + hxr;
  const T c24 = T(1.0 / 24.0), c12 = T(1.0 / 12.0);
  Sten<T> s;
  s.e = c24 * hxr * sy;
  s.w = c24 * hxl * sy;
  s.n = c24 * hyu * sx;
  s.s = c24 * hyd * sx;
  s.ne = c12 * hxr * hyu;
  s.sw = c12 * hxl * hyd;
  s.c = c12 * (T(2) * hxl * hyd + hxr * hyd + hxl * hyu + T(2) * hxr * hyu);
  return s;
}

}  // namespace eqf
