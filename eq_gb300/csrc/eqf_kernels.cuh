// Tile kernels of the trap field solver: matrix-free operator, Chebyshev-Jacobi
// smoothing, multigrid transfers, CG vector updates and the FP64 residual of the
// iterative-refinement loop.  Every kernel runs one CTA per tile of a level's
// tile list, so one launch covers every trap of a batch; a per-trap skip flag
// lets converged traps drop out without changing the launch sequence.
//
// Reductions are deterministic: each tile writes one FP64 partial, and the
// per-trap scalar kernels add a trap's partials in tile order.
#pragma once
#include "eqf_common.cuh"

namespace eqf {

constexpr int kThreads = 256;

// Walks the nodes k = k0 + tid, k0 + tid + bd, ... of a tile while keeping
// (i, j) = divmod(k - off, nx + 1) up to date with one division per thread.
struct NodeWalk {
  int k, i, j;
  int qi, qj, pitch;
  __device__ __forceinline__ NodeWalk(const LevelGeom& g, int k0) {
    pitch = g.nx + 1;
    k = k0 + threadIdx.x;
    i = k / pitch;
    j = k - i * pitch;
    qi = blockDim.x / pitch;
    qj = blockDim.x - qi * pitch;
  }
  __device__ __forceinline__ void next() {
    k += blockDim.x;
    i += qi;
    j += qj;
    if (j >= pitch) {
      j -= pitch;
      ++i;
    }
  }
};

// y_k = (A x)_k for node (i, j); x points at the trap's node (0,0).
template <class T>
__device__ __forceinline__ T apply_node(const LevelGeom& g, const T* __restrict__ x, int k, int i,
                                        int j, const Sten<T>& s) {
  const int P = g.nx + 1;
  if (is_uniform_interior(g, i, j)) {
    return s.c * x[k] + s.e * (x[k + 1] + x[k - 1]) + s.n * (x[k + P] + x[k - P]) +
           s.ne * (x[k + P + 1] + x[k - P - 1]);
  }
  T acc = s.c * x[k];
  if (j < g.nx) acc += s.e * x[k + 1];
  if (j > 0) acc += s.w * x[k - 1];
  if (i < g.ny) acc += s.n * x[k + P];
  if (i > 0) acc += s.s * x[k - P];
  if (i < g.ny && j < g.nx) acc += s.ne * x[k + P + 1];
  if (i > 0 && j > 0) acc += s.sw * x[k - P - 1];
  return acc;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

#define EQF_TILE_PROLOGUE(skipflags)                                  \
  const Tile tile = tiles[blockIdx.x];                                \
  const LevelGeom g = G[tile.geom];                                   \
  if (skipflags && skipflags[g.trap]) return;

// y = A x; optional per-tile partial of dot(x, y)
template <class T, bool DOT>
__global__ void __launch_bounds__(kThreads) k_apply(const LevelGeom* __restrict__ G,
                                                   const Tile* __restrict__ tiles,
                                                   const int* __restrict__ skip,
                                                   const T* __restrict__ x, T* __restrict__ y,
                                                   double* __restrict__ part) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (DOT && threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  const T* xs = x + g.off;
  T* ys = y + g.off;
  T acc = T(0);
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    const Sten<T> s = stencil_at<T>(g, w.i, w.j);
    const T v = apply_node<T>(g, xs, w.k, w.i, w.j, s);
    ys[w.k] = v;
    if (DOT) acc += v * xs[w.k];
  }
  if (DOT) {
    const double t = block_sum(double(acc));
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

// Chebyshev step coefficients for step index `step` (0-based) on [lmin, lmax].
struct ChebCoef {
  float c_old;  // multiplies the previous direction
  float c_res;  // multiplies D^-1 r
};
__device__ __forceinline__ ChebCoef cheb_coef(float lmin, float lmax, int step) {
  const float theta = 0.5f * (lmax + lmin), delta = 0.5f * (lmax - lmin);
  const float sigma = theta / delta;
  if (step == 0) return ChebCoef{0.f, 1.f / theta};
  float rho_old = 1.f / sigma, rho = rho_old;
  for (int s = 1; s <= step; ++s) {
    rho = 1.f / (2.f * sigma - rho_old);
    if (s < step) rho_old = rho;
  }
  return ChebCoef{rho * rho_old, 2.f * rho / delta};
}

// Chebyshev-Jacobi step on one level.
//   FIRST & ZERO: x_out = d = D^-1 b / theta                    (x_in = 0)
//   FIRST:        d = D^-1 (b - A x_in) / theta; x_out = x_in + d
//   otherwise:    d = c_old d + c_res D^-1 (b - A x_in); x_out = x_in + d
// `ratio` > 0 selects the smoothing interval [lmax/ratio, lmax], else the full
// interval [lmin, lmax] (coarsest-level solve).  DOT adds a partial of b.x_out.
template <class T, bool FIRST, bool ZERO, bool DOT>
__global__ void __launch_bounds__(kThreads) k_cheb(const LevelGeom* __restrict__ G,
                                                  const Tile* __restrict__ tiles,
                                                  const int* __restrict__ skip, float ratio,
                                                  int step, const T* __restrict__ b,
                                                  const T* __restrict__ xin, T* __restrict__ xout,
                                                  T* __restrict__ d, double* __restrict__ part) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (DOT && threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  const float lmax = g.lam_max, lmin = ratio > 0.f ? g.lam_max / ratio : g.lam_min;
  const ChebCoef cc = cheb_coef(lmin, lmax, FIRST ? 0 : step);
  const T* bs = b + g.off;
  const T* xi = xin + g.off;
  T* xo = xout + g.off;
  T* ds = d + g.off;
  T acc = T(0);
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    const Sten<T> s = stencil_at<T>(g, w.i, w.j);
    T r = bs[w.k];
    if (!ZERO) r -= apply_node<T>(g, xi, w.k, w.i, w.j, s);
    T dn = T(cc.c_res) * r / s.c;
    if (!FIRST) dn += T(cc.c_old) * ds[w.k];
    const T xn = ZERO ? dn : xi[w.k] + dn;
    xo[w.k] = xn;
    ds[w.k] = dn;
    if (DOT) acc += bs[w.k] * xn;
  }
  if (DOT) {
    const double t = block_sum(double(acc));
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

// t = b - A x
template <class T>
__global__ void __launch_bounds__(kThreads) k_resid(const LevelGeom* __restrict__ G,
                                                   const Tile* __restrict__ tiles,
                                                   const int* __restrict__ skip,
                                                   const T* __restrict__ b,
                                                   const T* __restrict__ x, T* __restrict__ t) {
  EQF_TILE_PROLOGUE(skip);
  const T* bs = b + g.off;
  const T* xs = x + g.off;
  T* ts = t + g.off;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    const Sten<T> s = stencil_at<T>(g, w.i, w.j);
    ts[w.k] = bs[w.k] - apply_node<T>(g, xs, w.k, w.i, w.j, s);
  }
}

// Per-axis map between a coarse level and its finer level.  A fine node either
// coincides with coarse node `lo` (hi == lo) or is the midpoint of coarse nodes
// lo and lo+1.  Coarse node K sits on fine node min(2K, n_fine) when the axis is
// halved, on fine node K otherwise.
__device__ __forceinline__ void fine_to_coarse(int f, int nf, int halved, int& lo, int& hi) {
  if (!halved) {
    lo = hi = f;
  } else if ((f & 1) == 0) {
    lo = hi = f >> 1;
  } else if (f == nf) {
    lo = hi = (f + 1) >> 1;
  } else {
    lo = (f - 1) >> 1;
    hi = lo + 1;
  }
}
__device__ __forceinline__ bool is_mid(int f, int nf, int halved) {
  return halved && (f & 1) && f != nf;
}
__device__ __forceinline__ int coarse_to_fine(int K, int nf, int halved) {
  return halved ? min(2 * K, nf) : K;
}

// b_c = R t_f = P^T t_f, gathered per coarse node (runs on coarse-level tiles).
// Coarse Dirichlet nodes get 0.
template <class T>
__global__ void __launch_bounds__(kThreads) k_restrict(const LevelGeom* __restrict__ G,
                                                      const Tile* __restrict__ tiles,
                                                      const int* __restrict__ skip,
                                                      const T* __restrict__ tf,
                                                      T* __restrict__ bc) {
  EQF_TILE_PROLOGUE(skip);
  const int nfx = g.fine_nx, nfy = g.fine_ny, PF = nfx + 1;
  const T* t = tf + g.fine_off;
  T* b = bc + g.off;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    if (g.walls && is_dirichlet(g, w.i, w.j)) {
      b[w.k] = T(0);
      continue;
    }
    const int fi = coarse_to_fine(w.i, nfy, g.cy), fj = coarse_to_fine(w.j, nfx, g.cx);
    const int kf = fj + fi * PF;
    T acc = t[kf];
    T half = T(0);
    const bool mE = fj + 1 <= nfx && is_mid(fj + 1, nfx, g.cx);
    const bool mW = fj - 1 >= 0 && is_mid(fj - 1, nfx, g.cx);
    const bool mN = fi + 1 <= nfy && is_mid(fi + 1, nfy, g.cy);
    const bool mS = fi - 1 >= 0 && is_mid(fi - 1, nfy, g.cy);
    if (mE) half += t[kf + 1];
    if (mW) half += t[kf - 1];
    if (mN) half += t[kf + PF];
    if (mS) half += t[kf - PF];
    if (mE && mN) half += t[kf + PF + 1];
    if (mW && mS) half += t[kf - PF - 1];
    b[w.k] = acc + T(0.5) * half;
  }
}

// x_f += P x_c (P1 interpolation of the coarse "right" mesh), on fine tiles.
// `Gc` is indexed like `G` (same trap order) and describes the coarse level.
template <class T>
__global__ void __launch_bounds__(kThreads) k_prolong(const LevelGeom* __restrict__ G,
                                                     const LevelGeom* __restrict__ Gc,
                                                     const Tile* __restrict__ tiles,
                                                     const int* __restrict__ skip,
                                                     const T* __restrict__ xc,
                                                     T* __restrict__ xf) {
  EQF_TILE_PROLOGUE(skip);
  const LevelGeom c = Gc[tile.geom];
  const int PC = c.nx + 1;
  const T* xcs = xc + c.off;
  T* xs = xf + g.off;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    int i0, i1, j0, j1;
    fine_to_coarse(w.i, g.ny, c.cy, i0, i1);
    fine_to_coarse(w.j, g.nx, c.cx, j0, j1);
    T v;
    if (i0 == i1 && j0 == j1)
      v = xcs[j0 + i0 * PC];
    else if (i0 == i1)
      v = T(0.5) * (xcs[j0 + i0 * PC] + xcs[j1 + i0 * PC]);
    else if (j0 == j1)
      v = T(0.5) * (xcs[j0 + i0 * PC] + xcs[j0 + i1 * PC]);
    else
      v = T(0.5) * (xcs[j0 + i0 * PC] + xcs[j1 + i1 * PC]);  // on the coarse diagonal
    xs[w.k] += v;
  }
}

// ---------------------------------------------------------------------------
// CG on the finest level.  Per-trap scalars live in CgState.
struct CgState {
  double rz, pq, rr, rr0, alpha, beta, bb, r64;
  int iters, sweeps, it_in_sweep, pad;
};

// p_out = z (FIRST) or z + beta p_in; q = A p_out; partial dot(p_out, q).
// p is ping-ponged because neighbours of p_out are recomputed from p_in.
template <class T, bool FIRST>
__global__ void __launch_bounds__(kThreads) k_cg_dir(const LevelGeom* __restrict__ G,
                                                    const Tile* __restrict__ tiles,
                                                    const int* __restrict__ skip,
                                                    const CgState* __restrict__ st,
                                                    const T* __restrict__ z,
                                                    const T* __restrict__ pin,
                                                    T* __restrict__ pout, T* __restrict__ q,
                                                    double* __restrict__ part) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  const T beta = FIRST ? T(0) : T(st[g.trap].beta);
  const T* zs = z + g.off;
  const T* ps = pin + g.off;
  T* po = pout + g.off;
  T* qs = q + g.off;
  const int P = g.nx + 1;
  T acc = T(0);
  auto pv = [&](int k) { return FIRST ? zs[k] : zs[k] + beta * ps[k]; };
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    const int k = w.k, i = w.i, j = w.j;
    const Sten<T> s = stencil_at<T>(g, i, j);
    const T pc = pv(k);
    T a = s.c * pc;
    if (j < g.nx) a += s.e * pv(k + 1);
    if (j > 0) a += s.w * pv(k - 1);
    if (i < g.ny) a += s.n * pv(k + P);
    if (i > 0) a += s.s * pv(k - P);
    if (i < g.ny && j < g.nx) a += s.ne * pv(k + P + 1);
    if (i > 0 && j > 0) a += s.sw * pv(k - P - 1);
    po[k] = pc;
    qs[k] = a;
    acc += pc * a;
  }
  const double t = block_sum(double(acc));
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// x += alpha p; r -= alpha q; partial dot(r, r)
template <class T>
__global__ void __launch_bounds__(kThreads) k_cg_update(const LevelGeom* __restrict__ G,
                                                       const Tile* __restrict__ tiles,
                                                       const int* __restrict__ skip,
                                                       const CgState* __restrict__ st,
                                                       const T* __restrict__ p,
                                                       const T* __restrict__ q, T* __restrict__ x,
                                                       T* __restrict__ r,
                                                       double* __restrict__ part) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  const T alpha = T(st[g.trap].alpha);
  const long long o = g.off;
  T acc = T(0);
  for (int k = tile.k0 + threadIdx.x; k < tile.k1; k += blockDim.x) {
    x[o + k] += alpha * p[o + k];
    const T rn = r[o + k] - alpha * q[o + k];
    r[o + k] = rn;
    acc += rn * rn;
  }
  const double t = block_sum(double(acc));
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// ---------------------------------------------------------------------------
// FP64 iterative refinement on the finest level.
//   FIRST: b = F + M u (stored), r = b - A u, partials |b|^2 and |r|^2
//   else : r = b - A u, partial |r|^2
// Dirichlet rows: b = 0 and r = -u (u is 0 there, so r = 0).
template <class T, bool FIRST>
__global__ void __launch_bounds__(kThreads) k_ir_residual(const LevelGeom* __restrict__ G,
                                                         const Tile* __restrict__ tiles,
                                                         const int* __restrict__ skip,
                                                         const double* __restrict__ F,
                                                         const double* __restrict__ u,
                                                         double* __restrict__ b64,
                                                         T* __restrict__ r,
                                                         double* __restrict__ part,
                                                         int ntiles) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (threadIdx.x == 0) {
      part[blockIdx.x] = 0.0;
      part[ntiles + blockIdx.x] = 0.0;
    }
    return;
  }
  const double* us = u + g.off;
  const double* Fs = F + g.off;
  double* bs = b64 + g.off;
  T* rs = r + g.off;
  const int P = g.nx + 1;
  double abb = 0.0, arr = 0.0;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    const int k = w.k, i = w.i, j = w.j;
    double bk;
    if (FIRST) {
      if (g.walls && is_dirichlet(g, i, j)) {
        bk = 0.0;
      } else {
        const Sten<double> m = mass_stencil<double>(g, i, j);
        double mu = m.c * us[k];
        if (j < g.nx) mu += m.e * us[k + 1];
        if (j > 0) mu += m.w * us[k - 1];
        if (i < g.ny) mu += m.n * us[k + P];
        if (i > 0) mu += m.s * us[k - P];
        if (i < g.ny && j < g.nx) mu += m.ne * us[k + P + 1];
        if (i > 0 && j > 0) mu += m.sw * us[k - P - 1];
        bk = Fs[k] + mu;
      }
      bs[k] = bk;
      abb += bk * bk;
    } else {
      bk = bs[k];
    }
    const Sten<double> s = stencil_at<double>(g, i, j);
    const double rk = bk - apply_node<double>(g, us, k, i, j, s);
    rs[k] = T(rk);
    arr += rk * rk;
  }
  const double tb = FIRST ? block_sum(abb) : 0.0;
  __syncthreads();
  const double tr = block_sum(arr);
  if (threadIdx.x == 0) {
    if (FIRST) part[blockIdx.x] = tb;
    part[ntiles + blockIdx.x] = tr;
  }
}

// u += x (the inner-solve correction)
template <class T>
__global__ void __launch_bounds__(kThreads) k_ir_update(const LevelGeom* __restrict__ G,
                                                       const Tile* __restrict__ tiles,
                                                       const int* __restrict__ skip,
                                                       const T* __restrict__ x,
                                                       double* __restrict__ u) {
  EQF_TILE_PROLOGUE(skip);
  const long long o = g.off;
  for (int k = tile.k0 + threadIdx.x; k < tile.k1; k += blockDim.x) u[o + k] += double(x[o + k]);
}

// ---------------------------------------------------------------------------
// Per-trap scalar phases (one thread per trap).  `range[t]` = first fine tile of
// trap t and its tile count; partials are added in tile order.
struct TileRange {
  int first, count;
};
__device__ __forceinline__ double trap_sum(const double* part, TileRange tr) {
  double s = 0.0;
  for (int i = 0; i < tr.count; ++i) s += part[tr.first + i];
  return s;
}

// After k_ir_residual: decide outer convergence, reset the inner solve.
__global__ void k_s_ir(int ntraps, const TileRange* __restrict__ range,
                       const double* __restrict__ part, int ntiles, int first_sweep, double rtol,
                       CgState* __restrict__ st, int* __restrict__ ir_done,
                       int* __restrict__ cg_skip) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps) return;
  if (ir_done[t]) {
    cg_skip[t] = 1;
    return;
  }
  CgState s = st[t];
  if (first_sweep) s.bb = trap_sum(part, range[t]);
  s.r64 = trap_sum(part + ntiles, range[t]);
  const bool conv = s.r64 <= rtol * rtol * s.bb || s.bb == 0.0;
  ir_done[t] = conv ? 1 : 0;
  cg_skip[t] = conv ? 1 : 0;
  s.rr0 = s.r64;
  s.rr = s.r64;
  s.it_in_sweep = 0;
  if (!conv) s.sweeps += 1;
  st[t] = s;
}

// After the preconditioner: rz = r.z and beta.
__global__ void k_s_rz(int ntraps, const TileRange* __restrict__ range,
                       const double* __restrict__ part, CgState* __restrict__ st,
                       const int* __restrict__ cg_skip) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || cg_skip[t]) return;
  const double rz = trap_sum(part, range[t]);
  CgState s = st[t];
  s.beta = s.it_in_sweep > 0 && s.rz != 0.0 ? rz / s.rz : 0.0;
  s.rz = rz;
  st[t] = s;
}

// After k_cg_dir: alpha = rz / pq.
__global__ void k_s_pq(int ntraps, const TileRange* __restrict__ range,
                       const double* __restrict__ part, CgState* __restrict__ st,
                       const int* __restrict__ cg_skip) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || cg_skip[t]) return;
  const double pq = trap_sum(part, range[t]);
  CgState s = st[t];
  s.pq = pq;
  s.alpha = pq != 0.0 ? s.rz / pq : 0.0;
  st[t] = s;
}

// After k_cg_update: inner convergence test |r| <= tol_rel |r0| or tol_abs^2 >= rr.
__global__ void k_s_rr(int ntraps, const TileRange* __restrict__ range,
                       const double* __restrict__ part, double tol_rel, double rtol_abs,
                       CgState* __restrict__ st, int* __restrict__ cg_skip) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || cg_skip[t]) return;
  CgState s = st[t];
  s.rr = trap_sum(part, range[t]);
  s.it_in_sweep += 1;
  s.iters += 1;
  if (s.rr <= tol_rel * tol_rel * s.rr0 || s.rr <= rtol_abs * rtol_abs * s.bb) cg_skip[t] = 1;
  st[t] = s;
}

}  // namespace eqf
