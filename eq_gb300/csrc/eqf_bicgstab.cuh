// Right-preconditioned BiCGSTAB on the finest level, for traps whose operator is
// not symmetric (advection).  Same conventions as the CG kernels: one CTA per row
// tile, per-trap scalars in CgState (rz = rho, pq = rhat.v, alpha, omega, beta),
// per-tile FP64 partials added in tile order by one thread per trap, and the
// per-trap skip flag doubling as the convergence flag.
//
// One iteration (x is the correction, r its residual, rhat the shadow residual):
//   p  = r + beta (p - omega v)          k_bs_dir     (first iteration: p = r, rhat = r)
//   ph = M^-1 p                          V-cycle
//   v  = A ph, (rhat, v)                 k_apply_dot<1>
//   alpha = rho / (rhat, v)              k_s_bs_alpha
//   x += alpha ph, s = r - alpha v, |s|  k_bs_half    (s overwrites r)
//   sh = M^-1 s                          V-cycle      (skipped once |s| is small)
//   t  = A sh, (t, s), (t, t)            k_apply_dot<2>
//   omega = (t, s) / (t, t)              k_s_bs_omega
//   x += omega sh, r = s - omega t       k_bs_full    (|r|^2, (rhat, r))
//   rho' = (rhat, r), beta               k_s_bs_rho
#pragma once
#include "eqf_kernels.cuh"

namespace eqf {

// p = r (FIRST, also rhat = r and partial (rhat, r)) or p = r + beta (p - omega v)
template <class T, bool FIRST>
__global__ void __launch_bounds__(kThreads)
    k_bs_dir(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
             const int* __restrict__ skip, const CgState* __restrict__ st,
             const T* __restrict__ r, const T* __restrict__ v, T* __restrict__ p,
             T* __restrict__ rhat, double* __restrict__ part, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (skip[g.trap]) {
    if (FIRST && threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  count_work(work, tile);
  const T beta = FIRST ? T(0) : T(st[g.trap].beta);
  const T omega = FIRST ? T(0) : T(st[g.trap].omega);
  const long long o = g.off;
  T acc = T(0);
  for (int k = tile.k0 + (int)threadIdx.x; k < tile.k1; k += blockDim.x) {
    const T rk = r[o + k];
    if (FIRST) {
      p[o + k] = rk;
      rhat[o + k] = rk;
      acc += rk * rk;
    } else {
      p[o + k] = fma_(beta, fma_(-omega, v[o + k], p[o + k]), rk);
    }
  }
  if (FIRST) {
    const double t = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

// y = A x with partials: NDOT = 1: (w, y); NDOT = 2: (y, w) and (y, y) (second
// partial array at part + ntiles).
template <class T, int NDOT>
__global__ void __launch_bounds__(kThreads, kStencilCtas<T>)
    k_apply_dot(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                const T* __restrict__ tabs, const int* __restrict__ skip,
                const T* __restrict__ x, const T* __restrict__ w, T* __restrict__ y,
                double* __restrict__ part, int ntiles, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (skip[g.trap]) {
    if (threadIdx.x == 0) {
      part[blockIdx.x] = 0.0;
      if (NDOT == 2) part[ntiles + blockIdx.x] = 0.0;
    }
    return;
  }
  count_work(work, tile);
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  Stager sg(eqf_smem);
  const int na = padded_len(g);
  const View<T> xv = sg.add_guarded(x + g.off, qhalo_lo(g, tile), qhalo_hi(g, tile), na);
  const View<T> wv = sg.add(w + g.off, tile.k0, tile.k1, na);
  const TableStage<T> tst = stage_table<T>(sg, tab, ci);
  const T* stab = tst.s;
  if (!sg.run(tst)) return;
  T* ys = y + g.off;
  const int P = g.P;
  T a0 = T(0), a1 = T(0);
  // tiles are whole rows: every quad lies inside the tile
  for_quads(g, QuadBlock{tile.r0, tile.r1, 0, P >> 2}, [&](int i, int cq, auto inner_) {
    constexpr bool INNER = decltype(inner_)::value;
    const int j = 4 * cq, k = i * P + j;
    Q4<T> xc, id;
    const Q4<T> ax = apply_quad<T, 0>(g, ci, stab, xv, k, P, i, j, INNER, xc, id);
    const Q4<T> wq = wv.quad(k);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      a0 += wq.v[e] * ax.v[e];
      if (NDOT == 2) a1 += ax.v[e] * ax.v[e];
    }
    vst4<T>(ys + k, ax);
  });
  const double t0 = block_sum(a0);
  const double t1 = NDOT == 2 ? block_sum(a1) : 0.0;
  if (threadIdx.x == 0) {
    part[blockIdx.x] = t0;
    if (NDOT == 2) part[ntiles + blockIdx.x] = t1;
  }
}

// x += alpha ph; s = r - alpha v (in place of r); partial |s|^2
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_bs_half(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
              const int* __restrict__ skip, const CgState* __restrict__ st,
              const T* __restrict__ ph, const T* __restrict__ v, T* __restrict__ x,
              T* __restrict__ r, double* __restrict__ part, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (skip[g.trap]) {
    if (threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  count_work(work, tile);
  const T alpha = T(st[g.trap].alpha);
  const long long o = g.off;
  T acc = T(0);
  for (int k = tile.k0 + (int)threadIdx.x; k < tile.k1; k += blockDim.x) {
    x[o + k] = fma_(alpha, ph[o + k], x[o + k]);
    const T sk = fma_(-alpha, v[o + k], r[o + k]);
    r[o + k] = sk;
    acc += sk * sk;
  }
  const double t = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// x += omega sh; r = s - omega t; partials |r|^2 and (rhat, r)
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_bs_full(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
              const int* __restrict__ skip, const CgState* __restrict__ st,
              const T* __restrict__ sh, const T* __restrict__ t, const T* __restrict__ rhat,
              T* __restrict__ x, T* __restrict__ r, double* __restrict__ part, int ntiles,
              unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (skip[g.trap]) {
    if (threadIdx.x == 0) {
      part[blockIdx.x] = 0.0;
      part[ntiles + blockIdx.x] = 0.0;
    }
    return;
  }
  count_work(work, tile);
  const T omega = T(st[g.trap].omega);
  const long long o = g.off;
  T a0 = T(0), a1 = T(0);
  for (int k = tile.k0 + (int)threadIdx.x; k < tile.k1; k += blockDim.x) {
    x[o + k] = fma_(omega, sh[o + k], x[o + k]);
    const T rk = fma_(-omega, t[o + k], r[o + k]);
    r[o + k] = rk;
    a0 += rk * rk;
    a1 += rhat[o + k] * rk;
  }
  const double t0 = block_sum(a0);
  const double t1 = block_sum(a1);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = t0;
    part[ntiles + blockIdx.x] = t1;
  }
}

// Scalar phases (one thread per trap; `part` partials in tile order).
// After k_bs_dir<FIRST>: rho = (rhat, r) = |r|^2.
__global__ void k_s_bs_rho0(int ntraps, const TileRange* __restrict__ range,
                            const double* __restrict__ part, CgState* __restrict__ st,
                            const int* __restrict__ skip) {
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || skip[t]) return;
  st[t].rz = trap_sum(part, range[t]);
}

// After v = A ph: alpha = rho / (rhat, v); a zero denominator (breakdown) stops the
// trap's inner solve (the refinement loop restarts it from the true residual).
__global__ void k_s_bs_alpha(int ntraps, const TileRange* __restrict__ range,
                             const double* __restrict__ part, CgState* __restrict__ st,
                             int* __restrict__ skip) {
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || skip[t]) return;
  CgState s = st[t];
  s.pq = trap_sum(part, range[t]);
  if (s.pq == 0.0 || !isfinite(s.pq)) {
    skip[t] = 1;
    s.alpha = 0.0;
  } else {
    s.alpha = s.rz / s.pq;
  }
  st[t] = s;
}

// After s = r - alpha v: stop when |s| already meets the inner tolerance.
__global__ void k_s_bs_half(int ntraps, const TileRange* __restrict__ range,
                            const double* __restrict__ part, double tol_rel, double rtol_abs,
                            CgState* __restrict__ st, int* __restrict__ skip) {
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || skip[t]) return;
  CgState s = st[t];
  s.rr = trap_sum(part, range[t]);
  if (s.rr <= tol_rel * tol_rel * s.rr0 || s.rr <= rtol_abs * rtol_abs * s.bb) {
    skip[t] = 1;
    s.it_in_sweep += 1;
    s.iters += 1;
  }
  st[t] = s;
}

// After t = A sh: omega = (t, s) / (t, t).
__global__ void k_s_bs_omega(int ntraps, const TileRange* __restrict__ range,
                             const double* __restrict__ part, int ntiles,
                             CgState* __restrict__ st, int* __restrict__ skip) {
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || skip[t]) return;
  const double ts = trap_sum(part, range[t]);
  const double tt = trap_sum(part + ntiles, range[t]);
  if (tt == 0.0 || !isfinite(tt) || ts == 0.0) {
    skip[t] = 1;
    st[t].omega = 0.0;
    return;
  }
  st[t].omega = ts / tt;
}

// After r = s - omega t: convergence, rho' = (rhat, r), beta = rho'/rho * alpha/omega.
__global__ void k_s_bs_rho(int ntraps, const TileRange* __restrict__ range,
                           const double* __restrict__ part, int ntiles, double tol_rel,
                           double rtol_abs, CgState* __restrict__ st, int* __restrict__ skip) {
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || skip[t]) return;
  CgState s = st[t];
  s.rr = trap_sum(part, range[t]);
  const double rho = trap_sum(part + ntiles, range[t]);
  s.it_in_sweep += 1;
  s.iters += 1;
  if (s.rr <= tol_rel * tol_rel * s.rr0 || s.rr <= rtol_abs * rtol_abs * s.bb || rho == 0.0 ||
      !isfinite(rho))
    skip[t] = 1;
  s.beta = s.rz != 0.0 ? (rho / s.rz) * (s.alpha / s.omega) : 0.0;
  s.rz = rho;
  st[t] = s;
}

}  // namespace eqf
