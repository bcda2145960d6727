// Temporally blocked multigrid level kernels: each computes several smoothing
// steps of one row tile in shared memory, on windows that shrink by one row (plus a
// few nodes) per step, so the level's vectors cross HBM once per half V-cycle.
//
//   k_down:  x1 = d1 = c0 D^-1 b                     (window W1 = tile +- 2 rows)
//            x2 = x1 + c_old d1 + c1 D^-1 (b - A x1) (window W2 = tile +- 1 row)
//            t  = b - A x2                           (tile)      -> writes x2, t
//   k_up:    x0 = x + P x_c                          (W1)
//            x1 = x0 + c0 D^-1 (b - A x0)            (W2)
//            x2 = x1 + c_old (x1 - x0) + c1 D^-1 (b - A x1)  (tile) -> writes x2
//
// These are the pre-smoothing (two Chebyshev-Jacobi steps from zero) + residual and
// the prolongation + post-smoothing (two steps) of a V(2,2) cycle.  k_down evaluates
// exactly the unfused sequence (same formulas, same operand order: bit-identical);
// k_up recomputes the first step's direction as x1 - x0 instead of storing it.
// Algorithmic bytes per node (FP32): k_down reads b, writes x, t (12); k_up reads x,
// b and a quarter-size x_c, writes x (13) -- against 44 and 45 for the unfused steps.
#pragma once
#include "eqf_kernels.cuh"

namespace eqf {

// Resident CTAs per SM the fused kernels are compiled for.
template <class T>
constexpr int kFusedCtas = sizeof(T) == 4 ? 3 : 2;

// Windows of the fused kernels (node ranges, multiples of 4), identical on host and
// device.  W1 = tile +- (2 rows + 16 nodes), W2 = tile +- (1 row + 8 nodes): every
// quad of W2 reads its neighbours inside W1, every quad of the tile inside W2.
struct FusedWin {
  int w1a, w1b, w2a, w2b;
};
EQF_HD FusedWin fused_win(int k0, int k1, int P) {
  FusedWin w;
  w.w1a = (k0 - 2 * P - 16) & ~3;
  w.w1b = (k1 + 2 * P + 16 + 3) & ~3;
  w.w2a = (k0 - P - 8) & ~3;
  w.w2b = (k1 + P + 8 + 3) & ~3;
  return w;
}
EQF_HD int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// Walks the quads k = ka + 4 tid, ka + 4 (tid + bd), ... of a window that may start
// before the trap (negative k), keeping (i, j) = floor-divmod(k, P).
struct WinWalk {
  int k, i, j, di, dj, P;
  __device__ __forceinline__ WinWalk(int ka, int P_) : P(P_) {
    k = ka + 4 * (int)threadIdx.x;
    i = floor_div(k, P);
    j = k - i * P;
    const int st = 4 * (int)blockDim.x;
    di = st / P;
    dj = st - di * P;
  }
  __device__ __forceinline__ void next() {
    k += 4 * (int)blockDim.x;
    i += di;
    j += dj;
    if (j >= P) {
      j -= P;
      ++i;
    }
  }
};

// The quad's nodes are all uniform-interior nodes (no tile bounds involved).
__device__ __forceinline__ bool quad_interior(const LevelGeom& g, int i, int j) {
  return !g.adv_on && i >= 2 && i <= g.ny - 2 && j >= 2 && j <= g.nx - 5;
}

// 1 / diagonal of the quad's nodes (the same values every stencil path uses).
template <class T>
__device__ __forceinline__ Q4<T> inv_diag_quad(const LevelGeom& g, const Interior<T>& ci,
                                               const T* __restrict__ stab, int P, int i0,
                                               int j0, bool inner) {
  Q4<T> id;
  if (inner) {
#pragma unroll
    for (int e = 0; e < 4; ++e) id.v[e] = ci.ic;
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      int i, j;
      quad_node(P, i0, j0, e, i, j);
      if (g.adv_on) {
        T c[8];
        coef_general<T>(g, i, j, c);
        id.v[e] = c[7];
      } else {
        id.v[e] = stab[node_class_clamped(g, i, j) * kTabStride + 7];
      }
    }
  }
  return id;
}

// Zeroes the nodes of a quad that lie outside the trap's grid [0, n).
template <class T>
__device__ __forceinline__ void mask_outside(Q4<T>& q, int k, int n) {
  if (k >= 0 && k + 4 <= n) return;
#pragma unroll
  for (int e = 0; e < 4; ++e)
    if (k + e < 0 || k + e >= n) q.v[e] = T(0);
}

template <class T>
__device__ __forceinline__ T* carve(Stager& st, int count) {
  T* p = reinterpret_cast<T*>(st.cur);
  st.cur += (((uint32_t)count * sizeof(T) + 15u) & ~15u) + 16u;
  return p;
}

// Pre-smoothing (two steps from zero) and residual of one row tile.
template <class T>
__global__ void __launch_bounds__(kThreads, kFusedCtas<T>)
    k_down(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
           const T* __restrict__ tabs, const int* __restrict__ skip, const T* __restrict__ b,
           T* __restrict__ x, T* __restrict__ t,
           unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) return;
  count_work(work, tile);
  const ChebCoef c0 = cheb_at(g, 0), c1 = cheb_at(g, 1);
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  const int P = g.nx + 1, n = P * (g.ny + 1), na = padded_len(g);
  const FusedWin w = fused_win(tile.k0, tile.k1, P);
  Stager st(eqf_smem);
  const View<T> bv = st.add_guarded(b + g.off, w.w1a, w.w1b, na);
  T* x1p = carve<T>(st, w.w1b - w.w1a);
  T* x2p = carve<T>(st, w.w2b - w.w2a);
  const T* stab = stage_table<T>(st, tab, ci);
  if (!st.run()) return;
  const View<T> x1v{x1p, w.w1a}, x2v{x2p, w.w2a};
  // step 1 from zero (pointwise) on W1
  for (WinWalk q(w.w1a, P); q.k < w.w1b; q.next()) {
    const Q4<T> bq = bv.quad(q.k);
    const Q4<T> id = inv_diag_quad<T>(g, ci, stab, P, q.i, q.j, quad_interior(g, q.i, q.j));
    Q4<T> d;
#pragma unroll
    for (int e = 0; e < 4; ++e) d.v[e] = (T(c0.c_res) * bq.v[e]) * id.v[e];
    mask_outside(d, q.k, n);
    vst4<T>(x1p + (q.k - w.w1a), d);
  }
  __syncthreads();
  // step 2 on W2 (d1 = x1)
  pitch_dispatch(P, [&](auto pm_) {
    constexpr int PM = decltype(pm_)::value;
    for (WinWalk q(w.w2a, P); q.k < w.w2b; q.next()) {
      Q4<T> xc, id;
      const Q4<T> ax = apply_quad<T, PM>(g, ci, stab, x1v, q.k, P, q.i, q.j,
                                     quad_interior(g, q.i, q.j), xc, id);
      const Q4<T> bq = bv.quad(q.k);
      Q4<T> xn;
#pragma unroll
      for (int e = 0; e < 4; ++e)
        xn.v[e] = xc.v[e] + cheb_dir<T, false>(c1, bq.v[e], ax.v[e], id.v[e], xc.v[e]);
      mask_outside(xn, q.k, n);
      vst4<T>(x2p + (q.k - w.w2a), xn);
    }
  });
  __syncthreads();
  // residual on the tile; store x2 and t
  T* xs = x + g.off;
  T* ts = t + g.off;
  const QuadGeom qg(g, tile);
  pitch_dispatch(P, [&](auto pm_) {
    constexpr int PM = decltype(pm_)::value;
    for (QuadWalk q(g, tile.k0 >> 2); 4 * q.q < tile.k1; q.next()) {
      const int k = 4 * q.q;
      const bool full = k >= tile.k0 && k + 4 <= tile.k1;
      Q4<T> xc, id;
      const Q4<T> ax =
          apply_quad<T, PM>(g, ci, stab, x2v, k, P, q.i, q.j, qg.interior(k, q.i, q.j), xc, id);
      const Q4<T> bq = bv.quad(k);
      Q4<T> r;
#pragma unroll
      for (int e = 0; e < 4; ++e) r.v[e] = bq.v[e] - ax.v[e];
      if (full) {
        vst4<T>(xs + k, xc);
        vst4<T>(ts + k, r);
      } else {
        store_masked<T>(xs, xc, k, tile.k0, tile.k1);
        store_masked<T>(ts, r, k, tile.k0, tile.k1);
      }
    }
  });
}

// Coarse rows a fused up-kernel tile stages: those the prolongation of the fine rows
// of W1 (clamped to the grid) reads.
EQF_HD void up_coarse_rows(const LevelGeom& g, const LevelGeom& c, const FusedWin& w, int& lo,
                           int& hi) {
  const int P = g.nx + 1;
  int fa = floor_div(w.w1a, P), fb = floor_div(w.w1b - 1, P);
  fa = fa < 0 ? 0 : (fa > g.ny ? g.ny : fa);
  fb = fb < 0 ? 0 : (fb > g.ny ? g.ny : fb);
  auto f2c_lo = [](int f, int nf, int h) {
    return !h ? f : ((f & 1) == 0 ? f / 2 : (f == nf ? (f + 1) / 2 : (f - 1) / 2));
  };
  auto f2c_hi = [](int f, int nf, int h) {
    return !h ? f : ((f & 1) == 0 ? f / 2 : (f == nf ? (f + 1) / 2 : (f - 1) / 2 + 1));
  };
  lo = f2c_lo(fa, g.ny, c.cy);
  hi = f2c_hi(fb, g.ny, c.cy);
}

// Prolongation and post-smoothing (two steps) of one row tile: reads x (xin) and the
// coarse correction, writes x2 to xout (another buffer: neighbouring tiles still
// stage xin).  DOT adds a partial of b.x2 (r.z of the Krylov iteration).
template <class T, bool DOT>
__global__ void __launch_bounds__(kThreads, kFusedCtas<T>)
    k_up(const LevelGeom* __restrict__ G, const LevelGeom* __restrict__ Gc,
         const Tile* __restrict__ tiles, const T* __restrict__ tabs,
         const int* __restrict__ skip, const T* __restrict__ xc,
         const T* __restrict__ b, const T* __restrict__ xin, T* __restrict__ xout,
         double* __restrict__ part, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (DOT && threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  count_work(work, tile);
  const LevelGeom& c = Gc[tile.geom];
  const ChebCoef c0 = cheb_at(g, 0), c1 = cheb_at(g, 1);
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  const int P = g.nx + 1, n = P * (g.ny + 1), na = padded_len(g);
  const int PC = c.nx + 1;
  const FusedWin w = fused_win(tile.k0, tile.k1, P);
  int clo, chi;
  up_coarse_rows(g, c, w, clo, chi);
  Stager st(eqf_smem);
  const View<T> xv = st.add_guarded(xin + g.off, w.w1a, w.w1b, na);
  const View<T> bv = st.add_guarded(b + g.off, w.w2a, w.w2b, na);
  const View<T> cv = st.add(xc + c.off, clo * PC, (chi + 1) * PC, padded_len(c));
  T* x1p = carve<T>(st, w.w2b - w.w2a);
  const T* stab = stage_table<T>(st, tab, ci);
  if (!st.run()) return;
  // x0 = x + P x_c on W1 (in place; nodes outside the grid stay zero)
  {
    T* x0 = const_cast<T*>(xv.p);
    const int ka = w.w1a > 0 ? w.w1a : 0, kb = w.w1b < n ? w.w1b : n;
    for (int k = ka + (int)threadIdx.x; k < kb; k += blockDim.x) {
      const int i = k / P, j = k - i * P;
      int i0, i1, j0, j1;
      fine_to_coarse(i, g.ny, c.cy, i0, i1);
      fine_to_coarse(j, g.nx, c.cx, j0, j1);
      T v;
      if (i0 == i1 && j0 == j1)
        v = cv[j0 + i0 * PC];
      else if (i0 == i1)
        v = T(0.5) * (cv[j0 + i0 * PC] + cv[j1 + i0 * PC]);
      else if (j0 == j1)
        v = T(0.5) * (cv[j0 + i0 * PC] + cv[j0 + i1 * PC]);
      else
        v = T(0.5) * (cv[j0 + i0 * PC] + cv[j1 + i1 * PC]);
      x0[k - xv.a] += v;
    }
  }
  __syncthreads();
  const View<T> x1v{x1p, w.w2a};
  // first step (no previous direction) on W2
  pitch_dispatch(P, [&](auto pm_) {
    constexpr int PM = decltype(pm_)::value;
    for (WinWalk q(w.w2a, P); q.k < w.w2b; q.next()) {
      Q4<T> x0q, id;
      const Q4<T> ax = apply_quad<T, PM>(g, ci, stab, xv, q.k, P, q.i, q.j,
                                     quad_interior(g, q.i, q.j), x0q, id);
      const Q4<T> bq = bv.quad(q.k);
      Q4<T> xn;
#pragma unroll
      for (int e = 0; e < 4; ++e)
        xn.v[e] = x0q.v[e] + cheb_dir<T, true>(c0, bq.v[e], ax.v[e], id.v[e], T(0));
      mask_outside(xn, q.k, n);
      vst4<T>(x1p + (q.k - w.w2a), xn);
    }
  });
  __syncthreads();
  // second step on the tile, d1 = x1 - x0
  T* xo = xout + g.off;
  const QuadGeom qg(g, tile);
  T acc = T(0);
  pitch_dispatch(P, [&](auto pm_) {
    constexpr int PM = decltype(pm_)::value;
    for (QuadWalk q(g, tile.k0 >> 2); 4 * q.q < tile.k1; q.next()) {
      const int k = 4 * q.q;
      const bool full = k >= tile.k0 && k + 4 <= tile.k1;
      Q4<T> x1q, id;
      const Q4<T> ax =
          apply_quad<T, PM>(g, ci, stab, x1v, k, P, q.i, q.j, qg.interior(k, q.i, q.j), x1q, id);
      const Q4<T> bq = bv.quad(k);
      const Q4<T> x0q = xv.quad(k);
      Q4<T> xn;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        xn.v[e] = x1q.v[e] + cheb_dir<T, false>(c1, bq.v[e], ax.v[e], id.v[e], x1q.v[e] - x0q.v[e]);
        if (DOT && (full || (k + e >= tile.k0 && k + e < tile.k1))) acc += bq.v[e] * xn.v[e];
      }
      if (full)
        vst4<T>(xo + k, xn);
      else
        store_masked<T>(xo, xn, k, tile.k0, tile.k1);
    }
  });
  if (DOT) {
    const double s = block_sum(double(acc));
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

}  // namespace eqf
