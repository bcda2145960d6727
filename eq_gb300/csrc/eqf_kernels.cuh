// Tile kernels of the trap field solver: matrix-free operator, Chebyshev-Jacobi
// smoothing, multigrid transfers, CG vector updates and the FP64 residual of the
// iterative-refinement loop.
//
// Work decomposition: every kernel runs one CTA per tile of a level's tile list;
// a tile is a block of whole rows of one trap, so one launch covers every trap of
// a batch.  Kernels that read neighbours stage their inputs (tile rows plus one
// halo row each side) into shared memory with bulk asynchronous copies
// (cp.async.bulk completed on one mbarrier), then compute from shared memory and
// store coalesced.  Rows outside the trap are zero-filled guard rows, so every
// node reads its seven neighbours without branches; the coefficients come from a
// per-trap table indexed by (row class, column class), classes {0, 1, interior,
// n-1, n}, which on a tensor grid with a ragged last cell determines the stencil
// exactly (walls and last-cell sizes included).  A per-trap skip flag lets
// converged traps drop out without changing the launch sequence.  Reductions are
// deterministic: each tile writes one FP64 partial and the per-trap scalar
// kernels add a trap's partials in tile order.
#pragma once
#include "eqf_common.cuh"

namespace eqf {

constexpr int kThreads = 256;
constexpr int kTabStride = 8;                 // c, e, w, n, s, ne, sw, 1/c
constexpr int kTabPerTrap = 25 * kTabStride;  // 5 x 5 node classes

// Device-side error flag: set when a bounded wait gives up (never expected).
__device__ int g_eqf_device_error = 0;

// ---------------------------------------------------------------------------
// Bulk-copy staging (global -> shared) completed on one mbarrier.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// A staged range of one array: node k (trap-relative) lives at p[k - a].
template <class T>
struct View {
  const T* p;
  int a;
  __device__ __forceinline__ T operator[](int k) const { return p[k - a]; }
};

constexpr int kMaxStaged = 4;
constexpr int kMaxGuards = 2 * kMaxStaged;

// Plans up to kMaxStaged ranges in dynamic shared memory; thread 0 then issues
// them as bulk copies.  Ranges are widened to 16-byte boundaries; trap segments
// are padded to 32 elements, so a widened range stays inside the allocation.
// Guarded ranges may reach outside [0, nalloc): those parts are zero-filled.
struct Stager {
  uint64_t* bar;
  char* cur;
  uint32_t total;
  int n, ng;
  const void* src[kMaxStaged];
  void* dst[kMaxStaged];
  uint32_t bytes[kMaxStaged];
  char* gptr[kMaxGuards];  // zero-fill regions (16-byte granules)
  uint32_t gbytes[kMaxGuards];

  __device__ __forceinline__ explicit Stager(char* smem) {
    bar = reinterpret_cast<uint64_t*>(smem);
    cur = smem + 16;
    total = 0;
    n = 0;
    ng = 0;
  }
  __device__ __forceinline__ void copy(const void* s, void* d, uint32_t nb) {
    if (nb) {
      src[n] = s;
      dst[n] = d;
      bytes[n] = nb;
      ++n;
      total += nb;
    }
  }
  // nodes [ka, kb) of `base` (trap-relative, inside [0, nalloc))
  template <class T>
  __device__ __forceinline__ View<T> add(const T* base, int ka, int kb, int nalloc) {
    constexpr int V = 16 / sizeof(T);
    const int a = (ka / V) * V;
    int b = ((kb + V - 1) / V) * V;
    b = b < nalloc ? b : nalloc;
    T* d = reinterpret_cast<T*>(cur);
    const uint32_t nb = b > a ? (uint32_t)(b - a) * (uint32_t)sizeof(T) : 0u;
    copy(base + a, d, nb);
    cur += (nb + 15u) & ~15u;
    return View<T>{d, a};
  }
  // nodes [ka, kb) with ka possibly < 0 and kb possibly > nalloc; the parts
  // outside [0, nalloc) read as zero
  template <class T>
  __device__ __forceinline__ View<T> add_guarded(const T* base, int ka, int kb, int nalloc) {
    constexpr int V = 16 / sizeof(T);
    const int wa = ka >= 0 ? (ka / V) * V : -(((-ka) + V - 1) / V) * V;
    const int wb = ((kb + V - 1) / V) * V;
    const int ca = wa > 0 ? wa : 0;
    const int cb = wb < nalloc ? wb : nalloc;
    T* d = reinterpret_cast<T*>(cur);
    if (cb > ca) copy(base + ca, d + (ca - wa), (uint32_t)(cb - ca) * sizeof(T));
    if (ca > wa) {
      gptr[ng] = reinterpret_cast<char*>(d);
      gbytes[ng++] = (uint32_t)(ca - wa) * sizeof(T);
    }
    const int lo = cb > ca ? cb : ca;
    if (wb > lo) {
      gptr[ng] = reinterpret_cast<char*>(d + (lo - wa));
      gbytes[ng++] = (uint32_t)(wb - lo) * sizeof(T);
    }
    cur += ((uint32_t)(wb - wa) * sizeof(T) + 15u) & ~15u;
    return View<T>{d, wa};
  }
  // Zero the guards, issue the copies and wait for them (bounded).  Returns
  // false, uniformly for the CTA, if the wait gave up (device error flag set).
  __device__ __forceinline__ bool run() {
    if (threadIdx.x == 0) mbar_init(bar, 1);
    for (int q = 0; q < ng; ++q) {
      uint4* z = reinterpret_cast<uint4*>(gptr[q]);
      for (uint32_t e = threadIdx.x; e < gbytes[q] / 16u; e += blockDim.x)
        z[e] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect_tx(bar, total);
      for (int q = 0; q < n; ++q) bulk_copy_g2s(dst[q], src[q], bytes[q], bar);
    }
    bool ok = false;
    for (int it = 0; it < (1 << 22) && !ok; ++it) ok = mbar_try_wait(bar, 0);
    if (!ok) {
      // give the copies in flight one more bounded chance to land before leaving
      for (int it = 0; it < (1 << 20) && !ok; ++it) ok = mbar_try_wait(bar, 0);
      if (!ok) atomicExch(&g_eqf_device_error, 1);
    }
    return __syncthreads_and(ok ? 1 : 0) != 0;
  }
};

__device__ __forceinline__ int padded_len(const LevelGeom& g) {
  const int n = (g.nx + 1) * (g.ny + 1);
  return (n + 31) & ~31;
}

// Walks the nodes k = k0 + tid, k0 + tid + bd, ... of a tile while keeping
// (i, j) = divmod(k, nx + 1) up to date with one division per thread.
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

// ---------------------------------------------------------------------------
// Stencil evaluation.
__device__ __forceinline__ int node_class(const LevelGeom& g, int i, int j) {
  const int ci = i < 2 ? i : (i > g.ny - 2 ? 4 - (g.ny - i) : 2);
  const int cj = j < 2 ? j : (j > g.nx - 2 ? 4 - (g.nx - j) : 2);
  return ci * 5 + cj;
}

template <class T>
struct Interior {
  T c, e, n, d, ic;
};
template <class T>
__device__ __forceinline__ Interior<T> interior(const LevelGeom& g);
template <>
__device__ __forceinline__ Interior<float> interior<float>(const LevelGeom& g) {
  return Interior<float>{g.fC, g.fE, g.fN, g.fD, g.fCinv};
}
template <>
__device__ __forceinline__ Interior<double> interior<double>(const LevelGeom& g) {
  return Interior<double>{g.cC, g.cE, g.cN, g.cD, g.cCinv};
}

// Advection rows: the full stencil from the cell sizes and the local velocity
// (out of line; only traps with advection take it, uniformly per CTA).
template <class T, class X>
__device__ __noinline__ T apply_general(const LevelGeom& g, const X& x, int k, int i, int j,
                                        T& idiag) {
  const Sten<T> s = stencil_general<T>(g, i, j);
  idiag = T(1) / s.c;
  const int P = g.nx + 1;
  return s.c * x[k] + s.e * x[k + 1] + s.w * x[k - 1] + s.n * x[k + P] + s.s * x[k - P] +
         s.ne * x[k + P + 1] + s.sw * x[k - P - 1];
}
template <class T>
__device__ __noinline__ T inv_diag_general(const LevelGeom& g, int i, int j) {
  return T(1) / stencil_general<T>(g, i, j).c;
}

// (A x)_k and 1/diagonal of node (i, j).  Every neighbour index must be readable
// (staged with guard rows); missing neighbours carry zero coefficients.
// MASS: the table holds a class-based operator that advection never changes.
template <class T, class X, bool MASS = false>
__device__ __forceinline__ T apply_tab(const LevelGeom& g, const Interior<T>& ci,
                                       const T* __restrict__ tab, const X& x, int k, int i,
                                       int j, T& idiag) {
  if (!MASS && g.adv_on) return apply_general<T, X>(g, x, k, i, j, idiag);
  const int P = g.nx + 1;
  const T x0 = x[k], xe = x[k + 1], xw = x[k - 1], xn = x[k + P], xs = x[k - P];
  const T xne = x[k + P + 1], xsw = x[k - P - 1];
  if (__all_sync(__activemask(), is_uniform_interior(g, i, j))) {
    idiag = ci.ic;
    return ci.c * x0 + ci.e * (xe + xw) + ci.n * (xn + xs) + ci.d * (xne + xsw);
  }
  const T* c = tab + node_class(g, i, j) * kTabStride;
  idiag = c[7];
  return c[0] * x0 + c[1] * xe + c[2] * xw + c[3] * xn + c[4] * xs + c[5] * xne + c[6] * xsw;
}

template <class T>
__device__ __forceinline__ T inv_diag_tab(const LevelGeom& g, const Interior<T>& ci,
                                          const T* __restrict__ tab, int i, int j) {
  if (g.adv_on) return inv_diag_general<T>(g, i, j);
  return is_uniform_interior(g, i, j) ? ci.ic : tab[node_class(g, i, j) * kTabStride + 7];
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
  __syncthreads();
  return t;  // valid in thread 0
}

// Optional profiling counter: nodes actually processed by a launch (tiles of
// skipped traps do not count).  One atomic per CTA, only when profiling.
__device__ __forceinline__ void count_work(unsigned long long* work, const Tile& t) {
  if (work && threadIdx.x == 0) atomicAdd(work, (unsigned long long)(t.k1 - t.k0));
}

extern __shared__ __align__(16) char eqf_smem[];

// halo window of a tile: one row plus one node each side (may leave the trap)
__device__ __forceinline__ int halo_lo(const LevelGeom& g, const Tile& t) {
  return t.k0 - g.nx - 2;
}
__device__ __forceinline__ int halo_hi(const LevelGeom& g, const Tile& t) {
  return t.k1 + g.nx + 2;
}

// ---------------------------------------------------------------------------
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
//   ZERO (x_in = 0): x_out = d = D^-1 b / theta            (streaming, no staging)
//   FIRST:           d = D^-1 (b - A x_in) / theta; x_out = x_in + d
//   otherwise:       d = c_old d + c_res D^-1 (b - A x_in); x_out = x_in + d
// `ratio` > 0 selects the smoothing interval [lmax/ratio, lmax], else the full
// interval [lmin, lmax] (coarsest-level solve).  DOT adds a partial of b.x_out.
template <class T, bool FIRST, bool ZERO, bool DOT>
__global__ void __launch_bounds__(kThreads)
    k_cheb(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
           const T* __restrict__ tabs, const int* __restrict__ skip, float ratio, int step,
           const T* __restrict__ b, const T* __restrict__ xin, T* __restrict__ xout,
           T* __restrict__ d, double* __restrict__ part, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (DOT && threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  count_work(work, tile);
  const float lmax = g.lam_max, lmin = ratio > 0.f ? g.lam_max / ratio : g.lam_min;
  const ChebCoef cc = cheb_coef(lmin, lmax, FIRST ? 0 : step);
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  const T* bs = b + g.off;
  T* xo = xout + g.off;
  T* ds = d + g.off;
  T acc = T(0);
  if (ZERO) {
    for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
      const T bk = bs[w.k];
      const T dn = T(cc.c_res) * bk * inv_diag_tab<T>(g, ci, tab, w.i, w.j);
      xo[w.k] = dn;
      ds[w.k] = dn;
      if (DOT) acc += bk * dn;
    }
  } else {
    Stager st(eqf_smem);
    const int na = padded_len(g);
    const View<T> xv = st.add_guarded(xin + g.off, halo_lo(g, tile), halo_hi(g, tile), na);
    const View<T> bv = st.add(bs, tile.k0, tile.k1, na);
    View<T> dv = bv;
    if (!FIRST) dv = st.add(static_cast<const T*>(ds), tile.k0, tile.k1, na);
    if (!st.run()) return;
    for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
      const T bk = bv[w.k];
      T id;
      const T r = bk - apply_tab<T>(g, ci, tab, xv, w.k, w.i, w.j, id);
      T dn = T(cc.c_res) * r * id;
      if (!FIRST) dn += T(cc.c_old) * dv[w.k];
      const T xn = xv[w.k] + dn;
      xo[w.k] = xn;
      ds[w.k] = dn;
      if (DOT) acc += bk * xn;
    }
  }
  if (DOT) {
    const double t = block_sum(double(acc));
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

// t = b - A x
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_resid(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
            const T* __restrict__ tabs, const int* __restrict__ skip, const T* __restrict__ b,
            const T* __restrict__ x, T* __restrict__ t, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) return;
  count_work(work, tile);
  Stager st(eqf_smem);
  const int na = padded_len(g);
  const View<T> xv = st.add_guarded(x + g.off, halo_lo(g, tile), halo_hi(g, tile), na);
  const View<T> bv = st.add(b + g.off, tile.k0, tile.k1, na);
  if (!st.run()) return;
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  T* ts = t + g.off;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    T id;
    ts[w.k] = bv[w.k] - apply_tab<T>(g, ci, tab, xv, w.k, w.i, w.j, id);
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
// Coarse Dirichlet nodes get 0.  Fine rows f(r0)-1 .. f(r1-1)+1 are staged.
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_restrict(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
               const int* __restrict__ skip, const T* __restrict__ tf, T* __restrict__ bc,
               unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) return;
  count_work(work, tile);
  const int nfx = g.fine_nx, nfy = g.fine_ny, PF = nfx + 1;
  int fr0 = coarse_to_fine(tile.r0, nfy, g.cy) - 1;
  int fr1 = coarse_to_fine(tile.r1 - 1, nfy, g.cy) + 2;
  fr0 = fr0 < 0 ? 0 : fr0;
  fr1 = fr1 > nfy + 1 ? nfy + 1 : fr1;
  const int naf = (((nfx + 1) * (nfy + 1)) + 31) & ~31;
  Stager st(eqf_smem);
  const View<T> t = st.add(tf + g.fine_off, fr0 * PF, fr1 * PF, naf);
  if (!st.run()) return;
  T* b = bc + g.off;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    if (g.walls && is_dirichlet(g, w.i, w.j)) {
      b[w.k] = T(0);
      continue;
    }
    const int fi = coarse_to_fine(w.i, nfy, g.cy), fj = coarse_to_fine(w.j, nfx, g.cx);
    const int kf = fj + fi * PF;
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
    b[w.k] = t[kf] + T(0.5) * half;
  }
}

// x_f += P x_c (P1 interpolation of the coarse "right" mesh), on fine tiles.
// `Gc` is indexed like `G` (same trap order) and describes the coarse level.
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_prolong(const LevelGeom* __restrict__ G, const LevelGeom* __restrict__ Gc,
              const Tile* __restrict__ tiles, const int* __restrict__ skip,
              const T* __restrict__ xc, T* __restrict__ xf, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) return;
  count_work(work, tile);
  const LevelGeom& c = Gc[tile.geom];
  const int PC = c.nx + 1;
  int lo0, hi0, lo1, hi1;
  fine_to_coarse(tile.r0, g.ny, c.cy, lo0, hi0);
  fine_to_coarse(tile.r1 - 1, g.ny, c.cy, lo1, hi1);
  Stager st(eqf_smem);
  const View<T> xcs = st.add(xc + c.off, lo0 * PC, (hi1 + 1) * PC, padded_len(c));
  if (!st.run()) return;
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

// Coarsest-level solve: one CTA per trap runs `deg` Chebyshev-Jacobi iterations
// on [lmin, lmax] from zero entirely in shared memory.  Layout after the staged
// rhs: two iterate buffers with gpad >= P+1 zero guard nodes each side, and d.
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_coarse_solve(const LevelGeom* __restrict__ G, const T* __restrict__ tabs,
                   const int* __restrict__ skip, int deg, const T* __restrict__ b,
                   T* __restrict__ xout) {
  const LevelGeom& g = G[blockIdx.x];
  if (skip && skip[g.trap]) return;
  const int n = (g.nx + 1) * (g.ny + 1);
  const int na = padded_len(g);
  const int gpad = ((g.nx + 2 + 7) / 8) * 8;
  Stager st(eqf_smem);
  const View<T> bv = st.add(b + g.off, 0, n, na);
  T* xa = reinterpret_cast<T*>(st.cur) + gpad;
  T* xb = xa + na + 2 * gpad;
  T* dd = xb + na + gpad;
  // zero both iterate buffers with their guards (disjoint from the staged rhs)
  for (int e = threadIdx.x; e < 2 * (na + 2 * gpad); e += blockDim.x) (xa - gpad)[e] = T(0);
  if (!st.run()) return;
  const View<T> xav{xa, 0}, xbv{xb, 0};
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  for (int it = 0; it < deg; ++it) {
    const ChebCoef cc = cheb_coef(g.lam_min, g.lam_max, it);
    const View<T>& xi = (it & 1) ? xbv : xav;
    T* xo = (it & 1) ? xa : xb;
    for (NodeWalk w(g, 0); w.k < n; w.next()) {
      T id;
      const T ax = apply_tab<T>(g, ci, tab, xi, w.k, w.i, w.j, id);
      T dn = T(cc.c_res) * (bv[w.k] - ax) * id;
      if (it > 0) dn += T(cc.c_old) * dd[w.k];
      dd[w.k] = dn;
      xo[w.k] = xi[w.k] + dn;
    }
    __syncthreads();
  }
  const T* xf = (deg & 1) ? xb : xa;
  T* out = xout + g.off;
  for (int k = threadIdx.x; k < n; k += blockDim.x) out[k] = xf[k];
}

// ---------------------------------------------------------------------------
// CG on the finest level.  Per-trap scalars live in CgState.
struct CgState {
  double rz, pq, rr, rr0, alpha, beta, bb, r64;
  double gamma;     // extrapolation factor of the initial guess
  double dn2_prev;  // |increment|^2 of the previous step
  int iters, sweeps, it_in_sweep, pad;
};

// p_out = z (FIRST) or z + beta p_in; q = A p_out; partial dot(p_out, q).
// p is ping-ponged because neighbours of p_out are recomputed from p_in.
template <class T, bool FIRST>
__global__ void __launch_bounds__(kThreads)
    k_cg_dir(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
             const T* __restrict__ tabs, const int* __restrict__ skip,
             const CgState* __restrict__ st, const T* __restrict__ z, const T* __restrict__ pin,
             T* __restrict__ pout, T* __restrict__ q, double* __restrict__ part,
             unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  count_work(work, tile);
  const T beta = FIRST ? T(0) : T(st[g.trap].beta);
  Stager sg(eqf_smem);
  const int na = padded_len(g);
  const int ka = halo_lo(g, tile), kb = halo_hi(g, tile);
  const View<T> zv = sg.add_guarded(z + g.off, ka, kb, na);
  View<T> pv = zv;
  if (!FIRST) pv = sg.add_guarded(pin + g.off, ka, kb, na);
  if (!sg.run()) return;
  struct PV {
    View<T> z, p;
    T beta;
    __device__ __forceinline__ T operator[](int k) const {
      return FIRST ? z[k] : z[k] + beta * p[k];
    }
  } pnew{zv, pv, beta};
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  T* po = pout + g.off;
  T* qs = q + g.off;
  T acc = T(0);
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    const T pc = pnew[w.k];
    T id;
    const T a = apply_tab<T>(g, ci, tab, pnew, w.k, w.i, w.j, id);
    po[w.k] = pc;
    qs[w.k] = a;
    acc += pc * a;
  }
  const double t = block_sum(double(acc));
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// x += alpha p; r -= alpha q; partial dot(r, r)   (streaming)
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_cg_update(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                const int* __restrict__ skip, const CgState* __restrict__ st,
                const T* __restrict__ p, const T* __restrict__ q, T* __restrict__ x,
                T* __restrict__ r, double* __restrict__ part, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  count_work(work, tile);
  const T alpha = T(st[g.trap].alpha);
  const long long o = g.off;
  T acc = T(0);
#pragma unroll 4
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
// FP64 iterative refinement on the finest level.  One step reads the field from
// u_in and writes the new field to u_out (the buffers swap every step, so halo
// reads of u_in never race with writes).  d_in / d_out hold the previous and the
// current step's increment (FP32), used as the extrapolated initial guess.

// First residual of a step (partials: [0] |b|^2, [1] |r|^2):
//   b = F + M u_in (stored), u0 = u_in + gamma d_in, u_out = u0, d_out = gamma d_in,
//   r = b - A u0.  Dirichlet rows: b = 0, r = 0.
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_ir_first(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
               const double* __restrict__ tabA, const double* __restrict__ tabM,
               const CgState* __restrict__ st, const double* __restrict__ F,
               const double* __restrict__ u_in, const float* __restrict__ d_in,
               double* __restrict__ b64, double* __restrict__ u_out, float* __restrict__ d_out,
               T* __restrict__ r, double* __restrict__ part, int ntiles,
               unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  count_work(work, tile);
  const double gamma = st[g.trap].gamma;
  Stager sg(eqf_smem);
  const int na = padded_len(g);
  const int ka = halo_lo(g, tile), kb = halo_hi(g, tile);
  const View<double> uv = sg.add_guarded(u_in + g.off, ka, kb, na);
  const View<double> fv = sg.add(F + g.off, tile.k0, tile.k1, na);
  const View<float> dv = sg.add_guarded(d_in + g.off, ka, kb, na);
  // the extrapolated guess u0 = u_in + gamma d_in over the window, formed once
  double* u0p = reinterpret_cast<double*>(sg.cur);
  if (!sg.run()) return;
  for (int k = ka + (int)threadIdx.x; k < kb; k += blockDim.x)
    u0p[k - ka] = uv[k] + gamma * (double)dv[k];
  __syncthreads();
  const View<double> u0{u0p, ka};
  const double* tA = tabA + (size_t)g.trap * kTabPerTrap;
  const double* tM = tabM + (size_t)g.trap * kTabPerTrap;
  const Interior<double> ci = interior<double>(g);
  const Interior<double> cm{g.mC, g.mE, g.mN, g.mD, 0.0};
  double* bs = b64 + g.off;
  double* uo = u_out + g.off;
  float* dout = d_out + g.off;
  T* rs = r + g.off;
  double abb = 0.0, arr = 0.0;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    const int k = w.k;
    double id;
    const double mu = apply_tab<double, View<double>, true>(g, cm, tM, uv, k, w.i, w.j, id);
    const bool dir = g.walls && is_dirichlet(g, w.i, w.j);
    const double bk = dir ? 0.0 : fv[k] + mu;
    const double rk = dir ? 0.0 : bk - apply_tab<double>(g, ci, tA, u0, k, w.i, w.j, id);
    bs[k] = bk;
    uo[k] = u0[k];
    dout[k] = (float)(u0[k] - uv[k]);
    rs[k] = T(rk);
    abb += bk * bk;
    arr += rk * rk;
  }
  const double tb = block_sum(abb);
  const double tr = block_sum(arr);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = tb;
    part[ntiles + blockIdx.x] = tr;
  }
}

// Later residuals of a step: r = b - A u (partial [1] |r|^2).  With FINAL the
// residual is only measured (not stored) and every trap also reports |d|^2
// (partial [2]) for the next step's extrapolation factor.
template <class T, bool FINAL>
__global__ void __launch_bounds__(kThreads)
    k_ir_residual(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                  const double* __restrict__ tabA, const int* __restrict__ skip,
                  const double* __restrict__ b64, const double* __restrict__ u,
                  const float* __restrict__ dcur, T* __restrict__ r, double* __restrict__ part,
                  int ntiles, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  const bool skipped = skip && skip[g.trap];
  if (skipped && !FINAL) {
    if (threadIdx.x == 0) part[ntiles + blockIdx.x] = 0.0;
    return;
  }
  double arr = 0.0, add = 0.0;
  if (FINAL) {
    const float* ds = dcur + g.off;
    for (int k = tile.k0 + threadIdx.x; k < tile.k1; k += blockDim.x) {
      const double v = ds[k];
      add += v * v;
    }
  }
  if (!skipped) {
    count_work(work, tile);
    Stager sg(eqf_smem);
    const int na = padded_len(g);
    const View<double> uv = sg.add_guarded(u + g.off, halo_lo(g, tile), halo_hi(g, tile), na);
    const View<double> bv = sg.add(b64 + g.off, tile.k0, tile.k1, na);
    if (!sg.run()) return;
    const double* tA = tabA + (size_t)g.trap * kTabPerTrap;
    const Interior<double> ci = interior<double>(g);
    T* rs = r + g.off;
    for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
      double id;
      const bool dir = g.walls && is_dirichlet(g, w.i, w.j);
      const double rk =
          dir ? 0.0 : bv[w.k] - apply_tab<double>(g, ci, tA, uv, w.k, w.i, w.j, id);
      if (!FINAL) rs[w.k] = T(rk);
      arr += rk * rk;
    }
  }
  const double tr = block_sum(arr);
  const double td = FINAL ? block_sum(add) : 0.0;
  if (threadIdx.x == 0) {
    part[ntiles + blockIdx.x] = tr;
    if (FINAL) part[2 * ntiles + blockIdx.x] = td;
  }
}

// u += x; d += x (the inner-solve correction)   (streaming)
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_ir_update(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                const int* __restrict__ skip, const T* __restrict__ x, double* __restrict__ u,
                float* __restrict__ d, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) return;
  count_work(work, tile);
  const long long o = g.off;
#pragma unroll 4
  for (int k = tile.k0 + threadIdx.x; k < tile.k1; k += blockDim.x) {
    const T v = x[o + k];
    u[o + k] += double(v);
    d[o + k] += float(v);
  }
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

// After a refinement residual: decide outer convergence, reset the inner solve.
__global__ void k_s_ir(int ntraps, const TileRange* __restrict__ range,
                       const double* __restrict__ part, int ntiles, int first_sweep, double rtol,
                       CgState* __restrict__ st, int* __restrict__ ir_done,
                       int* __restrict__ cg_skip) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps) return;
  if (first_sweep) ir_done[t] = 0;
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

// After the final check: convergence verdict and the next extrapolation factor
// gamma = |d_n| / |d_{n-1}| (clamped), from the increments of the last two steps.
// update_gamma is 0 for the extra checks of adaptive sweeps: the factor belongs to
// the step, so a trap's guess never depends on what the other traps needed.
__global__ void k_s_final(int ntraps, const TileRange* __restrict__ range,
                          const double* __restrict__ part, int ntiles, double rtol,
                          CgState* __restrict__ st, int* __restrict__ ir_done,
                          int* __restrict__ fail, int update_gamma) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps) return;
  CgState s = st[t];
  if (!ir_done[t]) {
    s.r64 = trap_sum(part + ntiles, range[t]);
    if (s.r64 <= rtol * rtol * s.bb || s.bb == 0.0)
      ir_done[t] = 1;
    else
      atomicAdd(fail, 1);
  }
  if (!update_gamma) {
    st[t] = s;
    return;
  }
  const double dn2 = trap_sum(part + 2 * ntiles, range[t]);
  double gm = 0.0;
  if (dn2 > 0.0) gm = s.dn2_prev > 0.0 ? sqrt(dn2 / s.dn2_prev) : 1.0;
  s.gamma = gm > 1.5 ? 1.5 : gm;
  s.dn2_prev = dn2;
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

// After k_cg_update: inner convergence test |r| <= tol_rel |r0| or |r| <= rtol |b|.
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
