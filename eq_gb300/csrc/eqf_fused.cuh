// Temporally blocked multigrid level kernels on 2-D tiles: each computes several
// smoothing steps of one tile (rows [r0, r1) x columns [c0, c1) of one trap) in
// shared memory, on windows that shrink by one row and four columns per step, so a
// level's vectors cross HBM once per half V-cycle:
//
//   k_down:  x1 = d1 = c0 D^-1 b                     (window W1 = tile + 2 rows, 8 cols)
//            x2 = x1 + c_old d1 + c1 D^-1 (b - A x1) (window W2 = tile + 1 row, 4 cols)
//            t  = b - A x2                           (tile)      -> writes x2, t
//   k_up:    x0 = x + P x_c                          (W1)
//            x1 = x0 + c0 D^-1 (b - A x0)            (W2)
//            x2 = x1 + c_old (x1 - x0) + c1 D^-1 (b - A x1)  (tile) -> writes x2
//
// These are the pre-smoothing (two Chebyshev-Jacobi steps from zero) + residual and
// the prolongation + post-smoothing (two steps) of a V(2,2) cycle.  k_down evaluates
// exactly the step-by-step sequence (same formulas, same operand order); k_up
// recomputes the first step's direction as x1 - x0 instead of storing it.
// Algorithmic bytes per node (FP32): k_down reads b, writes x, t (12); k_up reads x,
// b and a quarter-size x_c, writes x (13) -- against 44 and 45 for the steps one by one.
//
// Windows are staged row by row with bulk copies (every device row starts 16-byte
// aligned: the row pitch is a multiple of 4 nodes); window rows and columns outside
// the grid are zero-filled and take the all-zero pad class, so they stay zero.  In
// shared memory a window row is a multiple of 4 nodes long, so the neighbour rows of
// a quad are at compile-time misalignments (0 above, 3 below).
#pragma once
#include "eqf_kernels.cuh"

namespace eqf {

// GEN: the kernel runs on the tiles of general-path traps (advection, anisotropic
// tensor: per-node weights fetched inline); otherwise on the tiles of class-table traps
// only, so the class-table kernels carry no general path at all.
// Resident CTAs per SM the fused kernels are compiled for.
template <class T>
constexpr int kFusedCtas = sizeof(T) == 4 ? 3 : 2;

// One 2-D tile of a level: rows [r0, r1), columns [c0, c1) (multiples of 4, c1 <= P).
struct Tile2 {
  int geom;
  int r0, r1, c0, c1;
};

// A staged window: rows [ra, rb), columns [ca, cb) of a trap's array, `S = cb - ca`
// nodes per shared-memory row.
struct Win {
  int ra, rb, ca, cb;
  EQF_HD int S() const { return cb - ca; }
  EQF_HD int count() const { return (rb - ra) * (cb - ca); }
};
EQF_HD Win win_grow(const Tile2& t, int rows, int cols) {
  return Win{t.r0 - rows, t.r1 + rows, t.c0 - cols, t.c1 + cols};
}

// Coarse window of the prolongation into the fine window w1 (fine rows and columns
// clamped to the grid), columns widened to multiples of 4.
EQF_HD Win up_coarse_win(const LevelGeom& g, const LevelGeom& c, const Win& w1) {
  auto f2c_lo = [](int f, int nf, int h) {
    return !h ? f : ((f & 1) == 0 ? f / 2 : (f == nf ? (f + 1) / 2 : (f - 1) / 2));
  };
  auto f2c_hi = [](int f, int nf, int h) {
    return !h ? f : ((f & 1) == 0 ? f / 2 : (f == nf ? (f + 1) / 2 : (f - 1) / 2 + 1));
  };
  auto clampi = [](int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); };
  const int fa = clampi(w1.ra, 0, g.ny), fb = clampi(w1.rb - 1, 0, g.ny);
  const int ja = clampi(w1.ca, 0, g.nx), jb = clampi(w1.cb - 1, 0, g.nx);
  Win w;
  w.ra = f2c_lo(fa, g.ny, c.cy);
  w.rb = f2c_hi(fb, g.ny, c.cy) + 1;
  w.ca = f2c_lo(ja, g.nx, c.cx) & ~3;
  w.cb = (f2c_hi(jb, g.nx, c.cx) + 1 + 3) & ~3;
  return w;
}

// Shared-memory bytes of a window (with the 16-byte pad every region keeps after it).
EQF_HD size_t win_bytes(const Win& w, int tsize) {
  return (size_t)(((long long)w.count() * tsize + 15) & ~15ll) + 16;
}

// One array's window to stage: every thread zero-fills the out-of-grid parts,
// thread 0 counts the bytes, warp 0 issues one bulk copy per in-grid row segment.
template <class T>
struct RowStage {
  const T* src;  // trap base of the array (node (0,0))
  T* dst;        // window in shared memory
  Win w;
  int P, nrows;  // array row pitch and row count (ny + 1)
  __device__ __forceinline__ uint32_t row_bytes(int r, int& a, int& b) const {
    a = w.ca > 0 ? w.ca : 0;
    b = w.cb < P ? w.cb : P;
    if (r < 0 || r >= nrows || b <= a) return 0u;
    return (uint32_t)(b - a) * (uint32_t)sizeof(T);
  }
  // Only the guard parts are touched: whole rows outside the grid, and in grid rows
  // the columns left of 0 and right of the pitch (none for an interior tile).
  __device__ __forceinline__ void zero_guards() const {
    const int S = w.S();
    const int a = w.ca > 0 ? w.ca : 0, b = w.cb < P ? w.cb : P;
    const int lw = b > a ? a - w.ca : S;  // guard columns on the left (all: empty range)
    const int rw = b > a ? w.cb - b : 0;  // and on the right
    if (lw == 0 && rw == 0 && w.ra >= 0 && w.rb <= nrows) return;
    for (int r = w.ra + (int)(threadIdx.x >> 5); r < w.rb; r += (int)(blockDim.x >> 5)) {
      T* row = dst + (r - w.ra) * S;
      if (r < 0 || r >= nrows) {
        for (int c = (int)(threadIdx.x & 31); c < S; c += 32) row[c] = T(0);
      } else {
        for (int c = (int)(threadIdx.x & 31); c < lw; c += 32) row[c] = T(0);
        for (int c = (int)(threadIdx.x & 31); c < rw; c += 32) row[S - rw + c] = T(0);
      }
    }
  }
  __device__ __forceinline__ uint32_t total() const {  // in-grid rows x in-grid columns
    const int a = w.ca > 0 ? w.ca : 0, b = w.cb < P ? w.cb : P;
    const int r0 = w.ra > 0 ? w.ra : 0, r1 = w.rb < nrows ? w.rb : nrows;
    if (b <= a || r1 <= r0) return 0u;
    return (uint32_t)(r1 - r0) * (uint32_t)(b - a) * (uint32_t)sizeof(T);
  }
  __device__ __forceinline__ void issue(uint64_t* bar) const {  // warp 0
    for (int r = w.ra + (int)threadIdx.x; r < w.rb; r += 32) {
      int a, b;
      const uint32_t n = row_bytes(r, a, b);
      if (n)
        bulk_copy_g2s(dst + (r - w.ra) * w.S() + (a - w.ca), src + (size_t)r * P + a, n, bar);
    }
  }
};

// Stages the windows on one mbarrier: warp 0 issues the row copies, then every
// thread runs `fill` (the class table: its global loads overlap the copies) and
// zero-fills the guards.  Returns false, uniformly for the CTA, if the bounded wait
// gave up (device error flag set).
template <class T, int N, class F>
__device__ __forceinline__ bool stage_rows(uint64_t* bar, const RowStage<T> (&st)[N],
                                           const F& fill) {
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    uint32_t tot = 0;
#pragma unroll
    for (int q = 0; q < N; ++q) tot += st[q].total();
    mbar_expect_tx(bar, tot);
  }
  __syncwarp();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int q = 0; q < N; ++q) st[q].issue(bar);
  }
  fill();
#pragma unroll
  for (int q = 0; q < N; ++q) st[q].zero_guards();
  bool ok = true;
  if (threadIdx.x == 0) {
    ok = false;
    for (int it = 0; it < (1 << 22) && !ok; ++it) ok = mbar_try_wait(bar, 0);
    if (!ok) {
      for (int it = 0; it < (1 << 20) && !ok; ++it) ok = mbar_try_wait(bar, 0);
      if (!ok) atomicExch(&g_eqf_device_error, 1);
    }
  }
  return __syncthreads_and(ok ? 1 : 0) != 0;
}

// The tiles (row tiles or 2-D tiles) of the traps still iterating (skip[trap] == 0):
// class-table tiles (index < nc) into idx[0, ...), general-path tiles into idx[nc, ...),
// their numbers in counts[0] and counts[1] (zeroed before).  The order within a list
// does not matter: each tile's results and partial-sum slot are its own, whichever CTA
// computes it.
template <class TT>
__global__ void k_active_tiles(const LevelGeom* __restrict__ G, const TT* __restrict__ tiles,
                               int n, int nc, const int* __restrict__ skip,
                               int* __restrict__ idx, int* __restrict__ counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || skip[G[tiles[i].geom].trap]) return;
  const int k = i < nc ? 0 : 1;
  idx[(k ? nc : 0) + atomicAdd(&counts[k], 1)] = i;
}

// Quads of a window: quad q at window row q / QW, columns 4 (q % QW) .. +3.
struct WinQuads {
  int QW, n;
  float inv;
  __device__ __forceinline__ explicit WinQuads(const Win& w) {
    QW = w.S() >> 2;
    n = (w.rb - w.ra) * QW;
    inv = __fdividef(1.0f, (float)QW);  // div_pitch corrects the floor by one
  }
  __device__ __forceinline__ void at(int q, int& row, int& cq) const {
    div_pitch(q, QW, inv, row, cq);
  }
};

// The quads of a window, for for_quads.
__device__ __forceinline__ QuadBlock win_quads(const Win& w) {
  return QuadBlock{w.ra, w.rb, w.ca, w.S() >> 2};
}

// 1 / diagonal of the quad's nodes (the same values every stencil path uses).
template <class T, int GM>
__device__ __forceinline__ Q4<T> inv_diag_quad(const LevelGeom& g, const Interior<T>& ci,
                                               const T* __restrict__ stab, int i, int j0,
                                               bool inner) {
  Q4<T> id;
  if (inner) {
#pragma unroll
    for (int e = 0; e < 4; ++e) id.v[e] = ci.ic;
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (GM == 2 || (GM == 0 && g.adv_on)) {
        T c[8];
        if (GM == 2)
          coef_node<T>(g, i, j0 + e, c);
        else
          coef_general<T>(g, i, j0 + e, c);
        id.v[e] = c[7];
      } else {
        id.v[e] = stab[node_class_clamped(g, i, j0 + e) * kTabStride + 7];
      }
    }
  }
  return id;
}

// Local index of node (i, j) in window w.
__device__ __forceinline__ int wl(const Win& w, int i, int j) {
  return (i - w.ra) * w.S() + (j - w.ca);
}

// The previous Krylov iteration's update, folded into the finest level's k_down
// (UPD): r_out = r - alpha q and x_cg += alpha p, with a partial of (r_out, r_out).
template <class T>
struct CgFold {
  const T* q;      // A p of the previous iteration
  T* rout;         // the updated residual (another buffer: neighbours still stage r)
  const T* p;      // the previous direction
  T* xcg;          // the Krylov correction
  const CgState* st;
  double* part;    // (r_out, r_out) partials by 2-D tile index
  int first;       // the sweep's first update: x_cg = alpha p (x_cg is not read or zeroed)
};

// Pre-smoothing (two steps from zero) and residual of one tile.  UPD: b = r - alpha q
// is formed on the window from the staged r and q (the same expression k_cg_update
// evaluates, so the iterates do not change), stored to cf.rout on the tile, and the
// tile's correction takes cf.xcg += alpha cf.p.
// One tile (index ti in the launch's tile array); returns kTileSkipped, kTileDone or
// kTileFailed (a staging wait gave up).
template <class T, bool GEN, bool UPD>
__device__ __forceinline__ int down_tile(const LevelGeom* __restrict__ G, const Tile2& tile,
                                         int ti, const T* __restrict__ tabs,
                                         const int* __restrict__ skip, const T* __restrict__ b,
                                         T* __restrict__ x, T* __restrict__ t,
                                         const CgFold<T>& cf, unsigned long long* work) {
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (UPD && threadIdx.x == 0) cf.part[ti] = 0.0;
    return kTileSkipped;
  }
  if (work && threadIdx.x == 0)
    atomicAdd(work, (unsigned long long)(tile.r1 - tile.r0) * (tile.c1 - tile.c0));
  const ChebCoef c0 = cheb_at(g, 0), c1 = cheb_at(g, 1);
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  const int P = g.P;
  const Win w1 = win_grow(tile, 2, 8), w2 = win_grow(tile, 1, 4);
  const Win wt = win_grow(tile, 0, 0);
  Stager st(eqf_smem);  // used for the layout (barrier + regions) and the class table
  T* bp = carve<T>(st, w1.count());
  T* x1p = carve<T>(st, w1.count());
  T* x2p = carve<T>(st, w2.count());
  const TableStage<T> tst = stage_table<T>(st, tab, ci);
  const T* stab = tst.s;
  constexpr int NS = UPD ? 2 : 1;
  RowStage<T> rs[NS];
  rs[0] = RowStage<T>{b + g.off, bp, w1, P, g.ny + 1};
  if constexpr (UPD) rs[1] = RowStage<T>{cf.q + g.off, x1p, w1, P, g.ny + 1};  // q into x1's room
  if (!stage_rows<T, NS>(st.bar, rs, tst)) return kTileFailed;
  const T alpha = UPD ? T(cf.st[g.trap].alpha) : T(0);
  const int S1 = w1.S(), S2 = w2.S();
  // (UPD: b = r - alpha q, in place) step 1 from zero (pointwise) on W1
  for_quads(g, win_quads(w1), [&](int i, int cq, auto inner_) {
    constexpr bool INNER = decltype(inner_)::value;
    const int j = w1.ca + 4 * cq, kl = (i - w1.ra) * S1 + 4 * cq;
    Q4<T> bq = vld4<T>(bp + kl);
    if constexpr (UPD) {  // each quad is visited once: the in-place update is safe
      const Q4<T> qv = vld4<T>(x1p + kl);
#pragma unroll
      for (int e = 0; e < 4; ++e) bq.v[e] = fma_(-alpha, qv.v[e], bq.v[e]);
      vst4<T>(bp + kl, bq);
    }
    const Q4<T> id = inv_diag_quad<T, kGM<GEN>>(g, ci, stab, i, j, INNER);
    Q4<T> d;
#pragma unroll
    for (int e = 0; e < 4; ++e) d.v[e] = (T(c0.c_res) * bq.v[e]) * id.v[e];
    vst4<T>(x1p + kl, d);
  });
  __syncthreads();
  // step 2 on W2 (d1 = x1)
  {
    const View<T> x1v{x1p, 0};
    for_quads(g, win_quads(w2), [&](int i, int cq, auto inner_) {
      constexpr bool INNER = decltype(inner_)::value;
      const int j = w2.ca + 4 * cq;
      Q4<T> xc, id;
      const Q4<T> ax = apply_quad<T, 0, View<T>, kGM<GEN>>(g, ci, stab, x1v,
          wl(w1, i, j), S1, i, j, INNER, xc, id);
      const Q4<T> bq = vld4<T>(bp + wl(w1, i, j));
      Q4<T> xn;
#pragma unroll
      for (int e = 0; e < 4; ++e)
        xn.v[e] = xc.v[e] + cheb_dir<T, false>(c1, bq.v[e], ax.v[e], id.v[e], xc.v[e]);
      vst4<T>(x2p + (i - w2.ra) * S2 + 4 * cq, xn);
    });
  }
  __syncthreads();
  // residual on the tile; store x2 and t (UPD: and r, x_cg)
  T acc = T(0);
  {
    const View<T> x2v{x2p, 0};
    T* xs = x + g.off;
    T* ts = t + g.off;
    for_quads(g, win_quads(wt), [&](int i, int cq, auto inner_) {
      constexpr bool INNER = decltype(inner_)::value;
      const int j = tile.c0 + 4 * cq;
      const size_t k = (size_t)i * P + j;
      [[maybe_unused]] Q4<T> pv, xv;
      if constexpr (UPD) {  // issued before the stencil: their latency overlaps it
        pv = vld4<T>(cf.p + g.off + k);
        if (!cf.first) xv = vld4<T>(cf.xcg + g.off + k);
      }
      Q4<T> xc, id;
      const Q4<T> ax = apply_quad<T, 0, View<T>, kGM<GEN>>(g, ci, stab, x2v,
          wl(w2, i, j), S2, i, j, INNER, xc, id);
      const Q4<T> bq = vld4<T>(bp + wl(w1, i, j));
      Q4<T> r;
#pragma unroll
      for (int e = 0; e < 4; ++e) r.v[e] = bq.v[e] - ax.v[e];
      vst4<T>(xs + k, xc);
      vst4<T>(ts + k, r);
      if constexpr (UPD) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          // from a zero correction fma(alpha, p, 0) is the rounded product itself
          xv.v[e] = cf.first ? alpha * pv.v[e] : fma_(alpha, pv.v[e], xv.v[e]);
          acc += bq.v[e] * bq.v[e];
        }
        vst4<T>(cf.rout + g.off + k, bq);
        vst4<T>(cf.xcg + g.off + k, xv);
      }
    });
  }
  if constexpr (UPD) {
    const double s = block_sum(acc);
    if (threadIdx.x == 0) cf.part[ti] = s;
  }
  return kTileDone;
}

// LIST: the CTAs stride over a device-built list of the active traps' tiles (late
// refinement sweeps, where most traps are done: a grid of all tiles would be mostly
// CTAs that read their trap's skip flag and exit); otherwise CTA b takes tile b.
template <class T, bool GEN, bool UPD = false, bool LIST = false>
__global__ void __launch_bounds__(kThreads, kFusedCtas<T>)
    k_down(const LevelGeom* __restrict__ G, const Tile2* __restrict__ tiles,
           const T* __restrict__ tabs, const int* __restrict__ skip, const T* __restrict__ b,
           T* __restrict__ x, T* __restrict__ t, CgFold<T> cf, TileList tlist,
           unsigned long long* work) {
  if constexpr (!LIST) {
    const Tile2 tile = tiles[blockIdx.x];  // static: read before the wait
    prefetch_l1(G + tile.geom);
    grid_dep_sync();
    down_tile<T, GEN, UPD>(G, tile, (int)blockIdx.x, tabs, skip, b, x, t, cf, work);
  } else {
    grid_dep_sync();
    const int n = *tlist.count;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
      const int ti = tlist.idx[w];
      const int rc = down_tile<T, GEN, UPD>(G, tiles[ti], ti, tabs, skip, b, x, t, cf, work);
      if (rc == kTileFailed) return;
      next_listed_tile(rc);
    }
  }
}

// Prolongation and post-smoothing (two steps) of one tile: reads x (xin) and the
// coarse correction, writes x2 to xout (another buffer: neighbouring tiles still
// stage xin).  DOT adds a partial of b.x2 (r.z of the Krylov iteration).
template <class T, bool DOT, bool GEN>
__device__ __forceinline__ int up_tile(const LevelGeom* __restrict__ G,
                                       const LevelGeom* __restrict__ Gc, const Tile2& tile,
                                       int ti, const T* __restrict__ tabs,
                                       const int* __restrict__ skip, const T* __restrict__ xc,
                                       const T* __restrict__ b, const T* __restrict__ xin,
                                       T* __restrict__ xout, double* __restrict__ part,
                                       unsigned long long* work) {
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (DOT && threadIdx.x == 0) part[ti] = 0.0;
    return kTileSkipped;
  }
  if (work && threadIdx.x == 0)
    atomicAdd(work, (unsigned long long)(tile.r1 - tile.r0) * (tile.c1 - tile.c0));
  const LevelGeom& c = Gc[tile.geom];
  const ChebCoef c0 = cheb_at(g, 0), c1 = cheb_at(g, 1);
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  const int P = g.P;
  const Win w1 = win_grow(tile, 2, 8), w2 = win_grow(tile, 1, 4);
  const Win wt = win_grow(tile, 0, 0);
  const Win wc = up_coarse_win(g, c, w1);
  Stager st(eqf_smem);
  T* xp = carve<T>(st, w1.count());
  T* bp = carve<T>(st, w2.count());
  T* cp = carve<T>(st, wc.count());
  T* x1p = carve<T>(st, w2.count());
  const TableStage<T> tst = stage_table<T>(st, tab, ci);
  const T* stab = tst.s;
  const RowStage<T> rs[3] = {{xin + g.off, xp, w1, P, g.ny + 1},
                             {b + g.off, bp, w2, P, g.ny + 1},
                             {xc + c.off, cp, wc, c.P, c.ny + 1}};
  if (!stage_rows<T, 3>(st.bar, rs, tst)) return kTileFailed;
  const int S1 = w1.S(), S2 = w2.S(), SC = wc.S();
  // x0 = x + P x_c on the in-grid nodes of W1 (in place), one window quad per
  // thread.  Fine node (i, j) lies between coarse nodes (i0, j0) and (i1, j1) along
  // the cut's diagonal (i0 = i1 and/or j0 = j1 where it coincides with a coarse row,
  // column or node), and takes 0.5 (c[i0][j0] + c[i1][j1]): the coarse value itself,
  // an edge midpoint or a diagonal midpoint, bit for bit (0.5 (a + a) = a).
  {
    const WinQuads wq(w1);
    const int nx = g.nx, ny = g.ny;
    for (int q = threadIdx.x; q < wq.n; q += blockDim.x) {
      int row, cq;
      wq.at(q, row, cq);
      const int i = w1.ra + row, j = w1.ca + 4 * cq;  // j: a multiple of 4
      if (i < 0 || i > ny || j < 0 || j > nx) continue;  // j < 0 means j + 3 < 0
      int i0, i1;
      fine_to_coarse(i, ny, c.cy, i0, i1);
      const T* cr0 = cp + (i0 - wc.ra) * SC - wc.ca;
      const T* cr1 = cp + (i1 - wc.ra) * SC - wc.ca;
      int j0[4], j1[4];
      if (c.cx) {  // columns j, j+1, j+2, j+3 -> (J,J), (J,J+1), (J+1,J+1), (J+1,J+2);
        const int J = j >> 1;  // an odd last column nx coincides with coarse node (nx+1)/2
        j0[0] = J;
        j1[0] = J;
        j0[1] = j + 1 == nx ? J + 1 : J;
        j1[1] = J + 1;
        j0[2] = J + 1;
        j1[2] = J + 1;
        j0[3] = j + 3 == nx ? J + 2 : J + 1;
        j1[3] = J + 2;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) j0[e] = j1[e] = j + e;
      }
      T* xq = xp + row * S1 + 4 * cq;
      Q4<T> xv = vld4<T>(xq);
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (j + e <= nx) xv.v[e] += T(0.5) * (cr0[j0[e]] + cr1[j1[e]]);
      vst4<T>(xq, xv);
    }
  }
  __syncthreads();
  // first step (no previous direction) on W2
  {
    const View<T> xv{xp, 0};
    for_quads(g, win_quads(w2), [&](int i, int cq, auto inner_) {
      constexpr bool INNER = decltype(inner_)::value;
      const int j = w2.ca + 4 * cq, kl = (i - w2.ra) * S2 + 4 * cq;
      Q4<T> x0q, id;
      const Q4<T> ax = apply_quad<T, 0, View<T>, kGM<GEN>>(g, ci, stab, xv,
          wl(w1, i, j), S1, i, j, INNER, x0q, id);
      const Q4<T> bq = vld4<T>(bp + kl);
      Q4<T> xn;
#pragma unroll
      for (int e = 0; e < 4; ++e)
        xn.v[e] = add_(x0q.v[e], cheb_dir<T, true>(c0, bq.v[e], ax.v[e], id.v[e], T(0)));
      vst4<T>(x1p + kl, xn);
    });
  }
  __syncthreads();
  // second step on the tile, d1 = x1 - x0
  T acc = T(0);
  {
    const View<T> x1v{x1p, 0};
    T* xo = xout + g.off;
    for_quads(g, win_quads(wt), [&](int i, int cq, auto inner_) {
      constexpr bool INNER = decltype(inner_)::value;
      const int j = tile.c0 + 4 * cq;
      Q4<T> x1q, id;
      const Q4<T> ax = apply_quad<T, 0, View<T>, kGM<GEN>>(g, ci, stab, x1v,
          wl(w2, i, j), S2, i, j, INNER, x1q, id);
      const Q4<T> bq = vld4<T>(bp + wl(w2, i, j));
      const Q4<T> x0q = vld4<T>(xp + wl(w1, i, j));
      Q4<T> xn;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        xn.v[e] =
            x1q.v[e] + cheb_dir<T, false>(c1, bq.v[e], ax.v[e], id.v[e], x1q.v[e] - x0q.v[e]);
        if (DOT) acc += bq.v[e] * xn.v[e];
      }
      vst4<T>(xo + (size_t)i * P + j, xn);
    });
  }
  if (DOT) {
    const double s = block_sum(acc);
    if (threadIdx.x == 0) part[ti] = s;
  }
  return kTileDone;
}

// LIST as k_down's.
template <class T, bool DOT, bool GEN, bool LIST = false>
__global__ void __launch_bounds__(kThreads, kFusedCtas<T>)
    k_up(const LevelGeom* __restrict__ G, const LevelGeom* __restrict__ Gc,
         const Tile2* __restrict__ tiles, const T* __restrict__ tabs,
         const int* __restrict__ skip, const T* __restrict__ xc, const T* __restrict__ b,
         const T* __restrict__ xin, T* __restrict__ xout, double* __restrict__ part,
         TileList tlist, unsigned long long* work) {
  if constexpr (!LIST) {
    const Tile2 tile = tiles[blockIdx.x];  // static: read before the wait
    prefetch_l1(G + tile.geom);
    grid_dep_sync();
    up_tile<T, DOT, GEN>(G, Gc, tile, (int)blockIdx.x, tabs, skip, xc, b, xin, xout, part,
                         work);
  } else {
    grid_dep_sync();
    const int n = *tlist.count;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
      const int ti = tlist.idx[w];
      const int rc =
          up_tile<T, DOT, GEN>(G, Gc, tiles[ti], ti, tabs, skip, xc, b, xin, xout, part, work);
      if (rc == kTileFailed) return;
      next_listed_tile(rc);
    }
  }
}

}  // namespace eqf
