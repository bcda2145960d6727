// Refinement residuals of the FP32 form in double-float arithmetic.
//
// GB300 executes FP64 at 1/64 of the FP32 rate, so the residual r = b - A u of the
// iterative refinement (two seven-point stencils per node in the first pass) is
// evaluated on the FP32 pipe instead: every value is an unevaluated sum h + l of
// two floats ("pair", about 47 significant bits), products are split exactly with
// fused multiply-adds and the sums carry their rounding errors (two-sum).  The
// conversions between doubles and pairs are done with integer bit operations and
// the squared norms are accumulated in FP32, so the kernels issue almost no FP64
// instructions (one add per stored double, one per thread for the norms).
//
// Accuracy: a pair carries a relative error below 2^-47 (7e-15).  The residual of a
// stencil with cancellation factor C = sum|a_ij u_j| / |(A u)_i| is accurate to
// about 7 C 2^-47 |A u|; for the diffusion operators here (C up to ~1e4) that is
// 1e-9 of |b| or better, two orders below the tolerances the refinement is run to
// (rtol >= 1e-8), so the outer convergence test is unaffected.  Values of magnitude
// below 2^-126 (1.2e-38) flush to zero and values from 2^128 on become infinite.
//
// The plain FP64 form keeps its FP64 kernels (eqf_kernels.cuh).
#pragma once
#include "eqf_kernels.cuh"

namespace eqf {

struct DF {
  float h, l;
};

// Exact float -> double by repacking the bits (denormals flush to signed zero).
__device__ __forceinline__ double f2d(float f) { return to_double(f); }

// Low part of a value below 2^-80, where the integer scale below would leave the
// float range (rare: out of line so the common path carries no FP64 instructions).
__device__ __noinline__ float df_low_tiny(double v, float h) {
  return __double2float_rn(v - f2d(h));
}

// double -> pair: h = v truncated to 24 significant bits, l = the next 23 bits
// (|h + l - v| < 2^-46 |v|).  |v| < 2^-126 gives (0, 0); |v| >= 2^128 (+-inf, 0).
__device__ __forceinline__ DF df_split(double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const uint32_t wh = (uint32_t)(u >> 32), wl = (uint32_t)u;
  const uint32_t sg = wh & 0x80000000u;
  const int e = (int)((wh >> 20) & 0x7FFu);
  const uint32_t hb = sg | ((uint32_t)(e - 896) << 23) | ((wh & 0xFFFFFu) << 3) | (wl >> 29);
  // l = (low 29 mantissa bits >> 6) * 2^(e - 1069); the integer part is < 2^23,
  // so the magic-number conversion below is exact
  const uint32_t r = (wl & 0x1FFFFFFFu) >> 6;
  const float rf = __fsub_rn(__uint_as_float(0x4B000000u | r), 8388608.0f);
  const float sc = __uint_as_float((uint32_t)(e - 942) << 23);
  const float l = __uint_as_float(__float_as_uint(__fmul_rn(rf, sc)) | sg);
  DF o;
  if (e < 897) {
    o.h = 0.f;
    o.l = 0.f;
  } else if (e > 1150) {
    o.h = __uint_as_float(sg | 0x7F800000u);
    o.l = 0.f;
  } else {
    o.h = __uint_as_float(hb);
    // below 2^-80 the integer scale would leave the float range: FP64 fallback
    o.l = l;
    if (e < 943) o.l = df_low_tiny(v, o.h);
  }
  return o;
}

// pair -> double (one FP64 add)
__device__ __forceinline__ double df_to_double(DF a) { return __dadd_rn(f2d(a.h), f2d(a.l)); }

__device__ __forceinline__ float two_sum(float a, float b, float& err) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}
__device__ __forceinline__ DF df_norm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return DF{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  float err;
  const float s = two_sum(a.h, b.h, err);
  return df_norm(s, __fadd_rn(err, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }

// Sum of pair products c_m x_m: the high products are added with two-sum, every
// rounding error (of the products and of the sums) goes into e.
struct DFAcc {
  float s, e;
  __device__ __forceinline__ void first(DF c, DF x) {
    s = __fmul_rn(c.h, x.h);
    e = __fmaf_rn(c.h, x.l, __fmaf_rn(c.l, x.h, __fmaf_rn(c.h, x.h, -s)));
  }
  __device__ __forceinline__ void add(DF c, DF x) {
    const float p = __fmul_rn(c.h, x.h);
    const float pe = __fmaf_rn(c.h, x.l, __fmaf_rn(c.l, x.h, __fmaf_rn(c.h, x.h, -p)));
    float err;
    s = two_sum(s, p, err);
    e = __fadd_rn(e, __fadd_rn(err, pe));
  }
  __device__ __forceinline__ DF result() const { return df_norm(s, e); }
};

// Sum of squares in FP32 without underflow: values below 2^-40 are squared after
// scaling by 2^64 into a second accumulator (2^-128 times its sum is added back in
// FP64 once per thread).
struct SqAcc {
  float big = 0.f, tiny = 0.f;
  __device__ __forceinline__ void add(float v) {
    const bool small = fabsf(v) < 9.094947e-13f;  // 2^-40
    const float w = small ? v * 1.8446744e19f : v;  // 2^64
    if (small)
      tiny = __fmaf_rn(w, w, tiny);
    else
      big = __fmaf_rn(w, w, big);
  }
  __device__ __forceinline__ double total() const {
    return f2d(big) + f2d(tiny) * 2.9387358770557188e-39;  // 2^-128
  }
};
// CTA sum of the threads' sums of squares: both accumulators summed over the warp in
// FP32, the warps' totals in FP64.  Valid in thread 0.
__device__ __forceinline__ double block_sum(const SqAcc& a) {
  SqAcc w = a;
  for (int o = 16; o > 0; o >>= 1) {
    w.big += __shfl_down_sync(0xffffffffu, w.big, o);
    w.tiny += __shfl_down_sync(0xffffffffu, w.tiny, o);
  }
  return warps_sum(w.total());
}

// Per-trap pair tables: 25 classes x 8 pairs (c, e, w, n, s, ne, sw, unused), the
// interior class holding the interior weights (same layout as the FP64 tables).
// stage_pair_table carves the region; the returned filler runs inside Stager::run,
// after the bulk copies are issued.
struct PairTableStage {
  float2* s;
  const float2* tab;
  __device__ __forceinline__ void operator()() const {
    for (int e = threadIdx.x; e < kTabPerTrap; e += blockDim.x) s[e] = tab[e];
  }
};
__device__ __forceinline__ PairTableStage stage_pair_table(Stager& st, const float2* tab) {
  float2* s = reinterpret_cast<float2*>(st.cur);
  st.cur += kTabPerTrap * sizeof(float2);
  return PairTableStage{s, tab};
}

// (A x)_k for node (i, j) from a pair window x (node k at x[k - a]).
__device__ __forceinline__ DF df_apply(const LevelGeom& g, const float2* __restrict__ stab,
                                       bool general, const float2* x, int a, int k, int i,
                                       int j) {
  const int P = g.P;
  DF c[7];
  if (general) {
    double cg[8];
    coef_node<double>(g, i, j, cg);
#pragma unroll
    for (int m = 0; m < 7; ++m) c[m] = df_split(cg[m]);
  } else {
    const float2* t = stab + node_class(g, i, j) * kTabStride;
#pragma unroll
    for (int m = 0; m < 7; ++m) c[m] = DF{t[m].x, t[m].y};
  }
  const int idx[7] = {k, k + 1, k - 1, k + P, k - P, k + P + 1, k - P - 1};
  DFAcc acc;
  {
    const float2 v = x[idx[0] - a];
    acc.first(c[0], DF{v.x, v.y});
  }
#pragma unroll
  for (int m = 1; m < 7; ++m) {
    const float2 v = x[idx[m] - a];
    acc.add(c[m], DF{v.x, v.y});
  }
  return acc.result();
}

// A x on the quad of nodes k .. k+3 (row i, columns j .. j+3) from a pair window x
// (node k at x[k - a], k - a even, so four pairs are two aligned 16-byte loads) of a
// class-table trap.  The interior quads (INNER) take the interior weights `ci`, the
// others per-node weights from the table.  Every node accumulates its seven products
// in df_apply's order, so both paths give df_apply's bits.  (General-path traps take
// df_residual_general: their stencil fetch would cost this path its registers.)
template <bool INNER>
__device__ __forceinline__ void df_apply_quad(const LevelGeom& g, const float2* __restrict__ stab,
                                              const DF (&ci)[7], const float2* x, int a, int k,
                                              int i, int j, DF (&out)[4]) {
  const int P = g.P;
  const float2* xc = x + (k - a);
  auto ld2 = [](const float2* p, float2& u, float2& v) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    u = make_float2(q.x, q.y);
    v = make_float2(q.z, q.w);
  };
  // two nodes at a time (fewer values live): x[k+2h-1 .. k+2h+2], x[k+2h+P .. +2],
  // x[k+2h-P-1 .. k+2h-P+1]
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float2* xh = xc + 2 * h;
    float2 r0[4], rn[3], rs[3];
    r0[0] = xh[-1];
    ld2(xh, r0[1], r0[2]);
    r0[3] = xh[2];
    ld2(xh + P, rn[0], rn[1]);
    rn[2] = xh[P + 2];
    rs[0] = xh[-P - 1];
    ld2(xh - P, rs[1], rs[2]);
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const int e = 2 * h + f;
      DF c[7];
      if (INNER) {
#pragma unroll
        for (int m = 0; m < 7; ++m) c[m] = ci[m];
      } else {
        const float2* t = stab + node_class(g, i, j + e) * kTabStride;
#pragma unroll
        for (int m = 0; m < 7; ++m) c[m] = DF{t[m].x, t[m].y};
      }
      const float2 v[7] = {r0[f + 1], r0[f + 2], r0[f], rn[f], rs[f + 1], rn[f + 1], rs[f]};
      DFAcc acc;
      acc.first(c[0], DF{v[0].x, v[0].y});
#pragma unroll
      for (int m = 1; m < 7; ++m) acc.add(c[m], DF{v[m].x, v[m].y});
      out[e] = acc.result();
    }
  }
}

// The interior weights (class 12) of a staged pair table.
__device__ __forceinline__ void df_interior(const float2* stab, DF (&ci)[7]) {
  const float2* t = stab + 12 * kTabStride;
#pragma unroll
  for (int m = 0; m < 7; ++m) ci[m] = DF{t[m].x, t[m].y};
}

// r = b - A x on a quad (Dirichlet rows: 0, or b - x with wall values), stored when
// STORE; |r|^2 accumulated in `arr`.
template <bool INNER>
__device__ __forceinline__ void df_residual_quad(const LevelGeom& g, const float2* __restrict__ sA,
                                                 const DF (&ca)[7], const float2* x, int a, int k,
                                                 int i, int j, const float2* __restrict__ bs,
                                                 float* __restrict__ rs, SqAcc& arr, bool store) {
  DF ax[4];
  df_apply_quad<INNER>(g, sA, ca, x, a, k, i, j, ax);
  const float4 b01 = reinterpret_cast<const float4*>(bs + k)[0];
  const float4 b23 = reinterpret_cast<const float4*>(bs + k)[1];
  const DF bv[4] = {DF{b01.x, b01.y}, DF{b01.z, b01.w}, DF{b23.x, b23.y}, DF{b23.z, b23.w}};
  float rk[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const bool dir = !INNER && g.walls && is_dirichlet(g, i, j + e);
    rk[e] = 0.f;
    if (!dir) {
      const DF res = df_add(bv[e], df_neg(ax[e]));
      rk[e] = __fadd_rn(res.h, res.l);
    } else if (g.dvals) {
      const float2 xv = x[k + e - a];
      const DF res = df_add(bv[e], df_neg(DF{xv.x, xv.y}));
      rk[e] = __fadd_rn(res.h, res.l);
    }
    arr.add(rk[e]);
  }
  if (store) *reinterpret_cast<float4*>(rs + k) = make_float4(rk[0], rk[1], rk[2], rk[3]);
}

// The same residual node by node for a general-path trap (advection, anisotropic
// tensor), whose stencils come from coef_node.
__device__ __forceinline__ void df_residual_general(const LevelGeom& g, const Tile& tile,
                                                    const float2* x, int a,
                                                    const float2* __restrict__ bs,
                                                    float* __restrict__ rs, SqAcc& arr,
                                                    bool store) {
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    const bool dir = g.walls && is_dirichlet(g, w.i, w.j);
    float rk = 0.f;
    if (!dir) {
      const float2 b = bs[w.k];
      const DF res = df_add(DF{b.x, b.y}, df_neg(df_apply(g, nullptr, true, x, a, w.k, w.i, w.j)));
      rk = __fadd_rn(res.h, res.l);
    } else if (g.dvals) {
      const float2 b = bs[w.k], xv = x[w.k - a];
      const DF res = df_add(DF{b.x, b.y}, df_neg(DF{xv.x, xv.y}));
      rk = __fadd_rn(res.h, res.l);
    }
    if (store) rs[w.k] = rk;
    arr.add(rk);
  }
}

// Converts the staged doubles of window [ka, kb) to pairs in place (same 8 bytes).
__device__ __forceinline__ void window_to_pairs(const View<double>& v, int ka, int kb) {
  double* p = const_cast<double*>(v.p);
  for (int k = ka + (int)threadIdx.x; k < kb; k += blockDim.x) {
    const DF d = df_split(p[k - v.a]);
    reinterpret_cast<float2*>(p)[k - v.a] = make_float2(d.h, d.l);
  }
}

// First refinement residual of a step in the FP32 form (partials: [0] |b|^2,
// [1] |r|^2):  b = F + M u_in (stored as pairs), u0 = u_in + gamma d_in,
// u_out = u0, d_out = u0 - u_in, r = b - A u0.  Dirichlet rows: b = 0, r = 0.
__global__ void __launch_bounds__(kThreads)
    k_irf_first(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                const float2* __restrict__ tabA, const float2* __restrict__ tabM,
                const CgState* __restrict__ st, const double* __restrict__ F,
                const double* __restrict__ u_in, const float* __restrict__ d_in,
                float2* __restrict__ b2, double* __restrict__ u_out, float* __restrict__ d_out,
                float* __restrict__ r, double* __restrict__ part, int ntiles,
                const int* __restrict__ frozen, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (frozen[g.trap]) {  // inactive trap: its field is left as it is
    if (threadIdx.x == 0) part[blockIdx.x] = part[ntiles + blockIdx.x] = 0.0;
    return;
  }
  count_work(work, tile);
  Stager sg(eqf_smem);
  const int na = padded_len(g);
  const int ka = halo_lo(g, tile), kb = halo_hi(g, tile);
  const View<double> uv = sg.add_guarded(u_in + g.off, ka, kb, na);
  const View<float> dv = sg.add_guarded(d_in + g.off, ka, kb, na);
  const PairTableStage tA = stage_pair_table(sg, tabA + (size_t)g.trap * kTabPerTrap);
  const PairTableStage tM = stage_pair_table(sg, tabM + (size_t)g.trap * kTabPerTrap);
  const float2* sA = tA.s;
  const float2* sM = tM.s;
  if (!sg.run([&] {
        tA();
        tM();
      }))
    return;
  window_to_pairs(uv, ka, kb);
  __syncthreads();
  const float2* xw = reinterpret_cast<const float2*>(uv.p);
  const int xa = uv.a;
  const double* Fs = F + g.off;
  float2* bs = b2 + g.off;
  SqAcc abb, arr;
  const int P = g.P;
  // tiles are whole rows: every quad lies inside the tile
  const QuadBlock qb{tile.r0, tile.r1, 0, P >> 2};
  // b = F + M u_in (the mass operator: its interior weights from class 12 too)
  {
    DF cm[7];
    df_interior(sM, cm);
    for_quads(g, qb, [&](int i, int cq, auto inner_) {
      constexpr bool INNER = decltype(inner_)::value;
      const int j = 4 * cq, k = i * P + j;
      DF mu[4];
      df_apply_quad<INNER>(g, sM, cm, xw, xa, k, i, j, mu);
      const double2 f01 = *reinterpret_cast<const double2*>(Fs + k);
      const double2 f23 = *reinterpret_cast<const double2*>(Fs + k + 2);
      const double fv[4] = {f01.x, f01.y, f23.x, f23.y};
      float2 bo[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const bool dir = !INNER && g.walls && is_dirichlet(g, i, j + e);
        DF bk{0.f, 0.f};
        if (!dir)
          bk = df_add(df_split(fv[e]), mu[e]);
        else if (g.dvals)  // the identity row with the wall value held in F
          bk = df_split(fv[e]);
        bo[e] = make_float2(bk.h, bk.l);
        abb.add(bk.h);
      }
      reinterpret_cast<float4*>(bs + k)[0] = make_float4(bo[0].x, bo[0].y, bo[1].x, bo[1].y);
      reinterpret_cast<float4*>(bs + k)[1] = make_float4(bo[2].x, bo[2].y, bo[3].x, bo[3].y);
    });
  }
  __syncthreads();  // every read of u_in done: the window becomes u0 in place
  {
    const DF gm = df_split(st[g.trap].gamma);
    float2* x = const_cast<float2*>(xw);
    double* uo = u_out + g.off;
    float* dout = d_out + g.off;
    for (int k = ka + (int)threadIdx.x; k < kb; k += blockDim.x) {
      const float2 u = x[k - xa];
      const float dk = dv[k];
      const float p = __fmul_rn(gm.h, dk);
      const float pe = __fmaf_rn(gm.l, dk, __fmaf_rn(gm.h, dk, -p));
      const DF u0 = df_add(DF{u.x, u.y}, df_norm(p, pe));
      x[k - xa] = make_float2(u0.h, u0.l);
      if (k >= tile.k0 && k < tile.k1) {
        uo[k] = df_to_double(u0);
        dout[k] = __fadd_rn(p, pe);
      }
    }
  }
  __syncthreads();
  float* rs = r + g.off;
  if (g.adv_on) {
    df_residual_general(g, tile, xw, xa, bs, rs, arr, true);
  } else {
    DF ca[7];
    df_interior(sA, ca);
    for_quads(g, qb, [&](int i, int cq, auto inner_) {
      constexpr bool INNER = decltype(inner_)::value;
      const int j = 4 * cq, k = i * P + j;
      df_residual_quad<INNER>(g, sA, ca, xw, xa, k, i, j, bs, rs, arr, true);
    });
  }
  const double tb = block_sum(abb);
  const double tr = block_sum(arr);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = tb;
    part[ntiles + blockIdx.x] = tr;
  }
}

// Later residuals of a step in the FP32 form: r = b - A u (partial [1] |r|^2).
// With FINAL the residual is only measured and every trap also reports |d|^2
// (partial [2]) for the next step's extrapolation factor.
template <bool FINAL>
__global__ void __launch_bounds__(kThreads, 4)
    k_irf_residual(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                   const float2* __restrict__ tabA, const int* __restrict__ skip,
                   const float2* __restrict__ b2, const double* __restrict__ u,
                   const float* __restrict__ dcur, float* __restrict__ r,
                   double* __restrict__ part, int ntiles, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  const bool skipped = skip && skip[g.trap];
  if (skipped && !FINAL) {
    if (threadIdx.x == 0) part[ntiles + blockIdx.x] = 0.0;
    return;
  }
  SqAcc arr, add;
  // |d|^2 of the tile (tiles are whole rows of 16-byte-aligned quads)
  auto dnorm = [&] {
    if (FINAL) {
      const float4* ds = reinterpret_cast<const float4*>(dcur + g.off);
      for (int q = (tile.k0 >> 2) + (int)threadIdx.x; q < (tile.k1 >> 2); q += blockDim.x) {
        const float4 v = ds[q];
        add.add(v.x);
        add.add(v.y);
        add.add(v.z);
        add.add(v.w);
      }
    }
  };
  if (skipped) dnorm();
  if (!skipped) {
    count_work(work, tile);
    Stager sg(eqf_smem);
    const int na = padded_len(g);
    const int ka = halo_lo(g, tile), kb = halo_hi(g, tile);
    const View<double> uv = sg.add_guarded(u + g.off, ka, kb, na);
    const PairTableStage tA = stage_pair_table(sg, tabA + (size_t)g.trap * kTabPerTrap);
    const float2* sA = tA.s;
    if (!sg.run([&] {
          tA();
          dnorm();
        }))
      return;
    window_to_pairs(uv, ka, kb);
    __syncthreads();
    const float2* xw = reinterpret_cast<const float2*>(uv.p);
    const float2* bs = b2 + g.off;
    float* rs = r + g.off;
    const int P = g.P;
    if (g.adv_on) {
      df_residual_general(g, tile, xw, uv.a, bs, rs, arr, !FINAL);
    } else {
      DF ca[7];
      df_interior(sA, ca);
      // tiles are whole rows: every quad lies inside the tile
      for_quads(g, QuadBlock{tile.r0, tile.r1, 0, P >> 2}, [&](int i, int cq, auto inner_) {
        constexpr bool INNER = decltype(inner_)::value;
        const int j = 4 * cq, k = i * P + j;
        df_residual_quad<INNER>(g, sA, ca, xw, uv.a, k, i, j, bs, rs, arr, !FINAL);
      });
    }
  }
  const double tr = block_sum(arr);
  const double td = FINAL ? block_sum(add) : 0.0;
  if (threadIdx.x == 0) {
    part[ntiles + blockIdx.x] = tr;
    if (FINAL) part[2 * ntiles + blockIdx.x] = td;
  }
}

}  // namespace eqf
