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
#include <type_traits>

#include "eqf_common.cuh"

namespace eqf {

constexpr int kThreads = 256;
constexpr int kTabStride = 8;                 // c, e, w, n, s, ne, sw, 1/c
constexpr int kTabClasses = 26;                // 5 x 5 node classes + the pad class
constexpr int kClassPad = 25;                  // pad columns: all-zero row
constexpr int kTabPerTrap = kTabClasses * kTabStride;
// Resident CTAs per SM the staged stencil kernels are compiled for (register cap):
// FP32 tiles are small enough in shared memory for six per SM.
template <class T>
constexpr int kStencilCtas = sizeof(T) == 4 ? 4 : 2;

extern __shared__ __align__(16) char eqf_smem[];

// Device-side error flag: set when a bounded wait gives up (never expected).
__device__ int g_eqf_device_error = 0;

// Programmatic dependent launch.  The solver's kernels are launched with programmatic
// stream serialization, so a kernel's CTAs may be scheduled while its predecessor's
// last CTAs still run.  Every solver kernel calls this first: it returns once the
// predecessor grid has completed and its writes are visible (the hardware holds the
// CTA; no spinning), then allows the successor grid to be scheduled.  For a kernel
// launched without the attribute both instructions are no-ops.
__device__ __forceinline__ void grid_dep_sync() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Before grid_dep_sync a kernel may only read what no kernel of a step writes: its
// tile descriptor and the level geometry.  This pulls the geometry into L1 while the
// predecessor finishes.
template <class G>
__device__ __forceinline__ void prefetch_l1(const G* p) {
  const char* c = reinterpret_cast<const char*>(p);
  for (int o = (int)threadIdx.x * 128; o < (int)sizeof(G); o += (int)blockDim.x * 128)
    asm volatile("prefetch.global.L1 [%0];" ::"l"(c + o));
}

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
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// A launch over a device-built list of tiles: the CTAs stride over idx[0, *count)
// (absolute indices into the launch's tile array).
struct TileList {
  const int* idx;
  const int* count;
};

// Outcome of one tile of a staged kernel.
constexpr int kTileSkipped = 0, kTileDone = 1, kTileFailed = -1;

// Between two tiles of a listed launch: every thread is done with the staged windows
// before the next tile's copies overwrite them, and a used mbarrier (at the start of
// the dynamic shared memory) is invalidated before it is initialised again.
__device__ __forceinline__ void next_listed_tile(int rc) {
  __syncthreads();
  if (rc == kTileDone && threadIdx.x == 0) mbar_inval(reinterpret_cast<uint64_t*>(eqf_smem));
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
struct Q4;
template <class T>
struct View {
  const T* p;
  int a;
  __device__ __forceinline__ T operator[](int k) const { return p[k - a]; }
  __device__ __forceinline__ Q4<T> quad(int k) const;  // k a multiple of 4
  // x[k0 .. k0+4]; M = (k0 - a) mod 4, a compile-time constant of the caller
  template <int M>
  __device__ __forceinline__ void row(int k0, T (&out)[5]) const;
};

constexpr int kMaxStaged = 4;

// Plans up to kMaxStaged ranges in dynamic shared memory; thread 0 then issues
// them as bulk copies.  Ranges are widened to 16-byte boundaries; trap segments
// are padded to 32 elements, so a widened range stays inside the allocation.
// Guarded ranges may reach outside [0, nalloc): those parts are zero-filled.
// Every add() takes one copy slot and two guard slots, so the slot indices are
// compile-time constants and the bookkeeping stays in registers.
struct Stager {
  uint64_t* bar;
  char* cur;
  uint32_t total;
  int n;
  const void* src[kMaxStaged];
  void* dst[kMaxStaged];
  uint32_t bytes[kMaxStaged];
  char* gptr[2 * kMaxStaged];  // zero-fill regions (16-byte granules)
  uint32_t gbytes[2 * kMaxStaged];

  __device__ __forceinline__ explicit Stager(char* smem) {
    bar = reinterpret_cast<uint64_t*>(smem);
    cur = smem + 16;
    total = 0;
    n = 0;
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
    const uint32_t nb = cb > ca ? (uint32_t)(cb - ca) * (uint32_t)sizeof(T) : 0u;
    src[n] = base + ca;
    dst[n] = d + (ca - wa);
    bytes[n] = nb;
    total += nb;
    gptr[2 * n] = reinterpret_cast<char*>(d);
    gbytes[2 * n] = ca > wa ? (uint32_t)(ca - wa) * sizeof(T) : 0u;
    const int lo = cb > ca ? cb : ca;
    gptr[2 * n + 1] = reinterpret_cast<char*>(d + (lo - wa));
    gbytes[2 * n + 1] = wb > lo ? (uint32_t)(wb - lo) * sizeof(T) : 0u;
    ++n;
    // +16 bytes: vector row loads may read up to 8 bytes past the window (unused)
    cur += (((uint32_t)(wb - wa) * sizeof(T) + 15u) & ~15u) + 16u;
    return View<T>{d, wa};
  }
  // nodes [ka, kb) of `base` (trap-relative, inside [0, nalloc))
  template <class T>
  __device__ __forceinline__ View<T> add(const T* base, int ka, int kb, int nalloc) {
    return add_guarded<T>(base, ka, kb, nalloc);
  }
  // Issue the copies, run `fill` (other shared-memory staging that overlaps the
  // copies in flight: it must not touch the staged ranges), zero the guards and
  // wait for the copies (bounded).  Returns false, uniformly for the CTA, if the
  // wait gave up (device error flag set).
  template <class F>
  __device__ __forceinline__ bool run(const F& fill) {
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      mbar_expect_tx(bar, total);
#pragma unroll
      for (int q = 0; q < kMaxStaged; ++q)
        if (q < n && bytes[q]) bulk_copy_g2s(dst[q], src[q], bytes[q], bar);
    }
    fill();
#pragma unroll
    for (int q = 0; q < 2 * kMaxStaged; ++q) {
      if (q < 2 * n && gbytes[q]) {
        uint4* z = reinterpret_cast<uint4*>(gptr[q]);
        for (uint32_t e = threadIdx.x; e < gbytes[q] / 16u; e += blockDim.x)
          z[e] = make_uint4(0u, 0u, 0u, 0u);
      }
    }
    // One thread waits on the mbarrier (the others sleep in the barrier below
    // instead of spinning); the barrier then publishes the copied data CTA-wide.
    bool ok = true;
    if (threadIdx.x == 0) {
      ok = false;
      for (int it = 0; it < (1 << 22) && !ok; ++it) ok = mbar_try_wait(bar, 0);
      if (!ok) {
        // give the copies in flight one more bounded chance to land before leaving
        for (int it = 0; it < (1 << 20) && !ok; ++it) ok = mbar_try_wait(bar, 0);
        if (!ok) atomicExch(&g_eqf_device_error, 1);
      }
    }
    return __syncthreads_and(ok ? 1 : 0) != 0;
  }
  __device__ __forceinline__ bool run() {
    return run([] {});
  }
};

__device__ __forceinline__ int padded_len(const LevelGeom& g) {
  const int n = g.P * (g.ny + 1);
  return (n + 31) & ~31;
}

// (i, j) = floor-divmod(k, P) without an integer division (exact for |k| < 2^22).
__device__ __forceinline__ void div_pitch(int k, int P, float inv_p, int& i, int& j) {
  i = __float2int_rd(((float)k + 0.5f) * inv_p);
  j = k - i * P;
  if (j < 0) {
    --i;
    j += P;
  } else if (j >= P) {
    ++i;
    j -= P;
  }
}

// Walks the nodes k = k0 + tid, k0 + tid + bd, ... of a tile while keeping
// (i, j) = divmod(k, P) up to date with no division.
struct NodeWalk {
  int k, i, j;
  int qi, qj, pitch;
  __device__ __forceinline__ NodeWalk(const LevelGeom& g, int k0) {
    pitch = g.P;
    k = k0 + threadIdx.x;
    div_pitch(k, pitch, g.inv_pitch, i, j);
    div_pitch((int)blockDim.x, pitch, g.inv_pitch, qi, qj);
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
  if (j > g.nx) return kClassPad;
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

// One fixed evaluation order (explicit fused multiply-adds), shared by every code
// path, so a node's value never depends on which path evaluated it: the seven
// weights (c, e, w, n, s, ne, sw) are applied in that order.
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
// A sum the compiler may not fuse with the product that produced an operand (kernels
// that must give the same bits write it out where the product also has other uses).
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }

template <class T>
__device__ __forceinline__ T st_table(const T* c, T x0, T xe, T xw, T xn, T xs, T xne, T xsw) {
  return fma_(c[6], xsw, fma_(c[5], xne, fma_(c[4], xs, fma_(c[3], xn, fma_(c[2], xw,
              fma_(c[1], xe, c[0] * x0))))));
}
// The same order with the interior weights (e = w, n = s, ne = sw).
template <class T>
__device__ __forceinline__ T st_interior(const Interior<T>& ci, T x0, T xe, T xw, T xn, T xs,
                                         T xne, T xsw) {
  return fma_(ci.d, xsw, fma_(ci.d, xne, fma_(ci.n, xs, fma_(ci.n, xn, fma_(ci.e, xw,
              fma_(ci.e, xe, ci.c * x0))))));
}

// Advection rows and traps: the full stencil from the cell sizes and the local
// velocity (out of line; only traps with advection take it, uniformly per CTA).
// Pad columns and nodes outside the grid get an all-zero row.
template <class T>
__device__ __noinline__ void coef_general(const LevelGeom& g, int i, int j, T (&c)[8]) {
  if (j > g.nx || j < 0 || i < 0 || i > g.ny) {  // pad column or outside the grid
#pragma unroll
    for (int q = 0; q < 8; ++q) c[q] = T(0);
    return;
  }
  const T* pre = sizeof(T) == sizeof(float) ? (const T*)(const void*)g.coef_f
                                            : (const T*)(const void*)g.coef_d;
  if (pre) {  // an anisotropic level: the stencils built once (k_aniso_coefs)
    const T* q = pre + 8 * ((long long)i * g.P + j);
#pragma unroll
    for (int e = 0; e < 8; ++e) c[e] = q[e];
    return;
  }
  const T* row = sizeof(T) == sizeof(float) ? (const T*)(const void*)g.rowc_f
                                            : (const T*)(const void*)g.rowc_d;
  if (row) {  // an advective level: the row's stencils built once
    const T* q = row + 8 * ((long long)i * 5 + edge_class(j, g.nx));
#pragma unroll
    for (int e = 0; e < 8; ++e) c[e] = q[e];
    return;
  }
  const Sten<T> s = stencil_general<T, false>(g, i, j);  // advective rows
  c[0] = s.c;
  c[1] = s.e;
  c[2] = s.w;
  c[3] = s.n;
  c[4] = s.s;
  c[5] = s.ne;
  c[6] = s.sw;
  c[7] = T(1) / s.c;
}
// The stencil of a general-path node: an anisotropic level reads the stencil built
// once (k_aniso_coefs) inline, an advective level its row's (built once on the host);
// other general rows compute it out of line.
template <class T>
__device__ __forceinline__ void coef_node(const LevelGeom& g, int i, int j, T (&c)[8]) {
  const T* pre = sizeof(T) == sizeof(float) ? (const T*)(const void*)g.coef_f
                                            : (const T*)(const void*)g.coef_d;
  const T* row = sizeof(T) == sizeof(float) ? (const T*)(const void*)g.rowc_f
                                            : (const T*)(const void*)g.rowc_d;
  if ((pre || row) && j >= 0 && j <= g.nx && i >= 0 && i <= g.ny) {
    // anisotropic: per node; advective: per row and column class (L1-resident)
    const T* q = pre ? pre + 8 * ((long long)i * g.P + j)
                     : row + 8 * ((long long)i * 5 + edge_class(j, g.nx));
    if constexpr (sizeof(T) == sizeof(float)) {  // two aligned 16-byte vectors per node
      const float4 lo = __ldg(reinterpret_cast<const float4*>(q));
      const float4 hi = __ldg(reinterpret_cast<const float4*>(q) + 1);
      c[0] = (T)lo.x;
      c[1] = (T)lo.y;
      c[2] = (T)lo.z;
      c[3] = (T)lo.w;
      c[4] = (T)hi.x;
      c[5] = (T)hi.y;
      c[6] = (T)hi.z;
      c[7] = (T)hi.w;
    } else {
#pragma unroll
      for (int e = 0; e < 8; ++e) c[e] = __ldg(q + e);
    }
    return;
  }
  T t[8];
  coef_general<T>(g, i, j, t);
#pragma unroll
  for (int e = 0; e < 8; ++e) c[e] = t[e];
}
template <class T, class X>
__device__ __forceinline__ T apply_general(const LevelGeom& g, const X& x, int k, int i, int j,
                                           T& idiag) {
  T c[8];
  coef_node<T>(g, i, j, c);
  idiag = c[7];
  const int P = g.P;
  return st_table(c, x[k], x[k + 1], x[k - 1], x[k + P], x[k - P], x[k + P + 1], x[k - P - 1]);
}
template <class T>
__device__ __forceinline__ T inv_diag_general(const LevelGeom& g, int i, int j) {
  T c[8];
  coef_node<T>(g, i, j, c);
  return c[7];
}

// The per-node stencils of an anisotropic level: FP64 stencil_general (the same rows
// the host bounds use), kept in FP64 and rounded to FP32.
__global__ void k_aniso_coefs(const LevelGeom g, float* __restrict__ cf,
                              double* __restrict__ cd) {
  grid_dep_sync();
  const long long n = (long long)g.P * (g.ny + 1);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k / g.P), j = (int)(k - (long long)i * g.P);
    double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (j <= g.nx) {
      const Sten<double> s = stencil_general<double>(g, i, j);
      c[0] = s.c;
      c[1] = s.e;
      c[2] = s.w;
      c[3] = s.n;
      c[4] = s.s;
      c[5] = s.ne;
      c[6] = s.sw;
      c[7] = 1.0 / s.c;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      cd[8 * k + q] = c[q];
      cf[8 * k + q] = (float)c[q];
    }
  }
}

// (A x)_k and 1/diagonal of node (i, j).  Every neighbour index must be readable
// (staged with guard rows); missing neighbours carry zero coefficients.
// MASS: the table holds a class-based operator that advection never changes.
template <class T, class X, bool MASS = false>
__device__ __forceinline__ T apply_tab(const LevelGeom& g, const Interior<T>& ci,
                                       const T* __restrict__ tab, const X& x, int k, int i,
                                       int j, T& idiag) {
  if (!MASS && g.adv_on) return apply_general<T, X>(g, x, k, i, j, idiag);
  const int P = g.P;
  const T x0 = x[k], xe = x[k + 1], xw = x[k - 1], xn = x[k + P], xs = x[k - P];
  const T xne = x[k + P + 1], xsw = x[k - P - 1];
  if (is_uniform_interior(g, i, j)) {
    idiag = ci.ic;
    return st_interior(ci, x0, xe, xw, xn, xs, xne, xsw);
  }
  const T* c = tab + node_class(g, i, j) * kTabStride;
  idiag = c[7];
  return st_table(c, x0, xe, xw, xn, xs, xne, xsw);
}

// GM as apply_quad's: 0 general path when the trap has one, 1 table only, 2 general only.
template <class T, int GM = 0>
__device__ __forceinline__ T inv_diag_tab(const LevelGeom& g, const Interior<T>& ci,
                                          const T* __restrict__ tab, int i, int j) {
  if (GM == 2 || (GM == 0 && g.adv_on)) return inv_diag_general<T>(g, i, j);
  return is_uniform_interior(g, i, j) ? ci.ic : tab[node_class(g, i, j) * kTabStride + 7];
}

// ---------------------------------------------------------------------------
// Aligned quads: nodes [4q, 4q+4) of a trap (trap segments start 128-byte
// aligned, so a quad is one 16-byte vector in FP32).
template <class T>
struct Q4 {
  T v[4];
};
template <class T>
__device__ __forceinline__ Q4<T> vld4(const T* p);  // p 16-byte aligned (FP32) / 32 (FP64)
template <>
__device__ __forceinline__ Q4<float> vld4<float>(const float* p) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  return Q4<float>{{a.x, a.y, a.z, a.w}};
}
template <>
__device__ __forceinline__ Q4<double> vld4<double>(const double* p) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double2 b = reinterpret_cast<const double2*>(p)[1];
  return Q4<double>{{a.x, a.y, b.x, b.y}};
}
template <class T>
__device__ __forceinline__ void vst4(T* p, const Q4<T>& q);
template <>
__device__ __forceinline__ void vst4<float>(float* p, const Q4<float>& q) {
  *reinterpret_cast<float4*>(p) = make_float4(q.v[0], q.v[1], q.v[2], q.v[3]);
}
template <>
__device__ __forceinline__ void vst4<double>(double* p, const Q4<double>& q) {
  reinterpret_cast<double2*>(p)[0] = make_double2(q.v[0], q.v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(q.v[2], q.v[3]);
}
template <class T>
__device__ __forceinline__ Q4<T> ld4(const View<T>& w, int k) {
  return vld4<T>(w.p + (k - w.a));
}
template <class T>
__device__ __forceinline__ Q4<T> View<T>::quad(int k) const {
  return vld4<T>(p + (k - a));
}

// Five consecutive values x[k0 .. k0+4] of a staged row.  FP32: two aligned 16-byte
// loads and a compile-time selection by the misalignment M (the same for every quad
// of a trap: it only depends on the row pitch), free of shared-memory bank
// conflicts; FP64 loads scalars.
template <int M, class T>
struct Row5 {
  static __device__ __forceinline__ void load(const View<T>& w, int k0, T (&out)[5]) {
#pragma unroll
    for (int e = 0; e < 5; ++e) out[e] = w[k0 + e];
  }
};
template <int M>
struct Row5<M, float> {
  static __device__ __forceinline__ void load(const View<float>& w, int k0, float (&out)[5]) {
    const float4* base = reinterpret_cast<const float4*>(w.p + (k0 - w.a - M));
    const float4 A = base[0], B = base[1];
    const float v[8] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w};
#pragma unroll
    for (int e = 0; e < 5; ++e) out[e] = v[M + e];
  }
};
template <class T>
template <int M>
__device__ __forceinline__ void View<T>::row(int k0, T (&out)[5]) const {
  Row5<M, T>::load(*this, k0, out);
}

// A block of quads: grid rows [ra, rb), QW quads per row, quad cq covering columns
// ca + 4 cq .. ca + 4 cq + 3 (a row tile: ca = 0, QW = P / 4; a fused kernel's
// window: its own rows and columns).
struct QuadBlock {
  int ra, rb, ca, QW;
};

// Visits every quad of a block once, in two passes: first the rectangle of quads
// whose four nodes are all uniform-interior nodes (f(i, cq, true_type): every lane
// of a warp takes the interior path), then the rest (f(i, cq, false_type): the
// table path), so that no warp runs both paths with lanes masked off.
template <class F>
__device__ __forceinline__ void for_quads(const LevelGeom& g, const QuadBlock& b, F&& f) {
  // interior rows [2, ny - 2]; columns j = ca + 4 cq with 2 <= j and j + 3 <= nx - 2
  int ia = b.ra > 2 ? b.ra : 2, ib = b.rb - 1 < g.ny - 2 ? b.rb - 1 : g.ny - 2;
  int qa = 2 - b.ca > 0 ? (2 - b.ca + 3) >> 2 : 0;
  int qb = g.nx - 5 - b.ca >= 0 ? (g.nx - 5 - b.ca) >> 2 : -1;
  qb = qb < b.QW - 1 ? qb : b.QW - 1;
  if (g.adv_on || ib < ia || qb < qa) {  // no interior rectangle
    ia = b.ra;
    ib = b.ra - 1;
    qa = 0;
    qb = -1;
  }
  const int RW = qb - qa + 1, RH = ib - ia + 1;
  if (RH > 0) {
    const float inv = __fdividef(1.0f, (float)RW);  // div_pitch corrects the floor by one
    int r, c, dr, dc;
    div_pitch((int)threadIdx.x, RW, inv, r, c);
    div_pitch((int)blockDim.x, RW, inv, dr, dc);
    for (; r < RH;) {
      f(ia + r, qa + c, std::true_type{});
      r += dr;
      c += dc;
      if (c >= RW) {
        c -= RW;
        ++r;
      }
    }
  }
  // the rest: rows above the rectangle, the side quads of its rows, rows below it
  const int top = (RH > 0 ? ia - b.ra : b.rb - b.ra) * b.QW;
  const int nb = b.QW - (RH > 0 ? RW : 0);
  const int mid = RH > 0 ? RH * nb : 0;
  const int bot = RH > 0 ? (b.rb - 1 - ib) * b.QW : 0;
  const int n = top + mid + bot;
  if (n == 0) return;
  const float invq = __fdividef(1.0f, (float)b.QW);
  const float invb = nb > 0 ? __fdividef(1.0f, (float)nb) : 0.0f;
  for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
    int r, c;
    if (idx < top) {
      div_pitch(idx, b.QW, invq, r, c);
      r += b.ra;
    } else if (idx < top + mid) {
      int m;
      div_pitch(idx - top, nb, invb, r, m);
      r += ia;
      c = m < qa ? m : m + RW;
    } else {
      div_pitch(idx - top - mid, b.QW, invq, r, c);
      r += ib + 1;
    }
    f(r, c, std::false_type{});
  }
}

// Node (i, j) of node kk = 4q + e, from the quad's first node (i0, j0).
// Rows are padded to a multiple of 4 nodes, so a quad never leaves its row.
__device__ __forceinline__ void quad_node(int P, int i0, int j0, int e, int& i, int& j) {
  (void)P;
  i = i0;
  j = j0 + e;
}

// Class of a node that may lie outside the grid (guard rows and columns of staged
// windows): those take the all-zero pad class, so they stay exactly zero.
__device__ __forceinline__ int node_class_clamped(const LevelGeom& g, int i, int j) {
  if (i < 0 || i > g.ny || j < 0) return kClassPad;
  return node_class(g, i, j);
}

// The trap's class table in shared memory, with the interior class replaced by
// the interior weights, so that a node of the interior class evaluates to the same
// bits through the table as through the interior constants.  stage_table carves
// the region; the returned filler runs inside Stager::run / stage_rows, after the
// bulk copies are issued, so the table's global loads overlap them.
template <class T>
struct TableStage {
  T* s;
  const T* tab;
  Interior<T> ci;
  __device__ __forceinline__ void operator()() const {
    for (int e = threadIdx.x; e < kTabPerTrap; e += blockDim.x) {
      T v = tab[e];
      const int q = e - 12 * kTabStride;
      if (q >= 0 && q < kTabStride)
        v = q == 0 ? ci.c : (q <= 2 ? ci.e : (q <= 4 ? ci.n : (q <= 6 ? ci.d : ci.ic)));
      s[e] = v;
    }
  }
};
template <class T>
__device__ __forceinline__ TableStage<T> stage_table(Stager& st, const T* __restrict__ tab,
                                                     const Interior<T>& ci) {
  T* s = reinterpret_cast<T*>(st.cur);
  st.cur += kTabPerTrap * sizeof(T);
  return TableStage<T>{s, tab, ci};
}

// A region of `count` elements of shared memory after the staged ranges (16-byte
// aligned, with the 16-byte pad every region keeps after it).
template <class T>
__device__ __forceinline__ T* carve(Stager& st, int count) {
  T* p = reinterpret_cast<T*>(st.cur);
  st.cur += (((uint32_t)count * sizeof(T) + 15u) & ~15u) + 16u;
  return p;
}

// Quad halo window: one row and nine nodes each side, so that every vector load of
// a quad that overlaps the tile (quads start 4-aligned, up to 3 nodes before the
// tile) stays inside the staged, zero-guarded window.
__device__ __forceinline__ int qhalo_lo(const LevelGeom& g, const Tile& t) {
  return t.k0 - g.P - 8;
}
__device__ __forceinline__ int qhalo_hi(const LevelGeom& g, const Tile& t) {
  return t.k1 + g.P + 8;
}

// A x and 1/diagonal on a quad.  Every quad makes the same 13 loads (centre
// vector, two row ends, five above, five below); only the weights differ:
// interior quads use the interior constants, the others (walls, row ends, ragged
// last cells, advection traps) take per-node weights from the staged class table.
// PM = P mod 4, the row misalignment of the neighbour rows (0: device rows are
// padded to a multiple of 4 nodes); x's base index is a multiple of 4.
// GM selects the border path's weights: 0 the general path when the trap has one
// (g.adv_on), else the class table; 1 the class table only (kernels launched on the
// tiles of class-table traps); 2 the general path only, fetched inline (kernels
// launched on the tiles of general-path traps: the fetch's registers stay out of the
// class-table kernels).
template <bool GEN>
constexpr int kGM = GEN ? 2 : 1;  // apply_quad's border weights for a GEN kernel
template <class T, int PM, class X, int GM = 0>
__device__ __forceinline__ Q4<T> apply_quad(const LevelGeom& g, const Interior<T>& ci,
                                            const T* __restrict__ stab, const X& x, int k,
                                            int P, int i0, int j0, bool inner, Q4<T>& xc,
                                            Q4<T>& id) {
  xc = x.quad(k);
  const T xw = x[k - 1], xe = x[k + 4];
  T nr[5], sr[5];
  x.template row<PM>(k + P, nr);           // nr[e]: N of node e, NE of node e-1
  x.template row<3 - PM>(k - P - 1, sr);   // sr[e]: SW of node e, S of node e-1
  Q4<T> ax;
  if (inner) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const T w = e == 0 ? xw : xc.v[e - 1];
      const T ee = e == 3 ? xe : xc.v[e + 1];
      ax.v[e] = st_interior(ci, xc.v[e], ee, w, nr[e], sr[e + 1], nr[e + 1], sr[e]);
      id.v[e] = ci.ic;
    }
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      int i, j;
      quad_node(P, i0, j0, e, i, j);
      const T w = e == 0 ? xw : xc.v[e - 1];
      const T ee = e == 3 ? xe : xc.v[e + 1];
      if (GM == 2 || (GM == 0 && g.adv_on)) {
        T c[8];  // general rows: out of line in shared kernels (an inline fetch spills
        if (GM == 2)  // the class-table path), inline in the general-path kernels
          coef_node<T>(g, i, j, c);
        else
          coef_general<T>(g, i, j, c);
        ax.v[e] = st_table(c, xc.v[e], ee, w, nr[e], sr[e + 1], nr[e + 1], sr[e]);
        id.v[e] = c[7];
      } else {
        const T* t = stab + node_class_clamped(g, i, j) * kTabStride;
        const Q4<T> lo = vld4<T>(t), hi = vld4<T>(t + 4);
        const T c[8] = {lo.v[0], lo.v[1], lo.v[2], lo.v[3], hi.v[0], hi.v[1], hi.v[2], hi.v[3]};
        ax.v[e] = st_table(c, xc.v[e], ee, w, nr[e], sr[e + 1], nr[e + 1], sr[e]);
        id.v[e] = c[7];
      }
    }
  }
  return ax;
}

// Sum over the CTA of the warps' sums (lane 0 of each warp holds one): FP64 in
// warp 0, a shuffle tree over the warps present.  Valid in thread 0.
__device__ __forceinline__ double warps_sum(double v) {
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1)
      if (o < nw) t += __shfl_down_sync(0xffffffffu, t, o);  // (adding the zeros beyond
  }                                                           //  nw would change nothing)
  __syncthreads();
  return t;
}
__device__ __forceinline__ double block_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return warps_sum(v);
}
// FP32 partials: the warp stage in FP32 (five dependent FP64 adds would cost several
// hundred cycles on this part's narrow FP64 pipe), the warps' sums in FP64.
__device__ __forceinline__ double block_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return warps_sum((double)v);
}

// Optional profiling counter: nodes actually processed by a launch (tiles of
// skipped traps do not count).  One atomic per CTA, only when profiling.
__device__ __forceinline__ void count_work(unsigned long long* work, const Tile& t) {
  if (work && threadIdx.x == 0) atomicAdd(work, (unsigned long long)(t.k1 - t.k0));
}

// halo window of a tile: one row plus one node each side (may leave the trap)
__device__ __forceinline__ int halo_lo(const LevelGeom& g, const Tile& t) {
  return t.k0 - g.P - 1;
}
__device__ __forceinline__ int halo_hi(const LevelGeom& g, const Tile& t) {
  return t.k1 + g.P + 1;
}

// ---------------------------------------------------------------------------
// Chebyshev step coefficients of one step.
struct ChebCoef {
  float c_old;  // multiplies the previous direction
  float c_res;  // multiplies D^-1 r
};
// Step `s` of the level's Chebyshev table.
__device__ __forceinline__ ChebCoef cheb_at(const LevelGeom& g, int s) {
  return ChebCoef{g.ch_old[s], g.ch_res[s]};
}

// d_new = c_res (b - Ax) / diag (+ c_old d_old), one fixed evaluation order
template <class T, bool FIRST>
__device__ __forceinline__ T cheb_dir(const ChebCoef& cc, T bk, T ax, T id, T dold) {
  const T base = (T(cc.c_res) * (bk - ax)) * id;
  return FIRST ? base : fma_(T(cc.c_old), dold, base);
}

// Chebyshev-Jacobi step on one level.
//   ZERO (x_in = 0): x_out = d = D^-1 b / theta            (streaming, no staging)
//   FIRST:           d = D^-1 (b - A x_in) / theta; x_out = x_in + d
//   otherwise:       d = c_old d + c_res D^-1 (b - A x_in); x_out = x_in + d
// The coefficients come from the level's Chebyshev table (the smoothing interval,
// or the full interval on the coarsest level).  DOT adds a partial of b.x_out.
// GEN as k_cg_dir's: the launch covers general-path traps' tiles or class-table ones.
template <class T, bool FIRST, bool ZERO, bool DOT, bool GEN>
__global__ void __launch_bounds__(kThreads, kStencilCtas<T>)
    k_cheb(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
           const T* __restrict__ tabs, const int* __restrict__ skip, int step,
           const T* __restrict__ b, const T* __restrict__ xin, T* __restrict__ xout,
           T* __restrict__ d, double* __restrict__ part, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (DOT && threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  count_work(work, tile);
  const ChebCoef cc = cheb_at(g, FIRST ? 0 : step);
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  const T* bs = b + g.off;
  T* xo = xout + g.off;
  T* ds = d + g.off;
  const int P = g.P;
  T acc = T(0);
  // tiles are whole rows: every quad lies inside the tile
  const QuadBlock qb{tile.r0, tile.r1, 0, P >> 2};
  if (ZERO) {
    for_quads(g, qb, [&](int i, int cq, auto inner_) {
      constexpr bool INNER = decltype(inner_)::value;
      const int k = i * P + 4 * cq;
      const Q4<T> bq = vld4<T>(bs + k);
      Q4<T> id;
      if (INNER) {
#pragma unroll
        for (int e = 0; e < 4; ++e) id.v[e] = ci.ic;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          id.v[e] = inv_diag_tab<T, kGM<GEN>>(g, ci, tab, i, 4 * cq + e);
      }
      Q4<T> dn;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        dn.v[e] = (T(cc.c_res) * bq.v[e]) * id.v[e];
        if (DOT) acc += bq.v[e] * dn.v[e];
      }
      vst4<T>(xo + k, dn);
      vst4<T>(ds + k, dn);
    });
  } else {
    Stager st(eqf_smem);
    const int na = padded_len(g);
    const View<T> xv = st.add_guarded(xin + g.off, qhalo_lo(g, tile), qhalo_hi(g, tile), na);
    const View<T> bv = st.add(bs, tile.k0, tile.k1, na);
    View<T> dv = bv;
    if (!FIRST) dv = st.add(static_cast<const T*>(ds), tile.k0, tile.k1, na);
    const TableStage<T> tst = stage_table<T>(st, tab, ci);
    const T* stab = tst.s;
    if (!st.run(tst)) return;
    for_quads(g, qb, [&](int i, int cq, auto inner_) {
      constexpr bool INNER = decltype(inner_)::value;
      const int j = 4 * cq, k = i * P + j;
      Q4<T> xc, id;
      const Q4<T> ax =
          apply_quad<T, 0, View<T>, kGM<GEN>>(g, ci, stab, xv, k, P, i, j, INNER, xc, id);
      const Q4<T> bq = bv.quad(k);
      const Q4<T> dq = FIRST ? bq : dv.quad(k);
      Q4<T> dn, xn;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        dn.v[e] = cheb_dir<T, FIRST>(cc, bq.v[e], ax.v[e], id.v[e], dq.v[e]);
        xn.v[e] = xc.v[e] + dn.v[e];
        if (DOT) acc += bq.v[e] * xn.v[e];
      }
      vst4<T>(xo + k, xn);
      vst4<T>(ds + k, dn);
    });
  }
  if (DOT) {
    const double t = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

// t = b - A x
template <class T>
__global__ void __launch_bounds__(kThreads, kStencilCtas<T>)
    k_resid(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
            const T* __restrict__ tabs, const int* __restrict__ skip, const T* __restrict__ b,
            const T* __restrict__ x, T* __restrict__ t, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) return;
  count_work(work, tile);
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  Stager st(eqf_smem);
  const int na = padded_len(g);
  const View<T> xv = st.add_guarded(x + g.off, qhalo_lo(g, tile), qhalo_hi(g, tile), na);
  const View<T> bv = st.add(b + g.off, tile.k0, tile.k1, na);
  const TableStage<T> tst = stage_table<T>(st, tab, ci);
  const T* stab = tst.s;
  if (!st.run(tst)) return;
  T* ts = t + g.off;
  const int P = g.P;
  // tiles are whole rows: every quad lies inside the tile
  for_quads(g, QuadBlock{tile.r0, tile.r1, 0, P >> 2}, [&](int i, int cq, auto inner_) {
    constexpr bool INNER = decltype(inner_)::value;
    const int j = 4 * cq, k = i * P + j;
    Q4<T> xc, id;
    const Q4<T> ax = apply_quad<T, 0>(g, ci, stab, xv, k, P, i, j, INNER, xc, id);
    const Q4<T> bq = bv.quad(k);
    Q4<T> r;
#pragma unroll
    for (int e = 0; e < 4; ++e) r.v[e] = bq.v[e] - ax.v[e];
    vst4<T>(ts + k, r);
  });
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
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) return;
  count_work(work, tile);
  const int nfx = g.fine_nx, nfy = g.fine_ny, PF = g.fine_P;
  int fr0 = coarse_to_fine(tile.r0, nfy, g.cy) - 1;
  int fr1 = coarse_to_fine(tile.r1 - 1, nfy, g.cy) + 2;
  fr0 = fr0 < 0 ? 0 : fr0;
  fr1 = fr1 > nfy + 1 ? nfy + 1 : fr1;
  const int naf = ((PF * (nfy + 1)) + 31) & ~31;
  Stager st(eqf_smem);
  const View<T> t = st.add(tf + g.fine_off, fr0 * PF, fr1 * PF, naf);
  if (!st.run()) return;
  T* b = bc + g.off;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    if (w.j > g.nx || (g.walls && is_dirichlet(g, w.i, w.j))) {  // pad column or wall
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
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) return;
  count_work(work, tile);
  const LevelGeom& c = Gc[tile.geom];
  const int PC = c.P;
  int lo0, hi0, lo1, hi1;
  fine_to_coarse(tile.r0, g.ny, c.cy, lo0, hi0);
  fine_to_coarse(tile.r1 - 1, g.ny, c.cy, lo1, hi1);
  Stager st(eqf_smem);
  const View<T> xcs = st.add(xc + c.off, lo0 * PC, (hi1 + 1) * PC, padded_len(c));
  if (!st.run()) return;
  T* xs = xf + g.off;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    if (w.j > g.nx) continue;  // pad column stays zero
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
// 512 threads, the largest traps' CTAs first (order): the launch's time is its
// largest CTA's chain of `deg` barrier-separated sweeps.
constexpr int kCoarseThreads = 512;
template <class T>
__global__ void __launch_bounds__(kCoarseThreads)
    k_coarse_solve(const LevelGeom* __restrict__ G, const T* __restrict__ tabs,
                   const int* __restrict__ skip, int deg, const T* __restrict__ b,
                   T* __restrict__ xout, const int* __restrict__ order) {
  grid_dep_sync();
  const LevelGeom& g = G[order ? order[blockIdx.x] : (int)blockIdx.x];
  if (skip && skip[g.trap]) return;
  const int n = g.P * (g.ny + 1);
  const int na = padded_len(g);
  const int gpad = ((g.P + 1 + 7) / 8) * 8;
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
    const ChebCoef cc = cheb_at(g, it);
    const View<T>& xi = (it & 1) ? xbv : xav;
    T* xo = (it & 1) ? xa : xb;
    for (NodeWalk w(g, 0); w.k < n; w.next()) {
      T id;
      const T ax = apply_tab<T>(g, ci, tab, xi, w.k, w.i, w.j, id);
      T dn = (T(cc.c_res) * (bv[w.k] - ax)) * id;
      if (it > 0) dn = fma_(T(cc.c_old), dd[w.k], dn);
      dd[w.k] = dn;
      xo[w.k] = add_(xi[w.k], dn);
    }
    __syncthreads();
  }
  const T* xf = (deg & 1) ? xb : xa;
  T* out = xout + g.off;
  for (int k = threadIdx.x; k < n; k += blockDim.x) out[k] = xf[k];
}

// ---------------------------------------------------------------------------
// The bottom of the V-cycle in one CTA per trap: levels lb .. coarsest of one trap
// live in shared memory, and the kernel runs what the fused V(2,2) path does there
// (k_down's two pre-smoothing steps from zero and residual, k_restrict, k_coarse_solve,
// k_up's prolongation and two post-smoothing steps), node by node with the same
// expressions on the same operands, so its results are bit-identical to that path and
// the small levels cost one launch instead of seven, with no HBM round trips.
constexpr int kMaxBottom = 4;      // levels in the bottom kernel
constexpr int kBottomThreads = 512;
template <class T>
struct BottomArgs {
  const LevelGeom* G[kMaxBottom];  // per level lb + m: the level's geometry array (by trap)
  const T* tabs[kMaxBottom];       // and its class tables
  int nlev;                        // levels lb .. lb + nlev - 1 (the last the coarsest)
  int deg_pre, deg_coarse;  // (two post-smoothing steps, as k_up)
  const int* order;         // trap of each CTA, largest first (the tail is the largest
                            // trap's), or null: CTA b solves trap b
};
// Shared-memory bytes of one level: rhs b and direction d, iterates x and y with
// zero guards of gpad >= P + 1 nodes each side.
EQF_HD size_t bottom_level_bytes(int P, int ny, int tsize) {
  const long long na = (((long long)P * (ny + 1)) + 31) & ~31ll;
  const long long gp = ((P + 1 + 7) / 8) * 8;
  return (size_t)((4 * na + 4 * gp) * tsize);
}

template <class T>
struct BottomLevel {
  T *b, *x, *y, *d;  // x and y point at node 0 (guards before and after)
  int n, na, gp;
};

template <class T>
__device__ __forceinline__ void bottom_sweep(const LevelGeom& g, const Interior<T>& ci,
                                             const T* __restrict__ tab, const ChebCoef& cc,
                                             bool first, const T* b, const T* x, T* xo, T* d,
                                             int n) {
  const View<T> xv{x, 0};
  for (NodeWalk w(g, 0); w.k < n; w.next()) {
    T id;
    const T ax = apply_tab<T>(g, ci, tab, xv, w.k, w.i, w.j, id);
    const T dn = first ? (T(cc.c_res) * (b[w.k] - ax)) * id
                       : cheb_dir<T, false>(cc, b[w.k], ax, id, d[w.k]);
    d[w.k] = dn;
    xo[w.k] = add_(x[w.k], dn);
  }
  __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(kBottomThreads, 1)
    k_bottom(const BottomArgs<T> a, const int* __restrict__ skip, const T* __restrict__ b0,
             T* __restrict__ x0) {
  grid_dep_sync();
  const int trap = a.order ? a.order[blockIdx.x] : (int)blockIdx.x;
  if (skip && skip[trap]) return;
  BottomLevel<T> lv[kMaxBottom];
  Stager st(eqf_smem);
  const LevelGeom& g0 = a.G[0][trap];
  const int n0 = g0.P * (g0.ny + 1);
  const View<T> b0v = st.add(b0 + g0.off, 0, n0, padded_len(g0));  // level lb's rhs
  lv[0].b = const_cast<T*>(b0v.p);
  for (int m = 0; m < a.nlev; ++m) {
    const LevelGeom& g = a.G[m][trap];
    BottomLevel<T>& L = lv[m];
    L.n = g.P * (g.ny + 1);
    L.na = padded_len(g);
    L.gp = ((g.P + 1 + 7) / 8) * 8;
    if (m > 0) L.b = carve<T>(st, L.na);
    T* xg = carve<T>(st, 2 * (L.na + 2 * L.gp));  // x and y with their guards
    L.x = xg + L.gp;
    L.y = L.x + L.na + 2 * L.gp;
    L.d = carve<T>(st, L.na);
  }
  // zero the iterates and their guards (disjoint from the staged rhs) while it lands
  if (!st.run([&] {
        for (int m = 0; m < a.nlev; ++m) {
          T* xg = lv[m].x - lv[m].gp;
          for (int e = threadIdx.x; e < 2 * (lv[m].na + 2 * lv[m].gp); e += blockDim.x)
            xg[e] = T(0);
        }
      }))
    return;
  const int mc = a.nlev - 1;
  // down: pre-smoothing from zero, residual (into y), restriction
  for (int m = 0; m < mc; ++m) {
    const LevelGeom& g = a.G[m][trap];
    const T* tab = a.tabs[m] + (size_t)trap * kTabPerTrap;
    const Interior<T> ci = interior<T>(g);
    BottomLevel<T>& L = lv[m];
    {
      const ChebCoef cc = cheb_at(g, 0);
      for (NodeWalk w(g, 0); w.k < L.n; w.next()) {
        const T dn = (T(cc.c_res) * L.b[w.k]) * inv_diag_tab<T>(g, ci, tab, w.i, w.j);
        L.x[w.k] = dn;
        L.d[w.k] = dn;
      }
      __syncthreads();
    }
    for (int s = 1; s < a.deg_pre; ++s) {
      bottom_sweep<T>(g, ci, tab, cheb_at(g, s), false, L.b, L.x, L.y, L.d, L.n);
      T* t = L.x;
      L.x = L.y;
      L.y = t;
    }
    {
      const View<T> xv{L.x, 0};
      for (NodeWalk w(g, 0); w.k < L.n; w.next()) {
        T id;
        L.y[w.k] = L.b[w.k] - apply_tab<T>(g, ci, tab, xv, w.k, w.i, w.j, id);
      }
      __syncthreads();
    }
    // b_c = P^T t on the coarse level (k_restrict's gather)
    const LevelGeom& gc = a.G[m + 1][trap];
    const BottomLevel<T>& C = lv[m + 1];
    const T* t = L.y;
    const int nfx = gc.fine_nx, nfy = gc.fine_ny, PF = gc.fine_P;
    for (NodeWalk w(gc, 0); w.k < C.n; w.next()) {
      if (w.j > gc.nx || (gc.walls && is_dirichlet(gc, w.i, w.j))) {
        C.b[w.k] = T(0);
        continue;
      }
      const int fi = coarse_to_fine(w.i, nfy, gc.cy), fj = coarse_to_fine(w.j, nfx, gc.cx);
      const int kf = fj + fi * PF;
      T half = T(0);
      const bool mE = fj + 1 <= nfx && is_mid(fj + 1, nfx, gc.cx);
      const bool mW = fj - 1 >= 0 && is_mid(fj - 1, nfx, gc.cx);
      const bool mN = fi + 1 <= nfy && is_mid(fi + 1, nfy, gc.cy);
      const bool mS = fi - 1 >= 0 && is_mid(fi - 1, nfy, gc.cy);
      if (mE) half += t[kf + 1];
      if (mW) half += t[kf - 1];
      if (mN) half += t[kf + PF];
      if (mS) half += t[kf - PF];
      if (mE && mN) half += t[kf + PF + 1];
      if (mW && mS) half += t[kf - PF - 1];
      C.b[w.k] = t[kf] + T(0.5) * half;
    }
    __syncthreads();
  }
  // the coarsest level: deg_coarse Chebyshev iterations from zero (k_coarse_solve's)
  {
    const LevelGeom& g = a.G[mc][trap];
    const T* tab = a.tabs[mc] + (size_t)trap * kTabPerTrap;
    const Interior<T> ci = interior<T>(g);
    BottomLevel<T>& L = lv[mc];
    for (int it = 0; it < a.deg_coarse; ++it) {
      const ChebCoef cc = cheb_at(g, it);
      const View<T> xi{L.x, 0};
      for (NodeWalk w(g, 0); w.k < L.n; w.next()) {
        T id;
        const T ax = apply_tab<T>(g, ci, tab, xi, w.k, w.i, w.j, id);
        T dn = (T(cc.c_res) * (L.b[w.k] - ax)) * id;
        if (it > 0) dn = fma_(T(cc.c_old), L.d[w.k], dn);
        L.d[w.k] = dn;
        L.y[w.k] = add_(L.x[w.k], dn);
      }
      __syncthreads();
      T* t = L.x;
      L.x = L.y;
      L.y = t;
    }
  }
  // up: prolongation (k_prolong's), post-smoothing
  for (int m = mc - 1; m >= 0; --m) {
    const LevelGeom& g = a.G[m][trap];
    const LevelGeom& gc = a.G[m + 1][trap];
    const T* tab = a.tabs[m] + (size_t)trap * kTabPerTrap;
    const Interior<T> ci = interior<T>(g);
    BottomLevel<T>& L = lv[m];
    const T* xc = lv[m + 1].x;
    const int PC = gc.P;
    for (NodeWalk w(g, 0); w.k < L.n; w.next()) {
      if (w.j > g.nx) continue;  // pad column stays zero
      int i0, i1, j0, j1;
      fine_to_coarse(w.i, g.ny, gc.cy, i0, i1);
      fine_to_coarse(w.j, g.nx, gc.cx, j0, j1);
      T v;
      if (i0 == i1 && j0 == j1)
        v = xc[j0 + i0 * PC];
      else if (i0 == i1)
        v = T(0.5) * (xc[j0 + i0 * PC] + xc[j1 + i0 * PC]);
      else if (j0 == j1)
        v = T(0.5) * (xc[j0 + i0 * PC] + xc[j0 + i1 * PC]);
      else
        v = T(0.5) * (xc[j0 + i0 * PC] + xc[j1 + i1 * PC]);  // on the coarse diagonal
      L.x[w.k] += v;
    }
    __syncthreads();
    // post-smoothing as k_up does it: x1 = x0 + c0 D^-1 (b - A x0), then
    // x2 = x1 + c_old (x1 - x0) + c1 D^-1 (b - A x1), the direction recomputed as x1 - x0
    bottom_sweep<T>(g, ci, tab, cheb_at(g, 0), true, L.b, L.x, L.y, L.d, L.n);
    {
      const ChebCoef cc = cheb_at(g, 1);
      const View<T> x1v{L.y, 0};
      for (NodeWalk w(g, 0); w.k < L.n; w.next()) {
        T id;
        const T ax = apply_tab<T>(g, ci, tab, x1v, w.k, w.i, w.j, id);
        const T x1 = L.y[w.k], x0 = L.x[w.k];
        L.x[w.k] = x1 + cheb_dir<T, false>(cc, L.b[w.k], ax, id, x1 - x0);  // own node only
      }
      __syncthreads();
    }
  }
  T* out = x0 + g0.off;
  for (int k = threadIdx.x; k < lv[0].n; k += blockDim.x) out[k] = lv[0].x[k];
}

// ---------------------------------------------------------------------------
// CG on the finest level.  Per-trap scalars live in CgState.
struct CgState {
  double rz, pq, rr, rr0, alpha, beta, bb, r64;
  double gamma;     // extrapolation factor of the initial guess
  double dn2_prev;  // |increment|^2 of the previous step
  double omega;     // BiCGSTAB: stabilisation factor (rz = rho, pq = rhat.v)
  int iters, sweeps, it_in_sweep;
  int pend;  // alpha p of the last iteration is not yet in the correction x
};

// p_out = z (FIRST) or z + beta p_in; q = A p_out; partial dot(p_out, q).
// p is ping-ponged because neighbours of p_out are recomputed from p_in.
template <class T, bool FIRST>
struct PNew {  // p_out = z + beta p_in evaluated on the fly from the staged z, p_in
  View<T> z, p;
  T beta;
  __device__ __forceinline__ T operator[](int k) const {
    return FIRST ? z[k] : fma_(beta, p[k], z[k]);
  }
  __device__ __forceinline__ Q4<T> quad(int k) const {
    Q4<T> a = z.quad(k);
    if (!FIRST) {
      const Q4<T> b = p.quad(k);
#pragma unroll
      for (int e = 0; e < 4; ++e) a.v[e] = fma_(beta, b.v[e], a.v[e]);
    }
    return a;
  }
  template <int M>
  __device__ __forceinline__ void row(int k0, T (&out)[5]) const {
    z.template row<M>(k0, out);
    if (!FIRST) {
      T pr[5];
      p.template row<M>(k0, pr);
#pragma unroll
      for (int e = 0; e < 5; ++e) out[e] = fma_(beta, pr[e], out[e]);
    }
  }
};

// GEN: launched on the tiles of general-path traps (inline stencil fetch), else on
// the tiles of class-table traps only (see apply_quad).
// One row tile (index ti of the launch's tile array); returns kTileSkipped, kTileDone
// or kTileFailed.
template <class T, bool FIRST, bool GEN>
__device__ __forceinline__ int cgdir_tile(const LevelGeom* __restrict__ G, const Tile& tile,
                                          int ti, const T* __restrict__ tabs,
                                          const int* __restrict__ skip,
                                          const CgState* __restrict__ st, const T* __restrict__ z,
                                          const T* __restrict__ pin, T* __restrict__ pout,
                                          T* __restrict__ q, double* __restrict__ part,
                                          unsigned long long* work) {
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (threadIdx.x == 0) part[ti] = 0.0;
    return kTileSkipped;
  }
  count_work(work, tile);
  const T beta = FIRST ? T(0) : T(st[g.trap].beta);
  Stager sg(eqf_smem);
  const int na = padded_len(g);
  const int ka = qhalo_lo(g, tile), kb = qhalo_hi(g, tile);
  const View<T> zv = sg.add_guarded(z + g.off, ka, kb, na);
  View<T> pv = zv;
  if (!FIRST) pv = sg.add_guarded(pin + g.off, ka, kb, na);
  const T* tab = tabs + (size_t)g.trap * kTabPerTrap;
  const Interior<T> ci = interior<T>(g);
  const TableStage<T> tst = stage_table<T>(sg, tab, ci);
  const T* stab = tst.s;
  if (!sg.run(tst)) return kTileFailed;
  const PNew<T, FIRST> pnew{zv, pv, beta};
  T* po = pout + g.off;
  T* qs = q + g.off;
  const int P = g.P;
  T acc = T(0);
  // tiles are whole rows: every quad lies inside the tile
  for_quads(g, QuadBlock{tile.r0, tile.r1, 0, P >> 2}, [&](int i, int cq, auto inner_) {
    constexpr bool INNER = decltype(inner_)::value;
    const int j = 4 * cq, k = i * P + j;
    Q4<T> pc, id;
    const Q4<T> a =
        apply_quad<T, 0, PNew<T, FIRST>, kGM<GEN>>(g, ci, stab, pnew, k, P, i, j, INNER, pc, id);
#pragma unroll
    for (int e = 0; e < 4; ++e) acc += pc.v[e] * a.v[e];
    vst4<T>(po + k, pc);
    vst4<T>(qs + k, a);
  });
  const double t = block_sum(acc);
  if (threadIdx.x == 0) part[ti] = t;
  return kTileDone;
}

// LIST: the CTAs stride over a device-built list of the iterating traps' row tiles
// (late refinement sweeps); otherwise CTA b takes tile b.
template <class T, bool FIRST, bool GEN, bool LIST = false>
__global__ void __launch_bounds__(kThreads, kStencilCtas<T>)
    k_cg_dir(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
             const T* __restrict__ tabs, const int* __restrict__ skip,
             const CgState* __restrict__ st, const T* __restrict__ z, const T* __restrict__ pin,
             T* __restrict__ pout, T* __restrict__ q, double* __restrict__ part,
             TileList tlist, unsigned long long* work) {
  if constexpr (!LIST) {
    const Tile tile = tiles[blockIdx.x];  // static: read before the wait
    prefetch_l1(G + tile.geom);
    grid_dep_sync();
    cgdir_tile<T, FIRST, GEN>(G, tile, (int)blockIdx.x, tabs, skip, st, z, pin, pout, q, part,
                              work);
  } else {
    grid_dep_sync();
    const int n = *tlist.count;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
      const int ti = tlist.idx[w];
      const int rc = cgdir_tile<T, FIRST, GEN>(G, tiles[ti], ti, tabs, skip, st, z, pin, pout,
                                               q, part, work);
      if (rc == kTileFailed) return;
      next_listed_tile(rc);
    }
  }
}

// x += alpha p; r -= alpha q; partial dot(r, r)   (streaming, quads)
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_cg_update(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                const int* __restrict__ skip, const CgState* __restrict__ st,
                const T* __restrict__ p, const T* __restrict__ q, T* __restrict__ x,
                T* __restrict__ r, double* __restrict__ part, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) {
    if (threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  count_work(work, tile);
  const T alpha = T(st[g.trap].alpha);
  const long long o = g.off;
  T acc = T(0);
  const int qa = tile.k0 >> 2, qb = (tile.k1 + 3) >> 2;
  for (int qq = qa + threadIdx.x; qq < qb; qq += blockDim.x) {
    const int k = 4 * qq;
    if (k >= tile.k0 && k + 4 <= tile.k1) {
      const Q4<T> pq = vld4<T>(p + o + k), qv = vld4<T>(q + o + k);
      Q4<T> xq = vld4<T>(x + o + k), rq = vld4<T>(r + o + k);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        xq.v[e] = fma_(alpha, pq.v[e], xq.v[e]);
        rq.v[e] = fma_(-alpha, qv.v[e], rq.v[e]);
        acc += rq.v[e] * rq.v[e];
      }
      vst4<T>(x + o + k, xq);
      vst4<T>(r + o + k, rq);
    } else {
      for (int kk = k; kk < k + 4; ++kk) {
        if (kk < tile.k0 || kk >= tile.k1) continue;
        x[o + kk] = fma_(alpha, p[o + kk], x[o + kk]);
        const T rn = fma_(-alpha, q[o + kk], r[o + kk]);
        r[o + kk] = rn;
        acc += rn * rn;
      }
    }
  }
  const double t = block_sum(acc);
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
               const int* __restrict__ frozen, unsigned long long* work) {
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
  const LevelGeom& g = G[tile.geom];
  if (frozen[g.trap]) {
    if (threadIdx.x == 0) part[blockIdx.x] = part[ntiles + blockIdx.x] = 0.0;
    return;
  }
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
    // Dirichlet rows: the identity with the wall value (held in F) or 0
    const double bk = dir ? (g.dvals ? fv[k] : 0.0) : fv[k] + mu;
    const double rk = dir ? (g.dvals ? bk - u0[k] : 0.0)
                          : bk - apply_tab<double>(g, ci, tA, u0, k, w.i, w.j, id);
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
  const Tile tile = tiles[blockIdx.x];  // static: read before the wait
  prefetch_l1(G + tile.geom);
  grid_dep_sync();
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
      const double rk = dir ? (g.dvals ? bv[w.k] - uv[w.k] : 0.0)
                            : bv[w.k] - apply_tab<double>(g, ci, tA, uv, w.k, w.i, w.j, id);
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

// Exact conversion to double: floats by repacking their bits (no FP64-pipe convert).
__device__ __forceinline__ double to_double(double v) { return v; }
__device__ __forceinline__ double to_double(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xFFu;
  const unsigned long long s = (unsigned long long)(b & 0x80000000u) << 32;
  const unsigned long long ex = e == 0xFFu ? 0x7FFull : (unsigned long long)(e + 896u);
  const unsigned long long m = (unsigned long long)(b & 0x7FFFFFu) << 29;
  return __longlong_as_double(e == 0u ? s : (s | (ex << 52) | m));
}

// u += x; d += x (the inner-solve correction)   (streaming, quads).  A trap whose
// last Krylov update is pending (CgState::pend, folded CG) takes x + alpha p_last,
// the value k_cg_update would have left in x; after a single iteration the folded
// CG never wrote x (it is not zeroed per sweep), so x = alpha p_last.
template <class T>
__device__ __forceinline__ void irupd_tile(const LevelGeom* __restrict__ G, const Tile& tile,
                                           const int* __restrict__ skip,
                                           const T* __restrict__ x, double* __restrict__ u,
                                           float* __restrict__ d,
                                           const CgState* __restrict__ st,
                                           const T* __restrict__ plast,
                                           unsigned long long* work) {
  const LevelGeom& g = G[tile.geom];
  if (skip && skip[g.trap]) return;
  count_work(work, tile);
  const long long o = g.off;
  const bool pend = plast && st[g.trap].pend;
  const bool only = pend && st[g.trap].it_in_sweep == 1;  // x holds nothing of this sweep
  const T alpha = pend ? T(st[g.trap].alpha) : T(0);
  const int qa = tile.k0 >> 2, qb = (tile.k1 + 3) >> 2;
  for (int qq = qa + threadIdx.x; qq < qb; qq += blockDim.x) {
    const int k = 4 * qq;
    if (k >= tile.k0 && k + 4 <= tile.k1) {
      Q4<T> xq;
      if (only) {
        const Q4<T> pq = vld4<T>(plast + o + k);
#pragma unroll
        for (int e = 0; e < 4; ++e) xq.v[e] = alpha * pq.v[e];
      } else {
        xq = vld4<T>(x + o + k);
        if (pend) {
          const Q4<T> pq = vld4<T>(plast + o + k);
#pragma unroll
          for (int e = 0; e < 4; ++e) xq.v[e] = fma_(alpha, pq.v[e], xq.v[e]);
        }
      }
      Q4<double> uq = vld4<double>(u + o + k);
      Q4<float> dq = vld4<float>(d + o + k);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        uq.v[e] += to_double(xq.v[e]);
        dq.v[e] += float(xq.v[e]);
      }
      vst4<double>(u + o + k, uq);
      vst4<float>(d + o + k, dq);
    } else {
      for (int kk = k; kk < k + 4; ++kk) {
        if (kk < tile.k0 || kk >= tile.k1) continue;
        T v = only ? alpha * plast[o + kk] : x[o + kk];
        if (pend && !only) v = fma_(alpha, plast[o + kk], v);
        u[o + kk] += to_double(v);
        d[o + kk] += float(v);
      }
    }
  }
}

// LIST as k_cg_dir's (no shared memory: nothing to hand over between tiles).
template <class T, bool LIST = false>
__global__ void __launch_bounds__(kThreads)
    k_ir_update(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                const int* __restrict__ skip, const T* __restrict__ x, double* __restrict__ u,
                float* __restrict__ d, const CgState* __restrict__ st,
                const T* __restrict__ plast, TileList tlist, unsigned long long* work) {
  if constexpr (!LIST) {
    const Tile tile = tiles[blockIdx.x];  // static: read before the wait
    prefetch_l1(G + tile.geom);
    grid_dep_sync();
    irupd_tile<T>(G, tile, skip, x, u, d, st, plast, work);
  } else {
    grid_dep_sync();
    const int n = *tlist.count;
    for (int w = blockIdx.x; w < n; w += gridDim.x)
      irupd_tile<T>(G, tiles[tlist.idx[w]], skip, x, u, d, st, plast, work);
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
                       int* __restrict__ cg_skip, const int* __restrict__ frozen) {
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps) return;
  if (frozen[t]) {  // inactive trap: nothing to solve
    ir_done[t] = 1;
    cg_skip[t] = 1;
    return;
  }
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
  s.pend = 0;
  if (!conv) s.sweeps += 1;
  st[t] = s;
}

// After the final check: the convergence outcome and the next extrapolation factor
// gamma = |d_n| / |d_{n-1}| (clamped), from the increments of the last two steps.
// update_gamma is 0 for the extra checks of adaptive sweeps: the factor belongs to
// the step, so a trap's guess never depends on what the other traps needed.
__global__ void k_s_final(int ntraps, const TileRange* __restrict__ range,
                          const double* __restrict__ part, int ntiles, double rtol,
                          CgState* __restrict__ st, int* __restrict__ ir_done,
                          int* __restrict__ fail, int update_gamma) {
  grid_dep_sync();
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
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || cg_skip[t]) return;
  const double rz = trap_sum(part, range[t]);
  CgState s = st[t];
  s.beta = s.it_in_sweep > 0 && s.rz != 0.0 ? rz / s.rz : 0.0;
  s.rz = rz;
  st[t] = s;
}

// After k_cg_dir: alpha = rz / pq.  With `folded` the update x += alpha p, r -= alpha q
// is left to the next iteration's finest-level k_down (or, after the last iteration,
// to k_ir_update): the trap's update is marked pending and the iteration is counted
// here, since k_s_rr then runs one iteration later and not after the last one.
__global__ void k_s_pq(int ntraps, const TileRange* __restrict__ range,
                       const double* __restrict__ part, CgState* __restrict__ st,
                       const int* __restrict__ cg_skip, int folded) {
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || cg_skip[t]) return;
  const double pq = trap_sum(part, range[t]);
  CgState s = st[t];
  s.pq = pq;
  s.alpha = pq != 0.0 ? s.rz / pq : 0.0;
  if (folded) {
    s.pend = 1;
    s.it_in_sweep += 1;
    s.iters += 1;
  }
  st[t] = s;
}

// After the update (k_cg_update, or the finest-level k_down that folds it in: then
// `folded`): inner convergence test |r| <= tol_rel |r0| or |r| <= rtol |b|.
__global__ void k_s_rr(int ntraps, const TileRange* __restrict__ range,
                       const double* __restrict__ part, double tol_rel, double rtol_abs,
                       CgState* __restrict__ st, int* __restrict__ cg_skip, int folded) {
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraps || cg_skip[t]) return;
  CgState s = st[t];
  s.rr = trap_sum(part, range[t]);
  if (folded) {
    s.pend = 0;  // k_down has added alpha p to the correction
  } else {
    s.it_in_sweep += 1;
    s.iters += 1;
  }
  if (s.rr <= tol_rel * tol_rel * s.rr0 || s.rr <= rtol_abs * rtol_abs * s.bb) cg_skip[t] = 1;
  st[t] = s;
}

}  // namespace eqf
