// Batch runtime and C ABI of the GB300 trap field solver.
//
// A batch holds every trap's multigrid hierarchy in flat per-level arrays, the
// tile work lists that let one launch cover all traps, the FP64 field and load,
// and the device-resident per-trap solver state.  One backward-Euler step is a
// fixed launch sequence (refinement sweeps x preconditioned CG iterations x
// V-cycles); converged traps drop out through per-trap skip flags, so the same
// sequence can be captured once as a CUDA graph and replayed every step.
#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <exception>
#include <atomic>
#include <thread>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/eqfield.h"
#include "eqf_cells.cuh"
#include "eqf_common.cuh"
#include "eqf_kernels.cuh"
#include "eqf_refine.cuh"
#include "eqf_bicgstab.cuh"
#include "eqf_fused.cuh"
#include "eqf_rods.cuh"
#include "eqf_walls.cuh"
#include "eqf_balance.cuh"

namespace eqf {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define EQF_CK(call)                                                                       \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      throw ::eqf::Error(e_ == cudaErrorMemoryAllocation ? EQF_ERR_NOMEM : EQF_ERR_CUDA,   \
                         std::string(#call) + ": " + cudaGetErrorString(e_));              \
  } while (0)

#define EQF_LAUNCH_CHECK() EQF_CK(cudaGetLastError())

// The stream that device buffers are allocated and freed on while a batch's call runs
// (its own stream): cudaMallocAsync / cudaFreeAsync from the device's memory pool are
// ordered on that stream alone, where cudaMalloc / cudaFree can wait for the whole
// device, so batches created, grown or destroyed beside running ones (a server's
// cohorts) do not stall them.  Unset (outside any batch call): plain cudaMalloc.
thread_local cudaStream_t tl_alloc_stream = nullptr;
struct AllocStream {
  cudaStream_t prev;
  explicit AllocStream(cudaStream_t s) : prev(tl_alloc_stream) { tl_alloc_stream = s; }
  ~AllocStream() { tl_alloc_stream = prev; }
  AllocStream(const AllocStream&) = delete;
  AllocStream& operator=(const AllocStream&) = delete;
};

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;  // allocated on this stream (stream-ordered free), or plain
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) {
    o.p = nullptr;
    o.n = 0;
    o.s = nullptr;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      s = o.s;
      o.p = nullptr;
      o.n = 0;
      o.s = nullptr;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count == 0) return;
    if (tl_alloc_stream) {
      EQF_CK(cudaMallocAsync(reinterpret_cast<void**>(&p), count * sizeof(T), tl_alloc_stream));
      s = tl_alloc_stream;
    } else {
      EQF_CK(cudaMalloc(&p, count * sizeof(T)));
    }
    n = count;
    // the staged kernels' bulk copies and vector loads rely on 256-byte bases
    if (reinterpret_cast<uintptr_t>(p) & 255) {
      release();
      throw Error(EQF_ERR_CUDA, "device allocation not 256-byte aligned");
    }
  }
  void release() {
    if (p) {
      if (s)
        cudaFreeAsync(p, s);
      else
        cudaFree(p);
    }
    p = nullptr;
    n = 0;
    s = nullptr;
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    EQF_CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
};

// Page-locked host memory, grow-only: asynchronous copies from and to it do not
// synchronise the stream the way pageable copies do.
template <class T>
struct PinnedBuf {
  T* p = nullptr;
  size_t n = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  void grow(size_t count) {
    if (count <= n) return;
    if (p) cudaFreeHost(p);  // (waits for nothing: callers sync before growing)
    p = nullptr;
    n = 0;
    const size_t cap = count + count / 4 + 64;
    EQF_CK(cudaMallocHost(&p, cap * sizeof(T)));
    n = cap;
  }
};

constexpr int kTileNodes = 4096;
constexpr int kMaxLevels = 16;

static inline long long align_up(long long v, long long a) { return (v + a - 1) / a * a; }

// ---------------------------------------------------------------------------
// Spectrum bounds of D^-1 A on a level (host).
static void spectrum_bounds(LevelGeom& g) {
  // Fourier symbol of the uniform-interior stencil
  double smax = 0.0, smin = 1e300;
  const int NS = 48;
  for (int a = 0; a <= NS; ++a) {
    const double tx = M_PI * a / NS;
    for (int b = -NS; b <= NS; ++b) {
      const double ty = M_PI * b / NS;
      const double v =
          (g.cC + 2 * g.cE * cos(tx) + 2 * g.cN * cos(ty) + 2 * g.cD * cos(tx + ty)) / g.cC;
      smax = std::max(smax, v);
      smin = std::min(smin, v);
    }
  }
  // Gershgorin over every distinct row type (edges, corners, near-edge rows)
  double gmax = 0.0;
  const int is[] = {0, 1, 2, g.ny / 2, g.ny - 2, g.ny - 1, g.ny};
  const int js[] = {0, 1, 2, g.nx / 2, g.nx - 2, g.nx - 1, g.nx};
  for (int i : is) {
    if (i < 0 || i > g.ny) continue;
    for (int j : js) {
      if (j < 0 || j > g.nx) continue;
      if (g.walls && is_dirichlet(g, i, j)) continue;
      const Sten<double> s = stencil_general<double>(g, i, j);
      const double r = (std::fabs(s.c) + std::fabs(s.e) + std::fabs(s.w) + std::fabs(s.n) +
                        std::fabs(s.s) + std::fabs(s.ne) + std::fabs(s.sw)) /
                       s.c;
      gmax = std::max(gmax, r);
    }
  }
  if (g.htens) {
    // a varying tensor: the Gershgorin bound over every row (setup-time host loop)
    gmax = 0.0;
    for (int i = 0; i <= g.ny; ++i)
      for (int j = 0; j <= g.nx; ++j) {
        if (g.walls && is_dirichlet(g, i, j)) continue;
        const Sten<double> s = stencil_general<double>(g, i, j);
        gmax = std::max(gmax, (std::fabs(s.c) + std::fabs(s.e) + std::fabs(s.w) +
                               std::fabs(s.n) + std::fabs(s.s) + std::fabs(s.ne) +
                               std::fabs(s.sw)) / s.c);
      }
    g.lam_max = (float)gmax;
    g.lam_min = (float)(1e-3 * gmax);
    return;
  }
  g.lam_max = (float)std::min(gmax, 1.15 * smax);
  g.lam_min = (float)std::max(0.9 * smin, 1e-3 * smax);
}

template <class T>
static Lens<T> make_lens(const LevelGeom& g) {
  Lens<T> L;
  L.hx = (T)g.hx;
  L.hy = (T)g.hy;
  L.hxl = (T)g.hxl;
  L.hyl = (T)g.hyl;
  L.ihx = (T)(1.0 / g.hx);
  L.ihy = (T)(1.0 / g.hy);
  L.ihxl = (T)(1.0 / g.hxl);
  L.ihyl = (T)(1.0 / g.hyl);
  L.alpha = (T)g.alpha;
  L.beta = (T)g.beta;
  L.adv = (T)g.adv;
  for (int w = 0; w < 4; ++w) L.rob[w] = (T)g.rob[w];
  return L;
}

// Chebyshev-Jacobi coefficients of steps 0..15 on [lmin, lam_max] (three-term
// recurrence of the shifted Chebyshev polynomials, rho_s = 1 / (2 sigma - rho_{s-1})).
static void cheb_table(LevelGeom& g, double lmin) {
  const double lmax = g.lam_max;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
  const double sigma = theta / delta;
  g.ch_old[0] = 0.0f;
  g.ch_res[0] = (float)(1.0 / theta);
  double rho_prev = 1.0 / sigma;
  for (int s = 1; s < kMaxChebSteps; ++s) {
    const double rho = 1.0 / (2.0 * sigma - rho_prev);
    g.ch_old[s] = (float)(rho * rho_prev);
    g.ch_res[s] = (float)(2.0 * rho / delta);
    rho_prev = rho;
  }
}

static void interior_constants(LevelGeom& g) {
  g.adv_on = g.adv != 0.0 ? 1 : 0;
  g.ld = make_lens<double>(g);
  g.lf = make_lens<float>(g);
  LevelGeom q = g;
  q.nx = q.ny = 1000;
  q.walls = 0;
  q.adv = 0.0;
  q.adv_on = 0;
  q.tens = q.htens = nullptr;
  q.tensf = nullptr;
  q.coef_f = nullptr;
  q.coef_d = nullptr;
  q.rowc_f = nullptr;
  q.rowc_d = nullptr;
  const Sten<double> s = stencil_general<double>(q, 500, 500);
  g.cC = s.c;
  g.cE = s.e;
  g.cN = s.n;
  g.cD = s.ne;
  g.cCinv = 1.0 / s.c;
  g.fC = (float)s.c;
  g.fE = (float)s.e;
  g.fN = (float)s.n;
  g.fD = (float)s.ne;
  g.fCinv = (float)(1.0 / s.c);
  const Sten<double> m = mass_stencil<double>(q, 500, 500);
  g.mC = m.c;
  g.mE = m.e;
  g.mN = m.n;
  g.mD = m.ne;
}

// Shared-memory bytes of one staged range [ka, kb) (same widening as Stager::add).
static size_t staged_bytes(long long ka, long long kb, int tsize, long long nalloc) {
  const long long V = 16 / tsize;
  const long long a = (ka / V) * V;
  long long b = ((kb + V - 1) / V) * V;
  b = std::min(b, nalloc);
  const long long nb = b > a ? (b - a) * tsize : 0;
  return (size_t)((nb + 15) & ~15ll) + 16;  // + the 16-byte pad Stager leaves after a range
}

// Class tables: the stencil of every (row class, column class) pair of a trap on
// one level, classes {0, 1, interior, n-1, n} (as node_class), evaluated at a
// representative node of each class.  MASS selects the unscaled mass stencil.
template <class T, bool MASS>
static void build_table(const LevelGeom& g, T* out) {
  auto rep = [](int c, int n) { return c < 2 ? c : (c == 2 ? 2 : (c == 3 ? n - 1 : n)); };
  auto cls = [](int i, int n) { return i < 2 ? i : (i > n - 2 ? 4 - (n - i) : 2); };
  for (int ci = 0; ci < 5; ++ci)
    for (int cj = 0; cj < 5; ++cj) {
      T* e = out + (ci * 5 + cj) * kTabStride;
      for (int q = 0; q < kTabStride; ++q) e[q] = T(0);
      const int i = rep(ci, g.ny), j = rep(cj, g.nx);
      if (i < 0 || i > g.ny || j < 0 || j > g.nx || cls(i, g.ny) != ci || cls(j, g.nx) != cj)
        continue;  // class absent on this grid
      const Sten<T> s = MASS ? mass_stencil<T>(g, i, j) : stencil_general<T>(g, i, j);
      e[0] = s.c;
      e[1] = s.e;
      e[2] = s.w;
      e[3] = s.n;
      e[4] = s.s;
      e[5] = s.ne;
      e[6] = s.sw;
      e[7] = MASS ? T(0) : T(1) / s.c;
    }
}

// Shared-memory bytes of a guarded window (same widening as Stager::add_guarded).
static size_t guarded_bytes(long long ka, long long kb, int tsize) {
  const long long V = 16 / tsize;
  const long long wa = ka >= 0 ? (ka / V) * V : -(((-ka) + V - 1) / V) * V;
  const long long wb = ((kb + V - 1) / V) * V;
  return (size_t)(((wb - wa) * tsize + 15) & ~15ll) + 16;  // + pad as in Stager
}

struct Level {
  std::vector<LevelGeom> geom;  // per trap
  std::vector<Tile> tiles;
  std::vector<Tile2> tiles2;  // 2-D tiles of the fused level kernels
  DevBuf<Tile2> dtiles2;
  long long nodes = 0;
  DevBuf<LevelGeom> dgeom;
  DevBuf<Tile> dtiles;
  DevBuf<float> tabf;   // per-trap class tables (kTabPerTrap entries), FP32
  DevBuf<double> tabd;  // same in FP64
  // dynamic shared memory per staged kernel (max over this level's tiles)
  size_t sm_cheb = 0, sm_resid = 0, sm_cgdir = 0, sm_ir = 0;
  size_t sm_irf1 = 0, sm_irf = 0;  // pair-arithmetic refinement residuals (FP32 form)
  size_t sm_down = 0, sm_up = 0;   // fused level kernels (0: not built for this level)
  int ntiles2_cls = 0;  // tiles2[0, ntiles2_cls): class-table traps; the rest general-path
  int ntiles_cls = 0;   // the same split of the row tiles

  size_t sm_restrict = 0;  // restriction into this level (tiles of this level)
  size_t sm_prolong = 0;   // prolongation from the next coarser level (tiles of this level)
  size_t sm_coarse = 0;    // single-CTA coarsest solve (0 = not possible)
  int ntiles() const { return (int)tiles.size(); }
};

constexpr size_t kSmemHeader = 16;              // mbarrier
// CTAs of a listed launch over n tiles (late sweeps: a quarter of the tiles, which the
// CTAs stride over when more are still iterating).
static int listed_grid(int n) { return std::max(1, (n + 3) / 4); }
// Krylov iterations of a refinement sweep added after a step missed rtol (the step's
// own sweeps run opts.max_iters): such a sweep corrects a small residual.
constexpr int kExtraSweepIters = 6;
constexpr int kMaxExtraSweeps = 8;  // added sweeps per step before the step fails

// Adaptive refinement without a host round trip: run once after a graph-captured
// step's check (first = 1) and at the end of each added sweep, it sets the step graph's
// conditional loop to run another sweep while some trap of this step missed rtol and
// fewer than max_extra sweeps have run.  *fail counts failed trap-steps until the host
// reads and clears it; st[0] holds the part of it from earlier steps (a sweep restarts
// the count from there), st[1] the sweeps added in this step.
__global__ void k_sweep_loop(cudaGraphConditionalHandle h, int* fail, int* st, int first,
                             int max_extra) {
  if (first) st[1] = 0;
  const bool again = *fail > st[0] && st[1] < max_extra;
  if (again) {
    *fail = st[0];
    st[1] += 1;
  } else {
    st[0] = *fail;  // this step's remaining failures stay counted
  }
  cudaGraphSetConditional(h, again ? 1u : 0u);
}
constexpr size_t kMaxDynSmem = 200 * 1024;      // per CTA budget for staged kernels

// ---------------------------------------------------------------------------
// Kernel classes for the built-in profiler (CUDA events around each launch and a
// device counter of the nodes each launch actually processed).
enum KClass : int {
  KC_SMOOTH0 = 0,     // finest-level Chebyshev steps that apply the operator
  KC_SMOOTH0_FIRST,   // finest-level first pre-smoothing step (zero start, no operator)
  KC_RESID0,          // finest-level multigrid residual
  KC_RESTRICT0,       // restriction from the finest level (counts coarse nodes)
  KC_PROLONG0,        // prolongation to the finest level
  KC_COARSE,          // every kernel on coarser levels
  KC_CG_DIR,          // p = z + beta p, q = A p
  KC_CG_UPDATE,       // x += alpha p, r -= alpha q
  KC_IR_RESID_FIRST,  // FP64 b = F + M u, r = b - A u
  KC_IR_RESID,        // FP64 r = b - A u
  KC_IR_UPDATE,       // FP64 u += x
  KC_SCALAR,          // per-trap scalar phases
  KC_DOWN0,           // finest level, fused pre-smoothing + residual
  KC_UP0,             // finest level, fused prolongation + post-smoothing
  KC_ROD,             // rod-cell exchange waves (gather, membrane exchange, deposit)
  KC_BALANCE,         // per-step FP64 mass balance (eqf_mass_balance)
  KC_DOWN0_CG,        // finest level, fused pre-smoothing + residual + CG update
  KC_COUNT
};
static_assert(KC_COUNT == EQF_PROF_CLASSES, "profiler class count");

// algorithmic bytes per processed node: (words of the inner type, FP64 bytes)
static void class_bytes(int cls, int tsize, double& per_node) {
  switch (cls) {
    case KC_SMOOTH0: per_node = 5.0 * tsize; break;        // x, d, b in; x', d out
    case KC_SMOOTH0_FIRST: per_node = 3.0 * tsize; break;  // b in; x, d out
    case KC_RESID0: per_node = 3.0 * tsize; break;         // b, x in; t out
    case KC_RESTRICT0: per_node = 5.0 * tsize; break;      // ~4 fine in; 1 coarse out
    case KC_PROLONG0: per_node = 2.25 * tsize; break;      // x in/out; 1/4 coarse in
    case KC_CG_DIR: per_node = 4.0 * tsize; break;         // z, p in; p', q out
    case KC_CG_UPDATE: per_node = 6.0 * tsize; break;      // x, p, r, q in; x, r out
    case KC_IR_RESID_FIRST: per_node = 40.0 + tsize; break;  // F, u, d in; b, u, d, r out
    case KC_IR_RESID: per_node = 16.0 + tsize; break;      // b, u in; r out
    case KC_IR_UPDATE: per_node = 24.0 + tsize; break;     // x, u, d in; u, d out
    case KC_DOWN0: per_node = 3.0 * tsize; break;          // b in; x, t out
    case KC_DOWN0_CG: per_node = 8.0 * tsize; break;       // r, q, x_cg, p in; x, t, r,
                                                           // x_cg out
    case KC_UP0: per_node = 3.25 * tsize; break;           // x, b, 1/4 coarse in; x out
    default: per_node = 0.0;
  }
}

struct Prof {
  bool on = false;
  std::vector<cudaEvent_t> ev;  // pairs
  std::vector<int> cls;
  size_t used = 0;
  bool overflow = false;
  DevBuf<unsigned long long> work;  // one counter per record
};

// A byte range of device memory to zero (4-byte aligned, a multiple of 4 bytes).
struct ZeroRange {
  char* p;
  long long bytes;
};

// Zeroes every listed range, one CTA row (blockIdx.y) per range: a reused slot's
// vectors at every level in one launch instead of a memset each.
__global__ void k_zero_ranges(const ZeroRange* __restrict__ r) {
  const ZeroRange z = r[blockIdx.y];
  const long long n4 = z.bytes >> 2;
  unsigned* w = reinterpret_cast<unsigned*>(z.p);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
       i += (long long)gridDim.x * blockDim.x)
    w[i] = 0u;
}

struct WorkBase {
  virtual ~WorkBase() = default;
  // one refinement sweep of `iters` preconditioned Krylov iterations; `late`: a sweep
  // after the step's second, where few traps are still iterating
  virtual void enqueue_sweep(cudaStream_t s, bool first, int iters, bool late) = 0;
  virtual void enqueue_check(cudaStream_t s, bool update_gamma) = 0;
  // the byte ranges of every work vector over nodes [off, off + n) of level `lev`
  virtual void slot_ranges(int lev, long long off, long long n, std::vector<ZeroRange>& out) = 0;
};

class Batch;

template <class T>
struct Work : WorkBase {
  Batch& B;
  struct Lv {
    DevBuf<T> b, x, y, d, t;
  };
  std::vector<Lv> lv;
  DevBuf<T> xs, p0, p1, q;  // fine CG: correction, directions, A p
  DevBuf<T> r2;             // fine CG: the residual's second buffer (folded update)
  DevBuf<T> rh;             // BiCGSTAB shadow residual (only when BiCGSTAB is used)
  // The previous CG iteration's update, for the finest level's k_down to fold in, and
  // the inner convergence test k_s_rr runs right after it.
  struct Fold {
    CgFold<T> dev;
    double tol_rel, tol_abs;
  };
  explicit Work(Batch& b);
  void enqueue_sweep(cudaStream_t s, bool first, int iters, bool late) override;
  // Late sweeps of the folded CG: the finest level's fused kernels stride over a list
  // of the iterating traps' 2-D tiles (class-table tiles from act_idx[0], general-path
  // tiles from act_idx[ntiles2_cls]; counts in act_cnt[0..1]) with a quarter-size grid,
  // the CG direction and refinement update over one of their row tiles (act_ridx from
  // 0 and ntiles_cls, counts in act_cnt[2..3]).
  DevBuf<int> act_idx, act_cnt, act_ridx;
  bool late_lists = false;
  void enqueue_check(cudaStream_t s, bool update_gamma) override;
  void slot_ranges(int lev, long long off, long long n, std::vector<ZeroRange>& out) override {
    for (DevBuf<T>* v : {&lv[lev].b, &lv[lev].x, &lv[lev].y, &lv[lev].d, &lv[lev].t})
      out.push_back({reinterpret_cast<char*>(v->p + off), n * (long long)sizeof(T)});
    if (lev == 0)
      for (DevBuf<T>* v : {&xs, &p0, &p1, &q, &r2, &rh})
        if (v->p) out.push_back({reinterpret_cast<char*>(v->p + off), n * (long long)sizeof(T)});
  }
  T* vcycle(cudaStream_t s, int lev, bool dot, const T* rhs0 = nullptr,
            const Fold* fold = nullptr);
  void bicgstab(cudaStream_t s, T* r, double tol_rel, double tol_abs, int max_iters);
};

// Executable graphs that are no longer used.  Destroying one that holds a conditional
// node waits for the whole device, so they are kept here and destroyed in groups, a
// wait per kRetiredGraphs batches instead of one each (the last group stays until the
// process ends).
constexpr size_t kRetiredGraphs = 64;
static std::mutex g_retired_mu;
static std::vector<cudaGraphExec_t> g_retired;
static void retire_graph_exec(cudaGraphExec_t gx) {
  std::vector<cudaGraphExec_t> doomed;
  {
    std::lock_guard<std::mutex> lk(g_retired_mu);
    g_retired.push_back(gx);
    if (g_retired.size() >= kRetiredGraphs) doomed.swap(g_retired);
  }
  for (cudaGraphExec_t g : doomed) cudaGraphExecDestroy(g);
}

// f(0) .. f(n - 1) on up to 16 host threads (pure host work: no CUDA calls inside).
// The first exception a worker meets stops the others' remaining items and is
// rethrown on the calling thread.
template <class F>
static void parallel_for(int n, F&& f) {
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nt = std::min(std::min(hw, 16), (n + 3) / 4);
  if (nt <= 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int> next(0);
  std::exception_ptr err;
  std::mutex err_mu;
  auto work = [&] {
    try {
      for (int i; (i = next.fetch_add(1)) < n;) f(i);
    } catch (...) {
      std::lock_guard<std::mutex> lk(err_mu);
      if (!err) err = std::current_exception();
      next.store(n);
    }
  };
  std::vector<std::thread> th;
  th.reserve(nt - 1);
  try {
    for (int w = 1; w < nt; ++w) th.emplace_back(work);
  } catch (...) {  // no more threads: the ones started and this one share the items
  }
  work();  // the calling thread is a worker too
  for (auto& x : th) x.join();
  if (err) std::rethrow_exception(err);
}

class Batch {
 public:
  // Owns the batch's stream.  Declared first, so destroyed last: every buffer's
  // stream-ordered free is queued on the stream before it goes.
  struct StreamOwner {
    cudaStream_t s = nullptr;
    ~StreamOwner() {
      if (s) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
      }
    }
  } stream_owner;
  int ntraps = 0;
  int nlev = 0;
  // the V-cycle below level bottom_lb runs in k_bottom, one CTA per trap (-1: not used)
  int bottom_lb = -1;
  size_t sm_bottom = 0;
  DevBuf<int> bottom_order;  // k_bottom's traps by decreasing size of the first bottom level
  DevBuf<int> coarse_order;  // k_coarse_solve's traps by decreasing coarsest-grid size
  eqf_solver_opts opts{};
  std::vector<eqf_trap_params> params;
  std::vector<Level> L;
  // per level and trap: the nodes reserved for the trap's slot (its grid at creation;
  // eqf_replace_trap puts any grid that fits there), so replacing a trap moves no
  // other trap and reallocates no vector.  Empty until the first build_levels.
  std::vector<std::vector<long long>> slot_span;
  // per trap: its levels' geometry and class tables as last built (offsets aside);
  // build_levels reuses them unless the trap changed since (trap_dirty: replaced, new
  // walls or tensor), so rebuilding after a slot replacement costs the new traps only
  std::vector<char> trap_dirty;
  std::vector<std::vector<LevelGeom>> geom_cache;
  std::vector<std::vector<float>> tabf_cache;   // level-major, kTabPerTrap per level
  std::vector<std::vector<double>> tabd_cache;
  std::vector<std::vector<double>> tabm_cache;  // finest-level mass table
  std::vector<TileRange> range;  // fine tiles per trap
  DevBuf<TileRange> drange;
  DevBuf<TileRange> drange2;     // fine 2-D tiles per trap (partials of the fused kernels)
  bool fused0 = false;           // the finest level runs the fused level kernels
  DevBuf<CgState> dstate;
  DevBuf<int> d_ir_done, d_cg_skip, d_fail;
  DevBuf<int> d_frozen;  // per trap: nonzero = inactive (skipped by every kernel of a step)
  DevBuf<double> dpart;
  DevBuf<double> U[2];  // fine FP64 field; a step reads U[cur] and writes U[1 - cur]
  DevBuf<float> Dd[2];  // step increments (previous / current), for the initial guess
  int cur = 0;
  DevBuf<double> b64, F;  // refinement rhs, load
  DevBuf<double> tabM0;         // finest-level FP64 mass table
  DevBuf<float2> tabA2, tabM2;  // finest-level operator / mass tables as float pairs
  double* u_cur() { return U[cur].p; }
  std::unique_ptr<WorkBase> work;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one per step parity
  std::string err;
  long long steps_done = 0;
  Prof prof;
  int cur_cls = -1;
  int num_sms = 1;
  bool use_bicgstab = false;  // nonsymmetric operator (advection) or requested

  // profiling hooks: begin() returns the node counter of this launch (or null)
  unsigned long long* prof_begin(int c) {
    if (!prof.on) return nullptr;
    if (prof.used >= prof.cls.size()) {
      prof.overflow = true;
      cur_cls = -1;
      return nullptr;
    }
    cur_cls = c;
    EQF_CK(cudaEventRecord(prof.ev[2 * prof.used], stream));
    return prof.work.p + prof.used;
  }
  void prof_end() {
    if (!prof.on || cur_cls < 0) return;
    EQF_CK(cudaEventRecord(prof.ev[2 * prof.used + 1], stream));
    prof.cls[prof.used] = cur_cls;
    ++prof.used;
    cur_cls = -1;
  }

  // cells
  std::vector<std::vector<double>> cell_xy, cell_s;  // per trap (host copies)
  bool cells_dirty = false;
  // d_cell_s holds rates the host copies lack (eqf_set_cell_rates_all leaves the host
  // copies to pull_cell_s, so the per-step rate upload costs no host-side copy)
  bool cell_s_stale = false;
  int ncells = 0, nseg = 0;
  DevBuf<CellGeom> dcg;
  DevBuf<int> d_cell_trap, d_ent_node, d_perm, d_seg_start;
  DevBuf<double> d_cell_xy, d_cell_s, d_ent_w, d_ent_val, d_scale, d_cells_out;
  std::vector<int> cell_first;  // first cell index of each trap in the batch arrays
  // two-species couplings (species 1 on t1, species 2 on t2, same cells)
  struct Coupling {
    int t1, t2;
    CouplingLaw law;
    std::vector<int> sender;
  };
  std::vector<Coupling> couplings;
  int ncp = 0;  // coupled cells over all couplings
  DevBuf<int> d_cp_i1, d_cp_i2, d_cp_sender, d_cp_law;
  DevBuf<double> d_cp_prod, d_cp_c;
  DevBuf<CouplingLaw> d_cp_laws;
  void enqueue_coupling();
  // rod cells of the agent-based model (eqf_set_rods), one set per simulation
  struct RodSet {
    std::vector<int> layers;
    eqf_rod_law law{};
    RodLawDev dev{};
    int n = 0, nent = 0, waves = 0, grid = 0;
    int relax_passes = 0;  // passes the last wave relaxation took (0: no shared node)
    long long span = 0;  // lattice nodes of the layers' trap in device layout
    DevBuf<eqf_rod> rods;
    DevBuf<RodLawDev> dlaw;
    DevBuf<int> fp_off, fp_node, ent_cell, wave_cells, wave_off;
    DevBuf<int> cover, start, cursor, flag;  // wave analysis scratch
    // more scratch, kept between analyses (grow-only: a cudaFree would synchronise)
    DevBuf<int> sc_count, sc_perm, sc_pred, sc_succ, sc_wave, sc_wcount, sc_wstart;
    DevBuf<int4> winfo;     // wave order: (cell, footprint offset, size)
    DevBuf<double> cellk;   // per cell: volume constants
    DevBuf<double> ihsl, prod, ehsl;
    DevBuf<unsigned char> mode;
  };
  // wall conditions (eqf_set_boundaries) and the flow channels
  std::vector<eqf_boundaries> bcs;  // per trap
  bool walls_active = false;        // some trap carries wall values, Robin loads or channels
  std::vector<WallDev> hwalls;
  DevBuf<WallDev> d_walls;
  DevBuf<double> d_fbase;  // F of the point cells on the wall traps' rims
  int rim_max = 0;
  struct Chan {
    int trap = 0, n = 0, levels = 0;
    DevBuf<double> k1, k2, bfin, bl, bd, bu, c[2];
  };
  std::vector<std::unique_ptr<Chan>> chans;
  DevBuf<ChanDev> d_chans;
  int chan_n_max = 0;
  void setup_walls();
  DevBuf<int> d_wall_of;  // per trap: its index in d_walls, -1 for none
  // per-step FP64 mass balance (eqf_mass_balance): per trap record, tile partials
  bool bal_on = false;
  // the last balance's mass (of the field the next step starts from) and load still
  // hold: the next balance carries them over instead of summing c and F again
  bool bal_prev_ok = false, bal_load_ok = false;
  DevBuf<double> d_bal, bal_part, bal_rpart;
  void enqueue_balance();
  bool ops_dirty = false;  // walls or tensors changed: operators rebuilt before the next use
  void ensure_ops() {
    if (!ops_dirty) return;
    ops_dirty = false;
    build_levels();
    setup_walls();
    grow(dpart, 3 * std::max((size_t)L[0].ntiles(), L[0].tiles2.size()));
  }
  void trap_levels_geom(int t, std::vector<LevelGeom>& out,
                        std::vector<std::vector<double>>& rows) const;
  void check_replacement(int t, const eqf_trap_params& p) const;
  void replace_trap(int t, const eqf_trap_params& p);  // after zero_ranges(slot_ranges(t))
  void slot_ranges(int t, std::vector<ZeroRange>& out);
  void zero_ranges(const std::vector<ZeroRange>& r);
  PinnedBuf<ZeroRange> zero_stage;
  DevBuf<ZeroRange> d_zero;
  void enqueue_walls();
  void enqueue_channels();
  // anisotropic tensors (eqf_set_tensor): per trap the caller's D11, D22, D12 in grid
  // order (empty: isotropic), and per trap and level the pitched copy the stencil reads
  std::vector<std::vector<double>> tensor;
  std::map<std::pair<int, int>, std::vector<double>> htens;
  std::map<std::pair<int, int>, DevBuf<double>> dtens;
  std::map<std::pair<int, int>, DevBuf<float>> dtensf;
  std::map<std::pair<int, int>, DevBuf<float>> dcoef_f;
  std::map<std::pair<int, int>, DevBuf<double>> dcoef_d;
  // per (level, trap) of an advective trap: its rows' stencils (LevelGeom::rowc_*)
  std::map<std::pair<int, int>, DevBuf<float>> drowc_f;
  std::map<std::pair<int, int>, DevBuf<double>> drowc_d;
  void level_tensor(LevelGeom& g, int level, int t);
  // boundary wells (eqf_set_well)
  struct WellParams {
    double scale = 0.0, decay = 0.0;
  };
  std::vector<WellParams> well;
  DevBuf<double> d_well_c;
  DevBuf<long long> d_well_under;
  std::vector<WellDev> hwells;
  DevBuf<WellDev> d_wells;
  void setup_wells();
  void enqueue_wells();
  std::vector<std::unique_ptr<RodSet>> rod_sets;
  DevBuf<RodSetDev> d_rod_sets;        // one descriptor per set (blockIdx.y of a wave)
  int rod_launches = 0, rod_grid = 0;  // wave launches and blocks per set, as captured
  RodSet* rod_set_of(int layer0);
  void rod_analyse(RodSet& rs);
  // footprints and waves of several sets, phase by phase over all of them (one host
  // round trip per phase for the lot)
  void rod_analyse_sets(const std::vector<RodSet*>& sets);
  PinnedBuf<int> rod_hflags;  // per set: footprint size, shared flag, highest wave, unsettled
  PinnedBuf<int> rod_hwoff;   // per set: wave offsets
  PinnedBuf<unsigned char> rod_hstage;  // rods / production / readbacks of the batch calls
  void rod_publish();
  void enqueue_rods();
  // Marks the captured steps out of date: the next step of each parity recaptures it
  // (updating a plain graph in place; the old executable graph of a conditional loop
  // goes to the retired list, as destroying it would wait for the whole device).
  bool graph_stale[2] = {false, false};
  void drop_graphs() { graph_stale[0] = graph_stale[1] = true; }

  Batch(int n, const eqf_trap_params* p, const eqf_solver_opts& o, const int* tiles = nullptr,
        const int* cols = nullptr);
  std::vector<int> tile_target;  // per trap (0: opts.tile_nodes / the default)
  std::vector<int> tile_width;   // per trap 2-D tile columns (0: opts.tile_cols / 128)
  ~Batch();
  void build_levels();
  void step(int n);
  void run_step();
  // one step as a CUDA graph; with opts.adaptive the added refinement sweeps are a
  // conditional loop node inside it (no host round trip per step)
  void capture_step(cudaGraphExec_t& gx, bool device_loop);
  bool device_loop_ok = true;  // conditional graph nodes available (else the host loop)
  bool cond_failed = false;    // the last capture failed in a conditional-node call
  DevBuf<int> d_loop;          // k_sweep_loop's state: earlier failures, added sweeps
  void reset_fail() {
    EQF_CK(cudaMemsetAsync(d_fail.p, 0, sizeof(int), stream));
    if (d_loop.n) EQF_CK(cudaMemsetAsync(d_loop.p, 0, 2 * sizeof(int), stream));
  }
  void rebuild_cells();
  void pull_cell_s();
  void refresh_load();
  void build_segments(int nent, int* d_node, int* d_counts, DevBuf<int>& perm,
                      DevBuf<int>& seg_start, int& nseg_out, const double* xy, const double* s,
                      const double* val);
  // nodes of a trap (the caller's compact grid order, nx+1 per row) ...
  long long fine_nodes(int t) const {
    return (long long)(L[0].geom[t].nx + 1) * (L[0].geom[t].ny + 1);
  }
  // ... and the device span of its rows (pitch P per row)
  long long fine_span(int t) const { return (long long)L[0].geom[t].P * (L[0].geom[t].ny + 1); }
  // compact host grid <-> pitched device rows
  void copy_field_to_device(double* dst, const double* src, int t, cudaStream_t s) const {
    const LevelGeom& g = L[0].geom[t];
    EQF_CK(cudaMemcpy2DAsync(dst, g.P * sizeof(double), src, (g.nx + 1) * sizeof(double),
                             (g.nx + 1) * sizeof(double), g.ny + 1, cudaMemcpyHostToDevice, s));
  }
  void copy_field_to_host(double* dst, const double* src, int t, cudaStream_t s) const {
    const LevelGeom& g = L[0].geom[t];
    EQF_CK(cudaMemcpy2DAsync(dst, (g.nx + 1) * sizeof(double), src, g.P * sizeof(double),
                             (g.nx + 1) * sizeof(double), g.ny + 1, cudaMemcpyDeviceToHost, s));
  }
  void sync() { EQF_CK(cudaStreamSynchronize(stream)); }
  void check_fail();
  void scan(int n, const int* in, int* out);
  DevBuf<int> scan_sums;  // scan's block sums (grow-only)
  template <class U>
  static void grow(DevBuf<U>& b, size_t n) {
    if (b.n < n) b.alloc(n + n / 4 + 64);
  }
};

// ---------------------------------------------------------------------------
Batch::Batch(int n, const eqf_trap_params* p, const eqf_solver_opts& o, const int* tiles,
             const int* cols)
    : ntraps(n), opts(o), params(p, p + n) {
  if (tiles) tile_target.assign(tiles, tiles + n);
  if (cols) tile_width.assign(cols, cols + n);
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    throw Error(EQF_ERR_NO_DEVICE, "no CUDA device visible");
  EQF_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  stream_owner.s = stream;
  AllocStream scope(stream);
  {
    int dev = 0;
    EQF_CK(cudaGetDevice(&dev));
    EQF_CK(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
  }
  tensor.resize(ntraps);
  bcs.resize(ntraps);
  for (int t = 0; t < ntraps; ++t) {
    eqf_boundaries& bc = bcs[t];
    std::memset(&bc, 0, sizeof(bc));
    const unsigned bits[4] = {WALL_BOTTOM, WALL_TOP, WALL_LEFT, WALL_RIGHT};
    for (int w = 0; w < 4; ++w)
      bc.wall[w].kind = (params[t].walls & bits[w]) ? EQF_BC_DIRICHLET : EQF_BC_NEUMANN;
    bc.channel_substeps = 1;
    bc.well_scaling = 1.0;
  }
  build_levels();
  bool adv = false;
  for (const auto& p : params) adv = adv || (p.adv_u != 0.0 && p.adv_len > 0.0);
  use_bicgstab = opts.krylov == EQF_KRYLOV_BICGSTAB || (opts.krylov == EQF_KRYLOV_AUTO && adv);
  const long long N0 = L[0].nodes;
  for (int q = 0; q < 2; ++q) {
    U[q].alloc(N0);
    Dd[q].alloc(N0);
    EQF_CK(cudaMemsetAsync(U[q].p, 0, N0 * sizeof(double), stream));
    EQF_CK(cudaMemsetAsync(Dd[q].p, 0, N0 * sizeof(float), stream));
  }
  b64.alloc(N0);
  F.alloc(N0);
  EQF_CK(cudaMemsetAsync(F.p, 0, N0 * sizeof(double), stream));
  EQF_CK(cudaMemsetAsync(b64.p, 0, N0 * sizeof(double), stream));
  dstate.alloc(ntraps);
  EQF_CK(cudaMemsetAsync(dstate.p, 0, ntraps * sizeof(CgState), stream));
  d_ir_done.alloc(ntraps);
  d_frozen.alloc(ntraps);
  EQF_CK(cudaMemsetAsync(d_frozen.p, 0, ntraps * sizeof(int), stream));
  d_cg_skip.alloc(ntraps);
  d_fail.alloc(1);
  EQF_CK(cudaMemsetAsync(d_fail.p, 0, sizeof(int), stream));
  dpart.alloc(3 * std::max((size_t)L[0].ntiles(), L[0].tiles2.size()));
  if (opts.precision == EQF_PREC_FP32_IR)
    work.reset(new Work<float>(*this));
  else
    work.reset(new Work<double>(*this));
  cell_xy.resize(ntraps);
  cell_s.resize(ntraps);
  well.resize(ntraps);
  d_well_c.alloc(ntraps);
  d_well_under.alloc(ntraps);
  EQF_CK(cudaMemsetAsync(d_well_c.p, 0, ntraps * sizeof(double), stream));
  EQF_CK(cudaMemsetAsync(d_well_under.p, 0, ntraps * sizeof(long long), stream));
  d_wall_of.alloc(ntraps);
  {
    const std::vector<int> none(ntraps, -1);
    d_wall_of.upload(none.data(), ntraps, stream);
  }
  sync();
}

Batch::~Batch() {
  for (auto& gx : graph)
    if (gx) retire_graph_exec(gx);
  for (auto& e : prof.ev) cudaEventDestroy(e);
  work.reset();  // (the stream goes with stream_owner, after the members' frees)
}

// Multigrid levels a trap needs: coarsen until the Fourier number beta/h^2 drops to
// 4 or below (a batch uses the maximum over its traps).  There the coarsest solve's
// Chebyshev steps on [lmin, lmax] (16 in the FP32 form) already damp every mode; a
// criterion of 1 added a level whose launches cost more than it saved (measured on 512
// uneven traps: 16.79 -> 16.02 ms per step; a criterion of 16, two levels fewer, gave
// 16.20 ms with more iterations).
static int trap_levels(const eqf_trap_params& p) {
  const double hmin = std::min(p.width / p.nx, p.height / p.ny);
  const double beta = p.dt * p.D;
  int k = 0;
  double h = hmin;
  while (beta / (h * h) > 4.0 && k < kMaxLevels - 1) {
    h *= 2;
    ++k;
  }
  return k + 1;
}

}  // namespace eqf

// Multigrid depth of a trap (host helper shared with the serving loop).
int eqf_internal_trap_levels(const eqf_trap_params& p) { return eqf::trap_levels(p); }

// Nodes a trap's grid spans at each of nlev levels (rows x pitch, as build_levels lays
// them out): a trap fits a slot when it spans no more at any level.
void eqf_internal_trap_spans(const eqf_trap_params& p, int nlev, long long* spans) {
  int nx = p.nx, ny = p.ny;
  for (int l = 0; l < nlev; ++l) {
    if (l > 0) {  // build_levels' coarsening: halve an axis while it has >= 4 cells
      if (nx >= 4) nx = (nx + 1) / 2;
      if (ny >= 4) ny = (ny + 1) / 2;
    }
    spans[l] = (long long)((nx + 1 + 3) & ~3) * (ny + 1);
  }
}

namespace eqf {

// Device bytes of a batch (steady state plus the transient of the cell rebuild),
// from the same level shapes and buffers as the construction below.
static size_t estimate_bytes(int n, const eqf_trap_params* traps, const eqf_solver_opts& o,
                             long long ncells) {
  int nlev = 1;
  for (int t = 0; t < n; ++t) nlev = std::max(nlev, trap_levels(traps[t]));
  const double T = o.precision == EQF_PREC_FP32_IR ? 4.0 : 8.0;
  double n0 = 0, nall = 0;
  for (int t = 0; t < n; ++t) {
    long long nx = traps[t].nx, ny = traps[t].ny;
    for (int l = 0; l < nlev; ++l) {
      if (l > 0) {
        if (nx >= 4) nx = (nx + 1) / 2;
        if (ny >= 4) ny = (ny + 1) / 2;
      }
      const double nn = (double)((((nx + 1 + 3) & ~3ll) * (ny + 1) + 31) / 32 * 32);
      if (l == 0) n0 += nn;
      nall += nn;
    }
  }
  double bytes = 40.0 * n0                    // U[2], Dd[2], rhs, load
                 + T * (4 + 1) * n0            // Krylov vectors (CG: second residual;
                                               // BiCGSTAB: shadow residual)
                 + 5.0 * T * nall               // multigrid level vectors
                 + 12.0 * n0                    // cell rebuild transient (counts, scans)
                 + 140.0 * (double)ncells       // cell arrays, entries, segments, readout
                 + 64.0 * 1024;
  return (size_t)bytes;
}

// The tensor of trap t on `level` (pitched, D11 | D22 | D12): the caller's fields on
// the finest level, injection from the finer level below (coarse node (I, J) is fine
// node (2I, 2J), clamped to the last node, on coarsened axes).
void Batch::level_tensor(LevelGeom& g, int level, int t) {
  const long long st = (long long)g.P * (g.ny + 1);
  std::vector<double>& h = htens[{level, t}];
  h.assign(3 * st, 0.0);
  if (level == 0) {
    const std::vector<double>& src = tensor[t];
    const long long n = (long long)(g.nx + 1) * (g.ny + 1);
    for (int c = 0; c < 3; ++c)
      for (int i = 0; i <= g.ny; ++i)
        for (int j = 0; j <= g.nx; ++j)
          h[c * st + (long long)i * g.P + j] = src[c * n + (long long)i * (g.nx + 1) + j];
  } else {
    const std::vector<double>& f = htens[{level - 1, t}];
    const int fnx = g.fine_nx, fny = g.fine_ny, fP = (fnx + 1 + 3) & ~3;
    const long long fst = (long long)fP * (fny + 1);
    for (int c = 0; c < 3; ++c)
      for (int i = 0; i <= g.ny; ++i)
        for (int j = 0; j <= g.nx; ++j) {
          const int fi = g.cy ? std::min(2 * i, fny) : i, fj = g.cx ? std::min(2 * j, fnx) : j;
          h[c * st + (long long)i * g.P + j] = f[c * fst + (long long)fi * fP + fj];
        }
  }
  DevBuf<double>& d = dtens[{level, t}];
  d.alloc(h.size());
  d.upload(h.data(), h.size(), stream);
  std::vector<float> hf(h.begin(), h.end());
  DevBuf<float>& df = dtensf[{level, t}];
  df.alloc(hf.size());
  df.upload(hf.data(), hf.size(), stream);
  sync();  // hf is released on return
  g.htens = h.data();
  g.tens = d.p;
  g.tensf = df.p;
  g.tstride = st;
}

// Trap t's geometry at every level (sizes, spacings, constants, spectrum bounds and
// Chebyshev tables), and for an advective trap the FP64 stencils of each level's rows
// (rows[l]: (ny + 1) x 5 column classes x 8); no device work.  A trap with a tensor
// gets its isotropic levels here; build_levels adds the tensor.
void Batch::trap_levels_geom(int t, std::vector<LevelGeom>& out,
                             std::vector<std::vector<double>>& rows) const {
  out.assign(nlev, LevelGeom{});
  rows.assign(nlev, {});
  const auto& p = params[t];
  LevelGeom g{};
  g.nx = p.nx;
  g.ny = p.ny;
  g.trap = t;
  g.walls = p.walls;
  g.hx = g.hxl = p.width / p.nx;
  g.hy = g.hyl = p.height / p.ny;
  g.alpha = 1.0 + p.dt * p.decay;
  g.beta = p.dt * p.D;
  g.adv = (p.adv_u != 0.0 && p.adv_len > 0.0) ? p.dt * p.adv_u / p.adv_len : 0.0;
  const eqf_boundaries& bc = bcs[t];
  for (int w = 0; w < 4; ++w)
    g.rob[w] = bc.wall[w].kind == EQF_BC_ROBIN ? p.dt * bc.wall[w].rate : 0.0;
  for (int w = 0; w < 4; ++w)
    g.dvals = g.dvals || bc.wall[w].kind == EQF_BC_CHANNEL || bc.wall[w].kind == EQF_BC_WELL ||
              (bc.wall[w].kind == EQF_BC_DIRICHLET && bc.wall[w].value != 0.0);
  const bool aniso = !tensor[t].empty();
  for (int l = 0; l < nlev; ++l) {
    if (l > 0) {
      LevelGeom c = g;
      c.dvals = 0;  // coarse levels carry corrections: homogeneous walls
      c.fine_nx = g.nx;
      c.fine_ny = g.ny;
      c.cx = g.nx >= 4;
      c.cy = g.ny >= 4;
      if (c.cx) {
        c.nx = (g.nx + 1) / 2;
        c.hxl = (g.nx % 2 == 0) ? g.hx + g.hxl : g.hxl;
        c.hx = 2 * g.hx;
      }
      if (c.cy) {
        c.ny = (g.ny + 1) / 2;
        c.hyl = (g.ny % 2 == 0) ? g.hy + g.hyl : g.hyl;
        c.hy = 2 * g.hy;
      }
      g = c;
    }
    g.P = (g.nx + 1 + 3) & ~3;
    g.inv_pitch = 1.0f / (float)g.P;
    g.tens = g.htens = nullptr;
    g.tensf = nullptr;
    g.tstride = 0;
    g.coef_f = nullptr;
    g.coef_d = nullptr;
    g.rowc_f = nullptr;
    g.rowc_d = nullptr;
    interior_constants(g);
    if (aniso) {
      out[l] = g;  // the tensor, its stencils and bounds come in build_levels
      continue;
    }
    if (g.adv_on) {
      // advection: the stencil depends on the row (v_y(y)) and the column class only
      std::vector<double>& rd = rows[l];
      rd.assign((size_t)(g.ny + 1) * 5 * 8, 0.0);
      for (int i = 0; i <= g.ny; ++i)
        for (int c = 0; c < 5; ++c) {
          const int j = edge_rep(c, g.nx);
          if (j < 0 || j > g.nx || edge_class(j, g.nx) != c) continue;  // absent class
          const Sten<double> sd = stencil_general<double>(g, i, j);
          const double v[8] = {sd.c, sd.e, sd.w, sd.n, sd.s, sd.ne, sd.sw, 1.0 / sd.c};
          for (int q = 0; q < 8; ++q) rd[((size_t)i * 5 + c) * 8 + q] = v[q];
        }
    }
    spectrum_bounds(g);
    cheb_table(g, l == nlev - 1 ? (double)g.lam_min : (double)g.lam_max / opts.cheb_ratio);
    out[l] = g;
  }
}

void Batch::build_levels() {
  L.clear();
  int nl = 1;
  for (const auto& p : params) nl = std::max(nl, trap_levels(p));
  if (!slot_span.empty()) nl = (int)slot_span.size();  // the depth is fixed at creation
  nlev = nl;
  L.resize(nlev);
  for (int l = 0; l < nlev; ++l) L[l].geom.resize(ntraps);
  if ((int)trap_dirty.size() != ntraps) trap_dirty.assign(ntraps, 1);
  geom_cache.resize(ntraps);
  tabf_cache.resize(ntraps);
  tabd_cache.resize(ntraps);
  tabm_cache.resize(ntraps);
  auto cached = [&](int t) { return !trap_dirty[t] && (int)geom_cache[t].size() == nlev; };
  // the levels of every changed trap without a tensor: pure host work, on all host
  // threads (a slot replacement's traps, or a new batch's); their row tables' uploads
  // and the tensor traps (device work per level) follow in order
  std::vector<int> todo;
  for (int t = 0; t < ntraps; ++t)
    if (!cached(t) && tensor[t].empty()) todo.push_back(t);
  std::vector<std::vector<LevelGeom>> made(todo.size());
  std::vector<std::vector<std::vector<double>>> rows(todo.size());
  parallel_for((int)todo.size(), [&](int k) {
    trap_levels_geom(todo[k], made[k], rows[k]);
  });
  for (size_t k = 0; k < todo.size(); ++k) {
    const int t = todo[k];
    for (int l = 0; l < nlev; ++l) {
      LevelGeom& g = made[k][l];
      if (!rows[k][l].empty()) {  // advective: the rows' stencils, FP64 and rounded
        const std::vector<double>& rd = rows[k][l];
        const std::vector<float> rf(rd.begin(), rd.end());
        DevBuf<float>& bf = drowc_f[{l, t}];
        DevBuf<double>& bd = drowc_d[{l, t}];
        bf.alloc(rf.size());
        bf.upload(rf.data(), rf.size(), stream);
        bd.alloc(rd.size());
        bd.upload(rd.data(), rd.size(), stream);
        g.rowc_f = bf.p;
        g.rowc_d = bd.p;
      }
      L[l].geom[t] = g;
    }
  }
  for (int t = 0; t < ntraps; ++t) {
    if (cached(t)) {  // unchanged since the last build: its levels as built then
      for (int l = 0; l < nlev; ++l) L[l].geom[t] = geom_cache[t][l];
      continue;
    }
    if (!tensor[t].empty()) {  // an anisotropic trap: per-node stencils built on the device
      std::vector<LevelGeom> gl;
      std::vector<std::vector<double>> unused;
      trap_levels_geom(t, gl, unused);
      for (int l = 0; l < nlev; ++l) {
        LevelGeom& g = gl[l];
        level_tensor(g, l, t);
        g.adv_on = 1;  // per-node stencils: every kernel takes the general path
        const long long n = (long long)g.P * (g.ny + 1);
        DevBuf<float>& cf = dcoef_f[{l, t}];
        DevBuf<double>& cd = dcoef_d[{l, t}];
        cf.alloc(8 * n);
        cd.alloc(8 * n);
        k_aniso_coefs<<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, stream>>>(
            g, cf.p, cd.p);
        EQF_LAUNCH_CHECK();
        g.coef_f = cf.p;
        g.coef_d = cd.p;
        spectrum_bounds(g);  // with the tensor: every row
        cheb_table(g, l == nlev - 1 ? (double)g.lam_min : (double)g.lam_max / opts.cheb_ratio);
        L[l].geom[t] = g;
      }
    }
    geom_cache[t].resize(nlev);
    for (int l = 0; l < nlev; ++l) geom_cache[t][l] = L[l].geom[t];
    tabf_cache[t].clear();  // the tables follow below
    tabd_cache[t].clear();
    tabm_cache[t].clear();
  }
  // the class tables of the changed traps, every level, on all host threads
  std::vector<int> untabled;
  for (int t = 0; t < ntraps; ++t)
    if (tabf_cache[t].size() != (size_t)nlev * kTabPerTrap || tabm_cache[t].empty())
      untabled.push_back(t);
  parallel_for((int)untabled.size(), [&](int k) {  // each trap fills its own caches
    const int t = untabled[k];
    tabf_cache[t].assign((size_t)nlev * kTabPerTrap, 0.0f);
    tabd_cache[t].assign((size_t)nlev * kTabPerTrap, 0.0);
    tabm_cache[t].assign(kTabPerTrap, 0.0);
    for (int l = 0; l < nlev; ++l) {
      build_table<float, false>(L[l].geom[t], tabf_cache[t].data() + (size_t)l * kTabPerTrap);
      build_table<double, false>(L[l].geom[t], tabd_cache[t].data() + (size_t)l * kTabPerTrap);
    }
    build_table<double, true>(L[0].geom[t], tabm_cache[t].data());
  });
  // offsets, fine offsets and row tiles (about kTileNodes nodes each, whole rows)
  const int tsz = opts.precision == EQF_PREC_FP32_IR ? 4 : 8;
  const long long target =
      opts.tile_nodes > 0 ? opts.tile_nodes : (tsz == 4 ? kTileNodes : kTileNodes / 2);
  for (int l = 0; l < nlev; ++l) {
    long long off = 0;
    std::vector<Tile> gen1;   // row tiles of general-path traps: after the others
    std::vector<Tile2> gen2;  // 2-D tiles of general-path traps: after the others
    if ((int)slot_span.size() < nlev) slot_span.resize(nlev);
    std::vector<long long>& span = slot_span[l];
    if ((int)span.size() < ntraps) span.resize(ntraps, -1);
    for (int t = 0; t < ntraps; ++t) {
      LevelGeom& g = L[l].geom[t];
      g.off = off;
      const long long P = g.P;
      const long long n = P * (g.ny + 1);
      if (span[t] < 0) span[t] = n;
      if (n > span[t]) throw Error(EQF_ERR_INVALID, "trap grid larger than its slot");
      if (l > 0) {
        g.fine_off = L[l - 1].geom[t].off;
        g.fine_P = L[l - 1].geom[t].P;
      }
      const long long tgt =
          (!tile_target.empty() && tile_target[t] > 0) ? tile_target[t] : target;
      const int R = (int)std::max<long long>(1, tgt / P);
      for (int r0 = 0; r0 <= g.ny; r0 += R) {
        const int r1 = std::min(g.ny + 1, r0 + R);
        (g.adv_on ? gen1 : L[l].tiles).push_back(Tile{t, (int)(r0 * P), (int)(r1 * P), r0, r1});
      }
      // 2-D tiles of the fused kernels: column blocks of at most tile_cols (128) nodes
      const int cw = (!tile_width.empty() && tile_width[t] > 0) ? tile_width[t]
                     : opts.tile_cols > 0                        ? opts.tile_cols
                                                                 : 128;
      const int CW = (int)std::min<long long>(cw, P);
      const int R2 = (int)std::max<long long>(2, tgt / CW);
      for (int r0 = 0; r0 <= g.ny; r0 += R2)
        for (int c0 = 0; c0 < P; c0 += CW)
          (g.adv_on ? gen2 : L[l].tiles2)
              .push_back(Tile2{t, r0, std::min(g.ny + 1, r0 + R2), c0,
                               (int)std::min<long long>(P, c0 + CW)});
      off = align_up(off + span[t], 32);
    }
    if (l > 0) {
      // coarse levels carry no per-tile partials: their tiles go largest first, so the
      // long ones of the largest traps do not start last (level 0 keeps each trap's
      // tiles together, in order, for the partial sums)
      auto big1 = [](const Tile& a, const Tile& b) { return a.k1 - a.k0 > b.k1 - b.k0; };
      auto big2 = [](const Tile2& a, const Tile2& b) {
        return (long long)(a.r1 - a.r0) * (a.c1 - a.c0) > (long long)(b.r1 - b.r0) * (b.c1 - b.c0);
      };
      std::stable_sort(L[l].tiles.begin(), L[l].tiles.end(), big1);
      std::stable_sort(gen1.begin(), gen1.end(), big1);
      std::stable_sort(L[l].tiles2.begin(), L[l].tiles2.end(), big2);
      std::stable_sort(gen2.begin(), gen2.end(), big2);
    }
    L[l].ntiles_cls = (int)L[l].tiles.size();
    L[l].tiles.insert(L[l].tiles.end(), gen1.begin(), gen1.end());
    L[l].ntiles2_cls = (int)L[l].tiles2.size();
    L[l].tiles2.insert(L[l].tiles2.end(), gen2.begin(), gen2.end());
    L[l].nodes = off;
    if (off >= (1ll << 31)) throw Error(EQF_ERR_INVALID, "batch too large for 32-bit node indices");
    L[l].dgeom.alloc(ntraps);
    L[l].dgeom.upload(L[l].geom.data(), ntraps, stream);
    L[l].dtiles.alloc(L[l].tiles.size());
    L[l].dtiles.upload(L[l].tiles.data(), L[l].tiles.size(), stream);
    L[l].dtiles2.alloc(L[l].tiles2.size());
    L[l].dtiles2.upload(L[l].tiles2.data(), L[l].tiles2.size(), stream);
    std::vector<float> tf((size_t)ntraps * kTabPerTrap);
    std::vector<double> td((size_t)ntraps * kTabPerTrap);
    for (int t = 0; t < ntraps; ++t) {
      const size_t o = (size_t)l * kTabPerTrap;
      std::copy(tabf_cache[t].begin() + o, tabf_cache[t].begin() + o + kTabPerTrap,
                tf.data() + (size_t)t * kTabPerTrap);
      std::copy(tabd_cache[t].begin() + o, tabd_cache[t].begin() + o + kTabPerTrap,
                td.data() + (size_t)t * kTabPerTrap);
    }
    L[l].tabf.alloc(tf.size());
    L[l].tabf.upload(tf.data(), tf.size(), stream);
    L[l].tabd.alloc(td.size());
    L[l].tabd.upload(td.data(), td.size(), stream);
    if (l == 0) {
      std::vector<double> tm((size_t)ntraps * kTabPerTrap);
      for (int t = 0; t < ntraps; ++t)
        std::copy(tabm_cache[t].begin(), tabm_cache[t].end(), tm.data() + (size_t)t * kTabPerTrap);
      tabM0.alloc(tm.size());
      tabM0.upload(tm.data(), tm.size(), stream);
      // float pairs (h, l), h + l = the FP64 weight to ~2^-48; the interior class
      // holds the interior weights, as the FP64 kernels use them
      std::vector<float2> a2(tm.size()), m2(tm.size());
      auto pr = [](double v) {
        const float h = (float)v;
        return make_float2(h, (float)(v - (double)h));
      };
      for (int t = 0; t < ntraps; ++t) {
        const LevelGeom& g = L[0].geom[t];
        const size_t o = (size_t)t * kTabPerTrap;
        for (int e = 0; e < kTabPerTrap; ++e) {
          a2[o + e] = pr(td[o + e]);
          m2[o + e] = pr(tm[o + e]);
        }
        const double ia[8] = {g.cC, g.cE, g.cE, g.cN, g.cN, g.cD, g.cD, g.cCinv};
        const double im[8] = {g.mC, g.mE, g.mE, g.mN, g.mN, g.mD, g.mD, 0.0};
        for (int q = 0; q < kTabStride; ++q) {
          a2[o + 12 * kTabStride + q] = pr(ia[q]);
          m2[o + 12 * kTabStride + q] = pr(im[q]);
        }
      }
      tabA2.alloc(a2.size());
      tabA2.upload(a2.data(), a2.size(), stream);
      tabM2.alloc(m2.size());
      tabM2.upload(m2.data(), m2.size(), stream);
    }
    sync();  // host vectors go out of scope
  }
  // dynamic shared memory of the staged kernels
  for (int l = 0; l < nlev; ++l) {
    Level& Lv = L[l];
    for (const Tile& tl : Lv.tiles) {
      const LevelGeom& g = Lv.geom[tl.geom];
      const long long P = g.P, n = P * (g.ny + 1), na = align_up(n, 32);
      (void)n;
      const long long ka = (long long)tl.k0 - P - 1;  // guarded halo window
      const long long kb = (long long)tl.k1 + P + 1;
      // quad kernels: a wider halo (qhalo_lo / qhalo_hi) and the staged class table
      const size_t halo = guarded_bytes((long long)tl.k0 - P - 8, (long long)tl.k1 + P + 8, tsz);
      const size_t own = staged_bytes(tl.k0, tl.k1, tsz, na);
      const size_t tab = (size_t)kTabPerTrap * tsz;
      Lv.sm_cheb = std::max(Lv.sm_cheb, kSmemHeader + halo + 2 * own + tab);
      Lv.sm_resid = std::max(Lv.sm_resid, kSmemHeader + halo + own + tab);
      Lv.sm_cgdir = std::max(Lv.sm_cgdir, kSmemHeader + 2 * halo + tab);

      // first refinement residual: u (FP64, halo), F (FP64), d (FP32, halo)
      const size_t ptab = (size_t)kTabPerTrap * 8;
      Lv.sm_irf1 = std::max(Lv.sm_irf1, kSmemHeader + guarded_bytes(ka, kb, 8) +
                                            guarded_bytes(ka, kb, 4) + 2 * ptab);
      Lv.sm_irf = std::max(Lv.sm_irf, kSmemHeader + guarded_bytes(ka, kb, 8) + ptab);
      Lv.sm_ir = std::max(Lv.sm_ir, kSmemHeader + guarded_bytes(ka, kb, 8) +
                                        staged_bytes(tl.k0, tl.k1, 8, na) +
                                        guarded_bytes(ka, kb, 4) +
                                        (size_t)((kb - ka) * 8 + 15) / 16 * 16);
      if (l > 0) {  // restriction into level l stages fine rows f(r0)-1 .. f(r1-1)+1
        const LevelGeom& f = L[l - 1].geom[tl.geom];
        auto c2f = [](int K, int nf, int h) { return h ? std::min(2 * K, nf) : K; };
        const long long PF = f.P;
        long long fr0 = std::max(0, c2f(tl.r0, f.ny, g.cy) - 1);
        long long fr1 = std::min(f.ny + 1, c2f(tl.r1 - 1, f.ny, g.cy) + 2);
        Lv.sm_restrict = std::max(Lv.sm_restrict,
                                  kSmemHeader + staged_bytes(fr0 * PF, fr1 * PF, tsz,
                                                             align_up(PF * (f.ny + 1), 32)));
      }
      if (l + 1 < nlev) {  // prolongation into level l stages coarse rows lo(r0) .. hi(r1-1)
        const LevelGeom& c = L[l + 1].geom[tl.geom];
        auto f2c_lo = [](int f, int nf, int h) {
          return !h ? f : ((f & 1) == 0 ? f / 2 : (f == nf ? (f + 1) / 2 : (f - 1) / 2));
        };
        auto f2c_hi = [](int f, int nf, int h) {
          return !h ? f : ((f & 1) == 0 ? f / 2 : (f == nf ? (f + 1) / 2 : (f - 1) / 2 + 1));
        };
        const long long PC = c.P;
        const long long lo = f2c_lo(tl.r0, g.ny, c.cy), hi = f2c_hi(tl.r1 - 1, g.ny, c.cy);
        Lv.sm_prolong = std::max(Lv.sm_prolong,
                                 kSmemHeader + staged_bytes(lo * PC, (hi + 1) * PC, tsz,
                                                            align_up(PC * (c.ny + 1), 32)));
      }
    }
    if (l + 1 < nlev) {  // fused level kernels (windows as in k_down / k_up)
      const LevelGeom* gc = L[l + 1].geom.data();
      for (const Tile2& t2 : Lv.tiles2) {
        const LevelGeom& g = Lv.geom[t2.geom];
        const Win w1 = win_grow(t2, 2, 8), w2 = win_grow(t2, 1, 4);
        const Win wc = up_coarse_win(g, gc[t2.geom], w1);
        const size_t tab = (size_t)kTabPerTrap * tsz;
        Lv.sm_down = std::max(Lv.sm_down, kSmemHeader + 2 * win_bytes(w1, tsz) +
                                              win_bytes(w2, tsz) + tab);
        Lv.sm_up = std::max(Lv.sm_up, kSmemHeader + win_bytes(w1, tsz) + 2 * win_bytes(w2, tsz) +
                                          win_bytes(wc, tsz) + tab);
      }
    }
    for (size_t v : {Lv.sm_cheb, Lv.sm_resid, Lv.sm_cgdir, Lv.sm_restrict, Lv.sm_prolong})
      if (v > kMaxDynSmem)
        throw Error(EQF_ERR_INVALID, "trap rows too wide for shared-memory row tiles");
    // the fused level kernels are used where their windows fit (else the unfused steps)
    if (Lv.sm_down > kMaxDynSmem || Lv.sm_up > kMaxDynSmem) Lv.sm_down = Lv.sm_up = 0;
    if (l == 0 && std::max(Lv.sm_ir, Lv.sm_irf1) > kMaxDynSmem)
      throw Error(EQF_ERR_INVALID, "trap rows too wide for shared-memory row tiles");
  }
  {  // single-CTA coarsest solve when every trap's coarsest grid fits
    Level& Lc = L[nlev - 1];
    size_t need = 0;
    for (const LevelGeom& g : Lc.geom) {
      const long long n = (long long)g.P * (g.ny + 1), na = align_up(n, 32);
      const long long gpad = ((g.P + 1 + 7) / 8) * 8;
      need = std::max(need, kSmemHeader + staged_bytes(0, n, tsz, na) +
                                (size_t)(3 * na + 5 * gpad) * tsz);
    }
    Lc.sm_coarse = (nlev > 1 && need <= kMaxDynSmem) ? need : 0;
  }
  // the shallowest bottom level (>= 2) whose levels down to the coarsest fit one CTA's
  // shared memory for every trap (fused level path only: the step-by-step path stays
  // launch by launch)
  bottom_lb = -1;
  sm_bottom = 0;
  if (opts.fuse_levels >= 2 && opts.cheb_pre == 2 && opts.cheb_post == 2 &&
      L[nlev - 1].sm_coarse > 0) {
    for (int lb = std::max(2, nlev - kMaxBottom); lb <= nlev - 2; ++lb) {
      size_t need = 0;
      for (int t = 0; t < ntraps; ++t) {
        size_t b = kSmemHeader + 32;
        for (int l = lb; l < nlev; ++l)
          b += bottom_level_bytes(L[l].geom[t].P, L[l].geom[t].ny, tsz) + 96;
        need = std::max(need, b);
      }
      if (need <= kMaxDynSmem) {
        bottom_lb = lb;
        sm_bottom = need;
        break;
      }
    }
  }
  // one CTA per trap on the bottom and coarsest levels: largest traps first (the
  // launch's tail is the largest CTA's)
  auto by_size = [&](const Level& Lv, DevBuf<int>& out) {
    std::vector<int> ord(ntraps);
    for (int t = 0; t < ntraps; ++t) ord[t] = t;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
      return (long long)Lv.geom[a].P * (Lv.geom[a].ny + 1) >
             (long long)Lv.geom[b].P * (Lv.geom[b].ny + 1);
    });
    out.alloc(ntraps);
    out.upload(ord.data(), ntraps, stream);
  };
  if (bottom_lb >= 0) by_size(L[bottom_lb], bottom_order);
  by_size(L[nlev - 1], coarse_order);
  trap_dirty.assign(ntraps, 0);
  range.assign(ntraps, TileRange{0, 0});
  for (int i = 0; i < L[0].ntiles(); ++i) {
    const int t = L[0].tiles[i].geom;
    if (range[t].count == 0) range[t].first = i;
    range[t].count++;
  }
  drange.alloc(ntraps);
  drange.upload(range.data(), ntraps, stream);
  std::vector<TileRange> range2(ntraps, TileRange{0, 0});
  for (int i = 0; i < (int)L[0].tiles2.size(); ++i) {
    const int t = L[0].tiles2[i].geom;
    if (range2[t].count == 0) range2[t].first = i;
    range2[t].count++;
  }
  drange2.alloc(ntraps);
  drange2.upload(range2.data(), ntraps, stream);
  fused0 = nlev > 1 && opts.fuse_levels && opts.cheb_pre == 2 && opts.cheb_post == 2 &&
           L[0].sm_down > 0;
  sync();
}

// ---------------------------------------------------------------------------
template <class K>
static void smem_attrs(K kernel, int mx) {
  EQF_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
  EQF_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
}

template <class T>
static void allow_dyn_smem() {
  const int mx = (int)kMaxDynSmem;
  smem_attrs(k_cheb<T, true, false, true, false>, mx);
  smem_attrs(k_cheb<T, true, false, false, false>, mx);
  smem_attrs(k_cheb<T, false, false, true, false>, mx);
  smem_attrs(k_cheb<T, false, false, false, false>, mx);
  smem_attrs(k_cheb<T, true, false, true, true>, mx);
  smem_attrs(k_cheb<T, true, false, false, true>, mx);
  smem_attrs(k_cheb<T, false, false, true, true>, mx);
  smem_attrs(k_cheb<T, false, false, false, true>, mx);
  smem_attrs(k_resid<T>, mx);
  smem_attrs(k_restrict<T>, mx);
  smem_attrs(k_prolong<T>, mx);
  smem_attrs(k_coarse_solve<T>, mx);
  smem_attrs(k_cg_dir<T, true, false>, mx);
  smem_attrs(k_cg_dir<T, false, false>, mx);
  smem_attrs(k_cg_dir<T, true, true>, mx);
  smem_attrs(k_cg_dir<T, false, true>, mx);
  smem_attrs(k_cg_dir<T, true, false, true>, mx);
  smem_attrs(k_cg_dir<T, false, false, true>, mx);
  smem_attrs(k_cg_dir<T, true, true, true>, mx);
  smem_attrs(k_cg_dir<T, false, true, true>, mx);
  smem_attrs(k_ir_first<T>, mx);
  smem_attrs(k_ir_residual<T, true>, mx);
  smem_attrs(k_ir_residual<T, false>, mx);
  smem_attrs(k_irf_first, mx);
  smem_attrs(k_down<T, false>, mx);
  smem_attrs(k_down<T, true>, mx);
  smem_attrs(k_down<T, false, true>, mx);
  smem_attrs(k_down<T, true, true>, mx);
  smem_attrs(k_down<T, false, false, true>, mx);
  smem_attrs(k_down<T, true, false, true>, mx);
  smem_attrs(k_down<T, false, true, true>, mx);
  smem_attrs(k_down<T, true, true, true>, mx);
  smem_attrs(k_up<T, true, false, true>, mx);
  smem_attrs(k_up<T, true, true, true>, mx);
  smem_attrs(k_up<T, true, false>, mx);
  smem_attrs(k_up<T, false, false>, mx);
  smem_attrs(k_up<T, true, true>, mx);
  smem_attrs(k_up<T, false, true>, mx);
  smem_attrs(k_apply_dot<T, 1>, mx);
  smem_attrs(k_apply_dot<T, 2>, mx);
  smem_attrs(k_irf_residual<true>, mx);
  smem_attrs(k_irf_residual<false>, mx);
  smem_attrs(k_bottom<T>, mx);
}

template <class T>
Work<T>::Work(Batch& b) : B(b) {
  allow_dyn_smem<T>();
  lv.resize(B.nlev);
  for (int l = 0; l < B.nlev; ++l) {
    const size_t n = B.L[l].nodes;
    lv[l].b.alloc(n);
    lv[l].x.alloc(n);
    lv[l].y.alloc(n);
    lv[l].d.alloc(n);
    lv[l].t.alloc(n);
    // zero once so padding between traps never holds garbage
    for (DevBuf<T>* v : {&lv[l].b, &lv[l].x, &lv[l].y, &lv[l].d, &lv[l].t})
      EQF_CK(cudaMemsetAsync(v->p, 0, n * sizeof(T), B.stream));
  }
  const size_t n0 = B.L[0].nodes;
  for (DevBuf<T>* v : {&xs, &p0, &p1, &q}) {
    v->alloc(n0);
    EQF_CK(cudaMemsetAsync(v->p, 0, n0 * sizeof(T), B.stream));
  }
  if (!B.use_bicgstab) {  // the folded CG update writes the residual here
    // late sweeps' tile lists: allocated here, never in enqueue_sweep, which runs under
    // stream capture (a stream-ordered allocation there becomes a graph memory node)
    act_idx.alloc(std::max<size_t>(1, B.L[0].tiles2.size()));
    act_ridx.alloc(std::max<size_t>(1, (size_t)B.L[0].ntiles()));
    act_cnt.alloc(4);
    r2.alloc(n0);
    EQF_CK(cudaMemsetAsync(r2.p, 0, n0 * sizeof(T), B.stream));
  }
  if (B.use_bicgstab) {
    rh.alloc(n0);
    EQF_CK(cudaMemsetAsync(rh.p, 0, n0 * sizeof(T), B.stream));
  }
}

// Launch wrapper: profiler marks around one kernel launch.
// Launch of a solver kernel with programmatic stream serialization: its CTAs may be
// scheduled while the previous kernel's last CTAs run (each solver kernel starts
// with grid_dep_sync, which holds it until that grid has completed).
template <class... KArgs, class... Args>
static void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  EQF_CK(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
}

#define EQF_RUN(B_, cls_, launch_)                     \
  do {                                                 \
    unsigned long long* W = (B_).prof_begin(cls_);     \
    (void)W;                                           \
    launch_;                                           \
    EQF_LAUNCH_CHECK();                                \
    (B_).prof_end();                                   \
  } while (0)

// One Chebyshev step on a level (template flags chosen at run time).
template <class T>
static void cheb_step(Batch& B, cudaStream_t s, int lev, int nt, const LevelGeom* G,
                      const Tile* tl, const T* tab, const int* skip, int st,
                      bool first, bool zero, bool dot, const T* b, const T* xin, T* xout, T* d,
                      double* part) {
  const int cls = lev > 0 ? KC_COARSE : (zero ? KC_SMOOTH0_FIRST : KC_SMOOTH0);
  const size_t sm = zero ? 0 : B.L[lev].sm_cheb;
  // class-table traps' row tiles, then general-path traps' (part by tile index)
  const int nc = B.L[lev].ntiles_cls, ng = nt - nc;
  auto run = [&](auto kc, auto kg, int step) {
    if (nc > 0)
      EQF_RUN(B, cls, (launch_pdl(kc, nc, kThreads, sm, s, G, tl, tab, skip, step, b, xin, xout,
                                  d, part, W)));
    if (ng > 0)
      EQF_RUN(B, cls, (launch_pdl(kg, ng, kThreads, sm, s, G, tl + nc, tab, skip, step, b, xin,
                                  xout, d, part + nc, W)));
  };
  if (zero) {
    if (dot)
      run(k_cheb<T, true, true, true, false>, k_cheb<T, true, true, true, true>, 0);
    else
      run(k_cheb<T, true, true, false, false>, k_cheb<T, true, true, false, true>, 0);
  } else if (first) {
    if (dot)
      run(k_cheb<T, true, false, true, false>, k_cheb<T, true, false, true, true>, 0);
    else
      run(k_cheb<T, true, false, false, false>, k_cheb<T, true, false, false, true>, 0);
  } else {
    if (dot)
      run(k_cheb<T, false, false, true, false>, k_cheb<T, false, false, true, true>, st);
    else
      run(k_cheb<T, false, false, false, false>, k_cheb<T, false, false, false, true>, st);
  }
}

template <class T>
static const T* level_tab(const Level& L);
template <>
const float* level_tab<float>(const Level& L) {
  return L.tabf.p;
}
template <>
const double* level_tab<double>(const Level& L) {
  return L.tabd.p;
}

// V-cycle on level `lev` with rhs lv[lev].b (rhs0 on level 0 when given); returns
// the buffer holding x.
// With `dot`, the last smoothing step also writes partials of b.x (= r.z on level 0).
template <class T>
T* Work<T>::vcycle(cudaStream_t s, int lev, bool dot, const T* rhs0, const Fold* fold) {
  const Level& Lv_ = B.L[lev];
  Lv& v = lv[lev];
  const T* bl = (lev == 0 && rhs0) ? rhs0 : v.b.p;  // this level's rhs
  const int nt = Lv_.ntiles();
  const int* skip = B.d_cg_skip.p;
  const LevelGeom* G = Lv_.dgeom.p;
  const Tile* tl = Lv_.dtiles.p;
  const T* tab = level_tab<T>(Lv_);
  double* part = B.dpart.p;
  T* cur = v.x.p;
  T* oth = v.y.p;
  const bool coarsest = lev == B.nlev - 1;
  const int deg_pre = coarsest ? B.opts.cheb_coarse : B.opts.cheb_pre;
  if (lev == B.bottom_lb && !dot) {
    // levels lev .. coarsest in one CTA per trap
    BottomArgs<T> a{};
    a.nlev = B.nlev - lev;
    for (int m = 0; m < a.nlev; ++m) {
      a.G[m] = B.L[lev + m].dgeom.p;
      a.tabs[m] = level_tab<T>(B.L[lev + m]);
    }
    a.deg_pre = B.opts.cheb_pre;
    a.deg_coarse = B.opts.cheb_coarse;
    a.order = B.bottom_order.p;
    EQF_RUN(B, KC_COARSE,
            (launch_pdl(k_bottom<T>, B.ntraps, kBottomThreads, B.sm_bottom, s, a, skip, bl, cur)));
    return cur;
  }
  if (coarsest && Lv_.sm_coarse && !dot) {
    // the whole coarsest solve in one CTA per trap
    EQF_RUN(B, KC_COARSE,
            (launch_pdl(k_coarse_solve<T>, B.ntraps, kCoarseThreads, Lv_.sm_coarse, s, G, tab,
                        skip, deg_pre, bl, cur, (const int*)B.coarse_order.p)));
    return cur;
  }
  if (!coarsest && B.opts.fuse_levels && B.opts.cheb_pre == 2 && B.opts.cheb_post == 2 &&
      Lv_.sm_down > 0) {
    // temporally blocked: pre-smoothing + residual, restriction, coarse correction,
    // prolongation + post-smoothing
    // class-table traps' tiles first, general-path traps' tiles after: one kernel each
    const int nc2 = Lv_.ntiles2_cls, ng2 = (int)Lv_.tiles2.size() - nc2;
    const Tile2* tc2 = Lv_.dtiles2.p;
    const Tile2* tg2 = Lv_.dtiles2.p + nc2;
    const int cd = lev > 0 ? KC_COARSE : KC_DOWN0, cu = lev > 0 ? KC_COARSE : KC_UP0;
    const bool listed = lev == 0 && late_lists;
    const TileList lc{act_idx.p, act_cnt.p}, lg{act_idx.p + nc2, act_cnt.p + 1};
    const TileList none{nullptr, nullptr};
    if (lev == 0 && fold) {
      // the previous iteration's x += alpha p, r -= alpha q folded in; the partials
      // of (r, r) go to part[the tile's index in tiles2], the test follows at once
      CgFold<T> fc = fold->dev, fg = fold->dev;
      if (listed) {  // absolute tile indices: both kinds index the whole array
        if (nc2 > 0)
          EQF_RUN(B, KC_DOWN0_CG,
                  (launch_pdl(k_down<T, false, true, true>, listed_grid(nc2), kThreads,
                              Lv_.sm_down, s, G, tc2, tab, skip, bl, cur, v.t.p, fc, lc, W)));
        if (ng2 > 0)
          EQF_RUN(B, KC_DOWN0_CG,
                  (launch_pdl(k_down<T, true, true, true>, listed_grid(ng2), kThreads,
                              Lv_.sm_down, s, G, tc2, tab, skip, bl, cur, v.t.p, fg, lg, W)));
      } else {
        fg.part += nc2;
        if (nc2 > 0)
          EQF_RUN(B, KC_DOWN0_CG,
                  (launch_pdl(k_down<T, false, true>, nc2, kThreads, Lv_.sm_down, s, G, tc2, tab,
                              skip, bl, cur, v.t.p, fc, none, W)));
        if (ng2 > 0)
          EQF_RUN(B, KC_DOWN0_CG,
                  (launch_pdl(k_down<T, true, true>, ng2, kThreads, Lv_.sm_down, s, G, tg2, tab,
                              skip, bl, cur, v.t.p, fg, none, W)));
      }
      const int nb = (B.ntraps + 127) / 128;
      EQF_RUN(B, KC_SCALAR,
              (launch_pdl(k_s_rr, nb, 128, 0, s, B.ntraps, B.drange2.p, fold->dev.part,
                          fold->tol_rel, fold->tol_abs, B.dstate.p, B.d_cg_skip.p, 1)));
      bl = fold->dev.rout;  // the post-smoothing's right-hand side
    } else if (listed) {
      if (nc2 > 0)
        EQF_RUN(B, cd, (launch_pdl(k_down<T, false, false, true>, listed_grid(nc2), kThreads,
                                   Lv_.sm_down, s, G, tc2, tab, skip, bl, cur, v.t.p,
                                   CgFold<T>{}, lc, W)));
      if (ng2 > 0)
        EQF_RUN(B, cd, (launch_pdl(k_down<T, true, false, true>, listed_grid(ng2), kThreads,
                                   Lv_.sm_down, s, G, tc2, tab, skip, bl, cur, v.t.p,
                                   CgFold<T>{}, lg, W)));
    } else {
      if (nc2 > 0)
        EQF_RUN(B, cd, (launch_pdl(k_down<T, false>, nc2, kThreads, Lv_.sm_down, s, G, tc2,
                                   tab, skip, bl, cur, v.t.p, CgFold<T>{}, none, W)));
      if (ng2 > 0)
        EQF_RUN(B, cd, (launch_pdl(k_down<T, true>, ng2, kThreads, Lv_.sm_down, s, G, tg2,
                                   tab, skip, bl, cur, v.t.p, CgFold<T>{}, none, W)));
    }
    const Level& Lc = B.L[lev + 1];
    EQF_RUN(B, lev > 0 ? KC_COARSE : KC_RESTRICT0,
            (launch_pdl(k_restrict<T>, Lc.ntiles(), kThreads, Lc.sm_restrict, s,
                        Lc.dgeom.p, Lc.dtiles.p, skip, v.t.p, lv[lev + 1].b.p, W)));
    T* xc = vcycle(s, lev + 1, false);
    // the dot partials of a tile go to part[its index in tiles2]
    if (dot && listed) {
      if (nc2 > 0)
        EQF_RUN(B, cu, (launch_pdl(k_up<T, true, false, true>, listed_grid(nc2), kThreads,
                                   Lv_.sm_up, s, G, Lc.dgeom.p, tc2, tab, skip, xc, bl, cur,
                                   oth, part, lc, W)));
      if (ng2 > 0)
        EQF_RUN(B, cu, (launch_pdl(k_up<T, true, true, true>, listed_grid(ng2), kThreads,
                                   Lv_.sm_up, s, G, Lc.dgeom.p, tc2, tab, skip, xc, bl, cur,
                                   oth, part, lg, W)));
    } else if (dot) {
      if (nc2 > 0)
        EQF_RUN(B, cu, (launch_pdl(k_up<T, true, false>, nc2, kThreads, Lv_.sm_up, s, G,
                                   Lc.dgeom.p, tc2, tab, skip, xc, bl, cur, oth, part, none,
                                   W)));
      if (ng2 > 0)
        EQF_RUN(B, cu, (launch_pdl(k_up<T, true, true>, ng2, kThreads, Lv_.sm_up, s, G,
                                   Lc.dgeom.p, tg2, tab, skip, xc, bl, cur, oth, part + nc2,
                                   none, W)));
    } else {
      if (nc2 > 0)
        EQF_RUN(B, cu, (launch_pdl(k_up<T, false, false>, nc2, kThreads, Lv_.sm_up, s, G,
                                   Lc.dgeom.p, tc2, tab, skip, xc, bl, cur, oth, part, none,
                                   W)));
      if (ng2 > 0)
        EQF_RUN(B, cu, (launch_pdl(k_up<T, false, true>, ng2, kThreads, Lv_.sm_up, s, G,
                                   Lc.dgeom.p, tg2, tab, skip, xc, bl, cur, oth, part + nc2,
                                   none, W)));
    }
    return oth;
  }
  // pre-smoothing (or the coarsest-level solve) from zero
  cheb_step<T>(B, s, lev, nt, G, tl, tab, skip, 0, true, true,
               dot && coarsest && deg_pre == 1, bl, cur, cur, v.d.p, part);
  for (int st = 1; st < deg_pre; ++st) {
    cheb_step<T>(B, s, lev, nt, G, tl, tab, skip, st, false, false,
                 dot && coarsest && st == deg_pre - 1, bl, cur, oth, v.d.p, part);
    std::swap(cur, oth);
  }
  if (coarsest) return cur;
  // residual, restriction, coarse correction, prolongation
  const int c0 = lev > 0 ? KC_COARSE : KC_RESID0;
  EQF_RUN(B, c0,
          (launch_pdl(k_resid<T>, nt, kThreads, Lv_.sm_resid, s, G, tl, tab, skip, bl, cur, v.t.p,
                                                          W)));
  const Level& Lc = B.L[lev + 1];
  EQF_RUN(B, lev > 0 ? KC_COARSE : KC_RESTRICT0,
          (launch_pdl(k_restrict<T>, Lc.ntiles(), kThreads, Lc.sm_restrict, s, 
              Lc.dgeom.p, Lc.dtiles.p, skip, v.t.p, lv[lev + 1].b.p, W)));
  T* xc = vcycle(s, lev + 1, false);
  EQF_RUN(B, lev > 0 ? KC_COARSE : KC_PROLONG0,
          (launch_pdl(k_prolong<T>, nt, kThreads, Lv_.sm_prolong, s, G, Lc.dgeom.p, tl, skip, xc, cur,
                                                              W)));
  // post-smoothing from the corrected iterate
  const int deg_post = B.opts.cheb_post;
  for (int st = 0; st < deg_post; ++st) {
    cheb_step<T>(B, s, lev, nt, G, tl, tab, skip, st, st == 0, false,
                 dot && st == deg_post - 1, bl, cur, oth, v.d.p, part);
    std::swap(cur, oth);
  }
  return cur;
}

// One refinement sweep: FP64 residual, preconditioned CG on the correction,
// update.  The step reads U[cur] and writes U[1 - cur].
template <class T>
void Work<T>::enqueue_sweep(cudaStream_t s, bool first, int iters, bool late) {
  const Level& L0 = B.L[0];
  const int nt = L0.ntiles();
  const int nb = (B.ntraps + 127) / 128;
  const LevelGeom* G = L0.dgeom.p;
  const Tile* tl = L0.dtiles.p;
  const T* tab = level_tab<T>(L0);
  double* part = B.dpart.p;
  T* r = lv[0].b.p;  // CG residual = V-cycle rhs on level 0
  // FP32 inner solve: stop at inner_tol relative reduction, or once the correction
  // residual is below 0.3 rtol |b| (the outer check then passes); FP64: rtol |b|.
  const bool fp32 = std::is_same<T, float>::value;
  const double tol_rel = fp32 ? B.opts.inner_tol : 0.0;
  const double tol_abs = fp32 ? 0.3 * B.opts.rtol : B.opts.rtol;
  double* u_out = B.U[1 - B.cur].p;
  float* d_out = B.Dd[1 - B.cur].p;
  bool pairs = false;
  if constexpr (std::is_same<T, float>::value) {
    pairs = !B.opts.residual64;
    if (pairs) {
      // FP32 form: residuals in float-pair arithmetic, rhs b kept as pairs
      float2* b2 = reinterpret_cast<float2*>(B.b64.p);
      if (first)
        EQF_RUN(B, KC_IR_RESID_FIRST,
                (launch_pdl(k_irf_first, nt, kThreads, L0.sm_irf1, s,
                    G, tl, B.tabA2.p, B.tabM2.p, B.dstate.p, B.F.p, B.U[B.cur].p, B.Dd[B.cur].p,
                    b2, u_out, d_out, r, part, nt, B.d_frozen.p, W)));
      else
        EQF_RUN(B, KC_IR_RESID,
                (launch_pdl(k_irf_residual<false>, nt, kThreads, L0.sm_irf, s,
                    G, tl, B.tabA2.p, B.d_ir_done.p, b2, u_out, d_out, r, part, nt, W)));
    }
  }
  if (!pairs) {  // FP64 residuals (the plain form; the FP32 form with residual64)
    if (first)
      EQF_RUN(B, KC_IR_RESID_FIRST,
              (launch_pdl(k_ir_first<T>, nt, kThreads, L0.sm_ir, s, 
                  G, tl, L0.tabd.p, B.tabM0.p, B.dstate.p, B.F.p, B.U[B.cur].p, B.Dd[B.cur].p,
                  B.b64.p, u_out, d_out, r, part, nt, B.d_frozen.p, W)));
    else
      EQF_RUN(B, KC_IR_RESID,
              (launch_pdl(k_ir_residual<T, false>, nt, kThreads, L0.sm_ir, s, 
                  G, tl, L0.tabd.p, B.d_ir_done.p, B.b64.p, u_out, d_out, r, part, nt, W)));
  }
  EQF_RUN(B, KC_SCALAR,
          (launch_pdl(k_s_ir, nb, 128, 0, s, B.ntraps, B.drange.p, part, nt, first ? 1 : 0, B.opts.rtol,
                                     B.dstate.p, B.d_ir_done.p, B.d_cg_skip.p, B.d_frozen.p)));
  // the folded CG writes the correction at its first update (x = alpha p), so only the
  // other Krylov paths start from a zeroed correction
  const bool fold = !B.use_bicgstab && B.fused0 && r2.p;
  if (!fold) EQF_CK(cudaMemsetAsync(xs.p, 0, B.L[0].nodes * sizeof(T), s));
  const int n2 = (int)L0.tiles2.size();
  // (buffers sized at construction: a batch whose tiles outgrew them runs full grids)
  const bool listed = fold && late && act_idx.p && act_idx.n >= (size_t)n2 &&
                      act_ridx.n >= (size_t)nt;
  if (listed) {  // the iterating traps' finest-level 2-D tiles and row tiles
    EQF_CK(cudaMemsetAsync(act_cnt.p, 0, 4 * sizeof(int), s));
    EQF_RUN(B, KC_SCALAR,
            (k_active_tiles<Tile2><<<(n2 + 255) / 256, 256, 0, s>>>(
                G, L0.dtiles2.p, n2, L0.ntiles2_cls, B.d_cg_skip.p, act_idx.p, act_cnt.p)));
    EQF_RUN(B, KC_SCALAR,
            (k_active_tiles<Tile><<<(nt + 255) / 256, 256, 0, s>>>(
                G, tl, nt, L0.ntiles_cls, B.d_cg_skip.p, act_ridx.p, act_cnt.p + 2)));
  }
  late_lists = listed;
  if (B.use_bicgstab) {
    bicgstab(s, r, tol_rel, tol_abs, iters);
    EQF_RUN(B, KC_IR_UPDATE,
            (launch_pdl(k_ir_update<T>, nt, kThreads, 0, s, G, tl, B.d_ir_done.p, xs.p, u_out,
                        d_out, (const CgState*)nullptr, (const T*)nullptr,
                        TileList{nullptr, nullptr}, W)));
    return;
  }
  T* pin = p0.p;
  T* pout = p1.p;
  // With the fused finest level, iteration it's update x += alpha p, r -= alpha q is
  // folded into iteration it+1's k_down (residual ping-ponged between r and r2), and
  // the last iteration's x update into k_ir_update: no k_cg_update pass over the grid.
  T* rcur = r;
  T* ralt = r2.p;
  for (int it = 0; it < iters; ++it) {
    Fold fd;
    const bool use = fold && it > 0;
    if (use)
      fd = Fold{CgFold<T>{q.p, ralt, pin, xs.p, B.dstate.p, part, it == 1 ? 1 : 0}, tol_rel,
                tol_abs};
    T* z = vcycle(s, 0, true, rcur, use ? &fd : nullptr);
    if (use) std::swap(rcur, ralt);
    EQF_RUN(B, KC_SCALAR,
            (launch_pdl(k_s_rz, nb, 128, 0, s, B.ntraps, B.fused0 ? B.drange2.p : B.drange.p, part,
                                       B.dstate.p, B.d_cg_skip.p)));
    {  // class-table traps' row tiles, then general-path traps' (part by tile index)
      const int nc = L0.ntiles_cls, ng = nt - nc;
      int* sk = B.d_cg_skip.p;
      CgState* cs = B.dstate.p;
      const TileList none{nullptr, nullptr};
      if (listed) {  // absolute tile indices into the whole row-tile array
        const TileList rc{act_ridx.p, act_cnt.p + 2}, rg{act_ridx.p + nc, act_cnt.p + 3};
        if (it == 0) {
          if (nc > 0)
            EQF_RUN(B, KC_CG_DIR,
                    (launch_pdl(k_cg_dir<T, true, false, true>, listed_grid(nc), kThreads,
                                L0.sm_cgdir, s, G, tl, tab, sk, cs, z, pin, pout, q.p, part, rc,
                                W)));
          if (ng > 0)
            EQF_RUN(B, KC_CG_DIR,
                    (launch_pdl(k_cg_dir<T, true, true, true>, listed_grid(ng), kThreads,
                                L0.sm_cgdir, s, G, tl, tab, sk, cs, z, pin, pout, q.p, part, rg,
                                W)));
        } else {
          if (nc > 0)
            EQF_RUN(B, KC_CG_DIR,
                    (launch_pdl(k_cg_dir<T, false, false, true>, listed_grid(nc), kThreads,
                                L0.sm_cgdir, s, G, tl, tab, sk, cs, z, pin, pout, q.p, part, rc,
                                W)));
          if (ng > 0)
            EQF_RUN(B, KC_CG_DIR,
                    (launch_pdl(k_cg_dir<T, false, true, true>, listed_grid(ng), kThreads,
                                L0.sm_cgdir, s, G, tl, tab, sk, cs, z, pin, pout, q.p, part, rg,
                                W)));
        }
      } else if (it == 0) {
        if (nc > 0)
          EQF_RUN(B, KC_CG_DIR, (launch_pdl(k_cg_dir<T, true, false>, nc, kThreads, L0.sm_cgdir,
                                            s, G, tl, tab, sk, cs, z, pin, pout, q.p, part, none,
                                            W)));
        if (ng > 0)
          EQF_RUN(B, KC_CG_DIR, (launch_pdl(k_cg_dir<T, true, true>, ng, kThreads, L0.sm_cgdir, s,
                                            G, tl + nc, tab, sk, cs, z, pin, pout, q.p,
                                            part + nc, none, W)));
      } else {
        if (nc > 0)
          EQF_RUN(B, KC_CG_DIR, (launch_pdl(k_cg_dir<T, false, false>, nc, kThreads,
                                            L0.sm_cgdir, s, G, tl, tab, sk, cs, z, pin, pout,
                                            q.p, part, none, W)));
        if (ng > 0)
          EQF_RUN(B, KC_CG_DIR, (launch_pdl(k_cg_dir<T, false, true>, ng, kThreads,
                                            L0.sm_cgdir, s, G, tl + nc, tab, sk, cs, z, pin,
                                            pout, q.p, part + nc, none, W)));
      }
    }
    EQF_RUN(B, KC_SCALAR,
            (launch_pdl(k_s_pq, nb, 128, 0, s, B.ntraps, B.drange.p, part, B.dstate.p,
                        B.d_cg_skip.p, fold ? 1 : 0)));
    if (!fold) {
      EQF_RUN(B, KC_CG_UPDATE,
              (launch_pdl(k_cg_update<T>, nt, kThreads, 0, s, G, tl, B.d_cg_skip.p, B.dstate.p,
                          pout, q.p, xs.p, r, part, W)));
      EQF_RUN(B, KC_SCALAR,
              (launch_pdl(k_s_rr, nb, 128, 0, s, B.ntraps, B.drange.p, part, tol_rel, tol_abs,
                          B.dstate.p, B.d_cg_skip.p, 0)));
    }
    std::swap(pin, pout);
  }
  late_lists = false;
  // folded: traps still iterating at the end take their last alpha p here (pin now
  // holds the last direction)
  const T* plast = fold ? (const T*)pin : nullptr;
  if (listed) {  // the sweep's iterating traps are the ones not done (ir_done == cg_skip)
    const int nc = L0.ntiles_cls, ng = nt - nc;
    if (nc > 0)
      EQF_RUN(B, KC_IR_UPDATE,
              (launch_pdl(k_ir_update<T, true>, listed_grid(nc), kThreads, 0, s, G, tl,
                          B.d_ir_done.p, xs.p, u_out, d_out, (const CgState*)B.dstate.p, plast,
                          TileList{act_ridx.p, act_cnt.p + 2}, W)));
    if (ng > 0)
      EQF_RUN(B, KC_IR_UPDATE,
              (launch_pdl(k_ir_update<T, true>, listed_grid(ng), kThreads, 0, s, G, tl,
                          B.d_ir_done.p, xs.p, u_out, d_out, (const CgState*)B.dstate.p, plast,
                          TileList{act_ridx.p + nc, act_cnt.p + 3}, W)));
  } else {
    EQF_RUN(B, KC_IR_UPDATE,
            (launch_pdl(k_ir_update<T>, nt, kThreads, 0, s, G, tl, B.d_ir_done.p, xs.p, u_out,
                        d_out, (const CgState*)B.dstate.p, plast, TileList{nullptr, nullptr},
                        W)));
  }
}

// Right-preconditioned BiCGSTAB on the correction x (xs) from residual r (the
// V-cycle is the preconditioner); ceil(max_iters / 2) iterations of two
// preconditioner applications each.
template <class T>
void Work<T>::bicgstab(cudaStream_t s, T* r, double tol_rel, double tol_abs, int max_iters) {
  const Level& L0 = B.L[0];
  const int nt = L0.ntiles();
  const int nb = (B.ntraps + 127) / 128;
  const LevelGeom* G = L0.dgeom.p;
  const Tile* tl = L0.dtiles.p;
  const T* tab = level_tab<T>(L0);
  double* part = B.dpart.p;
  int* skip = B.d_cg_skip.p;
  CgState* st = B.dstate.p;
  T* p = p0.p;
  T* v = p1.p;
  T* t = q.p;
  const int iters = (max_iters + 1) / 2;
  for (int it = 0; it < iters; ++it) {
    if (it == 0) {
      EQF_RUN(B, KC_CG_UPDATE,
              (launch_pdl(k_bs_dir<T, true>, nt, kThreads, 0, s, G, tl, skip, st, r, v, p, rh.p, part,
                                                         W)));
      EQF_RUN(B, KC_SCALAR,
              (launch_pdl(k_s_bs_rho0, nb, 128, 0, s, B.ntraps, B.drange.p, part, st, skip)));
    } else {
      EQF_RUN(B, KC_CG_UPDATE,
              (launch_pdl(k_bs_dir<T, false>, nt, kThreads, 0, s, G, tl, skip, st, r, v, p, rh.p, part,
                                                          W)));
    }
    const T* ph = vcycle(s, 0, false, p);
    EQF_RUN(B, KC_CG_DIR,
            (launch_pdl(k_apply_dot<T, 1>, nt, kThreads, L0.sm_resid, s, G, tl, tab, skip, ph, rh.p, v,
                                                                  part, nt, W)));
    EQF_RUN(B, KC_SCALAR,
            (launch_pdl(k_s_bs_alpha, nb, 128, 0, s, B.ntraps, B.drange.p, part, st, skip)));
    EQF_RUN(B, KC_CG_UPDATE,
            (launch_pdl(k_bs_half<T>, nt, kThreads, 0, s, G, tl, skip, st, ph, v, xs.p, r, part, W)));
    EQF_RUN(B, KC_SCALAR,
            (launch_pdl(k_s_bs_half, nb, 128, 0, s, B.ntraps, B.drange.p, part, tol_rel, tol_abs, st,
                                            skip)));
    const T* sh = vcycle(s, 0, false, r);
    EQF_RUN(B, KC_CG_DIR,
            (launch_pdl(k_apply_dot<T, 2>, nt, kThreads, L0.sm_resid, s, G, tl, tab, skip, sh, r, t,
                                                                  part, nt, W)));
    EQF_RUN(B, KC_SCALAR,
            (launch_pdl(k_s_bs_omega, nb, 128, 0, s, B.ntraps, B.drange.p, part, nt, st, skip)));
    EQF_RUN(B, KC_CG_UPDATE,
            (launch_pdl(k_bs_full<T>, nt, kThreads, 0, s, G, tl, skip, st, sh, t, rh.p, xs.p, r, part,
                                                  nt, W)));
    EQF_RUN(B, KC_SCALAR,
            (launch_pdl(k_s_bs_rho, nb, 128, 0, s, B.ntraps, B.drange.p, part, nt, tol_rel, tol_abs, st,
                                           skip)));
  }
}

// Final FP64 residual check after the last sweep: marks converged traps, counts
// the others in d_fail and sets the next step's extrapolation factor.
template <class T>
void Work<T>::enqueue_check(cudaStream_t s, bool update_gamma) {
  const Level& L0 = B.L[0];
  const int nt = L0.ntiles();
  bool pairs = false;
  if constexpr (std::is_same<T, float>::value) {
    pairs = !B.opts.residual64;
    if (pairs)
      EQF_RUN(B, KC_IR_RESID,
              (launch_pdl(k_irf_residual<true>, nt, kThreads, L0.sm_irf, s,
                  L0.dgeom.p, L0.dtiles.p, B.tabA2.p, B.d_ir_done.p,
                  reinterpret_cast<const float2*>(B.b64.p), B.U[1 - B.cur].p, B.Dd[1 - B.cur].p,
                  lv[0].b.p, B.dpart.p, nt, W)));
  }
  if (!pairs)
    EQF_RUN(B, KC_IR_RESID,
            (launch_pdl(k_ir_residual<T, true>, nt, kThreads, L0.sm_ir, s, 
                L0.dgeom.p, L0.dtiles.p, L0.tabd.p, B.d_ir_done.p, B.b64.p, B.U[1 - B.cur].p,
                B.Dd[1 - B.cur].p, lv[0].b.p, B.dpart.p, nt, W)));
  EQF_RUN(B, KC_SCALAR,
          (launch_pdl(k_s_final, (B.ntraps + 127) / 128, 128, 0, s, B.ntraps, B.drange.p, B.dpart.p, nt,
                                                             B.opts.rtol, B.dstate.p,
                                                             B.d_ir_done.p, B.d_fail.p,
                                                             update_gamma ? 1 : 0)));
}

// Per-step sources of coupled species: gather every cell's concentration from the
// field at the start of the step, apply the sender/receiver law, re-deposit.
void Batch::enqueue_coupling() {
  if (ncp == 0) return;
  EQF_RUN(*this, KC_SCALAR,
          (k_cells_gather<<<(ncells + 255) / 256, 256, 0, stream>>>(ncells, d_ent_node.p, d_ent_w.p,
                                                                  u_cur(), d_cp_c.p)));
  EQF_RUN(*this, KC_SCALAR,
          (k_cells_qs_sources<<<(ncp + 255) / 256, 256, 0, stream>>>(
              ncp, d_cp_i1.p, d_cp_i2.p, d_cp_sender.p, d_cp_prod.p, d_cp_law.p, d_cp_laws.p,
              d_cp_c.p, d_cell_s.p)));
  refresh_load();
}

// ---------------------------------------------------------------------------
// Wall conditions with values, Robin loads and flow channels (eqf_set_boundaries).

// Device data of the traps whose walls carry values, Robin loads or channels: their
// rim slots, and per channel trap the Crank-Nicolson matrices of the sub-step with
// the parallel-cyclic-reduction multipliers of its left side.
void Batch::setup_walls() {
  hwalls.clear();
  chans.clear();
  rim_max = 0;
  chan_n_max = 0;
  int rim_total = 0;
  for (int t = 0; t < ntraps; ++t) {
    const eqf_boundaries& bc = bcs[t];
    const eqf_trap_params& p = params[t];
    bool active = false, channel = false;
    for (int w = 0; w < 4; ++w) {
      const eqf_wall& wl = bc.wall[w];
      active = active || wl.kind == EQF_BC_CHANNEL || wl.kind == EQF_BC_WELL ||
               (wl.kind != EQF_BC_NEUMANN && wl.value != 0.0);
      channel = channel || wl.kind == EQF_BC_CHANNEL;
    }
    if (!active) continue;
    WallDev wd{};
    wd.trap = t;
    wd.rim0 = rim_total;
    wd.well = d_well_c.p + t;
    for (int w = 0; w < 4; ++w) {
      wd.kind[w] = bc.wall[w].kind;
      wd.value[w] = bc.wall[w].value;
      wd.robs[w] = bc.wall[w].kind == EQF_BC_ROBIN ? p.dt * bc.wall[w].rate * bc.wall[w].value : 0.0;
    }
    const int nr = rim_count(p.nx, p.ny);
    rim_total += nr;
    rim_max = std::max(rim_max, nr);
    if (channel) {
      // the channel: nx cells of h_c = W/nx on [0, W], dt_c = dt / substeps
      auto ch = std::make_unique<Chan>();
      ch->trap = t;
      const int n = p.nx + 1;
      ch->n = n;
      const double h = p.width / p.nx, dtc = p.dt / bc.channel_substeps;
      const double D = bc.channel_D, v = bc.channel_velocity;
      // element matrices of fenics/AdvectionDiffusion.ufl (test row, trial column):
      // M h/6 [2 1; 1 2], K 1/h [1 -1; -1 1], C (w * du/dx) [-1/2 1/2; -1/2 1/2]
      std::vector<double> a(n, 0.0), b(n, 0.0), c(n, 0.0), bl(n, 0.0), bd(n, 0.0), bu(n, 0.0);
      const double me[2][2] = {{h / 3.0, h / 6.0}, {h / 6.0, h / 3.0}};
      const double ke[2][2] = {{1.0 / h, -1.0 / h}, {-1.0 / h, 1.0 / h}};
      const double ce[2][2] = {{-0.5, 0.5}, {-0.5, 0.5}};
      for (int e = 0; e < n - 1; ++e)
        for (int r = 0; r < 2; ++r)
          for (int q = 0; q < 2; ++q) {
            const double op = 0.5 * dtc * (D * ke[r][q] + v * ce[r][q]);
            const double lhs = me[r][q] + op, rhs = me[r][q] - op;
            const int i = e + r, jn = e + q;
            if (jn == i) {
              b[i] += lhs;
              bd[i] += rhs;
            } else if (jn == i + 1) {
              c[i] += lhs;
              bu[i] += rhs;
            } else {
              a[i] += lhs;
              bl[i] += rhs;
            }
          }
      // Robin ends: dt_c * r * (0.5 (c0 + c) - 0) w at x = 0 (ds(1)) and x = W (ds(2))
      b[0] += 0.5 * dtc * bc.channel_rate[0];
      bd[0] -= 0.5 * dtc * bc.channel_rate[0];
      b[n - 1] += 0.5 * dtc * bc.channel_rate[1];
      bd[n - 1] -= 0.5 * dtc * bc.channel_rate[1];
      // parallel cyclic reduction of the left side: at stride s, row i eliminates
      // x_{i-s} and x_{i+s} with rows i-s and i+s
      std::vector<double> k1, k2;
      int levels = 0;
      for (int st = 1; st < n; st <<= 1, ++levels) {
        std::vector<double> na(n, 0.0), nb(n, 0.0), nc(n, 0.0);
        k1.resize((size_t)(levels + 1) * n);
        k2.resize((size_t)(levels + 1) * n);
        for (int i = 0; i < n; ++i) {
          const double m1 = i - st >= 0 ? a[i] / b[i - st] : 0.0;
          const double m2 = i + st < n ? c[i] / b[i + st] : 0.0;
          k1[(size_t)levels * n + i] = m1;
          k2[(size_t)levels * n + i] = m2;
          na[i] = i - st >= 0 ? -a[i - st] * m1 : 0.0;
          nc[i] = i + st < n ? -c[i + st] * m2 : 0.0;
          nb[i] = b[i] - (i - st >= 0 ? c[i - st] * m1 : 0.0) - (i + st < n ? a[i + st] * m2 : 0.0);
        }
        a.swap(na);
        b.swap(nb);
        c.swap(nc);
      }
      ch->levels = levels;
      auto up = [&](DevBuf<double>& d, const std::vector<double>& h_) {
        d.alloc(std::max<size_t>(1, h_.size()));
        if (!h_.empty()) d.upload(h_.data(), h_.size(), stream);
      };
      for (double& v : b) v = 1.0 / v;  // the kernel multiplies by the reciprocal
      up(ch->k1, k1);
      up(ch->k2, k2);
      up(ch->bfin, b);
      up(ch->bl, bl);
      up(ch->bd, bd);
      up(ch->bu, bu);
      for (int side = 0; side < 2; ++side)
        if (bc.wall[side].kind == EQF_BC_CHANNEL) {
          ch->c[side].alloc(n);
          EQF_CK(cudaMemsetAsync(ch->c[side].p, 0, n * sizeof(double), stream));
          wd.chan[side] = ch->c[side].p;
        }
      chan_n_max = std::max(chan_n_max, n);
      chans.push_back(std::move(ch));
    }
    hwalls.push_back(wd);
  }
  walls_active = !hwalls.empty();
  d_walls.alloc(hwalls.size());
  if (walls_active) d_walls.upload(hwalls.data(), hwalls.size(), stream);
  {
    std::vector<int> of(ntraps, -1);
    for (size_t w = 0; w < hwalls.size(); ++w) of[hwalls[w].trap] = (int)w;
    d_wall_of.upload(of.data(), ntraps, stream);
  }
  d_fbase.alloc(std::max(rim_total, 1));
  EQF_CK(cudaMemsetAsync(d_fbase.p, 0, d_fbase.n * sizeof(double), stream));
  std::vector<ChanDev> hc;
  for (const auto& up : chans) {
    const Chan& ch = *up;
    const eqf_boundaries& bc = bcs[ch.trap];
    const eqf_trap_params& p = params[ch.trap];
    ChanDev d{};
    d.trap = ch.trap;
    d.n = ch.n;
    d.levels = ch.levels;
    d.substeps = bc.channel_substeps;
    d.h = p.height / p.ny;
    d.dtD = p.dt * p.D;
    d.well = bc.well_scaling;
    d.k1 = ch.k1.p;
    d.k2 = ch.k2.p;
    d.bfin = ch.bfin.p;
    d.bl = ch.bl.p;
    d.bd = ch.bd.p;
    d.bu = ch.bu.p;
    d.c[0] = ch.c[0].p;
    d.c[1] = ch.c[1].p;
    hc.push_back(d);
  }
  d_chans.alloc(hc.size());
  if (!hc.empty()) {
    d_chans.upload(hc.data(), hc.size(), stream);
    // the attribute belongs to the kernel, not to this batch: always the largest size
    EQF_CK(cudaFuncSetAttribute(k_channel_step<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)chan_smem_bytes(kChanMaxNodes)));
    EQF_CK(cudaFuncSetAttribute(k_channel_step<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)chan_smem_bytes(kChanMaxNodes)));
    EQF_CK(cudaFuncSetAttribute(k_channel_step<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)chan_smem_bytes(kChanMaxNodes)));
  }
  // the load vector restarts from the point cells alone (rims included)
  bal_load_ok = false;
  if (!cells_dirty) {
    EQF_CK(cudaMemsetAsync(F.p, 0, L[0].nodes * sizeof(double), stream));
    refresh_load();
  }
  drop_graphs();
  sync();
}

void Batch::setup_wells() {
  hwells.clear();
  for (int t = 0; t < ntraps; ++t) {
    if (!(well[t].scale > 0.0)) continue;
    WellDev w{};
    w.trap = t;
    w.scale = well[t].scale;
    w.decay_dt = params[t].dt * well[t].decay;
    w.Ddt = params[t].D * params[t].dt;
    w.conc = d_well_c.p + t;
    w.under = d_well_under.p + t;
    hwells.push_back(w);
  }
  d_wells.alloc(hwells.size());
  if (!hwells.empty()) d_wells.upload(hwells.data(), hwells.size(), stream);
  sync();
}

// After the step (and the channels): the boundary wells take the new field's flux.
void Batch::enqueue_wells() {
  if (hwells.empty()) return;
  EQF_RUN(*this, KC_SCALAR,
          (k_well_update<<<(unsigned)hwells.size(), kThreads, 0, stream>>>(
              d_wells.p, L[0].dgeom.p, U[1 - cur].p, d_frozen.p)));
}

// After the solve (and any extra sweeps): the step's FP64 balance from the new field
// U[1 - cur], the field the step started from U[cur] and the step's load F.
void Batch::enqueue_balance() {
  if (!bal_on) return;
  const int nt = L[0].ntiles();
  int longest = 1;  // outer ring, or the two-node rim of a trap with wall values
  for (int t = 0; t < ntraps; ++t) {
    const LevelGeom& g = L[0].geom[t];
    longest = std::max(longest, 2 * (g.nx + 1) + 2 * (g.ny - 1));
    if (g.nx >= 3 && g.ny >= 3) longest = std::max(longest, rim_count(g.nx, g.ny));
  }
  // one CTA per trap walks its ring (a few thousand nodes): more CTAs per trap only
  // add waves of this register-heavy kernel
  (void)longest;
  const int rim_blocks = 1;
  grow(bal_part, (size_t)nt * kBalTileParts);
  grow(bal_rpart, (size_t)ntraps * rim_blocks * kBalRimParts);
  // the field a step starts from is the last step's result unless the host or the rod
  // exchange changed it; the load stays unless the cells' rates, the coupling or the
  // wall values rebuilt it
  const bool old = !bal_prev_ok || !rod_sets.empty();
  const bool load = !bal_load_ok || ncp > 0 || walls_active;
  auto tiles = old ? (load ? k_balance_tiles<true, true> : k_balance_tiles<true, false>)
                   : (load ? k_balance_tiles<false, true> : k_balance_tiles<false, false>);
  EQF_RUN(*this, KC_BALANCE,
          (tiles<<<nt, kThreads, 0, stream>>>(L[0].dgeom.p, L[0].dtiles.p, U[1 - cur].p, U[cur].p,
                                              F.p, d_frozen.p, bal_part.p)));
  EQF_RUN(*this, KC_BALANCE,
          (k_balance_rim<<<dim3(rim_blocks, ntraps), kThreads, 0, stream>>>(
              L[0].dgeom.p, U[1 - cur].p, U[cur].p, F.p, d_wall_of.p, d_walls.p, d_fbase.p,
              d_frozen.p, old ? 1 : 0, load ? 1 : 0, bal_rpart.p)));
  EQF_RUN(*this, KC_BALANCE,
          (k_balance_finish<<<(ntraps + 3) / 4, 128, 0, stream>>>(
              L[0].dgeom.p, drange.p, bal_part.p, bal_rpart.p, rim_blocks, d_frozen.p, ntraps,
              old ? 1 : 0, load ? 1 : 0, d_bal.p)));
  bal_prev_ok = bal_load_ok = true;
}

void Batch::enqueue_walls() {
  if (!walls_active) return;
  const dim3 grid((rim_max + 255) / 256, (unsigned)hwalls.size());
  EQF_RUN(*this, KC_SCALAR,
          (k_wall_rim<2><<<grid, 256, 0, stream>>>(d_walls.p, L[0].dgeom.p, F.p, d_fbase.p)));
}

// After the step's solve (the new field is U[1 - cur]): fluxes into the channels and
// their sub-steps.
void Batch::enqueue_channels() {
  if (chans.empty()) return;
  // nodes per thread of the longest channel: the prefetching sweep up to 2 (more
  // would hold so many registers that fewer channels share an SM)
  const int npt = (chan_n_max + kChanThreads - 1) / kChanThreads;
  auto kern = npt == 1 ? k_channel_step<1> : npt == 2 ? k_channel_step<2> : k_channel_step<0>;
  EQF_RUN(*this, KC_SCALAR,
          (kern<<<dim3((unsigned)chans.size(), 2), kChanThreads, chan_smem_bytes(chan_n_max),
                  stream>>>(d_chans.p, L[0].dgeom.p, U[1 - cur].p, d_frozen.p)));
}

// ---------------------------------------------------------------------------
// Rod cells: footprints and dependency waves (at every geometry update), and the
// per-step exchange (one launch per wave, captured with the step).

Batch::RodSet* Batch::rod_set_of(int layer0) {
  for (auto& rs : rod_sets)
    if (rs->layers[0] == layer0) return rs.get();
  return nullptr;
}

void Batch::rod_analyse(RodSet& rs) { rod_analyse_sets({&rs}); }

constexpr int kRodFlags = 5;  // per set in rod_hflags

// Footprints (sizes, then nodes), the shared-node test, the waves of the sets with
// shared nodes and the wave offsets: each phase is queued for every set, then one
// round trip brings the sizes the next phase needs.
void Batch::rod_analyse_sets(const std::vector<RodSet*>& sets) {
  const int bs = 256, ns = (int)sets.size();
  if (ns == 0) return;
  // per set: footprint size, shared, highest wave, unsettled, relaxation passes
  rod_hflags.grow(kRodFlags * (size_t)ns);
  int* hf = rod_hflags.p;
  for (int q = 0; q < ns; ++q) {
    RodSet& rs = *sets[q];
    const int n = rs.n;
    rs.grid = std::max(1, std::min((n * 32 + bs - 1) / bs, num_sms * 16));
    grow(rs.sc_count, n);
    k_rod_footprint<false><<<rs.grid, bs, 0, stream>>>(n, rs.rods.p, rs.dlaw.p, rs.sc_count.p,
                                                       nullptr, nullptr, nullptr);
    EQF_LAUNCH_CHECK();
    scan(n, rs.sc_count.p, rs.fp_off.p);
    EQF_CK(cudaMemcpyAsync(hf + kRodFlags * q, rs.fp_off.p + n, sizeof(int), cudaMemcpyDeviceToHost,
                           stream));
  }
  sync();
  for (int q = 0; q < ns; ++q) {  // the footprints; does any node lie in two of them?
    RodSet& rs = *sets[q];
    const int n = rs.n, nent = hf[kRodFlags * q];
    if ((size_t)nent > rs.fp_node.n) {
      const size_t cap = (size_t)nent + (size_t)nent / 4 + 64;
      rs.fp_node.alloc(cap);
      rs.ent_cell.alloc(cap);
    }
    rs.nent = nent;
    k_rod_footprint<true><<<rs.grid, bs, 0, stream>>>(n, rs.rods.p, rs.dlaw.p, nullptr,
                                                      rs.fp_off.p, rs.fp_node.p, rs.ent_cell.p);
    EQF_LAUNCH_CHECK();
    const int ge = (nent + bs - 1) / bs;
    EQF_CK(cudaMemsetAsync(rs.cover.p, 0, rs.span * sizeof(int), stream));
    EQF_CK(cudaMemsetAsync(rs.flag.p, 0, sizeof(int), stream));
    k_rod_cover<<<ge, bs, 0, stream>>>(nent, rs.fp_node.p, 0, rs.cover.p, rs.flag.p);
    EQF_LAUNCH_CHECK();
    EQF_CK(cudaMemcpyAsync(hf + kRodFlags * q + 1, rs.flag.p, sizeof(int), cudaMemcpyDeviceToHost,
                           stream));
  }
  sync();
  bool any = false;
  for (int q = 0; q < ns; ++q) {  // waves: bucket the entries by node, each bucket in
    RodSet& rs = *sets[q];        // cell order; a cell's wave = its longest chain
    hf[kRodFlags * q + 2] = hf[kRodFlags * q + 3] = hf[kRodFlags * q + 4] = 0;
    if (!hf[kRodFlags * q + 1]) continue;
    any = true;
    const int n = rs.n, nent = rs.nent;
    const int ge = (nent + bs - 1) / bs, gc = (n + bs - 1) / bs;
    scan((int)rs.span, rs.cover.p, rs.start.p);
    EQF_CK(cudaMemsetAsync(rs.cursor.p, 0, rs.span * sizeof(int), stream));
    grow(rs.sc_perm, nent);
    grow(rs.sc_pred, nent);
    grow(rs.sc_succ, nent);
    grow(rs.sc_wave, n);
    grow(rs.sc_wcount, n);
    k_rod_place<<<ge, bs, 0, stream>>>(nent, rs.fp_node.p, 0, rs.start.p, rs.cursor.p,
                                       rs.sc_perm.p);
    EQF_LAUNCH_CHECK();
    k_rod_bucket_order<<<ge, bs, 0, stream>>>(nent, rs.fp_node.p, 0, rs.start.p, rs.cover.p,
                                              rs.sc_perm.p);
    EQF_LAUNCH_CHECK();
    k_rod_preds<<<ge, bs, 0, stream>>>(nent, rs.fp_node.p, 0, rs.start.p, rs.sc_perm.p,
                                       rs.ent_cell.p, rs.sc_pred.p, rs.sc_succ.p);
    EQF_LAUNCH_CHECK();
    EQF_CK(cudaMemsetAsync(rs.sc_wave.p, 0, n * sizeof(int), stream));
    // the whole relaxation in one CTA (no host round trip per pass); flag[1] reports a
    // relaxation that did not settle within its bound, flag[2] the passes it took
    EQF_CK(cudaMemsetAsync(rs.flag.p, 0, 3 * sizeof(int), stream));
    k_rod_relax_all<<<1, 1024, 0, stream>>>(nent, n, rs.sc_pred.p, rs.sc_succ.p, rs.sc_wave.p,
                                            rs.flag.p + 1, rs.flag.p + 2);
    EQF_LAUNCH_CHECK();
    EQF_CK(cudaMemsetAsync(rs.sc_wcount.p, 0, n * sizeof(int), stream));
    k_rod_wave_count<<<gc, bs, 0, stream>>>(n, rs.sc_wave.p, rs.sc_wcount.p, rs.flag.p);
    EQF_LAUNCH_CHECK();
    EQF_CK(cudaMemcpyAsync(hf + kRodFlags * q + 2, rs.flag.p, 3 * sizeof(int), cudaMemcpyDeviceToHost,
                           stream));
  }
  if (any) sync();
  // wave offsets: {0, n} when no node is shared, else the scan of the wave sizes
  std::vector<size_t> wo(ns + 1, 0);
  for (int q = 0; q < ns; ++q) {
    if (hf[kRodFlags * q + 1] && hf[kRodFlags * q + 3])
      throw Error(EQF_ERR_CUDA, "rod wave analysis did not settle");
    wo[q + 1] = wo[q] + (hf[kRodFlags * q + 1] ? (size_t)hf[kRodFlags * q + 2] + 2 : 2);
    sets[q]->relax_passes = hf[kRodFlags * q + 4];
  }
  rod_hwoff.grow(wo[ns]);
  int* hw = rod_hwoff.p;
  for (int q = 0; q < ns; ++q) {
    RodSet& rs = *sets[q];
    const int n = rs.n, gc = (n + bs - 1) / bs;
    if (!hf[kRodFlags * q + 1]) {
      k_rod_iota<<<gc, bs, 0, stream>>>(n, rs.wave_cells.p);
      EQF_LAUNCH_CHECK();
      hw[wo[q]] = 0;
      hw[wo[q] + 1] = n;
    } else {
      const int waves = hf[kRodFlags * q + 2] + 1;
      grow(rs.sc_wstart, waves + 1);
      scan(waves, rs.sc_wcount.p, rs.sc_wstart.p);
      EQF_CK(cudaMemsetAsync(rs.sc_wcount.p, 0, waves * sizeof(int), stream));
      k_rod_wave_place<<<gc, bs, 0, stream>>>(n, rs.sc_wave.p, rs.sc_wstart.p, rs.sc_wcount.p,
                                              rs.wave_cells.p);
      EQF_LAUNCH_CHECK();
      EQF_CK(cudaMemcpyAsync(hw + wo[q], rs.sc_wstart.p, (waves + 1) * sizeof(int),
                             cudaMemcpyDeviceToHost, stream));
    }
  }
  if (any) sync();
  for (int q = 0; q < ns; ++q) {
    RodSet& rs = *sets[q];
    const int n = rs.n, gc = (n + bs - 1) / bs;
    k_rod_cell_info<<<gc, bs, 0, stream>>>(n, rs.wave_cells.p, rs.fp_off.p, rs.rods.p,
                                           rs.dlaw.p, rs.winfo.p, rs.cellk.p);
    EQF_LAUNCH_CHECK();
    const size_t len = wo[q + 1] - wo[q];
    rs.waves = (int)len - 1;
    if (rs.wave_off.n < len) rs.wave_off.alloc(len + 8);
    EQF_CK(cudaMemcpyAsync(rs.wave_off.p, hw + wo[q], len * sizeof(int), cudaMemcpyHostToDevice,
                           stream));
  }
  sync();  // the pinned staging is reused by the next analysis
}

void Batch::rod_publish() {
  std::vector<RodSetDev> h;
  int waves = 0, grid = 1;
  for (auto& up : rod_sets) {
    RodSet& rs = *up;
    RodSetDev d;
    d.woff = rs.wave_off.p;
    d.winfo = rs.winfo.p;
    d.cellk = rs.cellk.p;
    d.rods = rs.rods.p;
    d.law = rs.dlaw.p;
    d.fp_node = rs.fp_node.p;
    d.ihsl = rs.ihsl.p;
    d.prod = rs.prod.p;
    d.mode = rs.mode.p;
    d.ehsl = rs.ehsl.p;
    d.waves = rs.waves;
    h.push_back(d);
    waves = std::max(waves, rs.waves);
    grid = std::max(grid, std::min((rs.n + kRodThreads - 1) / kRodThreads, num_sms * 4));
  }
  // the exchange's shared-memory stash exceeds the default 48 KB per block
  EQF_CK(cudaFuncSetAttribute(k_rod_exchange<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)rod_stash_bytes(1)));
  EQF_CK(cudaFuncSetAttribute(k_rod_exchange<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)rod_stash_bytes(2)));
  EQF_CK(cudaFuncSetAttribute(k_rod_exchange<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)rod_stash_bytes(3)));
  EQF_CK(cudaFuncSetAttribute(k_rod_exchange<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)rod_stash_bytes(4)));
  bool recapture = false;
  if (d_rod_sets.n != h.size()) {
    d_rod_sets.alloc(h.size());
    recapture = true;
  }
  if (!h.empty())
    EQF_CK(cudaMemcpyAsync(d_rod_sets.p, h.data(), h.size() * sizeof(RodSetDev),
                           cudaMemcpyHostToDevice, stream));
  sync();
  if (waves > rod_launches || grid > rod_grid || h.empty()) recapture = true;
  rod_launches = h.empty() ? 0 : std::max(rod_launches, waves);
  rod_grid = h.empty() ? 0 : std::max(rod_grid, grid);
  if (recapture) drop_graphs();
}

void Batch::enqueue_rods() {
  if (rod_launches == 0) return;
  const dim3 grid(rod_grid, (unsigned)rod_sets.size());
  int nl = 1;
  for (const auto& rs : rod_sets) nl = std::max(nl, (int)rs->layers.size());
  auto kern = nl == 1 ? k_rod_exchange<1>
              : nl == 2 ? k_rod_exchange<2>
              : nl == 3 ? k_rod_exchange<3>
                        : k_rod_exchange<4>;
  const size_t smem = rod_stash_bytes(nl);  // opted in by rod_publish
  for (int w = 0; w < rod_launches; ++w)
    EQF_RUN(*this, KC_ROD,
            (kern<<<grid, kRodThreads, smem, stream>>>(w, d_rod_sets.p, d_frozen.p, u_cur())));
}

void Batch::run_step() {
  enqueue_rods();
  enqueue_coupling();
  enqueue_walls();
  for (int sw = 0; sw < opts.max_sweeps; ++sw)
    work->enqueue_sweep(stream, sw == 0, opts.max_iters, sw >= 2);
  work->enqueue_check(stream, true);
}

void Batch::check_fail() {
  int derr = 0, f = 0;  // both flags in one round trip
  EQF_CK(cudaMemcpyFromSymbolAsync(&derr, g_eqf_device_error, sizeof(int), 0,
                                   cudaMemcpyDeviceToHost, stream));
  EQF_CK(cudaMemcpyAsync(&f, d_fail.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  sync();
  if (derr)
    throw Error(EQF_ERR_CUDA, "a device-side bounded wait gave up (staging copy never landed)");
  if (f > 0) {
    reset_fail();
    throw Error(EQF_ERR_NOT_CONVERGED,
                std::to_string(f) + " trap-step(s) missed rtol within the solver schedule");
  }
}

// Captures run_step() (and, with device_loop, the adaptive sweeps as a WHILE node
// whose body is one added sweep, its check and k_sweep_loop) and instantiates it.
void Batch::capture_step(cudaGraphExec_t& gx, bool device_loop) {
  const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  cudaGraph_t gr = nullptr;
  bool capturing = false;
  auto abandon = [&] {  // leave the stream out of capture mode on any error
    if (capturing) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(stream, &g);
      if (g) cudaGraphDestroy(g);
    }
    if (gr) cudaGraphDestroy(gr);
    cudaGetLastError();
  };
  cond_failed = false;
  // a failing conditional-node call marks the capture as one to redo without the loop
#define EQF_COND_CK(call)   \
  do {                      \
    cond_failed = true;     \
    EQF_CK(call);           \
    cond_failed = false;    \
  } while (0)
  try {
    cudaGraphConditionalHandle h{};
    std::vector<cudaGraphNode_t> leaf;
    if (device_loop && d_loop.n == 0) {
      d_loop.alloc(2);
      EQF_CK(cudaMemsetAsync(d_loop.p, 0, 2 * sizeof(int), stream));
    }
    EQF_CK(cudaStreamBeginCapture(stream, mode));
    capturing = true;
    run_step();
    if (device_loop) {
      cudaStreamCaptureStatus st;
      cudaGraph_t cg = nullptr;
      EQF_COND_CK(cudaStreamGetCaptureInfo(stream, &st, nullptr, &cg, nullptr, nullptr, nullptr));
      EQF_COND_CK(cudaGraphConditionalHandleCreate(&h, cg, 0, 0));
      k_sweep_loop<<<1, 1, 0, stream>>>(h, d_fail.p, d_loop.p, 1, kMaxExtraSweeps);
      EQF_COND_CK(cudaGetLastError());
      const cudaGraphNode_t* deps = nullptr;
      size_t nd = 0;
      EQF_COND_CK(cudaStreamGetCaptureInfo(stream, &st, nullptr, nullptr, &deps, nullptr, &nd));
      leaf.assign(deps, deps + nd);
    }
    capturing = false;
    EQF_CK(cudaStreamEndCapture(stream, &gr));
    if (device_loop) {
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t node = nullptr;
      EQF_COND_CK(cudaGraphAddNode(&node, gr, leaf.data(), nullptr, leaf.size(), &cp));
      EQF_COND_CK(cudaStreamBeginCaptureToGraph(stream, cp.conditional.phGraph_out[0], nullptr,
                                                nullptr, 0, mode));
      capturing = true;
      work->enqueue_sweep(stream, false, std::min(kExtraSweepIters, opts.max_iters), true);
      work->enqueue_check(stream, false);
      k_sweep_loop<<<1, 1, 0, stream>>>(h, d_fail.p, d_loop.p, 0, kMaxExtraSweeps);
      EQF_COND_CK(cudaGetLastError());
      cudaGraph_t body = nullptr;
      capturing = false;
      EQF_COND_CK(cudaStreamEndCapture(stream, &body));
    }
    if (gx) {
      // an out-of-date step of this parity: a plain graph is updated in place when the
      // topology allows; one with the conditional loop is replaced (its kernels name the
      // loop's handle, which belongs to the graph it was created on)
      cudaGraphExecUpdateResultInfo info{};
      if (!device_loop && cudaGraphExecUpdate(gx, gr, &info) == cudaSuccess) {
        cudaGraphDestroy(gr);
        return;
      }
      cudaGetLastError();
      retire_graph_exec(gx);
      gx = nullptr;
    }
    EQF_COND_CK(cudaGraphInstantiate(&gx, gr, 0));
    cudaGraphDestroy(gr);
  } catch (...) {
    abandon();
    throw;
  }
}

void Batch::step(int n) {
  ensure_ops();
  if (cells_dirty) rebuild_cells();
  for (int k = 0; k < n; ++k) {
    bool looped = false;  // the added sweeps ran inside the step's graph
    if (opts.use_graph && !prof.on) {
      cudaGraphExec_t& gx = graph[cur];
      if (!gx || graph_stale[cur]) {
        bool done = false;
        if (opts.adaptive && device_loop_ok) {
          try {
            capture_step(gx, true);
            done = true;
          } catch (const Error&) {
            if (!cond_failed) throw;
            // no conditional nodes here: the host adds the sweeps (below)
            device_loop_ok = false;
            drop_graphs();
          }
        }
        if (!done) capture_step(gx, false);
        graph_stale[cur] = false;
      }
      EQF_CK(cudaGraphLaunch(gx, stream));
      looped = opts.adaptive && device_loop_ok;
    } else {
      run_step();
    }
    if (opts.adaptive && !looped) {
      // add sweeps for traps that missed rtol (the others are skipped by ir_done)
      int f = 0;
      for (int extra = 0; extra < kMaxExtraSweeps; ++extra) {
        EQF_CK(cudaMemcpyAsync(&f, d_fail.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
        sync();
        if (f == 0) break;
        reset_fail();
        work->enqueue_sweep(stream, false, std::min(kExtraSweepIters, opts.max_iters), true);
        work->enqueue_check(stream, false);
      }
      if (f != 0) {
        reset_fail();
        enqueue_channels();
        enqueue_wells();
        cur = 1 - cur;
        bal_prev_ok = false;
        throw Error(EQF_ERR_NOT_CONVERGED, "trap(s) missed rtol after extra refinement sweeps");
      }
    }
    enqueue_balance();  // before the channels move the wall values of the next step
    enqueue_channels();
    enqueue_wells();
    cur = 1 - cur;
    ++steps_done;
  }
}

// Slot reuse: trap t becomes a new trap p whose grid fits t's slot at every level
// (the depth and the Krylov method of the batch stay; check_replacement first).  Its field, increments, solver
// state, cells, couplings, walls (p.walls, no values), tensor and well start afresh;
// the other traps keep their nodes and state.  Operators, tile lists and the cell
// index are rebuilt, and the captured steps recaptured, before the next step.
void Batch::check_replacement(int t, const eqf_trap_params& p) const {
  if (!(p.nx >= 1 && p.ny >= 1 && p.width > 0 && p.height > 0 && p.dt > 0 && p.D >= 0 &&
        p.decay >= 0 && (p.walls & ~15u) == 0))
    throw Error(EQF_ERR_INVALID, "invalid trap parameters");
  if (trap_levels(p) > nlev)
    throw Error(EQF_ERR_INVALID, "trap needs more multigrid levels than its batch has");
  const bool adv = p.adv_u != 0.0 && p.adv_len > 0.0;
  if (adv && !use_bicgstab)
    throw Error(EQF_ERR_INVALID, "advective trap in a batch that solves with CG");
  for (const auto& rs : rod_sets)
    for (int l : rs->layers)
      if (l == t) throw Error(EQF_ERR_INVALID, "trap carries rod cells");
  for (const auto& c : chans)
    if (c->trap == t) throw Error(EQF_ERR_INVALID, "trap carries a flow channel");
  {  // the grid of every level must fit the slot
    std::vector<long long> sp(nlev);
    eqf_internal_trap_spans(p, nlev, sp.data());
    for (int l = 0; l < nlev; ++l)
      if (sp[l] > slot_span[l][t]) throw Error(EQF_ERR_INVALID, "trap grid larger than its slot");
  }
}

// The slot's vectors at every level and its per-trap state, to zero before anything
// reads the slot under a new layout (pad columns and rows must hold zeros).
void Batch::slot_ranges(int t, std::vector<ZeroRange>& out) {
  for (int l = 0; l < nlev; ++l) work->slot_ranges(l, L[l].geom[t].off, slot_span[l][t], out);
  const long long off = L[0].geom[t].off, n0 = slot_span[0][t];
  auto add = [&](void* p, long long bytes) { out.push_back({static_cast<char*>(p), bytes}); };
  for (int q = 0; q < 2; ++q) {
    add(U[q].p + off, n0 * (long long)sizeof(double));
    add(Dd[q].p + off, n0 * (long long)sizeof(float));
  }
  add(F.p + off, n0 * (long long)sizeof(double));
  add(b64.p + off, n0 * (long long)sizeof(double));
  add(dstate.p + t, (long long)sizeof(CgState));
  add(d_frozen.p + t, (long long)sizeof(int));
  add(d_well_c.p + t, (long long)sizeof(double));
  add(d_well_under.p + t, (long long)sizeof(long long));
}

void Batch::zero_ranges(const std::vector<ZeroRange>& r) {
  if (r.empty()) return;
  // staged in page-locked memory: the copy does not wait for the stream; the caller
  // syncs before the staging is reused (build_levels does)
  zero_stage.grow(r.size());
  std::copy(r.begin(), r.end(), zero_stage.p);
  grow(d_zero, r.size());
  EQF_CK(cudaMemcpyAsync(d_zero.p, zero_stage.p, r.size() * sizeof(ZeroRange),
                         cudaMemcpyHostToDevice, stream));
  for (size_t k = 0; k < r.size(); k += 65535) {  // grid y limit
    const unsigned ny = (unsigned)std::min<size_t>(65535, r.size() - k);
    k_zero_ranges<<<dim3(8, ny), 256, 0, stream>>>(d_zero.p + k);
    EQF_LAUNCH_CHECK();
  }
}

void Batch::replace_trap(int t, const eqf_trap_params& p) {
  params[t] = p;
  eqf_boundaries& bc = bcs[t];
  std::memset(&bc, 0, sizeof(bc));
  const unsigned bits[4] = {WALL_BOTTOM, WALL_TOP, WALL_LEFT, WALL_RIGHT};
  for (int w = 0; w < 4; ++w)
    bc.wall[w].kind = (p.walls & bits[w]) ? EQF_BC_DIRICHLET : EQF_BC_NEUMANN;
  bc.channel_substeps = 1;
  bc.well_scaling = 1.0;
  tensor[t].clear();
  auto drop = [t](auto& m) {
    for (auto it = m.begin(); it != m.end();) it = it->first.second == t ? m.erase(it) : std::next(it);
  };
  drop(htens);
  drop(dtens);
  drop(dtensf);
  drop(dcoef_f);
  drop(dcoef_d);
  drop(drowc_f);
  drop(drowc_d);
  well[t] = WellParams{};
  pull_cell_s();  // the other traps' rates as the device holds them
  cell_xy[t].clear();
  cell_s[t].clear();
  couplings.erase(std::remove_if(couplings.begin(), couplings.end(),
                                 [t](const Coupling& c) { return c.t1 == t || c.t2 == t; }),
                  couplings.end());
  cells_dirty = true;
  ops_dirty = true;
  if ((int)trap_dirty.size() == ntraps) trap_dirty[t] = 1;
  bal_prev_ok = bal_load_ok = false;
  drop_graphs();
}

// ---------------------------------------------------------------------------
void Batch::scan(int n, const int* in, int* out) {
  if (n <= 0) return;
  const int nb = (n + kScanTile - 1) / kScanTile;
  grow(scan_sums, nb);  // stream-ordered reuse; callers sync before reading on the host
  k_scan_sums<<<nb, kScanBlock, 0, stream>>>(n, in, scan_sums.p);
  EQF_LAUNCH_CHECK();
  k_scan_top<<<1, kScanBlock, 0, stream>>>(nb, scan_sums.p);
  EQF_LAUNCH_CHECK();
  k_scan_apply<<<nb, kScanBlock, 0, stream>>>(n, in, scan_sums.p, out);
  EQF_LAUNCH_CHECK();
}

// Deterministic sort of entries by node: counting sort, then each bucket ordered
// by entry index; segments = buckets.  d_counts holds per-node counts on entry.
void Batch::build_segments(int nent, int* d_node, int* d_counts, DevBuf<int>& perm,
                           DevBuf<int>& seg_start, int& nseg_out, const double* xy,
                           const double* s, const double* val) {
  const long long N = L[0].nodes;
  DevBuf<int> start, cursor, head, head_scan;
  start.alloc(N + 1);
  cursor.alloc(N);
  scan((int)N, d_counts, start.p);
  EQF_CK(cudaMemsetAsync(cursor.p, 0, N * sizeof(int), stream));
  perm.alloc(std::max(nent, 1));
  head.alloc(std::max(nent, 1));
  head_scan.alloc(nent + 1);
  const int bs = 256, gb = (nent + bs - 1) / bs;
  k_cells_place<<<gb, bs, 0, stream>>>(nent, d_node, start.p, cursor.p, perm.p);
  EQF_LAUNCH_CHECK();
  k_cells_heads<<<gb, bs, 0, stream>>>(nent, d_node, start.p, perm.p, head.p);
  EQF_LAUNCH_CHECK();
  scan(nent, head.p, head_scan.p);
  int ns = 0;
  EQF_CK(cudaMemcpyAsync(&ns, head_scan.p + nent, sizeof(int), cudaMemcpyDeviceToHost, stream));
  sync();
  seg_start.alloc(ns + 1);
  k_cells_segments<<<gb, bs, 0, stream>>>(nent, head.p, head_scan.p, seg_start.p, ns);
  EQF_LAUNCH_CHECK();
  k_seg_sort<<<(ns + 255) / 256, 256, 0, stream>>>(ns, seg_start.p, perm.p, xy, s, val);
  EQF_LAUNCH_CHECK();
  sync();
  nseg_out = ns;
}

// Brings the host copies of the per-cell rates up to date with d_cell_s.
void Batch::pull_cell_s() {
  if (!cell_s_stale) return;
  cell_s_stale = false;
  if (ncells == 0) return;
  std::vector<double> sv(ncells);
  EQF_CK(cudaMemcpyAsync(sv.data(), d_cell_s.p, ncells * sizeof(double), cudaMemcpyDeviceToHost,
                         stream));
  sync();
  for (int t = 0; t < ntraps; ++t)
    std::copy(sv.begin() + cell_first[t], sv.begin() + cell_first[t + 1], cell_s[t].begin());
}

void Batch::rebuild_cells() {
  pull_cell_s();
  cells_dirty = false;
  ncp = 0;
  drop_graphs();
  cell_first.assign(ntraps + 1, 0);
  for (int t = 0; t < ntraps; ++t) cell_first[t + 1] = cell_first[t] + (int)cell_s[t].size();
  ncells = cell_first[ntraps];
  bal_load_ok = false;
  EQF_CK(cudaMemsetAsync(F.p, 0, L[0].nodes * sizeof(double), stream));
  if (ncells == 0) {
    nseg = 0;
    if (walls_active) EQF_CK(cudaMemsetAsync(d_fbase.p, 0, d_fbase.n * sizeof(double), stream));
    sync();
    return;
  }
  std::vector<double> xy(2 * (size_t)ncells), sv(ncells);
  std::vector<int> trap(ncells);
  std::vector<CellGeom> cg(ntraps);
  std::vector<double> scale(ntraps);
  for (int t = 0; t < ntraps; ++t) {
    const LevelGeom& g = L[0].geom[t];
    cg[t] = CellGeom{g.off, g.nx, g.ny, g.P, g.hx, g.hy};
    scale[t] = params[t].dt;
    std::copy(cell_xy[t].begin(), cell_xy[t].end(), xy.begin() + 2 * (size_t)cell_first[t]);
    std::copy(cell_s[t].begin(), cell_s[t].end(), sv.begin() + cell_first[t]);
    std::fill(trap.begin() + cell_first[t], trap.begin() + cell_first[t + 1], t);
  }
  d_cell_xy.alloc(xy.size());
  d_cell_xy.upload(xy.data(), xy.size(), stream);
  d_cell_s.alloc(ncells);
  d_cell_s.upload(sv.data(), ncells, stream);
  d_cell_trap.alloc(ncells);
  d_cell_trap.upload(trap.data(), ncells, stream);
  dcg.alloc(ntraps);
  dcg.upload(cg.data(), ntraps, stream);
  d_scale.alloc(ntraps);
  d_scale.upload(scale.data(), ntraps, stream);
  const int nent = 3 * ncells;
  d_ent_node.alloc(nent);
  d_ent_w.alloc(nent);
  d_ent_val.alloc(nent);
  DevBuf<int> counts;
  counts.alloc(L[0].nodes);
  EQF_CK(cudaMemsetAsync(counts.p, 0, L[0].nodes * sizeof(int), stream));
  k_cells_locate<<<(ncells + 255) / 256, 256, 0, stream>>>(ncells, dcg.p, d_cell_trap.p,
                                                           d_cell_xy.p, d_ent_node.p, d_ent_w.p,
                                                           counts.p);
  EQF_LAUNCH_CHECK();
  build_segments(nent, d_ent_node.p, counts.p, d_perm, d_seg_start, nseg, d_cell_xy.p,
                 d_cell_s.p, nullptr);
  // coupled cells: index maps, sender flags, production rates, laws
  ncp = 0;
  std::vector<int> i1, i2, snd, law_of;
  std::vector<double> prod;
  std::vector<CouplingLaw> laws;
  for (size_t c = 0; c < couplings.size(); ++c) {
    const Coupling& cp = couplings[c];
    const int n = (int)cell_s[cp.t1].size();
    if (n != (int)cell_s[cp.t2].size() || n != (int)cp.sender.size())
      throw Error(EQF_ERR_INVALID, "coupled traps' cells changed after eqf_couple_species");
    laws.push_back(cp.law);
    for (int i = 0; i < n; ++i) {
      i1.push_back(cell_first[cp.t1] + i);
      i2.push_back(cell_first[cp.t2] + i);
      snd.push_back(cp.sender[i]);
      prod.push_back(cell_s[cp.t1][i]);
      law_of.push_back((int)c);
    }
  }
  ncp = (int)i1.size();
  if (ncp > 0) {
    d_cp_i1.alloc(ncp);
    d_cp_i1.upload(i1.data(), ncp, stream);
    d_cp_i2.alloc(ncp);
    d_cp_i2.upload(i2.data(), ncp, stream);
    d_cp_sender.alloc(ncp);
    d_cp_sender.upload(snd.data(), ncp, stream);
    d_cp_law.alloc(ncp);
    d_cp_law.upload(law_of.data(), ncp, stream);
    d_cp_prod.alloc(ncp);
    d_cp_prod.upload(prod.data(), ncp, stream);
    d_cp_laws.alloc(laws.size());
    d_cp_laws.upload(laws.data(), laws.size(), stream);
    d_cp_c.alloc(ncells);
  }
  // captured steps hold pointers to the cell arrays just reallocated
  drop_graphs();
  refresh_load();
  sync();
}

// F = dt * sum_i s_i phi(x_i) from the current rates (segments fixed)
void Batch::refresh_load() {
  bal_load_ok = false;
  if (ncells == 0) return;
  const dim3 rim_grid((rim_max + 255) / 256, (unsigned)hwalls.size());
  if (walls_active)  // the rim takes the point cells' load alone, then is kept apart
    k_wall_rim<0><<<rim_grid, 256, 0, stream>>>(d_walls.p, L[0].dgeom.p, F.p, d_fbase.p);
  // rates changed: restore the canonical order of every node's contributions
  k_seg_sort<<<(nseg + 255) / 256, 256, 0, stream>>>(nseg, d_seg_start.p, d_perm.p, d_cell_xy.p,
                                                     d_cell_s.p, nullptr);
  EQF_LAUNCH_CHECK();
  k_cells_values<<<(ncells + 255) / 256, 256, 0, stream>>>(ncells, d_ent_w.p, d_cell_s.p,
                                                           d_scale.p, d_cell_trap.p, d_ent_val.p);
  EQF_LAUNCH_CHECK();
  k_seg_sum<false><<<(nseg + 255) / 256, 256, 0, stream>>>(nseg, d_seg_start.p, d_perm.p,
                                                           d_ent_node.p, d_ent_val.p, F.p);
  EQF_LAUNCH_CHECK();
  if (walls_active) {
    k_wall_rim<1><<<rim_grid, 256, 0, stream>>>(d_walls.p, L[0].dgeom.p, F.p, d_fbase.p);
    EQF_LAUNCH_CHECK();
  }
}

// ---------------------------------------------------------------------------
// Readouts: boundary flux and total mass of one trap (FP64, tile partials).
__global__ void k_trap_reduce(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                              int first_tile, const double* __restrict__ u, int what,
                              double* __restrict__ part) {
  const Tile tile = tiles[first_tile + blockIdx.x];
  const LevelGeom g = G[tile.geom];
  const double* us = u + g.off;
  const int P = g.P;
  double acc = 0.0;
  for (NodeWalk w(g, tile.k0); w.k < tile.k1; w.next()) {
    const int k = w.k, i = w.i, j = w.j;
    if (j > g.nx) continue;  // pad column
    if (what == 0) {  // 1^T M u
      const Sten<double> m = mass_stencil<double>(g, i, j);
      acc += (m.c + m.e + m.w + m.n + m.s + m.ne + m.sw) * us[k];
    } else {  // -int grad u . n ds, each boundary edge owned by one node
      if (i == 0 && j < g.nx) acc += (us[k + P + 1] - us[k + 1]) / g.hy * g.hx;
      if (i == g.ny && j < g.nx) acc += -(us[k] - us[k - P]) / g.hy * g.hx;
      if (j == 0 && i < g.ny) acc += (us[k + P + 1] - us[k + P]) / g.hx * g.hy;
      if (j == g.nx && i < g.ny) acc += -(us[k] - us[k - 1]) / g.hx * g.hy;
    }
  }
  const double t = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

}  // namespace eqf

// ===========================================================================
// C ABI
// ===========================================================================
using eqf::Batch;
using eqf::Error;

struct eqf_batch {
  std::unique_ptr<Batch> impl;
  std::string err;
};

static thread_local std::string g_create_err;

template <class F>
static int guarded(eqf_batch* b, F&& f) {
  eqf::AllocStream scope(b && b->impl ? b->impl->stream : nullptr);
  try {
    f();
    return EQF_OK;
  } catch (const Error& e) {
    if (b) b->err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    if (b) b->err = "host allocation failed";
    return EQF_ERR_NOMEM;
  } catch (const std::exception& e) {
    if (b) b->err = e.what();
    return EQF_ERR_INVALID;
  }
}

#define EQF_REQUIRE(cond, msg) \
  do {                         \
    if (!(cond)) throw Error(EQF_ERR_INVALID, msg); \
  } while (0)

extern "C" {

int eqf_default_opts(int32_t precision, eqf_solver_opts* o) {
  if (!o) return EQF_ERR_INVALID;
  std::memset(o, 0, sizeof(*o));
  o->precision = precision;
  o->cheb_pre = 2;
  o->cheb_post = 2;
  o->cheb_coarse = 12;
  o->cheb_ratio = 5.0;
  o->use_graph = 0;
  o->adaptive = 1;
  o->fuse_levels = 1;
  if (precision == EQF_PREC_FP32_IR) {
    // 4 inner iterations a sweep and 16 coarsest-level steps: 9-10 % faster steps than
    // 6 and 12 on the 512-trap workload at the same sweeps a step (the outer FP64 test
    // sets the accuracy either way).  rtol 3e-8 keeps the field within ~1e-7 of the
    // FP64 solution (relL2 about three times rtol on the uneven traps over 200 steps),
    // a tenfold margin under the form's 1e-6 accuracy target; 1e-8 costs 8 % more per
    // step, 1e-7 saves a further 10 % at ~3e-7
    o->rtol = 3e-8;
    o->max_sweeps = 2;
    o->max_iters = 4;
    o->inner_tol = 1e-5;
    o->cheb_coarse = 16;
  } else if (precision == EQF_PREC_FP64) {
    o->rtol = 1e-10;
    o->max_sweeps = 1;
    o->max_iters = 12;
    o->inner_tol = 0.0;
  } else {
    return EQF_ERR_INVALID;
  }
  return EQF_OK;
}

static int create_impl(int32_t n_traps, const eqf_trap_params* traps,
                       const eqf_solver_opts* opts, const int* tiles, const int* cols,
                       eqf_batch** out) {
  if (!out) return EQF_ERR_INVALID;
  *out = nullptr;
  auto* h = new (std::nothrow) eqf_batch();
  if (!h) return EQF_ERR_NOMEM;
  const int rc = guarded(h, [&] {
    EQF_REQUIRE(n_traps > 0 && traps, "need at least one trap");
    eqf_solver_opts o;
    if (opts)
      o = *opts;
    else
      eqf_default_opts(EQF_PREC_FP64, &o);
    EQF_REQUIRE(o.precision == EQF_PREC_FP64 || o.precision == EQF_PREC_FP32_IR,
                "unknown precision");
    EQF_REQUIRE(o.max_sweeps >= 1 && o.max_iters >= 1 && o.cheb_post >= 1 && o.cheb_pre >= 1 &&
                    o.cheb_coarse >= 1 && o.cheb_ratio > 1.0 && o.rtol > 0.0,
                "invalid solver options");
    EQF_REQUIRE(o.cheb_pre <= eqf::kMaxChebSteps && o.cheb_post <= eqf::kMaxChebSteps &&
                    o.cheb_coarse <= eqf::kMaxChebSteps,
                "Chebyshev degrees above 16");
    EQF_REQUIRE(o.tile_nodes >= 0 && o.tile_nodes <= 32768, "tile_nodes outside [0, 32768]");
    auto width_ok = [](int c) { return c == 0 || (c >= 16 && c <= 512 && c % 4 == 0); };
    EQF_REQUIRE(width_ok(o.tile_cols), "tile_cols not 0 or a multiple of 4 in [16, 512]");
    if (cols)
      for (int t = 0; t < n_traps; ++t)
        EQF_REQUIRE(width_ok(cols[t]), "tile width not 0 or a multiple of 4 in [16, 512]");
    EQF_REQUIRE(o.krylov >= EQF_KRYLOV_AUTO && o.krylov <= EQF_KRYLOV_BICGSTAB,
                "unknown Krylov method");
    for (int t = 0; t < n_traps; ++t) {
      const auto& p = traps[t];
      EQF_REQUIRE(p.nx >= 1 && p.ny >= 1 && p.width > 0 && p.height > 0 && p.dt > 0 &&
                      p.D >= 0 && p.decay >= 0 && (p.walls & ~15u) == 0,
                  "invalid trap parameters (trap " + std::to_string(t) + ")");
    }
    if (tiles)
      for (int t = 0; t < n_traps; ++t)
        EQF_REQUIRE(tiles[t] >= 0 && tiles[t] <= 32768, "tile target outside [0, 32768]");
    h->impl.reset(new Batch(n_traps, traps, o, tiles, cols));
  });
  if (rc != EQF_OK) {
    g_create_err = h->err;
    delete h;
    return rc;
  }
  *out = h;
  return EQF_OK;
}

int eqf_create(int32_t n_traps, const eqf_trap_params* traps, const eqf_solver_opts* opts,
               eqf_batch** out) {
  return create_impl(n_traps, traps, opts, nullptr, nullptr, out);
}

// Bucket of a trap in a tuning table: the first whose max_nodes holds it (the last
// bucket takes everything larger).
static int tune_bucket(const eqf_tune_table& tb, long long nodes) {
  for (int i = 0; i < tb.n; ++i)
    if (nodes <= tb.b[i].max_nodes) return i;
  return tb.n - 1;
}

int eqf_create_tuned(int32_t n_traps, const eqf_trap_params* traps, const eqf_solver_opts* opts,
                     const eqf_tune_table* table, eqf_batch** out) {
  if (!out || !traps || n_traps < 1) return EQF_ERR_INVALID;
  if (!table || table->n < 1 || table->n > EQF_TUNE_MAX_BUCKETS)
    return create_impl(n_traps, traps, opts, nullptr, nullptr, out);
  eqf_solver_opts o;
  if (opts)
    o = *opts;
  else
    eqf_default_opts(EQF_PREC_FP64, &o);
  // tile target per trap from its bucket; smoother degrees and Krylov schedule from
  // the bucket that holds most of the batch's nodes
  std::vector<int> tiles(n_traps), cols(n_traps);
  std::vector<long long> mass(table->n, 0);
  for (int t = 0; t < n_traps; ++t) {
    const long long nodes = (long long)(traps[t].nx + 1) * (traps[t].ny + 1);
    const int k = tune_bucket(*table, nodes);
    tiles[t] = table->b[k].tile_nodes;
    cols[t] = table->b[k].tile_cols;
    mass[k] += nodes;
  }
  const int kb = (int)(std::max_element(mass.begin(), mass.end()) - mass.begin());
  if (table->b[kb].cheb_pre > 0) o.cheb_pre = table->b[kb].cheb_pre;
  if (table->b[kb].cheb_post > 0) o.cheb_post = table->b[kb].cheb_post;
  if (table->b[kb].max_iters > 0) o.max_iters = table->b[kb].max_iters;
  if (table->b[kb].max_sweeps > 0) o.max_sweeps = table->b[kb].max_sweeps;
  return create_impl(n_traps, traps, &o, tiles.data(), cols.data(), out);
}

int eqf_destroy(eqf_batch* b) {
  if (!b) return EQF_ERR_INVALID;
  delete b;
  return EQF_OK;
}

const char* eqf_last_error(const eqf_batch* b) {
  return b ? b->err.c_str() : g_create_err.c_str();
}

#define EQF_TRAP_CHECK(b, trap)                                                     \
  EQF_REQUIRE((trap) >= 0 && (trap) < (b)->impl->ntraps, "trap index out of range")

int eqf_trap_info(const eqf_batch* b, int32_t trap, eqf_trap_params* out) {
  if (!b || !out || trap < 0 || trap >= b->impl->ntraps) return EQF_ERR_INVALID;
  *out = b->impl->params[trap];
  return EQF_OK;
}

int eqf_num_nodes(const eqf_batch* b, int32_t trap, int64_t* n) {
  if (!b || !n || trap < 0 || trap >= b->impl->ntraps) return EQF_ERR_INVALID;
  *n = b->impl->fine_nodes(trap);
  return EQF_OK;
}

int eqf_set_cells(eqf_batch* b, int32_t trap, int64_t n, const double* xy, const double* s) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(n >= 0 && (n == 0 || (xy && s)), "bad cell arrays");
    const auto& p = b->impl->params[trap];
    for (int64_t i = 0; i < n; ++i) {
      EQF_REQUIRE(std::isfinite(xy[2 * i]) && std::isfinite(xy[2 * i + 1]) && std::isfinite(s[i]),
                  "non-finite cell position or rate");
      EQF_REQUIRE(xy[2 * i] >= 0 && xy[2 * i] <= p.width && xy[2 * i + 1] >= 0 &&
                      xy[2 * i + 1] <= p.height,
                  "cell outside the trap");
    }
    b->impl->pull_cell_s();
    b->impl->cell_xy[trap].assign(xy, xy + 2 * n);
    b->impl->cell_s[trap].assign(s, s + n);
    b->impl->cells_dirty = true;
  });
}

int eqf_footprint_estimate(int32_t n_traps, const eqf_trap_params* traps,
                           const eqf_solver_opts* opts, int64_t n_cells, int64_t* bytes) {
  if (n_traps < 1 || !traps || !bytes || n_cells < 0) return EQF_ERR_INVALID;
  eqf_solver_opts o;
  if (opts)
    o = *opts;
  else
    eqf_default_opts(EQF_PREC_FP64, &o);
  for (int t = 0; t < n_traps; ++t)
    if (traps[t].nx < 1 || traps[t].ny < 1 || !(traps[t].width > 0) || !(traps[t].height > 0))
      return EQF_ERR_INVALID;
  *bytes = (int64_t)eqf::estimate_bytes(n_traps, traps, o, n_cells);
  return EQF_OK;
}

int eqf_set_active(eqf_batch* b, int32_t trap, int32_t active) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    Batch& B = *b->impl;
    const long long off = B.L[0].geom[trap].off;
    const size_t n = (size_t)B.fine_span(trap);
    if (!active) {
      // both field buffers hold the frozen field, so reads see it whatever the parity
      EQF_CK(cudaMemcpyAsync(B.U[1 - B.cur].p + off, B.U[B.cur].p + off, n * sizeof(double),
                             cudaMemcpyDeviceToDevice, B.stream));
    } else {
      // a resumed trap starts a fresh increment history for its initial guess
      for (int q = 0; q < 2; ++q)
        EQF_CK(cudaMemsetAsync(B.Dd[q].p + off, 0, n * sizeof(float), B.stream));
      EQF_CK(cudaMemsetAsync(reinterpret_cast<char*>(B.dstate.p + trap) +
                                 offsetof(eqf::CgState, gamma),
                             0, 2 * sizeof(double), B.stream));
    }
    // stream-ordered, no host memory involved: the call does not wait
    EQF_CK(cudaMemsetAsync(B.d_frozen.p + trap, active ? 0 : 1, sizeof(int), B.stream));
  });
}

int eqf_replace_traps(eqf_batch* b, int32_t n, const int32_t* traps,
                      const eqf_trap_params* p) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_REQUIRE(n >= 0 && (n == 0 || (traps && p)), "bad replacement arrays");
    Batch& B = *b->impl;
    for (int32_t k = 0; k < n; ++k) {
      EQF_TRAP_CHECK(b, traps[k]);
      for (int32_t m = 0; m < k; ++m) EQF_REQUIRE(traps[m] != traps[k], "trap listed twice");
    }
    for (int32_t k = 0; k < n; ++k) B.check_replacement(traps[k], p[k]);  // all or none
    if (n == 0) return;
    std::vector<eqf::ZeroRange> z;
    for (int32_t k = 0; k < n; ++k) B.slot_ranges(traps[k], z);
    B.zero_ranges(z);  // one launch for every slot's vectors and state
    for (int32_t k = 0; k < n; ++k) B.replace_trap(traps[k], p[k]);
    B.ensure_ops();  // the new geometry, for readouts before the next step
    B.sync();        // (the zeroing's page-locked staging may be reused next call)
  });
}

int eqf_replace_trap(eqf_batch* b, int32_t trap, const eqf_trap_params* p) {
  return eqf_replace_traps(b, 1, &trap, p);
}

int eqf_slot_fits(const eqf_batch* b, int32_t trap, const eqf_trap_params* p, int32_t* fits) {
  if (!b || !p || !fits || trap < 0 || trap >= b->impl->ntraps) return EQF_ERR_INVALID;
  try {
    b->impl->check_replacement(trap, *p);
    *fits = 1;
  } catch (const Error&) {
    *fits = 0;
  }
  return EQF_OK;
}

int eqf_poll(eqf_batch* b, int32_t* idle) {
  if (!b || !idle) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    const cudaError_t q = cudaStreamQuery(B.stream);
    if (q == cudaErrorNotReady) {
      *idle = 0;
      return;
    }
    EQF_CK(q);
    *idle = 1;
    B.check_fail();
  });
}

int eqf_read_cells_async(eqf_batch* b, int32_t trap, int64_t n, double* c) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    Batch& B = *b->impl;
    if (B.cells_dirty) B.rebuild_cells();
    EQF_REQUIRE(n == (int64_t)B.cell_s[trap].size() && (n == 0 || c), "cell count mismatch");
    if (n == 0) return;
    // stream-ordered (re)allocation: no wait for the steps queued before it
    if (B.d_cells_out.n < (size_t)B.ncells) B.d_cells_out.alloc(B.ncells);
    const int c0 = B.cell_first[trap];
    eqf::k_cells_gather<<<(int)((n + 255) / 256), 256, 0, B.stream>>>(
        (int)n, B.d_ent_node.p + 3 * (size_t)c0, B.d_ent_w.p + 3 * (size_t)c0, B.u_cur(),
        B.d_cells_out.p + c0);
    EQF_LAUNCH_CHECK();
    EQF_CK(cudaMemcpyAsync(c, B.d_cells_out.p + c0, n * sizeof(double), cudaMemcpyDeviceToHost,
                           B.stream));
  });
}

int eqf_fail_count_async(eqf_batch* b, int32_t* count) {
  if (!b || !count) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    EQF_CK(cudaMemcpyAsync(count, B.d_fail.p, sizeof(int), cudaMemcpyDeviceToHost, B.stream));
  });
}

int eqf_read_nodal_async(eqf_batch* b, int32_t trap, double* c) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(c != nullptr, "null output");
    Batch& B = *b->impl;
    B.copy_field_to_host(c, B.u_cur() + B.L[0].geom[trap].off, trap, B.stream);
  });
}

int eqf_couple_species(eqf_batch* b, int32_t trap1, int32_t trap2, const int32_t* sender,
                       double vmax, double K, double uptake) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap1);
    EQF_TRAP_CHECK(b, trap2);
    Batch& B = *b->impl;
    EQF_REQUIRE(trap1 != trap2, "a species cannot be coupled to itself");
    const auto &p1 = B.params[trap1], &p2 = B.params[trap2];
    EQF_REQUIRE(p1.nx == p2.nx && p1.ny == p2.ny && p1.width == p2.width &&
                    p1.height == p2.height,
                "coupled species must share the trap mesh");
    for (const auto& c : B.couplings)
      EQF_REQUIRE(c.t1 != trap1 && c.t2 != trap1 && c.t1 != trap2 && c.t2 != trap2,
                  "trap already coupled");
    EQF_REQUIRE(std::isfinite(vmax) && std::isfinite(K) && K > 0 && std::isfinite(uptake) &&
                    uptake >= 0,
                "bad coupling law");
    const size_t n = B.cell_s[trap1].size();
    EQF_REQUIRE(n == 0 || sender, "null sender flags");
    B.pull_cell_s();
    Batch::Coupling c{trap1, trap2, eqf::CouplingLaw{vmax, K, uptake}, {}};
    c.sender.assign(sender, sender + n);
    B.cell_xy[trap2] = B.cell_xy[trap1];
    B.cell_s[trap2].assign(n, 0.0);
    B.couplings.push_back(std::move(c));
    B.cells_dirty = true;
  });
}

int eqf_set_cell_rates(eqf_batch* b, int32_t trap, int64_t n, const double* s) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    Batch& B = *b->impl;
    EQF_REQUIRE(n == (int64_t)B.cell_s[trap].size() && (n == 0 || s), "rate count mismatch");
    for (int64_t i = 0; i < n; ++i) EQF_REQUIRE(std::isfinite(s[i]), "non-finite cell rate");
    B.pull_cell_s();
    B.cell_s[trap].assign(s, s + n);
    if (B.cells_dirty) return;  // the rebuild will pick the rates up
    if (n == 0) return;
    EQF_CK(cudaMemcpyAsync(B.d_cell_s.p + B.cell_first[trap], s, n * sizeof(double),
                           cudaMemcpyHostToDevice, B.stream));
    B.refresh_load();
    B.sync();
  });
}

int eqf_set_nodal(eqf_batch* b, int32_t trap, const double* c) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(c != nullptr, "null field");
    Batch& B = *b->impl;
    const long long off = B.L[0].geom[trap].off;
    B.bal_prev_ok = false;
    B.copy_field_to_device(B.u_cur() + off, c, trap, B.stream);
    // a new field invalidates the increment history of the initial guess
    EQF_CK(cudaMemsetAsync(B.Dd[B.cur].p + off, 0, B.fine_span(trap) * sizeof(float), B.stream));
    EQF_CK(cudaMemsetAsync(reinterpret_cast<char*>(B.dstate.p + trap) +
                               offsetof(eqf::CgState, gamma),
                           0, 2 * sizeof(double), B.stream));
    B.sync();
  });
}

int eqf_add_nodal(eqf_batch* b, int32_t trap, int64_t n, const int64_t* node,
                  const double* delta) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(n >= 0 && (n == 0 || (node && delta)), "bad nodal arrays");
    if (n == 0) return;
    Batch& B = *b->impl;
    B.bal_prev_ok = false;
    const int64_t nn = B.fine_nodes(trap);
    for (int64_t i = 0; i < n; ++i)
      EQF_REQUIRE(node[i] >= 0 && node[i] < nn && std::isfinite(delta[i]),
                  "node index out of range or non-finite increment");
    eqf::DevBuf<long long> dn;
    eqf::DevBuf<double> dv;
    eqf::DevBuf<int> ent, counts, perm, seg;
    dn.alloc(n);
    dn.upload(reinterpret_cast<const long long*>(node), n, B.stream);
    dv.alloc(n);
    dv.upload(delta, n, B.stream);
    ent.alloc(n);
    counts.alloc(B.L[0].nodes);
    EQF_CK(cudaMemsetAsync(counts.p, 0, B.L[0].nodes * sizeof(int), B.stream));
    const eqf::LevelGeom& g0 = B.L[0].geom[trap];
    eqf::k_nodal_entries<<<(int)((n + 255) / 256), 256, 0, B.stream>>>(
        (int)n, g0.off, g0.nx + 1, g0.P, dn.p, ent.p, counts.p);
    EQF_LAUNCH_CHECK();
    int ns = 0;
    B.build_segments((int)n, ent.p, counts.p, perm, seg, ns, nullptr, nullptr, dv.p);
    eqf::k_seg_sum<true><<<(ns + 255) / 256, 256, 0, B.stream>>>(ns, seg.p, perm.p, ent.p, dv.p,
                                                                  B.u_cur());
    EQF_LAUNCH_CHECK();
    B.sync();
  });
}

int eqf_step(eqf_batch* b, int32_t n_steps) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_REQUIRE(n_steps >= 0, "negative step count");
    b->impl->step(n_steps);
  });
}

int eqf_read_nodal(eqf_batch* b, int32_t trap, double* c) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(c != nullptr, "null output");
    Batch& B = *b->impl;
    B.copy_field_to_host(c, B.u_cur() + B.L[0].geom[trap].off, trap, B.stream);
    B.sync();
    B.check_fail();
  });
}

namespace {
// dof_from_vertex must be a permutation of 0 .. n-1
void check_dof_map(const int32_t* dof, long long n) {
  EQF_REQUIRE(dof != nullptr, "null DOF map");
  std::vector<unsigned char> seen((size_t)n, 0);
  for (long long v = 0; v < n; ++v) {
    const int32_t d = dof[v];
    EQF_REQUIRE(d >= 0 && d < n && !seen[(size_t)d], "the DOF map is not a permutation");
    seen[(size_t)d] = 1;
  }
}
}  // namespace

int eqf_read_nodal_dof(eqf_batch* b, int32_t trap, const int32_t* dof_from_vertex, double* c) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(c != nullptr, "null output");
    Batch& B = *b->impl;
    const long long n = B.fine_nodes(trap);
    check_dof_map(dof_from_vertex, n);
    std::vector<double> grid((size_t)n);
    B.copy_field_to_host(grid.data(), B.u_cur() + B.L[0].geom[trap].off, trap, B.stream);
    B.sync();
    B.check_fail();
    for (long long v = 0; v < n; ++v) c[dof_from_vertex[v]] = grid[(size_t)v];
  });
}

int eqf_set_nodal_dof(eqf_batch* b, int32_t trap, const int32_t* dof_from_vertex,
                      const double* c) {
  if (!b) return EQF_ERR_INVALID;
  std::vector<double> grid;
  const int rc = guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(c != nullptr, "null field");
    const long long n = b->impl->fine_nodes(trap);
    check_dof_map(dof_from_vertex, n);
    grid.resize((size_t)n);
    for (long long v = 0; v < n; ++v) grid[(size_t)v] = c[dof_from_vertex[v]];
  });
  if (rc != EQF_OK) return rc;
  return eqf_set_nodal(b, trap, grid.data());
}

int eqf_read_cells(eqf_batch* b, int32_t trap, int64_t n, double* c) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    Batch& B = *b->impl;
    if (B.cells_dirty) B.rebuild_cells();
    EQF_REQUIRE(n == (int64_t)B.cell_s[trap].size() && (n == 0 || c), "cell count mismatch");
    if (n == 0) return;
    eqf::DevBuf<double> out;
    out.alloc(n);
    const int c0 = B.cell_first[trap];
    eqf::k_cells_gather<<<(int)((n + 255) / 256), 256, 0, B.stream>>>(
        (int)n, B.d_ent_node.p + 3 * (size_t)c0, B.d_ent_w.p + 3 * (size_t)c0, B.u_cur(), out.p);
    EQF_LAUNCH_CHECK();
    EQF_CK(cudaMemcpyAsync(c, out.p, n * sizeof(double), cudaMemcpyDeviceToHost, B.stream));
    B.sync();
    B.check_fail();
  });
}

static double trap_reduce(Batch& B, int trap, int what) {
  const eqf::TileRange tr = B.range[trap];
  eqf::DevBuf<double> part;
  part.alloc(tr.count);
  eqf::k_trap_reduce<<<tr.count, eqf::kThreads, 0, B.stream>>>(
      B.L[0].dgeom.p, B.L[0].dtiles.p, tr.first, B.u_cur(), what, part.p);
  EQF_LAUNCH_CHECK();
  std::vector<double> h(tr.count);
  EQF_CK(cudaMemcpyAsync(h.data(), part.p, tr.count * sizeof(double), cudaMemcpyDeviceToHost,
                         B.stream));
  B.sync();
  double s = 0.0;
  for (double v : h) s += v;
  return s;
}

int eqf_boundary_flux(eqf_batch* b, int32_t trap, double* flux) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(flux != nullptr, "null output");
    Batch& B = *b->impl;
    *flux = B.params[trap].D * B.params[trap].dt * trap_reduce(B, trap, 1);
  });
}

int eqf_total_mass(eqf_batch* b, int32_t trap, double* mass) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(mass != nullptr, "null output");
    *mass = trap_reduce(*b->impl, trap, 0);
  });
}

int eqf_mass_balance(eqf_batch* b, int32_t enable) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    EQF_REQUIRE(enable == 0 || enable == 1, "enable must be 0 or 1");
    B.bal_on = enable != 0;
    B.bal_prev_ok = B.bal_load_ok = false;
    if (!B.bal_on) return;
    const size_t n = (size_t)B.ntraps * eqf::kBalFields;
    if (B.d_bal.n != n) B.d_bal.alloc(n);
    EQF_CK(cudaMemsetAsync(B.d_bal.p, 0, n * sizeof(double), B.stream));
    B.sync();
  });
}

int eqf_read_balance(eqf_batch* b, int32_t trap, eqf_balance* out) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(out != nullptr, "null output");
    Batch& B = *b->impl;
    EQF_REQUIRE(B.d_bal.n > 0, "the mass balance was never enabled (eqf_mass_balance)");
    double r[eqf::kBalFields];
    EQF_CK(cudaMemcpyAsync(r, B.d_bal.p + (size_t)trap * eqf::kBalFields, sizeof(r),
                           cudaMemcpyDeviceToHost, B.stream));
    B.sync();
    out->mass = r[eqf::BAL_MASS];
    out->mass_prev = r[eqf::BAL_MASS_PREV];
    out->load = r[eqf::BAL_LOAD];
    out->decay = r[eqf::BAL_DECAY];
    out->operator_loss = r[eqf::BAL_OPERATOR];
    out->wall_outflow = r[eqf::BAL_WALL];
    out->drift = r[eqf::BAL_DRIFT];
    out->drift_sum = r[eqf::BAL_DRIFT_SUM];
    out->drift_abs_sum = r[eqf::BAL_DRIFT_ABS_SUM];
    out->load_sum = r[eqf::BAL_LOAD_SUM];
    out->drift_rel_max = r[eqf::BAL_DRIFT_REL_MAX];
    out->steps = (int64_t)r[eqf::BAL_STEPS];
  });
}

int eqf_stats(eqf_batch* b, int32_t trap, int64_t* steps, int64_t* sweeps, int64_t* iters,
              double* last_rel_residual) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    Batch& B = *b->impl;
    eqf::CgState st;
    EQF_CK(cudaMemcpyAsync(&st, B.dstate.p + trap, sizeof(st), cudaMemcpyDeviceToHost, B.stream));
    B.sync();
    if (steps) *steps = B.steps_done;
    if (sweeps) *sweeps = st.sweeps;
    if (iters) *iters = st.iters;
    if (last_rel_residual) *last_rel_residual = st.bb > 0 ? std::sqrt(st.r64 / st.bb) : 0.0;
  });
}

int eqf_set_cell_rates_all(eqf_batch* b, int64_t n, const double* s) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    if (B.cells_dirty) B.rebuild_cells();
    EQF_REQUIRE(n == B.ncells && (n == 0 || s), "rate count mismatch");
    if (n == 0) return;
    EQF_CK(cudaMemcpyAsync(B.d_cell_s.p, s, n * sizeof(double), cudaMemcpyHostToDevice,
                           B.stream));
    B.refresh_load();
    B.cell_s_stale = true;  // the host copies follow on demand (pull_cell_s)
  });
}

int eqf_read_cells_all(eqf_batch* b, int64_t n, double* c) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    if (B.cells_dirty) B.rebuild_cells();
    EQF_REQUIRE(n == B.ncells && (n == 0 || c), "cell count mismatch");
    if (n == 0) return;
    if (B.d_cells_out.n < (size_t)n) B.d_cells_out.alloc(n);
    eqf::k_cells_gather<<<(int)((n + 255) / 256), 256, 0, B.stream>>>(
        (int)n, B.d_ent_node.p, B.d_ent_w.p, B.u_cur(), B.d_cells_out.p);
    EQF_LAUNCH_CHECK();
    EQF_CK(cudaMemcpyAsync(c, B.d_cells_out.p, n * sizeof(double), cudaMemcpyDeviceToHost,
                           B.stream));
    B.sync();
    B.check_fail();
  });
}

// Wall conditions and flow channels (eqfield.h: eqf_set_boundaries).
int eqf_set_boundaries(eqf_batch* b, int32_t trap, const eqf_boundaries* bc) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(bc != nullptr, "null boundaries");
    Batch& B = *b->impl;
    const eqf_trap_params& p = B.params[trap];
    unsigned walls = 0;
    bool channel = false, active = false;
    const unsigned bits[4] = {eqf::WALL_BOTTOM, eqf::WALL_TOP, eqf::WALL_LEFT, eqf::WALL_RIGHT};
    for (int w = 0; w < 4; ++w) {
      const eqf_wall& wl = bc->wall[w];
      EQF_REQUIRE(wl.kind >= EQF_BC_NEUMANN && wl.kind <= EQF_BC_WELL, "bad wall kind");
      EQF_REQUIRE(std::isfinite(wl.value) && std::isfinite(wl.rate), "non-finite wall value");
      EQF_REQUIRE(wl.kind != EQF_BC_ROBIN || wl.rate >= 0.0, "negative Robin rate");
      EQF_REQUIRE(wl.kind != EQF_BC_CHANNEL || w <= EQF_SIDE_TOP,
                  "channels border the bottom and top walls only");
      if (wl.kind == EQF_BC_DIRICHLET || wl.kind == EQF_BC_CHANNEL || wl.kind == EQF_BC_WELL)
        walls |= bits[w];
      channel = channel || wl.kind == EQF_BC_CHANNEL;
      active = active || wl.kind == EQF_BC_CHANNEL || wl.kind == EQF_BC_WELL ||
               (wl.kind != EQF_BC_NEUMANN && wl.value != 0.0);
    }
    if (active) EQF_REQUIRE(p.nx >= 3 && p.ny >= 3, "walls with values need nx, ny >= 3");
    if (channel) {
      EQF_REQUIRE(bc->channel_substeps >= 1 && std::isfinite(bc->channel_D) &&
                      bc->channel_D >= 0.0 && std::isfinite(bc->channel_velocity) &&
                      std::isfinite(bc->channel_rate[0]) && std::isfinite(bc->channel_rate[1]) &&
                      bc->channel_rate[0] >= 0.0 && bc->channel_rate[1] >= 0.0 &&
                      std::isfinite(bc->well_scaling) && bc->well_scaling > 0.0,
                  "bad channel parameters");
      EQF_REQUIRE(p.nx + 1 <= eqf::kChanMaxNodes, "channel longer than 4097 nodes");
      const double hx = p.width / p.nx, hy = p.height / p.ny;
      EQF_REQUIRE(std::fabs(hx - hy) <= 1e-12 * hx, "channel walls need a square lattice");
    }
    if (p.adv_u != 0.0 && p.adv_len > 0.0)
      EQF_REQUIRE(!active, "walls with values on advective traps are not supported");
    B.sync();
    B.bcs[trap] = *bc;
    B.params[trap].walls = walls;
    B.ops_dirty = true;
    if ((int)B.trap_dirty.size() == B.ntraps) B.trap_dirty[trap] = 1;
    // a new operator invalidates the initial-guess history of that trap
    const long long off = B.L[0].geom[trap].off;
    EQF_CK(cudaMemsetAsync(B.Dd[B.cur].p + off, 0, B.fine_span(trap) * sizeof(float), B.stream));
    EQF_CK(cudaMemsetAsync(reinterpret_cast<char*>(B.dstate.p + trap) +
                               offsetof(eqf::CgState, gamma),
                           0, 2 * sizeof(double), B.stream));
    B.sync();
  });
}

int eqf_set_tensor(eqf_batch* b, int32_t trap, const double* D11, const double* D22,
                   const double* D12) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    Batch& B = *b->impl;
    const eqf_trap_params& p = B.params[trap];
    const bool iso = !D11 && !D22 && !D12;
    EQF_REQUIRE(iso || (D11 && D22 && D12), "give all three tensor fields or none");
    const long long n = (long long)(p.nx + 1) * (p.ny + 1);
    std::vector<double> t;
    if (!iso) {
      t.resize(3 * n);
      for (long long k = 0; k < n; ++k) {
        const double a = D11[k], c = D22[k], d = D12[k];
        EQF_REQUIRE(std::isfinite(a) && std::isfinite(c) && std::isfinite(d) && a > 0.0 &&
                        c > 0.0 && a * c - d * d >= -1e-12 * a * c,
                    "tensor not symmetric positive definite at a node");
        t[k] = a;
        t[n + k] = c;
        t[2 * n + k] = d;
      }
    }
    B.sync();
    B.tensor[trap].swap(t);
    if (iso) {
      for (auto it = B.htens.begin(); it != B.htens.end();)
        it = it->first.second == trap ? B.htens.erase(it) : std::next(it);
      for (auto it = B.dtens.begin(); it != B.dtens.end();)
        it = it->first.second == trap ? B.dtens.erase(it) : std::next(it);
      for (auto it = B.dtensf.begin(); it != B.dtensf.end();)
        it = it->first.second == trap ? B.dtensf.erase(it) : std::next(it);
      for (auto it = B.dcoef_f.begin(); it != B.dcoef_f.end();)
        it = it->first.second == trap ? B.dcoef_f.erase(it) : std::next(it);
      for (auto it = B.dcoef_d.begin(); it != B.dcoef_d.end();)
        it = it->first.second == trap ? B.dcoef_d.erase(it) : std::next(it);
    }
    B.ops_dirty = true;
    if ((int)B.trap_dirty.size() == B.ntraps) B.trap_dirty[trap] = 1;
    const long long off = B.L[0].geom[trap].off;
    EQF_CK(cudaMemsetAsync(B.Dd[B.cur].p + off, 0, B.fine_span(trap) * sizeof(float), B.stream));
    EQF_CK(cudaMemsetAsync(reinterpret_cast<char*>(B.dstate.p + trap) +
                               offsetof(eqf::CgState, gamma),
                           0, 2 * sizeof(double), B.stream));
    B.sync();
  });
}

int eqf_set_well(eqf_batch* b, int32_t trap, double well_scaling, double decay_rate) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(std::isfinite(well_scaling) && well_scaling >= 0.0 && std::isfinite(decay_rate) &&
                    decay_rate >= 0.0,
                "bad well parameters");
    Batch& B = *b->impl;
    B.sync();
    B.well[trap].scale = well_scaling;
    B.well[trap].decay = decay_rate;
    B.setup_wells();
  });
}

int eqf_set_well_concentration(eqf_batch* b, int32_t trap, double concentration) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    EQF_REQUIRE(std::isfinite(concentration), "non-finite concentration");
    Batch& B = *b->impl;
    EQF_CK(cudaMemcpyAsync(B.d_well_c.p + trap, &concentration, sizeof(double),
                           cudaMemcpyHostToDevice, B.stream));
    B.sync();
  });
}

int eqf_read_well(eqf_batch* b, int32_t trap, double* concentration, int64_t* underflows) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    Batch& B = *b->impl;
    double c = 0.0;
    long long u = 0;
    EQF_CK(cudaMemcpyAsync(&c, B.d_well_c.p + trap, sizeof(double), cudaMemcpyDeviceToHost,
                           B.stream));
    EQF_CK(cudaMemcpyAsync(&u, B.d_well_under.p + trap, sizeof(long long),
                           cudaMemcpyDeviceToHost, B.stream));
    B.sync();
    if (concentration) *concentration = c;
    if (underflows) *underflows = u;
  });
}

static Batch::Chan* chan_of(Batch& B, int trap) {
  for (auto& c : B.chans)
    if (c->trap == trap) return c.get();
  return nullptr;
}

int eqf_read_channels(eqf_batch* b, int32_t trap, double* bottom, double* top) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    Batch& B = *b->impl;
    B.ensure_ops();
    Batch::Chan* ch = chan_of(B, trap);
    EQF_REQUIRE(ch != nullptr, "trap has no flow channel");
    double* out[2] = {bottom, top};
    for (int s = 0; s < 2; ++s) {
      if (!out[s]) continue;
      EQF_REQUIRE(ch->c[s].p != nullptr, "no channel on that wall");
      EQF_CK(cudaMemcpyAsync(out[s], ch->c[s].p, ch->n * sizeof(double), cudaMemcpyDeviceToHost,
                             B.stream));
    }
    B.sync();
  });
}

int eqf_set_channels(eqf_batch* b, int32_t trap, const double* bottom, const double* top) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    EQF_TRAP_CHECK(b, trap);
    Batch& B = *b->impl;
    B.ensure_ops();
    Batch::Chan* ch = chan_of(B, trap);
    EQF_REQUIRE(ch != nullptr, "trap has no flow channel");
    const double* in[2] = {bottom, top};
    for (int s = 0; s < 2; ++s) {
      if (!in[s]) continue;
      EQF_REQUIRE(ch->c[s].p != nullptr, "no channel on that wall");
      for (int j = 0; j < ch->n; ++j) EQF_REQUIRE(std::isfinite(in[s][j]), "non-finite channel value");
      EQF_CK(cudaMemcpyAsync(ch->c[s].p, in[s], ch->n * sizeof(double), cudaMemcpyHostToDevice,
                             B.stream));
    }
    B.sync();
  });
}

// Rod cells (eqfield.h: eqf_set_rods and the calls after it).
namespace {

// eQ::Cell::DEFAULT_CELL_WIDTH_MICRONS (src/eQcell.h:42)
constexpr double kRodCellWidth = 1.0;

void check_rods(const eqf_trap_params& p, const eqf_rod* rods, int64_t n) {
  auto in_trap = [&](const double* xy) {
    return std::isfinite(xy[0]) && std::isfinite(xy[1]) && xy[0] >= 0.0 && xy[1] >= 0.0 &&
           xy[0] <= p.width && xy[1] <= p.height;
  };
  for (int64_t c = 0; c < n; ++c) {
    const eqf_rod& r = rods[c];
    EQF_REQUIRE(in_trap(r.center) && in_trap(r.pole_a) && in_trap(r.pole_b),
                "rod centre or pole outside the trap");
    bool fin = std::isfinite(r.length) && std::isfinite(r.body_pos[0]) &&
               std::isfinite(r.body_pos[1]) && std::isfinite(r.body_rot[0]) &&
               std::isfinite(r.body_rot[1]);
    for (double v : r.verts) fin = fin && std::isfinite(v);
    EQF_REQUIRE(fin, "non-finite rod geometry");
    EQF_REQUIRE(r.length >= kRodCellWidth, "rod shorter than its width");
  }
}

}  // namespace

int eqf_set_rods(eqf_batch* b, int32_t n_layers, const int32_t* layers, const eqf_rod_law* law,
                 int64_t n_cells, const eqf_rod* rods, const double* ihsl,
                 const double* production, const uint8_t* mode) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    EQF_REQUIRE(n_layers >= 1 && n_layers <= EQF_MAX_ROD_LAYERS && layers && law,
                "bad rod layers or law");
    for (int l = 0; l < n_layers; ++l) {
      EQF_TRAP_CHECK(b, layers[l]);
      for (int m = 0; m < l; ++m) EQF_REQUIRE(layers[m] != layers[l], "repeated rod layer");
    }
    const eqf_trap_params& p0 = B.params[layers[0]];
    for (int l = 1; l < n_layers; ++l) {
      const eqf_trap_params& p = B.params[layers[l]];
      EQF_REQUIRE(p.nx == p0.nx && p.ny == p0.ny && p.width == p0.width &&
                      p.height == p0.height,
                  "rod layers must share the mesh");
    }
    const double npm = law->nodes_per_micron;
    EQF_REQUIRE(std::isfinite(npm) && npm > 0.0 && std::isfinite(law->dt) && law->dt >= 0.0,
                "bad rod law");
    for (int l = 0; l < n_layers; ++l)
      EQF_REQUIRE(std::isfinite(law->membrane_rate[l]), "non-finite membrane rate");
    // eQabm's lattice, nodesWide = size_t(W*npm) + 1 and nodesHigh = size_t(H*npm) + 1
    // (src/abm/eQabm.cpp:30-31), must be the mesh's nodes, with W*npm and H*npm
    // integral so that every point of the trap rounds to a lattice node
    EQF_REQUIRE(p0.width * npm == (double)p0.nx && p0.height * npm == (double)p0.ny,
                "rod coupling needs nx = W*npm and ny = H*npm exactly");
    size_t slot = B.rod_sets.size();
    for (size_t q = 0; q < B.rod_sets.size(); ++q) {
      const auto& rs = *B.rod_sets[q];
      if (rs.layers[0] == layers[0]) {
        slot = q;
        continue;
      }
      for (int l = 0; l < n_layers; ++l)
        for (int t : rs.layers)
          EQF_REQUIRE(t != layers[l], "trap already belongs to another rod set");
    }
    EQF_REQUIRE(n_cells >= 0 && n_cells <= (1 << 26), "bad rod cell count");
    if (n_cells == 0) {
      if (slot < B.rod_sets.size()) B.rod_sets.erase(B.rod_sets.begin() + slot);
      B.rod_publish();
      return;
    }
    EQF_REQUIRE(rods && ihsl && production && mode, "null rod arrays");
    check_rods(p0, rods, n_cells);
    const int64_t ns = n_cells * n_layers;
    for (int64_t i = 0; i < ns; ++i)
      EQF_REQUIRE(std::isfinite(ihsl[i]) && ihsl[i] >= 0.0 && std::isfinite(production[i]) &&
                      mode[i] <= EQF_ROD_INERT,
                  "bad rod state");
    auto rs = std::make_unique<Batch::RodSet>();
    rs->layers.assign(layers, layers + n_layers);
    rs->law = *law;
    rs->n = (int)n_cells;
    const eqf::LevelGeom& g = B.L[0].geom[layers[0]];
    eqf::RodLawDev& d = rs->dev;
    d.npm = npm;
    d.dt = law->dt;
    for (int l = 0; l < eqf::kRodLayers; ++l) {
      d.km[l] = l < n_layers ? law->membrane_rate[l] : 0.0;
      d.lay_off[l] = l < n_layers ? B.L[0].geom[layers[l]].off : 0;
    }
    d.trap0 = layers[0];
    d.nlayers = n_layers;
    d.nx = g.nx;
    d.ny = g.ny;
    d.P = g.P;
    // nodesToEdge = size_t(round(npm * W / 2)) (src/abm/eQabm.cpp:75)
    d.nte = (int)std::round(npm * kRodCellWidth / 2.0);
    // eQ::Cell (src/eQcell.h:51-59), same expressions
    const double pole_radius = kRodCellWidth / 2.0;
    d.k.cyl = M_PI * (pole_radius * pole_radius);
    d.k.pole = 4.0 / 3.0 * M_PI * (pole_radius * pole_radius * pole_radius);
    d.k.nm_per_molecule = 1.0 / 0.602;
    rs->span = B.fine_span(layers[0]);
    const size_t n = (size_t)n_cells, n4 = n * eqf::kRodLayers;
    rs->rods.alloc(n);
    rs->dlaw.alloc(1);
    rs->fp_off.alloc(n + 1);
    rs->wave_cells.alloc(n);
    rs->winfo.alloc(n);
    rs->cellk.alloc(3 * n);
    rs->cover.alloc(rs->span);
    rs->start.alloc(rs->span + 1);
    rs->cursor.alloc(rs->span);
    rs->flag.alloc(3);
    rs->ihsl.alloc(n4);
    rs->prod.alloc(n4);
    rs->ehsl.alloc(n4);
    rs->mode.alloc(n4);
    std::vector<double> hi(n4, 0.0), hp(n4, 0.0);
    std::vector<unsigned char> hm(n4, EQF_ROD_INERT);
    for (size_t c = 0; c < n; ++c)
      for (int l = 0; l < n_layers; ++l) {
        hi[c * eqf::kRodLayers + l] = ihsl[c * n_layers + l];
        hp[c * eqf::kRodLayers + l] = production[c * n_layers + l];
        hm[c * eqf::kRodLayers + l] = mode[c * n_layers + l];
      }
    rs->rods.upload(rods, n, B.stream);
    rs->dlaw.upload(&rs->dev, 1, B.stream);
    rs->ihsl.upload(hi.data(), n4, B.stream);
    rs->prod.upload(hp.data(), n4, B.stream);
    rs->mode.upload(hm.data(), n4, B.stream);
    EQF_CK(cudaMemsetAsync(rs->ehsl.p, 0, n4 * sizeof(double), B.stream));
    B.rod_analyse(*rs);
    if (slot < B.rod_sets.size())
      B.rod_sets[slot] = std::move(rs);
    else
      B.rod_sets.push_back(std::move(rs));
    B.rod_publish();
  });
}

int eqf_update_rods(eqf_batch* b, int32_t layer0, int64_t n_cells, const eqf_rod* rods,
                    const double* production) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    Batch::RodSet* rs = B.rod_set_of(layer0);
    EQF_REQUIRE(rs != nullptr, "no rod set on this layer");
    EQF_REQUIRE(n_cells == rs->n && rods, "rod count mismatch");
    check_rods(B.params[layer0], rods, n_cells);
    const int nl = (int)rs->layers.size();
    const size_t n = (size_t)n_cells, n4 = n * eqf::kRodLayers;
    if (production) {
      for (int64_t i = 0; i < n_cells * nl; ++i)
        EQF_REQUIRE(std::isfinite(production[i]), "non-finite production");
      std::vector<double> hp(n4, 0.0);
      for (size_t c = 0; c < n; ++c)
        for (int l = 0; l < nl; ++l) hp[c * eqf::kRodLayers + l] = production[c * nl + l];
      EQF_CK(cudaMemcpyAsync(rs->prod.p, hp.data(), n4 * sizeof(double), cudaMemcpyHostToDevice,
                             B.stream));
      B.sync();  // hp is released on return
    }
    EQF_CK(cudaMemcpyAsync(rs->rods.p, rods, n * sizeof(eqf_rod), cudaMemcpyHostToDevice,
                           B.stream));
    B.rod_analyse(*rs);
    B.rod_publish();
  });
}

int eqf_read_rods(eqf_batch* b, int32_t layer0, int64_t n_cells, double* ihsl, double* ehsl,
                  int32_t* points) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    Batch::RodSet* rs = B.rod_set_of(layer0);
    EQF_REQUIRE(rs != nullptr, "no rod set on this layer");
    EQF_REQUIRE(n_cells == rs->n, "rod count mismatch");
    const int nl = (int)rs->layers.size();
    const size_t n = (size_t)n_cells, n4 = n * eqf::kRodLayers;
    std::vector<double> hi(n4), he(n4);
    std::vector<int> off(n + 1);
    EQF_CK(cudaMemcpyAsync(hi.data(), rs->ihsl.p, n4 * sizeof(double), cudaMemcpyDeviceToHost,
                           B.stream));
    EQF_CK(cudaMemcpyAsync(he.data(), rs->ehsl.p, n4 * sizeof(double), cudaMemcpyDeviceToHost,
                           B.stream));
    EQF_CK(cudaMemcpyAsync(off.data(), rs->fp_off.p, (n + 1) * sizeof(int),
                           cudaMemcpyDeviceToHost, B.stream));
    B.sync();
    for (size_t c = 0; c < n; ++c) {
      for (int l = 0; l < nl; ++l) {
        if (ihsl) ihsl[c * nl + l] = hi[c * eqf::kRodLayers + l];
        if (ehsl) ehsl[c * nl + l] = he[c * eqf::kRodLayers + l];
      }
      if (points) points[c] = off[c + 1] - off[c];
    }
  });
}

// The batch's rod sets in increasing order of their first layer.
static std::vector<Batch::RodSet*> rod_sets_by_layer(Batch& B) {
  std::vector<Batch::RodSet*> v;
  for (auto& up : B.rod_sets) v.push_back(up.get());
  std::sort(v.begin(), v.end(), [](const Batch::RodSet* a, const Batch::RodSet* b) {
    return a->layers[0] < b->layers[0];
  });
  return v;
}

int eqf_update_rods_all(eqf_batch* b, int64_t n_total, const eqf_rod* rods,
                        const double* production) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    const std::vector<Batch::RodSet*> sets = rod_sets_by_layer(B);
    int64_t tot = 0, totp = 0;
    for (const Batch::RodSet* rs : sets) {
      tot += rs->n;
      totp += (int64_t)rs->n * (int64_t)rs->layers.size();
    }
    EQF_REQUIRE(n_total == tot && (n_total == 0 || rods), "rod count mismatch");
    if (production)
      for (int64_t i = 0; i < totp; ++i)
        EQF_REQUIRE(std::isfinite(production[i]), "non-finite production");
    // every set's rods are checked before anything is uploaded: a bad set leaves all
    // sets (device rods, footprints, waves) as they were
    {
      int64_t c = 0;
      for (const Batch::RodSet* rs : sets) {
        check_rods(B.params[rs->layers[0]], rods + c, rs->n);
        c += rs->n;
      }
    }
    // stage the rods and the productions (in the device's kRodLayers layout) in pinned
    // memory, so the uploads are asynchronous
    size_t prod4 = 0;
    for (const Batch::RodSet* rs : sets) prod4 += (size_t)rs->n * eqf::kRodLayers;
    const size_t rbytes = (size_t)tot * sizeof(eqf_rod);
    B.rod_hstage.grow(rbytes + (production ? prod4 * sizeof(double) : 0) + 16);
    unsigned char* st = B.rod_hstage.p;
    double* hp = reinterpret_cast<double*>(st + ((rbytes + 15) & ~size_t(15)));
    int64_t c0 = 0, p0 = 0;
    size_t q0 = 0;
    try {
      for (Batch::RodSet* rs : sets) {
        const int nl = (int)rs->layers.size();
        const size_t n = (size_t)rs->n;
        std::memcpy(st + (size_t)c0 * sizeof(eqf_rod), rods + c0, n * sizeof(eqf_rod));
        EQF_CK(cudaMemcpyAsync(rs->rods.p, st + (size_t)c0 * sizeof(eqf_rod),
                               n * sizeof(eqf_rod), cudaMemcpyHostToDevice, B.stream));
        if (production) {
          double* q = hp + q0;
          std::fill(q, q + n * eqf::kRodLayers, 0.0);
          for (size_t c = 0; c < n; ++c)
            for (int l = 0; l < nl; ++l) q[c * eqf::kRodLayers + l] = production[p0 + c * nl + l];
          EQF_CK(cudaMemcpyAsync(rs->prod.p, q, n * eqf::kRodLayers * sizeof(double),
                                 cudaMemcpyHostToDevice, B.stream));
        }
        c0 += rs->n;
        p0 += (int64_t)rs->n * nl;
        q0 += n * eqf::kRodLayers;
      }
      B.rod_analyse_sets(sets);  // ends with a sync: the staging may be reused
    } catch (...) {
      // copies may still read the pinned staging: let them finish before the next
      // call writes it
      cudaStreamSynchronize(B.stream);
      throw;
    }
    B.rod_publish();
  });
}

int eqf_read_rods_all(eqf_batch* b, int64_t n_total, double* ihsl, double* ehsl,
                      int32_t* points) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    const std::vector<Batch::RodSet*> sets = rod_sets_by_layer(B);
    int64_t tot = 0;
    size_t n4 = 0;
    for (const Batch::RodSet* rs : sets) {
      tot += rs->n;
      n4 += (size_t)rs->n * eqf::kRodLayers;
    }
    EQF_REQUIRE(n_total == tot, "rod count mismatch");
    const size_t dbytes = n4 * sizeof(double);
    B.rod_hstage.grow(2 * dbytes + ((size_t)tot + sets.size()) * sizeof(int) + 16);
    double* hi = reinterpret_cast<double*>(B.rod_hstage.p);
    double* he = hi + n4;
    int* ho = reinterpret_cast<int*>(he + n4);
    size_t q0 = 0, o0 = 0;
    for (const Batch::RodSet* rs : sets) {
      const size_t n = (size_t)rs->n, m = n * eqf::kRodLayers;
      EQF_CK(cudaMemcpyAsync(hi + q0, rs->ihsl.p, m * sizeof(double), cudaMemcpyDeviceToHost,
                             B.stream));
      EQF_CK(cudaMemcpyAsync(he + q0, rs->ehsl.p, m * sizeof(double), cudaMemcpyDeviceToHost,
                             B.stream));
      EQF_CK(cudaMemcpyAsync(ho + o0, rs->fp_off.p, (n + 1) * sizeof(int),
                             cudaMemcpyDeviceToHost, B.stream));
      q0 += m;
      o0 += n + 1;
    }
    B.sync();
    q0 = o0 = 0;
    int64_t c0 = 0, p0 = 0;
    for (const Batch::RodSet* rs : sets) {
      const int nl = (int)rs->layers.size();
      const size_t n = (size_t)rs->n;
      for (size_t c = 0; c < n; ++c) {
        for (int l = 0; l < nl; ++l) {
          if (ihsl) ihsl[p0 + c * nl + l] = hi[q0 + c * eqf::kRodLayers + l];
          if (ehsl) ehsl[p0 + c * nl + l] = he[q0 + c * eqf::kRodLayers + l];
        }
        if (points) points[c0 + c] = ho[o0 + c + 1] - ho[o0 + c];
      }
      q0 += n * eqf::kRodLayers;
      o0 += n + 1;
      c0 += rs->n;
      p0 += (int64_t)rs->n * nl;
    }
  });
}

int eqf_exchange_rods(eqf_batch* b) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    B.enqueue_rods();
    B.sync();
  });
}

int eqf_rod_waves(eqf_batch* b, int32_t* waves) {
  if (!b || !waves) return EQF_ERR_INVALID;
  int w = 0;
  for (const auto& rs : b->impl->rod_sets) w = std::max(w, rs->waves);
  *waves = w;
  return EQF_OK;
}

int eqf_rod_relax_passes(eqf_batch* b, int32_t* passes) {
  if (!b || !passes) return EQF_ERR_INVALID;
  int p = 0;
  for (const auto& rs : b->impl->rod_sets) p = std::max(p, rs->relax_passes);
  *passes = p;
  return EQF_OK;
}

int eqf_stream(eqf_batch* b, void** stream) {
  if (!b || !stream) return EQF_ERR_INVALID;
  *stream = (void*)b->impl->stream;
  return EQF_OK;
}

int eqf_profile(eqf_batch* b, int32_t enable) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    B.sync();
    eqf::Prof& P = B.prof;
    if (enable) {
      const size_t cap = 1u << 16;
      if (P.ev.empty()) {
        P.ev.resize(2 * cap);
        for (auto& e : P.ev) EQF_CK(cudaEventCreate(&e));
        P.cls.assign(cap, -1);
        P.work.alloc(cap);
      }
      EQF_CK(cudaMemsetAsync(P.work.p, 0, cap * sizeof(unsigned long long), B.stream));
      B.sync();
      P.used = 0;
      P.overflow = false;
      P.on = true;
    } else {
      P.on = false;
    }
  });
}

int eqf_profile_read(eqf_batch* b, int32_t n_classes, double* ms, int64_t* launches,
                     int64_t* nodes, double* bytes) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    Batch& B = *b->impl;
    EQF_REQUIRE(n_classes >= EQF_PROF_CLASSES && ms && launches && nodes && bytes,
                "profile arrays too short");
    B.sync();
    eqf::Prof& P = B.prof;
    EQF_REQUIRE(!P.overflow, "profiler record pool overflowed (profile fewer steps)");
    std::vector<unsigned long long> w(P.used);
    if (P.used)
      EQF_CK(cudaMemcpy(w.data(), P.work.p, P.used * sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost));
    for (int c = 0; c < n_classes; ++c) {
      ms[c] = 0.0;
      launches[c] = 0;
      nodes[c] = 0;
      bytes[c] = 0.0;
    }
    const int tsize = B.opts.precision == EQF_PREC_FP32_IR ? 4 : 8;
    for (size_t r = 0; r < P.used; ++r) {
      float t = 0.f;
      EQF_CK(cudaEventElapsedTime(&t, P.ev[2 * r], P.ev[2 * r + 1]));
      const int c = P.cls[r];
      ms[c] += t;
      launches[c] += 1;
      nodes[c] += (int64_t)w[r];
      double per = 0.0;
      eqf::class_bytes(c, tsize, per);
      bytes[c] += per * (double)w[r];
    }
  });
}

int eqf_sync(eqf_batch* b) {
  if (!b) return EQF_ERR_INVALID;
  return guarded(b, [&] {
    b->impl->sync();
    b->impl->check_fail();
  });
}

}  // extern "C"
