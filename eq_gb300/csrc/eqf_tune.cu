// Autotuner: per trap-size bucket, the finest-level row tile target, the fused
// kernels' 2-D tile width, the pre/post Chebyshev degrees and the Krylov schedule
// (inner iterations per refinement sweep, scheduled sweeps) that give the most
// DOF-steps/s at the solver tolerance (include/eqfield.h: eqf_autotune,
// eqf_create_tuned).
//
// Host code over the public C ABI.  Each candidate runs on a batch of the caller's
// traps from that bucket (replicated to fill the GPU) with seeded random point
// cells: three warm-up steps (graph capture, initial-guess history), then four
// timed steps between CUDA events on the batch's stream.  The default
// configuration is measured first, so a bucket whose exploration runs out of time
// keeps the defaults.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "../../include/eqfield.h"

namespace {

constexpr int kBuckets = 4;
constexpr int64_t kBucketMax[kBuckets] = {32768, 131072, 524288, INT64_MAX};
constexpr long long kFillNodes = 16ll << 20;  // nodes of a tuning batch (fills the GPU)
constexpr int kMaxTraps = 1024;
// warm-up and timed steps of the Krylov-schedule trials (the other trials: 3 and 4)
constexpr int kSchedWarm = 10, kSchedTimed = 8;

// splitmix64: a seeded stream of uniform doubles, identical on every platform
struct Rng {
  uint64_t s;
  double uniform() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  }
};

// DOF-steps/s of one candidate (0 if it cannot run: e.g. rows too wide for the tile)
// over `timed` steps after `warm` warm-up steps
double measure(const std::vector<eqf_trap_params>& traps, const eqf_solver_opts& o, int tile,
               int cols, int warm = 3, int timed = 4) {
  eqf_solver_opts c = o;
  c.tile_nodes = tile;
  c.tile_cols = cols;
  c.use_graph = 1;
  c.adaptive = 1;
  eqf_batch* b = nullptr;
  if (eqf_create((int32_t)traps.size(), traps.data(), &c, &b) != EQF_OK) return 0.0;
  double rate = 0.0;
  long long nodes = 0;
  Rng rng{12345};
  bool ok = true;
  for (size_t t = 0; t < traps.size() && ok; ++t) {
    const eqf_trap_params& p = traps[t];
    nodes += (long long)(p.nx + 1) * (p.ny + 1);
    const int64_t m = std::max<int64_t>(1, (int64_t)std::llround(0.02 * p.nx * p.ny));
    std::vector<double> xy(2 * m), s(m);
    for (int64_t i = 0; i < m; ++i) {
      xy[2 * i] = p.width * (0.05 + 0.9 * rng.uniform());
      xy[2 * i + 1] = p.height * (0.05 + 0.9 * rng.uniform());
      s[i] = 0.5 + rng.uniform();
    }
    ok = eqf_set_cells(b, (int32_t)t, m, xy.data(), s.data()) == EQF_OK;
  }
  void* stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ok && eqf_step(b, warm) == EQF_OK && eqf_stream(b, &stream) == EQF_OK &&
      cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
    const int steps = timed;
    cudaEventRecord(e0, (cudaStream_t)stream);
    const int rc = eqf_step(b, steps);
    cudaEventRecord(e1, (cudaStream_t)stream);
    float ms = 0.f;
    if (rc == EQF_OK && cudaEventSynchronize(e1) == cudaSuccess &&
        cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f)
      rate = (double)nodes * steps / (ms * 1e-3);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  eqf_destroy(b);
  return rate;
}

}  // namespace

extern "C" int eqf_autotune_log(int32_t n_traps, const eqf_trap_params* traps,
                                const eqf_solver_opts* opts, double budget_s,
                                eqf_tune_table* table, char* log, int64_t log_size) {
  if (n_traps < 1 || !traps || !table || !(budget_s > 0) || (log && log_size < 1))
    return EQF_ERR_INVALID;
  eqf_solver_opts o;
  if (opts)
    o = *opts;
  else
    eqf_default_opts(EQF_PREC_FP32_IR, &o);
  const auto t0 = std::chrono::steady_clock::now();
  auto elapsed = [&] {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  };
  std::string text;
  std::memset(table, 0, sizeof(*table));
  table->n = kBuckets;
  // stage 1: smoother degrees at the default tiles; stage 2: tile node targets x 2-D
  // tile widths at the best degrees (0 = the library default); stage 3: Krylov
  // schedules at the best of those (fewer inner iterations with more FP64 refinement
  // sweeps pays on some batches: the sweeps' residuals are exact, the inner solve FP32)
  const int degs[][2] = {{0, 0}, {1, 1}, {3, 3}, {2, 1}};
  const int tiles[] = {0, 2048, 6144};
  const int widths[] = {0, 64, 256, 512};
  const int scheds[][2] = {{2, 4}, {3, 3}};
  for (int k = 0; k < kBuckets; ++k) {
    eqf_tune_bucket& tb = table->b[k];
    tb.max_nodes = kBucketMax[k];
    tb.tile_nodes = 0;
    tb.tile_cols = 0;
    tb.cheb_pre = o.cheb_pre;
    tb.cheb_post = o.cheb_post;
    tb.max_iters = o.max_iters;
    tb.max_sweeps = o.max_sweeps;
    std::vector<eqf_trap_params> sel;
    for (int t = 0; t < n_traps; ++t) {
      const long long nodes = (long long)(traps[t].nx + 1) * (traps[t].ny + 1);
      const int64_t lo = k > 0 ? kBucketMax[k - 1] : 0;
      if (nodes > lo && nodes <= kBucketMax[k]) sel.push_back(traps[t]);
    }
    if (sel.empty()) continue;
    // replicate to a GPU-filling batch
    std::vector<eqf_trap_params> batch;
    long long nodes = 0;
    for (size_t i = 0; nodes < kFillNodes && (int)batch.size() < kMaxTraps; ++i) {
      const eqf_trap_params& p = sel[i % sel.size()];
      batch.push_back(p);
      nodes += (long long)(p.nx + 1) * (p.ny + 1);
    }
    double best = 0.0;
    auto trial = [&](int pre, int post, int tile, int cols, int iters, int sweeps,
                     bool longer = false) {
      if (elapsed() > budget_s && best > 0.0) return;
      eqf_solver_opts c = o;
      c.cheb_pre = pre;
      c.cheb_post = post;
      c.max_iters = iters;
      c.max_sweeps = sweeps;
      const double r = longer ? measure(batch, c, tile, cols, kSchedWarm, kSchedTimed)
                              : measure(batch, c, tile, cols);
      char line[192];
      std::snprintf(line, sizeof(line), "%d %d %d %d %d %d %d %.6e\n", k, tile, cols, pre,
                    post, iters, sweeps, r);
      text += line;
      if (r > best) {
        best = r;
        tb.tile_nodes = tile;
        tb.tile_cols = cols;
        tb.cheb_pre = pre;
        tb.cheb_post = post;
        tb.max_iters = iters;
        tb.max_sweeps = sweeps;
      }
    };
    const int it0 = o.max_iters, sw0 = o.max_sweeps;
    for (const auto& d : degs)
      trial(d[0] > 0 ? d[0] : o.cheb_pre, d[0] > 0 ? d[1] : o.cheb_post, 0, 0, it0, sw0);
    const int pre = tb.cheb_pre, post = tb.cheb_post;
    for (int tile : tiles)
      for (int cols : widths)
        if (tile != 0 || cols != 0) trial(pre, post, tile, cols, it0, sw0);
    const int tile = tb.tile_nodes, cols = tb.tile_cols;
    if (o.precision == EQF_PREC_FP32_IR) {  // the plain form keeps its one long sweep
      // schedules differ by a few percent once the fields have settled, which the
      // short trials above do not resolve: the incumbent is measured again the same
      // longer way and the schedules compete among themselves
      const double short_best = best;
      best = 0.0;
      trial(pre, post, tile, cols, it0, sw0, true);
      for (const auto& sc : scheds)
        if (sc[0] != it0 || sc[1] != sw0) trial(pre, post, tile, cols, sc[0], sc[1], true);
      if (best == 0.0) best = short_best;  // out of budget before the longer trials
    }
    tb.dof_steps_per_s = best;
  }
  if (log) {
    const size_t n = std::min<size_t>(text.size(), (size_t)log_size - 1);
    std::memcpy(log, text.data(), n);
    log[n] = '\0';
  }
  return EQF_OK;
}

extern "C" int eqf_autotune(int32_t n_traps, const eqf_trap_params* traps,
                            const eqf_solver_opts* opts, double budget_s, eqf_tune_table* table) {
  return eqf_autotune_log(n_traps, traps, opts, budget_s, table, nullptr, 0);
}
