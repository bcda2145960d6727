// eqserve: continuous-batching request loop over eqfield batches (include/eqserve.h).
//
// Host code only.  A cohort is one eqfield batch (its own CUDA stream) holding the
// traps of the requests admitted together; cohorts step concurrently.  Per cohort
// step: CUDA event, one graph-replayed step, asynchronous readout + freeze of the
// requests that finish at that step, a copy of the convergence-failure counter,
// CUDA event.  eqs_progress only queries events, so it never waits for the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/eqfield.h"
#include "../../include/eqserve.h"

// Multigrid depth of a trap and the nodes its grid spans per level (eqf_batch.cu).
int eqf_internal_trap_levels(const eqf_trap_params& p);
void eqf_internal_trap_spans(const eqf_trap_params& p, int nlev, long long* spans);

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  int64_t id = -1;
  eqs_request r{};
  std::vector<double> xy, s;
  std::vector<int32_t> sender;
  int64_t n_nodes = 0;
  double t_submit = 0, t_admit = -1, t_done = -1;
  int status = EQF_OK;
  int cohort = -1;
  int trap0 = -1;
  int step0 = 0;  // cohort steps queued before the request's first step
  int end_step() const { return step0 + r.steps; }
  double* h_cells = nullptr;  // pinned: n_species * n_cells
  double* h_nodal = nullptr;  // pinned: n_species * n_nodes (when asked for)
  bool done = false;
  bool taken = false;  // result handed out (the object lives until its cohort is released)
  int64_t klass = 0;   // cohort class: multigrid depth and symmetric / advective operator
  int levels = 0;      // the class's multigrid depth
  std::vector<long long> spans;  // per species and level: nodes its grid spans
  bool picked = false; // taken into the cohort being formed
  int ntraps() const { return r.n_species; }
};

struct StepMark {
  int step = 0;
  cudaEvent_t start = nullptr, end = nullptr;
  int32_t* fail = nullptr;  // pinned: the batch's failure counter after this step
};

// Page-locked host memory for the readouts, carved from large slabs and recycled by
// power-of-two size class.  A cudaMallocHost / cudaFreeHost per request or per step
// would stall the one host thread that keeps every cohort's queue filled.
struct PinnedArena {
  static constexpr size_t kSlab = (size_t)64 << 20;
  std::vector<void*> slabs;
  char* cur = nullptr;
  size_t left = 0;
  std::map<size_t, std::vector<void*>> free_by_class;
  static size_t size_class(size_t n) {
    size_t c = 256;
    while (c < n) c <<= 1;
    return c;
  }
  // nullptr when page-locked memory runs out
  void* get(size_t n) {
    const size_t c = size_class(n);
    std::vector<void*>& fl = free_by_class[c];
    if (!fl.empty()) {
      void* p = fl.back();
      fl.pop_back();
      return p;
    }
    void* p = nullptr;
    if (c > kSlab / 4) {  // large: a slab of its own
      if (cudaMallocHost(&p, c) != cudaSuccess) return nullptr;
      slabs.push_back(p);
      return p;
    }
    if (left < c) {
      if (cudaMallocHost(&p, kSlab) != cudaSuccess) return nullptr;
      slabs.push_back(p);
      cur = static_cast<char*>(p);
      left = kSlab;
    }
    p = cur;
    cur += c;
    left -= c;
    return p;
  }
  void put(void* p, size_t n) {
    if (p) free_by_class[size_class(n)].push_back(p);
  }
  ~PinnedArena() {
    for (void* p : slabs) cudaFreeHost(p);
  }
};

size_t cells_bytes(const Req* q) {
  return sizeof(double) * (size_t)std::max<int64_t>(1, q->r.n_cells * q->r.n_species);
}
size_t nodal_bytes(const Req* q) {
  return sizeof(double) * (size_t)(q->n_nodes * q->r.n_species);
}

struct Cohort {
  int id = 0;
  int64_t klass = 0;
  eqf_batch* b = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<Req*> reqs;  // the requests still running
  // per trap slot: the grid it was created with (its capacity) and the request
  // holding it (null: free since that request's last step was queued)
  std::vector<eqf_trap_params> slot_cap;
  std::vector<long long> cap_spans;  // per slot and level: the nodes the slot holds
  int levels = 0;
  std::vector<Req*> slot_owner;
  bool filling = false;  // queue no steps until the queued ones are done, then fill slots
  bool closing = false;  // no more requests: runs out to make room for another cohort
  bool refilled = false;  // slots filled since the last queued step
  bool slots_freed = false;    // a slot was freed since the last match
  bool was_ready = false;      // enough free slots at the last look
  int64_t seen_submitted = -1;  // the server's submissions at the last match
  int steps_target = 0, launched = 0;
  std::deque<StepMark> inflight;
  int64_t bytes = 0;
  int remaining = 0;
  int32_t fails_seen = 0;
  bool retired = false;  // every request done (its memory is released right after)
};

}  // namespace

struct eqs_server {
  eqs_config cfg{};
  std::string err;
  Clock::time_point t0 = Clock::now();
  double last_progress = 0;
  int64_t next_id = 0;
  int next_cohort = 0;
  std::deque<Req*> pending;
  std::map<int64_t, std::unique_ptr<Req>> reqs;
  std::vector<std::unique_ptr<Cohort>> cohorts;
  std::vector<int64_t> done_ids;
  std::vector<float> step_ms;
  eqs_stats st{};
  PinnedArena pinned;  // destroyed after the cohorts' copies into it are done
  // the device's memory pool keeps what released cohorts freed (up to the budget) for
  // the next admissions; its previous release threshold is restored at destruction
  cudaMemPool_t pool = nullptr;
  uint64_t pool_threshold0 = 0;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

struct Fail {
  int code;
  std::string msg;
};

void ck(int rc, const char* what) {
  if (rc != EQF_OK) throw Fail{rc, std::string(what) + " failed (" + std::to_string(rc) + ")"};
}
void ckb(int rc, eqf_batch* b) {
  if (rc != EQF_OK) throw Fail{rc, eqf_last_error(b)};
}
void ckc(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw Fail{EQF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}

template <class F>
int guarded(eqs_server* s, F&& f) {
  try {
    f();
    return EQF_OK;
  } catch (const Fail& e) {
    if (s) s->err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    if (s) s->err = "host allocation failed";
    return EQF_ERR_NOMEM;
  }
}

void trap_list(const std::vector<Req*>& rs, std::vector<eqf_trap_params>& tp, int64_t& cells) {
  tp.clear();
  cells = 0;
  for (const Req* q : rs) {
    for (int k = 0; k < q->r.n_species; ++k) tp.push_back(q->r.species[k]);
    cells += q->r.n_cells * q->r.n_species;
  }
}

int64_t estimate(const eqs_server* s, const std::vector<Req*>& rs) {
  std::vector<eqf_trap_params> tp;
  int64_t cells = 0, bytes = 0;
  trap_list(rs, tp, cells);
  ck(eqf_footprint_estimate((int32_t)tp.size(), tp.data(), &s->cfg.opts, cells, &bytes),
     "eqf_footprint_estimate");
  return bytes;
}

void release_cohort(eqs_server* s, Cohort& c) {
  for (StepMark& m : c.inflight) {
    cudaEventDestroy(m.start);
    cudaEventDestroy(m.end);
    s->pinned.put(m.fail, sizeof(int32_t));
  }
  c.inflight.clear();
  if (c.b) eqf_destroy(c.b);
  c.b = nullptr;
  s->st.bytes_in_use -= c.bytes;
}

// Marks a request finished (results are in its pinned buffers).
void finish(eqs_server* s, Req* q, int status) {
  if (q->done) return;
  q->done = true;
  q->status = status;
  q->t_done = s->now();
  s->done_ids.push_back(q->id);
  if (status == EQF_OK) {
    s->st.completed += 1;
    s->st.dof_steps += (double)q->n_nodes * q->r.n_species * q->r.steps;
  } else {
    s->st.failed += 1;
  }
}

void fail_cohort(eqs_server* s, Cohort& c, int code) {
  for (Req* q : c.reqs)
    if (!q->done) finish(s, q, code);
  c.remaining = 0;
}

// Queues one step of a cohort with its readouts and bookkeeping.
void launch_step(eqs_server* s, Cohort& c) {
  StepMark m;
  m.step = c.launched + 1;
  ckc(cudaEventCreate(&m.start), "cudaEventCreate");
  ckc(cudaEventCreate(&m.end), "cudaEventCreate");
  m.fail = static_cast<int32_t*>(s->pinned.get(sizeof(int32_t)));
  if (!m.fail) throw Fail{EQF_ERR_NOMEM, "page-locked host memory exhausted"};
  *m.fail = 0;
  ckc(cudaEventRecord(m.start, c.stream), "cudaEventRecord");
  ckb(eqf_step(c.b, 1), c.b);
  const double tr = s->now();
  for (Req* q : c.reqs) {
    if (q->end_step() != m.step) continue;
    for (int k = 0; k < q->r.n_species; ++k) {
      if (q->r.n_cells > 0)
        ckb(eqf_read_cells_async(c.b, q->trap0 + k, q->r.n_cells, q->h_cells + k * q->r.n_cells),
            c.b);
      if (q->h_nodal) ckb(eqf_read_nodal_async(c.b, q->trap0 + k, q->h_nodal + k * q->n_nodes), c.b);
      ckb(eqf_set_active(c.b, q->trap0 + k, 0), c.b);
      c.slot_owner[q->trap0 + k] = nullptr;  // reusable after these stream-ordered copies
      c.slots_freed = true;
    }
  }
  ckb(eqf_fail_count_async(c.b, m.fail), c.b);
  s->st.readout_s += s->now() - tr;
  ckc(cudaEventRecord(m.end, c.stream), "cudaEventRecord");
  c.inflight.push_back(m);
  c.launched = m.step;
}

void retire(eqs_server* s, Cohort& c) {
  while (!c.inflight.empty()) {
    StepMark& m = c.inflight.front();
    const cudaError_t e = cudaEventQuery(m.end);
    if (e == cudaErrorNotReady) break;
    if (e != cudaSuccess) {
      s->err = cudaGetErrorString(e);
      fail_cohort(s, c, EQF_ERR_CUDA);
      return;
    }
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, m.start, m.end) == cudaSuccess) s->step_ms.push_back(ms);
    const int32_t fails = *m.fail;
    const int status = fails > c.fails_seen ? EQF_ERR_NOT_CONVERGED : EQF_OK;
    if (status != EQF_OK) {
      // the counter is per batch: every request still running at this step is suspect
      for (Req* q : c.reqs)
        if (!q->done && q->step0 < m.step && q->end_step() >= m.step) q->status = status;
      c.fails_seen = fails;
    }
    for (Req* q : c.reqs)
      if (q->end_step() == m.step && !q->done) {
        finish(s, q, q->status);
        c.remaining -= 1;
      }
    c.reqs.erase(std::remove_if(c.reqs.begin(), c.reqs.end(), [](const Req* q) { return q->done; }),
                 c.reqs.end());
    cudaEventDestroy(m.start);
    cudaEventDestroy(m.end);
    s->pinned.put(m.fail, sizeof(int32_t));
    c.inflight.pop_front();
  }
}

// Frees the memory of retired cohorts.
bool release_retired(eqs_server* s) {
  const double t0 = s->now();
  bool any = false;
  for (auto& c : s->cohorts)
    if (c->b && c->retired) {
      release_cohort(s, *c);
      for (Req* q : c->reqs)
        if (q->taken) s->reqs.erase(q->id);
      any = true;
    }
  s->cohorts.erase(std::remove_if(s->cohorts.begin(), s->cohorts.end(),
                                  [](const std::unique_ptr<Cohort>& c) { return !c->b; }),
                   s->cohorts.end());
  s->st.release_s += s->now() - t0;
  return any;
}

// Puts request q into slots t .. t + n_species - 1 of cohort c (already holding its
// traps' grids): cells, coupling, readout buffers; its first step is the cohort's next.
void place(eqs_server* s, Cohort& c, Req* q, int t, double now) {
  for (int k = 0; k < q->r.n_species; ++k) c.slot_owner[t + k] = q;
  q->trap0 = t;
  q->step0 = c.launched;
  q->cohort = c.id;
  q->t_admit = now;
  if (q->r.n_cells > 0) {
    ckb(eqf_set_cells(c.b, t, q->r.n_cells, q->xy.data(), q->s.data()), c.b);
    if (q->r.n_species == 2)  // species 2 takes the same cells
      ckb(eqf_couple_species(c.b, t, t + 1, q->sender.data(), q->r.vmax, q->r.K, q->r.uptake),
          c.b);
  }
  q->h_cells = static_cast<double*>(s->pinned.get(cells_bytes(q)));
  if (q->r.want_nodal) q->h_nodal = static_cast<double*>(s->pinned.get(nodal_bytes(q)));
  if (!q->h_cells || (q->r.want_nodal && !q->h_nodal))
    throw Fail{EQF_ERR_NOMEM, "page-locked host memory exhausted"};
  c.steps_target = std::max(c.steps_target, q->end_step());
}

// Slots t .. are free and the request's grids fit them at every level (the spans
// eqf_slot_fits compares, computed once per request and per cohort)
bool fits(const Cohort& c, const Req* q, int t) {
  if (t + q->r.n_species > (int)c.slot_cap.size() || q->levels != c.levels) return false;
  const int L = c.levels;
  for (int k = 0; k < q->r.n_species; ++k) {
    if (c.slot_owner[t + k]) return false;
    const long long* cap = c.cap_spans.data() + (size_t)(t + k) * L;
    const long long* need = q->spans.data() + (size_t)k * L;
    for (int l = 0; l < L; ++l)
      if (need[l] > cap[l]) return false;
  }
  return true;
}

// Matches waiting requests of the cohort's class to its free slots, oldest first, each
// into the free run of slots with the smallest capacity that fits (so large slots stay
// for large requests).  Returns the matches as (request, first slot); with apply, also
// marks the slots taken.
std::vector<std::pair<Req*, int>> match_slots(eqs_server* s, Cohort& c, bool apply,
                                              bool first_only = false) {
  std::vector<std::pair<Req*, int>> out;
  std::vector<int> free_at;  // first slots of the free runs
  for (int t = 0; t < (int)c.slot_owner.size(); ++t)
    if (!c.slot_owner[t]) free_at.push_back(t);
  int free_slots = (int)free_at.size();
  if (free_slots == 0) return out;
  constexpr size_t kWindow = 1024;
  size_t seen = 0;
  for (Req* q : s->pending) {
    if (++seen > kWindow || free_slots == 0 || (first_only && !out.empty())) break;
    if (q->klass != c.klass || q->picked) continue;
    int best = -1;
    int64_t best_cap = 0;
    for (int t : free_at) {
      if (!fits(c, q, t)) continue;
      int64_t cap = 0;
      for (int k = 0; k < q->r.n_species; ++k)
        cap += (int64_t)(c.slot_cap[t + k].nx + 1) * (c.slot_cap[t + k].ny + 1);
      if (best < 0 || cap < best_cap) {
        best = t;
        best_cap = cap;
      }
    }
    if (best < 0) continue;
    for (int k = 0; k < q->r.n_species; ++k) c.slot_owner[best + k] = q;
    free_slots -= q->r.n_species;
    out.push_back({q, best});
  }
  if (!apply)
    for (auto& m : out)
      for (int k = 0; k < m.first->r.n_species; ++k) c.slot_owner[m.second + k] = nullptr;
  return out;
}

// Admits waiting requests into the cohort's free slots: one eqf_replace_traps call for
// all of them, then their cells.  Runs when the cohort has no step queued (the cell
// index rebuild at its next step then waits for nothing of its own).
bool fill_slots(eqs_server* s, Cohort& c) {
  const double t0 = s->now();
  std::vector<std::pair<Req*, int>> m = match_slots(s, c, true);
  if (m.empty()) return false;
  std::vector<int32_t> tr;
  std::vector<eqf_trap_params> tp;
  for (auto& e : m)
    for (int k = 0; k < e.first->r.n_species; ++k) {
      tr.push_back(e.second + k);
      tp.push_back(e.first->r.species[k]);
    }
  const int rc = eqf_replace_traps(c.b, (int32_t)tr.size(), tr.data(), tp.data());
  if (rc != EQF_OK) {  // nothing changed: the requests stay in the queue
    for (auto& e : m)
      for (int k = 0; k < e.first->r.n_species; ++k) c.slot_owner[e.second + k] = nullptr;
    s->err = eqf_last_error(c.b);
    return false;
  }
  const double now = s->now();
  size_t k = 0;
  auto take_placed = [&] {  // the placed requests leave the queue; the rest stay
    s->pending.erase(std::remove_if(s->pending.begin(), s->pending.end(),
                                    [](const Req* q) { return q->picked; }),
                     s->pending.end());
  };
  try {
    for (; k < m.size(); ++k) {
      place(s, c, m[k].first, m[k].second, now);
      m[k].first->picked = true;
      c.reqs.push_back(m[k].first);
      c.remaining += 1;
    }
  } catch (...) {
    for (size_t j = k; j < m.size(); ++j)
      for (int q = 0; q < m[j].first->r.n_species; ++q) c.slot_owner[m[j].second + q] = nullptr;
    take_placed();
    throw;
  }
  take_placed();
  s->st.admitted += (int64_t)m.size();
  s->st.slot_admitted += (int64_t)m.size();
  s->st.fills += 1;
  s->st.fill_s += s->now() - t0;
  c.refilled = true;
  return true;
}

// Forms one cohort from the queue within the budget: the oldest request first, then
// the waiting requests of its class with the nearest step counts (a cohort runs
// until its longest request is done; requests of similar length keep its slots
// busy), ties in arrival order.  Cohorts are class-pure (same multigrid depth and
// Krylov method), so a request's result is the same bits whichever requests share
// its cohort.
bool admit(eqs_server* s) {
  Req* head = s->pending.front();
  const int64_t klass = head->klass;
  // candidates: the oldest waiting requests of the head's class (a bounded window, so
  // an admission costs the same however long the queue is)
  constexpr size_t kWindow = 2048;
  std::vector<Req*> cand;
  for (Req* q : s->pending) {
    if (cand.size() >= kWindow) break;
    if (q != head && q->klass == klass) cand.push_back(q);
  }
  std::stable_sort(cand.begin(), cand.end(), [&](const Req* a, const Req* b) {
    return std::abs(a->r.steps - head->r.steps) < std::abs(b->r.steps - head->r.steps);
  });
  cand.insert(cand.begin(), head);
  std::vector<Req*> take;
  int traps = 0;
  int64_t free_bytes = s->cfg.hbm_budget - s->st.bytes_in_use;
  int64_t bytes = 0;
  for (Req* q : cand) {
    if (traps + q->ntraps() > s->cfg.max_cohort_traps) break;
    take.push_back(q);
    int64_t b = estimate(s, take);
    if (b > free_bytes && release_retired(s)) free_bytes = s->cfg.hbm_budget - s->st.bytes_in_use;
    if (b > free_bytes) {
      take.pop_back();
      break;
    }
    bytes = b;
    traps += q->ntraps();
  }
  if (take.empty()) return false;
  for (Req* q : take) q->picked = true;
  s->pending.erase(std::remove_if(s->pending.begin(), s->pending.end(),
                                  [](const Req* q) { return q->picked; }),
                   s->pending.end());
  std::unique_ptr<Cohort> c(new Cohort);
  c->id = s->next_cohort++;
  c->klass = klass;
  c->reqs = take;
  c->bytes = bytes;
  c->remaining = (int)take.size();
  std::vector<eqf_trap_params> tp;
  int64_t cells = 0;
  trap_list(take, tp, cells);
  eqf_solver_opts o = s->cfg.opts;
  o.adaptive = 1;  // the added sweeps run inside the step's graph: no host round trip
  o.use_graph = 1;
  const int rc = eqf_create((int32_t)tp.size(), tp.data(), &o, &c->b);
  if (rc != EQF_OK) {
    // put the requests back in arrival order and retry once memory frees up; with
    // nothing running no memory will free up: the oldest request fails
    for (Req* q : take) {
      q->picked = false;
      s->pending.push_back(q);
    }
    std::sort(s->pending.begin(), s->pending.end(),
              [](const Req* a, const Req* b) { return a->id < b->id; });
    if ((rc == EQF_ERR_NOMEM || rc == EQF_ERR_CUDA) && !s->cohorts.empty()) return false;
    Req* q = s->pending.front();
    s->pending.pop_front();
    s->err = eqf_last_error(nullptr);
    finish(s, q, rc);
    return true;
  }
  s->st.bytes_in_use += bytes;
  s->st.bytes_peak = std::max(s->st.bytes_peak, s->st.bytes_in_use);
  void* stream = nullptr;
  ckb(eqf_stream(c->b, &stream), c->b);
  c->stream = (cudaStream_t)stream;
  c->slot_cap = tp;
  c->levels = head->levels;
  c->cap_spans.resize(tp.size() * (size_t)c->levels);
  for (size_t k = 0; k < tp.size(); ++k)
    eqf_internal_trap_spans(tp[k], c->levels, c->cap_spans.data() + k * (size_t)c->levels);
  c->slot_owner.assign(tp.size(), nullptr);
  int t = 0;
  const double now = s->now();
  for (Req* q : take) {
    place(s, *c, q, t, now);
    t += q->ntraps();
  }
  s->st.admitted += (int64_t)take.size();
  s->st.cohorts += 1;
  s->cohorts.push_back(std::move(c));
  return true;
}

void progress(eqs_server* s) {
  const double now = s->now();
  bool running = false;
  for (auto& c : s->cohorts) running = running || (c->b && !c->retired);
  if (running) s->st.busy_s += now - s->last_progress;
  s->last_progress = now;
  // retire finished steps; a cohort whose requests are all done is retired and its
  // device memory goes back to the memory pool at once (stream-ordered frees: no wait
  // for the other cohorts' work)
  for (auto& c : s->cohorts) retire(s, *c);
  // slot reuse: a cohort with free slots (a quarter of them, or all its requests done)
  // that waiting requests of its class fit queues no further step; once its queued
  // steps are done the requests go into the slots (one rebuild) and it resumes.
  // Cohorts of fewer than half the traps a cohort may hold (formed while few requests
  // waited) are not refilled: they run out and make room for full-size ones.  So is
  // one cohort while the oldest waiting request has waited a second and fits no
  // resident cohort (another class, or a grid larger than the free slots): it runs out
  // and the request heads the next cohort.
  if (s->cfg.reuse_slots) {
    int live_now = 0;
    for (auto& c : s->cohorts) live_now += c->b && !c->retired ? 1 : 0;
    const bool starving = !s->pending.empty() && live_now >= s->cfg.max_cohorts &&
                          now - s->pending.front()->t_submit > 1.0;
    if (starving) {
      Req* head = s->pending.front();
      bool any_closing = false, fits_some = false;
      Cohort* victim = nullptr;
      for (auto& c : s->cohorts) {
        if (!c->b || c->retired) continue;
        any_closing = any_closing || c->closing;
        if (c->closing || c->klass != head->klass) continue;
        for (int t = 0; t + head->r.n_species <= (int)c->slot_cap.size() && !fits_some; ++t)
          fits_some = fits(*c, head, t);
      }
      if (!any_closing && !fits_some)
        for (auto& c : s->cohorts)
          if (c->b && !c->retired && !c->filling &&
              (!victim || c->remaining < victim->remaining))
            victim = c.get();
      if (victim) victim->closing = true;
    }
    for (auto& c : s->cohorts) {
      if (!c->b || c->retired || c->closing ||
          2 * (int)c->slot_owner.size() < s->cfg.max_cohort_traps)
        continue;
      if (!c->filling) {
        int free_slots = 0;
        for (Req* o : c->slot_owner) free_slots += o ? 0 : 1;
        const int n = (int)c->slot_owner.size();
        const bool ready = free_slots > 0 && (4 * free_slots >= n || c->remaining == 0);
        // match again only when that could change the answer
        if (ready && (!c->was_ready || c->seen_submitted != s->st.submitted || c->slots_freed)) {
          c->seen_submitted = s->st.submitted;
          c->slots_freed = false;
          c->filling = !match_slots(s, *c, false, true).empty();
        }
        c->was_ready = ready;
      }
      if (c->filling && c->inflight.empty()) {
        try {
          fill_slots(s, *c);
        } catch (const Fail& f) {
          s->err = f.msg;
          fail_cohort(s, *c, f.code);
        }
        c->filling = false;
      }
    }
  }
  bool retired_any = false;
  for (auto& c : s->cohorts)
    if (c->b && !c->retired && !c->filling && c->remaining == 0 && c->inflight.empty()) {
      int idle = 0;
      const int rc = eqf_poll(c->b, &idle);  // the steps are done: reports deferred errors
      if (rc == EQF_ERR_NOT_CONVERGED)
        for (Req* q : c->reqs) q->status = rc;
      c->retired = true;
      retired_any = true;
    }
  if (retired_any) release_retired(s);
  int live = 0;
  for (auto& c : s->cohorts) live += c->b && !c->retired ? 1 : 0;
  // admit: an idle GPU, enough waiting requests, or a request waiting too long
  const double ta = s->now();
  while (!s->pending.empty() && live < s->cfg.max_cohorts) {
    const bool idle = live == 0;
    const bool enough = (int)s->pending.size() >= s->cfg.min_batch;
    const bool late = (now - s->pending.front()->t_submit) * 1e3 >= s->cfg.max_wait_ms;
    if (!(idle || enough || late)) break;
    if (!admit(s)) break;
    ++live;
  }
  const double tl = s->now();
  s->st.admit_s += tl - ta;
  // keep every cohort's queue filled
  for (auto& c : s->cohorts) {
    if (c->retired || c->filling) continue;
    try {
      while (c->launched < c->steps_target && (int)c->inflight.size() < s->cfg.steps_in_flight) {
        const double t1 = s->now();
        const bool first = c->launched == 0, refill = c->refilled;
        c->refilled = false;
        launch_step(s, *c);
        if (first) s->st.first_step_s += s->now() - t1;
        if (refill) s->st.refill_step_s += s->now() - t1;
      }
    } catch (const Fail& f) {
      s->err = f.msg;
      fail_cohort(s, *c, f.code);
    }
  }
  s->st.launch_s += s->now() - tl;
  int64_t run = 0;
  for (auto& c : s->cohorts)
    if (!c->retired) run += (int64_t)c->reqs.size();
  s->st.pending = (int64_t)s->pending.size();
  s->st.running = run;
}

double percentile(std::vector<float> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = p * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int eqs_default_config(eqs_config* c) {
  if (!c) return EQF_ERR_INVALID;
  std::memset(c, 0, sizeof(*c));
  eqf_default_opts(EQF_PREC_FP32_IR, &c->opts);
  c->hbm_budget = (int64_t)150 << 30;
  c->max_cohorts = 8;
  c->max_cohort_traps = 256;
  c->min_batch = 16;
  c->max_wait_ms = 20.0;
  c->steps_in_flight = 4;
  c->reuse_slots = 1;
  return EQF_OK;
}

int eqs_create(const eqs_config* cfg, eqs_server** out) {
  if (!cfg || !out) return EQF_ERR_INVALID;
  if (cfg->hbm_budget <= 0 || cfg->max_cohorts < 1 || cfg->max_cohort_traps < 2 ||
      cfg->min_batch < 1 || cfg->steps_in_flight < 1 || !(cfg->max_wait_ms >= 0))
    return EQF_ERR_INVALID;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return EQF_ERR_NO_DEVICE;
  eqs_server* s = new (std::nothrow) eqs_server;
  if (!s) return EQF_ERR_NOMEM;
  s->cfg = *cfg;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&s->pool, dev) == cudaSuccess &&
      cudaMemPoolGetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &s->pool_threshold0) ==
          cudaSuccess) {
    uint64_t keep = (uint64_t)cfg->hbm_budget;
    if (keep > s->pool_threshold0)
      cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  } else {
    s->pool = nullptr;
  }
  *out = s;
  return EQF_OK;
}

int eqs_destroy(eqs_server* s) {
  if (!s) return EQF_ERR_INVALID;
  for (auto& c : s->cohorts)
    if (c->b) {
      eqf_sync(c->b);
      release_cohort(s, *c);
    }
  if (s->pool) {
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &s->pool_threshold0);
    cudaMemPoolTrimTo(s->pool, 0);
  }
  delete s;  // the arena's slabs go with it (no copy into them is left in flight)
  return EQF_OK;
}

const char* eqs_last_error(const eqs_server* s) { return s ? s->err.c_str() : ""; }

int eqs_submit(eqs_server* s, const eqs_request* r, int64_t* id) {
  if (!s || !r || !id) return EQF_ERR_INVALID;
  return guarded(s, [&] {
    if (!(r->n_species == 1 || r->n_species == 2) || r->steps < 1 || r->n_cells < 0 ||
        (r->n_cells > 0 && (!r->xy || !r->s)) ||
        (r->n_species == 2 && r->n_cells > 0 && !r->sender))
      throw Fail{EQF_ERR_INVALID, "bad request"};
    const eqf_trap_params& p = r->species[0];
    if (p.nx < 1 || p.ny < 1 || !(p.width > 0) || !(p.height > 0))
      throw Fail{EQF_ERR_INVALID, "bad trap"};
    if (r->n_species == 2) {
      const eqf_trap_params& p2 = r->species[1];
      if (p2.nx != p.nx || p2.ny != p.ny || p2.width != p.width || p2.height != p.height)
        throw Fail{EQF_ERR_INVALID, "the two species must share the mesh"};
    }
    std::unique_ptr<Req> q(new Req);
    q->r = *r;
    q->xy.assign(r->xy, r->xy + 2 * r->n_cells);
    q->s.assign(r->s, r->s + r->n_cells);
    if (r->n_species == 2) q->sender.assign(r->sender, r->sender + r->n_cells);
    q->r.xy = q->xy.data();
    q->r.s = q->s.data();
    q->r.sender = q->sender.data();
    q->n_nodes = (int64_t)(p.nx + 1) * (p.ny + 1);
    int levels = 0;
    bool adv = false;
    for (int k = 0; k < r->n_species; ++k) {
      levels = std::max(levels, eqf_internal_trap_levels(r->species[k]));
      adv = adv || (r->species[k].adv_u != 0.0 && r->species[k].adv_len > 0.0);
    }
    q->klass = 2 * (int64_t)levels + (adv ? 1 : 0);
    q->levels = levels;
    q->spans.resize((size_t)r->n_species * levels);
    for (int k = 0; k < r->n_species; ++k)
      eqf_internal_trap_spans(r->species[k], levels, q->spans.data() + (size_t)k * levels);
    if (estimate(s, {q.get()}) > s->cfg.hbm_budget)
      throw Fail{EQF_ERR_TOO_LARGE, "request larger than the server's memory budget"};
    q->id = s->next_id++;
    q->t_submit = s->now();
    *id = q->id;
    s->pending.push_back(q.get());
    s->reqs[q->id] = std::move(q);
    s->st.submitted += 1;
  });
}

int eqs_progress(eqs_server* s) {
  if (!s) return EQF_ERR_INVALID;
  return guarded(s, [&] { progress(s); });
}

int eqs_take_done(eqs_server* s, int64_t* ids, int32_t cap, int32_t* n) {
  if (!s || !n || cap < 0 || (cap > 0 && !ids)) return EQF_ERR_INVALID;
  const int32_t k = (int32_t)std::min<size_t>((size_t)cap, s->done_ids.size());
  std::copy(s->done_ids.begin(), s->done_ids.begin() + k, ids);
  s->done_ids.erase(s->done_ids.begin(), s->done_ids.begin() + k);
  *n = k;
  return EQF_OK;
}

int eqs_result(eqs_server* s, int64_t id, double* cells, double* nodal, eqs_result_info* info) {
  if (!s) return EQF_ERR_INVALID;
  return guarded(s, [&] {
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) throw Fail{EQF_ERR_INVALID, "unknown request id"};
    Req* q = it->second.get();
    if (!q->done) throw Fail{EQF_ERR_INVALID, "request not finished"};
    if (cells && q->h_cells && q->r.n_cells > 0)
      std::memcpy(cells, q->h_cells, sizeof(double) * q->r.n_cells * q->r.n_species);
    if (nodal && q->h_nodal)
      std::memcpy(nodal, q->h_nodal, sizeof(double) * q->n_nodes * q->r.n_species);
    if (info) {
      info->t_submit = q->t_submit;
      info->t_admit = q->t_admit;
      info->t_done = q->t_done;
      info->steps = q->r.steps;
      info->status = q->status;
      info->n_nodes = q->n_nodes;
      info->n_cells = q->r.n_cells;
      info->n_species = q->r.n_species;
      info->cohort = q->cohort;
    }
    // no copy writes these buffers after the request finished
    s->pinned.put(q->h_cells, cells_bytes(q));
    s->pinned.put(q->h_nodal, nodal_bytes(q));
    q->h_cells = q->h_nodal = nullptr;
    q->taken = true;
    // the object itself stays while a live cohort still refers to it
    bool live = false;
    for (auto& c : s->cohorts)
      for (Req* r : c->reqs) live = live || r == q;
    if (!live) s->reqs.erase(it);
  });
}

int eqs_get_stats(eqs_server* s, eqs_stats* out) {
  if (!s || !out) return EQF_ERR_INVALID;
  *out = s->st;
  out->step_samples = (int64_t)s->step_ms.size();
  out->step_ms_p50 = percentile(s->step_ms, 0.50);
  out->step_ms_p99 = percentile(s->step_ms, 0.99);
  out->step_ms_p999 = percentile(s->step_ms, 0.999);
  return EQF_OK;
}

int eqs_drain(eqs_server* s) {
  if (!s) return EQF_ERR_INVALID;
  return guarded(s, [&] {
    for (;;) {
      progress(s);
      bool live = false;
      for (auto& c : s->cohorts) live = live || (c->b && !c->retired);
      if (s->pending.empty() && !live) {
        release_retired(s);
        break;
      }
      bool any = false;
      for (auto& c : s->cohorts) any = any || !c->inflight.empty();
      if (any) {
        // wait for the oldest step of some cohort instead of spinning
        for (auto& c : s->cohorts)
          if (!c->inflight.empty()) {
            cudaEventSynchronize(c->inflight.front().end);
            break;
          }
      }
    }
  });
}

}  // extern "C"
