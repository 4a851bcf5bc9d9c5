// mcrg_batch.cu -- batched and served MCRG solves.
//
// Batched (mcrg_batch_run): every request in the fast acceptance regime of
// side <= MCRG_RESIDENT_MAX_L becomes one shared-memory-resident chain (one
// CTA; levels of side >= 64 as bit planes); all chains of one side run in one
// launch and the launches of different sides run concurrently on fork / join
// streams, captured into a CUDA graph when asked.  Larger sides and the other
// acceptance regimes run on the per-lattice path afterwards.  This replaces the reference's one chain per
// MPI rank + MPI_Allreduce (src/mcrg.cpp:42,101-103).
//
// Served (mcrg_server_*): a scheduler thread admits queued requests as slots
// and device memory free up.  Memory comes from one arena of
// hbm_budget_bytes allocated at creation, so admission never calls
// cudaMalloc; each admitted resident request is launched on the stream of its
// slot, so requests that arrive while others run overlap with them on the
// device.  A request's result depends only on its own seed / replica, never
// on what ran beside it.
#include <condition_variable>
#include <cstring>
#include <ctime>
#include <algorithm>
#include <deque>
#include <map>
#include <tuple>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "mcrg_internal.cuh"

using namespace mcrg;

namespace {

constexpr int64_t kBatchBin = int64_t(1) << 24;

double mono_s() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int ilog2i(int x) {
  int l = 0;
  while ((1 << l) < x) ++l;
  return l;
}

int resident_threads(int L, bool cluster = false) {
  if (cluster && L >= 64) return L >= 128 ? 512 : 256;  // cluster updates: labelling latency, not occupancy, bounds them
  if (L <= 32) return 32;
  if (L == 64) return 64;
  if (L == 128) return 128;
  return L >= 512 ? 512 : 256;
}

void add_into(mcrg_moments* dst, const mcrg_moments* src) {
  dst->n_samples += src->n_samples;
  for (int x = 0; x < (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS; ++x) dst->S[x] += src->S[x];
  for (int x = 0; x < MCRG_MAX_LEVELS * MCRG_MAX_COUPLINGS * MCRG_MAX_COUPLINGS; ++x) {
    __int128 a = ((__int128)dst->SbS[x].hi << 64) | dst->SbS[x].lo;
    a += ((__int128)src->SbS[x].hi << 64) | src->SbS[x].lo;
    dst->SbS[x].lo = (uint64_t)a;
    dst->SbS[x].hi = (int64_t)(a >> 64);
    __int128 b = ((__int128)dst->SbSb[x].hi << 64) | dst->SbSb[x].lo;
    b += ((__int128)src->SbSb[x].hi << 64) | src->SbSb[x].lo;
    dst->SbSb[x].lo = (uint64_t)b;
    dst->SbSb[x].hi = (int64_t)(b >> 64);
  }
}

// Validates a request; returns its resolved level count or a negative code.
int check_request(const mcrg_request* r) {
  if (!r) return MCRG_EINVAL;
  if (r->L < 4 || r->L > MCRG_MAX_L || (r->L & (r->L - 1))) return MCRG_EINVAL;
  if (r->n_couplings < 1 || r->n_couplings > MCRG_MAX_COUPLINGS) return MCRG_EINVAL;
  if (r->n_eq < 0 || r->n_samples < 0 || r->sweeps_between < 0) return MCRG_EINVAL;
  if (!(r->K == r->K)) return MCRG_EINVAL;
  if (r->flags != 0 && r->flags != MCRG_UPDATE_WOLFF && r->flags != MCRG_UPDATE_SWENDSEN_WANG) return MCRG_EINVAL;
  const int mx = ilog2i(r->L) - 1;
  const int nl = r->n_levels < 0 ? mx : r->n_levels;
  if (nl > mx) return MCRG_EINVAL;
  return nl;
}

int64_t n_dev_bins(const mcrg_request* r) { return r->n_samples > 0 ? (r->n_samples + kBatchBin - 1) / kBatchBin : 0; }

// Whether a request runs as a shared-memory-resident chain: sweeps in the
// fast acceptance regime up to MCRG_RESIDENT_MAX_L, cluster updates while
// labels, levels and moments fit one CTA (L <= 256).
bool runs_resident(const mcrg_request* r, int nl) {
  const bool fast = make_accept(r->K).fast;
  if (r->flags) return cluster_resident(r->L, nl, MCRG_MAX_COUPLINGS, fast);
  return r->L <= MCRG_RESIDENT_MAX_L && fast;
}

void fill_job(ChainJob* j, const mcrg_request* r, int nl, uint8_t* state, mcrg_moments* bins) {
  memset(j, 0, sizeof *j);
  j->L = r->L;
  j->n_levels = nl;
  j->C = r->n_couplings;
  j->threads = resident_threads(r->L, r->flags != 0);
  j->key = Key{(uint32_t)r->seed, (uint32_t)(r->seed >> 32)};
  j->replica = r->replica;
  j->init = 1;
  j->store = 1;
  j->n_eq = r->n_eq;
  j->n_samples = r->n_samples;
  j->sweeps_between = r->sweeps_between;
  j->bin_size = kBatchBin;
  j->update = r->flags;
  j->bond_tb = r->flags ? bond_threshold(r->K) : 0u;
  j->state = state;
  j->bins = bins;
  j->acc = make_accept(r->K);
}

// Runs one request on the HBM-tiled path through a temporary context.
int run_tiled_request(const mcrg_request* r, int device, mcrg_moments* out) {
  mcrg_cfg cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.L = r->L;
  cfg.b = 2;
  cfg.n_levels = r->n_levels;
  cfg.n_couplings = r->n_couplings;
  cfg.K = r->K;
  cfg.seed = r->seed;
  cfg.replica = r->replica;
  cfg.device = device;
  mcrg_ctx* c = nullptr;
  int rc = mcrg_alloc(&c, &cfg);
  if (rc) return rc;
  if (r->flags) {
    rc = mcrg_cluster_update(c, r->n_eq, r->flags, nullptr);
    if (!rc) rc = mcrg_measure_cluster(c, r->n_samples, r->sweeps_between, r->flags, out, 0, nullptr, 0);
  } else {
    rc = mcrg_sweep(c, r->n_eq);
    if (!rc) rc = mcrg_measure(c, r->n_samples, r->sweeps_between, out, 0, nullptr, 0);
  }
  mcrg_free(c);
  return rc;
}

// Device buffers, pinned staging and streams of mcrg_batch_run, kept per
// device between calls so a batch does not pay allocation or stream set-up.
constexpr int kMaxGroups = 8;

struct BatchWorkspace {
  std::mutex mu;
  bool ready = false;
  uint8_t* d_state = nullptr;
  size_t state_cap = 0;
  mcrg_moments* d_bins = nullptr;
  mcrg_moments* h_bins = nullptr;  // pinned
  size_t bins_cap = 0;
  ChainJob* d_jobs = nullptr;
  ChainJob* h_jobs = nullptr;      // pinned
  size_t jobs_cap = 0;
  cudaStream_t s0 = nullptr;
  cudaStream_t ss[kMaxGroups] = {};
  cudaEvent_t ev[kMaxGroups + 1] = {};

  int reserve(size_t state_bytes, size_t n_bins, size_t n_jobs) {
    if (!ready) {
      if (cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking) != cudaSuccess) return MCRG_EIO;
      for (auto& x : ss)
        if (cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking) != cudaSuccess) return MCRG_EIO;
      for (auto& e : ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return MCRG_EIO;
      ready = true;
    }
    if (state_bytes > state_cap) {
      cudaFree(d_state);
      d_state = nullptr;
      state_cap = 0;
      if (cudaMalloc(&d_state, state_bytes) != cudaSuccess) return MCRG_ENOMEM;
      state_cap = state_bytes;
    }
    if (n_bins > bins_cap) {
      cudaFree(d_bins);
      cudaFreeHost(h_bins);
      d_bins = nullptr;
      h_bins = nullptr;
      bins_cap = 0;
      if (cudaMalloc(&d_bins, sizeof(mcrg_moments) * n_bins) != cudaSuccess ||
          cudaMallocHost(&h_bins, sizeof(mcrg_moments) * n_bins) != cudaSuccess)
        return MCRG_ENOMEM;
      bins_cap = n_bins;
    }
    if (n_jobs > jobs_cap) {
      cudaFree(d_jobs);
      cudaFreeHost(h_jobs);
      d_jobs = nullptr;
      h_jobs = nullptr;
      jobs_cap = 0;
      if (cudaMalloc(&d_jobs, sizeof(ChainJob) * n_jobs) != cudaSuccess ||
          cudaMallocHost(&h_jobs, sizeof(ChainJob) * n_jobs) != cudaSuccess)
        return MCRG_ENOMEM;
      jobs_cap = n_jobs;
    }
    return MCRG_OK;
  }
};

BatchWorkspace& workspace(int device) {
  static BatchWorkspace ws[64];
  return ws[device & 63];
}

}  // namespace

extern "C" int mcrg_batch_run(const mcrg_request* reqs, int32_t n, mcrg_result* results, int32_t device,
                              int32_t use_graph) {
  if (n < 0 || (n > 0 && (!reqs || !results))) return MCRG_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return MCRG_EIO;
  const double t_submit = mono_s();
  std::vector<int> nl(n);
  for (int i = 0; i < n; ++i) {
    memset(&results[i], 0, sizeof results[i]);
    results[i].submit_s = t_submit;
    nl[i] = check_request(&reqs[i]);
    results[i].status = nl[i] < 0 ? nl[i] : MCRG_OK;
  }
  // group resident requests by side and chain form (bit planes, cluster updates)
  std::map<std::pair<int, int>, std::vector<int>> groups;
  std::vector<int> tiled;
  size_t state_bytes = 0;
  int64_t total_bins = 0;
  std::vector<size_t> state_off(n, 0);
  std::vector<int64_t> bin_off(n, 0);
  for (int i = 0; i < n; ++i) {
    if (results[i].status) continue;
    if (runs_resident(&reqs[i], nl[i])) {
      const int mode = (make_accept(reqs[i].K).fast && reqs[i].L >= 64 ? 1 : 0) | (reqs[i].flags ? 2 : 0);
      groups[{reqs[i].L, mode}].push_back(i);
      state_off[i] = state_bytes;
      state_bytes += (size_t)reqs[i].L * reqs[i].L;
      bin_off[i] = total_bins;
      total_bins += n_dev_bins(&reqs[i]);
    } else {
      tiled.push_back(i);
    }
  }
  int rc = MCRG_OK;
  if (!groups.empty()) {
    BatchWorkspace& w = workspace(device);
    std::lock_guard<std::mutex> lk(w.mu);
    std::vector<std::pair<int, int>> ranges;  // (first job, count) per group
    std::vector<int> modes;                   // chain form per group
    std::vector<int> order;                   // job index -> request index
    const size_t n_jobs = (size_t)n - tiled.size() - (size_t)std::count_if(results, results + n, [](const mcrg_result& r) {
                            return r.status != MCRG_OK;
                          });
    const size_t nb = (size_t)(total_bins > 0 ? total_bins : 1);
    rc = w.reserve(state_bytes + 16, nb, n_jobs);
    if (!rc) {
      // largest sides first so the longest chains start earliest
      size_t k = 0;
      for (auto it = groups.rbegin(); it != groups.rend(); ++it) {
        ranges.push_back({(int)k, (int)it->second.size()});
        modes.push_back(it->first.second);
        for (int i : it->second) {
          fill_job(&w.h_jobs[k++], &reqs[i], nl[i], w.d_state + state_off[i], w.d_bins + bin_off[i]);
          order.push_back(i);
        }
      }
      cudaStream_t s0 = w.s0;
      cudaMemcpyAsync(w.d_jobs, w.h_jobs, sizeof(ChainJob) * n_jobs, cudaMemcpyHostToDevice, s0);
      cudaMemsetAsync(w.d_bins, 0, sizeof(mcrg_moments) * nb, s0);
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      if (use_graph) cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal);
      cudaEventRecord(w.ev[kMaxGroups], s0);
      for (size_t g = 0; g < ranges.size(); ++g) {
        cudaStream_t sg = w.ss[g % kMaxGroups];
        cudaStreamWaitEvent(sg, w.ev[kMaxGroups], 0);
        const ChainJob& j0 = w.h_jobs[(size_t)ranges[g].first];
        int maxlev = 0;
        for (int q = 0; q < ranges[g].second; ++q) maxlev = std::max(maxlev, w.h_jobs[(size_t)ranges[g].first + q].n_levels);
        if (launch_chain(w.d_jobs + ranges[g].first, ranges[g].second, j0.L, maxlev, MCRG_MAX_COUPLINGS, j0.threads,
                         (modes[g] & 1) != 0, sg, (modes[g] & 2) != 0) != cudaSuccess)
          rc = MCRG_EIO;
        cudaEventRecord(w.ev[g % kMaxGroups], sg);
        cudaStreamWaitEvent(s0, w.ev[g % kMaxGroups], 0);
      }
      if (use_graph) {
        if (cudaStreamEndCapture(s0, &graph) != cudaSuccess ||
            cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess || cudaGraphLaunch(exec, s0) != cudaSuccess)
          rc = MCRG_EIO;
      }
      if (total_bins > 0)
        cudaMemcpyAsync(w.h_bins, w.d_bins, sizeof(mcrg_moments) * (size_t)total_bins, cudaMemcpyDeviceToHost, s0);
      if (cudaStreamSynchronize(s0) != cudaSuccess) rc = MCRG_EIO;
      const double t_done = mono_s();
      for (int i : order) {
        const int64_t nbi = n_dev_bins(&reqs[i]);
        if (nbi == 1) {
          results[i].moments = w.h_bins[(size_t)bin_off[i]];
        } else {
          results[i].moments.n_levels = nl[i];
          results[i].moments.n_couplings = reqs[i].n_couplings;
          for (int64_t q = 0; q < nbi; ++q) add_into(&results[i].moments, &w.h_bins[(size_t)(bin_off[i] + q)]);
        }
        results[i].moments.n_levels = nl[i];
        results[i].moments.n_couplings = reqs[i].n_couplings;
        results[i].done_s = t_done;
        if (rc) results[i].status = rc;
      }
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
    }
  }
  for (int i : tiled) {
    results[i].status = run_tiled_request(&reqs[i], device, &results[i].moments);
    results[i].done_s = mono_s();
  }
  return rc;
}

// ===========================================================================
// Server
// ===========================================================================
struct mcrg_server {
  mcrg_server_cfg cfg;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_hbm;
  std::thread worker;
  std::vector<std::thread> hbm_workers;  // run HBM-path requests concurrently
  std::deque<void*> hbm_queue;           // admitted slots waiting for an HBM worker
  bool hbm_stop = false;
  bool stop = false;
  uint64_t next_ticket = 1;
  struct Req {
    uint64_t ticket;
    mcrg_request r;
    int nl;
    size_t bytes;
    double submit_s;
  };
  std::deque<Req> pending;
  std::map<uint64_t, mcrg_result> done;
  std::map<uint64_t, double> submitted;  // ticket -> submit time (pending or running)
  int64_t admitted = 0, completed = 0, in_flight = 0, bytes_in_use = 0;
  // device arena (first-fit over [0, budget))
  uint8_t* arena = nullptr;
  std::map<size_t, size_t> free_list;  // offset -> size
  int64_t budget = 0;
};

namespace {

size_t arena_alloc(mcrg_server* s, size_t bytes) {
  bytes = (bytes + 255) & ~size_t(255);
  for (auto it = s->free_list.begin(); it != s->free_list.end(); ++it) {
    if (it->second >= bytes) {
      const size_t off = it->first, sz = it->second;
      s->free_list.erase(it);
      if (sz > bytes) s->free_list[off + bytes] = sz - bytes;
      return off;
    }
  }
  return (size_t)-1;
}

void arena_free(mcrg_server* s, size_t off, size_t bytes) {
  bytes = (bytes + 255) & ~size_t(255);
  auto it = s->free_list.emplace(off, bytes).first;
  auto nx = std::next(it);
  if (nx != s->free_list.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    s->free_list.erase(nx);
  }
  if (it != s->free_list.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      s->free_list.erase(it);
    }
  }
}

size_t request_bytes(const mcrg_request* r) {
  // state + device bins + job descriptor
  return (size_t)r->L * r->L + sizeof(mcrg_moments) * (size_t)(n_dev_bins(r) > 0 ? n_dev_bins(r) : 1) +
         sizeof(ChainJob) + 3 * 256;
}

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  bool busy = false;
  uint64_t ticket = 0;
  size_t off = 0, bytes = 0;
  int nl = 0;
  mcrg_request r{};
  double submit_s = 0;
  mcrg_moments* h_bins = nullptr;  // pinned
  int64_t nb = 0;
  bool tiled = false;
};

constexpr int kHbmWorkersDefault = 16;  // HBM-path requests are small, latency-bound launches: overlap many
constexpr int kHbmWorkersMax = 256;

// One HBM-path worker: takes admitted slots from the queue and runs them on
// contexts it keeps per (L, levels, couplings), re-initialised per request so
// that no request pays a device allocation (which can synchronise the device
// and stall the other slots).
void hbm_worker(mcrg_server* s) {
  cudaSetDevice(s->cfg.device);
  std::map<std::tuple<int, int, int>, mcrg_ctx*> cache;
  for (;;) {
    Slot* sl = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_hbm.wait(lk, [&] { return s->hbm_stop || !s->hbm_queue.empty(); });
      if (s->hbm_queue.empty()) break;  // stop requested and nothing left
      sl = static_cast<Slot*>(s->hbm_queue.front());
      s->hbm_queue.pop_front();
    }
    mcrg_result res;
    memset(&res, 0, sizeof res);
    res.submit_s = sl->submit_s;
    const mcrg_request& r = sl->r;
    if (r.L > MCRG_SMEM_MAX_L && make_accept(r.K).fast) {
      const auto key = std::make_tuple(r.L, sl->nl, r.n_couplings);
      mcrg_ctx* c = nullptr;
      int rc = MCRG_OK;
      auto it = cache.find(key);
      if (it != cache.end()) {
        c = it->second;
        rc = reinit_context(c, r.K, r.seed, r.replica);
      } else {
        mcrg_cfg cfg;
        memset(&cfg, 0, sizeof cfg);
        cfg.L = r.L;
        cfg.b = 2;
        cfg.n_levels = sl->nl;
        cfg.n_couplings = r.n_couplings;
        cfg.K = r.K;
        cfg.seed = r.seed;
        cfg.replica = r.replica;
        cfg.device = s->cfg.device;
        rc = mcrg_alloc(&c, &cfg);
        if (!rc) cache[key] = c;
      }
      if (r.flags) {
        if (!rc) rc = mcrg_cluster_update(c, r.n_eq, r.flags, nullptr);
        if (!rc) rc = mcrg_measure_cluster(c, r.n_samples, r.sweeps_between, r.flags, &res.moments, 0, nullptr, 0);
      } else {
        if (!rc) rc = mcrg_sweep(c, r.n_eq);
        if (!rc) rc = mcrg_measure(c, r.n_samples, r.sweeps_between, &res.moments, 0, nullptr, 0);
      }
      res.status = rc;
    } else {  // outside the fast acceptance regime: a one-off context
      res.status = run_tiled_request(&r, s->cfg.device, &res.moments);
    }
    res.done_s = mono_s();
    std::lock_guard<std::mutex> lk(s->mu);
    s->done[sl->ticket] = res;
    s->submitted.erase(sl->ticket);
    arena_free(s, sl->off, sl->bytes);
    s->bytes_in_use -= (int64_t)sl->bytes;
    s->in_flight--;
    s->completed++;
    sl->busy = false;
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
  for (auto& kv : cache) mcrg_free(kv.second);
}

void server_loop(mcrg_server* s) {
  cudaSetDevice(s->cfg.device);
  std::vector<Slot> slots((size_t)s->cfg.slots);
  for (auto& sl : slots) {
    cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
  }
  for (;;) {
    // ---- admit
    std::vector<std::pair<Slot*, mcrg_server::Req>> launch;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      bool any_busy = false;
      for (auto& sl : slots) any_busy |= sl.busy;
      if (!any_busy && s->pending.empty()) {
        if (s->stop) break;
        s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
        continue;
      }
      for (auto& sl : slots) {
        if (sl.busy || s->pending.empty()) continue;
        mcrg_server::Req& q = s->pending.front();
        size_t off = (size_t)-1;
        if ((int64_t)q.bytes + s->bytes_in_use <= s->budget) off = arena_alloc(s, q.bytes);
        if (off == (size_t)-1) break;  // wait for memory (keeps arrival order)
        sl.busy = true;
        sl.off = off;
        sl.bytes = q.bytes;
        s->bytes_in_use += (int64_t)q.bytes;
        s->admitted++;
        s->in_flight++;
        launch.push_back({&sl, q});
        s->pending.pop_front();
      }
    }
    for (auto& lp : launch) {
      Slot& sl = *lp.first;
      const mcrg_server::Req& q = lp.second;
      sl.ticket = q.ticket;
      sl.r = q.r;
      sl.nl = q.nl;
      sl.submit_s = q.submit_s;
      sl.nb = n_dev_bins(&q.r);
      sl.tiled = !runs_resident(&q.r, q.nl);
      if (sl.tiled) continue;  // handed to the HBM workers below
      uint8_t* base = s->arena + sl.off;
      ChainJob* d_job = reinterpret_cast<ChainJob*>(base);
      mcrg_moments* d_bins = reinterpret_cast<mcrg_moments*>(base + 256);
      uint8_t* d_state = base + 256 + ((sizeof(mcrg_moments) * (size_t)(sl.nb > 0 ? sl.nb : 1) + 255) & ~size_t(255));
      ChainJob j;
      fill_job(&j, &q.r, q.nl, d_state, d_bins);
      if (!sl.h_bins) cudaMallocHost(&sl.h_bins, sizeof(mcrg_moments) * 4);
      if (sl.nb > 4) {
        cudaFreeHost(sl.h_bins);
        cudaMallocHost(&sl.h_bins, sizeof(mcrg_moments) * (size_t)sl.nb);
      }
      cudaMemcpyAsync(d_job, &j, sizeof j, cudaMemcpyHostToDevice, sl.stream);
      cudaMemsetAsync(d_bins, 0, sizeof(mcrg_moments) * (size_t)(sl.nb > 0 ? sl.nb : 1), sl.stream);
      launch_chain(d_job, 1, j.L, j.n_levels, j.C, j.threads, j.acc.fast && j.L >= 64, sl.stream, j.update != 0);
      if (sl.nb > 0)
        cudaMemcpyAsync(sl.h_bins, d_bins, sizeof(mcrg_moments) * (size_t)sl.nb, cudaMemcpyDeviceToHost, sl.stream);
      cudaEventRecord(sl.done, sl.stream);
    }
    // ---- hand HBM-path admissions to the worker pool (they run concurrently, each on its own stream)
    {
      bool any = false;
      std::lock_guard<std::mutex> lk(s->mu);
      for (auto& lp : launch)
        if (lp.first->tiled) {
          s->hbm_queue.push_back(lp.first);
          any = true;
        }
      if (any) s->cv_hbm.notify_all();
    }
    // ---- retire finished slots
    bool progressed = false;
    for (auto& sl : slots) {
      if (sl.tiled || !sl.busy) continue;  // HBM-path slots are retired by their worker
      const cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) continue;
      mcrg_result res;
      memset(&res, 0, sizeof res);
      res.submit_s = sl.submit_s;
      res.status = q == cudaSuccess ? MCRG_OK : MCRG_EIO;
      res.moments.n_levels = sl.nl;
      res.moments.n_couplings = sl.r.n_couplings;
      for (int64_t b = 0; b < sl.nb; ++b) add_into(&res.moments, &sl.h_bins[b]);
      res.done_s = mono_s();
      std::lock_guard<std::mutex> lk(s->mu);
      s->done[sl.ticket] = res;
      s->submitted.erase(sl.ticket);
      arena_free(s, sl.off, sl.bytes);
      s->bytes_in_use -= (int64_t)sl.bytes;
      s->in_flight--;
      s->completed++;
      sl.busy = false;
      progressed = true;
      s->cv_done.notify_all();
    }
    if (!progressed && launch.empty()) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  for (auto& sl : slots) {
    cudaStreamSynchronize(sl.stream);
    cudaStreamDestroy(sl.stream);
    cudaEventDestroy(sl.done);
    if (sl.h_bins) cudaFreeHost(sl.h_bins);
  }
}

}  // namespace

extern "C" {

int mcrg_server_create(mcrg_server** out, const mcrg_server_cfg* cfg) {
  if (!out || !cfg || cfg->slots < 1 || cfg->slots > 4096 || cfg->hbm_budget_bytes <= 0 || cfg->queue_capacity < 1 ||
      cfg->hbm_workers < 0 || cfg->hbm_workers > kHbmWorkersMax)
    return MCRG_EINVAL;
  *out = nullptr;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return MCRG_EIO;
  mcrg_server* s = new (std::nothrow) mcrg_server();
  if (!s) return MCRG_ENOMEM;
  s->cfg = *cfg;
  s->budget = cfg->hbm_budget_bytes;
  if (cudaMalloc(&s->arena, (size_t)s->budget) != cudaSuccess) {
    delete s;
    return MCRG_ENOMEM;
  }
  s->free_list[0] = (size_t)s->budget & ~size_t(255);
  s->worker = std::thread(server_loop, s);
  const int nw = cfg->hbm_workers > 0 ? cfg->hbm_workers : kHbmWorkersDefault;
  for (int w = 0; w < nw; ++w) s->hbm_workers.emplace_back(hbm_worker, s);
  *out = s;
  return MCRG_OK;
}

int mcrg_submit(mcrg_server* s, const mcrg_request* r, uint64_t* ticket) {
  if (!s || !r || !ticket) return MCRG_EINVAL;
  const int nl = check_request(r);
  if (nl < 0) return nl;
  const size_t bytes = request_bytes(r);
  if ((int64_t)bytes > s->budget) return MCRG_ENOSPC;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return MCRG_ECANCELED;
  if ((int)s->pending.size() >= s->cfg.queue_capacity) return MCRG_EBUSY;
  mcrg_server::Req q{s->next_ticket++, *r, nl, bytes, mono_s()};
  s->pending.push_back(q);
  s->submitted[q.ticket] = q.submit_s;
  *ticket = q.ticket;
  s->cv_work.notify_one();
  return MCRG_OK;
}

int mcrg_cancel(mcrg_server* s, uint64_t ticket) {
  if (!s) return MCRG_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  for (auto it = s->pending.begin(); it != s->pending.end(); ++it)
    if (it->ticket == ticket) {  // not admitted yet: it never reaches the device
      mcrg_result res;
      memset(&res, 0, sizeof res);
      res.status = MCRG_ECANCELED;
      res.submit_s = it->submit_s;
      res.done_s = mono_s();
      s->done[ticket] = res;
      s->submitted.erase(ticket);
      s->pending.erase(it);
      s->cv_done.notify_all();
      return MCRG_OK;
    }
  if (s->submitted.count(ticket)) return MCRG_EBUSY;  // admitted: its chain is on the device
  return s->done.count(ticket) ? MCRG_EINVAL : MCRG_ENOENT;  // finished (result not collected yet) / unknown
}

int mcrg_poll(mcrg_server* s, uint64_t ticket, mcrg_result* out) {
  if (!s || !out) return MCRG_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->done.find(ticket);
  if (it != s->done.end()) {
    *out = it->second;
    s->done.erase(it);
    return MCRG_OK;
  }
  return s->submitted.count(ticket) ? MCRG_EAGAIN : MCRG_ENOENT;
}

int mcrg_wait(mcrg_server* s, uint64_t ticket, double timeout_s, mcrg_result* out) {
  if (!s || !out) return MCRG_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto deadline = std::chrono::steady_clock::now() +
                        std::chrono::microseconds((int64_t)(timeout_s > 0 ? timeout_s * 1e6 : 0));
  for (;;) {
    auto it = s->done.find(ticket);
    if (it != s->done.end()) {
      *out = it->second;
      s->done.erase(it);
      return MCRG_OK;
    }
    if (!s->submitted.count(ticket)) return MCRG_ENOENT;
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) {
      auto it2 = s->done.find(ticket);
      if (it2 != s->done.end()) {
        *out = it2->second;
        s->done.erase(it2);
        return MCRG_OK;
      }
      return MCRG_ETIMEDOUT;
    }
  }
}

int mcrg_server_stats(mcrg_server* s, int64_t* admitted, int64_t* completed, int64_t* in_flight,
                      int64_t* bytes_in_use) {
  if (!s) return MCRG_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  if (admitted) *admitted = s->admitted;
  if (completed) *completed = s->completed;
  if (in_flight) *in_flight = s->in_flight;
  if (bytes_in_use) *bytes_in_use = s->bytes_in_use;
  return MCRG_OK;
}

int mcrg_server_destroy(mcrg_server* s) {
  if (!s) return MCRG_EINVAL;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    // requests still queued are cancelled
    for (auto& q : s->pending) {
      mcrg_result res;
      memset(&res, 0, sizeof res);
      res.status = MCRG_ECANCELED;
      res.submit_s = q.submit_s;
      s->done[q.ticket] = res;
      s->submitted.erase(q.ticket);
    }
    s->pending.clear();
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();  // returns once every admitted request is done
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->hbm_stop = true;
    s->cv_hbm.notify_all();
  }
  for (auto& t : s->hbm_workers)
    if (t.joinable()) t.join();
  cudaSetDevice(s->cfg.device);
  cudaFree(s->arena);
  delete s;
  return MCRG_OK;
}

}  // extern "C"
