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

// ---------------------------------------------------------------------------
// Chain shapes, the schedule autotuner and packs of the persistent launch
// ---------------------------------------------------------------------------
// Chain form: bit 0 = levels of side >= 64 as bit planes (fast acceptance
// regime), bit 1 = cluster updates.
int chain_mode(const mcrg_request* r) {
  return (make_accept(r->K).fast && r->L >= 64 ? 1 : 0) | (r->flags ? 2 : 0);
}

int pack_stride(int L, int nl, int C, int mode, int threads) {
  return (make_plan(L, nl, C, (mode & 1) != 0, (mode & 2) != 0, threads).bytes + 15) / 16 * 16;
}

// Threads per chain the autotuner tries for a shape.  Every candidate gives
// the same chain bit for bit (the Philox stream is keyed by site, not thread).
std::vector<int> candidate_threads(int L, int mode) {
  if (mode & 2) {  // cluster labelling: latency-bound, wide groups
    if (L <= 32) return {32};
    if (L == 64) return {128, 256, 512};
    return {256, 512};
  }
  if (L <= 16) return {32};
  if (L == 32) return {32, 64};
  if (L == 64) return {32, 64, 128};
  if (L == 128) return {64, 128, 256};
  if (L == 256) return {128, 256, 512};
  return {256, 512};
}

// One timed candidate: threads per chain, seconds per sample of one chain in
// a full wave of the trial (its latency under load), and chain samples per
// second of the whole device running only this shape (its throughput).
struct Candidate {
  int threads = 0;
  double s_sample = 0;
  double rate = 0;
  // the same chains inside 512-wide CTAs (the width a batch takes when any of
  // its shapes runs 512 threads per chain); 0 when not timed or not fitting
  double s_sample512 = 0;
  double rate512 = 0;
};

struct Schedule {
  int threads = 0;       // threads per chain of the best-throughput candidate
  double s_sample = 0;   // its seconds per sample of one chain in a full wave
  double s_tiled = -1;   // seconds per sample of the same chain on the HBM path (-1: not timed)
  std::vector<Candidate> cand;  // every candidate that fits
};

std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int, int>, Schedule> g_tune;  // (device, L, mode, levels, couplings)

// Resident sides at which the autotuner also times the HBM path.
bool tiled_candidate(int L, int mode) { return mode == 1 && L > MCRG_SMEM_MAX_L; }

// A pool packing for chains of one shape at CTA width W.
bool pack_geometry(int L, int nl, int C, int mode, int g, int W, int* per_pack, int* stride) {
  if (g > W || W % g) return false;
  *stride = pack_stride(L, nl, C, mode, g);
  int m = std::min(W / g, kPoolMaxGroups);
  while (m > 0 && m * *stride > kPoolMaxSmem) --m;
  *per_pack = m;
  return m > 0;
}

// Device buffers, pinned staging, stream and the instantiated graph of the
// persistent batch, kept per device between calls: a batch pays neither
// allocation nor graph instantiation unless it outgrows them.
struct BatchWorkspace {
  std::mutex mu;
  bool ready = false;
  int sms = 0;
  cudaStream_t s0 = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  uint8_t* d_state = nullptr;
  size_t state_cap = 0;
  uint8_t* d_buf = nullptr;  // [PoolQueue | packs | jobs]
  uint8_t* h_buf = nullptr;  // pinned twin of d_buf
  size_t buf_cap = 0;
  uint8_t* d_out = nullptr;  // [pack counter (256 B) | bins]
  mcrg_moments* h_bins = nullptr;  // pinned
  size_t bins_cap = 0;
  // the graph: upload, clear, persistent kernel, download
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t n_up = nullptr, n_clr = nullptr, n_run = nullptr, n_down = nullptr;
  std::tuple<int, int, int, void*, void*> graph_key{0, 0, 0, nullptr, nullptr};
  int64_t n_runs = 0, n_graph_builds = 0;  // persistent launches, graph instantiations

  int init(int device) {
    if (ready) return MCRG_OK;
    if (cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking) != cudaSuccess) return MCRG_EIO;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return MCRG_EIO;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1) return MCRG_EIO;
    ready = true;
    return MCRG_OK;
  }

  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    graph_key = std::make_tuple(0, 0, 0, nullptr, nullptr);
  }

  int reserve(size_t state_bytes, size_t buf_bytes, size_t n_bins) {
    if (state_bytes > state_cap) {
      cudaFree(d_state);
      d_state = nullptr;
      state_cap = 0;
      if (cudaMalloc(&d_state, state_bytes) != cudaSuccess) return MCRG_ENOMEM;
      state_cap = state_bytes;
    }
    if (buf_bytes > buf_cap) {
      drop_graph();
      cudaFree(d_buf);
      cudaFreeHost(h_buf);
      d_buf = h_buf = nullptr;
      buf_cap = 0;
      if (cudaMalloc(&d_buf, buf_bytes) != cudaSuccess || cudaMallocHost(&h_buf, buf_bytes) != cudaSuccess)
        return MCRG_ENOMEM;
      buf_cap = buf_bytes;
    }
    if (n_bins > bins_cap) {
      drop_graph();
      cudaFree(d_out);
      cudaFreeHost(h_bins);
      d_out = nullptr;
      h_bins = nullptr;
      bins_cap = 0;
      if (cudaMalloc(&d_out, 256 + sizeof(mcrg_moments) * n_bins) != cudaSuccess ||
          cudaMallocHost(&h_bins, sizeof(mcrg_moments) * n_bins) != cudaSuccess)
        return MCRG_ENOMEM;
      bins_cap = n_bins;
    }
    return MCRG_OK;
  }

  mcrg_moments* d_bins() { return reinterpret_cast<mcrg_moments*>(d_out + 256); }

  // Issues upload, clear, persistent launch and download on s0: through the
  // graph (built once per CTA width / grid / shared memory and buffers, its
  // copy sizes updated per call) or directly.
  int run(int W, int grid, int smem, size_t up_bytes, size_t n_bins, bool use_graph) {
    const size_t clr = 256 + sizeof(mcrg_moments) * n_bins;
    const size_t down = sizeof(mcrg_moments) * std::max<size_t>(n_bins, 1);
    void* q = d_buf;
    void* args[] = {&q};
    if (!use_graph) {
      if (cudaMemcpyAsync(d_buf, h_buf, up_bytes, cudaMemcpyHostToDevice, s0) != cudaSuccess ||
          cudaMemsetAsync(d_out, 0, clr, s0) != cudaSuccess ||
          cudaLaunchKernel(pool_kernel_fn(W), dim3(grid), dim3(W), args, (size_t)smem, s0) != cudaSuccess)
        return MCRG_EIO;
      if (n_bins && cudaMemcpyAsync(h_bins, d_bins(), down, cudaMemcpyDeviceToHost, s0) != cudaSuccess)
        return MCRG_EIO;
      return MCRG_OK;
    }
    const auto key = std::make_tuple(W, grid, smem, (void*)d_buf, (void*)d_out);
    if (!exec || key != graph_key) {
      drop_graph();
      if (cudaGraphCreate(&graph, 0) != cudaSuccess) return MCRG_EIO;
      cudaMemsetParams ms;
      memset(&ms, 0, sizeof ms);
      ms.dst = d_out;
      ms.elementSize = 1;
      ms.width = clr;
      ms.height = 1;
      cudaKernelNodeParams kp;
      memset(&kp, 0, sizeof kp);
      kp.func = const_cast<void*>(pool_kernel_fn(W));
      kp.gridDim = dim3(grid);
      kp.blockDim = dim3(W);
      kp.sharedMemBytes = (unsigned)smem;
      kp.kernelParams = args;
      if (cudaGraphAddMemcpyNode1D(&n_up, graph, nullptr, 0, d_buf, h_buf, up_bytes, cudaMemcpyHostToDevice) !=
              cudaSuccess ||
          cudaGraphAddMemsetNode(&n_clr, graph, &n_up, 1, &ms) != cudaSuccess ||
          cudaGraphAddKernelNode(&n_run, graph, &n_clr, 1, &kp) != cudaSuccess ||
          cudaGraphAddMemcpyNode1D(&n_down, graph, &n_run, 1, h_bins, d_bins(), down, cudaMemcpyDeviceToHost) !=
              cudaSuccess ||
          cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        drop_graph();
        return MCRG_EIO;
      }
      graph_key = key;
      ++n_graph_builds;
    } else {
      cudaMemsetParams ms;
      memset(&ms, 0, sizeof ms);
      ms.dst = d_out;
      ms.elementSize = 1;
      ms.width = clr;
      ms.height = 1;
      if (cudaGraphExecMemcpyNodeSetParams1D(exec, n_up, d_buf, h_buf, up_bytes, cudaMemcpyHostToDevice) !=
              cudaSuccess ||
          cudaGraphExecMemsetNodeSetParams(exec, n_clr, &ms) != cudaSuccess ||
          cudaGraphExecMemcpyNodeSetParams1D(exec, n_down, h_bins, d_bins(), down, cudaMemcpyDeviceToHost) !=
              cudaSuccess)
        return MCRG_EIO;
    }
    return cudaGraphLaunch(exec, s0) == cudaSuccess ? MCRG_OK : MCRG_EIO;
  }
};

BatchWorkspace& workspace(int device) {
  static BatchWorkspace ws[64];
  return ws[device & 63];
}

// Lays out [PoolQueue | packs | jobs] in the workspace's pinned staging with
// device pointers, and returns the bytes used.
// The packs must be ordered by class; class_first[k] is the first pack of
// class k (class_first[n] = packs.size()), class_work[k] its estimated work.
size_t stage_queue(BatchWorkspace& w, const std::vector<PoolPack>& packs, const std::vector<ChainJob>& jobs,
                   const std::vector<int>& class_first = {}, const std::vector<double>& class_work = {}) {
  const size_t off_packs = 128;
  const size_t off_jobs = (off_packs + sizeof(PoolPack) * packs.size() + 255) & ~size_t(255);
  static_assert(sizeof(PoolQueue) <= 128, "queue header");
  PoolQueue q;
  memset(&q, 0, sizeof q);
  q.n_packs = (int32_t)packs.size();
  q.packs = reinterpret_cast<const PoolPack*>(w.d_buf + off_packs);
  q.jobs = reinterpret_cast<const ChainJob*>(w.d_buf + off_jobs);
  q.next = reinterpret_cast<unsigned*>(w.d_out);
  const char* pc = getenv("MCRG_POOL_CLASSES");
  const bool classes = !(pc && pc[0] == '0') && class_first.size() >= 2;
  if (!classes) {  // one class: every CTA takes every pack in order
    q.n_classes = 1;
    q.first[0] = 0;
    q.first[1] = (int32_t)packs.size();
  } else {
    const int nc = std::min((int)class_first.size() - 1, kPoolClasses);
    double tot = 0;
    for (int k = 0; k < nc; ++k) tot += class_work[(size_t)k];
    q.n_classes = nc;
    double acc = 0;
    for (int k = 0; k <= nc; ++k) {
      q.first[k] = class_first[(size_t)k];
      q.sm_edge[k] = (int32_t)(tot > 0 ? acc / tot * 65536.0 : 0.0);
      if (k < nc) acc += class_work[(size_t)k];
    }
  }
  memcpy(w.h_buf, &q, sizeof q);
  if (!packs.empty()) memcpy(w.h_buf + off_packs, packs.data(), sizeof(PoolPack) * packs.size());
  if (!jobs.empty()) memcpy(w.h_buf + off_jobs, jobs.data(), sizeof(ChainJob) * jobs.size());
  return off_jobs + sizeof(ChainJob) * jobs.size();
}

size_t queue_bytes(size_t n_packs, size_t n_jobs) {
  return ((128 + sizeof(PoolPack) * n_packs + 255) & ~size_t(255)) + sizeof(ChainJob) * n_jobs;
}

// One trial of the autotuner: a full wave of chains of one shape at `g`
// threads each, S samples per chain; returns seconds per sample of a chain
// (the wave's time / S) or -1 when the shape does not fit that way.
double trial_pool(BatchWorkspace& w, int L, int nl, int C, int mode, int g, int W) {
  int m = 0, stride = 0, occ = 0;
  if (!pack_geometry(L, nl, C, mode, g, W, &m, &stride)) return -1;
  if (pool_prepare(W, m * stride, &occ) != cudaSuccess || occ < 1) return -1;
  const int n_chains = std::min(w.sms * occ * m, 4096);
  const int S = std::max(2, std::min(64, 262144 / (L * L)));
  std::vector<ChainJob> jobs((size_t)n_chains);
  std::vector<PoolPack> packs;
  if (w.reserve((size_t)n_chains * L * L + 16, queue_bytes((size_t)n_chains, (size_t)n_chains), (size_t)n_chains))
    return -1;
  mcrg_request r;
  memset(&r, 0, sizeof r);
  r.L = L;
  r.n_couplings = C;
  r.K = -0.44068679350977147;  // critical coupling: the open-site rate of the batched workloads
  r.flags = (mode & 2) ? MCRG_UPDATE_SWENDSEN_WANG : 0;
  r.n_samples = S;
  r.sweeps_between = 1;
  for (int i = 0; i < n_chains; ++i) {
    r.seed = 0x7A11u + (uint64_t)i;
    fill_job(&jobs[(size_t)i], &r, nl, w.d_state + (size_t)i * L * L, w.d_bins() + i);
    jobs[(size_t)i].threads = g;
    jobs[(size_t)i].store = 0;
  }
  for (int i = 0; i < n_chains; i += m) packs.push_back(PoolPack{i, (int16_t)std::min(m, n_chains - i), (int16_t)g, stride, 0});
  const size_t up = stage_queue(w, packs, jobs);
  const int grid = std::min((int)packs.size(), w.sms * occ);
  double best = -1;
  for (int rep = 0; rep < 3; ++rep) {
    if (cudaEventRecord(w.e0, w.s0) != cudaSuccess || w.run(W, grid, m * stride, up, 0, false) != MCRG_OK ||
        cudaEventRecord(w.e1, w.s0) != cudaSuccess || cudaEventSynchronize(w.e1) != cudaSuccess)
      return -1;
    float ms = 0;
    cudaEventElapsedTime(&ms, w.e0, w.e1);
    if (rep > 0 && (best < 0 || ms < best)) best = ms;  // first run: warm-up
  }
  return best * 1e-3 / S;
}

double trial_tiled(int device, int L, int nl, int C) {
  mcrg_cfg cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.L = L;
  cfg.b = 2;
  cfg.n_levels = nl;
  cfg.n_couplings = C;
  cfg.K = -0.44068679350977147;
  cfg.seed = 0x7A11u;
  cfg.device = device;
  mcrg_ctx* c = nullptr;
  if (mcrg_alloc(&c, &cfg)) return -1;
  mcrg_moments m;
  const int S = 8;
  double best = -1;
  for (int rep = 0; rep < 3 && c; ++rep) {
    const double t0 = mono_s();
    if (mcrg_measure(c, S, 1, &m, 0, nullptr, 0)) break;
    const double dt = mono_s() - t0;
    if (rep > 0 && (best < 0 || dt < best)) best = dt;
  }
  mcrg_free(c);
  return best > 0 ? best / S : -1;
}

// The schedule of a shape: cached, or tuned now by timed trials on the
// workspace's stream.  MCRG_POOL_THREADS=<threads> forces the threads per
// chain of every shape it is a candidate for (not cached).
Schedule schedule_for(BatchWorkspace& w, int device, int L, int nl, int C, int mode) {
  const char* force = getenv("MCRG_POOL_THREADS");
  int forced = force ? atoi(force) : 0;
  {
    const std::vector<int> cand = candidate_threads(L, mode);
    if (std::find(cand.begin(), cand.end(), forced) == cand.end()) forced = 0;
  }
  const auto key = std::make_tuple(device, L, mode, nl, C);
  if (!forced) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return it->second;
  }
  Schedule best;
  double best_rate = -1;
  // chain samples per second of the device running only this shape at width W
  auto device_rate = [&](int g, int W, double t) {
    int m = 0, stride = 0, occ = 0;
    pack_geometry(L, nl, C, mode, g, W, &m, &stride);
    pool_prepare(W, m * stride, &occ);
    return (double)w.sms * occ * m / t;
  };
  for (int g : candidate_threads(L, mode)) {
    if (forced && g != forced) continue;
    const int W = g > 256 ? 512 : 256;
    const double t = trial_pool(w, L, nl, C, mode, g, W);
    if (t <= 0) continue;
    Candidate cd{g, t, device_rate(g, W, t), 0, 0};
    if (W == 512) {
      cd.s_sample512 = cd.s_sample;
      cd.rate512 = cd.rate;
    } else {
      const double t5 = trial_pool(w, L, nl, C, mode, g, 512);
      if (t5 > 0) {
        cd.s_sample512 = t5;
        cd.rate512 = device_rate(g, 512, t5);
      }
    }
    const double rate = cd.rate;
    best.cand.push_back(cd);
    if (rate > best_rate) {
      best_rate = rate;
      best.threads = g;
      best.s_sample = t;
    }
  }
  if (!best.threads) {  // nothing fit (should not happen for resident shapes): the fixed rule
    best.threads = resident_threads(L, (mode & 2) != 0);
    best.s_sample = 0;
    best.cand.push_back(Candidate{best.threads, 0.0, 0.0, 0.0, 0.0});
  }
  if (forced) return best;
  if (tiled_candidate(L, mode)) best.s_tiled = trial_tiled(device, L, nl, C);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = best;
  return best;
}

// Requests of one chain shape in a batch and their packing.
struct Shape {
  int L, mode, nl, C, g, per_pack, stride;
  std::vector<int> reqs;
};

// Work of a chain in sample units (a sample is one sweep or update plus one
// measurement; a bare sweep or update counts half).
double chain_samples(const mcrg_request& q) {
  const double sweeps = (double)q.n_eq + (double)q.n_samples * (double)(q.sweeps_between > 1 ? q.sweeps_between - 1 : 0);
  return (double)q.n_samples + 0.5 * sweeps;
}

// Threads per chain for every shape of a batch, and so the CTA width: the
// combination of timed candidates with the smallest estimated makespan,
// max(longest chain × its latency, Σ work / throughput), each shape's
// latency and throughput taken at the width the combination implies (512
// when any shape runs 512 threads per chain, else 256) -- the best-throughput
// pick alone can leave the batch waiting on a few long, narrow chains, and a
// 512-wide launch slows the shapes that did not need it.
void choose_threads(std::vector<Shape>& sh, const std::vector<std::vector<Candidate>>& cands,
                    const mcrg_request* reqs) {
  const size_t n = sh.size();
  double combos = 1;
  for (auto& c : cands) combos *= (double)std::max<size_t>(c.size(), 1);
  if (n == 0 || combos > 65536) return;  // keep each shape's best-throughput pick
  std::vector<double> longest(n, 0), total(n, 0);
  for (size_t k = 0; k < n; ++k)
    for (int i : sh[k].reqs) {
      const double w = chain_samples(reqs[i]);
      longest[k] = std::max(longest[k], w);
      total[k] += w;
    }
  std::vector<size_t> pick(n, 0), best(n, 0);
  double best_t = -1;
  for (;;) {
    bool wide = false;
    for (size_t k = 0; k < n; ++k) wide |= cands[k][pick[k]].threads > 256;
    double lat = 0, thr = 0;
    bool ok = true;
    for (size_t k = 0; k < n; ++k) {
      const Candidate& c = cands[k][pick[k]];
      const double sr = wide ? c.s_sample512 : c.s_sample, rt = wide ? c.rate512 : c.rate;
      if (rt <= 0 || sr <= 0) ok = false;
      lat = std::max(lat, longest[k] * sr);
      thr += rt > 0 ? total[k] / rt : 0;
    }
    const double t = std::max(lat, thr);
    if (ok && (best_t < 0 || t < best_t)) {
      best_t = t;
      best = pick;
    }
    size_t k = 0;
    while (k < n && ++pick[k] == cands[k].size()) pick[k++] = 0;
    if (k == n) break;
  }
  if (best_t < 0) return;
  for (size_t k = 0; k < n; ++k) sh[k].g = cands[k][best[k]].threads;
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
  // resident requests by shape (side, chain form)
  std::map<std::pair<int, int>, std::vector<int>> shapes;
  std::vector<int> tiled;
  for (int i = 0; i < n; ++i) {
    if (results[i].status) continue;
    if (runs_resident(&reqs[i], nl[i])) shapes[{reqs[i].L, chain_mode(&reqs[i])}].push_back(i);
    else tiled.push_back(i);
  }
  int rc = MCRG_OK;
  if (!shapes.empty()) {
    BatchWorkspace& w = workspace(device);
    std::lock_guard<std::mutex> lk(w.mu);
    rc = w.init(device);
    // schedules (autotuned once per shape), the CTA width and the packs
    std::vector<Shape> sh;
    std::vector<std::vector<Candidate>> cands;
    int W = 256;
    const char* se = getenv("MCRG_BATCH_SCHEDULE");
    const int sched_env = !se ? 0 : (!strcmp(se, "resident") ? 1 : (!strcmp(se, "tiled") ? 2 : 0));
    for (auto& kv : shapes) {
      if (rc) break;
      Shape s{kv.first.first, kv.first.second, 0, 0, 0, 0, 0, kv.second};
      for (int i : s.reqs) {
        s.nl = std::max(s.nl, nl[i]);
        s.C = std::max(s.C, reqs[i].n_couplings);
      }
      const Schedule sc = schedule_for(w, device, s.L, s.nl, s.C, s.mode);
      // resident vs tiled for the largest sides: tiled when running them one after
      // another on the whole device ends before a single resident chain would
      // (MCRG_BATCH_SCHEDULE=resident / tiled forces one)
      const bool go_tiled =
          tiled_candidate(s.L, s.mode) &&
          (sched_env == 2 ||
           (sched_env == 0 && sc.s_tiled > 0 && sc.s_sample > 0 && (double)s.reqs.size() * sc.s_tiled < sc.s_sample));
      if (go_tiled) {
        tiled.insert(tiled.end(), s.reqs.begin(), s.reqs.end());
        continue;
      }
      s.g = sc.threads;
      sh.push_back(s);
      cands.push_back(sc.cand);
    }
    choose_threads(sh, cands, reqs);
    for (auto& s : sh) W = std::max(W, s.g > 256 ? 512 : 256);
    std::vector<PoolPack> packs;
    std::vector<ChainJob> jobs;
    std::vector<int> order;  // job index -> request
    std::vector<size_t> state_off(n, 0);
    std::vector<int64_t> bin_off(n, 0);
    size_t state_bytes = 0;
    int64_t total_bins = 0;
    int smem = 16;
    struct Costed {
      int cls;      // chain code: 0 byte sweeps, 1 plane sweeps, 2 cluster updates
      double cost;  // of the pack's longest chain
      double work;  // of all its chains
      PoolPack pk;
    };
    std::vector<Costed> costed;
    for (auto it = sh.begin(); it != sh.end();) {  // a shape no pack holds runs on the tiled path
      if (!pack_geometry(it->L, it->nl, it->C, it->mode, it->g, W, &it->per_pack, &it->stride)) {
        tiled.insert(tiled.end(), it->reqs.begin(), it->reqs.end());
        it = sh.erase(it);
      } else {
        ++it;
      }
    }
    for (auto& s : sh) {
      if (rc) break;
      auto cost = [&](int i) {
        const mcrg_request& q = reqs[i];
        return (double)q.L * q.L * (double)(q.n_eq + q.n_samples * (q.sweeps_between + 1));
      };
      std::stable_sort(s.reqs.begin(), s.reqs.end(), [&](int a, int b) { return cost(a) > cost(b); });
      const int cls = (s.mode & 2) ? 2 : (s.mode & 1);
      for (size_t k = 0; k < s.reqs.size(); k += (size_t)s.per_pack) {
        const int cnt = (int)std::min(s.reqs.size() - k, (size_t)s.per_pack);
        double work = 0;
        for (int q = 0; q < cnt; ++q) work += cost(s.reqs[k + (size_t)q]);
        costed.push_back({cls, cost(s.reqs[k]), work,
                          PoolPack{(int32_t)(jobs.size() + k), (int16_t)cnt, (int16_t)s.g, s.stride, 0}});
      }
      for (int i : s.reqs) {
        state_off[i] = state_bytes;
        state_bytes += (size_t)reqs[i].L * reqs[i].L;
        bin_off[i] = total_bins;
        total_bins += n_dev_bins(&reqs[i]);
        jobs.emplace_back();
        order.push_back(i);
      }
      smem = std::max(smem, s.per_pack * s.stride);
    }
    // by chain code, and longest packs first within each: the tail of the launch is short chains
    std::stable_sort(costed.begin(), costed.end(), [](const Costed& a, const Costed& b) {
      return a.cls != b.cls ? a.cls < b.cls : a.cost > b.cost;
    });
    std::vector<int> class_first;
    std::vector<double> class_work;
    for (size_t k = 0; k < costed.size(); ++k) {
      if (k == 0 || costed[k].cls != costed[k - 1].cls) {
        class_first.push_back((int)k);
        class_work.push_back(0.0);
      }
      class_work.back() += costed[k].work;
      packs.push_back(costed[k].pk);
    }
    class_first.push_back((int)costed.size());
    if (!rc && !jobs.empty()) {
      rc = w.reserve(state_bytes + 16, queue_bytes(packs.size(), jobs.size()), (size_t)std::max<int64_t>(total_bins, 1));
      if (!rc) {
        size_t k = 0;
        for (auto& s : sh)
          for (int i : s.reqs) {
            fill_job(&jobs[k], &reqs[i], nl[i], w.d_state + state_off[i], w.d_bins() + bin_off[i]);
            jobs[k].threads = s.g;
            ++k;
          }
        int occ = 0;
        if (pool_prepare(W, smem, &occ) != cudaSuccess || occ < 1) rc = MCRG_EIO;
        const int grid = std::min((int)packs.size(), w.sms * std::max(occ, 1));
        const size_t up = stage_queue(w, packs, jobs, class_first, class_work);
        if (!rc) rc = w.run(W, grid, smem, up, (size_t)total_bins, use_graph != 0);
        ++w.n_runs;
        if (cudaStreamSynchronize(w.s0) != cudaSuccess) rc = MCRG_EIO;
        const double t_done = mono_s();
        for (int i : order) {
          const int64_t nbi = n_dev_bins(&reqs[i]);
          if (nbi == 1) {
            results[i].moments = w.h_bins[(size_t)bin_off[i]];
          } else {
            for (int64_t q = 0; q < nbi; ++q) add_into(&results[i].moments, &w.h_bins[(size_t)(bin_off[i] + q)]);
          }
          results[i].moments.n_levels = nl[i];
          results[i].moments.n_couplings = reqs[i].n_couplings;
          results[i].done_s = t_done;
          if (rc) results[i].status = rc;
        }
      }
    }
    if (rc)
      for (auto& s : sh)
        for (int i : s.reqs) results[i].status = rc;
  }
  for (int i : tiled) {
    results[i].status = run_tiled_request(&reqs[i], device, &results[i].moments);
    results[i].done_s = mono_s();
  }
  return rc;
}

extern "C" int mcrg_batch_schedule(const mcrg_request* r, int32_t device, int32_t* threads, double* s_sample,
                                   double* s_tiled) {
  if (!r || !threads) return MCRG_EINVAL;
  const int nl = check_request(r);
  if (nl < 0) return nl;
  if (!runs_resident(r, nl)) return MCRG_ENOSYS;
  if (cudaSetDevice(device) != cudaSuccess) return MCRG_EIO;
  BatchWorkspace& w = workspace(device);
  std::lock_guard<std::mutex> lk(w.mu);
  const int rc = w.init(device);
  if (rc) return rc;
  const Schedule sc = schedule_for(w, device, r->L, nl, r->n_couplings, chain_mode(r));
  *threads = sc.threads;
  if (s_sample) *s_sample = sc.s_sample;
  if (s_tiled) *s_tiled = sc.s_tiled;
  return MCRG_OK;
}

extern "C" int mcrg_batch_stats(int32_t device, int64_t* launches, int64_t* graph_builds) {
  if (device < 0 || device >= 64) return MCRG_EINVAL;
  BatchWorkspace& w = workspace(device);
  std::lock_guard<std::mutex> lk(w.mu);
  if (launches) *launches = w.n_runs;
  if (graph_builds) *graph_builds = w.n_graph_builds;
  return MCRG_OK;
}

// ===========================================================================
// Server
// ===========================================================================
// Resident requests are published as packs into a ring in page-locked host
// memory and run by the persistent serve kernel (mcrg_chain.cu), whose CTAs
// claim entries as they are published and write each chain's moments into
// page-locked host bins: admission, overlap and completion need no launch
// per request and no copy.  The scheduler thread admits, publishes, restarts
// the loop when it has gone idle, and retires finished entries.  Requests no
// resident chain holds run on host worker threads, each on a context whose
// device buffers are carved from the request's reservation in the arena.
namespace {

constexpr int kServeBinsPerChain = 4;        // host bins per resident chain (2^26 samples)
constexpr int kHbmWorkersDefault = 16;
constexpr int kHbmWorkersMax = 256;
constexpr unsigned long long kServeIdleNs = 20000000ull;  // a CTA leaves after 20 ms without work
constexpr double kServeHoldS = 1e-3;  // longest wait of a pack that is not full while the loop has a backlog

struct Member {  // one admitted request
  uint64_t ticket;
  mcrg_request r;
  int nl;
  double submit_s;
  size_t off, bytes;  // arena reservation
  int bin_slot;       // resident: its host bins; -1: HBM path
};

struct EntryState {
  bool busy = false;
  uint64_t seq = 0;  // entry index + 1
  std::vector<Member> members;
};

}  // namespace

struct mcrg_server {
  mcrg_server_cfg cfg;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_hbm;
  std::thread worker;
  std::vector<std::thread> hbm_workers;
  std::deque<Member> hbm_queue;  // admitted HBM-path requests waiting for a worker
  int hbm_running = 0;
  bool hbm_stop = false;
  bool stop = false;
  uint64_t next_ticket = 1;
  struct Req {
    uint64_t ticket;
    mcrg_request r;
    int nl;
    size_t bytes;
    int threads;  // resident: threads per chain in the serve loop; 0: HBM path
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
  // the ring and its control block (page-locked, mapped), the claim counter (device)
  int sms = 0;
  uint32_t cap = 0;
  ServeEntry* ring_h = nullptr;
  ServeCtl* ctl_h = nullptr;
  unsigned int* done_h = nullptr;
  mcrg_moments* bins_h = nullptr;  // slots x kServeBinsPerChain
  mcrg_moments* bins_d = nullptr;  // the same bins, device address
  ServeArgs args{};
  std::vector<int> free_bins;  // host bin slots not in use
  std::vector<EntryState> entries;
  uint64_t published = 0;
  // launches of the loop, each on a stream of its own (a launch queued behind a
  // running one on the same stream would not start until that one ended)
  static constexpr int kMaxLoopStreams = 256;
  struct LoopStream {
    cudaStream_t stream = nullptr;
    cudaEvent_t end = nullptr;  // recorded after the stream's last launch
    bool live = false;          // that launch may still run
  };
  std::vector<LoopStream> loop_streams;
  int serve_grid = 0;                  // CTAs that fill the device
  int64_t loop_launches = 0;
  int64_t ctas_launched = 0;
  int live_launches = 0;               // launches of the loop that may still run (last count)
  // device counters (claimed, started, left) and their page-locked read-back
  unsigned long long* h_ctr = nullptr;
  unsigned long long seen[3] = {0, 0, 0};
  cudaStream_t ctr_stream = nullptr;
  cudaEvent_t ctr_done = nullptr;
  bool ctr_pending = false;
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

// Whether a request runs in the serve loop: a resident chain whose bins fit
// its host bin slot.
int serve_threads(int device, const mcrg_request* r, int nl);

// Device bytes a request holds while admitted: the final configuration of a
// resident chain (its moments go to host bins), or every buffer of the
// context an HBM-path request runs on.
size_t request_bytes(const mcrg_request* r, int nl, bool resident) {
  if (resident) return ((size_t)r->L * r->L + 255) & ~size_t(255);
  return context_bytes(r->L, nl, r->n_couplings, r->flags, r->n_samples);
}

// Threads per chain of a shape in the serve loop.  A served request waits
// for its own chain, so among the candidates the autotuner has timed for the
// shape in this process the one with the lowest latency under load is taken,
// as long as its throughput is within 20 % of the best; without timings the
// fixed rule (the server does not time trials next to running requests).
int serve_threads(int device, const mcrg_request* r, int nl) {
  const int mode = chain_mode(r);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(std::make_tuple(device, r->L, mode, nl, r->n_couplings));
  if (it == g_tune.end()) return resident_threads(r->L, r->flags != 0);
  double best_rate = 0;
  for (const Candidate& c : it->second.cand) best_rate = std::max(best_rate, c.rate);
  int g = it->second.threads;
  double lat = -1;
  for (const Candidate& c : it->second.cand)
    if (c.rate >= 0.8 * best_rate && c.s_sample > 0 && (lat < 0 || c.s_sample < lat)) {
      lat = c.s_sample;
      g = c.threads;
    }
  return g;
}

// Threads per chain when the request runs in the serve loop, 0 when it runs
// on the HBM path (no resident chain holds it, its bins exceed the host bin
// slot, or no pack of the loop's CTA fits it).
int serve_plan(const mcrg_request* r, int nl, int device) {
  if (!runs_resident(r, nl) || n_dev_bins(r) > kServeBinsPerChain) return 0;
  const int g = serve_threads(device, r, nl);
  int per = 0, stride = 0;
  return pack_geometry(r->L, nl, r->n_couplings, chain_mode(r), g, kServeThreads, &per, &stride) ? g : 0;
}

void finish(mcrg_server* s, const Member& m, const mcrg_result& res) {
  s->done[m.ticket] = res;
  s->submitted.erase(m.ticket);
  arena_free(s, m.off, m.bytes);
  s->bytes_in_use -= (int64_t)m.bytes;
  s->in_flight--;
  s->completed++;
}

// One HBM-path worker: runs admitted requests on contexts built in their
// arena reservations (no cudaMalloc), one request at a time.
void hbm_worker(mcrg_server* s) {
  cudaSetDevice(s->cfg.device);
  for (;;) {
    Member m;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_hbm.wait(lk, [&] { return s->hbm_stop || !s->hbm_queue.empty(); });
      if (s->hbm_queue.empty()) break;  // stop requested and nothing left
      m = s->hbm_queue.front();
      s->hbm_queue.pop_front();
      s->hbm_running++;
    }
    mcrg_result res;
    memset(&res, 0, sizeof res);
    res.submit_s = m.submit_s;
    const mcrg_request& r = m.r;
    DevSpan span;
    span.base = s->arena + m.off;
    span.cap = m.bytes;
    mcrg_cfg cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.L = r.L;
    cfg.b = 2;
    cfg.n_levels = m.nl;
    cfg.n_couplings = r.n_couplings;
    cfg.K = r.K;
    cfg.seed = r.seed;
    cfg.replica = r.replica;
    cfg.device = s->cfg.device;
    mcrg_ctx* c = nullptr;
    int rc = context_create(&c, &cfg, &span);
    if (!rc) {
      if (r.flags) {
        rc = mcrg_cluster_update(c, r.n_eq, r.flags, nullptr);
        if (!rc) rc = mcrg_measure_cluster(c, r.n_samples, r.sweeps_between, r.flags, &res.moments, 0, nullptr, 0);
      } else {
        rc = mcrg_sweep(c, r.n_eq);
        if (!rc) rc = mcrg_measure(c, r.n_samples, r.sweeps_between, &res.moments, 0, nullptr, 0);
      }
    }
    if (c) mcrg_free(c);
    res.status = rc;
    res.done_s = mono_s();
    std::lock_guard<std::mutex> lk(s->mu);
    s->hbm_running--;
    finish(s, m, res);
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

// Keeps the serve loop at its width: reads the device counters back (one
// small asynchronous copy in flight at a time) and, while published entries
// are unclaimed and fewer CTAs than the target are running or queued,
// launches the difference on the next stream of the pool.  Returns MCRG_EIO
// when a launch of the loop has failed.
int ensure_loop(mcrg_server* s, bool hbm_waiting) {
  int live = 0;
  mcrg_server::LoopStream* idle = nullptr;
  for (auto& ls : s->loop_streams) {  // reap finished launches
    if (ls.live) {
      const cudaError_t q = cudaEventQuery(ls.end);
      if (q == cudaSuccess) ls.live = false;
      else if (q != cudaErrorNotReady) return MCRG_EIO;
    }
    if (ls.live) ++live;
    else if (!idle) idle = &ls;
  }
  s->live_launches = live;
  if (s->ctr_pending && cudaEventQuery(s->ctr_done) == cudaSuccess) {
    for (int k = 0; k < 3; ++k) s->seen[k] = std::max(s->seen[k], s->h_ctr[k]);
    s->ctr_pending = false;
  }
  if (!s->ctr_pending && live) {
    if (cudaMemcpyAsync(s->h_ctr, s->args.ctr, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                        s->ctr_stream) == cudaSuccess &&
        cudaEventRecord(s->ctr_done, s->ctr_stream) == cudaSuccess)
      s->ctr_pending = true;
  }
  // HBM-path kernels need SMs the loop would hold: the loop leaves room for them while they wait
  const int target = hbm_waiting ? std::max(1, s->serve_grid - std::max(2, s->sms / 8)) : s->serve_grid;
  __atomic_store_n(&s->ctl_h->max_live, target, __ATOMIC_RELAXED);
  if (!live) {  // nothing runs: every launched CTA has left
    for (int k = 1; k < 3; ++k) s->seen[k] = (unsigned long long)s->ctas_launched;
  }
  bool waiting = false;
  for (size_t k = 0; k < s->entries.size() && !waiting; ++k)
    waiting = s->entries[k].busy && __atomic_load_n(&s->done_h[k], __ATOMIC_ACQUIRE) != (unsigned)s->entries[k].seq;
  if (!waiting || s->published <= s->seen[0]) return MCRG_OK;  // nothing unclaimed
  const int64_t running = s->ctas_launched - (int64_t)s->seen[2];
  if (running >= target) return MCRG_OK;
  if (!idle) {  // every stream holds a running launch: one more, up to the cap
    if ((int)s->loop_streams.size() >= mcrg_server::kMaxLoopStreams) return MCRG_OK;
    mcrg_server::LoopStream ls;
    if (cudaStreamCreateWithFlags(&ls.stream, cudaStreamNonBlocking) != cudaSuccess) return MCRG_EIO;
    if (cudaEventCreateWithFlags(&ls.end, cudaEventDisableTiming) != cudaSuccess) {
      cudaStreamDestroy(ls.stream);
      return MCRG_EIO;
    }
    s->loop_streams.push_back(ls);
    idle = &s->loop_streams.back();
  }
  const int grid = (int)(target - running);
  ServeArgs a = s->args;
  void* argv[] = {&a};
  if (cudaLaunchKernel(serve_kernel_fn(), dim3(grid), dim3(kServeThreads), argv, (size_t)kPoolMaxSmem,
                       idle->stream) != cudaSuccess ||
      cudaEventRecord(idle->end, idle->stream) != cudaSuccess)
    return MCRG_EIO;
  idle->live = true;
  s->live_launches++;
  s->ctas_launched += grid;
  __atomic_add_fetch(&s->loop_launches, 1, __ATOMIC_RELAXED);
  return MCRG_OK;
}

void server_loop(mcrg_server* s) {
  cudaSetDevice(s->cfg.device);
  // Packs still filling, kept across passes: while the loop already has
  // entries nobody has claimed, a pack that is not full waits (up to
  // kServeHoldS) for more requests of its shape -- it could not start sooner
  // anyway -- so a saturated loop runs full packs instead of one small chain
  // per CTA.
  std::vector<std::vector<Member>> packs;
  std::vector<PoolPack> shapes;  // per pack: threads, stride (count filled at publish)
  std::vector<double> opened;    // when each pack was opened
  std::map<std::tuple<int, int, int, int, int>, size_t> open;  // shape -> pack index still filling
  for (;;) {
    bool progressed = false;
    // ---- admit: pending requests in arrival order while slots, bins and memory allow
    bool hbm_waiting = false;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      const bool idle = s->pending.empty() && s->in_flight == 0;
      if (idle) {
        if (s->stop) break;
        s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
        continue;
      }
      size_t free_entries = 0;  // ring slots free in publication order from the next one on
      while (free_entries < s->cap && !s->entries[(size_t)((s->published + free_entries) % s->cap)].busy)
        ++free_entries;
      while (!s->pending.empty()) {
        mcrg_server::Req& q = s->pending.front();
        const bool resident = q.threads > 0;
        if (resident && s->free_bins.empty()) break;
        const auto key = std::make_tuple(q.r.L, chain_mode(&q.r), q.nl, q.r.n_couplings, q.threads);
        auto it = resident ? open.find(key) : open.end();
        if (resident && it == open.end() && packs.size() >= free_entries) break;  // no ring slot
        size_t off = (size_t)-1;
        if ((int64_t)q.bytes + s->bytes_in_use <= s->budget) off = arena_alloc(s, q.bytes);
        if (off == (size_t)-1) break;  // wait for memory (keeps arrival order)
        Member m{q.ticket, q.r, q.nl, q.submit_s, off, q.bytes, -1};
        s->bytes_in_use += (int64_t)q.bytes;
        s->admitted++;
        s->in_flight++;
        if (resident) {
          m.bin_slot = s->free_bins.back();
          s->free_bins.pop_back();
          if (it == open.end()) {
            const int g = q.threads;
            int per = 0, stride = 0;
            pack_geometry(q.r.L, q.nl, q.r.n_couplings, chain_mode(&q.r), g, kServeThreads, &per, &stride);
            packs.emplace_back();
            shapes.push_back(PoolPack{0, (int16_t)std::max(per, 1), (int16_t)g, stride, 0});
            opened.push_back(mono_s());
            it = open.emplace(key, packs.size() - 1).first;
          }
          packs[it->second].push_back(m);
          if ((int)packs[it->second].size() >= shapes[it->second].count) open.erase(it);  // full: published next
        } else {
          s->hbm_queue.push_back(m);
          s->cv_hbm.notify_one();
        }
        s->pending.pop_front();
        progressed = true;
      }
      hbm_waiting = !s->hbm_queue.empty() || s->hbm_running > 0;
    }
    // ---- publish full packs, and the others unless the loop has a backlog (entry contents first,
    //      then the tail with release semantics)
    const bool backlog = s->live_launches > 0 && s->published > s->seen[0];
    const double now = mono_s();
    std::vector<size_t> keep;
    for (size_t p = 0; p < packs.size(); ++p) {
      const bool full = (int)packs[p].size() >= shapes[p].count;
      if (!full && backlog && now - opened[p] < kServeHoldS) {
        keep.push_back(p);
        continue;
      }
      const uint32_t slot = (uint32_t)(s->published % s->cap);  // free: admission counted it
      EntryState& es = s->entries[slot];
      ServeEntry& e = s->ring_h[slot];
      PoolPack pk = shapes[p];
      pk.count = (int16_t)packs[p].size();
      e.pk = pk;
      for (size_t k = 0; k < packs[p].size(); ++k) {
        const Member& m = packs[p][k];
        memset(s->bins_h + (size_t)m.bin_slot * kServeBinsPerChain, 0, sizeof(mcrg_moments) * kServeBinsPerChain);
        fill_job(&e.jobs[k], &m.r, m.nl, s->arena + m.off, s->bins_d + (size_t)m.bin_slot * kServeBinsPerChain);
        e.jobs[k].threads = pk.threads;
      }
      es.busy = true;
      es.seq = s->published + 1;
      es.members = packs[p];
      __atomic_store_n(&s->ctl_h->tail, (unsigned long long)(s->published + 1), __ATOMIC_RELEASE);
      __atomic_add_fetch(&s->published, 1, __ATOMIC_RELAXED);
      progressed = true;
    }
    if (keep.size() != packs.size()) {  // drop the published packs, keep the ones still filling
      std::vector<std::vector<Member>> kp;
      std::vector<PoolPack> ks;
      std::vector<double> ko;
      open.clear();
      for (size_t p : keep) {
        const Member& m0 = packs[p][0];
        open[std::make_tuple(m0.r.L, chain_mode(&m0.r), m0.nl, m0.r.n_couplings, (int)shapes[p].threads)] = kp.size();
        kp.push_back(std::move(packs[p]));
        ks.push_back(shapes[p]);
        ko.push_back(opened[p]);
      }
      packs.swap(kp);
      shapes.swap(ks);
      opened.swap(ko);
    }
    // ---- keep the loop running while entries wait
    if (ensure_loop(s, hbm_waiting) != MCRG_OK) {  // the loop failed: every entry it held fails
      std::lock_guard<std::mutex> lk(s->mu);
      for (auto& e : s->entries)
        if (e.busy) {
          for (auto& m : e.members) {
            mcrg_result res;
            memset(&res, 0, sizeof res);
            res.status = MCRG_EIO;
            res.submit_s = m.submit_s;
            res.done_s = mono_s();
            s->free_bins.push_back(m.bin_slot);
            finish(s, m, res);
          }
          e.busy = false;
          e.members.clear();
        }
      s->cv_done.notify_all();
    }
    // ---- retire finished entries
    for (uint32_t k = 0; k < s->cap; ++k) {
      EntryState& e = s->entries[k];
      if (!e.busy) continue;
      const unsigned int d = __atomic_load_n(&s->done_h[k], __ATOMIC_ACQUIRE);
      if (d != (unsigned int)e.seq) continue;
      const double t_done = mono_s();
      std::vector<mcrg_result> res(e.members.size());
      for (size_t q = 0; q < e.members.size(); ++q) {
        const Member& m = e.members[q];
        mcrg_result& r = res[q];
        memset(&r, 0, sizeof r);
        r.submit_s = m.submit_s;
        r.done_s = t_done;
        r.status = MCRG_OK;
        r.moments.n_levels = m.nl;
        r.moments.n_couplings = m.r.n_couplings;
        const mcrg_moments* hb = s->bins_h + (size_t)m.bin_slot * kServeBinsPerChain;
        for (int64_t b = 0; b < n_dev_bins(&m.r); ++b) add_into(&r.moments, &hb[b]);
        r.moments.n_levels = m.nl;
        r.moments.n_couplings = m.r.n_couplings;
      }
      std::lock_guard<std::mutex> lk(s->mu);
      for (size_t q = 0; q < e.members.size(); ++q) {
        s->free_bins.push_back(e.members[q].bin_slot);
        finish(s, e.members[q], res[q]);
      }
      e.busy = false;
      e.members.clear();
      progressed = true;
      s->cv_done.notify_all();
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  // stop: every admitted request has finished; the loop's CTAs leave
  __atomic_store_n(&s->ctl_h->stop, 1, __ATOMIC_RELEASE);
  for (auto& ls : s->loop_streams) {
    cudaStreamSynchronize(ls.stream);
    ls.live = false;
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
  int rc = MCRG_OK;
  do {
    if (cudaMalloc(&s->arena, (size_t)s->budget) != cudaSuccess) { rc = MCRG_ENOMEM; break; }
    s->free_list[0] = (size_t)s->budget & ~size_t(255);
    int occ = 0;
    if (cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, cfg->device) != cudaSuccess ||
        serve_prepare(kPoolMaxSmem, &occ) != cudaSuccess || occ < 1) {
      rc = MCRG_EIO;
      break;
    }
    s->serve_grid = s->sms * occ;
    s->cap = (uint32_t)(4 * cfg->slots);
    if (cudaHostAlloc(&s->ring_h, sizeof(ServeEntry) * s->cap, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostAlloc(&s->ctl_h, sizeof(ServeCtl), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostAlloc(&s->done_h, sizeof(unsigned int) * s->cap, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostAlloc(&s->bins_h, sizeof(mcrg_moments) * kServeBinsPerChain * (size_t)cfg->slots,
                      cudaHostAllocMapped) != cudaSuccess ||
        cudaHostAlloc(&s->h_ctr, 4 * sizeof(unsigned long long), cudaHostAllocDefault) != cudaSuccess ||
        cudaMalloc(&s->args.ctr, 4 * sizeof(unsigned long long)) != cudaSuccess) {
      rc = MCRG_ENOMEM;
      break;
    }
    memset(s->ring_h, 0, sizeof(ServeEntry) * s->cap);
    memset(s->ctl_h, 0, sizeof(ServeCtl));
    memset(s->done_h, 0, sizeof(unsigned int) * s->cap);
    s->ctl_h->idle_ns = kServeIdleNs;
    if (cudaHostGetDevicePointer((void**)&s->args.ring, s->ring_h, 0) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&s->args.ctl, s->ctl_h, 0) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&s->args.done, s->done_h, 0) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&s->bins_d, s->bins_h, 0) != cudaSuccess ||
        cudaMemset(s->args.ctr, 0, 4 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->ctr_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ctr_done, cudaEventDisableTiming) != cudaSuccess) {
      rc = MCRG_EIO;
      break;
    }
    memset(s->h_ctr, 0, 4 * sizeof(unsigned long long));
    s->ctl_h->max_live = s->serve_grid;
    s->args.cap = s->cap;
    s->entries.resize(s->cap);
    for (int b = cfg->slots - 1; b >= 0; --b) s->free_bins.push_back(b);
  } while (0);
  if (rc) {
    cudaFree(s->arena);
    cudaFree(s->args.ctr);
    if (s->ring_h) cudaFreeHost(s->ring_h);
    if (s->ctl_h) cudaFreeHost(s->ctl_h);
    if (s->done_h) cudaFreeHost(s->done_h);
    if (s->bins_h) cudaFreeHost(s->bins_h);
    if (s->h_ctr) cudaFreeHost(s->h_ctr);
    if (s->ctr_stream) cudaStreamDestroy(s->ctr_stream);
    if (s->ctr_done) cudaEventDestroy(s->ctr_done);
    delete s;
    return rc;
  }
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
  const int threads = serve_plan(r, nl, s->cfg.device);
  const size_t bytes = request_bytes(r, nl, threads > 0);
  if ((int64_t)bytes > s->budget) return MCRG_ENOSPC;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return MCRG_ECANCELED;
  if ((int)s->pending.size() >= s->cfg.queue_capacity) return MCRG_EBUSY;
  mcrg_server::Req q{s->next_ticket++, *r, nl, bytes, threads, mono_s()};
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

int mcrg_server_loop_stats(mcrg_server* s, int64_t* loop_launches, int64_t* entries_published) {
  if (!s) return MCRG_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);  // the scheduler thread updates both under its own order; a snapshot
  if (loop_launches) *loop_launches = __atomic_load_n(&s->loop_launches, __ATOMIC_RELAXED);
  if (entries_published) *entries_published = (int64_t)__atomic_load_n(&s->published, __ATOMIC_RELAXED);
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
  for (auto& ls : s->loop_streams) {
    cudaStreamSynchronize(ls.stream);
    cudaStreamDestroy(ls.stream);
    cudaEventDestroy(ls.end);
  }
  cudaStreamSynchronize(s->ctr_stream);
  cudaStreamDestroy(s->ctr_stream);
  cudaEventDestroy(s->ctr_done);
  cudaFree(s->arena);
  cudaFree(s->args.ctr);
  cudaFreeHost(s->ring_h);
  cudaFreeHost(s->ctl_h);
  cudaFreeHost(s->done_h);
  cudaFreeHost(s->bins_h);
  cudaFreeHost(s->h_ctr);
  delete s;
  return MCRG_OK;
}

}  // extern "C"
