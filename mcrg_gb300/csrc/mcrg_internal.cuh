// mcrg_internal.cuh -- job descriptors and launchers shared by the CUDA
// translation units of libmcrg.  Not part of the public ABI.
#pragma once
#include <cstdint>
#include <utility>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/mcrg.h"
#include "mcrg_device.cuh"

namespace mcrg {

// Device memory of a context: from cudaMalloc (span == nullptr), or -- for
// the contexts a server runs its HBM-path requests on -- carved out of a
// span of the server's arena that was reserved, and charged to its budget,
// when the request was admitted.  Span allocations are 256-byte aligned and
// bump-allocated; a release frees space once everything allocated after it
// is released as well (temporaries of one call are released in reverse
// order); the span goes back to the arena as a whole.
struct DevSpan {
  uint8_t* base = nullptr;
  size_t cap = 0, used = 0;
  std::vector<std::pair<size_t, size_t>> live;  // (offset, bytes) in allocation order; bytes 0 once released
};
cudaError_t dev_alloc(DevSpan* s, void** p, size_t bytes);
void dev_release(DevSpan* s, void* p);
template <class T>
inline cudaError_t dev_alloc(DevSpan* s, T** p, size_t bytes) {
  return dev_alloc(s, reinterpret_cast<void**>(p), bytes);
}

// One independent Markov chain run shared-memory resident by one CTA.
struct ChainJob {
  int32_t L, n_levels, C, threads;
  Key key;
  uint32_t replica;
  uint32_t t0;        // Philox time of the first sweep
  uint32_t n0;        // Philox time (sample index) of the first measurement
  uint32_t init;      // 1: draw the initial coin; 0: load `state`
  uint32_t store;     // 1: write the final configuration back to `state`
  int64_t n_eq, n_samples, sweeps_between, bin_size;
  uint8_t* state;     // L*L bytes: colour-0 array then colour-1 array
  mcrg_moments* bins; // ceil(n_samples / bin_size) outputs, zeroed by the host
  Accept acc;
  int32_t flow;       // 1: flow moments (sum S_l and S_l * S_0 of coupling 0) instead of the T-matrix moments
  int32_t update;     // 0: checkerboard sweeps; MCRG_UPDATE_WOLFF / MCRG_UPDATE_SWENDSEN_WANG: cluster updates (L <= 256)
  uint32_t bond_tb;   // cluster updates: floor((1 - exp(2K)) 2^32)
  uint32_t pad;
};

// Shared-memory plan of a resident lattice, its blocked levels and (when
// C > 0) the moment accumulators of one chain.  planes: every level of side
// >= 64 is kept as bit-plane words (m^2 / 8 bytes) instead of bytes, and the
// open-word queue of the bit-sliced sweep is added (mcrg_resident_bits.cuh).
struct SmemPlan {
  int off[MCRG_MAX_LEVELS + 2];
  int s_off;    // int32 S[(MCRG_MAX_LEVELS+1) * MCRG_MAX_COUPLINGS]
  int tab_off;  // int2 per moment entry: (x | y << 16, output index)
  int acc_off;  // int64 per moment entry
  int scr_off;  // uint32 open-site scratch: 64 per warp of the chain (at least 8 warps)
  int E;        // moment entries of the T-matrix moments
  int Ecap;     // entries the table holds (also fits the 2 (n_levels + 1) flow moments)
  int qn_off;   // planes: int qn[2] (padded to 16 bytes)
  int q_off;    // planes: uint4 queue entries (resident queue_cap(L))
  int cl_off;   // cluster updates: labels, coins and the seed's root (mcrg_resident_cluster.cuh)
  int bytes;
};

// Largest side of a chain with resident cluster updates (16-bit site labels).
constexpr int kClusterMaxL = 256;

// Largest side of a resident chain: bytes up to MCRG_SMEM_MAX_L, bit planes
// (fast acceptance regime) up to MCRG_RESIDENT_MAX_L.
__host__ __device__ inline bool resident_fits(int L, bool fast) {
  return L <= (fast ? MCRG_RESIDENT_MAX_L : MCRG_SMEM_MAX_L);
}

__host__ __device__ inline SmemPlan make_plan(int L, int n_levels, int C = 0, bool planes = false, bool cluster = false,
                                             int threads = 256) {
  SmemPlan p;
  int off = 0, n = L;
  for (int l = 0; l <= n_levels; ++l, n >>= 1) {
    p.off[l] = off;
    off += (planes && n >= 64) ? n * n / 8 : ((n * n + 15) / 16) * 16;
  }
  p.s_off = off;
  off += ((MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS * 4 + 15) / 16 * 16;
  p.E = C > 0 ? (n_levels + 1) * C + 2 * n_levels * C * C : 0;
  p.Ecap = C > 0 ? (p.E > 2 * (n_levels + 1) ? p.E : 2 * (n_levels + 1)) : 0;
  p.tab_off = off;
  off += ((p.Ecap * 8 + 15) / 16) * 16;
  p.acc_off = off;
  off += p.Ecap * 8;
  p.scr_off = off;
  off += (threads > 256 ? threads / 32 : 8) * 64 * 4;  // kOpenPerWarp words per warp of the chain
  p.qn_off = p.q_off = -1;
  if (planes) {
    off = (off + 15) / 16 * 16;  // the queue holds uint4 entries
    p.qn_off = off;
    off += 16;
    p.q_off = off;
    const int q = L * L / 256;
    off += (q < 32 ? 32 : (q > 2048 ? 2048 : q)) * 16;  // resident::queue_cap(L)
  }
  p.cl_off = -1;
  if (cluster) {  // rcluster::work_bytes(L)
    off = (off + 15) / 16 * 16;
    p.cl_off = off;
    off += ((L * L * 2 + 15) / 16) * 16 + 3 * ((L * L / 8 + 15) / 16) * 16 + 16;
  }
  p.bytes = (off + 15) / 16 * 16;
  return p;
}

inline int moment_entries(int n_levels, int C) { return (n_levels + 1) * C + 2 * n_levels * C * C; }

// Whether a chain with cluster updates fits one CTA's shared memory (227 KB).
inline bool cluster_resident(int L, int n_levels, int C, bool fast) {
  return L <= kClusterMaxL && make_plan(L, n_levels, C, fast && L >= 64, true).bytes <= 227 * 1024;
}

// Host: acceptance parameters for coupling K (FP64, see include/mcrg.h).
Accept make_accept(double K);

// Launch `n_jobs` chains (all with the same L, threads and acceptance regime:
// `planes` = acc.fast && L >= 64; n_levels and C bound the shared memory of
// every job; `cluster`: the jobs use cluster updates, L <= kClusterMaxL).
cudaError_t launch_chain(const ChainJob* d_jobs, int n_jobs, int L, int n_levels, int C, int threads, bool planes,
                         cudaStream_t stream, bool cluster = false);

// Persistent batch (pool_kernel, mcrg_chain.cu): packs of chains taken in
// queue order by the CTAs of one launch.  A pack is `count` chains (jobs
// first .. first+count-1) of `threads` threads each (a multiple of 32; 32,
// or 64 .. CTA width for named barriers), `stride` bytes of shared memory
// each; count * threads <= CTA width and count * stride <= the launch's
// dynamic shared memory.
constexpr int kPoolMaxGroups = 16;
constexpr int kPoolMaxSmem = 224 * 1024;  // dynamic shared memory per CTA (the kernel adds ~3 KB of its own)
struct PoolPack {
  int32_t first;
  int16_t count;
  int16_t threads;
  int32_t stride;
  int32_t pad;
};
// The packs are grouped into up to kPoolClasses classes by chain code (byte
// sweeps, plane sweeps, cluster updates): class k is packs [first[k],
// first[k+1]).  A CTA serves first the class of its SM (SM id ×
// n_classes-weighted by class work: sm_edge[k] = first SM fraction, in
// 1/65536, of class k), then takes from the others when it is empty, so that
// the CTAs of one SM mostly run one chain code and share its instructions in
// cache.  next[k * 16] counts the packs of class k handed out.
constexpr int kPoolClasses = 3;
struct PoolQueue {
  int32_t n_packs;
  int32_t n_classes;
  const PoolPack* packs;
  const ChainJob* jobs;
  unsigned* next;  // per class, 64 bytes apart; zero before the launch
  int32_t first[kPoolClasses + 1];
  int32_t sm_edge[kPoolClasses + 1];
};
// Served requests (serve_kernel, mcrg_chain.cu): a ring of packs in page-
// locked host memory that the server's scheduler fills and the persistent
// CTAs drain.  Entry k lives in slot k % cap; the host writes it, then
// publishes it by a release store of `tail` = k + 1; a CTA claims the next
// entry with a compare-and-swap of the device counter `head` after an
// acquire load of `tail`, runs its chains (the moments go to the jobs' bins,
// page-locked host memory) and stores done[k % cap] = k + 1 with release
// semantics.  A CTA with nothing to claim polls with growing sleeps and
// leaves after `idle_ns`; a CTA also leaves at its next claim while more than
// `max_live` CTAs run (room for HBM-path kernels), and all leave at stop.
// The device counters ctr[0..2] = entries claimed, CTAs started, CTAs left
// (monotonic) let the server keep the loop at its width: it launches more
// CTAs, on a pool of streams, while entries wait and fewer are running.
struct __align__(16) ServeEntry {
  PoolPack pk;  // pk.first unused: the jobs are inline
  ChainJob jobs[kPoolMaxGroups];
};
static_assert(sizeof(PoolPack) == 16 && sizeof(ServeEntry) % 16 == 0, "ring entries are copied as 16-byte words");
struct ServeCtl {
  unsigned long long tail;
  unsigned long long idle_ns;
  int32_t stop;
  int32_t max_live;
};
struct ServeArgs {
  const ServeEntry* ring;   // device address of the host ring
  ServeCtl* ctl;            // device address of the host control block
  unsigned int* done;       // device address of the host completion words
  unsigned long long* ctr;  // device memory: [0] entries claimed, [1] CTAs started, [2] CTAs left
  uint32_t cap;
  uint32_t pad;
};
constexpr int kServeThreads = 512;
const void* serve_kernel_fn();
// Shared-memory limit of the serve kernel (once per device); its resident
// CTAs per SM for `smem` bytes.
cudaError_t serve_prepare(int smem, int* blocks_per_sm);

// CTA widths of the pool kernel: 256 (3 CTAs per SM by registers) or 512 (one per SM).
const void* pool_kernel_fn(int cta_threads);
// Sets the kernel's shared-memory limit (once per device) and returns its
// resident CTAs per SM for `smem` bytes of dynamic shared memory.
cudaError_t pool_prepare(int cta_threads, int smem, int* blocks_per_sm);

// Stateless helpers on a device lattice in split layout (used by
// mcrg_block_lattice / mcrg_lattice_couplings and the HBM path's tail).
cudaError_t launch_block_once(const uint8_t* d_in, int N, uint8_t* d_out, const uint8_t* d_tie_nat,
                              Key key, uint32_t replica, int level, uint32_t sample, cudaStream_t s);
cudaError_t launch_couplings_once(const uint8_t* d_in, int N, int C, int* d_out, cudaStream_t s);
// Natural-layout int8 +-1 lattice -> split layout; *d_bad |= 1 on a value
// other than +-1.  Returns the launch's own status (no cudaGetLastError).
cudaError_t launch_nat_to_split(const int8_t* d_nat, int N, uint8_t* d_split, int* d_bad, cudaStream_t s);

// One cluster update (Wolff or Swendsen-Wang, mcrg_cluster.cu) of a split-
// layout lattice of side L at update index t: d_label holds
// cluster_label_ints(L) ints (L^2 labels, then two bond masks per 32 x 32 tile),
// *d_count gains the number of flipped spins, *d_err gets bit 2 / 4 when a
// find / union loop hits its bound.
cudaError_t launch_cluster_update(uint8_t* d_state, int L, int* d_label, int kind, Key key, uint32_t replica,
                                  uint32_t t, uint32_t bond_threshold, unsigned long long* d_count, int* d_err,
                                  int num_sms, cudaStream_t s);
inline size_t cluster_label_ints(int L) { return (size_t)L * L + (size_t)L * L / 512 + 2; }
// floor((1 - exp(2K)) 2^32), 0 when no bond can open (K >= 0).
uint32_t bond_threshold(double K);

// New chain on an HBM-resident context without allocating (mcrg_capi.cu).
int reinit_context(mcrg_ctx* c, double K, uint64_t seed, uint32_t replica);
// mcrg_alloc with every device buffer of the context's lifetime taken from
// `span` (nullptr: cudaMalloc).
int context_create(mcrg_ctx** out, const mcrg_cfg* cfg, DevSpan* span);
// Upper bound of the span bytes a context needs for mcrg_sweep / mcrg_measure
// of n_samples (update == 0) or mcrg_cluster_update / mcrg_measure_cluster
// (update != 0).
size_t context_bytes(int L, int n_levels, int C, int update, int64_t n_samples);

// Forward pass of the RG neural network (src/rgnn.cpp:281-307) on a split
// layout lattice of side n: the scalar output into *d_out (device), using
// `work` ((n/32)^2 + (n/1024)^2 + 2 doubles, not overlapping d_out).
cudaError_t launch_rgnn_scalar(const uint8_t* d_split, int n, const double W[4], double* work, double* d_out,
                               cudaStream_t s);

}  // namespace mcrg
