// mcrg_capi.cu -- host side of the C ABI declared in include/mcrg.h.
//
// A context (mcrg_ctx) holds one lattice and its chain counters on one
// device: lattices with L <= MCRG_SMEM_MAX_L run every sweep / measurement
// in one shared-memory-resident CTA (mcrg_chain.cu); larger lattices live in
// HBM and run the tiled streaming kernels (mcrg_tiled.cu).  Lattices cross
// the ABI in natural layout (int8 +-1) and are converted on the device.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <new>
#include <vector>

#include "mcrg_internal.cuh"
#include "mcrg_tiled.cuh"
#include "mcrg_tma.cuh"

using namespace mcrg;

struct mcrg_ctx {
  mcrg_cfg cfg;
  int n_levels;
  cudaStream_t stream = nullptr;
  uint8_t* d_state = nullptr;   // L*L bytes split layout (smem class)
  TiledLattice tiled;           // HBM class
  bool is_tiled = false;
  uint64_t t = 0;               // next sweep index
  uint64_t n = 0;               // next sample index
  ChainJob* d_job = nullptr;
  mcrg_moments* d_bins = nullptr;
  int64_t bins_cap = 0;
  int8_t* d_nat = nullptr;      // natural-layout staging (L*L)
  int* d_flag = nullptr;
  Accept acc;
  double* d_rgnn = nullptr;     // forward-pass work: (L/32)^2 + (L/1024)^2 + 3 doubles, the last one the result
  int* d_labels = nullptr;      // cluster updates: L^2 labels + tile-edge bond masks (allocated by the first update)
  unsigned long long* d_cl = nullptr;  // cluster updates: [0] flipped spins, [1] error flags
  mcrg_moments* d_cbins = nullptr;     // cluster measurement: one bin per sample of a chunk
  ChainJob* d_cjobs = nullptr;         // cluster measurement: one measurement job per sample of a chunk
  DevSpan* span = nullptr;             // where device buffers come from (nullptr: cudaMalloc)
};

namespace {

constexpr int64_t kMaxDeviceBin = int64_t(1) << 24;  // int64 headroom of the resident accumulators

int ilog2(int x) {
  int l = 0;
  while ((1 << l) < x) ++l;
  return l;
}

int to_status(cudaError_t e) { return e == cudaSuccess ? MCRG_OK : MCRG_EIO; }

#define CK(expr)                                  \
  do {                                            \
    cudaError_t _e = (expr);                      \
    if (_e != cudaSuccess) return MCRG_EIO;       \
  } while (0)

__global__ void nat_to_split_kernel(const int8_t* __restrict__ nat, int N, uint8_t* __restrict__ split,
                                    int* __restrict__ bad) {
  const int half = N / 2;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N * N; s += gridDim.x * blockDim.x) {
    const int i = s / N, j = s % N;
    const int8_t v = nat[s];
    if (v != 1 && v != -1) atomicOr(bad, 1);
    split[(size_t)((i + j) & 1) * N * half + (size_t)i * half + (j >> 1)] = v > 0 ? 1 : 0;
  }
}

__global__ void split_to_nat_kernel(const uint8_t* __restrict__ split, int N, int8_t* __restrict__ nat) {
  const int half = N / 2;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N * N; s += gridDim.x * blockDim.x) {
    const int i = s / N, j = s % N;
    nat[s] = split[(size_t)((i + j) & 1) * N * half + (size_t)i * half + (j >> 1)] ? 1 : -1;
  }
}

// 32 sites per thread (N >= 32): a natural row segment of 32 int8 +-1 is two
// 16-byte loads; its even and odd columns become 16 bytes of each colour.
// A byte is valid iff it is 0x01 or 0xFF: bit 0 set and bits 1..7 all equal.
__device__ __forceinline__ uint32_t pm1_to_01(uint32_t x, uint32_t& bad) {
  const uint32_t t = x & 0xFEFEFEFEu;
  bad |= ((x & 0x01010101u) ^ 0x01010101u) | (t ^ (((t >> 7) & 0x01010101u) * 0xFEu));
  return (~x >> 7) & 0x01010101u;
}

__global__ void nat_to_split_vec_kernel(const int8_t* __restrict__ nat, int N, uint8_t* __restrict__ split,
                                        int* __restrict__ bad) {
  const int half = N / 2, per_row = N / 32, lp = __ffs(per_row) - 1;  // N: a power of two
  uint32_t b = 0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < (long long)N * per_row;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q >> lp), j0 = (int)(q & (per_row - 1)) * 32;
    const uint4* src = reinterpret_cast<const uint4*>(nat + (size_t)i * N + j0);
    const uint4 a = src[0], c = src[1];
    const uint32_t w[8] = {pm1_to_01(a.x, b), pm1_to_01(a.y, b), pm1_to_01(a.z, b), pm1_to_01(a.w, b),
                           pm1_to_01(c.x, b), pm1_to_01(c.y, b), pm1_to_01(c.z, b), pm1_to_01(c.w, b)};
    const uint4 ev = make_uint4(__byte_perm(w[0], w[1], 0x6420), __byte_perm(w[2], w[3], 0x6420),
                                __byte_perm(w[4], w[5], 0x6420), __byte_perm(w[6], w[7], 0x6420));
    const uint4 od = make_uint4(__byte_perm(w[0], w[1], 0x7531), __byte_perm(w[2], w[3], 0x7531),
                                __byte_perm(w[4], w[5], 0x7531), __byte_perm(w[6], w[7], 0x7531));
    const int ce = i & 1;  // the colour whose sites sit on even columns of row i
    *reinterpret_cast<uint4*>(split + (size_t)ce * N * half + (size_t)i * half + (j0 >> 1)) = ev;
    *reinterpret_cast<uint4*>(split + (size_t)(1 - ce) * N * half + (size_t)i * half + (j0 >> 1)) = od;
  }
  if (b) atomicOr(bad, 1);
}

__global__ void split_to_nat_vec_kernel(const uint8_t* __restrict__ split, int N, int8_t* __restrict__ nat) {
  const int half = N / 2, per_row = N / 32, lp = __ffs(per_row) - 1;  // N: a power of two
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < (long long)N * per_row;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q >> lp), j0 = (int)(q & (per_row - 1)) * 32, ce = i & 1;
    const uint4 e = *reinterpret_cast<const uint4*>(split + (size_t)ce * N * half + (size_t)i * half + (j0 >> 1));
    const uint4 o = *reinterpret_cast<const uint4*>(split + (size_t)(1 - ce) * N * half + (size_t)i * half + (j0 >> 1));
    const uint32_t E[4] = {e.x, e.y, e.z, e.w}, O[4] = {o.x, o.y, o.z, o.w};
    uint32_t w[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      w[2 * k] = __byte_perm(E[k], O[k], 0x5140);
      w[2 * k + 1] = __byte_perm(E[k], O[k], 0x7362);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) w[k] |= (w[k] ^ 0x01010101u) * 0xFFu;  // 1 -> 0x01, 0 -> 0xFF
    uint4* dst = reinterpret_cast<uint4*>(nat + (size_t)i * N + j0);
    dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
    dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
  }
}

__global__ void nat01_kernel(const int8_t* __restrict__ nat, int n, uint8_t* __restrict__ out, int* bad) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const int8_t v = nat[s];
    if (v != 1 && v != -1) atomicOr(bad, 1);
    out[s] = v > 0 ? 1 : 0;
  }
}

int grid_for(int64_t work) {
  int64_t g = (work + 255) / 256;
  if (g < 1) g = 1;
  if (g > 8192) g = 8192;
  return (int)g;
}

bool valid_L(int L) { return L >= 4 && L <= MCRG_MAX_L && (L & (L - 1)) == 0; }

int resolve_levels(int L, int n_levels) {
  const int mx = ilog2(L) - 1;
  if (n_levels < 0) return mx;
  return n_levels <= mx ? n_levels : -1;
}

int threads_for(int L) {
  if (L <= 32) return 32;
  if (L == 64) return 64;
  if (L == 128) return 128;
  return 256;
}

void add_moments(mcrg_moments* dst, const mcrg_moments* src) {
  dst->n_samples += src->n_samples;
  for (int x = 0; x < (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS; ++x) dst->S[x] += src->S[x];
  for (int x = 0; x < MCRG_MAX_LEVELS * MCRG_MAX_COUPLINGS * MCRG_MAX_COUPLINGS; ++x) {
    __int128 a = ((__int128)dst->SbS[x].hi << 64) | dst->SbS[x].lo;
    __int128 b = ((__int128)src->SbS[x].hi << 64) | src->SbS[x].lo;
    a += b;
    dst->SbS[x].lo = (uint64_t)a;
    dst->SbS[x].hi = (int64_t)(a >> 64);
    a = ((__int128)dst->SbSb[x].hi << 64) | dst->SbSb[x].lo;
    b = ((__int128)src->SbSb[x].hi << 64) | src->SbSb[x].lo;
    a += b;
    dst->SbSb[x].lo = (uint64_t)a;
    dst->SbSb[x].hi = (int64_t)(a >> 64);
  }
}

int ensure_bins(mcrg_ctx* c, int64_t n) {
  if (n <= c->bins_cap) return MCRG_OK;
  dev_release(c->span, c->d_bins);
  c->d_bins = nullptr;
  c->bins_cap = 0;
  if (dev_alloc(c->span, &c->d_bins, sizeof(mcrg_moments) * (size_t)n) != cudaSuccess) return MCRG_ENOMEM;
  c->bins_cap = n;
  return MCRG_OK;
}

// Runs one resident chain job for the context and returns the device bins.
int run_resident(mcrg_ctx* c, int64_t n_eq, int64_t n_samples, int64_t sweeps_between, int64_t bin_size,
                 int64_t* n_bins_out, bool flow = false, int update = 0) {
  ChainJob j;
  memset(&j, 0, sizeof j);
  j.L = c->cfg.L;
  j.n_levels = c->n_levels;
  j.C = c->cfg.n_couplings;
  j.threads = update && c->cfg.L >= 64 ? 512 : threads_for(c->cfg.L);  // cluster labelling is latency-bound
  j.key = Key{(uint32_t)c->cfg.seed, (uint32_t)(c->cfg.seed >> 32)};
  j.replica = c->cfg.replica;
  j.t0 = (uint32_t)c->t;
  j.n0 = (uint32_t)c->n;
  j.init = 0;
  j.store = 1;
  j.n_eq = n_eq;
  j.n_samples = n_samples;
  j.sweeps_between = sweeps_between;
  j.bin_size = bin_size;
  j.state = c->d_state;
  j.acc = c->acc;
  j.flow = flow ? 1 : 0;
  j.update = update;
  j.bond_tb = update ? bond_threshold(c->cfg.K) : 0u;
  int64_t nb = n_samples > 0 ? (n_samples + bin_size - 1) / bin_size : 0;
  if (nb > 0) {
    int rc = ensure_bins(c, nb);
    if (rc) return rc;
    CK(cudaMemsetAsync(c->d_bins, 0, sizeof(mcrg_moments) * (size_t)nb, c->stream));
  }
  j.bins = c->d_bins;
  CK(cudaMemcpyAsync(c->d_job, &j, sizeof j, cudaMemcpyHostToDevice, c->stream));
  CK(launch_chain(c->d_job, 1, j.L, j.n_levels, j.C, j.threads, j.acc.fast && j.L >= 64, c->stream, update != 0));
  c->t += (uint64_t)(n_eq + n_samples * sweeps_between);
  c->n += (uint64_t)n_samples;
  *n_bins_out = nb;
  return MCRG_OK;
}

// One thread waits, with the kernels' bounded wait, on an mbarrier that
// nothing arrives at: the wait runs out after limit_ns and raises the flag.
// No copy is ever issued on the barrier, so the block can leave it pending.
__global__ void wait_selftest_kernel(uint64_t limit_ns, int* status, unsigned long long* waited_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tma::mbar_init(&bar, 1);
    tma::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint64_t t0 = tma::globaltimer_ns();
    if (!tma::mbar_wait_bounded(&bar, 0u, limit_ns)) atomicOr(status, 1);
    *waited_ns = tma::globaltimer_ns() - t0;
  }
}

}  // namespace

namespace mcrg {
cudaError_t launch_nat_to_split(const int8_t* d_nat, int N, uint8_t* d_split, int* d_bad, cudaStream_t s) {
  void* args[] = {(void*)&d_nat, (void*)&N, (void*)&d_split, (void*)&d_bad};
  return cudaLaunchKernel((const void*)nat_to_split_kernel, dim3(grid_for((int64_t)N * N)), dim3(256), args, 0, s);
}

Accept make_accept(double K) {
  Accept a;
  memset(&a, 0, sizeof a);
  uint8_t always[5];
  mcrg_thresholds(K, a.thr, always);
  for (int m = 0; m < 5; ++m) a.always_mask |= (uint32_t)always[m] << m;
  a.fast = (a.always_mask == 0x1Cu) && (a.thr[1] < 0x80000000u) && (a.thr[0] <= a.thr[1]);
  const uint32_t t0 = a.thr[0] >> 24, t1 = a.thr[1] >> 24;
  a.cx0 = (0x80u - t0) * 0x01010101u;
  a.cx1 = (0x80u - t1) * 0x01010101u;
  a.cy0 = (0x7Fu - t0) * 0x01010101u;
  a.cy1 = (0x7Fu - t1) * 0x01010101u;
  return a;
}
}  // namespace mcrg

extern "C" {

const char* mcrg_strerror(int code) {
  switch (code) {
    case MCRG_OK: return "ok";
    case MCRG_ENOENT: return "unknown ticket";
    case MCRG_EIO: return "CUDA error";
    case MCRG_EAGAIN: return "not finished";
    case MCRG_ENOMEM: return "out of memory";
    case MCRG_EBUSY: return "queue full";
    case MCRG_EINVAL: return "invalid argument";
    case MCRG_ENOSPC: return "request exceeds the memory budget";
    case MCRG_ENOSYS: return "not supported";
    case MCRG_ETIMEDOUT: return "timed out";
    case MCRG_ECANCELED: return "cancelled";
    default: return "unknown error";
  }
}

int mcrg_abi_version(void) { return MCRG_ABI_VERSION; }

int mcrg_thresholds(double K, uint32_t thr[5], uint8_t always[5]) {
  if (!thr || !always || !std::isfinite(K)) return MCRG_EINVAL;
  for (int m = 0; m < 5; ++m) {
    const double x = 2.0 * K * (double)(4 - 2 * m);
    if (x >= 0.0) {
      always[m] = 1;
      thr[m] = 0xFFFFFFFFu;
    } else {
      always[m] = 0;
      thr[m] = (uint32_t)std::floor(std::exp(x) * 4294967296.0);
    }
  }
  return MCRG_OK;
}

int mcrg_alloc(mcrg_ctx** out, const mcrg_cfg* cfg) { return context_create(out, cfg, nullptr); }

}  // extern "C"

namespace mcrg {

cudaError_t dev_alloc(DevSpan* s, void** p, size_t bytes) {
  if (!s) return cudaMalloc(p, bytes);
  if (bytes == 0) bytes = 1;
  const size_t off = (s->used + 255) & ~size_t(255);
  if (off > s->cap || bytes > s->cap - off) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  s->live.push_back({off, bytes});
  s->used = off + bytes;
  *p = s->base + off;
  return cudaSuccess;
}

void dev_release(DevSpan* s, void* p) {
  if (!p) return;
  if (!s) {
    cudaFree(p);
    return;
  }
  const size_t off = (size_t)(static_cast<uint8_t*>(p) - s->base);
  for (auto& e : s->live)
    if (e.first == off && e.second) {
      e.second = 0;
      break;
    }
  while (!s->live.empty() && s->live.back().second == 0) s->live.pop_back();
  s->used = s->live.empty() ? 0 : s->live.back().first + s->live.back().second;
}

size_t context_bytes(int L, int n_levels, int C, int update, int64_t n_samples) {
  auto a = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t LL = (size_t)L * L;
  const int64_t nb = n_samples > 0 ? (n_samples + kMaxDeviceBin - 1) / kMaxDeviceBin : 1;
  size_t b = a(sizeof(ChainJob)) + a(LL) + a(sizeof(int) * 64);  // job, natural staging, flags
  if (L <= MCRG_SMEM_MAX_L) {
    b += a(LL);  // state
  } else {       // ping-pong buffers, blocked levels (< LL / 3), sums, status, bins of the tiled path
    b += 2 * a(LL) + a(LL / 3 + 16) + a(sizeof(unsigned long long) * (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS) +
         a(sizeof(int)) + a(sizeof(mcrg_moments) * (size_t)nb);
  }
  b += a(sizeof(mcrg_moments) * (size_t)nb);  // the context's bins
  if (update)  // labels, counters, one chunk of per-sample bins and measurement jobs
    b += a(sizeof(int) * cluster_label_ints(L)) + a(2 * sizeof(unsigned long long)) + a(sizeof(mcrg_moments) * 256) +
         a(sizeof(ChainJob) * 256);
  (void)n_levels;
  (void)C;
  return b + 4096;
}

int context_create(mcrg_ctx** out, const mcrg_cfg* cfg, DevSpan* span) {
  if (!out || !cfg) return MCRG_EINVAL;
  *out = nullptr;
  if (!valid_L(cfg->L) || cfg->b != 2 || cfg->n_couplings < 1 || cfg->n_couplings > MCRG_MAX_COUPLINGS ||
      !std::isfinite(cfg->K))
    return MCRG_EINVAL;
  const int nl = resolve_levels(cfg->L, cfg->n_levels);
  if (nl < 0) return MCRG_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) return MCRG_EIO;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return MCRG_EIO;
  mcrg_ctx* c = new (std::nothrow) mcrg_ctx();
  if (!c) return MCRG_ENOMEM;
  c->cfg = *cfg;
  c->n_levels = nl;
  c->acc = make_accept(cfg->K);
  c->span = span;
  c->tiled.span = span;
  int rc = MCRG_OK;
  const size_t LL = (size_t)cfg->L * cfg->L;
  do {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { rc = MCRG_EIO; break; }
    if (dev_alloc(span, &c->d_job, sizeof(ChainJob)) != cudaSuccess) { rc = MCRG_ENOMEM; break; }
    if (dev_alloc(span, &c->d_nat, LL) != cudaSuccess) { rc = MCRG_ENOMEM; break; }
    if (dev_alloc(span, &c->d_flag, sizeof(int) * 64) != cudaSuccess) { rc = MCRG_ENOMEM; break; }
    const Key key{(uint32_t)cfg->seed, (uint32_t)(cfg->seed >> 32)};
    if (cfg->L <= MCRG_SMEM_MAX_L) {
      if (dev_alloc(span, &c->d_state, LL) != cudaSuccess) { rc = MCRG_ENOMEM; break; }
      ChainJob j;
      memset(&j, 0, sizeof j);
      j.L = cfg->L; j.n_levels = nl; j.C = cfg->n_couplings; j.threads = threads_for(cfg->L);
      j.key = key; j.replica = cfg->replica; j.init = 1; j.store = 1; j.bin_size = 1;
      j.state = c->d_state; j.acc = c->acc;
      if (cudaMemcpyAsync(c->d_job, &j, sizeof j, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) { rc = MCRG_EIO; break; }
      if (launch_chain(c->d_job, 1, j.L, nl, j.C, j.threads, j.acc.fast && j.L >= 64, c->stream) != cudaSuccess) {
        rc = MCRG_EIO;
        break;
      }
    } else {
      c->is_tiled = true;
      rc = tiled_alloc(&c->tiled, cfg->L, nl, cfg->n_couplings, key, cfg->replica, c->acc, c->stream);
      if (rc) break;
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) { rc = MCRG_EIO; break; }
  } while (0);
  if (rc) {
    mcrg_free(c);
    return rc;
  }
  *out = c;
  return MCRG_OK;
}

}  // namespace mcrg

extern "C" {

int mcrg_free(mcrg_ctx* c) {
  if (!c) return MCRG_EINVAL;
  cudaSetDevice(c->cfg.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->is_tiled) tiled_free(&c->tiled);
  DevSpan* sp = c->span;
  dev_release(sp, c->d_cjobs);
  dev_release(sp, c->d_cbins);
  dev_release(sp, c->d_cl);
  dev_release(sp, c->d_labels);
  dev_release(sp, c->d_rgnn);
  dev_release(sp, c->d_bins);
  dev_release(sp, c->d_state);
  dev_release(sp, c->d_flag);
  dev_release(sp, c->d_nat);
  dev_release(sp, c->d_job);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return MCRG_OK;
}

// Device address of a page-locked, 16-byte-aligned host buffer (the upload
// kernel then reads it directly over the host link), or nullptr for pageable
// memory, which goes through a staging copy.
static void* pinned_device_ptr(const void* host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer || ((uintptr_t)a.devicePointer & 15u)) return nullptr;
  return a.devicePointer;
}

int mcrg_set_spins(mcrg_ctx* c, const int8_t* host) {
  if (!c || !host) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  const int L = c->cfg.L;
  uint8_t* dst = c->is_tiled ? tiled_state(&c->tiled) : c->d_state;
  const void* direct = L >= 32 ? pinned_device_ptr(host) : nullptr;
  if (!direct) CK(cudaMemcpyAsync(c->d_nat, host, (size_t)L * L, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
  if (direct)  // pinned rows read in place: the copy and the layout conversion are one pass
    nat_to_split_vec_kernel<<<grid_for((int64_t)L * L / 32), 256, 0, c->stream>>>(
        static_cast<const int8_t*>(direct), L, dst, c->d_flag);
  else if (L >= 32)
    nat_to_split_vec_kernel<<<grid_for((int64_t)L * L / 32), 256, 0, c->stream>>>(c->d_nat, L, dst, c->d_flag);
  else
    nat_to_split_kernel<<<grid_for((int64_t)L * L), 256, 0, c->stream>>>(c->d_nat, L, dst, c->d_flag);
  CK(cudaGetLastError());
  int bad = 0;
  CK(cudaMemcpyAsync(&bad, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return bad ? MCRG_EINVAL : MCRG_OK;
}

// The HBM sweep kernel raises a flag when a bulk copy of its band does not
// land within its bounded wait (the lattice it wrote is then not a valid
// sweep).  Entry points that return results drain the stream, read and clear
// the flag, and report MCRG_ETIMEDOUT instead of the results.
static int sweep_status(mcrg_ctx* c) {
  if (!c->is_tiled) return MCRG_OK;
  const int h = tiled_status(&c->tiled, c->stream);
  return h < 0 ? MCRG_EIO : h ? MCRG_ETIMEDOUT : MCRG_OK;
}

int mcrg_get_spins(mcrg_ctx* c, int8_t* host) {
  if (!c || !host) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  const int L = c->cfg.L;
  const uint8_t* src = c->is_tiled ? tiled_state(&c->tiled) : c->d_state;
  // Converted on the device, then one copy-engine transfer: writing host rows
  // in place from the kernel measured 2.4x slower over the host link than
  // the DMA copy of the same bytes (reads in place are as fast as DMA, see
  // mcrg_set_spins).
  if (L >= 32)
    split_to_nat_vec_kernel<<<grid_for((int64_t)L * L / 32), 256, 0, c->stream>>>(src, L, c->d_nat);
  else
    split_to_nat_kernel<<<grid_for((int64_t)L * L), 256, 0, c->stream>>>(src, L, c->d_nat);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(host, c->d_nat, (size_t)L * L, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return sweep_status(c);
}

int mcrg_sweep(mcrg_ctx* c, int64_t n_sweeps) {
  if (!c || n_sweeps < 0) return MCRG_EINVAL;
  if (n_sweeps == 0) return MCRG_OK;
  CK(cudaSetDevice(c->cfg.device));
  if (c->is_tiled) {
    int rc = tiled_sweeps(&c->tiled, (uint32_t)c->t, n_sweeps, c->stream);
    if (rc) return rc;
    c->t += (uint64_t)n_sweeps;
    return MCRG_OK;
  }
  int64_t nb = 0;
  return run_resident(c, n_sweeps, 0, 0, 1, &nb);
}

// Sample loop shared by mcrg_measure (T-matrix moments) and
// mcrg_measure_flow (flow moments, flow = true).
// update: 0 = sweeps between samples; a cluster kind runs the whole loop in
// the resident chain (shared-memory contexts only).
static int measure_impl(mcrg_ctx* c, int64_t n_samples, int64_t sweeps_between, mcrg_moments* total,
                        int64_t bin_size, mcrg_moments* bins, int64_t n_bins_cap, bool flow, int update = 0) {
  if (!c || n_samples < 0 || sweeps_between < 0) return MCRG_EINVAL;
  if (bins && (bin_size <= 0 || bin_size > kMaxDeviceBin || n_bins_cap < 0)) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  const int nl = c->n_levels, C = c->cfg.n_couplings;
  if (total) {
    memset(total, 0, sizeof *total);
    total->n_levels = nl;
    total->n_couplings = C;
  }
  if (bins)
    for (int64_t q = 0; q < n_bins_cap; ++q) {
      memset(&bins[q], 0, sizeof bins[q]);
      bins[q].n_levels = nl;
      bins[q].n_couplings = C;
    }
  if (n_samples == 0) return MCRG_OK;
  const int64_t dev_bin = bins ? bin_size : (n_samples < kMaxDeviceBin ? n_samples : kMaxDeviceBin);
  std::vector<mcrg_moments> h;
  int64_t nb = 0;
  if (c->is_tiled) {
    int rc = tiled_measure(&c->tiled, (uint32_t)c->t, (uint32_t)c->n, n_samples, sweeps_between, dev_bin, &nb,
                           c->stream, flow);
    if (rc) return rc;
    c->t += (uint64_t)(n_samples * sweeps_between);
    c->n += (uint64_t)n_samples;
    h.resize((size_t)nb);
    CK(cudaMemcpyAsync(h.data(), tiled_bins(&c->tiled), sizeof(mcrg_moments) * (size_t)nb,
                       cudaMemcpyDeviceToHost, c->stream));
  } else {
    int rc = run_resident(c, 0, n_samples, sweeps_between, dev_bin, &nb, flow, update);
    if (rc) return rc;
    h.resize((size_t)nb);
    CK(cudaMemcpyAsync(h.data(), c->d_bins, sizeof(mcrg_moments) * (size_t)nb, cudaMemcpyDeviceToHost,
                       c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  if (int rc = sweep_status(c)) return rc;
  for (int64_t q = 0; q < nb; ++q) {
    if (total) add_moments(total, &h[(size_t)q]);
    if (bins && q < n_bins_cap) bins[q] = h[(size_t)q];
  }
  return MCRG_OK;
}

int mcrg_measure(mcrg_ctx* c, int64_t n_samples, int64_t sweeps_between, mcrg_moments* total, int64_t bin_size,
                 mcrg_moments* bins, int64_t n_bins_cap) {
  return measure_impl(c, n_samples, sweeps_between, total, bin_size, bins, n_bins_cap, false);
}

// n cluster updates at update indices c->t, c->t + 1, ...; queued on the
// context's stream.  The flipped count accumulates in c->d_cl[0].
static int cluster_updates(mcrg_ctx* c, int64_t n, int32_t kind) {
  const int L = c->cfg.L;
  if (!c->d_labels) {
    if (dev_alloc(c->span, &c->d_labels, sizeof(int) * cluster_label_ints(L)) != cudaSuccess) return MCRG_ENOMEM;
    if (dev_alloc(c->span, &c->d_cl, 2 * sizeof(unsigned long long)) != cudaSuccess) {
      dev_release(c->span, c->d_labels);
      c->d_labels = nullptr;
      return MCRG_ENOMEM;
    }
    CK(cudaMemsetAsync(c->d_cl, 0, 2 * sizeof(unsigned long long), c->stream));
  }
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->cfg.device));
  uint8_t* st = c->is_tiled ? tiled_state(&c->tiled) : c->d_state;
  const Key key{(uint32_t)c->cfg.seed, (uint32_t)(c->cfg.seed >> 32)};
  const uint32_t tb = bond_threshold(c->cfg.K);
  int* err = reinterpret_cast<int*>(c->d_cl + 1);
  for (int64_t k = 0; k < n; ++k)
    CK(launch_cluster_update(st, L, c->d_labels, kind, key, c->cfg.replica, (uint32_t)(c->t + (uint64_t)k), tb,
                             c->d_cl, err, sms, c->stream));
  c->t += (uint64_t)n;
  return MCRG_OK;
}

// Reads and clears the flipped count and the error flags of the cluster kernels.
static int cluster_readback(mcrg_ctx* c, int64_t* flipped) {
  unsigned long long h[2] = {0, 0};
  if (c->d_cl) {
    CK(cudaMemcpyAsync(h, c->d_cl, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemsetAsync(c->d_cl, 0, sizeof h, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  if (flipped) *flipped = (int64_t)h[0];
  return h[1] ? MCRG_EIO : MCRG_OK;
}

int mcrg_cluster_update(mcrg_ctx* c, int64_t n, int32_t kind, int64_t* flipped) {
  if (!c || n < 0 || (kind != MCRG_UPDATE_WOLFF && kind != MCRG_UPDATE_SWENDSEN_WANG)) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  int rc = cluster_updates(c, n, kind);
  if (rc) return rc;
  return cluster_readback(c, flipped);
}

int mcrg_measure_cluster(mcrg_ctx* c, int64_t n_samples, int64_t updates_between, int32_t kind, mcrg_moments* total,
                         int64_t bin_size, mcrg_moments* bins, int64_t n_bins_cap) {
  if (!c || n_samples < 0 || updates_between < 0 ||
      (kind != MCRG_UPDATE_WOLFF && kind != MCRG_UPDATE_SWENDSEN_WANG))
    return MCRG_EINVAL;
  if (bins && (bin_size <= 0 || n_bins_cap < 0)) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  const int nl = c->n_levels, C = c->cfg.n_couplings;
  // small shared-memory contexts: the whole loop in one resident chain launch.  From L = 128 on one
  // chain's CTA is slower per sample than the device-wide kernels (measured: 120 / 379 us against
  // 61 / 68 us per Wolff sample at L = 128 / 256; 47 against 61 us at L = 64); resident cluster
  // chains pay off in batches (mcrg_batch_run, the server), where many of them fill the GPU.  Both
  // give the same chain.
  if (!c->is_tiled && c->cfg.L <= 64 && cluster_resident(c->cfg.L, nl, C, c->acc.fast) &&
      (!bins || bin_size <= kMaxDeviceBin))
    return measure_impl(c, n_samples, updates_between, total, bin_size, bins, n_bins_cap, false, kind);
  if (total) {
    memset(total, 0, sizeof *total);
    total->n_levels = nl;
    total->n_couplings = C;
  }
  if (bins)
    for (int64_t q = 0; q < n_bins_cap; ++q) {
      memset(&bins[q], 0, sizeof bins[q]);
      bins[q].n_levels = nl;
      bins[q].n_couplings = C;
    }
  // chunks of samples: per sample the cluster updates and one measurement into its own device bin,
  // queued without a host round trip; one read-back per chunk
  constexpr int64_t kChunk = 256;
  if (!c->d_cbins && dev_alloc(c->span, &c->d_cbins, sizeof(mcrg_moments) * kChunk) != cudaSuccess)
    return MCRG_ENOMEM;
  if (!c->is_tiled && !c->d_cjobs && dev_alloc(c->span, &c->d_cjobs, sizeof(ChainJob) * kChunk) != cudaSuccess)
    return MCRG_ENOMEM;
  std::vector<mcrg_moments> h((size_t)kChunk);
  std::vector<ChainJob> jobs(c->is_tiled ? 0 : (size_t)kChunk);
  for (int64_t q0 = 0; q0 < n_samples; q0 += kChunk) {
    const int64_t k = n_samples - q0 < kChunk ? n_samples - q0 : kChunk;
    CK(cudaMemsetAsync(c->d_cbins, 0, sizeof(mcrg_moments) * (size_t)k, c->stream));
    if (!c->is_tiled) {  // measurement-only chain jobs (no sweeps, the state is read, not stored)
      for (int64_t q = 0; q < k; ++q) {
        ChainJob& j = jobs[(size_t)q];
        memset(&j, 0, sizeof j);
        j.L = c->cfg.L;
        j.n_levels = nl;
        j.C = C;
        j.threads = threads_for(c->cfg.L);
        j.key = Key{(uint32_t)c->cfg.seed, (uint32_t)(c->cfg.seed >> 32)};
        j.replica = c->cfg.replica;
        j.n0 = (uint32_t)(c->n + (uint64_t)q);
        j.n_samples = 1;
        j.bin_size = 1;
        j.state = c->d_state;
        j.bins = c->d_cbins + q;
        j.acc = c->acc;
      }
      CK(cudaMemcpyAsync(c->d_cjobs, jobs.data(), sizeof(ChainJob) * (size_t)k, cudaMemcpyHostToDevice,
                         c->stream));
    }
    for (int64_t q = 0; q < k; ++q) {
      int rc = cluster_updates(c, updates_between, kind);
      if (rc) return rc;
      if (c->is_tiled) {
        rc = tiled_measure_sample(&c->tiled, (uint32_t)(c->n + (uint64_t)q), c->d_cbins + q, c->stream);
        if (rc) return rc;
      } else {
        CK(launch_chain(c->d_cjobs + q, 1, c->cfg.L, nl, C, jobs[0].threads, c->acc.fast && c->cfg.L >= 64,
                        c->stream));
      }
    }
    CK(cudaMemcpyAsync(h.data(), c->d_cbins, sizeof(mcrg_moments) * (size_t)k, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->n += (uint64_t)k;
    for (int64_t q = 0; q < k; ++q) {
      if (total) add_moments(total, &h[(size_t)q]);
      if (bins && (q0 + q) / bin_size < n_bins_cap) add_moments(&bins[(q0 + q) / bin_size], &h[(size_t)q]);
    }
  }
  return cluster_readback(c, nullptr);
}

int mcrg_measure_flow(mcrg_ctx* c, int64_t n_samples, int64_t sweeps_between, mcrg_flow_moments* out) {
  if (!c || !out) return MCRG_EINVAL;
  mcrg_moments m;
  const int rc = measure_impl(c, n_samples, sweeps_between, &m, 0, nullptr, 0, true);
  if (rc) return rc;
  memset(out, 0, sizeof *out);
  out->n_levels = c->n_levels;
  out->n_samples = m.n_samples;
  for (int l = 0; l <= c->n_levels; ++l) {
    out->S[l] = m.S[l * MCRG_MAX_COUPLINGS];
    out->S0S[l] = m.SbSb[l * MCRG_MAX_COUPLINGS * MCRG_MAX_COUPLINGS];
  }
  return MCRG_OK;
}

int mcrg_block(mcrg_ctx* c, int level, int8_t* host_out) {
  if (!c || level < 0 || level > c->n_levels + 1 || (c->cfg.L >> level) < 2) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  const int L = c->cfg.L;
  const Key key{(uint32_t)c->cfg.seed, (uint32_t)(c->cfg.seed >> 32)};
  const uint32_t sample = (uint32_t)c->n;
  c->n += 1;
  const uint8_t* src = c->is_tiled ? tiled_state(&c->tiled) : c->d_state;
  uint8_t* tmp = nullptr;
  const size_t LL = (size_t)L * L;
  if (dev_alloc(c->span, &tmp, LL) != cudaSuccess) return MCRG_ENOMEM;
  uint8_t* buf[2] = {tmp, tmp + LL / 2};
  const uint8_t* cur = src;
  int n = L;
  int rc = MCRG_OK;
  for (int l = 0; l < level; ++l, n >>= 1) {
    uint8_t* nxt = buf[l & 1];
    if (launch_block_once(cur, n, nxt, nullptr, key, c->cfg.replica, l + 1, sample, c->stream) != cudaSuccess) {
      rc = MCRG_EIO;
      break;
    }
    cur = nxt;
  }
  if (!rc && host_out) {
    split_to_nat_kernel<<<grid_for((int64_t)n * n), 256, 0, c->stream>>>(cur, n, c->d_nat);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(host_out, c->d_nat, (size_t)n * n, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
      rc = MCRG_EIO;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = MCRG_EIO;
  if (!rc) rc = sweep_status(c);
  dev_release(c->span, tmp);
  return rc;
}

int mcrg_interactions(mcrg_ctx* c, int64_t* out) {
  if (!c || !out) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  const int L = c->cfg.L, C = c->cfg.n_couplings, nl = c->n_levels;
  const Key key{(uint32_t)c->cfg.seed, (uint32_t)(c->cfg.seed >> 32)};
  const uint32_t sample = (uint32_t)c->n;
  c->n += 1;
  const uint8_t* src = c->is_tiled ? tiled_state(&c->tiled) : c->d_state;
  uint8_t* tmp = nullptr;
  int* dS = nullptr;
  const size_t LL = (size_t)L * L;
  if (dev_alloc(c->span, &tmp, LL) != cudaSuccess) return MCRG_ENOMEM;
  if (dev_alloc(c->span, &dS, sizeof(int) * (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS) != cudaSuccess) {
    dev_release(c->span, tmp);
    return MCRG_ENOMEM;
  }
  int rc = MCRG_OK;
  uint8_t* buf[2] = {tmp, tmp + LL / 2};
  const uint8_t* cur = src;
  int n = L;
  if (cudaMemsetAsync(dS, 0, sizeof(int) * (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS, c->stream) != cudaSuccess)
    rc = MCRG_EIO;
  for (int l = 0; !rc && l <= nl; ++l, n >>= 1) {
    if (launch_couplings_once(cur, n, C, dS + l * MCRG_MAX_COUPLINGS, c->stream) != cudaSuccess) { rc = MCRG_EIO; break; }
    if (l == nl) break;
    uint8_t* nxt = buf[l & 1];
    if (launch_block_once(cur, n, nxt, nullptr, key, c->cfg.replica, l + 1, sample, c->stream) != cudaSuccess) {
      rc = MCRG_EIO;
      break;
    }
    cur = nxt;
  }
  int hS[(MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS];
  if (!rc && cudaMemcpyAsync(hS, dS, sizeof hS, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) rc = MCRG_EIO;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = MCRG_EIO;
  if (!rc) rc = sweep_status(c);
  dev_release(c->span, dS);
  dev_release(c->span, tmp);
  if (rc) return rc;
  for (int l = 0; l <= nl; ++l)
    for (int cc = 0; cc < C; ++cc) out[l * C + cc] = hS[l * MCRG_MAX_COUPLINGS + cc];
  return MCRG_OK;
}

int mcrg_set_counters(mcrg_ctx* c, uint64_t sweeps, uint64_t samples) {
  if (!c || sweeps > 0xFFFFFFFFull || samples > 0xFFFFFFFFull) return MCRG_EINVAL;  // 32-bit Philox time words
  c->t = sweeps;
  c->n = samples;
  return MCRG_OK;
}

int mcrg_counters(mcrg_ctx* c, uint64_t* sweeps, uint64_t* samples) {
  if (!c) return MCRG_EINVAL;
  if (sweeps) *sweeps = c->t;
  if (samples) *samples = c->n;
  return MCRG_OK;
}

int mcrg_tile_shape(mcrg_ctx* c, int32_t* tile_rows, int32_t* tile_cols) {
  if (!c || !c->is_tiled) return MCRG_EINVAL;
  int tr = 0, tc = 0;
  if (tiled_variant(&c->tiled, &tr, &tc) < 0) return MCRG_EAGAIN;
  if (tile_rows) *tile_rows = tr;
  if (tile_cols) *tile_cols = tc;
  return MCRG_OK;
}

int mcrg_stream(mcrg_ctx* c, void** stream) {
  if (!c || !stream) return MCRG_EINVAL;
  *stream = (void*)c->stream;
  return MCRG_OK;
}

int mcrg_sync(mcrg_ctx* c) {
  if (!c) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  const int rc = to_status(cudaStreamSynchronize(c->stream));
  return rc ? rc : sweep_status(c);
}

int mcrg_selftest_wait(int32_t device, int64_t limit_us, int32_t* status, double* waited_s) {
  if (!status || limit_us < 1 || limit_us > 1000000) return MCRG_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return MCRG_EIO;
  CK(cudaSetDevice(device));
  struct {
    int flag;
    int pad;
    unsigned long long waited;
  } h{}, *d = nullptr;
  CK(cudaMalloc(&d, sizeof h));
  int rc = MCRG_OK;
  if (cudaMemset(d, 0, sizeof h) != cudaSuccess) rc = MCRG_EIO;
  if (!rc) {
    wait_selftest_kernel<<<1, 32>>>((uint64_t)limit_us * 1000ull, &d->flag, &d->waited);
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = MCRG_EIO;
  }
  cudaFree(d);
  if (rc) return rc;
  *status = h.flag ? MCRG_ETIMEDOUT : MCRG_OK;
  if (waited_s) *waited_s = (double)h.waited * 1e-9;
  return MCRG_OK;
}

int mcrg_block_lattice(int32_t N, const int8_t* host_in, const int8_t* tie_values, uint64_t seed, uint32_t replica,
                       int32_t level, uint32_t sample, int8_t* host_out, int32_t device) {
  if (N < 2 || N > MCRG_MAX_L || (N & (N - 1)) || !host_in || !host_out || level < 1 || level > 255)
    return MCRG_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return MCRG_EIO;
  const size_t NN = (size_t)N * N, HH = NN / 4;
  int8_t* d_nat = nullptr;
  uint8_t *d_split = nullptr, *d_out = nullptr, *d_tie = nullptr;
  int* d_bad = nullptr;
  int rc = MCRG_OK;
  if (cudaMalloc(&d_nat, NN) != cudaSuccess || cudaMalloc(&d_split, NN) != cudaSuccess ||
      cudaMalloc(&d_out, HH + 16) != cudaSuccess || cudaMalloc(&d_tie, HH + 16) != cudaSuccess ||
      cudaMalloc(&d_bad, sizeof(int)) != cudaSuccess)
    rc = MCRG_ENOMEM;
  cudaStream_t s = 0;
  if (!rc) {
    cudaMemsetAsync(d_bad, 0, sizeof(int), s);
    cudaMemcpyAsync(d_nat, host_in, NN, cudaMemcpyHostToDevice, s);
    nat_to_split_kernel<<<grid_for((int64_t)NN), 256, 0, s>>>(d_nat, N, d_split, d_bad);
    const uint8_t* tie = nullptr;
    if (tie_values) {
      cudaMemcpyAsync(d_nat, tie_values, HH, cudaMemcpyHostToDevice, s);
      nat01_kernel<<<grid_for((int64_t)HH), 256, 0, s>>>(d_nat, (int)HH, d_tie, d_bad);
      tie = d_tie;
    }
    const Key key{(uint32_t)seed, (uint32_t)(seed >> 32)};
    launch_block_once(d_split, N, d_out, tie, key, replica, level, sample, s);
    split_to_nat_kernel<<<grid_for((int64_t)HH), 256, 0, s>>>(d_out, N / 2, d_nat);
    cudaMemcpyAsync(host_out, d_nat, HH, cudaMemcpyDeviceToHost, s);
    int bad = 0;
    cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = MCRG_EIO;
    else if (bad) rc = MCRG_EINVAL;
  }
  cudaFree(d_nat); cudaFree(d_split); cudaFree(d_out); cudaFree(d_tie); cudaFree(d_bad);
  return rc;
}

int mcrg_lattice_couplings(int32_t N, const int8_t* host_in, int32_t n_couplings, int64_t* out, int32_t device) {
  if (N < 2 || N > MCRG_MAX_L || (N & (N - 1)) || !host_in || !out || n_couplings < 1 ||
      n_couplings > MCRG_MAX_COUPLINGS)
    return MCRG_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return MCRG_EIO;
  const size_t NN = (size_t)N * N;
  int8_t* d_nat = nullptr;
  uint8_t* d_split = nullptr;
  int* d_S = nullptr;
  int rc = MCRG_OK;
  if (cudaMalloc(&d_nat, NN) != cudaSuccess || cudaMalloc(&d_split, NN) != cudaSuccess ||
      cudaMalloc(&d_S, sizeof(int) * 8) != cudaSuccess)
    rc = MCRG_ENOMEM;
  if (!rc) {
    cudaStream_t s = 0;
    cudaMemsetAsync(d_S, 0, sizeof(int) * 8, s);
    cudaMemcpyAsync(d_nat, host_in, NN, cudaMemcpyHostToDevice, s);
    nat_to_split_kernel<<<grid_for((int64_t)NN), 256, 0, s>>>(d_nat, N, d_split, d_S + 7);
    launch_couplings_once(d_split, N, n_couplings, d_S, s);
    int h[8];
    cudaMemcpyAsync(h, d_S, sizeof h, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = MCRG_EIO;
    else if (h[7]) rc = MCRG_EINVAL;
    else
      for (int c = 0; c < n_couplings; ++c) out[c] = h[c];
  }
  cudaFree(d_nat); cudaFree(d_split); cudaFree(d_S);
  return rc;
}

}  // extern "C"

int mcrg_rgnn_scalar_output(mcrg_ctx* c, const double* W, double* out) {
  if (!c || !W || !out) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  const int L = c->cfg.L;
  const size_t nwork = (size_t)(L / 32) * (L / 32) + (size_t)(L / 1024) * (L / 1024) + 3;
  if (!c->d_rgnn && dev_alloc(c->span, &c->d_rgnn, sizeof(double) * nwork) != cudaSuccess) return MCRG_ENOMEM;
  const uint8_t* state = c->is_tiled ? tiled_state(&c->tiled) : c->d_state;
  double* d_out = c->d_rgnn + nwork - 1;
  CK(launch_rgnn_scalar(state, L, W, c->d_rgnn, d_out, c->stream));
  CK(cudaMemcpyAsync(out, d_out, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return MCRG_OK;
}

namespace mcrg {

// Starts a new chain on an HBM-resident context (same L, levels, couplings
// and device) without allocating: new K, seed and replica, fresh initial
// coin, counters at zero.  Used by the server's workers to reuse contexts.
int reinit_context(mcrg_ctx* c, double K, uint64_t seed, uint32_t replica) {
  if (!c || !c->is_tiled || !std::isfinite(K)) return MCRG_EINVAL;
  CK(cudaSetDevice(c->cfg.device));
  const Accept acc = make_accept(K);
  const int rc = tiled_reinit(&c->tiled, Key{(uint32_t)seed, (uint32_t)(seed >> 32)}, replica, acc, c->stream);
  if (rc) return rc;
  c->cfg.K = K;
  c->cfg.seed = seed;
  c->cfg.replica = replica;
  c->acc = acc;
  c->t = 0;
  c->n = 0;
  return MCRG_OK;
}

}  // namespace mcrg
