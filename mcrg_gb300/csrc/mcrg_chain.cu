// mcrg_chain.cu -- shared-memory-resident MCRG chain (lattice side L <= 256;
// up to 1024 in the fast acceptance regime, where levels of side >= 64 are
// bit planes).
//
// One CTA owns one lattice for the whole launch: it draws (or loads) the
// configuration into shared memory, runs n_eq thermalisation sweeps, then
// n_samples x (sweeps_between sweeps + one measurement), where a measurement
// is every b=2 majority-rule blocking level (src/mcrg.cpp:314-348) with the
// coupling sums of each level (src/lattice.cpp:102-120) and the moment
// products of consecutive levels (src/mcrg.cpp:72-98).  Nothing touches HBM
// between the initial load and the final store except the per-bin moment
// flushes.
//
// Fast acceptance regime, L >= 64: every level of side >= 64 is kept only as
// bit-plane words; sweeps, coupling sums and blocking of those levels run
// bit-sliced (mcrg_resident_bits.cuh).  The levels of side <= 32 of every
// chain are measured by warp 0 from row words in registers
// (mcrg_small_levels.cuh), without shared memory or barriers per level.
// Sweep (L <= 32): the 16 sites of a 16-byte chunk of one colour row are updated with
// byte-SWAR arithmetic from one Philox block (one 8-bit draw per site).  A
// site whose 8-bit draw equals the top byte of its threshold is left open and
// queued; after the colour's pass the queue is resolved exactly with the
// remaining 24 bits from the P_SWEEP_LO stream.  Same-colour sites do not
// interact, so resolving them after the pass gives the same result as
// resolving them in place.
// Cluster chains (ChainJob.update = Wolff / Swendsen-Wang, L <= 256): each
// Monte Carlo step is a cluster update of level 0 in shared memory
// (mcrg_resident_cluster.cuh) instead of a sweep; the measurement is the same.
#include <atomic>

#include "mcrg_ops.cuh"
#include "mcrg_resident_bits.cuh"
#include "mcrg_resident_cluster.cuh"
#include "mcrg_small_levels.cuh"

namespace mcrg {

// One sweep of a resident lattice: colour 0, then colour 1.
__device__ __forceinline__ void chain_sweep(uint8_t* lat, int L, uint32_t t, Key key, uint32_t rep, const Accept& acc,
                                         bool vec, int tid, int T, uint32_t* scratch) {
  for (int c = 0; c < 2; ++c) {
    if (vec) {
      if (L >= 32) sweep_colour_vec<4>(lat, L, c, t, key, rep, acc, tid, T, scratch);
      else sweep_colour_vec<2>(lat, L, c, t, key, rep, acc, tid, T, scratch);
    } else {
      sweep_colour_scalar(lat, L, c, t, key, rep, acc, tid, T);
    }
    chain_sync(T);
  }
}

// ---------------------------------------------------------------------------
// One chain, run by T threads (tid = 0 .. T-1) on the shared memory at `smem`
// (make_plan(L, n_levels, C, planes, cluster, T).bytes of it): the whole CTA
// (chain_kernel) or one warp-aligned group of a CTA (pool_kernel).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void run_chain(const ChainJob& J, uint8_t* smem, int tid, int T) {
  const int L = J.L, nl = J.n_levels, C = J.C;
  const Key key = J.key;
  const uint32_t rep = J.replica;
  const Accept acc = J.acc;
  // L >= 64 in the fast regime: levels of side >= 64 are plane words
  const bool bits = acc.fast && L >= 64;
  const int upd = J.update;  // 0: sweeps, else the cluster update kind
  const SmemPlan plan = make_plan(L, nl, C, bits, upd != 0, T);
  uint8_t* lat = smem;
  int* S = reinterpret_cast<int*>(smem + plan.s_off);
  int2* tab = reinterpret_cast<int2*>(smem + plan.tab_off);
  long long* macc = reinterpret_cast<long long*>(smem + plan.acc_off);
  // moment entries: T-matrix moments (S, Sb S, Sb Sb) or flow moments (S_l, S_l S_0 of coupling 0)
  const int E = J.flow ? 2 * (nl + 1) : plan.E;
  uint32_t* scratch = reinterpret_cast<uint32_t*>(smem + plan.scr_off) + (tid >> 5) * kOpenPerWarp;
  const bool vec = acc.fast && L >= 16;
  uint32_t* pl = bits ? reinterpret_cast<uint32_t*>(smem) : nullptr;
  int* qn = bits ? reinterpret_cast<int*>(smem + plan.qn_off) : nullptr;
  uint4* oq = bits ? reinterpret_cast<uint4*>(smem + plan.q_off) : nullptr;

  // ---- configuration into shared memory
  if (bits) {
    if (J.init) resident::init_planes(pl, L, key, rep, tid, T);
    else resident::pack_lattice(J.state, pl, L, tid, T);
  } else if (J.init) {
    init_level0(lat, L, key, rep, tid, T);
  } else {
    const uint4* src = reinterpret_cast<const uint4*>(J.state);
    uint4* dst = reinterpret_cast<uint4*>(lat);
    for (int v = tid; v < L * L / 16; v += T) dst[v] = src[v];
  }
  // ---- moment entries: x | y << 16 (indices into S, y = 0xFFFF for a plain sum)
  //      and the output slot (kind << 16 | index into S / SbS / SbSb)
  for (int e = tid; e < E; e += T) {
    int x, y, out;
    if (J.flow) {
      // e <= nl: sum of S_e (coupling 0) into S[e*5]; else S_l S_0 into SbSb[l*25], l = e - nl - 1
      const int l = e <= nl ? e : e - nl - 1;
      x = l * MCRG_MAX_COUPLINGS;
      y = e <= nl ? 0xFFFF : 0;
      out = e <= nl ? x : ((2 << 16) | (l * MCRG_MAX_COUPLINGS * MCRG_MAX_COUPLINGS));
    } else if (e < (nl + 1) * C) {
      const int l = e / C, c = e % C;
      x = l * MCRG_MAX_COUPLINGS + c;
      y = 0xFFFF;
      out = x;
    } else {
      const int e2 = e - (nl + 1) * C, kind = e2 / (nl * C * C), e3 = e2 % (nl * C * C);
      const int l = e3 / (C * C), a = (e3 % (C * C)) / C, b = e3 % C;
      x = (l + 1) * MCRG_MAX_COUPLINGS + a;
      y = (kind == 0 ? l : l + 1) * MCRG_MAX_COUPLINGS + b;
      out = ((1 + kind) << 16) | ((l * MCRG_MAX_COUPLINGS + a) * MCRG_MAX_COUPLINGS + b);
    }
    tab[e] = make_int2(x | (y << 16), out);
    macc[e] = 0;
  }
  for (int x = tid; x < (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS; x += T) S[x] = 0;
  if (bits && tid < 2) qn[tid] = 0;
  chain_sync(T);

  // one Monte Carlo step at update index tt: a sweep, or a cluster update
  auto step = [&](uint32_t tt) {
    if (upd) {
      uint8_t* work = smem + plan.cl_off;
      if (bits) rcluster::update_planes(pl, L, work, key, rep, tt, J.bond_tb, upd, tid, T);
      else rcluster::update_bytes(lat, L, work, key, rep, tt, J.bond_tb, upd, tid, T);
    } else if (bits) {
      resident::sweep(pl, L, tt, key, rep, acc, tid, T, oq, qn);
    } else {
      chain_sweep(lat, L, tt, key, rep, acc, vec, tid, T, scratch);
    }
  };
  uint32_t t = J.t0;
  int64_t bin_fill = 0;           // samples in the current bin (warp 0)
  mcrg_moments* bin_out = J.bins;  // the current bin (warp 0)
  for (int64_t s = 0; s < J.n_eq; ++s) step(t++);
  for (int64_t n = 0; n < J.n_samples; ++n) {
    for (int64_t s = 0; s < J.sweeps_between; ++s) step(t++);
    // ---- measurement.  Levels of side >= 64: the whole chain, sums into S by
    //      shared-memory atomics (S is zero here), a barrier after each blocking.
    //      Levels of side <= 32: warp 0 from row words in registers.
    const uint32_t sample = J.n0 + (uint32_t)n;
    if (J.sweeps_between == 0) chain_sync(T);  // no step since the last measurement reset S
    int m = L, l = 0;
    bool in_regs = false;  // warp 0 holds level l as row words
    uint32_t row = 0;
    while (l <= nl && m >= 64) {
      const uint8_t* lev = smem + plan.off[l];
      int a5[5] = {0, 0, 0, 0, 0};
      if (bits) {
        const uint32_t* P = reinterpret_cast<const uint32_t*>(lev);
        if (C <= 2) resident::couplings_planes_c2(P, m, tid, T, a5);
        else resident::couplings_planes<5>(P, m, tid, T, a5);
      } else {
        if (C <= 2) couplings_vec<4, 2>(lev, m, tid, T, a5);
        else couplings_vec<4>(lev, m, tid, T, a5);
      }
      if (C <= 2) reduce_into<2>(a5, S + l * MCRG_MAX_COUPLINGS, C);
      else reduce_into<5>(a5, S + l * MCRG_MAX_COUPLINGS, C);
      if (l == nl) break;
      if (bits && m == 64) {  // the blocking into side 32 lands in warp 0's registers
        if (tid < 32) row = small::block_planes_row(reinterpret_cast<const uint32_t*>(lev), key, rep, l + 1, sample, tid);
        in_regs = true;
      } else {
        uint8_t* nxt = smem + plan.off[l + 1];
        if (bits) resident::block_planes(reinterpret_cast<const uint32_t*>(lev), m, nxt, key, rep, l + 1, sample, tid, T);
        else block_vec(lev, m, nxt, nullptr, key, rep, l + 1, sample, tid, T);
        chain_sync(T);
      }
      ++l;
      m >>= 1;
    }
    if (l <= nl && m <= 32 && tid < 32) {
      if (!in_regs) row = tid < m ? small::level_row(smem + plan.off[l], m, tid) : 0u;
      if (C <= 2) small::levels<2>(row, m, l, nl, C, key, rep, sample, S);
      else small::levels<5>(row, m, l, nl, C, key, rep, sample, S);
    }
    chain_sync(T);  // every sum in S; nobody reads this sample's levels any more
    // ---- moment products, bin flush and the reset of S: warp 0, each entry
    //      owned by one lane (the other warps go on with the next steps)
    if (tid < 32) {
      for (int e = tid; e < E; e += 32) {
        const int2 te = tab[e];
        const long long xv = S[te.x & 0xFFFF];
        const int yi = (te.x >> 16) & 0xFFFF;
        macc[e] += yi == 0xFFFF ? xv : xv * (long long)S[yi];
      }
      const bool last = n == J.n_samples - 1;
      if (++bin_fill == J.bin_size || last) {  // (a running count: no 64-bit division per sample)
        mcrg_moments* out = bin_out++;
        for (int e = tid; e < E; e += 32) {
          const int o = tab[e].y, kind = o >> 16, idx = o & 0xFFFF;
          const long long v = macc[e];
          if (kind == 0) {
            out->S[idx] = v;
          } else {
            mcrg_i128 w;
            w.lo = (uint64_t)v;
            w.hi = v >> 63;
            if (kind == 1) out->SbS[idx] = w;
            else out->SbSb[idx] = w;
          }
          macc[e] = 0;
        }
        if (tid == 0) {
          out->n_levels = nl;
          out->n_couplings = C;
          out->n_samples = bin_fill;
        }
        bin_fill = 0;
      }
      __syncwarp();
      for (int x = tid; x < (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS; x += 32) S[x] = 0;
    }
  }

  // ---- final configuration back to HBM
  if (bits) {
    if (J.store) resident::unpack_lattice(pl, J.state, L, tid, T);
  } else if (J.store) {
    const uint4* src = reinterpret_cast<const uint4*>(lat);
    uint4* dst = reinterpret_cast<uint4*>(J.state);
    for (int v = tid; v < L * L / 16; v += T) dst[v] = src[v];
  }
}

// One chain per CTA.  MAXT / MINB: launch bounds of the instantiation (256 x 3
// for L <= 256, 512 x 2 for the plane chains of L >= 512, which run one or
// two CTAs per SM).
template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) chain_kernel(const ChainJob* __restrict__ jobs) {
  extern __shared__ __align__(16) uint8_t smem[];
  run_chain(jobs[blockIdx.x], smem, threadIdx.x, blockDim.x);
}

// Persistent batch: every CTA takes packs from the queue in order (one
// atomicAdd per pack) until none is left.  A pack is `count` chains of
// `threads` threads each, laid out as consecutive warp-aligned groups of the
// CTA with `stride` bytes of shared memory apiece; threads beyond the pack's
// groups wait at the CTA barrier that ends the pack.  Each group copies its
// job into shared memory first, so the chain reads its descriptor from there.
template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) pool_kernel(const PoolQueue* __restrict__ q) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int s_pack;
  __shared__ ChainJob s_job[kPoolMaxGroups];
  // the class of this SM: its share of the SM ids
  int home = 0;
  if (threadIdx.x == 0) {
    unsigned smid, nsmid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(nsmid));
    const int frac = (int)(((unsigned long long)smid << 16) / (nsmid ? nsmid : 1u));
    for (int k = 1; k < q->n_classes; ++k)
      if (frac >= q->sm_edge[k]) home = k;
  }
  unsigned done_mask = 0;  // classes found empty (thread 0)
  for (;;) {
    if (threadIdx.x == 0) {
      int p = -1;
      for (int j = 0; j < q->n_classes && p < 0; ++j) {
        const int k = (home + j) % q->n_classes;
        if ((done_mask >> k) & 1u) continue;
        const int n_k = q->first[k + 1] - q->first[k];
        const int i = n_k > 0 ? (int)atomicAdd(q->next + 16 * k, 1u) : n_k;
        if (i < n_k) p = q->first[k] + i;
        else done_mask |= 1u << k;
      }
      s_pack = p;
    }
    __syncthreads();
    const int p = s_pack;
    if (p < 0) break;
    const PoolPack pk = q->packs[p];
    const int g = (int)threadIdx.x / pk.threads, tid = (int)threadIdx.x - g * pk.threads;
    if (g < pk.count) {
      if (tid == 0) s_job[g] = q->jobs[pk.first + g];
      chain_sync(pk.threads);
      run_chain(s_job[g], smem + (size_t)g * pk.stride, tid, pk.threads);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// The served request loop: persistent CTAs drain the host ring (ServeEntry,
// mcrg_internal.cuh).  Every wait is bounded: a CTA with nothing to claim
// leaves after ctl->idle_ns of device time, and the server launches the loop
// again when entries are published while no CTA is left.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_volatile_s32(const int32_t* p) { return *reinterpret_cast<const volatile int32_t*>(p); }
__device__ __forceinline__ void st_release_sys(unsigned int* p, unsigned int v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long serve_clock_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void __launch_bounds__(kServeThreads, 1) serve_kernel(ServeArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ long long s_idx;
  __shared__ __align__(16) ServeEntry s_entry;
  volatile unsigned long long* vctr = a.ctr;
  if (threadIdx.x == 0) atomicAdd(a.ctr + 1, 1ull);
  for (;;) {
    if (threadIdx.x == 0) {
      long long got = -1;
      const unsigned long long idle = *reinterpret_cast<const volatile unsigned long long*>(&a.ctl->idle_ns);
      const unsigned long long t0 = serve_clock_ns();
      unsigned ns = 128;
      for (;;) {
        if (ld_volatile_s32(&a.ctl->stop)) break;
        if ((long long)(vctr[1] - vctr[2]) > (long long)ld_volatile_s32(&a.ctl->max_live)) break;
        const unsigned long long tail = ld_acquire_sys(&a.ctl->tail);
        const unsigned long long h = vctr[0];
        if (h < tail) {
          if (atomicCAS(a.ctr, h, h + 1) == h) {
            got = (long long)h;
            break;
          }
          continue;
        }
        if (serve_clock_ns() - t0 > idle) break;
        __nanosleep(ns);
        if (ns < 4096) ns <<= 1;
      }
      s_idx = got;
      if (got < 0) atomicAdd(a.ctr + 2, 1ull);  // this CTA leaves
    }
    __syncthreads();
    const long long idx = s_idx;
    if (idx < 0) break;
    // the entry into shared memory (ordered after thread 0's acquire by the barrier)
    {
      const uint4* src = reinterpret_cast<const uint4*>(a.ring + (size_t)(idx % a.cap));
      uint4* dst = reinterpret_cast<uint4*>(&s_entry);
      for (int v = threadIdx.x; v < (int)(sizeof(ServeEntry) / 16); v += blockDim.x) dst[v] = src[v];
    }
    __syncthreads();
    const PoolPack pk = s_entry.pk;
    const int g = (int)threadIdx.x / pk.threads, tid = (int)threadIdx.x - g * pk.threads;
    if (g < pk.count) run_chain(s_entry.jobs[g], smem + (size_t)g * pk.stride, tid, pk.threads);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence_system();
      st_release_sys(a.done + (size_t)(idx % a.cap), (unsigned int)(idx + 1));
    }
  }
}

// ---------------------------------------------------------------------------
// Stateless helpers: one blocking step / one coupling evaluation on a device
// lattice in split layout (single CTA; sizes up to MCRG_MAX_L).
// ---------------------------------------------------------------------------
__global__ void block_once_kernel(const uint8_t* in, int N, uint8_t* out, const uint8_t* tie_nat, Key key,
                                  uint32_t rep, int level, uint32_t sample) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, T = gridDim.x * blockDim.x;
  if (N >= 32) block_vec(in, N, out, tie_nat, key, rep, level, sample, tid, T);
  else block_scalar(in, N, out, tie_nat, key, rep, level, sample, tid, T);
}

__global__ void couplings_once_kernel(const uint8_t* in, int N, int C, int* out) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, T = gridDim.x * blockDim.x;
  int a5[5] = {0, 0, 0, 0, 0};
  if (N >= 32) couplings_vec<4>(in, N, tid, T, a5);
  else if (N == 16) couplings_vec<2>(in, N, tid, T, a5);
  else couplings_scalar(in, N, tid, T, a5);
  reduce_into(a5, out, C);
}

cudaError_t launch_chain(const ChainJob* d_jobs, int n_jobs, int L, int n_levels, int C, int threads, bool planes,
                         cudaStream_t stream, bool cluster) {
  if (cluster && L > kClusterMaxL) return cudaErrorInvalidValue;
  const SmemPlan plan = make_plan(L, n_levels, C, planes, cluster, threads);
  constexpr int kMaxSmem = 227 * 1024;  // opt-in shared memory per CTA
  if (plan.bytes > kMaxSmem || threads > 512) return cudaErrorInvalidValue;
  const bool wide = threads > 256;
  // the attribute belongs to (instantiation, device): one bit per device, set once to the maximum;
  // host threads may race here, and setting it twice is harmless
  static std::atomic<uint64_t> configured[2];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = uint64_t(1) << (dev & 63);
  if (plan.bytes > 48 * 1024 && !(configured[wide].load(std::memory_order_acquire) & bit)) {
    e = wide ? cudaFuncSetAttribute(chain_kernel<512, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem)
             : cudaFuncSetAttribute(chain_kernel<256, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    if (e != cudaSuccess) return e;
    configured[wide].fetch_or(bit, std::memory_order_release);
  }
  if (wide) chain_kernel<512, 2><<<n_jobs, threads, plan.bytes, stream>>>(d_jobs);
  else chain_kernel<256, 3><<<n_jobs, threads, plan.bytes, stream>>>(d_jobs);
  return cudaGetLastError();
}

const void* serve_kernel_fn() { return (const void*)serve_kernel; }

cudaError_t serve_prepare(int smem, int* blocks_per_sm) {
  if (smem > kPoolMaxSmem) return cudaErrorInvalidValue;
  static std::atomic<uint64_t> configured;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = uint64_t(1) << (dev & 63);
  if (!(configured.load(std::memory_order_acquire) & bit)) {
    e = cudaFuncSetAttribute(serve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPoolMaxSmem);
    if (e != cudaSuccess) return e;
    configured.fetch_or(bit, std::memory_order_release);
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, serve_kernel, kServeThreads, smem);
}

// The 512-wide instantiation runs one CTA per SM: held to 64 registers for
// two, the chain code spills (measured 6-7 % slower on batches of cluster
// chains).  The 256-wide one runs two per SM: the plane sweep's two words per
// thread and step need ~120 registers (held to 80 for three CTAs it spilled,
// and three CTAs of the one-word sweep were 3 % slower on the batched mix).
const void* pool_kernel_fn(int cta_threads) {
  return cta_threads > 256 ? (const void*)pool_kernel<512, 1> : (const void*)pool_kernel<256, 2>;
}

cudaError_t pool_prepare(int cta_threads, int smem, int* blocks_per_sm) {
  if (smem > kPoolMaxSmem || (cta_threads != 256 && cta_threads != 512)) return cudaErrorInvalidValue;
  static std::atomic<uint64_t> configured[2];
  const bool wide = cta_threads > 256;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = uint64_t(1) << (dev & 63);
  if (!(configured[wide].load(std::memory_order_acquire) & bit)) {
    e = cudaFuncSetAttribute(pool_kernel_fn(cta_threads), cudaFuncAttributeMaxDynamicSharedMemorySize, kPoolMaxSmem);
    if (e != cudaSuccess) return e;
    configured[wide].fetch_or(bit, std::memory_order_release);
  }
  return wide ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pool_kernel<512, 1>, cta_threads, smem)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pool_kernel<256, 2>, cta_threads, smem);
}

cudaError_t launch_block_once(const uint8_t* d_in, int N, uint8_t* d_out, const uint8_t* d_tie_nat, Key key,
                              uint32_t replica, int level, uint32_t sample, cudaStream_t s) {
  const int work = (N >= 32) ? (N / 2) * (N / 32) : (N / 2) * (N / 2);
  int blocks = (work + 255) / 256;
  if (blocks < 1) blocks = 1;
  block_once_kernel<<<blocks, 256, 0, s>>>(d_in, N, d_out, d_tie_nat, key, replica, level, sample);
  return cudaGetLastError();
}

cudaError_t launch_couplings_once(const uint8_t* d_in, int N, int C, int* d_out, cudaStream_t s) {
  const int work = (N >= 32) ? 2 * N * (N / 32) : N * N;
  int blocks = (work + 255) / 256;
  if (blocks < 1) blocks = 1;
  if (blocks > 4096) blocks = 4096;
  void* args[] = {(void*)&d_in, (void*)&N, (void*)&C, (void*)&d_out};
  return cudaLaunchKernel((const void*)couplings_once_kernel, dim3(blocks), dim3(256), args, 0, s);
}

}  // namespace mcrg
