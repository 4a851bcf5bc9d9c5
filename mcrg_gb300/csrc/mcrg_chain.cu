// mcrg_chain.cu -- shared-memory-resident MCRG chain (lattice side L <= 256).
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
// Sweep: the 16 sites of a 16-byte chunk of one colour row are updated with
// byte-SWAR arithmetic from one Philox block (one 8-bit draw per site).  A
// site whose 8-bit draw equals the top byte of its threshold is left open and
// queued; after the colour's pass the queue is resolved exactly with the
// remaining 24 bits from the P_SWEEP_LO stream.  Same-colour sites do not
// interact, so resolving them after the pass gives the same result as
// resolving them in place.
#include "mcrg_ops.cuh"

namespace mcrg {

// ---------------------------------------------------------------------------
// One chain per CTA.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) chain_kernel(const ChainJob* __restrict__ jobs) {
  extern __shared__ __align__(16) uint8_t smem[];
  const ChainJob& J = jobs[blockIdx.x];
  const int L = J.L, nl = J.n_levels, C = J.C;
  const int tid = threadIdx.x, T = blockDim.x;
  const Key key = J.key;
  const uint32_t rep = J.replica;
  const Accept acc = J.acc;
  const SmemPlan plan = make_plan(L, nl);
  uint8_t* lat = smem;
  int* S = reinterpret_cast<int*>(smem + plan.s_off);
  int* qcount = reinterpret_cast<int*>(smem + plan.q_off);
  uint32_t* queue = reinterpret_cast<uint32_t*>(smem + plan.q_off + 16);
  const int qcap = plan.qcap;
  const bool vec = acc.fast && L >= 16;

  // ---- configuration into shared memory
  if (J.init) {
    init_level0(lat, L, key, rep, tid, T);
  } else {
    const uint4* src = reinterpret_cast<const uint4*>(J.state);
    uint4* dst = reinterpret_cast<uint4*>(lat);
    for (int v = tid; v < L * L / 16; v += T) dst[v] = src[v];
  }
  if (tid < 2) qcount[tid] = 0;

  // ---- moment entries owned by this thread
  const int E = (nl + 1) * C + 2 * nl * C * C;
  int16_t ox[kMaxOwned], oy[kMaxOwned];
  int oidx[kMaxOwned];
  int64_t oacc[kMaxOwned];
#pragma unroll
  for (int r = 0; r < kMaxOwned; ++r) {
    const int e = tid + r * T;
    oacc[r] = 0;
    ox[r] = -1; oy[r] = -1; oidx[r] = -1;
    if (e < (nl + 1) * C) {
      const int l = e / C, c = e % C;
      ox[r] = (int16_t)(l * MCRG_MAX_COUPLINGS + c);
      oidx[r] = l * MCRG_MAX_COUPLINGS + c;
    } else if (e < E) {
      const int e2 = e - (nl + 1) * C, kind = e2 / (nl * C * C), e3 = e2 % (nl * C * C);
      const int l = e3 / (C * C), a = (e3 % (C * C)) / C, b = e3 % C;
      ox[r] = (int16_t)((l + 1) * MCRG_MAX_COUPLINGS + a);
      oy[r] = (int16_t)((kind == 0 ? l : l + 1) * MCRG_MAX_COUPLINGS + b);
      oidx[r] = (1 + kind) * 100000 + (l * MCRG_MAX_COUPLINGS + a) * MCRG_MAX_COUPLINGS + b;
    }
  }
  sync_group();

  uint32_t t = J.t0;
  auto sweep = [&](uint32_t tt) {
    for (int c = 0; c < 2; ++c) {
      if (vec) {
        if (L >= 32) sweep_colour_vec<4>(lat, L, c, tt, key, rep, acc, &qcount[c], queue, qcap, tid, T);
        else sweep_colour_vec<2>(lat, L, c, tt, key, rep, acc, &qcount[c], queue, qcap, tid, T);
        sync_group();
        const int cnt = qcount[c];
        if (cnt) resolve_queue(lat, L, c, tt, key, rep, acc, cnt, queue, qcap, tid, T);
        sync_group();
        if (tid == 0) qcount[c] = 0;
      } else {
        sweep_colour_scalar(lat, L, c, tt, key, rep, acc, tid, T);
        sync_group();
      }
    }
  };

  for (int64_t s = 0; s < J.n_eq; ++s) sweep(t++);

  int64_t in_bin = 0, bin = 0;
  for (int64_t n = 0; n < J.n_samples; ++n) {
    for (int64_t s = 0; s < J.sweeps_between; ++s) sweep(t++);
    // ---- measurement: every level's coupling sums, blocking level by level
    const uint32_t sample = J.n0 + (uint32_t)n;
    for (int x = tid; x < (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS; x += T) S[x] = 0;
    sync_group();
    int m = L;
    for (int l = 0; l <= nl; ++l, m >>= 1) {
      const uint8_t* lev = smem + plan.off[l];
      int a5[5] = {0, 0, 0, 0, 0};
      if (m >= 32) couplings_vec<4>(lev, m, tid, T, a5);
      else if (m == 16) couplings_vec<2>(lev, m, tid, T, a5);
      else couplings_scalar(lev, m, tid, T, a5);
      reduce_into(a5, S + l * MCRG_MAX_COUPLINGS, C);
      if (l < nl) {
        uint8_t* nxt = smem + plan.off[l + 1];
        if (m >= 32) block_vec(lev, m, nxt, nullptr, key, rep, l + 1, sample, tid, T);
        else block_scalar(lev, m, nxt, nullptr, key, rep, l + 1, sample, tid, T);
      }
      sync_group();
    }
    // ---- moments
#pragma unroll
    for (int r = 0; r < kMaxOwned; ++r) {
      if (ox[r] >= 0) {
        const int64_t x = S[ox[r]];
        oacc[r] += oy[r] >= 0 ? x * (int64_t)S[oy[r]] : x;
      }
    }
    ++in_bin;
    if (in_bin == J.bin_size || n == J.n_samples - 1) {
      mcrg_moments* out = J.bins + bin;
#pragma unroll
      for (int r = 0; r < kMaxOwned; ++r) {
        if (oidx[r] < 0) continue;
        if (oidx[r] < 100000) {
          out->S[oidx[r]] = oacc[r];
        } else {
          mcrg_i128 v;
          v.lo = (uint64_t)oacc[r];
          v.hi = oacc[r] >> 63;
          if (oidx[r] < 200000) out->SbS[oidx[r] - 100000] = v;
          else out->SbSb[oidx[r] - 200000] = v;
        }
        oacc[r] = 0;
      }
      if (tid == 0) {
        out->n_levels = nl;
        out->n_couplings = C;
        out->n_samples = in_bin;
      }
      in_bin = 0;
      ++bin;
    }
    sync_group();
  }

  // ---- final configuration back to HBM
  if (J.store) {
    const uint4* src = reinterpret_cast<const uint4*>(lat);
    uint4* dst = reinterpret_cast<uint4*>(J.state);
    for (int v = tid; v < L * L / 16; v += T) dst[v] = src[v];
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

cudaError_t launch_chain(const ChainJob* d_jobs, int n_jobs, int L, int n_levels, int threads,
                         cudaStream_t stream) {
  const SmemPlan plan = make_plan(L, n_levels);
  static int configured = 0;
  if (plan.bytes > configured) {
    cudaError_t e = cudaFuncSetAttribute(chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    configured = 200 * 1024;
  }
  chain_kernel<<<n_jobs, threads, plan.bytes, stream>>>(d_jobs);
  return cudaGetLastError();
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
  couplings_once_kernel<<<blocks, 256, 0, s>>>(d_in, N, C, d_out);
  return cudaGetLastError();
}

}  // namespace mcrg
