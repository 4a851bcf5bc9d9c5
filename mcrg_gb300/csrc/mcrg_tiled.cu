// mcrg_tiled.cu -- HBM-resident lattices (MCRG_SMEM_MAX_L < L <= MCRG_MAX_L).
//
// Sweep: one fused two-colour pass per HBM round trip (bits::sweep_kernel,
// mcrg_sweep_bits.cuh): CTAs stream bands of full-width rows through shared
// memory with bulk copies, update them as bit-plane words and write both
// colours to the other buffer of a ping-pong pair.  HBM traffic: one read
// and one write of every site per sweep, plus four halo rows per band.
//
// Measurement: every level with side > MCRG_SMEM_MAX_L runs one grid kernel
// (coupling sums + blocking, straight from global memory); the remaining
// levels and the moment products run in one shared-memory CTA, accumulated
// exactly in int128 (per-sample products of the level-0 sums reach 2^60).
#include <cstring>

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <utility>

#include "mcrg_ops.cuh"
#include "mcrg_sweep_bits.cuh"
#include "mcrg_tiled.cuh"

namespace mcrg {

namespace {

__global__ void tiled_init_kernel(uint8_t* lat, int L, Key key, uint32_t rep) {
  init_level0(lat, L, key, rep, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Exact update of colour c of an HBM lattice (L >= 64) for any coupling: the
// acceptance outside the fast regime, where m = 0 or 1 anti-aligned
// neighbours can always flip and m >= 2 draws (or the reverse for K > 0).
// In place: a colour reads only the other colour.  One thread takes four
// consecutive sites of a colour row, which share the 32-site word's two
// high-byte blocks (groups 2w, 2w+1) and one low-bits block (group k >> 2):
// the same draws, site for site, as the resident exact path and the fast
// sweeps (u32 = r8 << 24 | r24, flip iff always[m] or u32 < thr[m]).
__global__ void __launch_bounds__(256) exact_colour_kernel(uint8_t* __restrict__ lat, int L, int c, uint32_t t,
                                                           Key key, uint32_t rep, Accept a) {
  const int half = L / 2;
  uint8_t* Cc = lat + (size_t)c * L * half;
  const uint8_t* Oc = lat + (size_t)(1 - c) * L * half;
  const long long quads = (long long)L * half / 4;
  for (long long qd = (long long)blockIdx.x * blockDim.x + threadIdx.x; qd < quads;
       qd += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(qd / (half / 4)), k0 = (int)(qd - (long long)i * (half / 4)) * 4, q = (i + c) & 1;
    const uint8_t* up = Oc + (size_t)((i - 1) & (L - 1)) * half;
    const uint8_t* dn = Oc + (size_t)((i + 1) & (L - 1)) * half;
    const uint8_t* mid = Oc + (size_t)i * half;
    uint8_t* row = Cc + (size_t)i * half;
    uint32_t m4[4], tv4[4];
    bool draw = false;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = k0 + j;
      const uint32_t tv = row[k];
      m4[j] = (up[k] != tv) + (dn[k] != tv) + (mid[(k - 1 + q) & (half - 1)] != tv) + (mid[(k + q) & (half - 1)] != tv);
      tv4[j] = tv;
      draw |= !((a.always_mask >> m4[j]) & 1u);
    }
    uint32_t flips = 0;
    if (draw) {
      const int w = k0 >> 5;
      const uint4 A = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(2 * w), t);
      const uint4 B = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(2 * w + 1), t);
      const uint4 lo = stream_block(key, rep, P_SWEEP_LO, (uint32_t)c, (uint32_t)i, (uint32_t)(k0 >> 2), t);
      const uint32_t W[8] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int p = (k0 + j) & 31, pos = 8 * (p & 3) + (p >> 2);
        uint32_t r8 = 0;
#pragma unroll
        for (int b = 0; b < 8; ++b) r8 |= ((W[b] >> pos) & 1u) << (7 - b);
        const uint32_t u32 = (r8 << 24) | (u4get(lo, j) & 0xFFFFFFu);
        if (((a.always_mask >> m4[j]) & 1u) || u32 < a.thr[m4[j]]) flips |= 1u << j;
      }
    } else {
      flips = 0xFu;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if ((flips >> j) & 1u) row[k0 + j] = (uint8_t)(tv4[j] ^ 1u);
  }
}

// Coupling sums of one HBM-resident level (and its blocking into the next).
__global__ void __launch_bounds__(256) level_kernel(const uint8_t* __restrict__ in, int n, uint8_t* __restrict__ out,
                                                    unsigned long long* __restrict__ S, int C, Key key, uint32_t rep,
                                                    int level_out, uint32_t sample, int do_block) {
  __shared__ int part[8][5];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, T = gridDim.x * blockDim.x;
  int a5[5] = {0, 0, 0, 0, 0};
  if (C <= 2) couplings_vec<4, 2, 2>(in, n, tid, T, a5);  // two couplings read four rows instead of six
  else couplings_vec<4, 5, 2>(in, n, tid, T, a5);
  if (do_block) block_vec(in, n, out, nullptr, key, rep, level_out, sample, tid, T);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    const int v = __reduce_add_sync(0xFFFFFFFFu, a5[c]);
    if (lane == 0) part[warp][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < C) {
    long long s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w][threadIdx.x];
    atomicAdd(&S[threadIdx.x], (unsigned long long)s);
  }
}

// Remaining levels (side <= MCRG_SMEM_MAX_L) in shared memory, then the
// exact moment products of this sample into `bin`, then S is cleared.
struct TailJob {
  int L, nl, C, lt;          // lt: first level handled here (level lt is read from `src`)
  const uint8_t* src;        // level lt, split layout (NULL when lt > nl)
  unsigned long long* S;     // [(nl+1)*5] sums of levels < lt, int64
  mcrg_moments* bin;
  Key key;
  uint32_t rep, sample;
  int flow;                  // 1: flow moments (sum S_l and S_l * S_0 of coupling 0)
};

__global__ void __launch_bounds__(256) tail_kernel(TailJob J) {
  extern __shared__ __align__(128) uint8_t smem[];
  const int tid = threadIdx.x, T = blockDim.x;
  const int nl = J.nl, C = J.C, lt = J.lt;
  __shared__ long long Sv[(MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS];
  __shared__ int St[(MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS];
  for (int x = tid; x < (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS; x += T) {
    Sv[x] = (long long)J.S[x];
    St[x] = 0;
  }
  if (lt <= nl) {
    const int nt = J.L >> lt;
    const SmemPlan plan = make_plan(nt, nl - lt);
    const uint4* src = reinterpret_cast<const uint4*>(J.src);
    uint4* dst = reinterpret_cast<uint4*>(smem);
    for (int v = tid; v < nt * nt / 16; v += T) dst[v] = src[v];
    __syncthreads();
    int m = nt;
    for (int l = lt; l <= nl; ++l, m >>= 1) {
      const uint8_t* lev = smem + plan.off[l - lt];
      int a5[5] = {0, 0, 0, 0, 0};
      if (m >= 32) {
        if (C <= 2) couplings_vec<4, 2>(lev, m, tid, T, a5);
        else couplings_vec<4>(lev, m, tid, T, a5);
      } else if (m == 16) {
        if (C <= 2) couplings_vec<2, 2>(lev, m, tid, T, a5);
        else couplings_vec<2>(lev, m, tid, T, a5);
      } else {
        couplings_scalar(lev, m, tid, T, a5);
      }
      reduce_into(a5, St + l * MCRG_MAX_COUPLINGS, C);
      if (l < nl) {
        uint8_t* nxt = smem + plan.off[l + 1 - lt];
        if (m >= 32) block_vec(lev, m, nxt, nullptr, J.key, J.rep, l + 1, J.sample, tid, T);
        else block_scalar(lev, m, nxt, nullptr, J.key, J.rep, l + 1, J.sample, tid, T);
      }
      __syncthreads();
    }
    for (int x = tid; x < (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS; x += T)
      if (x >= lt * MCRG_MAX_COUPLINGS) Sv[x] = St[x];
  }
  __syncthreads();
  const int E = J.flow ? 2 * (nl + 1) : (nl + 1) * C + 2 * nl * C * C;
  mcrg_moments* out = J.bin;
  for (int e = tid; e < E; e += T) {
    if (J.flow) {
      // e <= nl: sum of S_e (coupling 0); else S_l S_0 into SbSb[l*25], l = e - nl - 1
      const int l = e <= nl ? e : e - nl - 1;
      if (e <= nl) {
        out->S[l * MCRG_MAX_COUPLINGS] += Sv[l * MCRG_MAX_COUPLINGS];
      } else {
        mcrg_i128* dstv = out->SbSb + l * MCRG_MAX_COUPLINGS * MCRG_MAX_COUPLINGS;
        __int128 cur = ((__int128)dstv->hi << 64) | (__int128)dstv->lo;
        cur += (__int128)Sv[l * MCRG_MAX_COUPLINGS] * (__int128)Sv[0];
        dstv->lo = (uint64_t)cur;
        dstv->hi = (int64_t)(cur >> 64);
      }
    } else if (e < (nl + 1) * C) {
      const int l = e / C, c = e % C;
      out->S[l * MCRG_MAX_COUPLINGS + c] += Sv[l * MCRG_MAX_COUPLINGS + c];
    } else {
      const int e2 = e - (nl + 1) * C, kind = e2 / (nl * C * C), e3 = e2 % (nl * C * C);
      const int l = e3 / (C * C), aa = (e3 % (C * C)) / C, bb = e3 % C;
      const __int128 x = (__int128)Sv[(l + 1) * MCRG_MAX_COUPLINGS + aa];
      const __int128 y = (__int128)Sv[(kind == 0 ? l : l + 1) * MCRG_MAX_COUPLINGS + bb];
      mcrg_i128* dstv = (kind == 0 ? out->SbS : out->SbSb) + (l * MCRG_MAX_COUPLINGS + aa) * MCRG_MAX_COUPLINGS + bb;
      __int128 cur = ((__int128)dstv->hi << 64) | (__int128)dstv->lo;
      cur += x * y;
      dstv->lo = (uint64_t)cur;
      dstv->hi = (int64_t)(cur >> 64);
    }
  }
  if (tid == 0) {
    out->n_levels = nl;
    out->n_couplings = C;
    out->n_samples += 1;
  }
  __syncthreads();
  for (int x = tid; x < (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS; x += T) J.S[x] = 0ull;
}


// Variants of the fused sweep: one instantiation per lattice side (L = 64 <<
// lw) and CTA size; the autotuner picks one per (L, device) by timing each
// eligible variant on the live lattice.
struct Variant {
  int threads, lw, lead;  // threads per CTA, L = 64 << lw, row groups in flight ahead of packing
  int wpt;                // plane words per thread per colour and group
  const void* kern;
  size_t smem;
  int waves;              // bands = waves x resident CTAs (two waves measured slower: more halo rows)
};

#define BITS_VARIANT_X(NT_, WPT_, MINB_, LEAD_, LW_)                                                    \
  Variant {                                                                                              \
    NT_, LW_, LEAD_, WPT_, (const void*)bits::sweep_kernel<NT_, WPT_, MINB_, LEAD_, LW_>,               \
        bits::smem_bytes<NT_ * WPT_, LEAD_>(), 1                                                         \
  }
#define BITS_VARIANT(NT_, MINB_, LEAD_, LW_) BITS_VARIANT_X(NT_, 1, MINB_, LEAD_, LW_)
// per side: 256 threads x 3 CTAs per SM (copy lead 2), x 4 (lead 1), x 2 (lead 3), 512 x 1, 128 x 4;
// and 128 threads with two words each (x 4 CTAs per SM, lead 1 or 2).  L = 16384 adds two words per
// thread at 256 x 2 (lead 1)
#define BITS_VARIANTS_L(LW_)                                                                             \
  BITS_VARIANT(256, 3, 2, LW_), BITS_VARIANT(256, 4, 1, LW_), BITS_VARIANT(256, 2, 3, LW_),             \
      BITS_VARIANT(512, 1, 3, LW_), BITS_VARIANT(128, 4, 3, LW_), BITS_VARIANT_X(128, 2, 4, 1, LW_)

const Variant kVariants[] = {BITS_VARIANT(256, 4, 1, 8),        BITS_VARIANT(256, 3, 2, 8),
                             BITS_VARIANT(256, 2, 3, 8),        BITS_VARIANT(512, 1, 3, 8),
                             BITS_VARIANT_X(128, 2, 4, 1, 8),    BITS_VARIANT_X(128, 2, 4, 2, 8),
                             BITS_VARIANT_X(256, 2, 2, 1, 8),
                             BITS_VARIANTS_L(7),
                             BITS_VARIANTS_L(6),                 BITS_VARIANTS_L(5),
                             BITS_VARIANTS_L(4),                 BITS_VARIANTS_L(3)};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

int block_threads(const Variant& v) { return v.threads; }

bool variant_fits(const Variant& v, int L) { return (64 << v.lw) == L && (v.threads * v.wpt) >= (L / 64); }

// rows per pipeline group
int variant_rows(const Variant& v) { return (v.threads * v.wpt) >> v.lw; }

void launch_variant(const TiledLattice* t, int vi, const uint8_t* in, uint8_t* out, uint32_t tt, cudaStream_t s) {
  const Variant& v = kVariants[vi];
  bits::Params P;
  memset(&P, 0, sizeof P);
  bits::fill_params(P, t->key, t->replica, t->acc.thr[0], t->acc.thr[1]);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v.kern, block_threads(v), v.smem);
  if (per_sm < 1) per_sm = 1;
  // bands of at least four row groups, `waves` times as many as fit the GPU at once
  int bands = t->L / (4 * variant_rows(v));
  if (bands > v.waves * t->sms * per_sm) bands = v.waves * t->sms * per_sm;
  if (bands < 1) bands = 1;
  void* args[] = {(void*)&in, (void*)&out, (void*)&P, (void*)&tt, (void*)&t->d_status};
  // programmatic dependent launch: the CTAs of this sweep are scheduled while
  // the previous kernel drains and wait for it inside the kernel
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(bands);
  cfg.blockDim = dim3(block_threads(v));
  cfg.dynamicSmemBytes = v.smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelExC(&cfg, v.kern, args);
}

int first_tail_level(int L) {
  int l = 0;
  while ((L >> l) > MCRG_SMEM_MAX_L) ++l;
  return l;
}

}  // namespace

int tiled_alloc(TiledLattice* t, int L, int nl, int C, Key key, uint32_t replica, const Accept& acc,
                cudaStream_t s) {
  t->L = L;
  t->nl = nl;
  t->C = C;
  t->key = key;
  t->replica = replica;
  t->acc = acc;  // outside the fast regime the sweeps take the exact per-site path (exact_colour_kernel)
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&t->sms, cudaDevAttrMultiProcessorCount, dev);
    if (t->sms <= 0) t->sms = 1;
  }
  const size_t LL = (size_t)L * L;
  if (dev_alloc(t->span, &t->buf[0], LL) != cudaSuccess || dev_alloc(t->span, &t->buf[1], LL) != cudaSuccess)
    return MCRG_ENOMEM;
  // blocked levels 1 .. min(lt, nl)
  const int lt = first_tail_level(L);
  size_t off = 0;
  for (int l = 1; l <= nl && l <= lt; ++l) {
    t->level_off[l] = off;
    off += (size_t)(L >> l) * (L >> l);
  }
  t->n_hbm = lt;
  if (off && dev_alloc(t->span, &t->levels, off) != cudaSuccess) return MCRG_ENOMEM;
  if (dev_alloc(t->span, &t->d_S, sizeof(unsigned long long) * (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS) !=
      cudaSuccess)
    return MCRG_ENOMEM;
  if (dev_alloc(t->span, &t->d_status, sizeof(int)) != cudaSuccess) return MCRG_ENOMEM;
  cudaMemsetAsync(t->d_S, 0, sizeof(unsigned long long) * (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS, s);
  cudaMemsetAsync(t->d_status, 0, sizeof(int), s);
  for (int v = 0; v < kNumVariants; ++v)
    if (cudaFuncSetAttribute(kVariants[v].kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kVariants[v].smem) != cudaSuccess)
      return MCRG_EIO;
  cudaFuncSetAttribute(tail_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
  t->variant = -1;
  tiled_init_kernel<<<t->sms * 8, 256, 0, s>>>(t->buf[0], L, key, replica);
  t->cur = 0;
  return cudaGetLastError() == cudaSuccess ? MCRG_OK : MCRG_EIO;
}

int tiled_reinit(TiledLattice* t, Key key, uint32_t replica, const Accept& acc, cudaStream_t s) {
  t->key = key;
  t->replica = replica;
  t->acc = acc;
  cudaMemsetAsync(t->d_S, 0, sizeof(unsigned long long) * (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS, s);
  cudaMemsetAsync(t->d_status, 0, sizeof(int), s);
  tiled_init_kernel<<<t->sms * 8, 256, 0, s>>>(t->buf[0], t->L, key, replica);
  t->cur = 0;
  return cudaGetLastError() == cudaSuccess ? MCRG_OK : MCRG_EIO;
}

void tiled_free(TiledLattice* t) {
  dev_release(t->span, t->d_bins);
  dev_release(t->span, t->d_status);
  dev_release(t->span, t->d_S);
  dev_release(t->span, t->levels);
  dev_release(t->span, t->buf[1]);
  dev_release(t->span, t->buf[0]);
  *t = TiledLattice();
}

uint8_t* tiled_state(TiledLattice* t) { return t->buf[t->cur]; }
mcrg_moments* tiled_bins(TiledLattice* t) { return t->d_bins; }

// Picks the fastest eligible tile shape for this lattice side on this device
// (MCRG_TILE=<TR>x<TC> forces one).  Each candidate runs a few sweeps that
// write the idle ping-pong buffer only, so the chain state does not move.
static int autotune(TiledLattice* t, cudaStream_t s) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  if (const char* force = getenv("MCRG_TILE")) {  // "b<threads>l<lead>[x<words per thread>]" forces a variant
    int nt = 0, lead = 2, wpt = 1;
    if (force[0] == 'b' && sscanf(force + 1, "%dl%dx%d", &nt, &lead, &wpt) >= 1)
      for (int v = 0; v < kNumVariants; ++v)
        if (kVariants[v].threads == nt && kVariants[v].lead == lead && kVariants[v].wpt == wpt &&
            variant_fits(kVariants[v], t->L))
          return v;
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({t->L, dev});
    if (it != cache.end()) return it->second;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // two rounds of 20 launches per variant, best round kept: the leading
  // variants differ by ~1 %, below the spread of a single short round
  int best = -1;
  float best_ms = 1e30f;
  float round_best[kNumVariants];
  for (int v = 0; v < kNumVariants; ++v) round_best[v] = 1e30f;
  const int reps = 20;
  for (int round = 0; round < 2; ++round)
    for (int v = 0; v < kNumVariants; ++v) {
      if (!variant_fits(kVariants[v], t->L)) continue;
      launch_variant(t, v, t->buf[t->cur], t->buf[t->cur ^ 1], 0xFFFFFFF0u, s);  // warm-up
      cudaEventRecord(e0, s);
      for (int r = 0; r < reps; ++r) launch_variant(t, v, t->buf[t->cur], t->buf[t->cur ^ 1], 0xFFFFFFF0u + r, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < round_best[v]) round_best[v] = ms;
    }
  for (int v = 0; v < kNumVariants; ++v)
    if (round_best[v] < best_ms) {
      best_ms = round_best[v];
      best = v;
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best < 0) return -1;
  std::lock_guard<std::mutex> lk(mu);
  cache[{t->L, dev}] = best;
  return best;
}

int tiled_variant(TiledLattice* t, int* rows, int* threads) {
  if (t->variant < 0) return -1;
  if (rows) *rows = variant_rows(kVariants[t->variant]);
  if (threads) *threads = kVariants[t->variant].threads;
  return t->variant;
}

int tiled_sweeps(TiledLattice* t, uint32_t t0, int64_t n, cudaStream_t s) {
  if (n <= 0) return MCRG_OK;
  if (!t->acc.fast) {  // two in-place colour passes per sweep
    int grid = (int)(((long long)t->L * t->L / 8 + 255) / 256);
    if (grid > t->sms * 8) grid = t->sms * 8;
    for (int64_t k = 0; k < n; ++k)
      for (int c = 0; c < 2; ++c)
        exact_colour_kernel<<<grid, 256, 0, s>>>(t->buf[t->cur], t->L, c, t0 + (uint32_t)k, t->key, t->replica, t->acc);
    return cudaGetLastError() == cudaSuccess ? MCRG_OK : MCRG_EIO;
  }
  if (t->variant < 0) {
    t->variant = autotune(t, s);
    if (t->variant < 0) return MCRG_ENOSYS;
  }
  for (int64_t k = 0; k < n; ++k) {
    launch_variant(t, t->variant, t->buf[t->cur], t->buf[t->cur ^ 1], t0 + (uint32_t)k, s);
    t->cur ^= 1;
  }
  return cudaGetLastError() == cudaSuccess ? MCRG_OK : MCRG_EIO;
}

static int measure_one(TiledLattice* t, uint32_t sample, mcrg_moments* bin, bool flow, cudaStream_t s) {
  const int L = t->L, nl = t->nl, lt = t->n_hbm;
  const uint8_t* cur = t->buf[t->cur];
  for (int l = 0; l < lt && l <= nl; ++l) {
    const int n = L >> l;
    const int do_block = l < nl;
    uint8_t* nxt = do_block ? t->levels + t->level_off[l + 1] : nullptr;
    const int64_t work = 2 * (int64_t)n * (n / 32);
    int grid = (int)((work + 255) / 256);
    if (grid > t->sms * 8) grid = t->sms * 8;
    if (grid < 1) grid = 1;
    level_kernel<<<grid, 256, 0, s>>>(cur, n, nxt, t->d_S + l * MCRG_MAX_COUPLINGS, t->C, t->key, t->replica, l + 1,
                                      sample, do_block);
    cur = nxt;
  }
  TailJob J;
  J.L = L;
  J.nl = nl;
  J.C = t->C;
  J.lt = lt;
  J.src = (lt <= nl) ? t->levels + t->level_off[lt] : nullptr;
  J.S = t->d_S;
  J.bin = bin;
  J.key = t->key;
  J.rep = t->replica;
  J.sample = sample;
  J.flow = flow ? 1 : 0;
  const size_t sm = (lt <= nl) ? (size_t)make_plan(L >> lt, nl - lt).bytes : 16;
  tail_kernel<<<1, 256, sm, s>>>(J);
  return cudaGetLastError() == cudaSuccess ? MCRG_OK : MCRG_EIO;
}

int tiled_measure(TiledLattice* t, uint32_t t0, uint32_t n0, int64_t n_samples, int64_t sweeps_between,
                  int64_t bin_size, int64_t* n_bins, cudaStream_t s, bool flow) {
  const int64_t nb = (n_samples + bin_size - 1) / bin_size;
  if (nb > t->bins_cap) {
    dev_release(t->span, t->d_bins);
    t->d_bins = nullptr;
    t->bins_cap = 0;
    if (dev_alloc(t->span, &t->d_bins, sizeof(mcrg_moments) * (size_t)nb) != cudaSuccess) return MCRG_ENOMEM;
    t->bins_cap = nb;
  }
  if (cudaMemsetAsync(t->d_bins, 0, sizeof(mcrg_moments) * (size_t)nb, s) != cudaSuccess) return MCRG_EIO;
  uint32_t tt = t0;
  for (int64_t k = 0; k < n_samples; ++k) {
    int rc = tiled_sweeps(t, tt, sweeps_between, s);
    if (rc) return rc;
    tt += (uint32_t)sweeps_between;
    rc = measure_one(t, n0 + (uint32_t)k, t->d_bins + k / bin_size, flow, s);
    if (rc) return rc;
  }
  *n_bins = nb;
  return MCRG_OK;
}

int tiled_measure_sample(TiledLattice* t, uint32_t sample, mcrg_moments* bin, cudaStream_t s) {
  return measure_one(t, sample, bin, false, s);
}

int tiled_status(TiledLattice* t, cudaStream_t s) {
  int h = 0;
  if (cudaMemcpyAsync(&h, t->d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  if (h != 0 && (cudaMemsetAsync(t->d_status, 0, sizeof(int), s) != cudaSuccess ||
                 cudaStreamSynchronize(s) != cudaSuccess))
    return -1;
  return h;
}

}  // namespace mcrg
