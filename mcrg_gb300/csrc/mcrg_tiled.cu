// mcrg_tiled.cu -- HBM-resident lattices (MCRG_SMEM_MAX_L < L <= MCRG_MAX_L).
//
// Sweep: one fused two-colour pass per HBM round trip.  A persistent CTA
// takes tiles of TR rows x TC bytes (per colour).  For each tile it stages,
// with TMA bulk copies (cp.async.bulk + mbarrier), the old colour-1 rows
// r0-2 .. r0+TR+1 and colour-0 rows r0-1 .. r0+TR, each widened by 16 bytes
// on both sides (periodic wrap split into separate copies).  It updates
// colour 0 on the tile plus its halo, then colour 1 on the tile from the new
// colour 0, and writes the tile to the other buffer of a ping-pong pair.
// Halo sites are updated by both neighbouring tiles; the counter-based draws
// are keyed by the global site, so both compute the same value.  Reads come
// from one buffer and writes go to the other, so tiles never see each
// other's output within a sweep.  HBM traffic: one read and one write of
// every site per sweep (halo re-reads hit L2).
//
// Measurement: every level with side > MCRG_SMEM_MAX_L runs one grid kernel
// (coupling sums + blocking, straight from global memory); the remaining
// levels and the moment products run in one shared-memory CTA, accumulated
// exactly in int128 (per-sample products of the level-0 sums reach 2^60).
#include <cstring>

#include "mcrg_ops.cuh"
#include "mcrg_tiled.cuh"

namespace mcrg {

namespace {

struct TileParams {
  int L, h, TR, TC, pitch, tiles_x, n_tiles, qcap;
  Key key;
  uint32_t rep;
  Accept acc;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Copies global bytes [k - 16, k - 16 + len) (mod h) of one row into dst.
__device__ __forceinline__ void stage_row(uint8_t* dst, const uint8_t* row, int h, int k0, int len, uint64_t* bar) {
  int g = k0 - 16;
  if (g < 0) g += h;
  int z = 0;
  while (z < len) {
    const int run = min(len - z, h - g);
    bulk_g2s(dst + z, row + g, (uint32_t)run, bar);
    z += run;
    g = 0;
  }
}

constexpr uint32_t kWaitLimit = 1u << 24;

__global__ void __launch_bounds__(256, 2)
    tiled_sweep_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, TileParams P, uint32_t t,
                       int* __restrict__ status) {
  extern __shared__ __align__(128) uint8_t smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  int* qcount = reinterpret_cast<int*>(smem + 16);
  uint32_t* queue = reinterpret_cast<uint32_t*>(smem + 32);
  uint8_t* Ws = smem + 32 + ((P.qcap * 4 + 127) / 128) * 128;
  uint8_t* Bs = Ws + (size_t)(P.TR + 4) * P.pitch;
  const int tid = threadIdx.x, T = blockDim.x;
  const int L = P.L, h = P.h, TR = P.TR, TC = P.TC, pitch = P.pitch;
  const size_t plane = (size_t)L * h;
  const Accept a = P.acc;
  const Key key = P.key;
  const uint32_t rep = P.rep;
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (tid < 4) qcount[tid] = 0;
  __syncthreads();
  uint32_t phase = 0;
  const int rows_staged = 2 * TR + 6;
  const int cpr_all = pitch / 16;  // chunks per staged row (tile + both halos)
  for (int tile = blockIdx.x; tile < P.n_tiles; tile += gridDim.x) {
    const int r0 = (tile / P.tiles_x) * TR, k0 = (tile % P.tiles_x) * TC;
    // ---- stage the tile (one warp issues the bulk copies)
    if (tid < 32) {
      if (tid == 0) {
        fence_proxy_async();
        mbar_expect_tx(bar, (uint32_t)(rows_staged * pitch));
      }
      __syncwarp();
      for (int r = tid; r < rows_staged; r += 32) {
        if (r < TR + 4) {
          const int g = (r0 - 2 + r + L) & (L - 1);
          stage_row(Ws + (size_t)r * pitch, in + plane + (size_t)g * h, h, k0, pitch, bar);
        } else {
          const int rr = r - (TR + 4);
          const int g = (r0 - 1 + rr + L) & (L - 1);
          stage_row(Bs + (size_t)rr * pitch, in + (size_t)g * h, h, k0, pitch, bar);
        }
      }
    }
    bool ok = false;
    for (uint32_t it = 0; it < kWaitLimit && !ok; ++it) ok = mbar_try_wait(bar, phase);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(status, 1);
      return;
    }
    phase ^= 1u;

    // ---- colour 0 on rows r0-1 .. r0+TR (tile + halo), all staged columns
    for (int task = tid; task < (TR + 2) * cpr_all; task += T) {
      const int y = task / cpr_all, z0 = (task % cpr_all) * 16;
      const int gr = (r0 - 1 + y + L) & (L - 1);
      const uint32_t q = (uint32_t)(gr & 1);
      int gk = k0 - 16 + z0;
      if (gk < 0) gk += h;
      if (gk >= h) gk -= h;
      uint8_t* tp = Bs + (size_t)y * pitch + z0;
      const uint8_t* mid = Ws + (size_t)(y + 1) * pitch;
      uint32_t tw[4], uw[4], dw[4], mw[4], nw[4], ties[4];
      load_words4(tp, tw);
      load_words4(Ws + (size_t)y * pitch + z0, uw);
      load_words4(Ws + (size_t)(y + 2) * pitch + z0, dw);
      load_words4(mid + z0, mw);
      uint32_t e = 0;
      if (q) { if (z0 + 16 < pitch) e = mid[z0 + 16]; }
      else if (z0 > 0) e = mid[z0 - 1];
      const uint4 R = stream_block(key, rep, P_SWEEP_HI, 0u, (uint32_t)gr, (uint32_t)(gk >> 4), t);
      if (chunk_update<4>(tw, uw, dw, mw, e, q, R, a, nw, ties)) {
        queue_ties<4>(tw, uw, dw, mw, e, q, ties, nw, &qcount[0], queue, P.qcap,
                      [&](int kb, uint32_t m) { return tie_entry(y, z0 + kb, m); },
                      [&](int kb, uint32_t m) { return resolve_tie(key, rep, 0, gr, gk + kb, m, t, a); });
      }
      store_words<4>(tp, nw);
    }
    __syncthreads();
    {
      const int cnt = min(qcount[0], P.qcap);
      for (int x = tid; x < cnt; x += T) {
        const uint32_t v = queue[x];
        const int y = (int)(v >> 14), z = (int)((v >> 1) & 0x1FFFu);
        const uint32_t m = v & 1u;
        const int gr = (r0 - 1 + y + L) & (L - 1);
        int gk = k0 - 16 + z;
        if (gk < 0) gk += h;
        if (gk >= h) gk -= h;
        if (resolve_tie(key, rep, 0, gr, gk, m, t, a)) Bs[(size_t)y * pitch + z] ^= 1u;
      }
    }
    __syncthreads();
    if (tid == 0) qcount[0] = 0;

    // ---- colour 1 on the tile rows r0 .. r0+TR-1, tile columns
    const int cpr_in = TC / 16;
    for (int task = tid; task < TR * cpr_in; task += T) {
      const int x = 2 + task / cpr_in, z0 = 16 + (task % cpr_in) * 16;
      const int gr = r0 + x - 2;
      const uint32_t q = (uint32_t)((gr + 1) & 1);
      const int gk = k0 - 16 + z0;
      uint8_t* tp = Ws + (size_t)x * pitch + z0;
      const uint8_t* mid = Bs + (size_t)(x - 1) * pitch;
      uint32_t tw[4], uw[4], dw[4], mw[4], nw[4], ties[4];
      load_words4(tp, tw);
      load_words4(Bs + (size_t)(x - 2) * pitch + z0, uw);
      load_words4(Bs + (size_t)x * pitch + z0, dw);
      load_words4(mid + z0, mw);
      const uint32_t e = q ? mid[z0 + 16] : mid[z0 - 1];
      const uint4 R = stream_block(key, rep, P_SWEEP_HI, 1u, (uint32_t)gr, (uint32_t)(gk >> 4), t);
      if (chunk_update<4>(tw, uw, dw, mw, e, q, R, a, nw, ties)) {
        queue_ties<4>(tw, uw, dw, mw, e, q, ties, nw, &qcount[1], queue, P.qcap,
                      [&](int kb, uint32_t m) { return tie_entry(x, z0 + kb, m); },
                      [&](int kb, uint32_t m) { return resolve_tie(key, rep, 1, gr, gk + kb, m, t, a); });
      }
      store_words<4>(tp, nw);
    }
    __syncthreads();
    {
      const int cnt = min(qcount[1], P.qcap);
      for (int xx = tid; xx < cnt; xx += T) {
        const uint32_t v = queue[xx];
        const int x = (int)(v >> 14), z = (int)((v >> 1) & 0x1FFFu);
        const uint32_t m = v & 1u;
        if (resolve_tie(key, rep, 1, r0 + x - 2, k0 - 16 + z, m, t, a)) Ws[(size_t)x * pitch + z] ^= 1u;
      }
    }
    __syncthreads();
    if (tid == 0) qcount[1] = 0;

    // ---- write the tile (both colours) to the output buffer
    for (int task = tid; task < 2 * TR * cpr_in; task += T) {
      const int c = task / (TR * cpr_in), rem = task % (TR * cpr_in);
      const int rr = rem / cpr_in, z0 = 16 + (rem % cpr_in) * 16;
      const uint8_t* src = c == 0 ? Bs + (size_t)(rr + 1) * pitch + z0 : Ws + (size_t)(rr + 2) * pitch + z0;
      uint8_t* dst = out + (size_t)c * plane + (size_t)(r0 + rr) * h + (k0 - 16 + z0);
      *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(src);
    }
    __syncthreads();
  }
}

__global__ void tiled_init_kernel(uint8_t* lat, int L, Key key, uint32_t rep) {
  init_level0(lat, L, key, rep, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Coupling sums of one HBM-resident level (and its blocking into the next).
__global__ void __launch_bounds__(256) level_kernel(const uint8_t* __restrict__ in, int n, uint8_t* __restrict__ out,
                                                    unsigned long long* __restrict__ S, int C, Key key, uint32_t rep,
                                                    int level_out, uint32_t sample, int do_block) {
  __shared__ int part[8][5];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, T = gridDim.x * blockDim.x;
  int a5[5] = {0, 0, 0, 0, 0};
  couplings_vec<4>(in, n, tid, T, a5);
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
      if (m >= 32) couplings_vec<4>(lev, m, tid, T, a5);
      else if (m == 16) couplings_vec<2>(lev, m, tid, T, a5);
      else couplings_scalar(lev, m, tid, T, a5);
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
  const int E = (nl + 1) * C + 2 * nl * C * C;
  mcrg_moments* out = J.bin;
  for (int e = tid; e < E; e += T) {
    if (e < (nl + 1) * C) {
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

int g_num_sms = 0;

TileParams tile_params(const TiledLattice* t) {
  TileParams P;
  memset(&P, 0, sizeof P);
  P.L = t->L;
  P.h = t->L / 2;
  P.TR = t->tile_rows;
  P.TC = t->tile_cols;
  P.pitch = P.TC + 32;
  P.tiles_x = P.h / P.TC;
  P.n_tiles = (P.L / P.TR) * P.tiles_x;
  P.qcap = 1024;
  P.key = t->key;
  P.rep = t->replica;
  P.acc = t->acc;
  return P;
}

size_t sweep_smem(const TileParams& P) {
  return 32 + (size_t)((P.qcap * 4 + 127) / 128) * 128 + (size_t)(2 * P.TR + 6) * P.pitch;
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
  t->acc = acc;
  t->tile_rows = 32;
  t->tile_cols = (L / 2) < 1024 ? (L / 2) : 1024;
  if (!acc.fast) return MCRG_ENOSYS;  // the tiled sweep implements the K < -ln2/4 fast path only
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  const size_t LL = (size_t)L * L;
  if (cudaMalloc(&t->buf[0], LL) != cudaSuccess || cudaMalloc(&t->buf[1], LL) != cudaSuccess) return MCRG_ENOMEM;
  // blocked levels 1 .. min(lt, nl)
  const int lt = first_tail_level(L);
  size_t off = 0;
  for (int l = 1; l <= nl && l <= lt; ++l) {
    t->level_off[l] = off;
    off += (size_t)(L >> l) * (L >> l);
  }
  t->n_hbm = lt;
  if (off && cudaMalloc(&t->levels, off) != cudaSuccess) return MCRG_ENOMEM;
  if (cudaMalloc(&t->d_S, sizeof(unsigned long long) * (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS) != cudaSuccess)
    return MCRG_ENOMEM;
  if (cudaMalloc(&t->d_status, sizeof(int)) != cudaSuccess) return MCRG_ENOMEM;
  cudaMemsetAsync(t->d_S, 0, sizeof(unsigned long long) * (MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS, s);
  cudaMemsetAsync(t->d_status, 0, sizeof(int), s);
  const TileParams P = tile_params(t);
  if (cudaFuncSetAttribute(tiled_sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem(P)) !=
      cudaSuccess)
    return MCRG_EIO;
  cudaFuncSetAttribute(tail_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tiled_sweep_kernel, 256, sweep_smem(P));
  if (per_sm < 1) per_sm = 1;
  t->ctas = g_num_sms * per_sm;
  if (t->ctas > P.n_tiles) t->ctas = P.n_tiles;
  tiled_init_kernel<<<g_num_sms * 8, 256, 0, s>>>(t->buf[0], L, key, replica);
  t->cur = 0;
  return cudaGetLastError() == cudaSuccess ? MCRG_OK : MCRG_EIO;
}

void tiled_free(TiledLattice* t) {
  cudaFree(t->buf[0]);
  cudaFree(t->buf[1]);
  cudaFree(t->levels);
  cudaFree(t->d_S);
  cudaFree(t->d_status);
  cudaFree(t->d_bins);
  *t = TiledLattice();
}

uint8_t* tiled_state(TiledLattice* t) { return t->buf[t->cur]; }
mcrg_moments* tiled_bins(TiledLattice* t) { return t->d_bins; }

int tiled_sweeps(TiledLattice* t, uint32_t t0, int64_t n, cudaStream_t s) {
  const TileParams P = tile_params(t);
  const size_t sm = sweep_smem(P);
  for (int64_t k = 0; k < n; ++k) {
    tiled_sweep_kernel<<<t->ctas, 256, sm, s>>>(t->buf[t->cur], t->buf[t->cur ^ 1], P, t0 + (uint32_t)k,
                                                t->d_status);
    t->cur ^= 1;
  }
  return cudaGetLastError() == cudaSuccess ? MCRG_OK : MCRG_EIO;
}

static int measure_one(TiledLattice* t, uint32_t sample, mcrg_moments* bin, cudaStream_t s) {
  const int L = t->L, nl = t->nl, lt = t->n_hbm;
  const uint8_t* cur = t->buf[t->cur];
  for (int l = 0; l < lt && l <= nl; ++l) {
    const int n = L >> l;
    const int do_block = l < nl;
    uint8_t* nxt = do_block ? t->levels + t->level_off[l + 1] : nullptr;
    const int64_t work = 2 * (int64_t)n * (n / 32);
    int grid = (int)((work + 255) / 256);
    if (grid > g_num_sms * 8) grid = g_num_sms * 8;
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
  const size_t sm = (lt <= nl) ? (size_t)make_plan(L >> lt, nl - lt).bytes : 16;
  tail_kernel<<<1, 256, sm, s>>>(J);
  return cudaGetLastError() == cudaSuccess ? MCRG_OK : MCRG_EIO;
}

int tiled_measure(TiledLattice* t, uint32_t t0, uint32_t n0, int64_t n_samples, int64_t sweeps_between,
                  int64_t bin_size, int64_t* n_bins, cudaStream_t s) {
  const int64_t nb = (n_samples + bin_size - 1) / bin_size;
  if (nb > t->bins_cap) {
    cudaFree(t->d_bins);
    t->d_bins = nullptr;
    t->bins_cap = 0;
    if (cudaMalloc(&t->d_bins, sizeof(mcrg_moments) * (size_t)nb) != cudaSuccess) return MCRG_ENOMEM;
    t->bins_cap = nb;
  }
  if (cudaMemsetAsync(t->d_bins, 0, sizeof(mcrg_moments) * (size_t)nb, s) != cudaSuccess) return MCRG_EIO;
  uint32_t tt = t0;
  for (int64_t k = 0; k < n_samples; ++k) {
    int rc = tiled_sweeps(t, tt, sweeps_between, s);
    if (rc) return rc;
    tt += (uint32_t)sweeps_between;
    rc = measure_one(t, n0 + (uint32_t)k, t->d_bins + k / bin_size, s);
    if (rc) return rc;
  }
  *n_bins = nb;
  return MCRG_OK;
}

int tiled_status(TiledLattice* t, cudaStream_t s) {
  int h = 0;
  if (cudaMemcpyAsync(&h, t->d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  return h;
}

}  // namespace mcrg
