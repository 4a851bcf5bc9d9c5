// mcrg_sweep_stream.cuh -- band-streaming fused two-colour sweep of an
// HBM-resident lattice (one read and one write of every site per sweep).
//
// One 512-thread CTA per SM owns a band of full-width rows [b0, b1) and walks
// it top to bottom, R rows per step (R = 512 threads / chunks per row, so
// every thread updates one 16-byte chunk of each colour per step).  Rows live
// in a ring of shared-memory slots (8R rows per colour, 128 KB per CTA) that
// a single warp fills with TMA bulk copies (cp.async.bulk + one mbarrier per
// stage) five steps ahead of the compute.  Step s:
//   colour 0, rows b0+sR+1 .. b0+(s+1)R   (reads old colour-1 rows)
//   -- barrier --
//   colour 1, rows b0+sR   .. b0+(s+1)R-1 (reads new colour-0 rows), storing
//   both colours of these rows to the output buffer.
// Rows of the two phases never overlap across consecutive steps, so one block
// barrier per step suffices; slots are refilled only after that barrier, when
// every thread has finished the step that last read them.  A prologue updates
// colour 0 on rows b0-1 and b0; rows b0-1 and b1 are halo rows also computed
// by the neighbouring bands (same Philox keys, same values) and not stored.
// Full-width rows need no horizontal halo.
#pragma once
#include "mcrg_ops.cuh"

namespace mcrg {
namespace stream {

struct Params {
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

constexpr int kThreads = 512;
constexpr int kStages = 8;     // mbarriers (stage k uses bar[(k+1) % kStages])
constexpr int kAhead = 5;      // stages in flight ahead of the compute

template <int R>
constexpr size_t smem_bytes() {
  return 128 + 2 * (size_t)(8 * R) * (size_t)(kThreads / R) * 16;
}

// Ring of row slots of one CTA (rows b0-2 .. b1+1 map to slot (r-b0+2) mod SLOTS).
template <int R>
struct Ring {
  static constexpr int CPR = kThreads / R;  // 16-byte chunks per colour row
  static constexpr int H = CPR * 16;        // bytes per colour row
  static constexpr int L = 2 * H;
  static constexpr int SLOTS = 8 * R;
  uint8_t* Ws;
  uint8_t* Bs;
  int b0;
  __device__ __forceinline__ uint8_t* w(int r) const { return Ws + ((r - b0 + 2) & (SLOTS - 1)) * H; }
  __device__ __forceinline__ uint8_t* b(int r) const { return Bs + ((r - b0 + 2) & (SLOTS - 1)) * H; }
};

// Stage k >= 0 brings colour-1 rows [b0+kR+2, b0+(k+1)R+1] and colour-0 rows
// [b0+kR+1, b0+(k+1)R] (clipped to b1+1 / b1); stage -1 brings colour-1 rows
// b0-2 .. b0+1 and colour-0 rows b0-1, b0.  Called by all of warp 0.
template <int R>
__device__ __forceinline__ void issue_stage(const Ring<R>& g, int k, int b1, const uint8_t* in, uint64_t* bar,
                                            int lane) {
  constexpr int H = Ring<R>::H, L = Ring<R>::L;
  constexpr size_t PLANE = (size_t)L * H;
  const int b0 = g.b0;
  int w_lo, w_hi, b_lo, b_hi;
  if (k < 0) {
    w_lo = b0 - 2; w_hi = b0 + 1; b_lo = b0 - 1; b_hi = b0;
  } else {
    w_lo = b0 + k * R + 2; w_hi = min(b0 + (k + 1) * R + 1, b1 + 1);
    b_lo = b0 + k * R + 1; b_hi = min(b0 + (k + 1) * R, b1);
  }
  const int nw = max(0, w_hi - w_lo + 1), nb = max(0, b_hi - b_lo + 1);
  uint64_t* br = &bar[(k + 1) & (kStages - 1)];
  if (lane == 0) {
    fence_proxy_async();
    mbar_expect_tx(br, (uint32_t)((nw + nb) * H));
  }
  __syncwarp();
  for (int x = lane; x < nw + nb; x += 32) {
    if (x < nw) {
      const int r = w_lo + x;
      bulk_g2s(g.w(r), in + PLANE + (size_t)((r + L) & (L - 1)) * H, H, br);
    } else {
      const int r = b_lo + x - nw;
      bulk_g2s(g.b(r), in + (size_t)((r + L) & (L - 1)) * H, H, br);
    }
  }
}

__device__ __forceinline__ bool wait_stage(uint64_t* bar, int k) {
  const uint32_t parity = (uint32_t)(((k + 1) / kStages) & 1);
  bool ok = false;
  for (uint32_t it = 0; it < (1u << 24) && !ok; ++it) ok = mbar_try_wait(&bar[(k + 1) & (kStages - 1)], parity);
  return ok;
}

// Colour-0 chunk c of row r (update in place, then resolve its open sites).
template <int R>
__device__ __forceinline__ void black_chunk(const Ring<R>& g, int r, int c, const Params& P, uint32_t tt) {
  constexpr int H = Ring<R>::H, L = Ring<R>::L;
  const int k0 = c * 16;
  uint8_t* row = g.b(r);
  const uint8_t* mid = g.w(r);
  const uint8_t* up = g.w(r - 1);
  const uint8_t* dn = g.w(r + 1);
  uint32_t tw[4], uw[4], dw[4], mw[4];
  load_words4(row + k0, tw);
  load_words4(up + k0, uw);
  load_words4(dn + k0, dw);
  load_words4(mid + k0, mw);
  const uint32_t prv = load_word(mid + ((k0 - 4) & (H - 1))), nxt = load_word(mid + ((k0 + 16) & (H - 1)));
  const int gr = (r + L) & (L - 1), q = gr & 1;
  const uint4 Rn = stream_block(P.key, P.rep, P_SWEEP_HI, 0u, (uint32_t)gr, (uint32_t)c, tt);
  uint32_t bits = update_chunk<4>(tw, uw, dw, mw, prv, nxt, (uint32_t)q, Rn, P.acc);
  store_words<4>(row + k0, tw);
  while (bits) {
    const int p = __ffs(bits) - 1;
    bits &= bits - 1;
    const int k = k0 + open_byte(p);
    if (resolve_open(row[k], up[k], dn[k], mid[(k - 1 + q) & (H - 1)], mid[(k + q) & (H - 1)], P.key, P.rep, 0u, gr,
                     k, tt, P.acc))
      row[k] ^= 1u;
  }
}

template <int R>
__global__ void __launch_bounds__(kThreads, 1)
    sweep_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, Params P, uint32_t tt,
                 int* __restrict__ status) {
  constexpr int CPR = Ring<R>::CPR, H = Ring<R>::H, L = Ring<R>::L, SLOTS = Ring<R>::SLOTS;
  constexpr size_t PLANE = (size_t)L * H;
  extern __shared__ __align__(128) uint8_t smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  const int tid = threadIdx.x;
  Ring<R> g;
  g.Ws = smem + 128;
  g.Bs = g.Ws + SLOTS * H;
  g.b0 = (int)(((long long)blockIdx.x * L) / gridDim.x);
  const int b0 = g.b0;
  const int b1 = (int)(((long long)(blockIdx.x + 1) * L) / gridDim.x);
  const int nsteps = (b1 - b0 + R - 1) / R;

  if (tid < kStages) mbar_init(&bar[tid], 1);
  if (tid == 0) fence_mbar_init();
  __syncthreads();
  if (tid < 32)
    for (int k = -1; k < kAhead - 1 && k < nsteps; ++k) issue_stage<R>(g, k, b1, in, bar, tid);

  // ---- prologue: colour 0 on rows b0-1 and b0
  bool ok = wait_stage(bar, -1);
  if (ok)
    for (int x = tid; x < 2 * CPR; x += kThreads) black_chunk<R>(g, b0 - 1 + x / CPR, x % CPR, P, tt);

  for (int s = 0; s < nsteps; ++s) {
    if (!wait_stage(bar, s)) ok = false;
    // ---- colour 0, rows b0+sR+1 .. b0+(s+1)R (<= b1)
    {
      const int r = b0 + s * R + 1 + tid / CPR;
      if (ok && r <= b1) black_chunk<R>(g, r, tid % CPR, P, tt);
    }
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(status, 1);
      return;
    }
    if (tid < 32 && s + kAhead - 1 < nsteps) issue_stage<R>(g, s + kAhead - 1, b1, in, bar, tid);
    // ---- colour 1, rows b0+sR .. b0+(s+1)R-1 (<= b1-1); both colours of the row are stored
    const int r = b0 + s * R + tid / CPR, c = tid % CPR;
    if (r <= b1 - 1) {
      const int k0 = c * 16;
      uint8_t* row = g.w(r);
      const uint8_t* mid = g.b(r);
      const uint8_t* up = g.b(r - 1);
      const uint8_t* dn = g.b(r + 1);
      uint32_t tw[4], uw[4], dw[4], mw[4];
      load_words4(row + k0, tw);
      load_words4(up + k0, uw);
      load_words4(dn + k0, dw);
      load_words4(mid + k0, mw);
      const uint32_t prv = load_word(mid + ((k0 - 4) & (H - 1))), nxt = load_word(mid + ((k0 + 16) & (H - 1)));
      *reinterpret_cast<uint4*>(out + (size_t)r * H + k0) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
      const uint4 Rn = stream_block(P.key, P.rep, P_SWEEP_HI, 1u, (uint32_t)r, (uint32_t)c, tt);
      const int q = (r + 1) & 1;
      uint32_t bits = update_chunk<4>(tw, uw, dw, mw, prv, nxt, (uint32_t)q, Rn, P.acc);
      if (bits) {
        store_words<4>(row + k0, tw);
        while (bits) {
          const int p = __ffs(bits) - 1;
          bits &= bits - 1;
          const int k = k0 + open_byte(p);
          if (resolve_open(row[k], up[k], dn[k], mid[(k - 1 + q) & (H - 1)], mid[(k + q) & (H - 1)], P.key, P.rep,
                           1u, r, k, tt, P.acc))
            row[k] ^= 1u;
        }
        load_words4(row + k0, tw);
      }
      *reinterpret_cast<uint4*>(out + PLANE + (size_t)r * H + k0) = make_uint4(tw[0], tw[1], tw[2], tw[3]);
    }
  }
}

}  // namespace stream
}  // namespace mcrg

// ===========================================================================
// Two-CTA-per-SM form for one row per step: NT threads, each updating CH =
// CPR / NT chunks of each colour per step in one straight-line block (CH
// independent Philox chains give the scheduler instruction-level
// parallelism), a ring of SL slots per colour (modulo indexing) so that two
// CTAs fit one SM and one CTA's barrier is covered by the other's work.
// Prefetch: the stage of step s + SL - 4 is issued after step s's barrier.
// ===========================================================================
namespace mcrg {
namespace stream2 {

using stream::Params;

template <int CPR, int NT, int SL>
struct Geo {
  static constexpr int CH = CPR / NT;
  static constexpr int H = CPR * 16;
  static constexpr int L = 2 * H;
  static constexpr int AHEAD = SL - 4;  // stages issued ahead (prologue stage + AHEAD)
};

template <int CPR, int NT, int SL>
constexpr size_t smem_bytes() {
  return 128 + 2 * (size_t)SL * (size_t)CPR * 16;
}

template <int SL>
__device__ __forceinline__ int slot_of(int r, int b0) {
  return (r - b0 + 2) % SL;
}

template <int CPR, int NT, int SL>
__global__ void __launch_bounds__(NT, 2)
    sweep_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, Params P, uint32_t tt,
                 int* __restrict__ status) {
  using G = Geo<CPR, NT, SL>;
  constexpr int H = G::H, L = G::L, CH = G::CH;
  constexpr size_t PLANE = (size_t)L * H;
  extern __shared__ __align__(128) uint8_t smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  uint8_t* Ws = smem + 128;
  uint8_t* Bs = Ws + SL * H;
  const int tid = threadIdx.x;
  const int b0 = (int)(((long long)blockIdx.x * L) / gridDim.x);
  const int b1 = (int)(((long long)(blockIdx.x + 1) * L) / gridDim.x);
  const int nsteps = b1 - b0;
  const Key key = P.key;
  const uint32_t rep = P.rep;
  auto W = [&](int r) { return Ws + slot_of<SL>(r, b0) * H; };
  auto B = [&](int r) { return Bs + slot_of<SL>(r, b0) * H; };

  // stage k >= 0: colour-1 row b0+k+2 (<= b1+1) and colour-0 row b0+k+1 (<= b1);
  // stage -1: colour-1 rows b0-2 .. b0+1, colour-0 rows b0-1, b0
  auto issue = [&](int k) {
    int w_lo, w_hi, b_lo, b_hi;
    if (k < 0) {
      w_lo = b0 - 2; w_hi = b0 + 1; b_lo = b0 - 1; b_hi = b0;
    } else {
      w_lo = b0 + k + 2; w_hi = min(b0 + k + 2, b1 + 1);
      b_lo = b0 + k + 1; b_hi = min(b0 + k + 1, b1);
    }
    const int nw = max(0, w_hi - w_lo + 1), nb = max(0, b_hi - b_lo + 1);
    uint64_t* br = &bar[(k + 1) & (stream::kStages - 1)];
    if (tid == 0) {
      stream::fence_proxy_async();
      stream::mbar_expect_tx(br, (uint32_t)((nw + nb) * H));
    }
    __syncwarp();
    for (int x = tid; x < nw + nb; x += 32) {
      if (x < nw) {
        const int r = w_lo + x;
        stream::bulk_g2s(W(r), in + PLANE + (size_t)((r + L) & (L - 1)) * H, H, br);
      } else {
        const int r = b_lo + x - nw;
        stream::bulk_g2s(B(r), in + (size_t)((r + L) & (L - 1)) * H, H, br);
      }
    }
  };

  // CH chunks of colour `colour` of row r, chunks tid + h*NT; tp = own-colour row,
  // up/dn/mid = other-colour rows r-1, r+1, r.  Returns nothing; stores in place
  // (colour 0) and optionally to `gout` (colour 1).
  if (tid < stream::kStages) stream::mbar_init(&bar[tid], 1);
  if (tid == 0) stream::fence_mbar_init();
  __syncthreads();
  if (tid < 32)
    for (int k = -1; k < G::AHEAD && k < nsteps; ++k) issue(k);

  bool ok = stream::wait_stage(bar, -1);
  // ---- prologue: colour 0 on rows b0-1, b0
  for (int pr = 0; pr < 2; ++pr) {
    const int r = b0 - 1 + pr;
    const int gr = (r + L) & (L - 1), q = gr & 1;
    uint8_t* row = B(r);
    const uint8_t* mid = W(r);
    const uint8_t* up = W(r - 1);
    const uint8_t* dn = W(r + 1);
    uint32_t bits[CH];
#pragma unroll
    for (int h = 0; h < CH; ++h) {
      const int c = tid + h * NT, k0 = c * 16;
      uint32_t tw[4], uw[4], dw[4], mw[4];
      load_words4(row + k0, tw);
      load_words4(up + k0, uw);
      load_words4(dn + k0, dw);
      load_words4(mid + k0, mw);
      const uint4 Rn = stream_block(key, rep, P_SWEEP_HI, 0u, (uint32_t)gr, (uint32_t)c, tt);
      bits[h] = update_chunk<4>(tw, uw, dw, mw, load_word(mid + ((k0 - 4) & (H - 1))),
                                load_word(mid + ((k0 + 16) & (H - 1))), (uint32_t)q, Rn, P.acc);
      if (ok) store_words<4>(row + k0, tw);
    }
#pragma unroll
    for (int h = 0; h < CH; ++h) {
      uint32_t b = ok ? bits[h] : 0u;
      const int k0 = (tid + h * NT) * 16;
      while (b) {
        const int p = __ffs(b) - 1;
        b &= b - 1;
        const int k = k0 + open_byte(p);
        if (resolve_open(row[k], up[k], dn[k], mid[(k - 1 + q) & (H - 1)], mid[(k + q) & (H - 1)], key, rep, 0u, gr,
                         k, tt, P.acc))
          row[k] ^= 1u;
      }
    }
  }

  for (int s = 0; s < nsteps; ++s) {
    if (!stream::wait_stage(bar, s)) ok = false;
    // ---- colour 0, row rb = b0+s+1 (<= b1)
    {
      const int rb = b0 + s + 1;
      const int gr = (rb + L) & (L - 1), q = gr & 1;
      uint8_t* row = B(rb);
      const uint8_t* mid = W(rb);
      const uint8_t* up = W(rb - 1);
      const uint8_t* dn = W(rb + 1);
      uint32_t bits[CH];
#pragma unroll
      for (int h = 0; h < CH; ++h) {
        const int c = tid + h * NT, k0 = c * 16;
        uint32_t tw[4], uw[4], dw[4], mw[4];
        load_words4(row + k0, tw);
        load_words4(up + k0, uw);
        load_words4(dn + k0, dw);
        load_words4(mid + k0, mw);
        const uint4 Rn = stream_block(key, rep, P_SWEEP_HI, 0u, (uint32_t)gr, (uint32_t)c, tt);
        bits[h] = update_chunk<4>(tw, uw, dw, mw, load_word(mid + ((k0 - 4) & (H - 1))),
                                  load_word(mid + ((k0 + 16) & (H - 1))), (uint32_t)q, Rn, P.acc);
        if (ok) store_words<4>(row + k0, tw);
      }
#pragma unroll
      for (int h = 0; h < CH; ++h) {
        uint32_t b = ok ? bits[h] : 0u;
        const int k0 = (tid + h * NT) * 16;
        while (b) {
          const int p = __ffs(b) - 1;
          b &= b - 1;
          const int k = k0 + open_byte(p);
          if (resolve_open(row[k], up[k], dn[k], mid[(k - 1 + q) & (H - 1)], mid[(k + q) & (H - 1)], key, rep, 0u,
                           gr, k, tt, P.acc))
            row[k] ^= 1u;
        }
      }
    }
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(status, 1);
      return;
    }
    if (tid < 32 && s + G::AHEAD < nsteps) issue(s + G::AHEAD);
    // ---- colour 1, row r = b0+s; both colours of the row are stored
    {
      const int r = b0 + s;
      const int q = (r + 1) & 1;
      uint8_t* row = W(r);
      const uint8_t* mid = B(r);
      const uint8_t* up = B(r - 1);
      const uint8_t* dn = B(r + 1);
      uint32_t bits[CH];
      uint32_t keep[CH][4];
#pragma unroll
      for (int h = 0; h < CH; ++h) {
        const int c = tid + h * NT, k0 = c * 16;
        uint32_t uw[4], dw[4], mw[4];
        load_words4(row + k0, keep[h]);
        load_words4(up + k0, uw);
        load_words4(dn + k0, dw);
        load_words4(mid + k0, mw);
        *reinterpret_cast<uint4*>(out + (size_t)r * H + k0) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
        const uint4 Rn = stream_block(key, rep, P_SWEEP_HI, 1u, (uint32_t)r, (uint32_t)c, tt);
        bits[h] = update_chunk<4>(keep[h], uw, dw, mw, load_word(mid + ((k0 - 4) & (H - 1))),
                                  load_word(mid + ((k0 + 16) & (H - 1))), (uint32_t)q, Rn, P.acc);
      }
#pragma unroll
      for (int h = 0; h < CH; ++h) {
        const int k0 = (tid + h * NT) * 16;
        uint32_t b = bits[h];
        if (b) {
          store_words<4>(row + k0, keep[h]);
          while (b) {
            const int p = __ffs(b) - 1;
            b &= b - 1;
            const int k = k0 + open_byte(p);
            if (resolve_open(row[k], up[k], dn[k], mid[(k - 1 + q) & (H - 1)], mid[(k + q) & (H - 1)], key, rep, 1u,
                             r, k, tt, P.acc))
              row[k] ^= 1u;
          }
          load_words4(row + k0, keep[h]);
        }
        *reinterpret_cast<uint4*>(out + PLANE + (size_t)r * H + k0) =
            make_uint4(keep[h][0], keep[h][1], keep[h][2], keep[h][3]);
      }
    }
  }
}

}  // namespace stream2
}  // namespace mcrg
