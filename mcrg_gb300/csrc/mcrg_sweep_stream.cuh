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
  return 128 + 2 * (size_t)(8 * R) * (size_t)(kThreads / R) * 16 + (kThreads / 32) * 64 * 4;
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

// One open site resolved exactly: returns true when it flips.
template <int R>
__device__ __forceinline__ void resolve_site(const Ring<R>& g, uint32_t colour, int r, int k, const Params& P,
                                             uint32_t tt) {
  constexpr int H = Ring<R>::H, L = Ring<R>::L;
  uint8_t* row = colour ? g.w(r) : g.b(r);
  const uint8_t* up = colour ? g.b(r - 1) : g.w(r - 1);
  const uint8_t* dn = colour ? g.b(r + 1) : g.w(r + 1);
  const uint8_t* mid = colour ? g.b(r) : g.w(r);
  const int gr = (r + L) & (L - 1), q = (gr + (int)colour) & 1;
  if (resolve_open(row[k], up[k], dn[k], mid[(k - 1 + q) & (H - 1)], mid[(k + q) & (H - 1)], P.key, P.rep, colour, gr,
                   k, tt, P.acc))
    row[k] ^= 1u;
}

// Open-site descriptor: colour << 31 | (row - b0 + 2) << 13 | k.
constexpr int kWarpOpen = 64;  // descriptors one warp resolves cooperatively per pass

// Resolves the open sites of the warp: this lane's colour-0 chunk (row rb)
// and its deferred colour-1 chunk (row rw), both at chunk byte offset k0.
// Sites are spread over the warp's lanes (one Philox block each) instead of
// each owner resolving its own, which would serialise the warp.
template <int R>
__device__ __forceinline__ void warp_resolve(const Ring<R>& g, uint32_t* scratch, uint32_t bits_b, int rb,
                                             uint32_t bits_w, int rw, int k0, const Params& P, uint32_t tt) {
  const int lane = threadIdx.x & 31;
  const int cnt = __popc(bits_b) + __popc(bits_w);
  if (__ballot_sync(0xFFFFFFFFu, cnt != 0) == 0) return;
  int off = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xFFFFFFFFu, off, d);
    if (lane >= d) off += y;
  }
  const int total = __shfl_sync(0xFFFFFFFFu, off, 31);
  int slot = off - cnt;
  while (bits_b) {
    const int p = __ffs(bits_b) - 1;
    bits_b &= bits_b - 1;
    const int k = k0 + open_byte(p);
    if (slot < kWarpOpen) scratch[slot] = ((uint32_t)(rb - g.b0 + 2) << 13) | (uint32_t)k;
    else resolve_site<R>(g, 0u, rb, k, P, tt);
    ++slot;
  }
  while (bits_w) {
    const int p = __ffs(bits_w) - 1;
    bits_w &= bits_w - 1;
    const int k = k0 + open_byte(p);
    if (slot < kWarpOpen) scratch[slot] = 0x80000000u | ((uint32_t)(rw - g.b0 + 2) << 13) | (uint32_t)k;
    else resolve_site<R>(g, 1u, rw, k, P, tt);
    ++slot;
  }
  __syncwarp();
  for (int j = lane; j < min(total, kWarpOpen); j += 32) {
    const uint32_t d = scratch[j];
    resolve_site<R>(g, d >> 31, (int)((d >> 13) & 0x3FFFFu) + g.b0 - 2, (int)(d & 0x1FFFu), P, tt);
  }
  __syncwarp();
}

// SWAR update of one chunk at k0 of `row` from the other colour's rows.
// The parity q of the row is uniform across a warp (a warp never straddles
// rows), so the two directions are separate code paths.
template <int R, int QT>
__device__ __forceinline__ uint32_t chunk_step(uint32_t (&tw)[4], const uint8_t* row, const uint8_t* up,
                                               const uint8_t* dn, const uint8_t* mid, int k0, int q, const uint4& Rn,
                                               const Accept& a, uint32_t (&mw)[4]) {
  constexpr int H = Ring<R>::H;
  uint32_t uw[4], dw[4];
  load_words4(row + k0, tw);
  load_words4(up + k0, uw);
  load_words4(dn + k0, dw);
  load_words4(mid + k0, mw);
  if (QT) {  // two code paths, direction fixed at compile time (the branch is warp-uniform)
    if (q) return update_chunk_q<4, 1>(tw, uw, dw, mw, 0u, load_word(mid + ((k0 + 16) & (H - 1))), Rn, a);
    return update_chunk_q<4, 0>(tw, uw, dw, mw, load_word(mid + ((k0 - 4) & (H - 1))), 0u, Rn, a);
  }
  return update_chunk<4>(tw, uw, dw, mw, load_word(mid + ((k0 - 4) & (H - 1))), load_word(mid + ((k0 + 16) & (H - 1))),
                         (uint32_t)q, Rn, a);
}

template <int R>
__device__ __forceinline__ uint4 black_draw(int r, int c, const Params& P, uint32_t tt) {
  constexpr int L = Ring<R>::L;
  return stream_block(P.key, P.rep, P_SWEEP_HI, 0u, (uint32_t)((r + L) & (L - 1)), (uint32_t)c, tt);
}

// Per-thread resolution of the open sites of one chunk (the owner resolves).
template <int R>
__device__ __noinline__ void own_resolve(const Ring<R>& g, uint32_t colour, int r, int k0, uint32_t bits,
                                         const Params& P, uint32_t tt) {
  while (bits) {
    const int p = __ffs(bits) - 1;
    bits &= bits - 1;
    resolve_site<R>(g, colour, r, k0 + open_byte(p), P, tt);
  }
}

// PIPE: compute the next step's draws alongside this step's update.
// COOP: resolve open sites warp-cooperatively once per step (colour-1 sites
//       deferred by one step) instead of by their owners right away.
// QT:   side-neighbour direction as two compile-time code paths instead of
//       selects.
template <int R, int PIPE, int COOP, int QT>
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
  uint32_t* scratch = reinterpret_cast<uint32_t*>(g.Bs + SLOTS * H) + (tid >> 5) * kWarpOpen;
  g.b0 = (int)(((long long)blockIdx.x * L) / gridDim.x);
  const int b0 = g.b0;
  const int b1 = (int)(((long long)(blockIdx.x + 1) * L) / gridDim.x);
  const int nsteps = (b1 - b0 + R - 1) / R;
  // with one row per step every thread of the block works on the same row
  const int rr = (R == 1) ? 0 : tid / CPR;
  const int c = (R == 1) ? tid : tid % CPR, k0 = c * 16;

  if (tid < kStages) mbar_init(&bar[tid], 1);
  if (tid == 0) fence_mbar_init();
  __syncthreads();
  if (tid < 32)
    for (int k = -1; k < kAhead - 1 && k < nsteps; ++k) issue_stage<R>(g, k, b1, in, bar, tid);

  // ---- prologue: colour 0 on rows b0-1 and b0
  bool ok = wait_stage(bar, -1);
  for (int x = tid; x < 2 * CPR; x += kThreads) {
    const int r = b0 - 1 + x / CPR, cc = x % CPR;
    uint32_t tw[4], mw[4];
    uint8_t* row = g.b(r);
    const int q = ((r + L) & (L - 1)) & 1;
    const uint32_t bits = chunk_step<R, QT>(tw, row, g.w(r - 1), g.w(r + 1), g.w(r), cc * 16, q,
                                        black_draw<R>(r, cc, P, tt), P.acc, mw);
    if (ok) store_words<4>(row + cc * 16, tw);
    if (COOP) warp_resolve<R>(g, scratch, ok ? bits : 0u, r, 0u, r, cc * 16, P, tt);
    else if (ok && bits) own_resolve<R>(g, 0u, r, cc * 16, bits, P, tt);
  }

  uint4 Rb = black_draw<R>(b0 + 1 + rr, c, P, tt);
  uint4 Rw = stream_block(P.key, P.rep, P_SWEEP_HI, 1u, (uint32_t)(b0 + rr), (uint32_t)c, tt);
  uint32_t pend = 0;  // open colour-1 sites of the previous step (row r - R), COOP only
  for (int s = 0; s < nsteps; ++s) {
    if (!wait_stage(bar, s)) ok = false;
    const int rb = b0 + s * R + 1 + rr;  // colour-0 row of this step
    const int r = rb - 1;                // colour-1 row of this step
    uint4 Rb_next, Rw_next;
    if (PIPE) {
      Rb_next = black_draw<R>(rb + R, c, P, tt);
      Rw_next = stream_block(P.key, P.rep, P_SWEEP_HI, 1u, (uint32_t)((r + R) & (L - 1)), (uint32_t)c, tt);
    } else {
      Rb = black_draw<R>(rb, c, P, tt);
    }
    // ---- colour 0 (rows past b1 in the last step run on stale slots and are not stored)
    uint32_t bits_b;
    {
      uint8_t* row = g.b(rb);
      const int q = ((rb + L) & (L - 1)) & 1;
      uint32_t tw[4], mw[4];
      bits_b = chunk_step<R, QT>(tw, row, g.w(rb - 1), g.w(rb + 1), g.w(rb), k0, q, Rb, P.acc, mw);
      if (ok && rb <= b1) store_words<4>(row + k0, tw);
      if (!(ok && rb <= b1)) bits_b = 0;
    }
    if (COOP) {
      warp_resolve<R>(g, scratch, bits_b, rb, pend, r - R, k0, P, tt);
      if (pend)
        *reinterpret_cast<uint4*>(out + PLANE + (size_t)(r - R) * H + k0) =
            *reinterpret_cast<const uint4*>(g.w(r - R) + k0);
    } else if (bits_b) {
      own_resolve<R>(g, 0u, rb, k0, bits_b, P, tt);
    }
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(status, 1);
      return;
    }
    if (tid < 32 && s + kAhead - 1 < nsteps) issue_stage<R>(g, s + kAhead - 1, b1, in, bar, tid);
    // ---- colour 1, rows b0+sR .. b0+(s+1)R-1 (<= b1-1); both colours of the row are stored
    if (!PIPE) Rw = stream_block(P.key, P.rep, P_SWEEP_HI, 1u, (uint32_t)(r & (L - 1)), (uint32_t)c, tt);
    {
      uint8_t* row = g.w(r);
      const int q = (r + 1) & 1;
      uint32_t tw[4], mw[4];
      uint32_t bits = chunk_step<R, QT>(tw, row, g.b(r - 1), g.b(r + 1), g.b(r), k0, q, Rw, P.acc, mw);
      if (r <= b1 - 1) {
        *reinterpret_cast<uint4*>(out + (size_t)r * H + k0) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
        if (bits) {
          store_words<4>(row + k0, tw);
          if (!COOP) {
            own_resolve<R>(g, 1u, r, k0, bits, P, tt);
            load_words4(row + k0, tw);
          }
        }
        if (!COOP || !bits)
          *reinterpret_cast<uint4*>(out + PLANE + (size_t)r * H + k0) = make_uint4(tw[0], tw[1], tw[2], tw[3]);
      } else {
        bits = 0;
      }
      pend = COOP ? bits : 0u;
    }
    if (PIPE) {
      Rb = Rb_next;
      Rw = Rw_next;
    }
  }
  if (COOP) {
    // ---- the last step's open colour-1 sites
    const int rlast = b0 + (nsteps - 1) * R + rr;
    warp_resolve<R>(g, scratch, 0u, rlast, pend, rlast, k0, P, tt);
    if (pend)
      *reinterpret_cast<uint4*>(out + PLANE + (size_t)rlast * H + k0) =
          *reinterpret_cast<const uint4*>(g.w(rlast) + k0);
  }
}

}  // namespace stream
}  // namespace mcrg
