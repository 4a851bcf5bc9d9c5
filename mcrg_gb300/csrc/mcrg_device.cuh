// mcrg_device.cuh -- device primitives shared by the MCRG kernels (sm_103a).
//
// Spin storage: one byte per site, 0 = spin -1, 1 = spin +1, in a split
// checkerboard layout.  For a lattice of side n, colour c in {0,1} holds the
// sites (i, j) with (i + j) & 1 == c; array c is n rows x n/2 bytes,
// row-major, and byte k of row i is site (i, 2k + ((i + c) & 1)).
// Neighbours of colour-c site (i, k) with q = (i + c) & 1, O the other colour:
//   up/down    O[i-1][k], O[i+1][k]
//   left/right O[i][k-1+q], O[i][k+q]
// so a 16-byte chunk of one row is updated from three aligned 16-byte chunks
// of the other colour plus one byte-shifted copy of the centre chunk.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mcrg {

// Philox4x32-10 stream layout (mirrored by the oracle):
//   key = (seed lo32, seed hi32)
//   ctr = (row, purpose << 28 | sub << 20 | group, time, replica)
enum : uint32_t { P_INIT = 1, P_SWEEP_HI = 2, P_SWEEP_LO = 3, P_TIE = 4, P_BOND = 5, P_CLUSTER = 6 };

struct Key {
  uint32_t k0, k1;
};

// Philox4x32-10 (Salmon et al., SC'11).  Round keys are bumped by the Weyl
// constants; mulhi/mullo pairs come from 32x32->64 products.
__device__ __forceinline__ uint4 philox10(uint4 c, Key key) {
  uint32_t k0 = key.k0, k1 = key.k1;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
    c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1,
                   (uint32_t)p0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ uint4 stream_block(Key key, uint32_t replica, uint32_t purpose, uint32_t sub,
                                              uint32_t row, uint32_t group, uint32_t time) {
  return philox10(make_uint4(row, (purpose << 28) | (sub << 20) | group, time, replica), key);
}

__device__ __forceinline__ uint32_t u4get(const uint4& v, int w) {
  return w == 0 ? v.x : (w == 1 ? v.y : (w == 2 ? v.z : v.w));
}

// Acceptance parameters of one lattice.  m = number of anti-aligned
// neighbours (0..4), flip iff always[m] or u32 < thr[m].  The fast path
// applies when always = {0,0,1,1,1} and thr[1] < 2^31 (K < -ln2/4): then only
// m = 0, 1 draw, and the top byte of each threshold is below 0x80.
struct Accept {
  uint32_t thr[5];
  uint32_t always_mask;  // bit m set when always[m]
  uint32_t fast;
  uint32_t cx0, cx1;     // (0x80 - T8[m]) replicated in 4 bytes, m = 0, 1
  uint32_t cy0, cy1;     // (0x7F - T8[m]) replicated
};

// ---------------------------------------------------------------------------
// SWAR update of 4 sites packed in one word (bytes 0/1).
//   t: the sites; u, d, l, r: their four neighbours; R: four random bytes.
// Returns the updated word; *tie receives bit 7 of each byte whose decision
// is still open (top byte of the draw equals the threshold's top byte).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t swar_update(uint32_t t, uint32_t u, uint32_t d, uint32_t l, uint32_t r,
                                                uint32_t R, const Accept& a, uint32_t* tie) {
  const uint32_t H = 0x80808080u;
  const uint32_t n = u + d + l + r;           // up-neighbour count per byte (0..4)
  const uint32_t m = (n ^ (t * 7u)) - t * 3u;  // anti-aligned count: t ? 4-n : n
  const uint32_t gm1 = m + 0x7F7F7F7Fu;        // bit 7: m >= 1
  const uint32_t gm2 = m + 0x7E7E7E7Eu;        // bit 7: m >= 2
  const uint32_t Rl = R & 0x7F7F7F7Fu;
  const uint32_t x0 = Rl + a.cx0, x1 = Rl + a.cx1;  // bit 7: low7(R) >= T
  const uint32_t y0 = Rl + a.cy0, y1 = Rl + a.cy1;  // bit 7: low7(R) >= T+1
  const uint32_t ge0 = x0 | R, ge1 = x1 | R;        // bit 7: r8 >= T
  const uint32_t f = (gm2 | (gm1 & ~ge1) | ~ge0) & H;
  const uint32_t eq0 = x0 & ~y0 & ~R, eq1 = x1 & ~y1 & ~R;  // bit 7: r8 == T
  *tie = ((gm1 & ~gm2 & eq1) | (~gm1 & eq0)) & H;
  return t ^ (f >> 7);
}

// m of byte b of an update word (for tie bookkeeping; slow path only).
__device__ __forceinline__ uint32_t swar_m(uint32_t t, uint32_t u, uint32_t d, uint32_t l, uint32_t r) {
  const uint32_t n = u + d + l + r;
  return (n ^ (t * 7u)) - t * 3u;
}

// Exact decision for one site given its draw u32 (general path).
__device__ __forceinline__ bool accept_site(const Accept& a, uint32_t m, uint32_t u32) {
  return ((a.always_mask >> m) & 1u) || u32 < a.thr[m];
}

// Byte shifts over a chunk.  w[0..NW-1] are the chunk's words, wp the word
// before it and wn the word after it (both wrapped within the row).
// shifted(d)[j] = bytes 4j+d .. 4j+d+3 of [wp | w | wn], d in {-1, 0, 1, 2}.
template <int NW>
__device__ __forceinline__ uint32_t shifted_word(const uint32_t (&w)[NW], uint32_t wp, uint32_t wn, int j,
                                                 int d) {
  const uint32_t cur = w[j];
  const uint32_t nxt = (j + 1 < NW) ? w[j + 1] : wn;
  const uint32_t prv = (j > 0) ? w[j - 1] : wp;
  if (d == 0) return cur;
  if (d > 0) return __funnelshift_r(cur, nxt, 8 * d);
  return __funnelshift_r(prv, cur, 24);
}

// Byte sum of a word whose bytes total at most 255.
__device__ __forceinline__ uint32_t bytesum(uint32_t w) { return (w * 0x01010101u) >> 24; }

// 4 bits -> 4 bytes (bit b to bit 0 of byte b).
__device__ __forceinline__ uint32_t spread4(uint32_t x) { return ((x & 0xFu) * 0x00204081u) & 0x01010101u; }

// Barrier of the T threads that run one resident chain.  A chain owns the
// whole CTA (T == blockDim.x: __syncthreads), one warp (T == 32: the lanes
// synchronise and order their shared-memory accesses with __syncwarp), or a
// warp-aligned group of T = 64..512 threads of a larger CTA (named barrier
// 1 + threadIdx.x / T; at most 15 such groups per CTA).
__device__ __forceinline__ void chain_sync(int T) {
  if (T == (int)blockDim.x) {
    __syncthreads();
  } else if (T == 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)threadIdx.x / T), "r"(T) : "memory");
  }
}

}  // namespace mcrg
