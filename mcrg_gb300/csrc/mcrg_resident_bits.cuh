// mcrg_resident_bits.cuh -- bit-sliced sweeps of a shared-memory-resident
// lattice (64 <= L <= 256), the same update and draws as the HBM sweep.
//
// The chain keeps a plane-word copy of level 0 (mcrg_planes.cuh) next to the
// byte lattice: sweeps run on the planes, and the bytes are refreshed from
// them before every measurement (blocking and coupling sums read bytes).  A
// colour pass updates every plane word of the colour from the other colour's
// words; words with open sites (8-bit draw equal to the threshold's top byte,
// ~0.1 per word at Kc) are appended to a shared-memory queue and, after a
// barrier, decided by the whole CTA from their P_SWEEP_LO draws, so that no
// warp stalls on its own open sites.  Same-colour sites do not interact, so
// deciding them after the pass equals deciding them in place.
#pragma once
#include "mcrg_ops.cuh"
#include "mcrg_planes.cuh"

namespace mcrg {
namespace resident {

// Queue entries of one colour pass: a quarter of the words (overflow is
// decided by the word's owner).
__host__ __device__ inline int queue_cap(int L) { return L * L / 256 > 32 ? L * L / 256 : 32; }

// byte lattice (split layout) -> plane words, colour c at pl + c * L * L / 64
__device__ __forceinline__ void pack_lattice(const uint8_t* lat, uint32_t* pl, int L, int tid, int T) {
  const int words = L * L / 64;  // per colour; word r covers bytes 32r .. 32r + 31 of the colour array
  for (int x = tid; x < 2 * words; x += T) {
    const uint4* src = reinterpret_cast<const uint4*>(lat + (size_t)x * 32);
    pl[x] = planes::pack_bytes(src[0], src[1]);
  }
}

__device__ __forceinline__ void unpack_lattice(const uint32_t* pl, uint8_t* lat, int L, int tid, int T) {
  const int words = L * L / 64;
  for (int x = tid; x < 2 * words; x += T) {
    uint4 a, b;
    planes::unpack_bytes(pl[x], a, b);
    uint4* dst = reinterpret_cast<uint4*>(lat + (size_t)x * 32);
    dst[0] = a;
    dst[1] = b;
  }
}

// Open sites of plane word w (row i) of colour c that flip at sweep t.
__device__ __forceinline__ uint32_t open_flips(Key key, uint32_t rep, const Accept& a, int c, int i, int w,
                                               uint32_t open, uint32_t zero, uint32_t t) {
  uint32_t flips = 0;
  while (open) {
    const int pos = __ffs(open) - 1;
    open &= open - 1;
    const int k = 32 * w + planes::plane_site(pos);
    const uint4 lo = stream_block(key, rep, P_SWEEP_LO, (uint32_t)c, (uint32_t)i, (uint32_t)(k >> 2), t);
    const uint32_t th = ((zero >> pos) & 1u) ? a.thr[0] : a.thr[1];
    if ((u4get(lo, k & 3) & 0xFFFFFFu) < (th & 0xFFFFFFu)) flips |= 1u << pos;
  }
  return flips;
}

// One colour pass (fast acceptance regime).  qn[c] must be 0 on entry; the
// caller clears it again once the other colour's pass has started.
__device__ __forceinline__ void sweep_colour(uint32_t* pl, int L, int c, uint32_t t, Key key, uint32_t rep,
                                             const Accept& a, int tid, int T, uint4* q, int* qn) {
  const int wpr = L / 64, words = L * wpr, cap = queue_cap(L);
  int lw = 0;
  while ((1 << lw) < wpr) ++lw;
  uint32_t* Cc = pl + (size_t)c * words;
  const uint32_t* Oc = pl + (size_t)(1 - c) * words;
  uint32_t tz[8], to[8];
  {
    const uint32_t T0 = a.thr[0] >> 24, T1 = a.thr[1] >> 24;
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      tz[p] = 0u - ((T0 >> (7 - p)) & 1u);
      to[p] = 0u - ((T1 >> (7 - p)) & 1u);
    }
  }
  for (int r = tid; r < words; r += T) {
    const int i = r >> lw, w = r & (wpr - 1);
    const uint32_t* orow = Oc + (size_t)i * wpr;
    const uint32_t tv = Cc[r];
    const uint32_t u = Oc[(size_t)((i - 1) & (L - 1)) * wpr + w];
    const uint32_t d = Oc[(size_t)((i + 1) & (L - 1)) * wpr + w];
    const uint32_t mid = orow[w];
    const uint32_t side = ((i + c) & 1) ? planes::right_sites(mid, orow[(w + 1) & (wpr - 1)])
                                        : planes::left_sites(mid, orow[(w - 1) & (wpr - 1)]);
    const uint4 A = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(2 * w), t);
    const uint4 B = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(2 * w + 1), t);
    uint32_t open, zero;
    uint32_t nt = planes::decide(tv, u, d, mid, side, A, B, tz, to, open, zero);
    if (open) {
      const int slot = atomicAdd(&qn[c], 1);
      if (slot < cap)
        q[slot] = make_uint4(open, zero & open, (uint32_t)i, (uint32_t)w);
      else
        nt ^= open_flips(key, rep, a, c, i, w, open, zero, t);
    }
    Cc[r] = nt;
  }
  __syncthreads();
  const int nq = min(qn[c], cap);
  for (int e = tid; e < nq; e += T) {
    const uint4 en = q[e];
    const uint32_t fl = open_flips(key, rep, a, c, (int)en.z, (int)en.w, en.x, en.y, t);
    if (fl) Cc[(size_t)en.z * wpr + en.w] ^= fl;  // one entry per word: no two threads touch the same word
  }
  __syncthreads();
}

// One sweep: colour 0, then colour 1 (qn[0..1] zero on entry and on return).
__device__ __forceinline__ void sweep(uint32_t* pl, int L, uint32_t t, Key key, uint32_t rep, const Accept& a,
                                      int tid, int T, uint4* q, int* qn) {
  sweep_colour(pl, L, 0, t, key, rep, a, tid, T, q, qn);
  if (tid == 0) qn[0] = 0;  // colour 0's queue was read before the last barrier; its next use is after more barriers
  sweep_colour(pl, L, 1, t, key, rep, a, tid, T, q, qn);
  if (tid == 0) qn[1] = 0;
}

}  // namespace resident
}  // namespace mcrg
