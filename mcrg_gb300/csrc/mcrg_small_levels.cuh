// mcrg_small_levels.cuh -- the blocking levels of side m <= 32 of a resident
// chain, run by one warp from registers.
//
// Lane i (< m) holds row i of the level as one word: bit j = site (i, j),
// 1 = up.  The coupling sums take the right-hand neighbours of a row from
// rotations of its word and the rows below from warp shuffles; b = 2 majority
// blocking takes the two input rows of an output row by shuffle and counts the
// four sites of every block bit-sliced (planes::majority4).  A tied block
// (two up, two down) takes bit jb of word 0 of the P_TIE block (level_out,
// ib, 0, sample), as block_vec and block_scalar do for jb < 32; the tie words
// of every blocking below are drawn up front, one Philox block per lane
// (output side h at lanes 32 - 2h .. 31 - h).  The sums are exact integers,
// so the results equal couplings_vec / couplings_scalar and block_vec /
// block_scalar on the same level (src/lattice.cpp:102-120, src/mcrg.cpp:314-348).
//
// Replaces, per measurement, one CTA-group barrier per level, a pass through
// shared memory per level and a Philox block per tied site with about sixty
// warp instructions per level.
#pragma once
#include "mcrg_ops.cuh"
#include "mcrg_planes.cuh"

namespace mcrg {
namespace small {

constexpr unsigned kFull = 0xFFFFFFFFu;

// Row word of the sites (i, j + s) of every site (i, j) of a row of side m
// (torus): the window at s of two copies of the row.  One expression for
// every m: a form that branched on m == 32 into a funnel shift gave the
// unrotated row for the first level of the 512-thread chain kernel (and only
// there), which the cluster-chain parity tests caught.
__device__ __forceinline__ uint32_t row_rot(uint32_t x, int s, int m) {
  const uint64_t xx = ((uint64_t)x << m) | x;
  return (uint32_t)(xx >> (s & (m - 1))) & (0xFFFFFFFFu >> (32 - m));
}

// Inverse of planes::unshuffle: bit k (< 16) to bit 2k, bit 16 + k to bit 2k + 1.
__device__ __forceinline__ uint32_t shuffle_bits(uint32_t x) {
  uint32_t t;
  t = (x ^ (x >> 8)) & 0x0000FF00u; x ^= t ^ (t << 8);
  t = (x ^ (x >> 4)) & 0x00F000F0u; x ^= t ^ (t << 4);
  t = (x ^ (x >> 2)) & 0x0C0C0C0Cu; x ^= t ^ (t << 2);
  t = (x ^ (x >> 1)) & 0x22222222u; x ^= t ^ (t << 1);
  return x;
}

// Four bytes 0/1 -> four bits (byte b to bit b): the partial products of the
// multiply land on distinct bits, bits 24..27 holding the four bytes.
__device__ __forceinline__ uint32_t nibble4(uint32_t w) { return (w * 0x01020408u) >> 24; }

// n bytes 0/1 (n <= 16, p aligned to n) -> bit k = byte k.  Rows of 16 and 8
// bytes are read as one vector, so that the lanes of a warp (one row each)
// read consecutive 16 / 8-byte pieces without shared-memory bank conflicts.
__device__ __forceinline__ uint32_t bytes_to_bits(const uint8_t* p, int n) {
  if (n == 16) {
    const uint4 v = *reinterpret_cast<const uint4*>(p);
    return nibble4(v.x) | (nibble4(v.y) << 4) | (nibble4(v.z) << 8) | (nibble4(v.w) << 12);
  }
  if (n == 8) {
    const uint2 v = *reinterpret_cast<const uint2*>(p);
    return nibble4(v.x) | (nibble4(v.y) << 4);
  }
  if (n == 4) return nibble4(*reinterpret_cast<const uint32_t*>(p));
  uint32_t v = 0;
  for (int k = 0; k < n; ++k) v |= (uint32_t)p[k] << k;
  return v;
}

// Row i of a split-layout byte level of side m <= 32: natural column j = 2k
// is byte k of colour i & 1, j = 2k + 1 byte k of the other colour.
__device__ __forceinline__ uint32_t level_row(const uint8_t* lev, int m, int i) {
  const int half = m / 2;
  const uint8_t* ev = lev + (size_t)(i & 1) * m * half + (size_t)i * half;
  const uint8_t* od = lev + (size_t)((i + 1) & 1) * m * half + (size_t)i * half;
  return shuffle_bits(bytes_to_bits(ev, half) | (bytes_to_bits(od, half) << 16));
}

// Row ib (= lane, 0..31) of the blocking of a plane level of side 64 into side
// 32, the rule of resident::block_planes: bit pos(jb) of the majority word is
// block (ib, jb), brought back to natural order by planes::plane_to_nat.
__device__ __forceinline__ uint32_t block_planes_row(const uint32_t* P, Key key, uint32_t rep, int level_out,
                                                     uint32_t sample, int ib) {
  const uint4 tb = stream_block(key, rep, P_TIE, (uint32_t)level_out, (uint32_t)ib, 0u, sample);
  const uint2 c0 = *reinterpret_cast<const uint2*>(P + 2 * ib);       // rows 2ib, 2ib + 1 of colour 0
  const uint2 c1 = *reinterpret_cast<const uint2*>(P + 64 + 2 * ib);  // and of colour 1
  uint32_t ge3, eq2;
  planes::majority4(c0.x, c1.x, c0.y, c1.y, ge3, eq2);
  const uint32_t res = ge3 | (eq2 & planes::nat_to_plane(tb.x));
  return planes::plane_to_nat(res);
}

// Levels l .. nl of side m, m/2, ... (m <= 32) from `row` (lane i: row i of
// level l).  Writes S[level * MCRG_MAX_COUPLINGS + c], c < C, from lane 0.
// NC: couplings computed (2 when C <= 2, else 5).  Every lane of the warp
// calls it.
template <int NC>
__device__ __forceinline__ void levels(uint32_t row, int m, int l, int nl, int C, Key key, uint32_t rep,
                                       uint32_t sample, int* S) {
  const int lane = (int)(threadIdx.x & 31u);
  // tie words of the blockings below level l: output side h at lane 32 - 2h + ib
  uint32_t tie = 0;
  {
    const int h = lane < 16 ? 16 : lane < 24 ? 8 : lane < 28 ? 4 : lane < 30 ? 2 : lane < 31 ? 1 : 0;
    if (h > 0 && h < m) {
      const int lo = l + __clz(h) - __clz(m);
      if (lo <= nl)
        tie = stream_block(key, rep, P_TIE, (uint32_t)lo, (uint32_t)(lane - (32 - 2 * h)), 0u, sample).x;
    }
  }
  for (;;) {
    const bool own = lane < m;
    const uint32_t r1 = row_rot(row, 1, m);
    const uint32_t d1 = __shfl_sync(kFull, row, (lane + 1) & (m - 1));
    const uint32_t d1r = row_rot(d1, 1, m), d1l = row_rot(d1, m - 1, m);
    int v[5];
    v[0] = 4 * m - 4 * (__popc(row ^ r1) + __popc(row ^ d1));
    v[1] = 4 * m - 4 * (__popc(row ^ d1r) + __popc(row ^ d1l));
    if (NC > 2) {
      const uint32_t r2 = row_rot(row, 2, m), r3 = row_rot(row, 3, m);
      const uint32_t d2 = __shfl_sync(kFull, row, (lane + 2) & (m - 1));
      const uint32_t d3 = __shfl_sync(kFull, row, (lane + 3) & (m - 1));
      v[2] = 4 * m - 4 * (__popc(row ^ r2) + __popc(row ^ d2));
      v[3] = m - 2 * __popc(row ^ d1 ^ r1 ^ d1r);
      v[4] = 2 * m - 2 * (__popc(row ^ r1 ^ r2 ^ r3) + __popc(row ^ d1 ^ d2 ^ d3));
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const int s = __reduce_add_sync(kFull, own ? v[c] : 0);
      if (lane == 0 && c < C) S[l * MCRG_MAX_COUPLINGS + c] = s;
    }
    if (l == nl) break;
    // blocking into level l + 1 of side h: rows 2ib, 2ib + 1 -> row ib
    const int h = m >> 1;
    const uint32_t a = __shfl_sync(kFull, row, (2 * lane) & 31);
    const uint32_t b = __shfl_sync(kFull, row, (2 * lane + 1) & 31);
    uint32_t ge3, eq2;
    planes::majority4(a, a >> 1, b, b >> 1, ge3, eq2);  // block jb at bit 2jb
    const uint32_t u = planes::unshuffle((ge3 & 0x55555555u) | ((eq2 & 0x55555555u) << 1));
    const uint32_t t = __shfl_sync(kFull, tie, (32 - 2 * h + lane) & 31);
    row = ((u & 0xFFFFu) | ((u >> 16) & t)) & ((1u << h) - 1u);
    m = h;
    ++l;
  }
}

}  // namespace small
}  // namespace mcrg
