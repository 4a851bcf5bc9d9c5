// mcrg_planes.cuh -- bit-plane words of a colour row and the bit-sliced
// Metropolis decision, shared by the HBM sweep (mcrg_sweep_bits.cuh) and the
// shared-memory-resident chains (mcrg_chain.cu).
//
// 32 consecutive sites k = 32w .. 32w+31 of one colour row form plane word w;
// site k = 32w + p sits at bit pos(p) = 8*(p&3) + (p>>2).  That order makes
// packing 32 int8 sites (bytes 0/1) a sum of eight shifted 32-bit loads and
// unpacking eight shift-and-mask pairs.  The eight random planes of a word are
// the words of its two P_SWEEP_HI Philox blocks (groups 2w, 2w+1): bit pos(p)
// of plane q is bit 7-q of the site's 8-bit draw r8.
#pragma once
#include <cstdint>

namespace mcrg {
namespace planes {

// plane bit of site p (0..31) of a word, and its inverse
__device__ __forceinline__ int plane_pos(int p) { return 8 * (p & 3) + (p >> 2); }
__device__ __forceinline__ int plane_site(int pos) { return 4 * (pos & 7) + (pos >> 3); }

// 32 sites (bytes 0/1, a = bytes 0..15, b = bytes 16..31) -> plane word
__device__ __forceinline__ uint32_t pack_bytes(const uint4& a, const uint4& b) {
  return a.x + (a.y << 1) + (a.z << 2) + (a.w << 3) + (b.x << 4) + (b.y << 5) + (b.z << 6) + (b.w << 7);
}

__device__ __forceinline__ void unpack_bytes(uint32_t x, uint4& a, uint4& b) {
  const uint32_t M = 0x01010101u;
  a = make_uint4(x & M, (x >> 1) & M, (x >> 2) & M, (x >> 3) & M);
  b = make_uint4((x >> 4) & M, (x >> 5) & M, (x >> 6) & M, (x >> 7) & M);
}

// Word of the sites k+1 (right) / k-1 (left) of every site k of word x;
// xn / xp is the next / previous word of the row.
__device__ __forceinline__ uint32_t right_sites(uint32_t x, uint32_t xn) {
  return (x >> 8) | ((x << 23) & 0x7F000000u) | (xn << 31);
}
__device__ __forceinline__ uint32_t left_sites(uint32_t x, uint32_t xp) {
  return (x << 8) | ((x >> 23) & 0xFEu) | (xp >> 31);
}

// Rotates the 5-bit bit index right by one: the bits at even positions go to
// the low half in order, the odd ones to the high half (outer perfect
// unshuffle, four delta swaps).
__device__ __forceinline__ uint32_t unshuffle(uint32_t x) {
  uint32_t t;
  t = (x ^ (x >> 1)) & 0x22222222u; x ^= t ^ (t << 1);
  t = (x ^ (x >> 2)) & 0x0C0C0C0Cu; x ^= t ^ (t << 2);
  t = (x ^ (x >> 4)) & 0x00F000F0u; x ^= t ^ (t << 4);
  t = (x ^ (x >> 8)) & 0x0000FF00u; x ^= t ^ (t << 8);
  return x;
}

// Swap of index bits i < j of every bit position (delta d = 2^j - 2^i, m =
// the positions whose index has bit i set and bit j clear).
template <int D, uint32_t M>
__device__ __forceinline__ uint32_t index_swap(uint32_t x) {
  const uint32_t t = (x ^ (x >> D)) & M;
  return x ^ t ^ (t << D);
}

// Natural bit order (bit p = site p) -> plane order (bit pos(p)): pos(p)
// rotates the 5-bit index of p right by two, (a2 a1 a0 b1 b0) -> (b1 b0 a2
// a1 a0), four index-bit swaps: (1,4), (0,3), (0,2), (1,2).
__device__ __forceinline__ uint32_t nat_to_plane(uint32_t v) {
  v = index_swap<14, 0x0000CCCCu>(v);
  v = index_swap<7, 0x00AA00AAu>(v);
  v = index_swap<3, 0x0A0A0A0Au>(v);
  return index_swap<2, 0x0C0C0C0Cu>(v);
}

// Plane order -> natural order: the same swaps in reverse.
__device__ __forceinline__ uint32_t plane_to_nat(uint32_t v) {
  v = index_swap<2, 0x0C0C0C0Cu>(v);
  v = index_swap<3, 0x0A0A0A0Au>(v);
  v = index_swap<7, 0x00AA00AAu>(v);
  return index_swap<14, 0x0000CCCCu>(v);
}

// Bit-sliced count of four words: ge3 = at least three bits set, eq2 = exactly two.
__device__ __forceinline__ void majority4(uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t& ge3,
                                          uint32_t& eq2) {
  const uint32_t s1 = a ^ b, c1 = a & b, s2 = c ^ d, c2 = c & d;
  const uint32_t lo = s1 ^ s2, any2 = c1 | c2 | (s1 & s2), both = c1 & c2;
  ge3 = both | (any2 & lo);
  eq2 = any2 & ~both & ~lo;
}

// Bit-sliced update of 32 sites t from their neighbours u, d (other colour,
// rows above and below), mid (same byte index) and side (the other
// horizontal neighbour).  tz / to: the top bytes of thr[0] / thr[1] as
// all-ones / all-zero masks per plane (plane 0 = most significant bit).
// Returns the new word; `open` gets the sites whose draw ties the
// threshold's top byte, `zero` the sites with m = 0.
__device__ __forceinline__ uint32_t decide(uint32_t t, uint32_t u, uint32_t d, uint32_t mid, uint32_t side,
                                           const uint4& A, const uint4& B, const uint32_t (&tz)[8],
                                           const uint32_t (&to)[8], uint32_t& open, uint32_t& zero) {
  const uint32_t s1 = (u ^ t) | (d ^ t), p1 = (u ^ t) & (d ^ t);
  const uint32_t s2 = (mid ^ t) | (side ^ t), p2 = (mid ^ t) & (side ^ t);
  const uint32_t ge2 = p1 | p2 | (s1 & s2);  // m >= 2: always flips
  zero = ~(s1 | s2);
  const uint32_t W[8] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w};
  uint32_t br = 0u, eq = ~0u;  // borrow of r8 - T8 (r8 < T8), r8 == T8
#pragma unroll
  for (int q = 7; q >= 0; --q) {
    const uint32_t th = (zero & tz[q]) | (~zero & to[q]);
    br = (~W[q] & (th | br)) | (th & br);
    eq &= ~(W[q] ^ th);
  }
  open = eq & ~ge2;
  return t ^ (ge2 | br);
}

}  // namespace planes
}  // namespace mcrg
