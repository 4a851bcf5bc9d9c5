// mcrg_resident_bits.cuh -- bit-sliced chains of a shared-memory-resident
// lattice (64 <= L <= 1024, fast acceptance regime): sweeps, coupling sums
// and b=2 majority blocking on plane words (mcrg_planes.cuh), the same update,
// draws and measurement as the byte and HBM paths.
//
// Every level of side m >= 64 lives only as plane words (m^2 / 8 bytes), so
// an L = 1024 chain with all its levels fits one CTA's shared memory.  A
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

// Queue entries of one colour pass: a quarter of the words, 32 .. 2048
// (overflow is decided by the word's owner).
__host__ __device__ inline int queue_cap(int L) {
  const int q = L * L / 256;
  return q < 32 ? 32 : (q > 2048 ? 2048 : q);
}

__device__ __forceinline__ int log2_words(int wpr) {
  int lw = 0;
  while ((1 << lw) < wpr) ++lw;
  return lw;
}

// Initial coin (P_INIT) straight into plane words: site k of (colour c, row i)
// is bit k & 31 of word (k & 127) >> 5 of block (row i, group k >> 7, sub c).
__device__ __forceinline__ void init_planes(uint32_t* pl, int L, Key key, uint32_t rep, int tid, int T) {
  const int wpr = L / 64, lw = log2_words(wpr), words = L * wpr;
  for (int x = tid; x < 2 * words; x += T) {
    const int c = x >= words, r = x - c * words, i = r >> lw, w = r & (wpr - 1);
    const uint4 b = stream_block(key, rep, P_INIT, (uint32_t)c, (uint32_t)i, (uint32_t)(w >> 2), 0u);
    pl[x] = planes::nat_to_plane(u4get(b, w & 3));
  }
}

// Coupling sums of a plane level of side m >= 64 (the directional forms of
// couplings_vec: down / right bonds of every site, each counted from one end
// and scaled by two).  NC: couplings wanted (1..5).
template <int NC>
__device__ __forceinline__ void couplings_planes(const uint32_t* P, int m, int tid, int T, int (&acc)[5]) {
  using planes::right_sites;
  using planes::left_sites;
  const int wpr = m / 64, lw = log2_words(wpr), words = m * wpr;
  int a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, nw = 0;
  for (int x = tid; x < 2 * words; x += T) {
    const int c = x >= words, r = x - c * words, i = r >> lw, w = r & (wpr - 1);
    const bool q = ((i + c) & 1) != 0;
    const uint32_t* Cc = P + (size_t)c * words;
    const uint32_t* Oc = P + (size_t)(1 - c) * words;
    const int wn = (w + 1) & (wpr - 1), wp = (w - 1) & (wpr - 1);
    const int r0 = i * wpr, r1 = ((i + 1) & (m - 1)) * wpr;
    const uint32_t xv = Cc[r0 + w];
    const uint32_t od = Oc[r1 + w];                                   // O[i+1][k]
    const uint32_t oi = Oc[r0 + w], oin = Oc[r0 + wn];
    const uint32_t oi1 = right_sites(oi, oin);                        // O[i][k+1]
    const uint32_t oiq = q ? oi1 : oi;                                 // O[i][k+q]
    a0 += __popc(xv ^ od) + __popc(xv ^ oiq);
    uint32_t cdq = 0, ci1 = 0, cd2 = 0;
    if (NC > 1) {
      const uint32_t cd = Cc[r1 + w];
      cdq = q ? right_sites(cd, Cc[r1 + wn]) : cd;                    // C[i+1][k+q]
      const uint32_t cdqm = q ? cd : left_sites(cd, Cc[r1 + wp]);     // C[i+1][k+q-1]
      a1 += __popc(xv ^ cdq) + __popc(xv ^ cdqm);
    }
    if (NC > 2) {
      cd2 = Cc[((i + 2) & (m - 1)) * wpr + w];                        // C[i+2][k]
      ci1 = right_sites(xv, Cc[r0 + wn]);                             // C[i][k+1]
      a2 += __popc(xv ^ cd2) + __popc(xv ^ ci1);
    }
    if (NC > 3) a3 += __popc(xv ^ od ^ oiq ^ cdq);
    if (NC > 4) {
      const uint32_t oiq1 = q ? right_sites(oi1, oin >> 8) : oi1;     // O[i][k+q+1]
      const uint32_t od3 = Oc[((i + 3) & (m - 1)) * wpr + w];         // O[i+3][k]
      a4 += __popc(xv ^ oiq ^ ci1 ^ oiq1) + __popc(xv ^ od ^ cd2 ^ od3);
    }
    ++nw;
  }
  acc[0] += 128 * nw - 4 * a0;
  if (NC > 1) acc[1] += 128 * nw - 4 * a1;
  if (NC > 2) acc[2] += 128 * nw - 4 * a2;
  if (NC > 3) acc[3] += 32 * nw - 2 * a3;
  if (NC > 4) acc[4] += 64 * nw - 2 * a4;
}

// The first two coupling sums of a plane level (couplings_planes<2>), one
// item per row i covering both colours: the colour with q = 0 (its right and
// down-right neighbours share its word index) and the colour with q = 1 read
// the words of rows i and i + 1 once each, walking the row's words with the
// neighbours of word w carried over from word w - 1 (four loads per pair of
// words instead of six per word).  Row i starts its walk at word
// (i / (32 / wpr)) mod wpr, so that the lanes of a warp, one row each, read
// 32 different shared-memory banks at every step (rows 32 / wpr apart share
// a bank set).
__device__ __forceinline__ void couplings_planes_c2(const uint32_t* P, int m, int tid, int T, int (&acc)[5]) {
  using planes::right_sites;
  using planes::left_sites;
  const int wpr = m / 64, words = m * wpr, lw = log2_words(wpr);
  const int lr = lw >= 5 ? 0 : 5 - lw;  // log2 of the rows that share a bank set
  int a0 = 0, a1 = 0, nw = 0;
  for (int i = tid; i < m; i += T) {
    const int i1 = (i + 1) & (m - 1);
    const uint32_t* Ce = P + (size_t)(i & 1) * words + (size_t)i * wpr;         // row i, colour i & 1: q = 0
    const uint32_t* Co = P + (size_t)((i + 1) & 1) * words + (size_t)i * wpr;   // row i, the other colour: q = 1
    const uint32_t* De = P + (size_t)(i & 1) * words + (size_t)i1 * wpr;        // row i + 1, colour i & 1
    const uint32_t* Dd = P + (size_t)((i + 1) & 1) * words + (size_t)i1 * wpr;  // row i + 1, the other colour
    const int w0 = (i >> lr) & (wpr - 1);
    const uint32_t ce0 = Ce[w0], dd0 = Dd[w0];
    uint32_t ce = ce0, de = De[w0], dd = dd0, dep = De[(w0 - 1) & (wpr - 1)];
    for (int k = 0; k < wpr; ++k) {
      const int w = (w0 + k) & (wpr - 1), wn = (w + 1) & (wpr - 1);
      const bool more = k + 1 < wpr;
      const uint32_t co = Co[w];
      const uint32_t cen = more ? Ce[wn] : ce0, ddn = more ? Dd[wn] : dd0;
      // q = 0: down O[i+1][k] = dd, right O[i][k] = co;  q = 1: down de, right O[i][k+1]
      a0 += __popc(ce ^ dd) + __popc(ce ^ co) + __popc(co ^ de) + __popc(co ^ right_sites(ce, cen));
      // q = 0: C[i+1][k] = de and C[i+1][k-1];  q = 1: C[i+1][k+1] and C[i+1][k] = dd
      a1 += __popc(ce ^ de) + __popc(ce ^ left_sites(de, dep)) + __popc(co ^ right_sites(dd, ddn)) +
            __popc(co ^ dd);
      dep = de;
      de = more ? De[wn] : de;
      ce = cen;
      dd = ddn;
    }
    nw += wpr;
  }
  acc[0] += 256 * nw - 4 * a0;
  acc[1] += 256 * nw - 4 * a1;
}

// b = 2 majority blocking of a plane level of side m >= 128 into the plane
// level of side m/2 (the blocking of side 64 into 32 lands in one warp's
// registers: small::block_planes_row).  Block (ib, jb)
// counts split column jb of rows 2ib, 2ib+1 in both colours (bit pos(jb & 31)
// of word jb >> 5); a tie takes bit jb & 31 of word (jb & 127) >> 5 of the
// P_TIE block (level_out, ib, jb >> 7, sample), as block_vec does.  Output
// (ib, jb) has colour (ib + jb) & 1 and split index jb >> 1: the bits of one
// parity of two neighbouring input words form one output word, which is the
// index rotation `unshuffle` once the parity is moved to index bit 3.
__device__ __forceinline__ void block_planes(const uint32_t* P, int m, uint8_t* out, Key key, uint32_t rep,
                                             int level_out, uint32_t sample, int tid, int T) {
  const int wpr = m / 64, words = m * wpr, h = m / 2;
  const uint32_t* P0 = P;
  const uint32_t* P1 = P + words;
  {
    uint32_t* Q = reinterpret_cast<uint32_t*>(out);
    const int wpr1 = wpr / 2, lw1 = log2_words(wpr1), words1 = h * wpr1;
    // input word w of rows 2 ib, 2 ib + 1 (both colours) -> its blocks in plane order; t: the
    // tie word of w (natural order)
    auto block_word = [](uint32_t a0, uint32_t a1, uint32_t b0, uint32_t b1, uint32_t t) {
      uint32_t ge3, eq2;
      planes::majority4(a0, a1, b0, b1, ge3, eq2);
      return ge3 | (eq2 & planes::nat_to_plane(t));
    };
    // output word x of both colours from the blocks of input words 2 w1, 2 w1 + 1
    auto out_word = [](uint32_t r0, uint32_t r1, uint32_t& even, uint32_t& odd) {
      even = planes::unshuffle((r0 & 0x00FF00FFu) | ((r1 & 0x00FF00FFu) << 8));  // even jb
      odd = planes::unshuffle(((r0 >> 8) & 0x00FF00FFu) | (r1 & 0xFF00FF00u));  // odd jb
    };
    if (wpr1 >= 2) {
      // item y: output words 2y, 2y + 1 of row ib from input words 4a .. 4a + 3 (a = group of the
      // tie block), read as one 16-byte vector per row and colour; consecutive lanes take
      // consecutive groups, so a quarter warp's vectors fall on at most two bank sets
      for (int y = tid; y < words1 / 2; y += T) {
        const int x = 2 * y, ib = x >> lw1, w1 = x & (wpr1 - 1), w = 2 * w1;
        const uint4 tb = stream_block(key, rep, P_TIE, (uint32_t)level_out, (uint32_t)ib, (uint32_t)(w1 >> 1), sample);
        const size_t ra = (size_t)2 * ib * wpr + w, rb = ra + wpr;
        const uint4 a0 = *reinterpret_cast<const uint4*>(P0 + ra), a1 = *reinterpret_cast<const uint4*>(P1 + ra);
        const uint4 b0 = *reinterpret_cast<const uint4*>(P0 + rb), b1 = *reinterpret_cast<const uint4*>(P1 + rb);
        uint32_t e0, o0, e1, o1;
        out_word(block_word(a0.x, a1.x, b0.x, b1.x, tb.x), block_word(a0.y, a1.y, b0.y, b1.y, tb.y), e0, o0);
        out_word(block_word(a0.z, a1.z, b0.z, b1.z, tb.z), block_word(a0.w, a1.w, b0.w, b1.w, tb.w), e1, o1);
        *reinterpret_cast<uint2*>(Q + (size_t)(ib & 1) * words1 + x) = make_uint2(e0, e1);
        *reinterpret_cast<uint2*>(Q + (size_t)((ib + 1) & 1) * words1 + x) = make_uint2(o0, o1);
      }
    } else {  // m = 128: one output word per row (x = ib) from input words 0, 1 (8-byte vectors)
      for (int ib = tid; ib < h; ib += T) {
        const uint4 tb = stream_block(key, rep, P_TIE, (uint32_t)level_out, (uint32_t)ib, 0u, sample);
        const size_t ra = (size_t)4 * ib, rb = ra + 2;
        const uint2 a0 = *reinterpret_cast<const uint2*>(P0 + ra), a1 = *reinterpret_cast<const uint2*>(P1 + ra);
        const uint2 b0 = *reinterpret_cast<const uint2*>(P0 + rb), b1 = *reinterpret_cast<const uint2*>(P1 + rb);
        uint32_t e, o;
        out_word(block_word(a0.x, a1.x, b0.x, b1.x, tb.x), block_word(a0.y, a1.y, b0.y, b1.y, tb.y), e, o);
        Q[(size_t)(ib & 1) * words1 + ib] = e;
        Q[(size_t)((ib + 1) & 1) * words1 + ib] = o;
      }
    }
  }
}

// byte lattice (split layout, shared or global memory) -> plane words, colour c at pl + c * L * L / 64
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
  const int wpr = L / 64, words = L * wpr, cap = queue_cap(L), lw = log2_words(wpr);
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
  // two words per thread and step (r and r + T): two independent Philox and
  // decision chains in flight per thread
  auto neighbours = [&](int r, int& i, int& w, uint32_t& tv, uint32_t& u, uint32_t& d, uint32_t& mid,
                        uint32_t& side) {
    i = r >> lw;
    w = r & (wpr - 1);
    const uint32_t* orow = Oc + (size_t)i * wpr;
    tv = Cc[r];
    u = Oc[(size_t)((i - 1) & (L - 1)) * wpr + w];
    d = Oc[(size_t)((i + 1) & (L - 1)) * wpr + w];
    mid = orow[w];
    side = ((i + c) & 1) ? planes::right_sites(mid, orow[(w + 1) & (wpr - 1)])
                         : planes::left_sites(mid, orow[(w - 1) & (wpr - 1)]);
  };
  auto finish = [&](int r, int i, int w, uint32_t nt, uint32_t open, uint32_t zero) {
    if (open) {
      const int slot = atomicAdd(&qn[c], 1);
      if (slot < cap)
        q[slot] = make_uint4(open, zero & open, (uint32_t)i, (uint32_t)w);
      else
        nt ^= open_flips(key, rep, a, c, i, w, open, zero, t);
    }
    Cc[r] = nt;
  };
  int r = tid;
  for (; r + T < words; r += 2 * T) {
    const int r2 = r + T;
    int i1, w1, i2, w2;
    uint32_t tv1, u1, d1, m1, s1, tv2, u2, d2, m2, s2;
    neighbours(r, i1, w1, tv1, u1, d1, m1, s1);
    neighbours(r2, i2, w2, tv2, u2, d2, m2, s2);
    const uint4 A1 = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i1, (uint32_t)(2 * w1), t);
    const uint4 A2 = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i2, (uint32_t)(2 * w2), t);
    const uint4 B1 = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i1, (uint32_t)(2 * w1 + 1), t);
    const uint4 B2 = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i2, (uint32_t)(2 * w2 + 1), t);
    uint32_t o1, z1, o2, z2;
    const uint32_t n1 = planes::decide(tv1, u1, d1, m1, s1, A1, B1, tz, to, o1, z1);
    const uint32_t n2 = planes::decide(tv2, u2, d2, m2, s2, A2, B2, tz, to, o2, z2);
    finish(r, i1, w1, n1, o1, z1);
    finish(r2, i2, w2, n2, o2, z2);
  }
  if (r < words) {  // one word left for this thread (words per thread odd, e.g. one when T = words)
    int i1, w1;
    uint32_t tv1, u1, d1, m1, s1;
    neighbours(r, i1, w1, tv1, u1, d1, m1, s1);
    const uint4 A1 = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i1, (uint32_t)(2 * w1), t);
    const uint4 B1 = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i1, (uint32_t)(2 * w1 + 1), t);
    uint32_t o1, z1;
    const uint32_t n1 = planes::decide(tv1, u1, d1, m1, s1, A1, B1, tz, to, o1, z1);
    finish(r, i1, w1, n1, o1, z1);
  }
  chain_sync(T);
  const int nq = min(qn[c], cap);
  for (int e = tid; e < nq; e += T) {
    const uint4 en = q[e];
    const uint32_t fl = open_flips(key, rep, a, c, (int)en.z, (int)en.w, en.x, en.y, t);
    if (fl) Cc[(size_t)en.z * wpr + en.w] ^= fl;  // one entry per word: no two threads touch the same word
  }
  chain_sync(T);
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
