// mcrg_ops.cuh -- per-chunk device routines shared by the resident chain
// kernel (mcrg_chain.cu) and the HBM-tiled kernels (mcrg_tiled.cu): the
// initial coin, the SWAR checkerboard update of a chunk, deferred tie
// resolution, the coupling sums of one level and b=2 majority-rule blocking.
// Every routine takes plain pointers, so the same code runs on shared or
// global memory.
#pragma once
#include "mcrg_internal.cuh"

namespace mcrg {
namespace {

__device__ __forceinline__ void load_words4(const uint8_t* p, uint32_t (&w)[4]) {
  const uint4 v = *reinterpret_cast<const uint4*>(p);
  w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
}
__device__ __forceinline__ void load_words2(const uint8_t* p, uint32_t (&w)[2]) {
  const uint2 v = *reinterpret_cast<const uint2*>(p);
  w[0] = v.x; w[1] = v.y;
}
template <int NW>
__device__ __forceinline__ void load_words(const uint8_t* p, uint32_t (&w)[NW]) {
  if constexpr (NW == 4) load_words4(p, w); else load_words2(p, w);
}
template <int NW>
__device__ __forceinline__ void store_words(uint8_t* p, const uint32_t (&w)[NW]) {
  if constexpr (NW == 4) *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
  else *reinterpret_cast<uint2*>(p) = make_uint2(w[0], w[1]);
}
__device__ __forceinline__ uint32_t load_word(const uint8_t* p) { return *reinterpret_cast<const uint32_t*>(p); }

// ---------------------------------------------------------------------------
// Initial coin (P_INIT): spin bit of (colour c, row i, k) = bit (k&127) of
// the block (row i, group k>>7, sub c, time 0).
// ---------------------------------------------------------------------------
__device__ void init_level0(uint8_t* lat, int L, Key key, uint32_t rep, int tid, int T) {
  const int half = L / 2;
  if (half >= 16) {
    const int cpr = half / 16;
    for (int task = tid; task < 2 * L * cpr; task += T) {
      const int c = task / (L * cpr), rem = task % (L * cpr), i = rem / cpr, k0 = (rem % cpr) * 16;
      const uint4 b = stream_block(key, rep, P_INIT, (uint32_t)c, (uint32_t)i, (uint32_t)(k0 >> 7), 0u);
      const uint32_t bits = (u4get(b, (k0 & 127) >> 5) >> (k0 & 31)) & 0xFFFFu;
      *reinterpret_cast<uint4*>(lat + (size_t)c * L * half + (size_t)i * half + k0) =
          make_uint4(spread4(bits), spread4(bits >> 4), spread4(bits >> 8), spread4(bits >> 12));
    }
  } else {
    for (int s = tid; s < 2 * L * half; s += T) {
      const int c = s / (L * half), rem = s % (L * half), i = rem / half, k = rem % half;
      const uint4 b = stream_block(key, rep, P_INIT, (uint32_t)c, (uint32_t)i, (uint32_t)(k >> 7), 0u);
      lat[(size_t)c * L * half + (size_t)i * half + k] = (uint8_t)((u4get(b, (k & 127) >> 5) >> (k & 31)) & 1u);
    }
  }
}

// ---------------------------------------------------------------------------
// SWAR update of one chunk of NW words (4*NW sites) of colour c.  tw: the
// chunk (updated in place); uw / dw: the other colour's chunks in the rows
// above / below; mw: the other colour's chunk in the same row; prv / nxt: the
// aligned words just before / after mw in that row (only their top / low byte
// is used); q: the side neighbour is O[i][k+1] when q = 1, O[i][k-1] when
// q = 0; R: the chunk's P_SWEEP_HI block.  Returns the still-open sites as
// a mask with bit (8*b + 7 - j) for byte b of word j.
// ---------------------------------------------------------------------------
template <int NW>
__device__ __forceinline__ uint32_t update_chunk(uint32_t (&tw)[NW], const uint32_t (&uw)[NW],
                                                 const uint32_t (&dw)[NW], const uint32_t (&mw)[NW], uint32_t prv,
                                                 uint32_t nxt, uint32_t q, const uint4& R, const Accept& a) {
  uint32_t V[NW + 1];
  V[0] = q ? mw[0] : prv;
#pragma unroll
  for (int j = 1; j < NW; ++j) V[j] = q ? mw[j] : mw[j - 1];
  V[NW] = q ? nxt : mw[NW - 1];
  const uint32_t sh = 24u - 16u * q;
  uint32_t open = 0;
#pragma unroll
  for (int j = 0; j < NW; ++j) {
    uint32_t tie;
    const uint32_t side = __funnelshift_r(V[j], V[j + 1], sh);
    tw[j] = swar_update(tw[j], uw[j], dw[j], mw[j], side, u4get(R, j), a, &tie);
    open |= tie >> j;
  }
  return open;
}

// Chunk byte of bit p of an open-site mask.
__device__ __forceinline__ int open_byte(int p) { return 4 * (7 - (p & 7)) + (p >> 3); }

// Exact decision for an open site (top byte of its draw equal to the top
// byte of its threshold): flip iff the low 24 bits of the P_SWEEP_LO draw
// are below the threshold's.  t: the site; n0..n3: its neighbours.
__device__ __forceinline__ bool resolve_open(uint32_t t, uint32_t n0, uint32_t n1, uint32_t n2, uint32_t n3,
                                             Key key, uint32_t rep, uint32_t c, int i, int k, uint32_t tt,
                                             const Accept& a) {
  const uint32_t m = (n0 != t) + (n1 != t) + (n2 != t) + (n3 != t);
  if (m > 1) return false;  // only reachable for unused halo bytes of a staged tile
  const uint4 lo = stream_block(key, rep, P_SWEEP_LO, c, (uint32_t)i, (uint32_t)(k >> 2), tt);
  return (u4get(lo, k & 3) & 0xFFFFFFu) < (a.thr[m] & 0xFFFFFFu);
}

// Descriptors one warp resolves cooperatively per pass (scratch entries).
constexpr int kOpenPerWarp = 64;
// Resident sweeps resolve open sites warp-cooperatively (true) or per thread.
#ifndef MCRG_RESIDENT_WARP_RESOLVE
#define MCRG_RESIDENT_WARP_RESOLVE 0
#endif
constexpr bool kResolveInWarp = MCRG_RESIDENT_WARP_RESOLVE != 0;

// Resolves the open sites of the warp's chunks of one round.  om[r] is the
// open mask of this lane's chunk r (row i_r, first byte k_r).  The sites are
// spread over the warp's lanes (one Philox block each) instead of each owner
// resolving its own, which would serialise the warp.  All lanes must call it.
template <int NW>
__device__ __forceinline__ void warp_resolve_resident(uint8_t* lat, int n, int c, uint32_t t, Key key, uint32_t rep,
                                                      const Accept& a, const uint32_t (&om)[8], int base, int tid,
                                                      int T, int cpr, uint32_t* scratch) {
  constexpr int CB = 4 * NW;
  const int half = n / 2, lane = threadIdx.x & 31;
  uint8_t* Cc = lat + (size_t)c * n * half;
  const uint8_t* Oc = lat + (size_t)(1 - c) * n * half;
  int cnt = 0;
#pragma unroll
  for (int r = 0; r < 8; ++r) cnt += __popc(om[r]);
  if (__ballot_sync(0xFFFFFFFFu, cnt != 0) == 0) return;
  int off = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xFFFFFFFFu, off, d);
    if (lane >= d) off += y;
  }
  const int total = __shfl_sync(0xFFFFFFFFu, off, 31);
  int slot = off - cnt;
  auto resolve = [&](int i, int k) {
    const int q = (i + c) & 1;
    uint8_t* sp = Cc + (size_t)i * half + k;
    const uint8_t* orow = Oc + (size_t)i * half;
    if (resolve_open(*sp, Oc[(size_t)((i - 1) & (n - 1)) * half + k], Oc[(size_t)((i + 1) & (n - 1)) * half + k],
                     orow[(k - 1 + q) & (half - 1)], orow[(k + q) & (half - 1)], key, rep, (uint32_t)c, i, k, t, a))
      *sp ^= 1u;
  };
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    uint32_t bits = om[r];
    if (!bits) continue;
    const int task = base + tid + r * T;
    const int i = task >> (__ffs(cpr) - 1), k0 = (task & (cpr - 1)) * CB;
    while (bits) {
      const int p = __ffs(bits) - 1;
      bits &= bits - 1;
      const int k = k0 + open_byte(p);
      if (slot < kOpenPerWarp) scratch[slot] = ((uint32_t)i << 13) | (uint32_t)k;
      else resolve(i, k);
      ++slot;
    }
  }
  __syncwarp();
  for (int j = lane; j < min(total, kOpenPerWarp); j += 32) {
    const uint32_t d = scratch[j];
    resolve((int)(d >> 13), (int)(d & 0x1FFFu));
  }
  __syncwarp();
}

// Vector sweep of colour c of a resident n x n lattice (n >= 16).  Threads
// take chunks in rounds of up to 8 per thread; the open sites of a round are
// resolved by the warp together at the end of the round.
template <int NW>
__device__ void sweep_colour_vec(uint8_t* lat, int n, int c, uint32_t t, Key key, uint32_t rep,
                                 const Accept& a, int tid, int T, uint32_t* scratch) {
  constexpr int CB = 4 * NW;  // chunk bytes
  const int half = n / 2, cpr = half / CB, ntask = n * cpr, lc = __ffs(cpr) - 1;  // cpr: a power of two
  uint8_t* Cc = lat + (size_t)c * n * half;
  const uint8_t* Oc = lat + (size_t)(1 - c) * n * half;
  for (int base = 0; base < ntask; base += 8 * T) {
    uint32_t om[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int task = base + tid + r * T;
      om[r] = 0;
      if (task < ntask) {
        const int i = task >> lc, k0 = (task & (cpr - 1)) * CB;
        const uint32_t q = (uint32_t)((i + c) & 1);
        uint8_t* tp = Cc + (size_t)i * half + k0;
        const uint8_t* orow = Oc + (size_t)i * half;
        uint32_t tw[NW], uw[NW], dw[NW], mw[NW];
        load_words<NW>(tp, tw);
        load_words<NW>(Oc + (size_t)((i - 1) & (n - 1)) * half + k0, uw);
        load_words<NW>(Oc + (size_t)((i + 1) & (n - 1)) * half + k0, dw);
        load_words<NW>(orow + k0, mw);
        // the words before and after the chunk (wrapped in the row); a row of one chunk
        // (L = 16, 32) has them in mw already (word loads at a 16-byte stride would put
        // four lanes on each bank)
        const uint32_t prv = cpr == 1 ? mw[NW - 1] : load_word(orow + ((k0 - 4) & (half - 1)));
        const uint32_t nxt = cpr == 1 ? mw[0] : load_word(orow + ((k0 + CB) & (half - 1)));
        const uint4 R = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(k0 >> 4), t);
        om[r] = update_chunk<NW>(tw, uw, dw, mw, prv, nxt, q, R, a);
        store_words<NW>(tp, tw);
      }
    }
    if (kResolveInWarp) {
      warp_resolve_resident<NW>(lat, n, c, t, key, rep, a, om, base, tid, T, cpr, scratch);
    } else {
      // each thread resolves the open sites of its own chunks (inline: a call
      // would make every warp save and restore its registers)
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        uint32_t bits = om[r];
        if (!bits) continue;
        const int task = base + tid + r * T;
        const int i = task >> lc, k0 = (task & (cpr - 1)) * CB, q = (i + c) & 1;
        const uint8_t* orow = Oc + (size_t)i * half;
        while (bits) {
          const int p = __ffs(bits) - 1;
          bits &= bits - 1;
          const int k = k0 + open_byte(p);
          uint8_t* sp = Cc + (size_t)i * half + k;
          if (resolve_open(*sp, Oc[(size_t)((i - 1) & (n - 1)) * half + k],
                           Oc[(size_t)((i + 1) & (n - 1)) * half + k], orow[(k - 1 + q) & (half - 1)],
                           orow[(k + q) & (half - 1)], key, rep, (uint32_t)c, i, k, t, a))
            *sp ^= 1u;
        }
      }
    }
  }
}

// Scalar sweep of colour c (any n >= 4, any K): exact 32-bit draw per site;
// the 8-bit part r8 comes from bytes for n <= 32 and from bit planes for
// n >= 64 (the layouts of the byte-SWAR and bit-sliced sweeps).
__device__ void sweep_colour_scalar(uint8_t* lat, int n, int c, uint32_t t, Key key, uint32_t rep,
                                    const Accept& a, int tid, int T) {
  const int half = n / 2, lh = __ffs(half) - 1;  // half is a power of two
  uint8_t* Cc = lat + (size_t)c * n * half;
  const uint8_t* Oc = lat + (size_t)(1 - c) * n * half;
  for (int s = tid; s < n * half; s += T) {
    const int i = s >> lh, k = s & (half - 1), q = (i + c) & 1;
    const uint32_t tv = Cc[(size_t)i * half + k];
    const uint32_t m = (Oc[(size_t)((i - 1) & (n - 1)) * half + k] != tv) +
                       (Oc[(size_t)((i + 1) & (n - 1)) * half + k] != tv) +
                       (Oc[(size_t)i * half + ((k - 1 + q) & (half - 1))] != tv) +
                       (Oc[(size_t)i * half + ((k + q) & (half - 1))] != tv);
    bool flip;
    if ((a.always_mask >> m) & 1u) {
      flip = true;
    } else {
      uint32_t r8;
      if (n >= 64) {  // bit-plane draws (groups 2w, 2w+1; bit 7-q of r8 = plane bit of word q)
        const int w = k >> 5, p = k & 31, pos = 8 * (p & 3) + (p >> 2);
        const uint4 A = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(2 * w), t);
        const uint4 B = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(2 * w + 1), t);
        const uint32_t W[8] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w};
        r8 = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) r8 |= ((W[q] >> pos) & 1u) << (7 - q);
      } else {  // byte draws
        const uint4 hi = stream_block(key, rep, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(k >> 4), t);
        r8 = (u4get(hi, (k & 15) >> 2) >> (8 * (k & 3))) & 0xFFu;
      }
      // u32 = r8 << 24 | r24 < thr: the top byte decides unless it ties, and only
      // then is the P_SWEEP_LO draw needed
      const uint32_t th = a.thr[m];
      if (r8 != (th >> 24)) {
        flip = r8 < (th >> 24);
      } else {
        const uint4 lo = stream_block(key, rep, P_SWEEP_LO, (uint32_t)c, (uint32_t)i, (uint32_t)(k >> 2), t);
        flip = (u4get(lo, k & 3) & 0xFFFFFFu) < (th & 0xFFFFFFu);
      }
    }
    if (flip) Cc[(size_t)i * half + k] = (uint8_t)(tv ^ 1u);
  }
}

// ---------------------------------------------------------------------------
// Coupling sums of one level.  Per site, downward / rightward forms of the
// directional sums (each symmetric pair counted twice, as src/lattice.cpp
// counts every bond from both ends).  Accumulates final values in acc[5].
// ---------------------------------------------------------------------------
// NC: number of couplings wanted (1..5); the sums past NC stay 0.
// U: tasks per thread and step (2 on HBM levels: twice the loads in flight).
template <int NW, int NC = 5, int U = 1>
__device__ void couplings_vec(const uint8_t* lev, int n, int tid, int T, int (&acc)[5]) {
  constexpr int CB = 4 * NW;
  const int half = n / 2, cpr = half / CB, lc = __ffs(cpr) - 1, lnc = __ffs(n * cpr) - 1;  // powers of two
  const int ntask = 2 * n * cpr;
  auto body = [&](int task) {
    const int c = task >> lnc, rem = task & (n * cpr - 1), i = rem >> lc, k0 = (rem & (cpr - 1)) * CB;
    const uint32_t q = (uint32_t)((i + c) & 1);
    const uint8_t* C = lev + (size_t)c * n * half;
    const uint8_t* O = lev + (size_t)(1 - c) * n * half;
    const uint8_t* Ci = C + (size_t)i * half;
    const uint8_t* Cd = C + (size_t)((i + 1) & (n - 1)) * half;
    const uint8_t* Cd2 = C + (size_t)((i + 2) & (n - 1)) * half;
    const uint8_t* Oi = O + (size_t)i * half;
    const uint8_t* Od = O + (size_t)((i + 1) & (n - 1)) * half;
    const uint8_t* Od3 = O + (size_t)((i + 3) & (n - 1)) * half;
    uint32_t ci[NW], cd[NW], cd2[NW], oi[NW], od[NW], od3[NW];
    load_words<NW>(Ci + k0, ci);
    load_words<NW>(Oi + k0, oi);
    load_words<NW>(Od + k0, od);
    if (NC > 1) load_words<NW>(Cd + k0, cd);
    if (NC > 2) load_words<NW>(Cd2 + k0, cd2);
    if (NC > 4) load_words<NW>(Od3 + k0, od3);
    const int kn = (k0 + CB) & (half - 1), kp = (k0 - 4) & (half - 1);
    const uint32_t ci_n = NC > 2 ? load_word(Ci + kn) : 0u, oi_n = load_word(Oi + kn);
    const uint32_t cd_n = NC > 1 ? load_word(Cd + kn) : 0u, cd_p = NC > 1 ? load_word(Cd + kp) : 0u;
    uint32_t a = 0, b = 0, e = 0, p = 0, h = 0;
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      const uint32_t ci_nx = (j + 1 < NW) ? ci[j + 1] : ci_n;
      const uint32_t oi_nx = (j + 1 < NW) ? oi[j + 1] : oi_n;
      const uint32_t cd_nx = (j + 1 < NW) ? cd[j + 1] : cd_n;
      const uint32_t cd_pv = (j > 0) ? cd[j - 1] : cd_p;
      const uint32_t ci1 = __funnelshift_r(ci[j], ci_nx, 8);             // C[i][k+1]
      const uint32_t oiq = __funnelshift_r(oi[j], oi_nx, 8 * q);         // O[i][k+q]
      const uint32_t oiq1 = __funnelshift_rc(oi[j], oi_nx, 8 * q + 8);   // O[i][k+q+1]
      const uint32_t cdq = __funnelshift_r(cd[j], cd_nx, 8 * q);         // C[i+1][k+q]
      const uint32_t cdqm = __funnelshift_rc(cd_pv, cd[j], 24 + 8 * q);  // C[i+1][k+q-1]
      const uint32_t x = ci[j];
      a += (x ^ od[j]) + (x ^ oiq);
      if (NC > 1) b += (x ^ cdq) + (x ^ cdqm);
      if (NC > 2) e += (x ^ cd2[j]) + (x ^ ci1);
      if (NC > 3) p += x ^ od[j] ^ oiq ^ cdq;
      if (NC > 4) h += (x ^ oiq ^ ci1 ^ oiq1) + (x ^ od[j] ^ cd2[j] ^ od3[j]);
    }
    acc[0] += 4 * CB - 4 * (int)bytesum(a);
    if (NC > 1) acc[1] += 4 * CB - 4 * (int)bytesum(b);
    if (NC > 2) acc[2] += 4 * CB - 4 * (int)bytesum(e);
    if (NC > 3) acc[3] += CB - 2 * (int)bytesum(p);
    if (NC > 4) acc[4] += 2 * CB - 2 * (int)bytesum(h);
  };
  int task = tid;
  if (U > 1)
    for (; task + T < ntask; task += 2 * T) {  // no stores: the two tasks' loads may all be issued first
      body(task);
      body(task + T);
    }
  for (; task < ntask; task += T) body(task);
}

__device__ __forceinline__ int spin_at(const uint8_t* lev, int n, int i, int j) {
  i &= n - 1;
  j &= n - 1;
  const int half = n / 2;
  return 2 * (int)lev[(size_t)((i + j) & 1) * n * half + (size_t)i * half + (j >> 1)] - 1;
}

// Direct directional sums (any n >= 2), one site per thread-iteration.
__device__ void couplings_scalar(const uint8_t* lev, int n, int tid, int T, int (&acc)[5]) {
  for (int s = tid; s < n * n; s += T) {
    const int i = s / n, j = s % n;
    const int v = spin_at(lev, n, i, j);
    acc[0] += v * (spin_at(lev, n, i + 1, j) + spin_at(lev, n, i - 1, j) + spin_at(lev, n, i, j + 1) +
                   spin_at(lev, n, i, j - 1));
    acc[1] += v * (spin_at(lev, n, i + 1, j + 1) + spin_at(lev, n, i - 1, j + 1) +
                   spin_at(lev, n, i + 1, j - 1) + spin_at(lev, n, i - 1, j - 1));
    acc[2] += v * (spin_at(lev, n, i + 2, j) + spin_at(lev, n, i - 2, j) + spin_at(lev, n, i, j + 2) +
                   spin_at(lev, n, i, j - 2));
    acc[3] += v * spin_at(lev, n, i + 1, j) * spin_at(lev, n, i, j + 1) * spin_at(lev, n, i + 1, j + 1);
    acc[4] += v * spin_at(lev, n, i + 1, j) * spin_at(lev, n, i + 2, j) * spin_at(lev, n, i + 3, j) +
              v * spin_at(lev, n, i, j + 1) * spin_at(lev, n, i, j + 2) * spin_at(lev, n, i, j + 3);
  }
}

// ---------------------------------------------------------------------------
// b = 2 majority rule, level n -> n/2.  Block (ib, jb) sums colour arrays
// B[2ib][jb] + W[2ib][jb] + B[2ib+1][jb] + W[2ib+1][jb] (same split column
// jb in all four rows).  Output (ib, jb) has colour (ib+jb)&1, index jb>>1.
// tie_nat (optional): natural-layout (n/2)^2 bytes, 1 = +1, 0 = -1.
// ---------------------------------------------------------------------------
__device__ void block_vec(const uint8_t* in, int n, uint8_t* out, const uint8_t* tie_nat, Key key,
                          uint32_t rep, int level_out, uint32_t sample, int tid, int T) {
  const int half = n / 2, hn = n / 2, ohalf = hn / 2, cpr = hn / 16;
  const uint8_t* B = in;
  const uint8_t* W = in + (size_t)n * half;
  const int lc = __ffs(cpr) - 1;  // cpr: a power of two
  for (int task = tid; task < hn * cpr; task += T) {
    const int ib = task >> lc, jb0 = (task & (cpr - 1)) * 16;
    uint32_t b0[4], w0[4], b1[4], w1[4];
    load_words4(B + (size_t)(2 * ib) * half + jb0, b0);
    load_words4(W + (size_t)(2 * ib) * half + jb0, w0);
    load_words4(B + (size_t)(2 * ib + 1) * half + jb0, b1);
    load_words4(W + (size_t)(2 * ib + 1) * half + jb0, w1);
    uint32_t tb[4];
    if (tie_nat) {
      load_words4(tie_nat + (size_t)ib * hn + jb0, tb);
    } else {
      const uint4 r = stream_block(key, rep, P_TIE, (uint32_t)level_out, (uint32_t)ib, (uint32_t)(jb0 >> 7), sample);
      const uint32_t bits = (u4get(r, (jb0 & 127) >> 5) >> (jb0 & 31)) & 0xFFFFu;
      tb[0] = spread4(bits); tb[1] = spread4(bits >> 4); tb[2] = spread4(bits >> 8); tb[3] = spread4(bits >> 12);
    }
    uint32_t res[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t s = b0[j] + w0[j] + b1[j] + w1[j];  // up spins per block, 0..4
      const uint32_t g3 = s + 0x7D7D7D7Du, g2 = s + 0x7E7E7E7Eu;
      res[j] = ((g3 >> 7) & 0x01010101u) | (((g2 & ~g3) >> 7) & tb[j] & 0x01010101u);
    }
    const uint32_t e0 = __byte_perm(res[0], res[1], 0x6420), e1 = __byte_perm(res[2], res[3], 0x6420);
    const uint32_t o0 = __byte_perm(res[0], res[1], 0x7531), o1 = __byte_perm(res[2], res[3], 0x7531);
    const int ce = ib & 1;
    *reinterpret_cast<uint2*>(out + (size_t)ce * hn * ohalf + (size_t)ib * ohalf + (jb0 >> 1)) = make_uint2(e0, e1);
    *reinterpret_cast<uint2*>(out + (size_t)(1 - ce) * hn * ohalf + (size_t)ib * ohalf + (jb0 >> 1)) =
        make_uint2(o0, o1);
  }
}

__device__ void block_scalar(const uint8_t* in, int n, uint8_t* out, const uint8_t* tie_nat, Key key,
                             uint32_t rep, int level_out, uint32_t sample, int tid, int T) {
  const int hn = n / 2, ohalf = hn / 2 > 0 ? hn / 2 : 1;
  for (int s = tid; s < hn * hn; s += T) {
    const int ib = s / hn, jb = s % hn;
    const int tot = spin_at(in, n, 2 * ib, 2 * jb) + spin_at(in, n, 2 * ib, 2 * jb + 1) +
                    spin_at(in, n, 2 * ib + 1, 2 * jb) + spin_at(in, n, 2 * ib + 1, 2 * jb + 1);
    uint32_t v;
    if (tot > 0) v = 1;
    else if (tot < 0) v = 0;
    else if (tie_nat) v = tie_nat[(size_t)ib * hn + jb];
    else {
      const uint4 r = stream_block(key, rep, P_TIE, (uint32_t)level_out, (uint32_t)ib, (uint32_t)(jb >> 7), sample);
      v = (u4get(r, (jb & 127) >> 5) >> (jb & 31)) & 1u;
    }
    out[(size_t)((ib + jb) & 1) * hn * ohalf + (size_t)ib * ohalf + (jb >> 1)] = (uint8_t)v;
  }
}

// Warp sums of acc[0 .. NC-1] added into S[c], c < C (NC >= C).
template <int NC = 5>
__device__ __forceinline__ void reduce_into(int (&acc)[5], int* S, int C) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int v = __reduce_add_sync(0xFFFFFFFFu, acc[c]);
    if (lane == 0 && c < C) atomicAdd(&S[c], v);
  }
}


}  // namespace
}  // namespace mcrg
