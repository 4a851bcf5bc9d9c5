// mcrg_sweep_bits.cuh -- bit-sliced fused two-colour sweep of an HBM-resident
// lattice (L = 512 .. 16384): one read and one write of every int8 site per
// sweep, the update itself on 32 sites per 32-bit word.
//
// Bit-plane words.  32 consecutive sites k = 32w .. 32w+31 of one colour row
// form plane word w; site k = 32w + p sits at bit pos(p) = 8*(p&3) + (p>>2).
// That order makes packing 32 int8 sites (bytes 0/1) a sum of eight shifted
// 32-bit loads and unpacking eight shift-and-mask pairs.  The update draws
// eight random planes per word from two Philox blocks (row, P_SWEEP_HI,
// colour, group 2w and 2w+1, sweep): bit pos(p) of plane q is bit 7-q of the
// site's 8-bit draw r8.  For the fast acceptance regime (m >= 2 always flips,
// m in {0,1} flips iff r8:r24 < thr[m]) the decision for all 32 sites is a
// bit-sliced borrow chain r8 - T8[m] plus an equality mask; a site whose r8
// equals T8[m] is "open" and is decided from the low 24 bits of its
// P_SWEEP_LO draw exactly as the byte form does.
//
// Schedule.  Each CTA owns a band of rows [b0, b1) and walks it in groups of
// R = NT / (L/64) rows (one plane word per thread per colour per group).  A
// group g covers rows b0-2+gR .. b0-2+(g+1)R-1.  Phase p (one barrier each):
//   - resolve the open sites queued by colour 0 of group p-3 (flip bits of
//     the packed colour-0 rows in shared memory) and by colour 1 of group p-6
//     (patch the bytes already written to HBM);
//   - one warp issues the bulk copies of group p+LEAD (both colours);
//   - pack group p from its landed byte rows into plane words;
//   - update colour 0 of group p-2 (reads old colour-1 planes), queue its
//     open sites;
//   - update colour 1 of group p-5 (reads new colour-0 planes of groups p-6 ..
//     p-4, all resolved), queue its open sites, and write both colours of its
//     rows to the output buffer.
// The lags make every read in a phase depend only on work that finished
// before the previous barrier, so one barrier per phase suffices and the
// rare open sites are resolved compactly by a few lanes instead of stalling
// every warp that holds one (a queue entry is one plane word with open sites:
// its open, m = 0 and old-value masks).  Colour 0 is updated on rows b0-1 .. b1 and
// colour 1 on b0 .. b1-1; halo rows are also updated by the neighbouring
// band with the same draws, so both compute the same values.  Input and
// output are the two buffers of a ping-pong pair.
#pragma once
#include "mcrg_ops.cuh"
#include "mcrg_planes.cuh"
#include "mcrg_tma.cuh"

#include <type_traits>

namespace mcrg {
namespace bits {

struct Params {
  uint32_t rep;
  uint32_t thr0, thr1;  // acceptance thresholds for m = 0 and m = 1
  uint32_t rk[20];      // Philox round keys: rk[2r] = k0 + r*W0, rk[2r+1] = k1 + r*W1
  uint32_t tz[8], to[8];  // threshold top bytes as all-ones / all-zero masks, plane q (q = 0 MSB)
};

// Kernel parameters live in the constant bank, so the round keys and the
// threshold masks enter the logic ops as constant operands instead of
// occupying registers or being recomputed per Philox call.
inline void fill_params(Params& P, Key key, uint32_t rep, uint32_t thr0, uint32_t thr1) {
  P.rep = rep;
  P.thr0 = thr0;
  P.thr1 = thr1;
  uint32_t k0 = key.k0, k1 = key.k1;
  for (int r = 0; r < 10; ++r) {
    P.rk[2 * r] = k0;
    P.rk[2 * r + 1] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  const uint32_t T0 = thr0 >> 24, T1 = thr1 >> 24;
  for (int q = 0; q < 8; ++q) {
    P.tz[q] = 0u - ((T0 >> (7 - q)) & 1u);
    P.to[q] = 0u - ((T1 >> (7 - q)) & 1u);
  }
}

// Philox4x32-10 with precomputed round keys (same stream as philox10()).
__device__ __forceinline__ uint4 draw(const Params& P, uint32_t purpose, uint32_t sub, uint32_t row, uint32_t group,
                                      uint32_t tt) {
  uint4 c = make_uint4(row, (purpose << 28) | (sub << 20) | group, tt, P.rep);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
    c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ P.rk[2 * r], (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ P.rk[2 * r + 1],
                   (uint32_t)p0);
  }
  return c;
}

// Row groups of byte rows in flight ahead of packing: LEAD; LEAD + 1 are held
// per colour.
constexpr int kPackSlots = 8;          // plane-word groups held per colour
// Open-site queue entries per buffer: one entry per plane word with open
// sites (about 0.1 per word at the critical coupling, 51 +- 7 of 512); a word
// that finds its buffer full is resolved by its owner.
template <int NT, int LEAD>
constexpr int queue_cap() {
  static_assert(LEAD >= 1, "at least one row group of bulk copies in flight ahead of packing");
  return NT / 4;
}

template <int NT, int LEAD>
constexpr size_t smem_bytes() {
  return 128 + 6 * (size_t)queue_cap<NT, LEAD>() * 16 + 2 * (size_t)(LEAD + 1) * NT * 32 +
         2 * (size_t)kPackSlots * NT * 4;
}

using planes::left_sites;
using planes::pack_bytes;
using planes::plane_pos;
using planes::plane_site;
using planes::right_sites;
using planes::unpack_bytes;

__device__ __forceinline__ uint32_t decide(uint32_t t, uint32_t u, uint32_t d, uint32_t mid, uint32_t side,
                                           const uint4& A, const uint4& B, const Params& P, uint32_t& open,
                                           uint32_t& zero) {
  return planes::decide(t, u, d, mid, side, A, B, P.tz, P.to, open, zero);
}

// Open sites of one plane word of colour c (row gr, word w) that flip:
// each is decided from the low 24 bits of its P_SWEEP_LO draw.
__device__ __forceinline__ uint32_t open_flips(const Params& P, uint32_t c, int gr, int w, uint32_t open,
                                               uint32_t zero, uint32_t tt) {
  uint32_t flips = 0;
  while (open) {
    const int pos = __ffs(open) - 1;
    open &= open - 1;
    const int k = 32 * w + plane_site(pos);
    const uint4 lo = draw(P, P_SWEEP_LO, c, (uint32_t)gr, (uint32_t)(k >> 2), tt);
    const uint32_t th = ((zero >> pos) & 1u) ? P.thr0 : P.thr1;
    if ((u4get(lo, k & 3) & 0xFFFFFFu) < (th & 0xFFFFFFu)) flips |= 1u << pos;
  }
  return flips;
}

// Queues plane word w (band offset off) of colour c, which has open sites;
// returns their flips when the buffer is full (resolved here), else 0.  (One
// shared atomic per lane measured faster than a warp-aggregated slot range.)
template <int NT, int LEAD>
__device__ __forceinline__ uint32_t enqueue(uint32_t open, uint32_t zero, uint32_t t, int off, int w, int gr,
                                            int c, int qi, int* qn, uint4* Q, const Params& P, uint32_t tt) {
  constexpr int CAP = queue_cap<NT, LEAD>();
  const int slot = atomicAdd(&qn[qi], 1);
  if (slot < CAP) {
    Q[qi * CAP + slot] = make_uint4(open, zero & open, t & open, ((uint32_t)off << 8) | (uint32_t)w);
    return 0u;
  }
  return open_flips(P, (uint32_t)c, gr, w, open, zero, tt);
}

// Geometry of one instantiation: lattice side L = 64 << LW, NT threads.
template <int NT, int LW, int LEAD>
struct Geo {
  static constexpr int L = 64 << LW;
  static constexpr int H = L / 2;              // bytes per colour row
  static constexpr int WPR = 1 << LW;          // plane words per colour row
  static constexpr int R = NT >> LW;           // rows per group
  static constexpr int RAW_ROWS = (LEAD + 1) * R;
  static constexpr int PK_ROWS = kPackSlots * R;
  static constexpr size_t PLANE = (size_t)L * H;
  static_assert(R >= 1, "one plane word per thread per group row");
};

// Lattice row of band row x: odd bands walk their rows bottom-up (ms = b0 +
// b1 - 1 mirrors them, ms < 0 keeps them), so that the halo rows two
// neighbouring bands share are read at about the same time (one DRAM read,
// one L2 hit) instead of at opposite ends of the sweep.  The update is
// symmetric in up / down, so only the row numbers change.
__device__ __forceinline__ int lattice_row(int x, int ms, int L) { return ((ms >= 0 ? ms - x : x) + L) & (L - 1); }

template <int NT, int LW, int LEAD>
__device__ __forceinline__ void issue_group(int g, int top, int b0, int b1, int ms, const uint8_t* in, uint8_t* raw,
                                            uint64_t* bar, int lane) {
  using G = Geo<NT, LW, LEAD>;
  const int x0 = top + g * G::R;
  // rows wanted: colour 0 on [b0-1, b1], colour 1 on [b0-2, b1+1]
  const int n0 = max(0, min(b1, x0 + G::R - 1) - max(b0 - 1, x0) + 1);
  const int n1 = max(0, min(b1 + 1, x0 + G::R - 1) - max(b0 - 2, x0) + 1);
  uint64_t* br = &bar[g % (LEAD + 1)];
  tma::fence_proxy_async();
  if (lane == 0) tma::mbar_expect_tx(br, (uint32_t)((n0 + n1) * G::H));
  __syncwarp();
  for (int e = lane; e < 2 * G::R; e += 32) {
    const int c = e >= G::R, x = x0 + (e - c * G::R);
    const bool want = c ? (x >= b0 - 2 && x <= b1 + 1) : (x >= b0 - 1 && x <= b1);
    if (want)
      tma::bulk_g2s(raw + ((size_t)c * G::RAW_ROWS + (x - top) % G::RAW_ROWS) * G::H,
                    in + c * G::PLANE + (size_t)lattice_row(x, ms, G::L) * G::H, (uint32_t)G::H, br);
  }
}

// Resolves the open sites queued for colour c by group g: entries first,
// first + stride, ... of the buffer; flips go to the packed colour-0 row in
// shared memory (c = 0) or to the bytes already written to HBM (c = 1).
template <int NT, int LW, int LEAD>
__device__ __forceinline__ void resolve_queue(int c, int g, int first, int stride, const int* qn, const uint4* Q,
                                              uint32_t* pk, uint8_t* out, int top, int ms, const Params& P,
                                              uint32_t tt) {
  using G = Geo<NT, LW, LEAD>;
  constexpr int CAP = queue_cap<NT, LEAD>();
  const int qi = c * 3 + g % 3;
  const int n = min(qn[qi], CAP);
  for (int e = first; e < n; e += stride) {
    const uint4 ent = Q[qi * CAP + e];
    const int off = (int)(ent.w >> 8), ww = (int)(ent.w & 0xFFu);
    const int gr = lattice_row(top + off, ms, G::L);
    const uint32_t fl = open_flips(P, (uint32_t)c, gr, ww, ent.x, ent.y, tt);
    if (fl == 0u) continue;
    if (c == 0) {
      atomicXor(&pk[(off & (G::PK_ROWS - 1)) * G::WPR + ww], fl);
    } else {
      uint32_t f = fl;
      while (f) {
        const int pos = __ffs(f) - 1;
        f &= f - 1;
        out[G::PLANE + (size_t)gr * G::H + 32 * ww + plane_site(pos)] = (uint8_t)(((ent.z >> pos) & 1u) ^ 1u);
      }
    }
  }
}

// NT compute threads, one plane word per colour per group each; warp 0 also
// issues the bulk copies.  (A dedicated helper warp for the copies and the
// open sites, and drawing the Philox blocks ahead of the copy wait, both
// measured slower on GB300.)
// WPT plane words per thread per colour and group: a group is NS = NT * WPT
// words; slot s = tid + j NT (j < WPT) of a thread is row s / WPR, word s % WPR
// of the group, so that a thread's words are independent chains (ILP) and the
// per-phase fixed work is shared by more sites.
template <int NT, int WPT, int MINB, int LEAD, int LW>
__global__ void __launch_bounds__(NT, MINB)
    sweep_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, const __grid_constant__ Params P,
                 uint32_t tt, int* __restrict__ status) {
  constexpr int NS = NT * WPT;
  using G = Geo<NS, LW, LEAD>;
  constexpr int L = G::L, H = G::H, WPR = G::WPR, R = G::R, RAW_ROWS = G::RAW_ROWS, PK_ROWS = G::PK_ROWS;
  constexpr size_t PLANE = G::PLANE;
  constexpr int kRawSlots = LEAD + 1, CAP = queue_cap<NS, LEAD>();
  extern __shared__ __align__(128) uint8_t smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  int* qn = reinterpret_cast<int*>(smem + 64);                    // [colour][3] queue lengths
  uint4* Q = reinterpret_cast<uint4*>(smem + 128);                // [colour][3][CAP] entries
  uint8_t* raw = smem + 128 + 6 * CAP * 16;                       // [colour][RAW_ROWS][H] bytes
  uint32_t* pk = reinterpret_cast<uint32_t*>(raw + 2 * (size_t)RAW_ROWS * H);  // [colour][PK_ROWS][WPR]
  uint32_t* pk1 = pk + PK_ROWS * WPR;

  const int tid = threadIdx.x, lane = tid & 31;
  int wj[WPT], rj[WPT];  // word and row (within the group) of each slot of this thread
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    wj[j] = (tid + j * NT) % WPR;
    rj[j] = (R == 1) ? 0 : (tid + j * NT) / WPR;  // uniform when groups are one row
  }
  const int b0 = (int)(((long long)blockIdx.x * L) / gridDim.x);
  const int b1 = (int)(((long long)(blockIdx.x + 1) * L) / gridDim.x);
  const int top = b0 - 2;
  const int J = (b1 - b0 + 4 + R - 1) / R;
  const int ms = (blockIdx.x & 1) ? b0 + b1 - 1 : -1;

  if (tid < kRawSlots) tma::mbar_init(&bar[tid], 1);
  if (tid < 6) qn[tid] = 0;
  if (tid == 0) tma::fence_mbar_init();
  __syncthreads();
  // Launched as a programmatic dependent of the previous sweep: its output is
  // this launch's input and its input this launch's output, so every thread
  // waits for it before the first copy or store.
  tma::griddep_wait();
  tma::griddep_launch_dependents();
  if (tid < 32)
    for (int g = 0; g < LEAD && g < J; ++g) issue_group<NS, LW, LEAD>(g, top, b0, b1, ms, in, raw, bar, lane);

  // ok turns false when a bulk copy does not land in time; the phase's work
  // then runs on stale shared memory (all indices stay in bounds) and the
  // kernel reports the error at the phase barrier.  Keeping ok out of the
  // work conditions leaves them uniform across each warp.
  bool ok = true;
  // One phase; STEADY: every action of the phase is valid for every row (no
  // band-edge checks).
  auto phase = [&](int p, auto steady_tag) {
    constexpr bool STEADY = decltype(steady_tag)::value;
    // queue lengths of buffers no phase touches now (read last phase, next appended after this one)
    if (tid == 0) {
      if (STEADY || p >= 4) qn[(p - 4) % 3] = 0;
      if (STEADY || p >= 7) qn[3 + (p - 7) % 3] = 0;
    }
    // ---- open sites queued last phase: colour 0 of group p-3, colour 1 of group p-6.  The first
    //      entries go to the last warps (warp 0 also issues the bulk copies): warp NW-1-k takes
    //      colour k & 1, entries 32 (k >> 1) + lane, ...
    {
      const int rw = NT / 32 - 1 - (tid >> 5), c = rw & 1, g = p - (c ? 6 : 3);
      if (STEADY || (g >= 0 && g < J))
        resolve_queue<NS, LW, LEAD>(c, g, (rw >> 1) * 32 + lane, NT / 2, qn, Q, pk, out, top, ms, P, tt);
    }
    // ---- bulk copies of group p + LEAD (its slot was packed last phase)
    if (tid < 32 && p + LEAD < J) issue_group<NS, LW, LEAD>(p + LEAD, top, b0, b1, ms, in, raw, bar, lane);
    // ---- pack group p (waits for its copy)
    if (STEADY || p < J) {
      if (!tma::mbar_wait_bounded(&bar[p % kRawSlots], (uint32_t)((p / kRawSlots) & 1))) ok = false;
#pragma unroll
      for (int j = 0; j < WPT; ++j) {
        const int w = wj[j], off = p * R + rj[j], x = top + off;
        const int ri = off % RAW_ROWS, pi = off & (PK_ROWS - 1);
        if (STEADY || (x >= b0 - 1 && x <= b1)) {
          const uint4* sp = reinterpret_cast<const uint4*>(raw + (size_t)ri * H + 32 * w);
          pk[pi * WPR + w] = pack_bytes(sp[0], sp[1]);
        }
        if (STEADY || x <= b1 + 1) {
          const uint4* sp = reinterpret_cast<const uint4*>(raw + ((size_t)RAW_ROWS + ri) * H + 32 * w);
          pk1[pi * WPR + w] = pack_bytes(sp[0], sp[1]);
        }
      }
    }
    // ---- colour 0 of group p-2
#pragma unroll
    for (int j = 0; j < WPT; ++j) {
      const int w = wj[j], off = (p - 2) * R + rj[j], x = top + off;
      if (STEADY || (p >= 2 && p - 2 < J && x >= b0 - 1 && x <= b1)) {
        const int gr = lattice_row(x, ms, L), pi = off & (PK_ROWS - 1);
        const uint32_t t = pk[pi * WPR + w];
        const uint32_t u = pk1[((pi - 1) & (PK_ROWS - 1)) * WPR + w];
        const uint32_t d = pk1[((pi + 1) & (PK_ROWS - 1)) * WPR + w];
        const uint32_t* mr = pk1 + pi * WPR;
        const uint32_t mid = mr[w];
        const uint32_t side =
            (gr & 1) ? right_sites(mid, mr[(w + 1) & (WPR - 1)]) : left_sites(mid, mr[(w - 1) & (WPR - 1)]);
        const uint4 A = draw(P, P_SWEEP_HI, 0u, (uint32_t)gr, (uint32_t)(2 * w), tt);
        const uint4 B = draw(P, P_SWEEP_HI, 0u, (uint32_t)gr, (uint32_t)(2 * w + 1), tt);
        uint32_t open, zero;
        uint32_t nt = decide(t, u, d, mid, side, A, B, P, open, zero);
        if (open) nt ^= enqueue<NS, LEAD>(open, zero, t, off, w, gr, 0, (p - 2) % 3, qn, Q, P, tt);
        pk[pi * WPR + w] = nt;
      }
    }
    // ---- colour 1 of group p-5, then both colours of its rows to the output
#pragma unroll
    for (int j = 0; j < WPT; ++j) {
      const int w = wj[j], off = (p - 5) * R + rj[j], x = top + off;
      if (STEADY || (p >= 5 && p - 5 < J && x >= b0 && x <= b1 - 1)) {
        const int gr = lattice_row(x, ms, L), pi = off & (PK_ROWS - 1);
        const uint32_t t = pk1[pi * WPR + w];
        const uint32_t u = pk[((pi - 1) & (PK_ROWS - 1)) * WPR + w];
        const uint32_t d = pk[((pi + 1) & (PK_ROWS - 1)) * WPR + w];
        const uint32_t* mr = pk + pi * WPR;
        const uint32_t mid = mr[w];
        const uint32_t side =
            ((gr + 1) & 1) ? right_sites(mid, mr[(w + 1) & (WPR - 1)]) : left_sites(mid, mr[(w - 1) & (WPR - 1)]);
        const uint4 A = draw(P, P_SWEEP_HI, 1u, (uint32_t)gr, (uint32_t)(2 * w), tt);
        const uint4 B = draw(P, P_SWEEP_HI, 1u, (uint32_t)gr, (uint32_t)(2 * w + 1), tt);
        uint32_t open, zero;
        uint32_t nt = decide(t, u, d, mid, side, A, B, P, open, zero);
        if (open) nt ^= enqueue<NS, LEAD>(open, zero, t, off, w, gr, 1, 3 + (p - 5) % 3, qn, Q, P, tt);
        uint4 a, b;
        unpack_bytes(mid, a, b);
        uint4* o0 = reinterpret_cast<uint4*>(out + (size_t)gr * H + 32 * w);
        o0[0] = a;
        o0[1] = b;
        unpack_bytes(nt, a, b);
        uint4* o1 = reinterpret_cast<uint4*>(out + PLANE + (size_t)gr * H + 32 * w);
        o1[0] = a;
        o1[1] = b;
      }
    }
  };
  // steady phases: groups p (pack), p-2, p-5 and the queues of p-3, p-6 all
  // lie inside the band with every row valid
  const int p_lo = 7;  // the colour-1 queue reset (group p-7) is the last action to become valid
  const int p_hi = (b1 - b0 + 3 - R) / R;  // last phase whose pack group is all valid colour-0 rows
  for (int p = 0; p <= J + 5; ++p) {
    if (p >= p_lo && p <= p_hi) {
      phase(p, std::true_type());
    } else {
      phase(p, std::false_type());
    }
    if (__syncthreads_or(!ok)) {
      // a copy did not land: wait (bounded) for the copies still in flight, then report
      if (tid == 0) {
        for (int g = p; g < J && g <= p + LEAD; ++g)
          tma::mbar_wait_bounded(&bar[g % kRawSlots], (uint32_t)((g / kRawSlots) & 1));
        atomicOr(status, 1);
      }
      __syncthreads();
      return;
    }
  }
}

}  // namespace bits
}  // namespace mcrg
