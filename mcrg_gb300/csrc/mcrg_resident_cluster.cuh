// mcrg_resident_cluster.cuh -- Wolff / Swendsen-Wang updates of a
// shared-memory-resident lattice (L <= 256) inside a chain's CTA.
//
// The same update as the device-wide kernels of mcrg_cluster.cu and the
// reference's Wolff step it restates (src/ising.cpp:87-155): bonds between
// aligned nearest neighbours open from the purpose-5 Philox stream, clusters
// are the connected components of the open bonds, Wolff flips the seed's
// component, Swendsen-Wang every component whose smallest site index draws a
// set coin.  Here one CTA labels its own lattice with a union-find over
// 16-bit labels in shared memory (L^2 <= 65536 sites): a label only
// decreases (compare-and-swap minimum on the 32-bit word that holds it), so
// a root is always the smallest index of its tree and, once all bonds are
// united, of its component -- the same roots as the device-wide labelling,
// hence the same flips.  The lattice is the chain's level 0: bytes (split
// layout) or bit-plane words.  For L >= 32 a warp owns 32-column row
// segments: the segment's open horizontal bonds are one ballot mask, every
// site points at the first site of its run, and only vertical bonds (one per
// pair of runs) and segment-crossing bonds are united, with path halving;
// a flatten pass leaves every label at its root before the flips.
#pragma once
#include "mcrg_planes.cuh"

namespace mcrg {
namespace rcluster {

constexpr int kLoopLimit = 1 << 20;  // bound of every find / union loop (never reached: labels only decrease)

// Level 0 as split-layout bytes.
struct ByteLevel {
  uint8_t* lat;
  int L;
  __device__ __forceinline__ uint32_t spin(int i, int j) const {
    const int h = L / 2;
    return lat[(size_t)((i + j) & 1) * L * h + (size_t)i * h + (j >> 1)];
  }
};

// Level 0 as plane words: colour c, row i, word w at pl[c * L * L / 64 + i * L / 64 + w].
struct PlaneLevel {
  uint32_t* pl;
  int L;
  __device__ __forceinline__ uint32_t spin(int i, int j) const {
    const int k = j >> 1, wpr = L / 64;
    const uint32_t w = pl[(size_t)((i + j) & 1) * L * wpr + (size_t)i * wpr + (k >> 5)];
    return (w >> planes::plane_pos(k & 31)) & 1u;
  }
};

__device__ __forceinline__ int find16(const uint16_t* lab, int x) {
  const volatile uint16_t* v = lab;
  for (int it = 0; it < kLoopLimit; ++it) {
    const int p = v[x];
    if (p == x) break;
    x = p;
  }
  return x;
}

// Lowers label x to at most b; returns the label it held before.
__device__ __forceinline__ int min16(uint16_t* lab, int x, int b) {
  uint32_t* w = reinterpret_cast<uint32_t*>(lab) + (x >> 1);
  const int sh = (x & 1) * 16;
  uint32_t old = *reinterpret_cast<volatile uint32_t*>(w);
  for (int it = 0; it < kLoopLimit; ++it) {
    const int cur = (int)((old >> sh) & 0xFFFFu);
    if (cur <= b) return cur;
    const uint32_t upd = (old & ~(0xFFFFu << sh)) | ((uint32_t)b << sh);
    const uint32_t prev = atomicCAS(w, old, upd);
    if (prev == old) return cur;
    old = prev;
  }
  return b;
}

// Root of x with path halving (each visited label lowered to its grandparent).
__device__ __forceinline__ int find_halve16(uint16_t* lab, int x) {
  const volatile uint16_t* v = lab;
  for (int it = 0; it < kLoopLimit; ++it) {
    const int p = v[x];
    if (p == x) break;
    const int gp = v[p];
    if (gp == p) return p;
    min16(lab, x, gp);
    x = gp;
  }
  return x;
}

// Links the larger of the two roots under the smaller (retrying while
// another thread relinks them).
template <bool HALVE = false>
__device__ __forceinline__ void unite16(uint16_t* lab, int a, int b) {
  for (int it = 0; it < kLoopLimit; ++it) {
    a = HALVE ? find_halve16(lab, a) : find16(lab, a);
    b = HALVE ? find_halve16(lab, b) : find16(lab, b);
    if (a == b) return;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    const int old = min16(lab, a, b);
    if (old == a) return;
    a = old;
  }
}

// Shared-memory work area of one update: L^2 labels, L^2 / 32 coin words,
// the horizontal and vertical bond masks of every 32-column row segment
// (L >= 32) and the seed's root.
__host__ __device__ inline int work_bytes(int L) {
  return ((L * L * 2 + 15) / 16) * 16 + 3 * ((L * L / 8 + 15) / 16) * 16 + 16;
}
__device__ __forceinline__ int coin_off(int n) { return ((n * 2 + 15) / 16) * 16; }
__device__ __forceinline__ int hb_off(int n) { return coin_off(n) + ((n / 8 + 15) / 16) * 16; }
__device__ __forceinline__ int vb_off(int n) { return hb_off(n) + ((n / 8 + 15) / 16) * 16; }
__device__ __forceinline__ int seed_off(int n) { return vb_off(n) + ((n / 8 + 15) / 16) * 16; }

// Labels and flips the components of the level's open bonds at update index t.
// kind: MCRG_UPDATE_WOLFF or MCRG_UPDATE_SWENDSEN_WANG; tb: the bond threshold.
template <class Level>
__device__ void update(const Level& lv, int L, uint8_t* work, Key key, uint32_t rep, uint32_t t, uint32_t tb,
                       int kind, int tid, int T) {
  const int n = L * L, m = L - 1, half = L / 2;
  uint16_t* lab = reinterpret_cast<uint16_t*>(work);
  uint32_t* coin = reinterpret_cast<uint32_t*>(work + coin_off(n));
  int* seed_root = reinterpret_cast<int*>(work + seed_off(n));
  const bool wolff = kind == MCRG_UPDATE_WOLFF;
  if (!wolff)
    for (int x = tid; x < (n + 31) / 32; x += T) coin[x] = 0u;
  if (L >= 32) {
    uint32_t* hb = reinterpret_cast<uint32_t*>(work + hb_off(n));
    uint32_t* vb = reinterpret_cast<uint32_t*>(work + vb_off(n));
    const int segs = L / 32, units = L * segs, lane = tid & 31, warp = tid >> 5, nw = T >> 5;
    const int ls = __ffs(segs) - 1;  // L is a power of two: divisions by segs are shifts
    // runs: unit u = row u / segs, columns 32 (u % segs) .. +31; two units per pass,
    // lane l draws pair l & 15 of unit 2v + (l >> 4)
    for (int v = warp; v < units / 2; v += nw) {
      const int ud = 2 * v + (lane >> 4), di = ud >> ls, dj = (ud & (segs - 1)) * 32;
      const uint4 R = stream_block(key, rep, P_BOND, 0u, (uint32_t)di, (uint32_t)((dj >> 1) + (lane & 15)), t);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int u = 2 * v + h, i = u >> ls, j0 = (u & (segs - 1)) * 32, src = h * 16 + (lane >> 1);
        const uint32_t wx = __shfl_sync(0xFFFFFFFFu, R.x, src), wy = __shfl_sync(0xFFFFFFFFu, R.y, src);
        const uint32_t wz = __shfl_sync(0xFFFFFFFFu, R.z, src), ww = __shfl_sync(0xFFFFFFFFu, R.w, src);
        const uint32_t ur = (lane & 1) ? wz : wx, udn = (lane & 1) ? ww : wy;
        const int j = j0 + lane;
        const uint32_t s = lv.spin(i, j);
        const bool right = ur < tb && lv.spin(i, (j + 1) & m) == s;  // lane 31: the bond into the next segment
        const bool down = udn < tb && lv.spin((i + 1) & m, j) == s;
        const uint32_t hm = __ballot_sync(0xFFFFFFFFu, right), vm = __ballot_sync(0xFFFFFFFFu, down);
        const uint32_t starts = ~(hm << 1);
        const uint32_t low = lane == 31 ? 0xFFFFFFFFu : ((2u << lane) - 1u);
        lab[i * L + j] = (uint16_t)(i * L + j0 + (31 - __clz(starts & low)));
        if (lane == 0) {
          hb[u] = hm;
          vb[u] = vm;
        }
      }
    }
    chain_sync(T);
    for (int u = warp; u < units; u += nw) {
      const int i = u >> ls, sg = u & (segs - 1), j0 = sg * 32, in = (i + 1) & m;
      const uint32_t vv = vb[u], hr = hb[u], hn = hb[in * segs + sg];
      const uint32_t dup = (vv & hr & hn) << 1;  // column c-1 already joins the same two runs
      if (((vv & ~dup) >> lane) & 1u) unite16<true>(lab, i * L + j0 + lane, in * L + j0 + lane);
      if (lane == 31 && (hr >> 31)) unite16<true>(lab, i * L + j0 + 31, i * L + ((j0 + 32) & m));
    }
  } else {
    for (int x = tid; x < n; x += T) lab[x] = (uint16_t)x;
    chain_sync(T);
    // open bonds of site pairs (i, j0), (i, j0 + 1): one Philox block each
    for (int y = tid; y < n / 2; y += T) {
      const int i = y >> (__ffs(half) - 1), j0 = 2 * (y & (half - 1)), id = (i + 1) & m, x0 = i * L + j0;
      const uint4 r = stream_block(key, rep, P_BOND, 0u, (uint32_t)i, (uint32_t)(j0 >> 1), t);
      const uint32_t s0 = lv.spin(i, j0), s1 = lv.spin(i, j0 + 1);
      if (r.x < tb && s1 == s0) unite16(lab, x0, x0 + 1);
      if (r.y < tb && lv.spin(id, j0) == s0) unite16(lab, x0, id * L + j0);
      if (r.z < tb && lv.spin(i, (j0 + 2) & m) == s1) unite16(lab, x0 + 1, i * L + ((j0 + 2) & m));
      if (r.w < tb && lv.spin(id, j0 + 1) == s1) unite16(lab, x0 + 1, id * L + j0 + 1);
    }
  }
  chain_sync(T);
  for (int x = tid; x < n; x += T) lab[x] = (uint16_t)find16(lab, x);  // flatten: every label at its root
  chain_sync(T);
  if (wolff) {
    if (tid == 0) {
      const uint4 r = stream_block(key, rep, P_CLUSTER, 0u, 0u, 0u, t);
      *seed_root = lab[r.x & (uint32_t)(n - 1)];
    }
  } else {
    for (int x = tid; x < n; x += T)
      if (lab[x] == x &&
          (stream_block(key, rep, P_CLUSTER, 1u, (uint32_t)x >> 16, (uint32_t)x & 0xFFFFu, t).x & 1u))
        atomicOr(&coin[x >> 5], 1u << (x & 31));
  }
  chain_sync(T);
}

// Whether site x flips, after update() has labelled the level (labels flattened).
__device__ __forceinline__ bool flips(const uint8_t* work, int L, int x, bool wolff) {
  const int n = L * L;
  const int r = reinterpret_cast<const uint16_t*>(work)[x];
  if (wolff) return r == *reinterpret_cast<const int*>(work + seed_off(n));
  return (reinterpret_cast<const uint32_t*>(work + coin_off(n))[r >> 5] >> (r & 31)) & 1u;
}

// One cluster update of a byte level 0.
__device__ __forceinline__ void update_bytes(uint8_t* lat, int L, uint8_t* work, Key key, uint32_t rep, uint32_t t,
                                             uint32_t tb, int kind, int tid, int T) {
  update(ByteLevel{lat, L}, L, work, key, rep, t, tb, kind, tid, T);
  const int h = L / 2;
  const bool wolff = kind == MCRG_UPDATE_WOLFF;
  for (int x = tid; x < L * L; x += T)
    if (flips(work, L, x, wolff)) {
      const int i = x >> (__ffs(L) - 1), j = x & (L - 1);
      lat[(size_t)((i + j) & 1) * L * h + (size_t)i * h + (j >> 1)] ^= 1u;
    }
  chain_sync(T);
}

// One cluster update of a plane level 0 (L >= 64): one thread per plane word.
__device__ __forceinline__ void update_planes(uint32_t* pl, int L, uint8_t* work, Key key, uint32_t rep, uint32_t t,
                                              uint32_t tb, int kind, int tid, int T) {
  update(PlaneLevel{pl, L}, L, work, key, rep, t, tb, kind, tid, T);
  const int wpr = L / 64, words = L * wpr;
  const bool wolff = kind == MCRG_UPDATE_WOLFF;
  for (int x = tid; x < 2 * words; x += T) {
    const int c = x >= words, r = x - c * words, i = r >> (__ffs(wpr) - 1), w = r & (wpr - 1), q = (i + c) & 1;
    // site p of the word has label word (i L + 64 w + 2 p + q) / 2, bank p: the lanes start at
    // p = lane and go round, so that they read 32 different banks at every step
    const int lane = tid & 31;
    uint32_t mask = 0;
    for (int s = 0; s < 32; ++s) {
      const int p = (s + lane) & 31;
      if (flips(work, L, i * L + 2 * (32 * w + p) + q, wolff)) mask |= 1u << planes::plane_pos(p);
    }
    pl[x] ^= mask;
  }
  chain_sync(T);
}

}  // namespace rcluster
}  // namespace mcrg
