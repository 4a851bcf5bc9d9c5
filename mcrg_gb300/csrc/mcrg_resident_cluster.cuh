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
// layout) or bit-plane words.
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

// Links the larger of the two roots under the smaller (retrying while
// another thread relinks them).
__device__ __forceinline__ void unite16(uint16_t* lab, int a, int b) {
  for (int it = 0; it < kLoopLimit; ++it) {
    a = find16(lab, a);
    b = find16(lab, b);
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

// Shared-memory work area of one update: L^2 labels, L^2 / 32 coin words
// and the seed's root.
__host__ __device__ inline int work_bytes(int L) { return ((L * L * 2 + 15) / 16) * 16 + ((L * L / 8 + 15) / 16) * 16 + 16; }

// Labels and flips the components of the level's open bonds at update index t.
// kind: MCRG_UPDATE_WOLFF or MCRG_UPDATE_SWENDSEN_WANG; tb: the bond threshold.
template <class Level>
__device__ void update(const Level& lv, int L, uint8_t* work, Key key, uint32_t rep, uint32_t t, uint32_t tb,
                       int kind, int tid, int T) {
  const int n = L * L, m = L - 1, half = L / 2;
  uint16_t* lab = reinterpret_cast<uint16_t*>(work);
  uint32_t* coin = reinterpret_cast<uint32_t*>(work + ((n * 2 + 15) / 16) * 16);
  int* seed_root = reinterpret_cast<int*>(work + ((n * 2 + 15) / 16) * 16 + ((n / 8 + 15) / 16) * 16);
  const bool wolff = kind == MCRG_UPDATE_WOLFF;
  for (int x = tid; x < n; x += T) lab[x] = (uint16_t)x;
  if (!wolff)
    for (int x = tid; x < (n + 31) / 32; x += T) coin[x] = 0u;
  __syncthreads();
  // open bonds of site pairs (i, j0), (i, j0 + 1): one Philox block each
  for (int y = tid; y < n / 2; y += T) {
    const int i = y / half, j0 = 2 * (y - i * half), id = (i + 1) & m, x0 = i * L + j0;
    const uint4 r = stream_block(key, rep, P_BOND, 0u, (uint32_t)i, (uint32_t)(j0 >> 1), t);
    const uint32_t s0 = lv.spin(i, j0), s1 = lv.spin(i, j0 + 1);
    if (r.x < tb && s1 == s0) unite16(lab, x0, x0 + 1);
    if (r.y < tb && lv.spin(id, j0) == s0) unite16(lab, x0, id * L + j0);
    if (r.z < tb && lv.spin(i, (j0 + 2) & m) == s1) unite16(lab, x0 + 1, i * L + ((j0 + 2) & m));
    if (r.w < tb && lv.spin(id, j0 + 1) == s1) unite16(lab, x0 + 1, id * L + j0 + 1);
  }
  __syncthreads();
  if (wolff) {
    if (tid == 0) {
      const uint4 r = stream_block(key, rep, P_CLUSTER, 0u, 0u, 0u, t);
      *seed_root = find16(lab, (int)(r.x & (uint32_t)(n - 1)));
    }
  } else {
    for (int x = tid; x < n; x += T)
      if (lab[x] == x &&
          (stream_block(key, rep, P_CLUSTER, 1u, (uint32_t)x >> 16, (uint32_t)x & 0xFFFFu, t).x & 1u))
        atomicOr(&coin[x >> 5], 1u << (x & 31));
  }
  __syncthreads();
}

// Whether site x flips, after update() has labelled the level.
__device__ __forceinline__ bool flips(const uint8_t* work, int L, int x, bool wolff) {
  const int n = L * L;
  const uint16_t* lab = reinterpret_cast<const uint16_t*>(work);
  const uint32_t* coin = reinterpret_cast<const uint32_t*>(work + ((n * 2 + 15) / 16) * 16);
  const int r = find16(lab, x);
  if (wolff) return r == *reinterpret_cast<const int*>(work + ((n * 2 + 15) / 16) * 16 + ((n / 8 + 15) / 16) * 16);
  return (coin[r >> 5] >> (r & 31)) & 1u;
}

// One cluster update of a byte level 0.
__device__ __forceinline__ void update_bytes(uint8_t* lat, int L, uint8_t* work, Key key, uint32_t rep, uint32_t t,
                                             uint32_t tb, int kind, int tid, int T) {
  update(ByteLevel{lat, L}, L, work, key, rep, t, tb, kind, tid, T);
  const int h = L / 2;
  const bool wolff = kind == MCRG_UPDATE_WOLFF;
  for (int x = tid; x < L * L; x += T)
    if (flips(work, L, x, wolff)) {
      const int i = x / L, j = x - i * L;
      lat[(size_t)((i + j) & 1) * L * h + (size_t)i * h + (j >> 1)] ^= 1u;
    }
  __syncthreads();
}

// One cluster update of a plane level 0 (L >= 64): one thread per plane word.
__device__ __forceinline__ void update_planes(uint32_t* pl, int L, uint8_t* work, Key key, uint32_t rep, uint32_t t,
                                              uint32_t tb, int kind, int tid, int T) {
  update(PlaneLevel{pl, L}, L, work, key, rep, t, tb, kind, tid, T);
  const int wpr = L / 64, words = L * wpr;
  const bool wolff = kind == MCRG_UPDATE_WOLFF;
  for (int x = tid; x < 2 * words; x += T) {
    const int c = x >= words, r = x - c * words, i = r / wpr, w = r - i * wpr, q = (i + c) & 1;
    uint32_t mask = 0;
    for (int p = 0; p < 32; ++p)
      if (flips(work, L, i * L + 2 * (32 * w + p) + q, wolff)) mask |= 1u << planes::plane_pos(p);
    pl[x] ^= mask;
  }
  __syncthreads();
}

}  // namespace rcluster
}  // namespace mcrg
