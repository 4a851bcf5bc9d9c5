// mcrg_cluster.cu -- cluster updates (Wolff, Swendsen-Wang) of a lattice held
// in split layout in device memory: bond draws, union-find labelling, flips.
//
// The reference grows one Wolff cluster per sample breadth first
// (src/ising.cpp:87-155): every aligned nearest neighbour of a cluster site
// that is not in the cluster yet joins with probability P = 1 - exp(2K)
// (src/ising.cpp:9), and every such bond is tried once, from whichever end
// joined first.  The cluster is therefore the connected component of the
// seed site in a graph of independently open bonds, and the device labels
// that graph in parallel, in three launches per update:
//   1. cl_tile_kernel: a CTA draws the bonds of a T x T tile (T = 32, or L
//      below that), unites the sites of open in-tile bonds with a
//      shared-memory union-find and writes every site's label: the smallest
//      natural index i*L + j of its in-tile component;
//   2. cl_merge_kernel (L > 32): every open bond that crosses a tile edge
//      unites the two trees of the global forest; atomicMin links the larger
//      root under the smaller, so a root is always the smallest index of its
//      tree and, at the end, of its cluster;
//   3. cl_flip_kernel: every site finds its root; Wolff flips the sites that
//      share the seed's root, Swendsen-Wang the sites whose root draws a set
//      bit; the flips are counted.
// The result depends only on the bond draws, never on the order in which
// threads unite, so it is reproducible and equal to the oracle's labelling.
// Union and find loops make progress by construction (labels only decrease);
// they are bounded anyway and raise an error flag when the bound is hit.
#include <cmath>

#include "mcrg_internal.cuh"

namespace mcrg {
namespace {

constexpr uint32_t P_BOND = 5, P_CLUSTER = 6;
constexpr int kTile = 32;
constexpr int kFindLimit = 1 << 28;  // > L^2 for every supported L

__device__ __forceinline__ uint32_t nat_spin(const uint8_t* st, int L, int i, int j) {
  const int h = L / 2;
  return st[(size_t)((i + j) & 1) * L * h + (size_t)i * h + (j >> 1)];
}

// Open bonds of the site pair (i, j0), (i, j0 + 1), j0 even: bit 0 / 1 = the
// right / down bond of (i, j0), bit 2 / 3 = those of (i, j0 + 1).
__device__ __forceinline__ uint32_t pair_bonds(const uint8_t* st, int L, int i, int j0, Key key, uint32_t rep,
                                               uint32_t t, uint32_t tb) {
  const uint4 r = stream_block(key, rep, P_BOND, 0u, (uint32_t)i, (uint32_t)(j0 >> 1), t);
  const int m = L - 1, id = (i + 1) & m;
  const uint32_t s0 = nat_spin(st, L, i, j0), s1 = nat_spin(st, L, i, (j0 + 1) & m);
  const uint32_t s2 = nat_spin(st, L, i, (j0 + 2) & m);
  uint32_t b = 0;
  if (r.x < tb && s1 == s0) b |= 1u;
  if (r.y < tb && nat_spin(st, L, id, j0) == s0) b |= 2u;
  if (r.z < tb && s2 == s1) b |= 4u;
  if (r.w < tb && nat_spin(st, L, id, (j0 + 1) & m) == s1) b |= 8u;
  return b;
}

// Root of x in a forest whose links only decrease (volatile reads: other
// threads lower links concurrently while a tile or the merge unites).
__device__ __forceinline__ int find_root(const int* par, int x, int* err) {
  const volatile int* vp = par;
  for (int it = 0; it < kFindLimit; ++it) {
    const int p = vp[x];
    if (p == x) return x;
    x = p;
  }
  atomicOr(err, 2);
  return x;
}

// Unites the trees of a and b: the larger root is linked under the smaller.
__device__ __forceinline__ void unite(int* par, int a, int b, int* err) {
  for (int it = 0; it < kFindLimit; ++it) {
    a = find_root(par, a, err);
    b = find_root(par, b, err);
    if (a == b) return;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    const int old = atomicMin(&par[a], b);
    if (old == a) return;  // a was still a root: linked
    a = old;               // someone linked a first: continue from its new parent
  }
  atomicOr(err, 4);
}

__global__ void __launch_bounds__(256) cl_tile_kernel(const uint8_t* __restrict__ st, int L, int* __restrict__ label,
                                                      Key key, uint32_t rep, uint32_t t, uint32_t tb, int* err) {
  __shared__ int par[kTile * kTile];
  __shared__ uint8_t bd[kTile * kTile];
  const int T = L < kTile ? L : kTile, tpr = L / T, n = T * T;
  const int ti = blockIdx.x / tpr, tj = blockIdx.x - ti * tpr;
  const int i0 = ti * T, j0 = tj * T;
  for (int x = threadIdx.x; x < n; x += blockDim.x) par[x] = x;
  for (int y = threadIdx.x; y < n / 2; y += blockDim.x) {  // one Philox block per site pair
    const int x = 2 * y, li = x / T, lj = x - li * T;
    const uint32_t b = pair_bonds(st, L, i0 + li, j0 + lj, key, rep, t, tb);
    bd[x] = (uint8_t)(b & 3u);
    bd[x + 1] = (uint8_t)(b >> 2);
  }
  __syncthreads();
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    const int li = x / T, lj = x - li * T;
    const uint32_t b = bd[x];
    if (b & 1u) {
      if (lj + 1 < T) unite(par, x, x + 1, err);
      else if (T == L) unite(par, x, x - lj, err);  // periodic wrap inside a one-tile lattice
    }
    if (b & 2u) {
      if (li + 1 < T) unite(par, x, x + T, err);
      else if (T == L) unite(par, x, lj, err);
    }
  }
  __syncthreads();
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    const int li = x / T, lj = x - li * T;
    const int r = find_root(par, x, err), ri = r / T, rj = r - ri * T;
    label[(size_t)(i0 + li) * L + j0 + lj] = (i0 + ri) * L + j0 + rj;  // row-major: the tile's order is the lattice's
  }
}

// Open bonds that cross a tile edge (L > kTile): the right bonds of column
// T-1 and the down bonds of row T-1 of every tile (periodic wrap included).
__global__ void __launch_bounds__(256) cl_merge_kernel(const uint8_t* __restrict__ st, int L, int* label, Key key,
                                                       uint32_t rep, uint32_t t, uint32_t tb, int* err) {
  const int tpr = L / kTile, m = L - 1;
  const long long right = (long long)L * tpr, total = 2 * right;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    if (e < right) {
      const int i = (int)(e / tpr), j = (int)(e - (long long)i * tpr) * kTile + kTile - 1;  // odd
      const uint4 r = stream_block(key, rep, P_BOND, 0u, (uint32_t)i, (uint32_t)(j >> 1), t);
      if (r.z < tb && nat_spin(st, L, i, j) == nat_spin(st, L, i, (j + 1) & m))
        unite(label, i * L + j, i * L + ((j + 1) & m), err);
    } else {
      const long long e2 = e - right;
      const int i = (int)(e2 / L) * kTile + kTile - 1, j = (int)(e2 - (e2 / L) * L);
      const uint4 r = stream_block(key, rep, P_BOND, 0u, (uint32_t)i, (uint32_t)(j >> 1), t);
      const uint32_t u = (j & 1) ? r.w : r.y;
      if (u < tb && nat_spin(st, L, i, j) == nat_spin(st, L, (i + 1) & m, j))
        unite(label, i * L + j, ((i + 1) & m) * L + j, err);
    }
  }
}

__global__ void __launch_bounds__(256) cl_flip_kernel(uint8_t* __restrict__ st, int L, const int* __restrict__ label,
                                                      int kind, Key key, uint32_t rep, uint32_t t,
                                                      unsigned long long* count, int* err) {
  __shared__ int seed_root;
  __shared__ unsigned long long warp_cnt[8];
  if (kind == MCRG_UPDATE_WOLFF && threadIdx.x == 0) {
    const uint4 r = stream_block(key, rep, P_CLUSTER, 0u, 0u, 0u, t);
    seed_root = find_root(label, (int)(r.x & (uint32_t)(L * L - 1)), err);
  }
  __syncthreads();
  const int h = L / 2;
  unsigned long long cnt = 0;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < (long long)L * L;
       s += (long long)gridDim.x * blockDim.x) {
    const int r = find_root(label, (int)s, err);
    bool flip;
    if (kind == MCRG_UPDATE_WOLFF) {
      flip = r == seed_root;
    } else {
      const uint4 b = stream_block(key, rep, P_CLUSTER, 1u, (uint32_t)r >> 16, (uint32_t)r & 0xFFFFu, t);
      flip = (b.x & 1u) != 0;
    }
    if (flip) {
      const int i = (int)(s / L), j = (int)(s - (long long)i * L);
      st[(size_t)((i + j) & 1) * L * h + (size_t)i * h + (j >> 1)] ^= 1u;
      ++cnt;
    }
  }
  cnt = __reduce_add_sync(0xFFFFFFFFu, (unsigned)cnt);
  if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += warp_cnt[w];
    if (tot) atomicAdd(count, tot);
  }
}

}  // namespace

cudaError_t launch_cluster_update(uint8_t* d_state, int L, int* d_label, int kind, Key key, uint32_t replica,
                                  uint32_t t, uint32_t bond_threshold, unsigned long long* d_count, int* d_err,
                                  int num_sms, cudaStream_t s) {
  const int T = L < kTile ? L : kTile, tiles = (L / T) * (L / T);
  cl_tile_kernel<<<tiles, 256, 0, s>>>(d_state, L, d_label, key, replica, t, bond_threshold, d_err);
  if (L > kTile) {
    const long long edges = 2LL * L * (L / kTile);
    long long blocks = (edges + 255) / 256;
    if (blocks > 8LL * num_sms) blocks = 8LL * num_sms;
    cl_merge_kernel<<<(int)blocks, 256, 0, s>>>(d_state, L, d_label, key, replica, t, bond_threshold, d_err);
  }
  long long blocks = ((long long)L * L + 255) / 256;
  if (blocks > 16LL * num_sms) blocks = 16LL * num_sms;
  cl_flip_kernel<<<(int)blocks, 256, 0, s>>>(d_state, L, d_label, kind, key, replica, t, d_count, d_err);
  return cudaGetLastError();
}

uint32_t bond_threshold(double K) {
  const double p = 1.0 - exp(2.0 * K);
  if (!(p > 0.0)) return 0u;
  const double x = floor(p * 4294967296.0);
  return x >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)x;
}

}  // namespace mcrg
