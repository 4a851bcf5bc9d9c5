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
//      natural index i*L + j of its in-tile component.  With T = 32 a warp
//      owns a tile row: the row's open horizontal bonds form a ballot mask,
//      every site points at the first site of its run (count leading zeros),
//      and only vertical bonds are united, one per pair of runs, taken by
//      all threads from one list for the whole tile;
//      It also records, as two 32-bit masks per tile, which of its bonds into
//      the next tiles (right of column 31, below row 31) are open: it draws
//      them anyway and holds the spins on both sides;
//   2. cl_merge_kernel (L > 32): every open bond that crosses a tile edge (a
//      set mask bit) unites the two trees of the global forest; atomicMin
//      links the larger root under the smaller, so a root is always the
//      smallest index of its tree and, at the end, of its cluster (finds halve
//      the paths they walk: a cluster spanning thousands of tiles would
//      otherwise leave long chains);
//   3. cl_flip_kernel: every site finds its root; Wolff flips the sites that
//      share the seed's root, Swendsen-Wang the sites whose root draws a set
//      bit; the flips are counted.  With T = 32 a CTA loads its tile's labels
//      and resolves the global root (and coin) once per entry of a compacted
//      list: each in-tile component's root, and each tile root the merge
//      linked into another tile.
// The result depends only on the bond draws, never on the order in which
// threads unite, so it is reproducible and equal to the oracle's labelling.
// Union and find loops make progress by construction (labels only decrease);
// they are bounded anyway and raise an error flag when the bound is hit.
#include <cmath>

#include "mcrg_internal.cuh"

namespace mcrg {
namespace {

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

// Root of x with path halving: each visited link is lowered to its
// grandparent by atomicMin, so links still only decrease.
__device__ __forceinline__ int find_halve(int* par, int x, int* err) {
  const volatile int* vp = par;
  for (int it = 0; it < kFindLimit; ++it) {
    const int p = vp[x];
    if (p == x) return x;
    const int gp = vp[p];
    if (gp == p) return p;
    atomicMin(&par[x], gp);
    x = gp;
  }
  atomicOr(err, 2);
  return x;
}

// Unites the trees of a and b: the larger root is linked under the smaller.
template <bool HALVE = false>
__device__ __forceinline__ void unite(int* par, int a, int b, int* err) {
  for (int it = 0; it < kFindLimit; ++it) {
    a = HALVE ? find_halve(par, a, err) : find_root(par, a, err);
    b = HALVE ? find_halve(par, b, err) : find_root(par, b, err);
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

// Tiles of 32 x 32 (L >= 32): warp w owns rows w, w+8, w+16, w+24.  Sites
// point at the first site of their horizontal run; vertical bonds unite runs.
// Besides the in-tile labels it records the tile's bonds into the next tiles
// (L > 32), whose draws it makes anyway: edges[2 tile] bit r = the right bond
// of (i0 + r, j0 + 31), edges[2 tile + 1] bit c = the down bond of
// (i0 + 31, j0 + c).  The merge then reads these masks instead of drawing the
// bonds and reading the spins again.
__global__ void __launch_bounds__(256) cl_tile32_kernel(const uint8_t* __restrict__ st, int L,
                                                        int* __restrict__ label, uint32_t* __restrict__ edges,
                                                        Key key, uint32_t rep, uint32_t t, uint32_t tb, int* err) {
  __shared__ int par[1024];
  __shared__ uint8_t sp[33 * 32];  // spins of the tile's rows and of the row below it
  __shared__ uint8_t ecol[32];     // spins of column j0 + 32 (the next tile's first column)
  __shared__ uint32_t hb[32], vb[32], redge;
  __shared__ int vlist[1024], nv;  // vertical bonds that join two runs, as their upper site
  const int tpr = L >> 5, ti = blockIdx.x / tpr, tj = blockIdx.x - ti * tpr;
  const int i0 = ti << 5, j0 = tj << 5, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool one = L == 32;  // a one-tile lattice: its wrap bonds are in-tile bonds
  const int h = L / 2;
  if (threadIdx.x == 0) {
    nv = 0;
    redge = 0;
  }
  if (threadIdx.x < 66) {  // 33 rows x 2 colours: 16 bytes each, de-interleaved into natural order
    const int r = threadIdx.x >> 1, c = threadIdx.x & 1, i = (i0 + r) & (L - 1);
    const uint4 v = *reinterpret_cast<const uint4*>(st + (size_t)c * L * h + (size_t)i * h + (j0 >> 1));
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    const int q = (i + c) & 1;  // column parity of colour c in row i (j0 is even)
#pragma unroll
    for (int b = 0; b < 16; ++b) sp[r * 32 + 2 * b + q] = (uint8_t)((w[b >> 2] >> (8 * (b & 3))) & 0xFFu);
  } else if (threadIdx.x >= 96 && threadIdx.x < 128 && !one) {  // site (i, j0 + 32): colour i & 1 (j0 + 32 is even)
    const int r = threadIdx.x - 96, i = i0 + r;
    ecol[r] = st[(size_t)(i & 1) * L * h + (size_t)i * h + (((j0 + 32) & (L - 1)) >> 1)];
  }
  __syncthreads();
  for (int rp = warp; rp < 16; rp += 8) {  // row pairs 2rp, 2rp+1: lane l draws pair l & 15 of row 2rp + (l >> 4)
    const uint4 R = stream_block(key, rep, P_BOND, 0u, (uint32_t)(i0 + 2 * rp + (lane >> 4)),
                                 (uint32_t)((j0 >> 1) + (lane & 15)), t);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = 2 * rp + h, src = h * 16 + (lane >> 1);
      const uint32_t wx = __shfl_sync(0xFFFFFFFFu, R.x, src), wy = __shfl_sync(0xFFFFFFFFu, R.y, src);
      const uint32_t wz = __shfl_sync(0xFFFFFFFFu, R.z, src), ww = __shfl_sync(0xFFFFFFFFu, R.w, src);
      const uint32_t ur = (lane & 1) ? wz : wx, ud = (lane & 1) ? ww : wy;
      const uint32_t s = sp[r * 32 + lane];
      const bool right = ur < tb && (lane < 31 || one) && sp[r * 32 + ((lane + 1) & 31)] == s;
      const bool down = ud < tb && (r < 31 || one) && sp[(r + 1) * 32 + lane] == s;
      const uint32_t hm = __ballot_sync(0xFFFFFFFFu, right), vm = __ballot_sync(0xFFFFFFFFu, down);
      if (!one) {  // the bonds into the next tiles: right of column 31, below row 31
        if (lane == 31 && ur < tb && ecol[r] == s) atomicOr(&redge, 1u << r);
        if (r == 31) {
          const uint32_t dm = __ballot_sync(0xFFFFFFFFu, ud < tb && sp[32 * 32 + lane] == s);
          if (lane == 0) edges[2 * (size_t)blockIdx.x + 1] = dm;
        }
      }
      const uint32_t starts = ~(hm << 1);  // bit c: the bond (c-1, c) is closed (bit 0 always); the wrap bit drops out
      const uint32_t low = lane == 31 ? 0xFFFFFFFFu : ((2u << lane) - 1u);
      par[r * 32 + lane] = r * 32 + (31 - __clz(starts & low));
      if (lane == 0) {
        hb[r] = hm;
        vb[r] = vm;
      }
    }
  }
  __syncthreads();
  // The unions go through one list for the whole tile, so that the rows with
  // the longest union chains do not hold every other warp at the barrier.
  for (int r = warp; r < 32; r += 8) {
    const int rn = (r + 1) & 31;
    const uint32_t v = vb[r], hr = hb[r], hn = hb[rn];
    const uint32_t dup = (v & hr & hn) << 1;  // column c-1 already joins the same two runs
    const uint32_t m = v & ~dup;
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(&nv, __popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if ((m >> lane) & 1u) vlist[base + __popc(m & ((1u << lane) - 1u))] = r * 32 + lane;
  }
  __syncthreads();
  if (!one && threadIdx.x == 0) edges[2 * (size_t)blockIdx.x] = redge;
  for (int e = threadIdx.x; e < nv; e += 256) {
    const int x = vlist[e];
    unite<true>(par, x, (x + 32) & 1023, err);
  }
  if (one && threadIdx.x < 32 && (hb[threadIdx.x] >> 31))  // horizontal wrap of a one-tile lattice
    unite<true>(par, threadIdx.x * 32 + 31, threadIdx.x * 32, err);
  __syncthreads();
  for (int x = threadIdx.x; x < 1024; x += 256) {
    const int r = find_root(par, x, err);
    label[(size_t)(i0 + (x >> 5)) * L + j0 + (x & 31)] = (i0 + (r >> 5)) * L + j0 + (r & 31);
  }
}

// Open bonds that cross a tile edge (L > kTile), from the masks the tile
// kernel recorded: the right bonds of column 31 and the down bonds of row 31
// of every tile (periodic wrap included).  One thread per mask bit; a warp
// reads one mask.
__global__ void __launch_bounds__(256) cl_merge_kernel(const uint32_t* __restrict__ edges, int L, int* label,
                                                       int* err) {
  const int tpr = L / kTile, m = L - 1;
  const long long total = 64LL * tpr * tpr;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long tile = e >> 6;
    const int b = (int)(e & 63), k = b & 31;
    if (!((edges[2 * tile + (b >> 5)] >> k) & 1u)) continue;
    const int ti = (int)(tile / tpr), tj = (int)(tile - (long long)ti * tpr);
    const int i0 = ti * kTile, j0 = tj * kTile;
    if (b < 32) {
      const int i = i0 + k, j = j0 + kTile - 1;
      unite<true>(label, i * L + j, i * L + ((j + 1) & m), err);
    } else {
      const int i = i0 + kTile - 1, j = j0 + k;
      unite<true>(label, i * L + j, ((i + 1) & m) * L + j, err);
    }
  }
}

// Every other bit of x (bits 0, 2, .., 30) packed into the low 16 bits.
__device__ __forceinline__ uint32_t even_bits(uint32_t x) {
  x &= 0x55555555u;
  x = (x | (x >> 1)) & 0x33333333u;
  x = (x | (x >> 2)) & 0x0F0F0F0Fu;
  x = (x | (x >> 4)) & 0x00FF00FFu;
  return (x | (x >> 8)) & 0x0000FFFFu;
}

// Flips of a 32 x 32 tile (L >= 32): the global root and the coin of every
// in-tile component are resolved once, then every site looks them up; a
// warp owns a tile row and applies its flips as two 16-byte XORs.
__global__ void __launch_bounds__(256) cl_flip32_kernel(uint8_t* __restrict__ st, int L, int lg,
                                                        int* label, int kind, Key key, uint32_t rep,
                                                        uint32_t t, unsigned long long* count, int* err) {
  __shared__ int lbl[1024], groot[1024], todo[1024];
  __shared__ uint8_t need[1024], coin[1024];
  __shared__ int seed_root, n_todo;
  __shared__ unsigned long long warp_cnt[8];
  const int tpr = L >> 5, ti = blockIdx.x >> (lg - 5), tj = blockIdx.x & (tpr - 1);
  const int i0 = ti << 5, j0 = tj << 5, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool wolff = kind == MCRG_UPDATE_WOLFF;
  if (wolff && threadIdx.x == 0) {
    const uint4 r = stream_block(key, rep, P_CLUSTER, 0u, 0u, 0u, t);
    seed_root = find_halve(label, (int)(r.x & (uint32_t)(L * L - 1)), err);
  }
  for (int x = threadIdx.x; x < 1024; x += 256) need[x] = 0;
  if (threadIdx.x == 0) n_todo = 0;
  __syncthreads();
  // the in-tile index of a label, or -1 when it lies outside the tile
  auto loc = [&](int v) {
    const int vi = (v >> lg) - i0, vj = (v & (L - 1)) - j0;
    return ((unsigned)vi < 32u && (unsigned)vj < 32u) ? (vi << 5) + vj : -1;
  };
  // Every site resolves through one entry of the list: its label's site when
  // that lies in the tile (a member's in-tile root, or the root another
  // in-tile root was linked to), else itself (a root the merge linked to
  // another tile).
  for (int x = threadIdx.x; x < 1024; x += 256) {
    const int v = label[((size_t)(i0 + (x >> 5)) << lg) + j0 + (x & 31)];
    lbl[x] = v;
    const int q = loc(v);
    need[q >= 0 ? q : x] = 1;
  }
  __syncthreads();
  // the in-tile components' roots as a dense list (one shared atomic per warp and pass), so that
  // their global root lookups and coins keep every lane busy
  for (int x = threadIdx.x; x < 1024; x += 256) {
    const bool nd = need[x] != 0;
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, nd);
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(&n_todo, __popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (nd) todo[base + __popc(m & ((1u << lane) - 1u))] = x;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n_todo; e += 256) {
    const int x = todo[e];
    const int r = find_halve(label, ((i0 + (x >> 5)) << lg) + j0 + (x & 31), err);
    groot[x] = r;
    if (!wolff)
      coin[x] = (uint8_t)(stream_block(key, rep, P_CLUSTER, 1u, (uint32_t)r >> 16, (uint32_t)r & 0xFFFFu, t).x & 1u);
  }
  __syncthreads();
  const int h = L / 2;
  unsigned cnt = 0;
  for (int r = warp; r < 32; r += 8) {
    const int x = (r << 5) + lane, q = loc(lbl[x]), k = q >= 0 ? q : x;
    const bool flip = wolff ? groot[k] == seed_root : coin[k] != 0;
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, flip);
    if (lane < 2 && m) {  // lane c: the 16 bytes of colour c in this row segment
      const int i = i0 + r, c = lane, par = (i + c) & 1;  // colour c holds the columns of parity (i + c) & 1
      const uint32_t bits = even_bits(m >> par);
      if (bits) {
        uint4* p = reinterpret_cast<uint4*>(st + (size_t)c * L * h + (size_t)i * h + (j0 >> 1));
        uint4 v4 = *p;
        v4.x ^= spread4(bits);
        v4.y ^= spread4(bits >> 4);
        v4.z ^= spread4(bits >> 8);
        v4.w ^= spread4(bits >> 12);
        *p = v4;
      }
    }
    if (lane == 0) cnt += (unsigned)__popc(m);
  }
  if (lane == 0) warp_cnt[warp] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int w = 0; w < 8; ++w) tot += warp_cnt[w];
    if (tot) atomicAdd(count, tot);
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
  uint32_t* edges = reinterpret_cast<uint32_t*>(d_label + (size_t)L * L);  // 2 masks per tile
  if (L >= kTile)
    cl_tile32_kernel<<<tiles, 256, 0, s>>>(d_state, L, d_label, edges, key, replica, t, bond_threshold, d_err);
  else
    cl_tile_kernel<<<tiles, 256, 0, s>>>(d_state, L, d_label, key, replica, t, bond_threshold, d_err);
  if (L > kTile) {
    const long long bits = 64LL * tiles;
    long long blocks = (bits + 255) / 256;
    if (blocks > 8LL * num_sms) blocks = 8LL * num_sms;
    cl_merge_kernel<<<(int)blocks, 256, 0, s>>>(edges, L, d_label, d_err);
  }
  if (L >= kTile) {
    int lg = 0;
    while ((1 << lg) < L) ++lg;
    cl_flip32_kernel<<<tiles, 256, 0, s>>>(d_state, L, lg, d_label, kind, key, replica, t, d_count, d_err);
  } else {
    cl_flip_kernel<<<1, 256, 0, s>>>(d_state, L, d_label, kind, key, replica, t, d_count, d_err);
  }
  return cudaGetLastError();
}

uint32_t bond_threshold(double K) {
  const double p = 1.0 - exp(2.0 * K);
  if (!(p > 0.0)) return 0u;
  const double x = floor(p * 4294967296.0);
  return x >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)x;
}

}  // namespace mcrg
