// mcrg_sweep_tiled.cuh -- the fused two-colour checkerboard sweep of an
// HBM-resident lattice (one read and one write of every site per sweep).
//
// A persistent CTA walks tiles of TR rows x TC bytes (per colour).  For each
// tile one warp stages, with TMA bulk copies (cp.async.bulk + mbarrier), the
// old colour-1 rows r0-2 .. r0+TR+1 and colour-0 rows r0-1 .. r0+TR, each
// widened by 16 bytes on both sides (periodic wraps split into separate
// copies).  Colour 0 is updated on the tile plus its halo, colour 1 on the
// tile from the new colour 0, and the tile is written to the other buffer of
// a ping-pong pair.  Halo sites are updated by both neighbouring tiles; the
// counter-based draws are keyed by the global site, so both compute the same
// value, and reads come from one buffer while writes go to the other.
//
// Per 16-site chunk: one Philox block gives an 8-bit draw per site; the SWAR
// update decides every site whose 8-bit draw differs from the top byte of its
// threshold and flags the rest (1/256 of the draws).  Each thread keeps the
// flags of its chunks in registers and resolves them itself at the end of the
// colour's pass with the remaining 24 bits (P_SWEEP_LO); same-colour sites do
// not interact, so no other thread waits for them except through the barrier
// that ends the pass.  Two block barriers per tile.
#pragma once
#include "mcrg_ops.cuh"

namespace mcrg {
namespace tiled {

struct Params {
  int L, h, tiles_x, n_tiles;
  Key key;
  uint32_t rep;
  Accept acc;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Copies global bytes [k0 - 16, k0 - 16 + len) (mod h) of one row into dst.
__device__ __forceinline__ void stage_row(uint8_t* dst, const uint8_t* row, int h, int k0, int len, uint64_t* bar) {
  int g = k0 - 16;
  if (g < 0) g += h;
  int z = 0;
  while (z < len) {
    const int run = min(len - z, h - g);
    bulk_g2s(dst + z, row + g, (uint32_t)run, bar);
    z += run;
    g = 0;
  }
}

__device__ __forceinline__ uint4 lds128(const uint8_t* p) { return *reinterpret_cast<const uint4*>(p); }
__device__ __forceinline__ uint32_t lds32(const uint8_t* p) { return *reinterpret_cast<const uint32_t*>(p); }

// SWAR update of one 16-byte chunk.  prv / nxt: the aligned words just
// before / after the chunk in the side-neighbour row (only their top / low
// byte is used).  Updates tw in place and returns the open sites as a mask
// with bit (8*b + 7 - j) for byte b of word j.
__device__ __forceinline__ uint32_t update16(uint32_t (&tw)[4], const uint4& U, const uint4& D, const uint4& Mw,
                                             uint32_t prv, uint32_t nxt, uint32_t q, const uint4& R,
                                             const Accept& a) {
  const uint32_t mw[4] = {Mw.x, Mw.y, Mw.z, Mw.w};
  const uint32_t uw[4] = {U.x, U.y, U.z, U.w};
  const uint32_t dw[4] = {D.x, D.y, D.z, D.w};
  const uint32_t rw[4] = {R.x, R.y, R.z, R.w};
  // side neighbour: the row shifted by one byte towards k+1 (q = 1) or k-1 (q = 0)
  uint32_t V[5];
  V[0] = q ? mw[0] : prv;
  V[1] = q ? mw[1] : mw[0];
  V[2] = q ? mw[2] : mw[1];
  V[3] = q ? mw[3] : mw[2];
  V[4] = q ? nxt : mw[3];
  const uint32_t sh = 24u - 16u * q;
  uint32_t tie[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const uint32_t side = __funnelshift_r(V[j], V[j + 1], sh);
    tw[j] = swar_update(tw[j], uw[j], dw[j], mw[j], side, rw[j], a, &tie[j]);
  }
  return tie[0] | (tie[1] >> 1) | (tie[2] >> 2) | (tie[3] >> 3);
}

// Exact resolution of one open site: t its value, its four neighbours
// n0..n3; returns true when it flips (r24 below the threshold's low 24 bits).
__device__ __forceinline__ bool resolve_open(uint32_t t, uint32_t n0, uint32_t n1, uint32_t n2, uint32_t n3,
                                             const Params& P, uint32_t c, int gr, int gk, uint32_t tt) {
  const uint32_t m = (n0 != t) + (n1 != t) + (n2 != t) + (n3 != t);
  if (m > 1) return false;  // only reachable for the unused outermost halo bytes
  const uint4 lo = stream_block(P.key, P.rep, P_SWEEP_LO, c, (uint32_t)gr, (uint32_t)(gk >> 2), tt);
  return (u4get(lo, gk & 3) & 0xFFFFFFu) < (P.acc.thr[m] & 0xFFFFFFu);
}

template <int TR, int TC, int NT>
__global__ void __launch_bounds__(NT, 2)
    sweep_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, Params P, uint32_t tt,
                 int* __restrict__ status) {
  constexpr int CPR = TC / 16;         // tile chunks per row
  constexpr int CPA = CPR + 2;         // staged chunks per row (halo chunk on each side)
  constexpr int PITCH = TC + 32;
  constexpr int NB = (TR + 2) * CPA;   // colour-0 chunks (tile + halo)
  constexpr int NBI = (NB + NT - 1) / NT;
  constexpr int NW = TR * CPR;         // colour-1 chunks
  constexpr int NWI = (NW + NT - 1) / NT;
  constexpr int ROWS = 2 * TR + 6;
  extern __shared__ __align__(128) uint8_t smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  uint8_t* Ws = smem + 128;
  uint8_t* Bs = Ws + (TR + 4) * PITCH;
  const int tid = threadIdx.x;
  const int L = P.L, h = P.h;
  const size_t plane = (size_t)L * h;
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t phase = 0;
  for (int tile = blockIdx.x; tile < P.n_tiles; tile += gridDim.x) {
    const int r0 = (tile / P.tiles_x) * TR, k0 = (tile % P.tiles_x) * TC;
    if (tid < 32) {
      if (tid == 0) {
        fence_proxy_async();
        mbar_expect_tx(bar, (uint32_t)(ROWS * PITCH));
      }
      __syncwarp();
      for (int r = tid; r < ROWS; r += 32) {
        if (r < TR + 4) {
          const int g = (r0 - 2 + r) & (L - 1);
          stage_row(Ws + r * PITCH, in + plane + (size_t)g * h, h, k0, PITCH, bar);
        } else {
          const int g = (r0 - 1 + r - (TR + 4)) & (L - 1);
          stage_row(Bs + (r - (TR + 4)) * PITCH, in + (size_t)g * h, h, k0, PITCH, bar);
        }
      }
    }
    bool ok = false;
    for (uint32_t it = 0; it < (1u << 24) && !ok; ++it) ok = mbar_try_wait(bar, phase);
    phase ^= 1u;

    // ---- colour 0: rows r0-1 .. r0+TR, all staged chunks
    uint32_t tm[NBI];
#pragma unroll
    for (int i = 0; i < NBI; ++i) {
      const int task = tid + i * NT;
      tm[i] = 0;
      if (ok && (NB % NT == 0 || task < NB)) {
        const int y = task / CPA, zc = task - (task / CPA) * CPA, z0 = zc * 16;
        const int gr = (r0 - 1 + y) & (L - 1);
        int gk = k0 - 16 + z0;
        gk += gk < 0 ? h : 0;
        gk -= gk >= h ? h : 0;
        uint8_t* tp = Bs + y * PITCH + z0;
        const uint8_t* mid = Ws + (y + 1) * PITCH;
        const uint4 T = lds128(tp), U = lds128(Ws + y * PITCH + z0), D = lds128(Ws + (y + 2) * PITCH + z0);
        const uint4 Mw = lds128(mid + z0);
        const uint32_t prv = zc > 0 ? lds32(mid + z0 - 4) : 0u;
        const uint32_t nxt = zc < CPA - 1 ? lds32(mid + z0 + 16) : 0u;
        const uint4 R = stream_block(P.key, P.rep, P_SWEEP_HI, 0u, (uint32_t)gr, (uint32_t)(gk >> 4), tt);
        uint32_t tw[4] = {T.x, T.y, T.z, T.w};
        tm[i] = update16(tw, U, D, Mw, prv, nxt, (uint32_t)(gr & 1), R, P.acc);
        *reinterpret_cast<uint4*>(tp) = make_uint4(tw[0], tw[1], tw[2], tw[3]);
      }
    }
#pragma unroll
    for (int i = 0; i < NBI; ++i) {
      uint32_t bits = tm[i];
      if (!bits) continue;
      const int task = tid + i * NT;
      const int y = task / CPA, z0 = (task - y * CPA) * 16;
      const int gr = (r0 - 1 + y) & (L - 1);
      const int q = gr & 1;
      while (bits) {
        const int p = __ffs(bits) - 1;
        bits &= bits - 1;
        const int z = z0 + 4 * (7 - (p & 7)) + (p >> 3);
        const int zl = max(z - 1 + q, 0), zr = min(z + q, PITCH - 1);
        int gk = k0 - 16 + z;
        gk += gk < 0 ? h : 0;
        gk -= gk >= h ? h : 0;
        uint8_t* sp = Bs + y * PITCH + z;
        if (resolve_open(*sp, Ws[y * PITCH + z], Ws[(y + 2) * PITCH + z], Ws[(y + 1) * PITCH + zl],
                         Ws[(y + 1) * PITCH + zr], P, 0u, gr, gk, tt))
          *sp ^= 1u;
      }
    }
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(status, 1);
      return;
    }

    // ---- colour 1: tile rows and columns; colour-0 tile rows are final now
    uint32_t tmw[NWI];
#pragma unroll
    for (int i = 0; i < NWI; ++i) {
      const int task = tid + i * NT;
      tmw[i] = 0;
      if (NW % NT == 0 || task < NW) {
        const int xr = task / CPR, zc = 1 + task - (task / CPR) * CPR, z0 = zc * 16, x = xr + 2;
        const int gr = r0 + xr, gk = k0 + 16 * (zc - 1);
        const uint8_t* mid = Bs + (x - 1) * PITCH;
        const uint4 T = lds128(Ws + x * PITCH + z0), U = lds128(Bs + (x - 2) * PITCH + z0);
        const uint4 D = lds128(Bs + x * PITCH + z0), Mw = lds128(mid + z0);
        const uint32_t prv = lds32(mid + z0 - 4), nxt = lds32(mid + z0 + 16);
        *reinterpret_cast<uint4*>(out + (size_t)gr * h + gk) = Mw;  // final colour-0 chunk of this row
        const uint4 R = stream_block(P.key, P.rep, P_SWEEP_HI, 1u, (uint32_t)gr, (uint32_t)(gk >> 4), tt);
        uint32_t tw[4] = {T.x, T.y, T.z, T.w};
        tmw[i] = update16(tw, U, D, Mw, prv, nxt, (uint32_t)((gr + 1) & 1), R, P.acc);
        const uint4 nv = make_uint4(tw[0], tw[1], tw[2], tw[3]);
        if (tmw[i] == 0) *reinterpret_cast<uint4*>(out + plane + (size_t)gr * h + gk) = nv;
        else *reinterpret_cast<uint4*>(Ws + x * PITCH + z0) = nv;
      }
    }
#pragma unroll
    for (int i = 0; i < NWI; ++i) {
      uint32_t bits = tmw[i];
      if (!bits) continue;
      const int task = tid + i * NT;
      const int xr = task / CPR, zc = 1 + task - xr * CPR, z0 = zc * 16, x = xr + 2;
      const int gr = r0 + xr, gk0 = k0 + 16 * (zc - 1);
      const int q = (gr + 1) & 1;
      while (bits) {
        const int p = __ffs(bits) - 1;
        bits &= bits - 1;
        const int zo = 4 * (7 - (p & 7)) + (p >> 3), z = z0 + zo;
        uint8_t* sp = Ws + x * PITCH + z;
        if (resolve_open(*sp, Bs[(x - 2) * PITCH + z], Bs[x * PITCH + z], Bs[(x - 1) * PITCH + z - 1 + q],
                         Bs[(x - 1) * PITCH + z + q], P, 1u, gr, gk0 + zo, tt))
          *sp ^= 1u;
      }
      *reinterpret_cast<uint4*>(out + plane + (size_t)gr * h + gk0) = lds128(Ws + x * PITCH + z0);
    }
    __syncthreads();
  }
}

template <int TR, int TC>
constexpr size_t sweep_smem_bytes() {
  return 128 + (size_t)(2 * TR + 6) * (TC + 32);
}

}  // namespace tiled
}  // namespace mcrg
