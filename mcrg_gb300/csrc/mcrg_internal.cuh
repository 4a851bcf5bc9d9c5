// mcrg_internal.cuh -- job descriptors and launchers shared by the CUDA
// translation units of libmcrg.  Not part of the public ABI.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mcrg.h"
#include "mcrg_device.cuh"

namespace mcrg {

// One independent Markov chain run shared-memory resident by one CTA.
struct ChainJob {
  int32_t L, n_levels, C, threads;
  Key key;
  uint32_t replica;
  uint32_t t0;        // Philox time of the first sweep
  uint32_t n0;        // Philox time (sample index) of the first measurement
  uint32_t init;      // 1: draw the initial coin; 0: load `state`
  uint32_t store;     // 1: write the final configuration back to `state`
  int64_t n_eq, n_samples, sweeps_between, bin_size;
  uint8_t* state;     // L*L bytes: colour-0 array then colour-1 array
  mcrg_moments* bins; // ceil(n_samples / bin_size) outputs, zeroed by the host
  Accept acc;
  int32_t flow;       // 1: flow moments (sum S_l and S_l * S_0 of coupling 0) instead of the T-matrix moments
  int32_t pad;
};

// Shared-memory plan of a resident lattice, its blocked levels and (when
// C > 0) the moment accumulators of one chain.
struct SmemPlan {
  int off[MCRG_MAX_LEVELS + 2];
  int s_off;    // int32 S[(MCRG_MAX_LEVELS+1) * MCRG_MAX_COUPLINGS]
  int tab_off;  // int2 per moment entry: (x | y << 16, output index)
  int acc_off;  // int64 per moment entry
  int scr_off;  // uint32 open-site scratch: 64 per warp, up to 8 warps
  int E;        // moment entries of the T-matrix moments
  int Ecap;     // entries the table holds (also fits the 2 (n_levels + 1) flow moments)
  int pl_off;   // L >= 64: plane words of level 0 (2 L^2 / 64 uint32), then qn[2] and the open-word queue
  int q_off;    // uint4 queue entries (resident::queue_cap(L))
  int bytes;
};

__host__ __device__ inline SmemPlan make_plan(int L, int n_levels, int C = 0) {
  SmemPlan p;
  int off = 0, n = L;
  for (int l = 0; l <= n_levels; ++l, n >>= 1) {
    p.off[l] = off;
    off += ((n * n + 15) / 16) * 16;
  }
  p.s_off = off;
  off += ((MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS * 4 + 15) / 16 * 16;
  p.E = C > 0 ? (n_levels + 1) * C + 2 * n_levels * C * C : 0;
  p.Ecap = C > 0 ? (p.E > 2 * (n_levels + 1) ? p.E : 2 * (n_levels + 1)) : 0;
  p.tab_off = off;
  off += ((p.Ecap * 8 + 15) / 16) * 16;
  p.acc_off = off;
  off += p.Ecap * 8;
  p.scr_off = off;
  off += 8 * 64 * 4;
  p.pl_off = p.q_off = -1;
  if (L >= 64) {  // bit-sliced sweeps (mcrg_resident_bits.cuh)
    off = (off + 15) / 16 * 16;
    p.pl_off = off;
    off += 2 * (L * L / 64) * 4 + 16;  // planes + qn[2] (padded)
    p.q_off = off;
    off += (L * L / 256 > 32 ? L * L / 256 : 32) * 16;
  }
  p.bytes = (off + 15) / 16 * 16;
  return p;
}

inline int moment_entries(int n_levels, int C) { return (n_levels + 1) * C + 2 * n_levels * C * C; }

// Host: acceptance parameters for coupling K (FP64, see include/mcrg.h).
Accept make_accept(double K);

// Launch `n_jobs` chains (all with the same L and threads; n_levels and C
// bound the shared memory of every job).
cudaError_t launch_chain(const ChainJob* d_jobs, int n_jobs, int L, int n_levels, int C, int threads,
                         cudaStream_t stream);

// Stateless helpers on a device lattice in split layout (used by
// mcrg_block_lattice / mcrg_lattice_couplings and the HBM path's tail).
cudaError_t launch_block_once(const uint8_t* d_in, int N, uint8_t* d_out, const uint8_t* d_tie_nat,
                              Key key, uint32_t replica, int level, uint32_t sample, cudaStream_t s);
cudaError_t launch_couplings_once(const uint8_t* d_in, int N, int C, int* d_out, cudaStream_t s);

// New chain on an HBM-resident context without allocating (mcrg_capi.cu).
int reinit_context(mcrg_ctx* c, double K, uint64_t seed, uint32_t replica);

// Forward pass of the RG neural network (src/rgnn.cpp:281-307) on a split
// layout lattice of side n: the scalar output into *d_out (device), using
// `work` ((n/32)^2 + (n/1024)^2 + 2 doubles, not overlapping d_out).
cudaError_t launch_rgnn_scalar(const uint8_t* d_split, int n, const double W[4], double* work, double* d_out,
                               cudaStream_t s);

}  // namespace mcrg
