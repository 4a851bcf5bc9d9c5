// mcrg_tiled.cuh -- HBM-resident lattices (MCRG_SMEM_MAX_L < L <= MCRG_MAX_L).
#pragma once
#include "mcrg_internal.cuh"

namespace mcrg {

struct TiledLattice {
  int L = 0, nl = 0, C = 0;
  Key key{0, 0};
  uint32_t replica = 0;
  Accept acc{};
  uint8_t* buf[2] = {nullptr, nullptr};  // ping-pong level-0 configurations
  int cur = 0;
  uint8_t* levels = nullptr;             // blocked levels 1..n_hbm (HBM-resident sizes) + tail level
  size_t level_off[MCRG_MAX_LEVELS + 2] = {};
  int n_hbm = 0;                          // levels 0..n_hbm-1 are measured from HBM; level n_hbm by the tail CTA
  unsigned long long* d_S = nullptr;      // per-sample coupling sums [(nl+1)*5] (int64)
  int* d_status = nullptr;                // kernel error flags
  mcrg_moments* d_bins = nullptr;
  int64_t bins_cap = 0;
  int variant = -1;                       // sweep variant picked by the autotuner
  int sms = 0;                            // multiprocessors of the lattice's device
  DevSpan* span = nullptr;                // where the buffers come from (nullptr: cudaMalloc)
};

int tiled_alloc(TiledLattice* t, int L, int nl, int C, Key key, uint32_t replica, const Accept& acc,
                cudaStream_t s);
void tiled_free(TiledLattice* t);
// New chain on an allocated lattice: new key, replica and acceptance, fresh
// initial coin, the autotuned sweep variant kept (no allocation).
int tiled_reinit(TiledLattice* t, Key key, uint32_t replica, const Accept& acc, cudaStream_t s);
uint8_t* tiled_state(TiledLattice* t);
// n sweeps starting at sweep index t0 (one fused two-colour pass per sweep).
int tiled_sweeps(TiledLattice* t, uint32_t t0, int64_t n, cudaStream_t s);
// n_samples x (sweeps_between sweeps + measurement); bins of bin_size samples.
// flow: accumulate the flow moments (sum S_l in S[l*5], sum S_l S_0 in
// SbSb[l*25], coupling 0) instead of the T-matrix moments.
int tiled_measure(TiledLattice* t, uint32_t t0, uint32_t n0, int64_t n_samples, int64_t sweeps_between,
                  int64_t bin_size, int64_t* n_bins, cudaStream_t s, bool flow = false);
mcrg_moments* tiled_bins(TiledLattice* t);
// One measurement of the current configuration (no sweeps) at tie-stream
// sample index `sample`, added into *bin (device; n_samples counts it).
int tiled_measure_sample(TiledLattice* t, uint32_t sample, mcrg_moments* bin, cudaStream_t s);
// Sweep schedule in use (after the first sweep): rows per pipeline group
// and threads per CTA; returns the variant index.
int tiled_variant(TiledLattice* t, int* rows, int* threads);
// Drains the stream and returns the sweep kernel's error flags since the
// last call (1 = a bulk copy did not land within the bounded wait), clearing
// them; -1 when the stream itself failed.
int tiled_status(TiledLattice* t, cudaStream_t s);

}  // namespace mcrg
