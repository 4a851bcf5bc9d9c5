/*
 * mcrg.h -- C ABI of the GB300-native MCRG hot path (libmcrg.so).
 *
 * Drop-in boundary for kim-jane/MCRG.  The reference has no FFI: its hot path
 * is the C++ classes Lattice (src/lattice.hpp:5-37), IsingModel
 * (src/ising.hpp:8-41) and MonteCarloRenormalizationGroup (src/mcrg.hpp:6-40),
 * called from src/main.cpp:15-17 and src/rgnn.cpp:85-123.  Each entry point
 * below names the reference interface it replaces.
 *
 * Conventions
 *   - Every function returns 0 (MCRG_OK) or a negative errno-style code;
 *     mcrg_strerror() names it.  No C++ exception crosses this ABI.
 *   - A context owns its device memory and one CUDA stream; the caller owns
 *     every host buffer.  Use one context per host thread.  mcrg_submit /
 *     mcrg_poll / mcrg_wait of a server are thread-safe.
 *   - Host lattices are int8 +-1, row-major: site (i, j) at i*L + j, i being
 *     the first index of the reference's Lattice::spins_(i, j).
 *   - Weight exp(-K sum_bonds s s); K < 0 is ferromagnetic (src/ising.cpp:9).
 *
 * Monte Carlo update.  The reference grows one Wolff cluster per sample
 * (src/ising.cpp:87-149).  Here one "sweep" updates every site once with a
 * checkerboard Metropolis rule (mcrg_cluster_update / mcrg_measure_cluster
 * and mcrg_request.flags give the reference's own cluster rule instead): flip iff always[m] or u32 < thr[m], where
 * m = number of anti-aligned neighbours, p[m] = min(1, exp(2K(4-2m))),
 * always[m] = (p[m] == 1), thr[m] = floor(p[m] 2^32).  Both chains sample the
 * same Boltzmann distribution.
 *
 * Random streams: Philox4x32-10, key = (seed lo32, seed hi32), counter =
 * (row, purpose<<28 | sub<<20 | group, time, replica):
 *   init   purpose 1, sub = colour, group = k>>7, time 0:
 *          spin bit = bit (k&127) of the 128-bit block;
 *   sweep  purpose 2, sub = colour, time = sweep index t; the 8-bit draw r8:
 *          L <= 32: group = k>>4, r8 = byte (k&15);
 *          L >= 64: groups 2w, 2w+1 with w = k>>5 give eight
 *            plane words W0..W7; bit 7-q of r8 is bit 8*(p&3)+(p>>2) of Wq,
 *            p = k&31;
 *          purpose 3, group = k>>2: r24 = low 24 bits of word (k&3);
 *          u32 = r8<<24 | r24;
 *   ties   purpose 4, sub = level produced, row = ib, group = jb>>7,
 *          time = sample index: tie value = bit (jb&127) ? +1 : -1.
 *   bonds  purpose 5 (cluster updates), row = i, group = j>>1, time = update
 *          index t: the bond of site (i, j) to (i, j+1) draws word 2*(j&1),
 *          the bond to (i+1, j) word 2*(j&1)+1; a bond is open iff both
 *          spins are equal and the word is below floor((1 - exp(2K)) 2^32);
 *   cluster purpose 6, time = t: Wolff seed site i*L + j = word 0 of block
 *          (row 0, sub 0, group 0) mod L^2; Swendsen-Wang flips the
 *          cluster whose smallest site index is r iff bit 0 of word 0 of
 *          block (row r>>16, sub 1, group r & 0xFFFF) is set.
 * Site (i, j) has colour c = (i+j)&1 and split index k = j>>1.  Colour 0 is
 * updated before colour 1 within a sweep.
 *
 * Coupling sums (per level, over directional offsets, periodic):
 *   0 nn    sum_x s(x) sum_{(+-1,0),(0,+-1)} s(x+d)   (src/lattice.cpp:102-120)
 *   1 nnn   sum_x s(x) sum_{(+-1,+-1)} s(x+d)         (src/lattice.cpp:102-120)
 *   2 third sum_x s(x) sum_{(+-2,0),(0,+-2)} s(x+d)   (no reference counterpart)
 *   3 plaq  sum_x s(i,j)s(i+1,j)s(i,j+1)s(i+1,j+1)     (no reference counterpart)
 *   4 line4 sum_x s(i,j)..s(i+3,j) + s(i,j)..s(i,j+3)  (no reference counterpart)
 * Blocking is b = 2 majority rule (src/mcrg.cpp:314-348).
 */
#ifndef MCRG_H_
#define MCRG_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCRG_ABI_VERSION 1
#define MCRG_MAX_LEVELS 14     /* L <= 32768 */
#define MCRG_MAX_COUPLINGS 5
#define MCRG_MAX_L 16384
#define MCRG_SMEM_MAX_L 256    /* lattices up to this side run shared-memory resident */
#define MCRG_RESIDENT_MAX_L 1024 /* batched / served chains in the fast acceptance regime run
                                    shared-memory resident up to this side (bit-plane levels) */

enum {
  MCRG_OK = 0,
  MCRG_ENOENT = -2,      /* unknown ticket */
  MCRG_EIO = -5,         /* CUDA error */
  MCRG_EAGAIN = -11,     /* not finished yet */
  MCRG_ENOMEM = -12,     /* device or host allocation failed */
  MCRG_EBUSY = -16,      /* server queue full */
  MCRG_EINVAL = -22,     /* bad argument */
  MCRG_ENOSPC = -28,     /* request exceeds the memory budget */
  MCRG_ENOSYS = -38,     /* operation not supported for this configuration */
  MCRG_ETIMEDOUT = -110, /* bounded wait ran out */
  MCRG_ECANCELED = -125  /* request cancelled / server shut down */
};

typedef struct {
  uint64_t lo;
  int64_t hi;
} mcrg_i128;

/* Lattice(N) + IsingModel(K) + MonteCarloRenormalizationGroup(b) parameters. */
typedef struct {
  int32_t L;           /* lattice side N, power of two, 4..MCRG_MAX_L */
  int32_t b;           /* block factor; 2 is the only supported value */
  int32_t n_levels;    /* RG levels; < 0 selects log2(L)-1 (src/mcrg.cpp:43) */
  int32_t n_couplings; /* 1..5; 2 = the reference's {nn, nnn} */
  double K;            /* coupling */
  uint64_t seed;       /* Philox key */
  uint32_t replica;    /* Philox counter word 3: independent chains */
  int32_t device;      /* CUDA device ordinal */
} mcrg_cfg;

/* Moment sums of src/mcrg.cpp:56-98 (exact integers, not averages):
 *   S[l*MAX_C + c]             = sum_samples S_l,c
 *   SbS[(l*MAX_C + a)*MAX_C + b]  = sum S_{l+1},a * S_l,b      (l < n_levels)
 *   SbSb[(l*MAX_C + a)*MAX_C + b] = sum S_{l+1},a * S_{l+1},b
 * The reference flattens the same products column-major (a + b*C). */
typedef struct {
  int32_t n_levels;
  int32_t n_couplings;
  int64_t n_samples;
  int64_t S[(MCRG_MAX_LEVELS + 1) * MCRG_MAX_COUPLINGS];
  mcrg_i128 SbS[MCRG_MAX_LEVELS * MCRG_MAX_COUPLINGS * MCRG_MAX_COUPLINGS];
  mcrg_i128 SbSb[MCRG_MAX_LEVELS * MCRG_MAX_COUPLINGS * MCRG_MAX_COUPLINGS];
} mcrg_moments;

/* Renormalisation-flow moments of one chain (coupling 0, nearest
 * neighbours): S[l] = sum over samples of S_nn at level l, S0S[l] = sum of
 * S_nn(level l) * S_nn(level 0), for l = 0 .. n_levels.  They are the sums of
 * the sample loop of approx_critical_point (src/mcrg.cpp:225-258): for the
 * lattice of side L, SL = S[0], SLb(n) = S[n+1], SLb*SL = S0S[n+1]; for the
 * lattice of side L/b, SS = S[0], SSb(n) = S[n], SSb*SS = S0S[n]. */
typedef struct {
  int32_t n_levels;
  int32_t pad;
  int64_t n_samples;
  int64_t S[MCRG_MAX_LEVELS + 1];
  mcrg_i128 S0S[MCRG_MAX_LEVELS + 1];
} mcrg_flow_moments;

typedef struct mcrg_ctx mcrg_ctx;

const char* mcrg_strerror(int code);
int mcrg_abi_version(void);

/* Acceptance table the sweep kernels use (host FP64, as described above). */
int mcrg_thresholds(double K, uint32_t thr[5], uint8_t always[5]);

/* Replaces `new Lattice(N)` + `new IsingModel(K)` (src/lattice.cpp:3-15,
 * src/ising.cpp:3-11): allocates the device lattice and draws the initial
 * +-1 coin from the init stream (src/lattice.cpp:33-41). */
int mcrg_alloc(mcrg_ctx** out, const mcrg_cfg* cfg);
int mcrg_free(mcrg_ctx* ctx);

/* Replaces writes / reads of the public Lattice::spins_ (src/lattice.hpp:16;
 * read directly by src/rgnn.cpp:113-114,175).  Values must be +-1.
 * mcrg_set_spins reads a page-locked, 16-byte-aligned host buffer (L >= 32)
 * in place with the layout-conversion kernel over the host link; other
 * buffers go through a staging copy.  mcrg_get_spins converts on the device
 * and copies the rows out with one transfer (at host-link speed when the
 * buffer is page-locked).  Both return after the transfer completed. */
int mcrg_set_spins(mcrg_ctx* ctx, const int8_t* host_spins);
int mcrg_get_spins(mcrg_ctx* ctx, int8_t* host_spins);

/* Replaces n_sweeps calls of IsingModel::sample_new_configuration
 * (src/ising.cpp:87-93) and IsingModel::equilibrate(lat, n, false)
 * (src/ising.cpp:14-84). */
int mcrg_sweep(mcrg_ctx* ctx, int64_t n_sweeps);

/* Replaces `level` chained calls of block_spin_transformation
 * (src/mcrg.cpp:314-348) on the current configuration; ties come from the
 * tie stream at the context's next sample index, which is consumed.  Copies
 * the (L>>level)^2 result to host_out when it is not NULL. */
int mcrg_block(mcrg_ctx* ctx, int level, int8_t* host_out);

/* Replaces Lattice::calc_interactions at every level (src/lattice.cpp:102-120,
 * src/mcrg.cpp:78-84) for the current configuration: out[l*n_couplings + c].
 * Consumes one sample index for the tie stream. */
int mcrg_interactions(mcrg_ctx* ctx, int64_t* out);

/* Replaces the sample loop of calc_critical_exponent (src/mcrg.cpp:72-98):
 * n_samples x (sweeps_between sweeps, then blocking + coupling sums at every
 * level + moment accumulation), all on the device.  `total` receives the
 * moment sums over all samples.  When bins != NULL and bin_size > 0, bins[q]
 * receives the sums over samples [q*bin_size, (q+1)*bin_size) for
 * q < n_bins_cap (binned error bars). */
int mcrg_measure(mcrg_ctx* ctx, int64_t n_samples, int64_t sweeps_between, mcrg_moments* total,
                 int64_t bin_size, mcrg_moments* bins, int64_t n_bins_cap);

/* Replaces RenormalizationGroupNeuralNetwork::scalar_output(spins_)
 * (src/rgnn.cpp:281-307) on the current configuration, on the device: the 2x2
 * filter out(i, j) = || W * block(2i, 2j, 2, 2) ||_1 applied until one value
 * remains, W(r, k) = W[2r + k], FP64 in the reference's order of operations
 * (same result bit for bit).  Does not move the chain or its counters, and
 * spares the spins_ copy the reference's RGNN reads (src/rgnn.cpp:113-114). */
int mcrg_rgnn_scalar_output(mcrg_ctx* ctx, const double W[4], double* out);

/* Replaces the sample loop of approx_critical_point (src/mcrg.cpp:225-258)
 * for one of its two lattices: n_samples x (sweeps_between sweeps, then the
 * nearest-neighbour sums of every level and their products with level 0),
 * on the device, exactly in integers.  The host matching step
 * (src/mcrg.cpp:283-301) combines the moments of a context of side L and one
 * of side L/b at the same K. */
int mcrg_measure_flow(mcrg_ctx* ctx, int64_t n_samples, int64_t sweeps_between, mcrg_flow_moments* out);

/* Cluster updates on the device: the reference's own update rule
 * (IsingModel::sample_new_configuration, src/ising.cpp:87-155: one Wolff
 * cluster grown from a random site through aligned nearest neighbours, each
 * bond open with probability 1 - exp(2K) (src/ising.cpp:9), then flipped) and
 * its all-cluster form (Swendsen-Wang: every cluster of the same bond
 * configuration flipped with probability 1/2).  A Wolff cluster is the
 * connected component of the seed under open bonds, so it is labelled
 * order-independently (union-find) from per-bond draws of the stream above.
 * Each update consumes one sweep index (the time word t); *flipped (may be
 * NULL) receives the number of spins flipped over the n updates (for Wolff,
 * the summed cluster sizes).  kind: MCRG_UPDATE_WOLFF or
 * MCRG_UPDATE_SWENDSEN_WANG.  The first call allocates 4 L^2 bytes of
 * labels for the context. */
enum { MCRG_UPDATE_WOLFF = 1, MCRG_UPDATE_SWENDSEN_WANG = 2 };
int mcrg_cluster_update(mcrg_ctx* ctx, int64_t n, int32_t kind, int64_t* flipped);

/* mcrg_measure with cluster updates in place of sweeps: n_samples x
 * (updates_between cluster updates of the given kind, then blocking + coupling
 * sums at every level + moment accumulation) -- the sample loop of
 * calc_critical_exponent (src/mcrg.cpp:72-98) with the reference's update
 * rule. */
int mcrg_measure_cluster(mcrg_ctx* ctx, int64_t n_samples, int64_t updates_between, int32_t kind,
                         mcrg_moments* total, int64_t bin_size, mcrg_moments* bins, int64_t n_bins_cap);

/* Sweep and sample counters (the Philox time words of the next sweep / sample). */
int mcrg_counters(mcrg_ctx* ctx, uint64_t* sweeps, uint64_t* samples);
/* Sets them: with mcrg_set_spins, a context of the same mcrg_cfg resumes a
 * saved chain (mcrg_get_spins + mcrg_counters) exactly, draw for draw.  The
 * reference has no checkpoint (its only persistence is the final spin dump of
 * Lattice::write_spins, src/lattice.cpp:63-75). */
int mcrg_set_counters(mcrg_ctx* ctx, uint64_t sweeps, uint64_t samples);
/* Sweep schedule the autotuner picked for an HBM-resident context: rows per
 * pipeline group (tile_rows) and threads per CTA (tile_cols); MCRG_EINVAL
 * for shared-memory-resident contexts and MCRG_EAGAIN before the first
 * sweep.  No counterpart in the reference. */
int mcrg_tile_shape(mcrg_ctx* ctx, int32_t* tile_rows, int32_t* tile_cols);
/* The context's CUDA stream (cudaStream_t), for event timing. */
int mcrg_stream(mcrg_ctx* ctx, void** stream);
/* Drains the context's stream.  Like every entry point that returns results
 * (mcrg_get_spins, mcrg_block, mcrg_interactions, mcrg_measure*), it returns
 * MCRG_ETIMEDOUT when an HBM sweep since the last such call gave up waiting
 * for a bulk copy of its band (bounded wait of 1 s; the lattice is then not
 * a valid chain state), and clears that flag. */
int mcrg_sync(mcrg_ctx* ctx);

/* Self-test of the bounded device waits, without a fault: one kernel on
 * `device` waits with the library's bounded wait on a barrier that nothing
 * completes, for limit_us (1 .. 1e6) microseconds.  Returns MCRG_OK when the
 * kernel ran and the device stays usable, with *status = MCRG_ETIMEDOUT (the
 * wait ran out and raised the error flag, the expected outcome) and
 * *waited_s = the device time the wait took.  No counterpart in the
 * reference. */
int mcrg_selftest_wait(int32_t device, int64_t limit_us, int32_t* status, double* waited_s);

/* Stateless device forms of block_spin_transformation (src/mcrg.cpp:314-348)
 * and calc_interactions (src/lattice.cpp:102-120) on a host lattice.
 * tie_values (N/2 x N/2, +-1) gives the value of every tied block; NULL uses
 * the tie stream (seed, replica, level, sample). */
int mcrg_block_lattice(int32_t N, const int8_t* host_in, const int8_t* tie_values, uint64_t seed,
                       uint32_t replica, int32_t level, uint32_t sample, int8_t* host_out, int32_t device);
int mcrg_lattice_couplings(int32_t N, const int8_t* host_in, int32_t n_couplings, int64_t* out,
                           int32_t device);

/* Same result as mcrg_lattice_couplings, for callers that must not allocate
 * device memory while they run (a program that has given the rest of the GPU
 * to its own memory pool or works under a fixed budget, where a cudaMalloc
 * can fail, or one that cannot accept the device-wide synchronisation that
 * cudaMalloc / cudaFree may cause).  It allocates nothing: the device-side
 * working copy lives in a fixed scratch array that is part of libmcrg.so and
 * stays reserved on every GPU that loads the library until the process ends
 * (2 * MCRG_NOALLOC_MAX_L^2 + 256 bytes).  N above MCRG_NOALLOC_MAX_L is
 * rejected with MCRG_ENOSPC.  The first call on a device sets it up: it
 * looks the array's address up for that device and creates the one
 * non-blocking stream all calls on the device use (so a call neither uses the
 * legacy default stream nor waits for the caller's streams); make that first
 * call before any stream capture.  All calls share the array and it keeps
 * the last call's data; the sums are cleared at the start of each call.
 * Calls on one device are serialised by a lock inside the library, held until
 * the call's device work is done; device work that overlaps with a call in
 * any other way races on the array.  No counterpart in the reference. */
#define MCRG_NOALLOC_MAX_L 1024
int mcrg_lattice_couplings_noalloc(int32_t N, const int8_t* host_in, int32_t n_couplings, int64_t* out,
                                   int32_t device);

/* ---------------------------------------------------------------------- */
/* Batched solves: many independent chains (the reference runs one chain   */
/* per MPI rank and sums with MPI_Allreduce, src/mcrg.cpp:101-103).         */
/* ---------------------------------------------------------------------- */
typedef struct {
  int32_t L;
  int32_t n_levels;    /* < 0: log2(L)-1 */
  int32_t n_couplings;
  int32_t flags;       /* update rule: 0 = checkerboard sweeps, MCRG_UPDATE_WOLFF or
                          MCRG_UPDATE_SWENDSEN_WANG = cluster updates (n_eq and sweeps_between
                          then count cluster updates); cluster requests up to L = 256 run as
                          resident chains */
  double K;
  uint64_t seed;
  uint32_t replica;
  uint32_t pad;
  int64_t n_eq;        /* thermalisation sweeps */
  int64_t n_samples;   /* measurements */
  int64_t sweeps_between;
} mcrg_request;

typedef struct {
  int32_t status;      /* MCRG_OK or an error code */
  int32_t pad;
  double submit_s;     /* host clock (CLOCK_MONOTONIC seconds) at submission */
  double done_s;       /* host clock when the result was observed complete */
  mcrg_moments moments;
} mcrg_result;

/* Runs a batch of independent chains on `device` and fills results[i]
 * (the GPU form of the reference's one chain per MPI rank + MPI_Allreduce,
 * src/mcrg.cpp:42,101-103).  Every request that fits a shared-memory-
 * resident chain (fast acceptance regime up to MCRG_RESIDENT_MAX_L; other K
 * up to MCRG_SMEM_MAX_L; cluster updates up to 256) runs in ONE persistent
 * launch: the chains are grouped into packs (one chain per warp-aligned
 * group of a CTA's threads), ordered longest first, and the CTAs take packs
 * from a queue until it is empty.  The threads per chain of each shape
 * (side, chain form, levels, couplings) are picked once per process by the
 * schedule autotuner from timed trial launches (mcrg_batch_schedule); for
 * resident sides above MCRG_SMEM_MAX_L it also times the tiled HBM path and
 * runs those requests there when that ends sooner.  With `use_graph` != 0
 * the upload, clear, launch and download are one CUDA graph, instantiated
 * once per device, CTA width, grid and buffer set and re-launched with
 * updated copy sizes.  Requests that no chain holds run on the tiled HBM
 * path after the resident launch.  The packs are queued by chain code (byte
 * sweeps, plane sweeps, cluster updates) and each SM serves first the code
 * its share of SM ids was given (shares by estimated work), so that the CTAs
 * of one SM share their instructions in cache.  Environment:
 * MCRG_POOL_THREADS=<n> forces n threads per chain where n is a candidate;
 * MCRG_BATCH_SCHEDULE=resident | tiled forces the choice for the largest
 * resident sides; MCRG_POOL_CLASSES=0 puts every pack in one queue. */
int mcrg_batch_run(const mcrg_request* reqs, int32_t n, mcrg_result* results, int32_t device,
                   int32_t use_graph);

/* The schedule the autotuner picked (tuning it now if needed) for chains of
 * the request's shape: threads per chain, seconds per sample of one chain in
 * a full wave of the trial, and seconds per sample of the tiled HBM path
 * (-1 when not timed).  MCRG_ENOSYS when the request has no resident form.
 * No counterpart in the reference. */
int mcrg_batch_schedule(const mcrg_request* r, int32_t device, int32_t* threads, double* s_sample,
                        double* s_tiled);
/* Persistent batch launches and CUDA graph instantiations so far on a
 * device.  No counterpart in the reference. */
int mcrg_batch_stats(int32_t device, int64_t* launches, int64_t* graph_builds);

/* ---------------------------------------------------------------------- */
/* Serving: continuous batching of MCRG requests.                          */
/* ---------------------------------------------------------------------- */
/* A server admits requests in arrival order as slots and memory free up and
 * runs them while others run.  Requests that fit a shared-memory-resident
 * chain go, packed by shape, into a ring in page-locked host memory that a
 * device-resident loop of persistent CTAs drains (one CTA per SM, relaunched
 * when it has gone idle for 20 ms); their moments are written straight to
 * page-locked host memory.  The others run on host worker threads, each on a
 * context built inside the request's share of the arena.  The arena of
 * hbm_budget_bytes is allocated once at creation and is all the device
 * memory the server uses for requests: a request is charged every device
 * byte it holds (the final configuration of a resident chain, the whole
 * context of an HBM-path request), and waits while the budget is spent.  A
 * result depends only on its request's seed and replica, never on what ran
 * beside it.  No counterpart in the reference (it runs one chain per MPI
 * rank, src/mcrg.cpp:42). */
typedef struct {
  int32_t device;
  int32_t slots;            /* resident chains admitted at a time (host result slots) */
  int64_t hbm_budget_bytes; /* device bytes the server may hold for requests (one arena) */
  int32_t queue_capacity;   /* pending requests before mcrg_submit returns EBUSY */
  int32_t hbm_workers;      /* host threads running requests no resident chain holds (L > 1024, or
                               other acceptance regimes above MCRG_SMEM_MAX_L) concurrently;
                               0 selects 16, at most 256 */
} mcrg_server_cfg;

typedef struct mcrg_server mcrg_server;

int mcrg_server_create(mcrg_server** out, const mcrg_server_cfg* cfg);
int mcrg_submit(mcrg_server* srv, const mcrg_request* req, uint64_t* ticket);
int mcrg_poll(mcrg_server* srv, uint64_t ticket, mcrg_result* out);   /* MCRG_EAGAIN while running */
/* Withdraws a request that is still queued: its result (mcrg_poll / mcrg_wait)
 * has status MCRG_ECANCELED.  MCRG_EBUSY once it is admitted (its chain runs
 * to the end), MCRG_EINVAL when it has finished, MCRG_ENOENT for an unknown
 * ticket.  No counterpart in the reference. */
int mcrg_cancel(mcrg_server* srv, uint64_t ticket);
int mcrg_wait(mcrg_server* srv, uint64_t ticket, double timeout_s, mcrg_result* out);
int mcrg_server_stats(mcrg_server* srv, int64_t* admitted, int64_t* completed, int64_t* in_flight,
                      int64_t* bytes_in_use);
/* The device-resident request loop: how many times the server launched it
 * (it runs until no request has arrived for 20 ms) and how many packs of
 * requests it published to it.  No counterpart in the reference. */
int mcrg_server_loop_stats(mcrg_server* srv, int64_t* loop_launches, int64_t* entries_published);
int mcrg_server_destroy(mcrg_server* srv);

#ifdef __cplusplus
}
#endif
#endif /* MCRG_H_ */
