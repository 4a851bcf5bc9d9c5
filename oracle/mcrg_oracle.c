/*
 * mcrg_oracle.c -- CPU oracle for the MCRG Monte-Carlo / block-spin hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs may
 * load it.  The product (libmcrg, the CUDA path) never links or calls it.
 *
 * It restates, in plain C on a natural-layout lattice (int8 +-1, row-major,
 * element (i,j) at i*N+j, periodic), every step of the hot path:
 *
 *   - majority-rule b=2 blocking with ties resolved either from an injected
 *     list consumed in ib-outer / jb-inner order (kim-jane/MCRG
 *     src/mcrg.cpp:314-348, ties drawn by rand_spin() in that order) or from
 *     the Philox tie stream the device uses;
 *   - coupling sums over directional offsets (src/lattice.cpp:102-120 for
 *     nn / nnn, with the periodic neighbour tables of src/lattice.cpp:124-151);
 *     the third-neighbour, plaquette and 4-spin-line sums are extensions with
 *     no counterpart in the reference;
 *   - the checkerboard Metropolis sweep driven by the same counter-based
 *     Philox4x32-10 keys as the device (the new update rule; it has the same
 *     stationary distribution as the Wolff step of src/ising.cpp:87-149);
 *   - the reference's own Wolff single-cluster step (src/ising.cpp:87-155),
 *     with bond probability 1-exp(2K) (src/ising.cpp:9), used for the
 *     statistical comparison and as the timed CPU baseline;
 *   - exact enumeration of the 4x4 lattice (2^16 states).
 *
 * Weight convention (src/ising.cpp:9, :158-173): w(s) = exp(-K * sum_bonds s s),
 * K < 0 ferromagnetic.  A Metropolis flip of s with local field h is accepted
 * with min(1, exp(2 K s h)).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11, "Parallel random   */
/* numbers: as easy as 1, 2, 3").                                      */
/* ------------------------------------------------------------------ */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += PHILOX_W0;
        k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Stream layout shared with the device (documented in include/mcrg.h):
 *   key = (seed lo32, seed hi32)
 *   ctr = (row, purpose<<28 | sub<<20 | group, time, replica)          */
enum { P_INIT = 1, P_SWEEP_HI = 2, P_SWEEP_LO = 3, P_TIE = 4 };

static void stream(uint64_t seed, uint32_t replica, uint32_t purpose, uint32_t sub,
                   uint32_t row, uint32_t group, uint32_t time, uint32_t out[4]) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {row, (purpose << 28) | (sub << 20) | group, time, replica};
    orc_philox4x32_10(ctr, key, out);
}

/* ------------------------------------------------------------------ */
/* Acceptance table                                                    */
/* ------------------------------------------------------------------ */
/* m = number of anti-aligned neighbours (0..4); s*h = 4 - 2m.
 * p = min(1, exp(2K(4-2m))); always[m] when p >= 1, else thr = floor(p 2^32). */
void orc_thresholds(double K, uint32_t thr[5], uint8_t always[5]) {
    for (int m = 0; m < 5; ++m) {
        double x = 2.0 * K * (double)(4 - 2 * m);
        if (x >= 0.0) { always[m] = 1; thr[m] = 0xFFFFFFFFu; continue; }
        double p = exp(x);
        always[m] = 0;
        thr[m] = (uint32_t)floor(p * 4294967296.0);
    }
}

/* ------------------------------------------------------------------ */
/* Initial configuration: fair coin from the P_INIT stream.             */
/* Site (i,j) has colour c=(i+j)&1 and split index k=j>>1.             */
/* ------------------------------------------------------------------ */
void orc_init_spins(int N, uint64_t seed, uint32_t replica, int8_t* s) {
    uint32_t out[4];
    for (int i = 0; i < N; ++i)
        for (int c = 0; c < 2; ++c) {
            int last_g = -1;
            for (int j = (i + c) & 1; j < N; j += 2) {
                int k = j >> 1;
                if ((k >> 7) != last_g) {
                    last_g = k >> 7;
                    stream(seed, replica, P_INIT, (uint32_t)c, (uint32_t)i, (uint32_t)last_g, 0u, out);
                }
                int bit = (out[(k & 127) >> 5] >> (k & 31)) & 1;
                s[i * N + j] = bit ? 1 : -1;
            }
        }
}

/* ------------------------------------------------------------------ */
/* Checkerboard Metropolis sweep (black (i+j even) then white).         */
/* Site (i, j) of colour c = (i+j)&1 is byte k = j>>1 of its colour     */
/* row.  Site random u32 = r8 << 24 | r24 where r8 depends on N:        */
/*   N <  ORC_PLANE_MIN_L (byte draws):                                 */
/*     r8 = byte (k&15) of the P_SWEEP_HI block (row i, group k>>4,     */
/*          sub = colour c, time = sweep t); byte b of a block is byte  */
/*          (b&3) of word (b>>2), little-endian;                        */
/*   N >= ORC_PLANE_MIN_L (bit-plane draws, 32 sites per plane word):   */
/*     with w = k>>5, p = k&31 and pos = 8*(p&3) + (p>>2), the planes   */
/*     W0..W7 are the words of the P_SWEEP_HI blocks (row i, group 2w   */
/*     and 2w+1, sub = c, time = t) in order, and bit 7-q of r8 is bit  */
/*     pos of Wq (W0 carries the most significant bit);                 */
/*   r24 = low 24 bits of word (k&3) of the P_SWEEP_LO block            */
/*         (row i, group k>>2, sub = c, time = t), both layouts.        */
/* Flip iff always[m] or u32 < thr[m].                                  */
/* ------------------------------------------------------------------ */
#define ORC_PLANE_MIN_L 64   /* one colour row holds whole plane words */

static uint32_t plane_r8(const uint32_t planes[8], int k) {
    int p = k & 31, pos = 8 * (p & 3) + (p >> 2);
    uint32_t r8 = 0;
    for (int q = 0; q < 8; ++q) r8 |= ((planes[q] >> pos) & 1u) << (7 - q);
    return r8;
}
void orc_sweep(int N, int8_t* s, double K, uint64_t seed, uint32_t replica,
               uint32_t t0, int64_t n_sweeps) {
    uint32_t thr[5]; uint8_t always[5];
    orc_thresholds(K, thr, always);
    uint32_t hi[4], lo[4], planes[8];
    const int bit_planes = N >= ORC_PLANE_MIN_L;
    for (int64_t n = 0; n < n_sweeps; ++n) {
        uint32_t t = t0 + (uint32_t)n;
        for (int c = 0; c < 2; ++c)
            for (int i = 0; i < N; ++i) {
                int last_g = -1;
                for (int j = ((i + c) & 1); j < N; j += 2) {
                    int k = j >> 1;
                    if (bit_planes && (k >> 5) != last_g) {
                        last_g = k >> 5;
                        stream(seed, replica, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(2 * last_g), t, planes);
                        stream(seed, replica, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)(2 * last_g + 1), t,
                               planes + 4);
                    } else if (!bit_planes && (k >> 4) != last_g) {
                        last_g = k >> 4;
                        stream(seed, replica, P_SWEEP_HI, (uint32_t)c, (uint32_t)i, (uint32_t)last_g, t, hi);
                    }
                    int sv = s[i * N + j];
                    int ip = (i + 1) % N, im = (i - 1 + N) % N, jp = (j + 1) % N, jm = (j - 1 + N) % N;
                    int m = (s[ip * N + j] != sv) + (s[im * N + j] != sv) +
                            (s[i * N + jp] != sv) + (s[i * N + jm] != sv);
                    if (always[m]) { s[i * N + j] = (int8_t)-sv; continue; }
                    uint32_t r8 = bit_planes ? plane_r8(planes, k) : (hi[(k & 15) >> 2] >> (8 * (k & 3))) & 0xFFu;
                    uint32_t t8 = thr[m] >> 24;
                    int flip;
                    if (r8 != t8) {
                        flip = r8 < t8; /* u32 < thr decided by the top byte */
                    } else {
                        stream(seed, replica, P_SWEEP_LO, (uint32_t)c, (uint32_t)i, (uint32_t)(k >> 2), t, lo);
                        uint32_t u = (r8 << 24) | (lo[k & 3] & 0xFFFFFFu);
                        flip = u < thr[m];
                    }
                    if (flip) s[i * N + j] = (int8_t)-sv;
                }
            }
    }
}

/* ------------------------------------------------------------------ */
/* Majority-rule blocking, b = 2 (src/mcrg.cpp:314-348).                */
/* tie_mode 0: ties take values from tie_vals[] in ib-outer, jb-inner   */
/*             order (the order rand_spin() is consumed in the          */
/*             reference); returns -1 if tie_vals runs out.             */
/* tie_mode 1: tie (ib,jb) = bit (jb&127) of P_TIE block (row ib,       */
/*             group jb>>7, sub = level, time = sample).                */
/* Returns the number of ties.                                          */
/* ------------------------------------------------------------------ */
int orc_block(int N, const int8_t* s, int8_t* out, int tie_mode, const int8_t* tie_vals,
              int tie_len, uint64_t seed, uint32_t replica, int level, uint32_t sample) {
    int Nb = N / 2, ties = 0;
    uint32_t w[4];
    for (int ib = 0; ib < Nb; ++ib)
        for (int jb = 0; jb < Nb; ++jb) {
            int tot = 0;
            for (int i = 2 * ib; i < 2 * ib + 2; ++i)
                for (int j = 2 * jb; j < 2 * jb + 2; ++j) tot += s[i * N + j];
            int v;
            if (tot > 0) v = 1;
            else if (tot < 0) v = -1;
            else {
                if (tie_mode == 0) {
                    if (ties >= tie_len) return -1;
                    v = tie_vals[ties];
                } else {
                    stream(seed, replica, P_TIE, (uint32_t)level, (uint32_t)ib, (uint32_t)(jb >> 7), sample, w);
                    v = ((w[(jb & 127) >> 5] >> (jb & 31)) & 1) ? 1 : -1;
                }
                ++ties;
            }
            out[ib * Nb + jb] = (int8_t)v;
        }
    return ties;
}

/* ------------------------------------------------------------------ */
/* Coupling sums over directional offsets.                             */
/*   0 nn    : sum_x s(x) sum_{(+-1,0),(0,+-1)} s(x+d)  (lattice.cpp:102-120) */
/*   1 nnn   : sum_x s(x) sum_{(+-1,+-1)} s(x+d)        (lattice.cpp:102-120) */
/*   2 third : sum_x s(x) sum_{(+-2,0),(0,+-2)} s(x+d)  (extension)           */
/*   3 plaq  : sum_x s(i,j)s(i+1,j)s(i,j+1)s(i+1,j+1)   (extension)           */
/*   4 line4 : sum_x s(i,j)..s(i+3,j) + s(i,j)..s(i,j+3) (extension)          */
/* ------------------------------------------------------------------ */
static inline int wrap(int x, int N) {
    x %= N;
    return x < 0 ? x + N : x;
}

void orc_couplings(int N, const int8_t* s, int C, int64_t* out) {
    int64_t acc[5] = {0, 0, 0, 0, 0};
    int jj[7];
    for (int i = 0; i < N; ++i) {
        const int8_t* r0 = s + (size_t)i * N;
        const int8_t* rp1 = s + (size_t)wrap(i + 1, N) * N;
        const int8_t* rm1 = s + (size_t)wrap(i - 1, N) * N;
        const int8_t* rp2 = s + (size_t)wrap(i + 2, N) * N;
        const int8_t* rm2 = s + (size_t)wrap(i - 2, N) * N;
        const int8_t* rp3 = s + (size_t)wrap(i + 3, N) * N;
        for (int j = 0; j < N; ++j) {
            for (int d = -2; d <= 3; ++d) jj[d + 2] = wrap(j + d, N);
            const int jm2 = jj[0], jm1 = jj[1], jp1 = jj[3], jp2 = jj[4], jp3 = jj[5];
            const int v = r0[j];
            acc[0] += v * (rp1[j] + rm1[j] + r0[jp1] + r0[jm1]);
            if (C > 1) acc[1] += v * (rp1[jp1] + rm1[jp1] + rp1[jm1] + rm1[jm1]);
            if (C > 2) acc[2] += v * (rp2[j] + rm2[j] + r0[jp2] + r0[jm2]);
            if (C > 3) acc[3] += v * rp1[j] * r0[jp1] * rp1[jp1];
            if (C > 4) acc[4] += v * rp1[j] * rp2[j] * rp3[j] + v * r0[jp1] * r0[jp2] * r0[jp3];
        }
    }
    for (int c = 0; c < C; ++c) out[c] = acc[c];
}

/* ------------------------------------------------------------------ */
/* One measurement: S[l][c] for l = 0..n_levels on the current lattice, */
/* blocking with the Philox tie stream at sample index `sample`.        */
/* ------------------------------------------------------------------ */
static void measure(int N, const int8_t* s, int C, int n_levels, uint64_t seed, uint32_t replica,
                    uint32_t sample, int64_t* S, int8_t* work) {
    const int8_t* cur = s;
    int n = N;
    int8_t* bufs[2] = {work, work + (size_t)N * N / 4};
    orc_couplings(n, cur, C, S);
    for (int l = 1; l <= n_levels; ++l) {
        int8_t* nxt = bufs[l & 1];
        orc_block(n, cur, nxt, 1, NULL, 0, seed, replica, l, sample);
        n /= 2;
        cur = nxt;
        orc_couplings(n, cur, C, S + (size_t)l * C);
    }
}

/* A full chain as the device runs it: init (or given spins), n_eq sweeps,
 * then n_samples x (sweeps_between sweeps + measurement).  Writes the
 * per-sample S trace [n_samples][n_levels+1][C] and the final spins.
 * Sweep t and sample n are counted from t0 / n0.                        */
int orc_chain(int N, double K, int C, int n_levels, uint64_t seed, uint32_t replica,
              int init_from_spins, int8_t* spins, uint32_t t0, uint32_t n0, int64_t n_eq,
              int64_t n_samples, int64_t sweeps_between, int64_t* S_trace) {
    if (N < 4 || (N & (N - 1)) || C < 1 || C > 5 || n_levels < 0) return -1;
    int8_t* work = (int8_t*)malloc((size_t)N * N / 2 + 16);
    if (!work) return -2;
    if (!init_from_spins) orc_init_spins(N, seed, replica, spins);
    uint32_t t = t0;
    orc_sweep(N, spins, K, seed, replica, t, n_eq);
    t += (uint32_t)n_eq;
    for (int64_t n = 0; n < n_samples; ++n) {
        orc_sweep(N, spins, K, seed, replica, t, sweeps_between);
        t += (uint32_t)sweeps_between;
        measure(N, spins, C, n_levels, seed, replica, n0 + (uint32_t)n,
                S_trace + (size_t)n * (n_levels + 1) * C, work);
    }
    free(work);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Reference update rule: Wolff single-cluster step                     */
/* (src/ising.cpp:87-155).  The reference grows the cluster with a BFS  */
/* frontier, tests the 4 neighbours in the order (i+1,j),(i-1,j),       */
/* (i,j+1),(i,j-1), adds an aligned neighbour not yet queued with        */
/* probability P = 1-exp(2K) and flips each site after its neighbours   */
/* were examined.  The restatement keeps that order and semantics; a    */
/* per-site "queued" stamp replaces the linear std::find of in_cluster  */
/* (same membership test: a site is never queued twice).  Its own RNG   */
/* is xoshiro256** (Blackman & Vigna), not the reference's mt19937_64,  */
/* so chains agree with the reference statistically, not bitwise.       */
/* ------------------------------------------------------------------ */
typedef struct { uint64_t s[4]; } xo_t;
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline uint64_t xo_next(xo_t* r) {
    uint64_t res = rotl(r->s[1] * 5, 7) * 9, t = r->s[1] << 17;
    r->s[2] ^= r->s[0]; r->s[3] ^= r->s[1]; r->s[1] ^= r->s[2]; r->s[0] ^= r->s[3];
    r->s[2] ^= t; r->s[3] = rotl(r->s[3], 45);
    return res;
}
static void xo_seed(xo_t* r, uint64_t seed) {
    for (int i = 0; i < 4; ++i) { /* splitmix64 */
        uint64_t z = (seed += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        r->s[i] = z ^ (z >> 31);
    }
}
static inline double xo_unif(xo_t* r) { return (double)(xo_next(r) >> 11) * (1.0 / 9007199254740992.0); }

typedef struct {
    int N;
    double P;
    xo_t rng;
    int32_t* queue;   /* BFS frontier, capacity N*N */
    uint32_t* stamp;  /* queued-in-step stamp */
    uint32_t step;
} orc_wolff_t;

static int64_t wolff_step(orc_wolff_t* w, int8_t* s) {
    int N = w->N;
    w->step++;
    int head = 0, tail = 0;
    int k0 = (int)(xo_next(&w->rng) % (uint64_t)(N * N));
    w->queue[tail++] = k0;
    w->stamp[k0] = w->step;
    while (head < tail) {
        int k = w->queue[head++];
        int i = k / N, j = k % N;
        int sv = s[k];
        int nb[4] = {((i + 1) % N) * N + j, ((i - 1 + N) % N) * N + j, i * N + (j + 1) % N,
                     i * N + (j - 1 + N) % N};
        for (int l = 0; l < 4; ++l) {
            int n = nb[l];
            if (s[n] == sv && w->stamp[n] != w->step) {
                if (xo_unif(&w->rng) < w->P) {
                    w->stamp[n] = w->step;
                    w->queue[tail++] = n;
                }
            }
        }
        s[k] = (int8_t)-sv;
    }
    return tail;
}

orc_wolff_t* orc_wolff_new(int N, double K, uint64_t seed) {
    orc_wolff_t* w = (orc_wolff_t*)calloc(1, sizeof(orc_wolff_t));
    if (!w) return NULL;
    w->N = N;
    w->P = 1.0 - exp(2.0 * K);
    xo_seed(&w->rng, seed);
    w->queue = (int32_t*)malloc(sizeof(int32_t) * (size_t)N * N);
    w->stamp = (uint32_t*)calloc((size_t)N * N, sizeof(uint32_t));
    if (!w->queue || !w->stamp) {
        free(w->queue); free(w->stamp); free(w);
        return NULL;
    }
    return w;
}

void orc_wolff_free(orc_wolff_t* w) {
    if (!w) return;
    free(w->queue); free(w->stamp); free(w);
}

/* n Wolff steps; returns the number of flipped sites. */
int64_t orc_wolff_steps(orc_wolff_t* w, int8_t* spins, int64_t n) {
    int64_t flipped = 0;
    for (int64_t k = 0; k < n; ++k) flipped += wolff_step(w, spins);
    return flipped;
}

/* ------------------------------------------------------------------ */
/* Cluster updates with the device's bond and cluster streams           */
/* (include/mcrg.h).  The bond of (i,j) to (i,j+1) is word 2*(j&1), the */
/* bond to (i+1,j) word 2*(j&1)+1 of the purpose-5 block (row i, group  */
/* j>>1, time t); it is open iff both spins are equal and the word is   */
/* below tb = floor((1 - exp(2K)) 2^32).  Clusters are labelled by a     */
/* sequential union-find that keeps the smallest index as the root.     */
/* kind 1 (Wolff): flip the component of the seed site, word 0 of the   */
/* purpose-6 block (sub 0, row 0, group 0) mod N^2 -- the component the */
/* reference's breadth-first step grows from that site with the same    */
/* bond outcomes (src/ising.cpp:87-155).  kind 2 (Swendsen-Wang): flip  */
/* every component whose root r draws bit 0 of word 0 of the purpose-6  */
/* block (sub 1, row r>>16, group r&0xFFFF) set.  Returns the number of */
/* flipped spins, -1 when out of memory.                                 */
/* ------------------------------------------------------------------ */
static int dsu_find(int* p, int x) {
    while (p[x] != x) {
        p[x] = p[p[x]];
        x = p[x];
    }
    return x;
}

static void dsu_union(int* p, int a, int b) {
    a = dsu_find(p, a);
    b = dsu_find(p, b);
    if (a == b) return;
    if (a < b) p[b] = a;
    else p[a] = b;
}

uint32_t orc_bond_threshold(double K) {
    double p = 1.0 - exp(2.0 * K);
    if (!(p > 0.0)) return 0u;
    double x = floor(p * 4294967296.0);
    return x >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)x;
}

int64_t orc_cluster_update(int N, int8_t* s, double K, uint64_t seed, uint32_t replica, uint32_t t, int kind) {
    const uint32_t tb = orc_bond_threshold(K);
    const int n = N * N;
    int* par = (int*)malloc((size_t)n * sizeof(int));
    signed char* dec = (signed char*)malloc((size_t)n);
    if (!par || !dec) { free(par); free(dec); return -1; }
    for (int x = 0; x < n; ++x) par[x] = x;
    uint32_t w[4];
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; j += 2) {
            stream(seed, replica, 5u, 0u, (uint32_t)i, (uint32_t)(j >> 1), t, w);
            for (int d = 0; d < 2; ++d) {
                const int jj = j + d, x = i * N + jj;
                const int xr = i * N + (jj + 1) % N, xd = ((i + 1) % N) * N + jj;
                if (w[2 * d] < tb && s[x] == s[xr]) dsu_union(par, x, xr);
                if (w[2 * d + 1] < tb && s[x] == s[xd]) dsu_union(par, x, xd);
            }
        }
    int64_t flipped = 0;
    if (kind == 1) {
        stream(seed, replica, 6u, 0u, 0u, 0u, t, w);
        const int r0 = dsu_find(par, (int)(w[0] & (uint32_t)(n - 1)));
        for (int x = 0; x < n; ++x)
            if (dsu_find(par, x) == r0) { s[x] = (int8_t)-s[x]; ++flipped; }
    } else {
        memset(dec, -1, (size_t)n);
        for (int x = 0; x < n; ++x) {
            const int r = dsu_find(par, x);
            if (dec[r] < 0) {
                stream(seed, replica, 6u, 1u, (uint32_t)r >> 16, (uint32_t)r & 0xFFFFu, t, w);
                dec[r] = (signed char)(w[0] & 1u);
            }
            if (dec[r]) { s[x] = (int8_t)-s[x]; ++flipped; }
        }
    }
    free(par);
    free(dec);
    return flipped;
}

/* One measurement (all levels, Philox tie stream at `sample`). */
int orc_measure(int N, const int8_t* spins, int C, int n_levels, uint64_t seed, uint32_t replica,
                uint32_t sample, int64_t* S) {
    int8_t* work = (int8_t*)malloc((size_t)N * N / 2 + 16);
    if (!work) return -2;
    measure(N, spins, C, n_levels, seed, replica, sample, S, work);
    free(work);
    return 0;
}

/* Runs the reference's MCRG sample loop (src/mcrg.cpp:72-98) with the
 * Wolff update: n_eq Wolff steps, then n_samples x (one Wolff step +
 * measurement at every level).  Ties come from the Philox tie stream.
 * Returns the number of flipped sites; writes the S trace if non-null. */
int64_t orc_wolff_chain(int N, double K, int C, int n_levels, uint64_t seed, int8_t* spins,
                        int64_t n_eq, int64_t n_samples, int64_t* S_trace) {
    if (N < 4 || (N & (N - 1))) return -1;
    orc_wolff_t* w = orc_wolff_new(N, K, seed);
    int8_t* work = (int8_t*)malloc((size_t)N * N / 2 + 16);
    int64_t* Sbuf = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n_levels + 1) * (C > 0 ? C : 1));
    if (!w || !work || !Sbuf) return -2;
    w->step = 0;
    int64_t flipped = orc_wolff_steps(w, spins, n_eq);
    for (int64_t n = 0; n < n_samples; ++n) {
        flipped += wolff_step(w, spins);
        if (C > 0) {
            int64_t* dst = S_trace ? S_trace + (size_t)n * (n_levels + 1) * C : Sbuf;
            measure(N, spins, C, n_levels, seed, 0u, (uint32_t)n, dst, work);
        }
    }
    orc_wolff_free(w); free(work); free(Sbuf);
    return flipped;
}

/* ------------------------------------------------------------------ */
/* Exact enumeration of the 4x4 periodic lattice.                       */
/* out[0] = Z-normalised <E> per site (E = K S_nn / N^2, ising.cpp:158) */
/* out[1] = <M^2> per site^2 (M = sum s / N^2)                          */
/* Then, for the one blocking level 4 -> 2 with ties averaged (each tie  */
/* value with weight 1/2), exact moments for C couplings:                */
/*   S0[C], S1[C], S1S0[C*C] (a*C+b = <S1_a S0_b>), S1S1[C*C].          */
/* ------------------------------------------------------------------ */
void orc_exact4(double K, int C, double* out) {
    const int N = 4;
    double Z = 0, E = 0, M2 = 0;
    double S0[5] = {0}, S1[5] = {0}, S1S0[25] = {0}, S1S1[25] = {0};
    int8_t s[16], b[4];
    int64_t c0[5], c1[5];
    double wmin = 0.0;
    /* shift the exponent by the ground-state energy to avoid overflow */
    wmin = -K * 32.0;
    for (uint32_t cfg = 0; cfg < (1u << 16); ++cfg) {
        for (int x = 0; x < 16; ++x) s[x] = ((cfg >> x) & 1) ? 1 : -1;
        orc_couplings(N, s, 5, c0);
        double w = exp(-K * (double)c0[0] / 2.0 - wmin);
        int mag = 0;
        for (int x = 0; x < 16; ++x) mag += s[x];
        Z += w;
        E += w * K * (double)c0[0] / 16.0;
        M2 += w * ((double)mag / 16.0) * ((double)mag / 16.0);
        /* blocked sums; enumerate tie assignments */
        int tot[4], tieidx[4], nt = 0;
        for (int ib = 0; ib < 2; ++ib)
            for (int jb = 0; jb < 2; ++jb) {
                int t = s[(2 * ib) * 4 + 2 * jb] + s[(2 * ib) * 4 + 2 * jb + 1] +
                        s[(2 * ib + 1) * 4 + 2 * jb] + s[(2 * ib + 1) * 4 + 2 * jb + 1];
                tot[ib * 2 + jb] = t;
                if (t == 0) tieidx[nt++] = ib * 2 + jb;
            }
        double wt = w / (double)(1 << nt);
        for (int a = 0; a < (1 << nt); ++a) {
            for (int x = 0; x < 4; ++x) b[x] = tot[x] > 0 ? 1 : -1;
            for (int q = 0; q < nt; ++q) b[tieidx[q]] = ((a >> q) & 1) ? 1 : -1;
            orc_couplings(2, b, 5, c1);
            for (int p = 0; p < C; ++p) {
                S1[p] += wt * (double)c1[p];
                for (int q = 0; q < C; ++q) {
                    S1S0[p * C + q] += wt * (double)c1[p] * (double)c0[q];
                    S1S1[p * C + q] += wt * (double)c1[p] * (double)c1[q];
                }
            }
        }
        for (int p = 0; p < C; ++p) S0[p] += w * (double)c0[p];
    }
    out[0] = E / Z;
    out[1] = M2 / Z;
    double* o = out + 2;
    for (int p = 0; p < C; ++p) o[p] = S0[p] / Z;
    o += C;
    for (int p = 0; p < C; ++p) o[p] = S1[p] / Z;
    o += C;
    for (int p = 0; p < C * C; ++p) o[p] = S1S0[p] / Z;
    o += C * C;
    for (int p = 0; p < C * C; ++p) o[p] = S1S1[p] / Z;
}
