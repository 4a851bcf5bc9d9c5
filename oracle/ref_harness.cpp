// ref_harness.cpp -- exposes the reference's own classes through a C ABI so
// tests/golden/make_golden.py can record golden vectors from the reference
// itself.  TEST INFRASTRUCTURE ONLY; compiled together with the reference's
// unmodified sources (src/definitions.cpp, lattice.cpp, ising.cpp, mcrg.cpp
// of kim-jane/MCRG) into oracle/_ref/libmcrg_ref.so by oracle/build.py.
//
// Lattices cross this ABI in natural layout: int8 +-1, element (i,j) at
// i*N+j, i being the first index of Lattice::spins_(i,j).

#include "definitions.hpp"   // std headers and Eigen first
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unistd.h>
#define private public       // reach MonteCarloRenormalizationGroup::block_spin_transformation
#include "mcrg.hpp"
#include "rgnn.hpp"
#undef private

namespace {

std::shared_ptr<Lattice> make_lattice(int N, const int8_t* nat) {
    imat m(N, N);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) m(i, j) = nat[i * N + j];
    return std::shared_ptr<Lattice>(new Lattice(1, m));
}

void export_lattice(const Lattice& lat, int8_t* out) {
    int N = lat.N_;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) out[i * N + j] = (int8_t)lat.spins_(i, j);
}

}  // namespace

extern "C" {

void ref_seed(uint64_t s) { rng.seed(s); }

// rand_spin() draws after reseeding: the tie values block_spin_transformation
// would consume, in order (src/definitions.hpp:34-36).
void ref_tie_draws(uint64_t seed, int n, int8_t* out) {
    rng.seed(seed);
    for (int k = 0; k < n; ++k) out[k] = (int8_t)rand_spin();
}

// src/mcrg.cpp:314-348 after rng.seed(seed).
void ref_block(int N, const int8_t* nat, uint64_t seed, int8_t* out) {
    MonteCarloRenormalizationGroup mcrg(2);
    auto lat = make_lattice(N, nat);
    rng.seed(seed);
    auto b = mcrg.block_spin_transformation(lat);
    export_lattice(*b, out);
}

// src/lattice.cpp:102-120.
void ref_interactions(int N, const int8_t* nat, double* out) {
    auto lat = make_lattice(N, nat);
    vec2D s = lat->calc_interactions();
    out[0] = s(0);
    out[1] = s(1);
}

// src/lattice.cpp:84-99.
double ref_nn_interaction(int N, const int8_t* nat) {
    auto lat = make_lattice(N, nat);
    return lat->calc_nearest_neighbor_interaction();
}

// src/ising.cpp:158-173.
double ref_energy(double K, int N, const int8_t* nat) {
    IsingModel m(K);
    auto lat = make_lattice(N, nat);
    return m.calc_energy(lat);
}

// The sequence calc_critical_exponent (src/mcrg.cpp:22-108) runs, step for
// step, through the reference's own methods, recording per sample the level-0
// spins, the blocked lattices of levels 1..n_lev (concatenated) and S[l][0..1].
// With the same rng seed it visits the same configurations as
// calc_critical_exponent itself.
int ref_trace(uint64_t seed, int n_eq, int n_samples, int N, double K, int8_t* spins_trace,
              int8_t* blocked_trace, double* S_trace) {
    MonteCarloRenormalizationGroup mcrg(2);
    int n_tr = (int)floor(log(N) / log(2)) - 1;
    rng.seed(seed);
    std::unique_ptr<IsingModel> ising(new IsingModel(K));
    std::shared_ptr<Lattice> lat(new Lattice(N));
    ising->equilibrate(lat, n_eq, false);
    size_t blocked_per_sample = 0;
    for (int n = 1, M = N / 2; n <= n_tr; ++n, M /= 2) blocked_per_sample += (size_t)M * M;
    for (int s = 0; s < n_samples; ++s) {
        ising->sample_new_configuration(lat);
        export_lattice(*lat, spins_trace + (size_t)s * N * N);
        vec2D S = lat->calc_interactions();
        double* Srow = S_trace + (size_t)s * (n_tr + 1) * 2;
        Srow[0] = S(0);
        Srow[1] = S(1);
        std::shared_ptr<Lattice> b = lat;
        int8_t* bt = blocked_trace + (size_t)s * blocked_per_sample;
        for (int n = 1; n <= n_tr; ++n) {
            b = mcrg.block_spin_transformation(b);
            export_lattice(*b, bt);
            bt += (size_t)b->N_ * b->N_;
            S = b->calc_interactions();
            Srow[2 * n] = S(0);
            Srow[2 * n + 1] = S(1);
        }
    }
    return n_tr;
}

// Runs the reference's calc_critical_exponent (src/mcrg.cpp:22-144) in
// directory `dir` after rng.seed(seed) and returns the largest eigenvalue of
// each level pair, parsed from the critical_exponent_N_*.txt it writes.
int ref_critical_exponent(uint64_t seed, int n_eq, int n_samples, int N, double K, const char* dir,
                          double* lambdas, int max_levels) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1;
    if (chdir(dir) != 0) return -2;
    rng.seed(seed);
    MonteCarloRenormalizationGroup mcrg(2);
    mcrg.calc_critical_exponent(n_eq, n_samples, N, K);
    std::string fn = "critical_exponent_N_" + std::to_string(N) + "_K_" + get_rounded_str(K, 7) + ".txt";
    FILE* f = fopen(fn.c_str(), "r");
    int got = 0;
    if (f) {
        char line[512];
        while (fgets(line, sizeof line, f)) {
            if (line[0] == '#') continue;
            int n;
            double lam, nu;
            if (sscanf(line, " %d , %lf , %lf", &n, &lam, &nu) == 3 && got < max_levels) lambdas[got++] = lam;
        }
        fclose(f);
    }
    if (chdir(cwd) != 0) return -3;
    return got;
}

// Runs the reference's locate_critical_point (src/mcrg.cpp:145-189) in
// directory `dir` after rng.seed(seed).  Writes the "Approximate Kc" column of
// the critical_point_L_*.txt it produces (one row per iteration and level)
// into kc, the returned K into *k_final, and returns the number of rows.
int ref_locate_critical_point(uint64_t seed, int n_iterations, int n_eq, int n_samples, int L, double K0,
                              const char* dir, double* kc, int max_rows, double* k_final) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1;
    if (chdir(dir) != 0) return -2;
    rng.seed(seed);
    MonteCarloRenormalizationGroup mcrg(2);
    *k_final = mcrg.locate_critical_point(n_iterations, n_eq, n_samples, L, K0);
    std::string fn = "critical_point_L_" + std::to_string(L) + "_K_" + get_rounded_str(K0, 7) + ".txt";
    FILE* f = fopen(fn.c_str(), "r");
    int got = 0;
    if (f) {
        char line[512];
        while (fgets(line, sizeof line, f)) {
            if (line[0] == '#') continue;
            int it, n;
            double k, k_c;
            if (sscanf(line, " %d , %d , %lf , %lf", &it, &n, &k, &k_c) == 4 && got < max_rows) kc[got++] = k_c;
        }
        fclose(f);
    }
    if (chdir(cwd) != 0) return -3;
    return got;
}

// Runs the reference's IsingModel::equilibrate(lattice, n, true)
// (src/ising.cpp:14-84) in directory `dir` after rng.seed(seed); it writes
// equilibrate_N_<N>_K_<K>.txt there.  Returns 0.
int ref_equilibrate_log(uint64_t seed, int N, double K, int n, const char* dir) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1;
    if (chdir(dir) != 0) return -2;
    rng.seed(seed);
    IsingModel m(K);
    std::shared_ptr<Lattice> lat(new Lattice(N));
    m.equilibrate(lat, n, true);
    if (chdir(cwd) != 0) return -3;
    return 0;
}

// RenormalizationGroupNeuralNetwork::scalar_output (src/rgnn.cpp:281-307)
// of a +-1 lattice (row-major, site (i, j) at i*N + j = spins_(i, j)) with
// weights W(r, k) = W[2r + k].
// The reference's own Wolff step (IsingModel::sample_new_configuration,
// src/ising.cpp:87-155) on a fresh Lattice(N) after rng.seed(seed): n_eq steps,
// then per step s < n_steps the number of spins it flipped (sizes[s]) and the
// bond sum sum_(i,j) s(i,j) (s(i+1,j) + s(i,j+1)) after it (bonds[s]).
int ref_wolff_sizes(uint64_t seed, int N, double K, int n_eq, int n_steps, int32_t* sizes, int32_t* bonds) {
    rng.seed(seed);
    IsingModel ising(K);
    std::shared_ptr<Lattice> lat(new Lattice(N));
    for (int s = 0; s < n_eq; ++s) ising.sample_new_configuration(lat);
    imat prev = lat->spins_;
    for (int s = 0; s < n_steps; ++s) {
        ising.sample_new_configuration(lat);
        int changed = 0, b = 0;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                const int v = lat->spins_(i, j);
                changed += v != prev(i, j);
                b += v * (lat->spins_((i + 1) % N, j) + lat->spins_(i, (j + 1) % N));
            }
        sizes[s] = changed;
        bonds[s] = b;
        prev = lat->spins_;
    }
    return 0;
}

double ref_rgnn_scalar_output(int N, const int8_t* spins, const double* W) {
    imat s(N, N);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) s(i, j) = spins[i * N + j];
    RenormalizationGroupNeuralNetwork net(2);
    mat w(2, 2);
    for (int r = 0; r < 2; ++r)
        for (int k = 0; k < 2; ++k) w(r, k) = W[2 * r + k];
    net.set_weights(w);
    return net.scalar_output(s);
}

// n Wolff steps of the reference (src/ising.cpp:87-149) on a lattice of side
// N started from rng.seed(seed); returns the final lattice.
void ref_wolff(uint64_t seed, int N, double K, int n_steps, int8_t* out) {
    rng.seed(seed);
    IsingModel m(K);
    std::shared_ptr<Lattice> lat(new Lattice(N));
    for (int s = 0; s < n_steps; ++s) m.sample_new_configuration(lat);
    export_lattice(*lat, out);
}

}  // extern "C"
