// mcrg_classes.hpp -- the reference's host classes over the libmcrg C ABI.
//
// Same names, signatures and argument meaning as kim-jane/MCRG's
//   Lattice                          (src/lattice.hpp:5-37)
//   IsingModel                       (src/ising.hpp:8-41)
//   MonteCarloRenormalizationGroup   (src/mcrg.hpp:6-40)
// so src/main.cpp's call sites compile against this header.  Differences a
// caller can observe:
//   - the lattice lives on the GPU; spins_ is a host mirror refreshed after
//     every device operation (set mirror_spins_ = false to skip the copy);
//   - sample_new_configuration() is one checkerboard Metropolis sweep by
//     default (same stationary distribution as the reference's Wolff step);
//     update_ = Update::Wolff makes it the reference's own rule, one Wolff
//     cluster grown and flipped on the device (Update::SwendsenWang: every
//     cluster flipped with probability 1/2);
//   - the RG eigen-solve is a small FP64 routine (tmatrix.hpp) instead of
//     Eigen, applied to exact integer moment sums;
//   - errors from the device surface as McrgError exceptions on the C++ side
//     (the reference has no error reporting).
#pragma once

#include <cstdint>
#include <cstdio>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mcrg.h"

class McrgError : public std::runtime_error {
 public:
  McrgError(int code, const std::string& what)
      : std::runtime_error(what + ": " + mcrg_strerror(code)), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

#ifdef MCRG_EIGEN_SPINS
// The drop-in build (headers in dropin/, compiled with the reference's own
// definitions.hpp and vendored Eigen): spins_ and the neighbour tables are the
// reference's `imat`, calc_interactions returns its `vec2D`, so callers that
// hand spins_ to Eigen code (src/rgnn.cpp:113-114,175) compile unchanged.
#include "definitions.hpp"
using SpinMatrix = imat;
using Interactions = vec2D;
#else
// Minimal stand-in for the reference's `imat` (Eigen column-major int
// matrix): spins_(i, j) indexing, rows(), cols(), sum().
class SpinMatrix {
 public:
  SpinMatrix() = default;
  SpinMatrix(int n, int m) : n_(n), m_(m), d_((size_t)n * m, 0) {}
  int& operator()(int i, int j) { return d_[(size_t)j * n_ + i]; }
  int operator()(int i, int j) const { return d_[(size_t)j * n_ + i]; }
  int rows() const { return n_; }
  int cols() const { return m_; }
  long long sum() const {
    long long s = 0;
    for (int v : d_) s += v;
    return s;
  }

 private:
  int n_ = 0, m_ = 0;
  std::vector<int> d_;
};
using Interactions = std::vector<double>;
#endif

class Lattice {
 public:
  explicit Lattice(int N, double K = -0.44068679350977147, uint64_t seed = 1, uint32_t replica = 0,
                   int n_couplings = 2, int device = 0);
  Lattice(int a, const SpinMatrix& spins, double K = -0.44068679350977147, uint64_t seed = 1);
  ~Lattice();
  Lattice(const Lattice&) = delete;
  Lattice& operator=(const Lattice&) = delete;

  int N_;
  int n_spins_;
  int a_;
  SpinMatrix spins_;
  bool mirror_spins_ = true;

  // src/lattice.cpp:102-120 -> (S_nn, S_nnn) of the current configuration
  // (every coupling of the context in the stand-alone build)
  Interactions calc_interactions();
  double calc_nearest_neighbor_interaction();

  // src/lattice.cpp:63-75: "\n" then one "# s, s, ..., " line per row of the
  // host mirror spins_
  void write_spins(FILE* fptr);
  // src/lattice.cpp:44-60: the mirror as coloured O (+1) / X (-1) on stdout
  void display_spins();
  // src/lattice.cpp:78-81: a uniform site index in [0, N^2) from the
  // lattice's own mt19937_64 (seeded from seed and replica)
  int choose_random_spin();
  // src/lattice.cpp:124-151: periodic neighbours of (i, j) as a 4 x 2 matrix
  // of (row, column): (i+1, j), (i-1, j), (i, j+1), (i, j-1) and diagonals
  // (i+1, j+1), (i-1, j+1), (i+1, j-1), (i-1, j-1)
  SpinMatrix nearest_neighbors(int i, int j) const;
  SpinMatrix next_nearest_neighbors(int i, int j) const;

  // push host edits of spins_ to the device / pull the device state
  void upload_spins();
  void sync_spins();

  // RenormalizationGroupNeuralNetwork::scalar_output(spins_) (src/rgnn.cpp:281-307)
  // on the device, W(r, k) = W[2r + k]
  double rgnn_scalar_output(const double W[4]) const;

  mcrg_ctx* ctx() const { return ctx_; }
  void refresh() {
    if (mirror_spins_) sync_spins();
  }

 private:
  mcrg_ctx* ctx_ = nullptr;
  std::mt19937_64 site_rng_;
};

// Update rule of a Monte Carlo step: a checkerboard Metropolis sweep, or a
// cluster update on the device (mcrg_cluster_update).
enum class Update { Metropolis, Wolff, SwendsenWang };

class IsingModel {
 public:
  explicit IsingModel(double K);
  ~IsingModel() {}

  Update update_ = Update::Metropolis;

  void equilibrate(std::shared_ptr<Lattice> pLattice, int n_samples_eq, bool write);
  void sample_new_configuration(std::shared_ptr<Lattice> pLattice);
  double calc_magnetization(std::shared_ptr<Lattice> pLattice);
  double calc_energy(std::shared_ptr<Lattice> pLattice);

 private:
  double K_, P_;
};

class MonteCarloRenormalizationGroup {
 public:
  explicit MonteCarloRenormalizationGroup(int b);
  ~MonteCarloRenormalizationGroup() {}

  int b_;

  // src/mcrg.cpp:22-144: prints and writes critical_exponent_N_<N>_K_<K>.txt;
  // equilibration and the step between samples use update_
  void calc_critical_exponent(int n_samples_eq, int n_samples, int N, double K);
  Update update_ = Update::Metropolis;

  // src/mcrg.cpp:145-189: iterated flow matching of lattices of side L and
  // L/b; prints, writes critical_point_L_<L>_K_<K0>.txt, returns the last Kc
  double locate_critical_point(int n_iterations, int n_samples_eq, int n_samples, int L, double K0);

  // Kc estimate of every blocking level of the last matching iteration
  std::vector<double> kc_estimates_;

  // results of the last calc_critical_exponent (one entry per level pair)
  std::vector<double> lambdas_;
  std::vector<double> nus_;
  uint64_t seed_ = 1;
  int n_couplings_ = 2;
  int device_ = 0;

 private:
  int iter_ = 0;
  FILE* fptr_ = nullptr;
  // src/mcrg.cpp:191-301: one matching step at K, returns the Kc of the largest level
  double approx_critical_point(int n_samples_eq, int n_samples, int L, double K);
};
