// mcrg_classes.cpp -- implementation of the reference-named host classes
// (see mcrg_classes.hpp) on top of the libmcrg C ABI.
#include "mcrg_classes.hpp"

#include <cmath>
#include <cstdio>
#include <iomanip>
#include <sstream>

#include "tmatrix.hpp"

namespace {

void check(int rc, const char* what) {
  if (rc != MCRG_OK) throw McrgError(rc, what);
}

// the reference's get_rounded_str(K, 7) (src/definitions.cpp:70-77)
std::string rounded(double x, int precision) {
  std::stringstream ss;
  ss << std::setprecision(precision) << x;
  return ss.str();
}

}  // namespace

Lattice::Lattice(int N, double K, uint64_t seed, uint32_t replica, int n_couplings, int device)
    : N_(N), n_spins_(N * N), a_(1), spins_(N, N) {
  mcrg_cfg cfg{};
  cfg.L = N;
  cfg.b = 2;
  cfg.n_levels = -1;
  cfg.n_couplings = n_couplings;
  cfg.K = K;
  cfg.seed = seed;
  cfg.replica = replica;
  cfg.device = device;
  check(mcrg_alloc(&ctx_, &cfg), "mcrg_alloc");
  refresh();
}

Lattice::Lattice(int a, const SpinMatrix& spins, double K, uint64_t seed)
    : N_(spins.rows()), n_spins_(spins.rows() * spins.rows()), a_(a), spins_(spins) {
  mcrg_cfg cfg{};
  cfg.L = N_;
  cfg.b = 2;
  cfg.n_levels = -1;
  cfg.n_couplings = 2;
  cfg.K = K;
  cfg.seed = seed;
  check(mcrg_alloc(&ctx_, &cfg), "mcrg_alloc");
  upload_spins();
}

Lattice::~Lattice() {
  if (ctx_) mcrg_free(ctx_);
}

void Lattice::upload_spins() {
  std::vector<int8_t> h((size_t)N_ * N_);
  for (int i = 0; i < N_; ++i)
    for (int j = 0; j < N_; ++j) h[(size_t)i * N_ + j] = (int8_t)spins_(i, j);
  check(mcrg_set_spins(ctx_, h.data()), "mcrg_set_spins");
}

void Lattice::sync_spins() {
  std::vector<int8_t> h((size_t)N_ * N_);
  check(mcrg_get_spins(ctx_, h.data()), "mcrg_get_spins");
  for (int i = 0; i < N_; ++i)
    for (int j = 0; j < N_; ++j) spins_(i, j) = h[(size_t)i * N_ + j];
}

std::vector<double> Lattice::calc_interactions() {
  const int nl = (int)std::lround(std::log2((double)N_)) - 1;
  std::vector<int64_t> S((size_t)(nl + 1) * 2 + 8, 0);
  // level 0 only is returned, as the reference's calc_interactions does
  check(mcrg_interactions(ctx_, S.data()), "mcrg_interactions");
  return {(double)S[0], (double)S[1]};
}

double Lattice::calc_nearest_neighbor_interaction() { return calc_interactions()[0]; }

IsingModel::IsingModel(double K) : K_(K), P_(1.0 - std::exp(2.0 * K)) {}

void IsingModel::equilibrate(std::shared_ptr<Lattice> p, int n_samples_eq, bool /*write*/) {
  check(mcrg_sweep(p->ctx(), n_samples_eq), "mcrg_sweep");
  p->refresh();
}

void IsingModel::sample_new_configuration(std::shared_ptr<Lattice> p) {
  check(mcrg_sweep(p->ctx(), 1), "mcrg_sweep");
  p->refresh();
}

double IsingModel::calc_energy(std::shared_ptr<Lattice> p) {
  return K_ * p->calc_interactions()[0] / ((double)p->N_ * p->N_);
}

double IsingModel::calc_magnetization(std::shared_ptr<Lattice> p) {
  p->sync_spins();
  return (double)p->spins_.sum() / ((double)p->N_ * p->N_);
}

MonteCarloRenormalizationGroup::MonteCarloRenormalizationGroup(int b) : b_(b) {
  if (b != 2) throw McrgError(MCRG_EINVAL, "block factor");
  printf("\n=============================================\n");
  printf("==========       MONTE CARLO       ==========\n");
  printf("==========  RENORMALIZATION GROUP  ==========\n");
  printf("=============================================\n\n");
  printf("* Using 1 GPU process\n");
  printf("* Scaling factor b = %i\n", b_);
}

void MonteCarloRenormalizationGroup::calc_critical_exponent(int n_samples_eq, int n_samples, int N, double K) {
  printf("* Calculating critical exponent at K = %lf\n\n", K);
  const std::string filename = "critical_exponent_N_" + std::to_string(N) + "_K_" + rounded(K, 7) + ".txt";
  FILE* f = fopen(filename.c_str(), "w");
  if (f) {
    fprintf(f, "# Number of parallel processes = %i\n", 1);
    fprintf(f, "# Number of equilibration samples = %i\n", n_samples_eq);
    fprintf(f, "# Number of samples = %i\n", n_samples);
    fprintf(f, "# %23s  %25s  %25s\n", "Blocking Level n", "Largest Eigenvalue", "Critical Exponent nu");
  }
  mcrg_cfg cfg{};
  cfg.L = N;
  cfg.b = b_;
  cfg.n_levels = -1;
  cfg.n_couplings = n_couplings_;
  cfg.K = K;
  cfg.seed = seed_;
  cfg.device = device_;
  mcrg_ctx* ctx = nullptr;
  check(mcrg_alloc(&ctx, &cfg), "mcrg_alloc");
  mcrg_moments mom;
  int rc = mcrg_sweep(ctx, n_samples_eq);
  printf("Sampling %i configurations...\n", n_samples);
  if (rc == MCRG_OK) rc = mcrg_measure(ctx, n_samples, 1, &mom, 0, nullptr, 0);
  mcrg_free(ctx);
  if (rc != MCRG_OK) {
    if (f) fclose(f);
    throw McrgError(rc, "calc_critical_exponent");
  }
  lambdas_.clear();
  nus_.clear();
  double nu = 0.0;
  for (int n = 0; n < mom.n_levels; ++n) {
    const double lambda = mcrg_host::leading_eigenvalue(mom, n);
    nu = std::log((double)b_) / std::log(lambda);
    lambdas_.push_back(lambda);
    nus_.push_back(nu);
    printf("n = %i: lambda = %lf, nu = %lf\n", n, lambda, nu);
    if (f) fprintf(f, "%25i, %25.10lf, %25.10lf\n", n, lambda, nu);
  }
  printf("\n* Critical exponent: nu = %lf\n", nu);
  if (f) fclose(f);
}
