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
    : N_(N), n_spins_(N * N), a_(1), spins_(N, N), site_rng_(seed ^ ((uint64_t)replica << 32)) {
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
    : N_(spins.rows()), n_spins_(spins.rows() * spins.rows()), a_(a), spins_(spins), site_rng_(seed) {
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

Interactions Lattice::calc_interactions() {
  const int nl = (int)std::lround(std::log2((double)N_)) - 1;
  std::vector<int64_t> S((size_t)(nl + 1) * 2 + 8, 0);
  // level 0 only is returned, as the reference's calc_interactions does
  check(mcrg_interactions(ctx_, S.data()), "mcrg_interactions");
#ifdef MCRG_EIGEN_SPINS
  Interactions r;
  r(0) = (double)S[0];
  r(1) = (double)S[1];
  return r;
#else
  return {(double)S[0], (double)S[1]};
#endif
}

double Lattice::calc_nearest_neighbor_interaction() { return calc_interactions()[0]; }

void Lattice::write_spins(FILE* fptr) {
  fprintf(fptr, "\n");
  for (int i = 0; i < N_; ++i) {
    fprintf(fptr, "# ");
    for (int j = 0; j < N_; ++j) fprintf(fptr, "%i, ", spins_(i, j));
    fprintf(fptr, "\n");
  }
}

void Lattice::display_spins() {
  for (int i = 0; i < N_; ++i) {
    for (int j = 0; j < N_; ++j)
      printf(spins_(i, j) == 1 ? "\033[34m%2s\033[0m" : "\033[37m%2s\033[0m", spins_(i, j) == 1 ? "O" : "X");
    printf("\n");
  }
  printf("(Lattice spacing a = %i)\n\n", a_);
}

int Lattice::choose_random_spin() { return std::uniform_int_distribution<int>(0, n_spins_ - 1)(site_rng_); }

SpinMatrix Lattice::nearest_neighbors(int i, int j) const {
  const int N = N_;
  auto w = [N](int x) { return (x % N + N) % N; };
  SpinMatrix nn(4, 2);
  const int r[4][2] = {{w(i + 1), j}, {w(i - 1), j}, {i, w(j + 1)}, {i, w(j - 1)}};
  for (int k = 0; k < 4; ++k) nn(k, 0) = r[k][0], nn(k, 1) = r[k][1];
  return nn;
}

SpinMatrix Lattice::next_nearest_neighbors(int i, int j) const {
  const int N = N_;
  auto w = [N](int x) { return (x % N + N) % N; };
  SpinMatrix nnn(4, 2);
  const int r[4][2] = {{w(i + 1), w(j + 1)}, {w(i - 1), w(j + 1)}, {w(i + 1), w(j - 1)}, {w(i - 1), w(j - 1)}};
  for (int k = 0; k < 4; ++k) nnn(k, 0) = r[k][0], nnn(k, 1) = r[k][1];
  return nnn;
}

IsingModel::IsingModel(double K) : K_(K), P_(1.0 - std::exp(2.0 * K)) {}

namespace {

// the reference's write_iter (src/definitions.cpp:44-68): logged iterations
bool logged_iteration(int i) {
  if (i < 10) return true;
  if (i < 100) return i % 10 == 0;
  if (i < 1000) return i % 100 == 0;
  if (i < 10000) return i % 1000 == 0;
  if (i < 100000) return i % 10000 == 0;
  return i % 100000 == 0;
}

// S_nn of a +-1 matrix (each bond counted twice, src/lattice.cpp:102-120)
long long nn_sum(const SpinMatrix& s) {
  const int N = s.rows();
  long long S = 0;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      S += (long long)s(i, j) * (s((i + 1) % N, j) + s((i + N - 1) % N, j) + s(i, (j + 1) % N) + s(i, (j + N - 1) % N));
  return S;
}

}  // namespace

// n Monte Carlo steps of the given rule on the context.
static int advance(mcrg_ctx* ctx, Update u, int64_t n) {
  if (u == Update::Metropolis) return mcrg_sweep(ctx, n);
  return mcrg_cluster_update(ctx, n, u == Update::Wolff ? MCRG_UPDATE_WOLFF : MCRG_UPDATE_SWENDSEN_WANG, nullptr);
}

// src/ising.cpp:14-84.  The sweeps between two logged iterations run in one
// device call (the chain is the same as sweeping one by one).  The logged
// columns follow the reference's arithmetic with one process: E = K S_nn / N^2
// (calc_energy) divided again by the number of sites, |M| from the integer
// division of calc_magnetization (src/ising.cpp:176-179), spreads over the
// processes (zero here).
void IsingModel::equilibrate(std::shared_ptr<Lattice> p, int n_samples_eq, bool write) {
  if (!write) {
    check(advance(p->ctx(), update_, n_samples_eq), "equilibrate");
    p->refresh();
    return;
  }
  const std::string filename = "equilibrate_N_" + std::to_string(p->N_) + "_K_" + rounded(K_, 7) + ".txt";
  FILE* f = fopen(filename.c_str(), "w");
  if (!f) throw McrgError(MCRG_EIO, "equilibrate: cannot open the output file");
  fprintf(f, "# Nearest neighbor coupling K = %lf\n", K_);
  fprintf(f, "# Temperature T = %lf\n", -1 / K_);
  fprintf(f, "# Number of lattice sites = %i\n", p->N_ * p->N_);
  fprintf(f, "# Lattice spacing = %i\n", p->a_);
  fprintf(f, "# Using %i parallel processes\n", 1);
  fprintf(f, "# %s, %s, %s, %s, %s, %s, %s\n", "Iteration", "Avg E/spin", "Stddev E/spin", "Heat Capacity",
          "Avg |M|/spin", "Stddev |M|/spin", "Susceptibility");
  int done = 0;
  try {
    for (int n = 1; n <= n_samples_eq; ++n) {
      if (!logged_iteration(n)) continue;
      check(advance(p->ctx(), update_, n - done), "equilibrate");
      done = n;
      p->sync_spins();
      const int NN = p->N_ * p->N_;
      const double E = K_ * (double)nn_sum(p->spins_) / NN;
      const double M = std::abs((double)(int)(p->spins_.sum() / NN));
      const double E2 = E * E, M2 = M * M;
      double E_sigma = E2 - E * E, M_sigma = M2 - M * M;
      const double C = E_sigma * K_ * K_, Chi = -M_sigma * K_;
      E_sigma = std::sqrt(E_sigma);
      M_sigma = std::sqrt(M_sigma);
      fprintf(f, "%i, %10.7e, %10.7e, %10.7e, %10.7e, %10.7e, %10.7e\n", n, E / p->n_spins_, E_sigma / p->n_spins_, C,
              M / p->n_spins_, M_sigma / p->n_spins_, Chi);
    }
    if (done < n_samples_eq) check(advance(p->ctx(), update_, n_samples_eq - done), "equilibrate");
  } catch (...) {
    fclose(f);
    throw;
  }
  p->sync_spins();
  p->write_spins(f);
  fclose(f);
}

void IsingModel::sample_new_configuration(std::shared_ptr<Lattice> p) {
  check(advance(p->ctx(), update_, 1), "sample_new_configuration");
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
  int rc = advance(ctx, update_, n_samples_eq);
  printf("Sampling %i configurations...\n", n_samples);
  if (rc == MCRG_OK) {
    if (update_ == Update::Metropolis)
      rc = mcrg_measure(ctx, n_samples, 1, &mom, 0, nullptr, 0);
    else
      rc = mcrg_measure_cluster(ctx, n_samples, 1,
                                update_ == Update::Wolff ? MCRG_UPDATE_WOLFF : MCRG_UPDATE_SWENDSEN_WANG, &mom, 0,
                                nullptr, 0);
  }
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

// ---------------------------------------------------------------------------
// Critical point by flow matching (src/mcrg.cpp:145-301).  The sample loop of
// both lattices runs on the device (mcrg_measure_flow); the connected parts
// <x y> - <x><y> are formed from the exact integer sums before dividing.
// ---------------------------------------------------------------------------
namespace {

// (n sum_xy - sum_x sum_y) / n^2
long double connected(const mcrg_i128& sum_xy, int64_t sum_x, int64_t sum_y, int64_t n) {
  const __int128 xy = ((__int128)sum_xy.hi << 64) | (__int128)sum_xy.lo;
  const __int128 num = xy * (__int128)n - (__int128)sum_x * (__int128)sum_y;
  return (long double)num / ((long double)n * (long double)n);
}

void flow_of(int side, double K, uint64_t seed, uint32_t replica, int device, int n_eq, int n_samples,
             mcrg_flow_moments* out) {
  mcrg_cfg cfg{};
  cfg.L = side;
  cfg.b = 2;
  cfg.n_levels = -1;
  cfg.n_couplings = 1;
  cfg.K = K;
  cfg.seed = seed;
  cfg.replica = replica;
  cfg.device = device;
  mcrg_ctx* ctx = nullptr;
  check(mcrg_alloc(&ctx, &cfg), "mcrg_alloc");
  int rc = mcrg_sweep(ctx, n_eq);
  if (rc == MCRG_OK) rc = mcrg_measure_flow(ctx, n_samples, 1, out);
  mcrg_free(ctx);
  if (rc != MCRG_OK) throw McrgError(rc, "mcrg_measure_flow");
}

}  // namespace

double MonteCarloRenormalizationGroup::approx_critical_point(int n_samples_eq, int n_samples, int L, double K) {
  if (L < 8 || (L & (L - 1))) throw McrgError(MCRG_EINVAL, "approx_critical_point: L");
  const int n_transformations = (int)std::floor(std::log((double)L) / std::log((double)b_)) - 1;
  mcrg_flow_moments mL, mS;
  const uint64_t seed = seed_ + 1000003ull * (uint64_t)iter_;
  printf("Sampling %i configurations each...\n", n_samples);
  flow_of(L, K, seed, 0, device_, n_samples_eq, n_samples, &mL);
  flow_of(L / b_, K, seed, 1, device_, n_samples_eq, n_samples, &mS);
  const int64_t n = n_samples;
  double Kc = 0.0;
  kc_estimates_.clear();
  for (int lev = 0; lev < n_transformations; ++lev) {
    const long double dSL_dK = connected(mL.S0S[lev + 1], mL.S[lev + 1], mL.S[0], n);
    const long double dSS_dK = connected(mS.S0S[lev], mS.S[lev], mS.S[0], n);
    const long double dK = ((long double)(mL.S[lev + 1] - mS.S[lev]) / (long double)n) / (dSL_dK - dSS_dK);
    Kc = (double)((long double)K + dK);
    kc_estimates_.push_back(Kc);
    printf("n = %i: Kc = %lf\n", lev, Kc);
    if (fptr_) {
      fprintf(fptr_, "%25i, %25i, %25.10lf, %25.10lf\n", iter_, lev, K, Kc);
      fflush(fptr_);
    }
  }
  return Kc;
}

double MonteCarloRenormalizationGroup::locate_critical_point(int n_iterations, int n_samples_eq, int n_samples,
                                                            int L, double K0) {
  printf("* Locating critical point starting from K0 = %lf\n", K0);
  const std::string filename = "critical_point_L_" + std::to_string(L) + "_K_" + rounded(K0, 7) + ".txt";
  fptr_ = fopen(filename.c_str(), "w");
  if (fptr_) {
    fprintf(fptr_, "# Number of parallel processes = %i\n", 1);
    fprintf(fptr_, "# Number of equilibration samples = %i\n", n_samples_eq);
    fprintf(fptr_, "# Number of samples = %i\n", n_samples);
    fprintf(fptr_, "# %23s  %25s  %25s  %25s\n", "Iteration", "Blocking Level n", "Starting K", "Approximate Kc");
  }
  double K = K0;
  try {
    for (iter_ = 1; iter_ <= n_iterations; ++iter_) {
      printf("\nIteration %i:\n", iter_);
      K = approx_critical_point(n_samples_eq, n_samples, L, K);
    }
  } catch (...) {
    if (fptr_) fclose(fptr_);
    fptr_ = nullptr;
    throw;
  }
  printf("\n* Critical point: Kc = %lf\n", K);
  printf("* Critical temperature: Tc = %lf\n", -1.0 / K);
  if (fptr_) fclose(fptr_);
  fptr_ = nullptr;
  return K;
}

double Lattice::rgnn_scalar_output(const double W[4]) const {
  double out = 0.0;
  check(mcrg_rgnn_scalar_output(ctx_, W, &out), "mcrg_rgnn_scalar_output");
  return out;
}
