// run_mcrg -- the reference's src/main.cpp call sequence against the
// GB300 library: MonteCarloRenormalizationGroup(b).calc_critical_exponent.
// Usage: run_mcrg N n_eq n_samples K [seed] [n_couplings] [metropolis|wolff|sw]
//        run_mcrg locate L n_iterations n_eq n_samples K0 [seed]
//          (MonteCarloRenormalizationGroup::locate_critical_point)
//        run_mcrg rgnn N seed W00 W01 W10 W11  (Lattice::rgnn_scalar_output of the initial coin)
//        run_mcrg equilibrate N n K [seed] [metropolis|wolff|sw]
//          (IsingModel::equilibrate(lattice, n, true): writes equilibrate_N_*.txt)
//        run_mcrg lattice N seed n_draws
//          (the Lattice members: neighbour tables, write_spins, display_spins,
//           choose_random_spin, Lattice(a, spins))
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>

#include "mcrg_classes.hpp"

int main(int argc, char** argv) {
  if (argc > 7 && std::string(argv[1]) == "rgnn") {
    try {
      Lattice lat(atoi(argv[2]), -0.44068679350977147, strtoull(argv[3], nullptr, 10));
      const double W[4] = {atof(argv[4]), atof(argv[5]), atof(argv[6]), atof(argv[7])};
      printf("RGNN %.17g\n", lat.rgnn_scalar_output(W));
    } catch (const McrgError& e) {
      fprintf(stderr, "error: %s\n", e.what());
      return 1;
    }
    return 0;
  }
  if (argc > 1 && std::string(argv[1]) == "equilibrate") {
    const int N = argc > 2 ? atoi(argv[2]) : 8;
    const int n = argc > 3 ? atoi(argv[3]) : 1000;
    const double K = argc > 4 ? atof(argv[4]) : -0.44068679350977147;
    const uint64_t seed = argc > 5 ? strtoull(argv[5], nullptr, 10) : 1;
    const std::string u = argc > 6 ? argv[6] : "metropolis";
    try {
      std::shared_ptr<Lattice> lat(new Lattice(N, K, seed));
      IsingModel model(K);
      model.update_ = u == "wolff" ? Update::Wolff : u == "sw" ? Update::SwendsenWang : Update::Metropolis;
      model.equilibrate(lat, n, true);
    } catch (const McrgError& e) {
      fprintf(stderr, "error: %s\n", e.what());
      return 1;
    }
    return 0;
  }
  if (argc > 4 && std::string(argv[1]) == "lattice") {
    const int N = atoi(argv[2]);
    const uint64_t seed = strtoull(argv[3], nullptr, 10);
    const int n_draws = atoi(argv[4]);
    try {
      Lattice lat(N, -0.44068679350977147, seed);
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
          const SpinMatrix nn = lat.nearest_neighbors(i, j), nnn = lat.next_nearest_neighbors(i, j);
          printf("NB %d %d", i, j);
          for (int k = 0; k < 4; ++k) printf(" %d %d", nn(k, 0), nn(k, 1));
          for (int k = 0; k < 4; ++k) printf(" %d %d", nnn(k, 0), nnn(k, 1));
          printf("\n");
        }
      printf("DRAWS");
      for (int k = 0; k < n_draws; ++k) printf(" %d", lat.choose_random_spin());
      printf("\nSPINS");
      fflush(stdout);
      lat.write_spins(stdout);
      printf("DISPLAY\n");
      lat.display_spins();
      // Lattice(a, spins): the mirror flipped, spacing 2
      SpinMatrix flipped(N, N);
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) flipped(i, j) = -lat.spins_(i, j);
      Lattice lat2(2, flipped);
      lat2.sync_spins();
      printf("A2 %d SNN %.0f SNN2 %.0f\nFLIPPED", lat2.a_, lat.calc_nearest_neighbor_interaction(),
             lat2.calc_nearest_neighbor_interaction());
      lat2.write_spins(stdout);
    } catch (const McrgError& e) {
      fprintf(stderr, "error: %s\n", e.what());
      return 1;
    }
    return 0;
  }
  if (argc > 1 && std::string(argv[1]) == "locate") {
    const int L = argc > 2 ? atoi(argv[2]) : 16;
    const int n_it = argc > 3 ? atoi(argv[3]) : 1;
    const int n_eq = argc > 4 ? atoi(argv[4]) : 1000;
    const int n_samples = argc > 5 ? atoi(argv[5]) : 10000;
    const double K0 = argc > 6 ? atof(argv[6]) : -0.44;
    try {
      MonteCarloRenormalizationGroup MCRG(2);
      if (argc > 7) MCRG.seed_ = strtoull(argv[7], nullptr, 10);
      const double Kc = MCRG.locate_critical_point(n_it, n_eq, n_samples, L, K0);
      for (size_t n = 0; n < MCRG.kc_estimates_.size(); ++n) printf("KC %zu %.12f\n", n, MCRG.kc_estimates_[n]);
      printf("KCFINAL %.12f\n", Kc);
    } catch (const McrgError& e) {
      fprintf(stderr, "error: %s\n", e.what());
      return 1;
    }
    return 0;
  }
  int N = argc > 1 ? atoi(argv[1]) : 128;
  int n_eq = argc > 2 ? atoi(argv[2]) : 10000;
  int n_samples = argc > 3 ? atoi(argv[3]) : 1000000;
  double K = argc > 4 ? atof(argv[4]) : -0.44068679350977147;
  try {
    MonteCarloRenormalizationGroup MCRG(2);
    if (argc > 5) MCRG.seed_ = strtoull(argv[5], nullptr, 10);
    if (argc > 6) MCRG.n_couplings_ = atoi(argv[6]);
    if (argc > 7) {  // update rule: metropolis (default), wolff, sw
      const std::string u = argv[7];
      MCRG.update_ = u == "wolff" ? Update::Wolff : (u == "sw" ? Update::SwendsenWang : Update::Metropolis);
    }
    MCRG.calc_critical_exponent(n_eq, n_samples, N, K);
    for (size_t n = 0; n < MCRG.lambdas_.size(); ++n) printf("LAMBDA %zu %.12f\n", n, MCRG.lambdas_[n]);
  } catch (const McrgError& e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
