// run_mcrg -- the reference's src/main.cpp call sequence against the
// GB300 library: MonteCarloRenormalizationGroup(b).calc_critical_exponent.
// Usage: run_mcrg N n_eq n_samples K [seed] [n_couplings]
#include <cstdio>
#include <cstdlib>

#include "mcrg_classes.hpp"

int main(int argc, char** argv) {
  int N = argc > 1 ? atoi(argv[1]) : 128;
  int n_eq = argc > 2 ? atoi(argv[2]) : 10000;
  int n_samples = argc > 3 ? atoi(argv[3]) : 1000000;
  double K = argc > 4 ? atof(argv[4]) : -0.44068679350977147;
  try {
    MonteCarloRenormalizationGroup MCRG(2);
    if (argc > 5) MCRG.seed_ = strtoull(argv[5], nullptr, 10);
    if (argc > 6) MCRG.n_couplings_ = atoi(argv[6]);
    MCRG.calc_critical_exponent(n_eq, n_samples, N, K);
    for (size_t n = 0; n < MCRG.lambdas_.size(); ++n) printf("LAMBDA %zu %.12f\n", n, MCRG.lambdas_[n]);
  } catch (const McrgError& e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
