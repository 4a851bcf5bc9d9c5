// Prints the real parts of the eigenvalues of matrices read from stdin
// (n, then n*n row-major values) using the shim's FP64 routine.
#include <cstdio>
#include <vector>
#include "../mcrg_gb300/shim/tmatrix.hpp"
int main() {
  int n;
  while (scanf("%d", &n) == 1) {
    std::vector<double> a((size_t)n * n);
    for (auto& x : a) scanf("%lf", &x);
    auto re = mcrg_host::eig_real_parts(a, n);
    double best = -1e300;
    for (double r : re) best = r > best ? r : best;
    printf("%.15g\n", best);
  }
  return 0;
}
