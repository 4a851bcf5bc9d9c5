// tmatrix.hpp -- host FP64 linearised RG matrix of src/mcrg.cpp:110-137.
//
// From exact moment sums (mcrg_moments) of one level pair:
//   A = <Sb S^T> - <Sb><S>^T,  B = <Sb Sb^T> - <Sb><Sb>^T,  T = B^{-1} A,
// and the largest real part of T's eigenvalues.  Connected parts are formed
// exactly in 128-bit integers (n*sum(xy) - sum(x)sum(y)) before the division.
// The eigenvalues of the small (C <= 5) real matrix come from Householder
// reduction to Hessenberg form and Francis double-shift QR iterations
// (Golub & Van Loan, Matrix Computations, Alg. 7.4.2 / 7.5.2).
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/mcrg.h"

namespace mcrg_host {

inline __int128 i128(const mcrg_i128& v) { return ((__int128)v.hi << 64) | (__int128)v.lo; }

// Solves B X = A (n x n, row-major) by Gaussian elimination with partial
// pivoting; returns false when B is singular.
inline bool solve(std::vector<double> B, std::vector<double> A, int n, std::vector<double>& X) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int r = k + 1; r < n; ++r)
      if (std::fabs(B[r * n + k]) > std::fabs(B[p * n + k])) p = r;
    if (B[p * n + k] == 0.0) return false;
    if (p != k)
      for (int c = 0; c < n; ++c) {
        std::swap(B[k * n + c], B[p * n + c]);
        std::swap(A[k * n + c], A[p * n + c]);
      }
    for (int r = k + 1; r < n; ++r) {
      const double f = B[r * n + k] / B[k * n + k];
      for (int c = k; c < n; ++c) B[r * n + c] -= f * B[k * n + c];
      for (int c = 0; c < n; ++c) A[r * n + c] -= f * A[k * n + c];
    }
  }
  X.assign((size_t)n * n, 0.0);
  for (int c = 0; c < n; ++c)
    for (int r = n - 1; r >= 0; --r) {
      double s = A[r * n + c];
      for (int q = r + 1; q < n; ++q) s -= B[r * n + q] * X[q * n + c];
      X[r * n + c] = s / B[r * n + r];
    }
  return true;
}

// Real parts of the eigenvalues of a real n x n matrix (row-major).
inline std::vector<double> eig_real_parts(std::vector<double> H, int n) {
  auto at = [&](int i, int j) -> double& { return H[(size_t)i * n + j]; };
  // Householder reduction to upper Hessenberg form
  for (int k = 0; k + 2 < n; ++k) {
    double alpha = 0;
    for (int i = k + 1; i < n; ++i) alpha += at(i, k) * at(i, k);
    alpha = std::sqrt(alpha);
    if (alpha == 0) continue;
    if (at(k + 1, k) > 0) alpha = -alpha;
    std::vector<double> v(n, 0.0);
    v[k + 1] = at(k + 1, k) - alpha;
    for (int i = k + 2; i < n; ++i) v[i] = at(i, k);
    double vn = 0;
    for (int i = k + 1; i < n; ++i) vn += v[i] * v[i];
    if (vn == 0) continue;
    for (int j = 0; j < n; ++j) {  // H = (I - 2vv^T/vn) H
      double s = 0;
      for (int i = k + 1; i < n; ++i) s += v[i] * at(i, j);
      s = 2 * s / vn;
      for (int i = k + 1; i < n; ++i) at(i, j) -= s * v[i];
    }
    for (int i = 0; i < n; ++i) {  // H = H (I - 2vv^T/vn)
      double s = 0;
      for (int j = k + 1; j < n; ++j) s += at(i, j) * v[j];
      s = 2 * s / vn;
      for (int j = k + 1; j < n; ++j) at(i, j) -= s * v[j];
    }
  }
  std::vector<double> re;
  int hi = n - 1, iter = 0;
  while (hi >= 0) {
    if (hi == 0) {
      re.push_back(at(0, 0));
      break;
    }
    // find a negligible subdiagonal entry
    int l = hi;
    for (; l > 0; --l) {
      const double s = std::fabs(at(l - 1, l - 1)) + std::fabs(at(l, l));
      if (std::fabs(at(l, l - 1)) <= 1e-15 * (s == 0 ? 1.0 : s)) break;
    }
    if (l == hi) {  // 1x1 block
      re.push_back(at(hi, hi));
      --hi;
      iter = 0;
      continue;
    }
    if (l == hi - 1) {  // 2x2 block: eigenvalues in closed form
      const double a = at(hi - 1, hi - 1), b = at(hi - 1, hi), c = at(hi, hi - 1), d = at(hi, hi);
      const double tr = a + d, det = a * d - b * c, disc = tr * tr / 4 - det;
      if (disc >= 0) {
        const double r = std::sqrt(disc);
        re.push_back(tr / 2 + r);
        re.push_back(tr / 2 - r);
      } else {
        re.push_back(tr / 2);
        re.push_back(tr / 2);
      }
      hi -= 2;
      iter = 0;
      continue;
    }
    if (++iter > 200) {  // give up on convergence: report the diagonal
      for (int i = l; i <= hi; ++i) re.push_back(at(i, i));
      break;
    }
    // Francis double-shift step on the active block [l, hi]
    const double s = at(hi - 1, hi - 1) + at(hi, hi);
    const double t = at(hi - 1, hi - 1) * at(hi, hi) - at(hi - 1, hi) * at(hi, hi - 1);
    double x = at(l, l) * at(l, l) + at(l, l + 1) * at(l + 1, l) - s * at(l, l) + t;
    double y = at(l + 1, l) * (at(l, l) + at(l + 1, l + 1) - s);
    double z = (l + 2 <= hi) ? at(l + 2, l + 1) * at(l + 1, l) : 0.0;
    for (int k = l; k <= hi - 2; ++k) {
      double v[3] = {x, y, z};
      double nv = std::sqrt(x * x + y * y + z * z);
      if (nv != 0) {
        const double alpha = (x > 0) ? -nv : nv;
        v[0] = x - alpha;
        const double vn = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        if (vn != 0) {
          const int q = k > l ? k - 1 : l;
          for (int j = q; j < n; ++j) {
            double sum = v[0] * at(k, j) + v[1] * at(k + 1, j) + v[2] * at(k + 2, j);
            sum = 2 * sum / vn;
            at(k, j) -= sum * v[0];
            at(k + 1, j) -= sum * v[1];
            at(k + 2, j) -= sum * v[2];
          }
          const int r = std::min(k + 3, hi);
          for (int i = 0; i <= r; ++i) {
            double sum = at(i, k) * v[0] + at(i, k + 1) * v[1] + at(i, k + 2) * v[2];
            sum = 2 * sum / vn;
            at(i, k) -= sum * v[0];
            at(i, k + 1) -= sum * v[1];
            at(i, k + 2) -= sum * v[2];
          }
        }
      }
      x = at(k + 1, k);
      y = at(k + 2, k);
      if (k < hi - 2) z = at(k + 3, k);
    }
    // final 2-element reflector
    {
      const int k = hi - 1;
      double nv = std::sqrt(x * x + y * y);
      if (nv != 0) {
        const double alpha = (x > 0) ? -nv : nv;
        double v0 = x - alpha, v1 = y;
        const double vn = v0 * v0 + v1 * v1;
        if (vn != 0) {
          for (int j = k - 1; j < n; ++j) {
            if (j < 0) continue;
            double sum = v0 * at(k, j) + v1 * at(k + 1, j);
            sum = 2 * sum / vn;
            at(k, j) -= sum * v0;
            at(k + 1, j) -= sum * v1;
          }
          for (int i = 0; i <= hi; ++i) {
            double sum = at(i, k) * v0 + at(i, k + 1) * v1;
            sum = 2 * sum / vn;
            at(i, k) -= sum * v0;
            at(i, k + 1) -= sum * v1;
          }
        }
      }
    }
  }
  return re;
}

// Largest real eigenvalue part of T for level pair `l`; NaN when B is singular.
inline double leading_eigenvalue(const mcrg_moments& m, int l) {
  const int C = m.n_couplings, MC = MCRG_MAX_COUPLINGS;
  const __int128 n = m.n_samples;
  std::vector<int> keep;
  for (int a = 0; a < C; ++a) {
    const __int128 sa = m.S[(l + 1) * MC + a];
    if (n * i128(m.SbSb[(l * MC + a) * MC + a]) - sa * sa != 0) keep.push_back(a);
  }
  const int k = (int)keep.size();
  if (k == 0) return NAN;
  std::vector<double> A((size_t)k * k), B((size_t)k * k), T;
  const double n2 = (double)m.n_samples * (double)m.n_samples;
  for (int p = 0; p < k; ++p)
    for (int q = 0; q < k; ++q) {
      const int a = keep[p], b = keep[q];
      const __int128 sba = m.S[(l + 1) * MC + a], sb = m.S[l * MC + b], sbb = m.S[(l + 1) * MC + b];
      A[(size_t)p * k + q] = (double)(n * i128(m.SbS[(l * MC + a) * MC + b]) - sba * sb) / n2;
      B[(size_t)p * k + q] = (double)(n * i128(m.SbSb[(l * MC + a) * MC + b]) - sba * sbb) / n2;
    }
  if (!solve(B, A, k, T)) return NAN;
  for (double x : T)
    if (!std::isfinite(x)) return NAN;
  const std::vector<double> re = eig_real_parts(T, k);
  double best = -INFINITY;
  for (double r : re) best = r > best ? r : best;
  return best;
}

}  // namespace mcrg_host
