// Oracle (test infrastructure only): small dense FP64 linear algebra that
// stands in for the Eigen decompositions the reference calls. These are
// written from the textbook algorithms (Golub & Van Loan, "Matrix
// Computations", 4th ed.): they agree with Eigen to rounding, not bit for bit.
#pragma once

#include <cmath>
#include <cstring>
#include <vector>

namespace oracle {

// utils::gaussElimination<_Size> (src/pygcransac/include/math_utils.h:45-87):
// a bubble pivoting pre-pass on the first column entries, forward elimination
// without further pivoting, back substitution. `a` is _Size x (_Size + 1).
template <int S>
void gauss_elimination(double a[S][S + 1], double x[S]) {
  for (int i = 0; i < S; i++)
    for (int k = i + 1; k < S; k++)
      if (std::fabs(a[i][i]) < std::fabs(a[k][i]))
        for (int j = 0; j <= S; j++) {
          const double t = a[i][j];
          a[i][j] = a[k][j];
          a[k][j] = t;
        }
  for (int i = 0; i < S - 1; i++)
    for (int k = i + 1; k < S; k++) {
      const double t = a[k][i] / a[i][i];
      for (int j = 0; j <= S; j++) a[k][j] = a[k][j] - t * a[i][j];
    }
  for (int i = S - 1; i >= 0; i--) {
    x[i] = a[i][S];
    for (int j = i + 1; j < S; j++) x[i] = x[i] - a[i][j] * x[j];
    x[i] = x[i] / a[i][i];
  }
}

// Least-squares solve of the m x n (m >= n) system A x = b by Householder QR
// with column pivoting (Businger-Golub), the algorithm behind Eigen's
// colPivHouseholderQr().solve(). A is row-major and is overwritten. Like
// Eigen's solve, it always returns a solution: columns after an exactly zero
// pivot get zero coefficients (a basic solution).
inline bool lstsq_colpiv_qr(std::vector<double>& A, std::vector<double>& b, int m, int n, double* x) {
  std::vector<int> perm(n);
  std::vector<double> norms(n);
  for (int j = 0; j < n; ++j) {
    perm[j] = j;
    double s = 0;
    for (int i = 0; i < m; ++i) s += A[i * n + j] * A[i * n + j];
    norms[j] = s;
  }
  double first_pivot = 0;
  int rank = n;
  (void)first_pivot;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = -1;
    for (int j = k; j < n; ++j) {
      double s = 0;
      for (int i = k; i < m; ++i) s += A[i * n + j] * A[i * n + j];
      norms[j] = s;
      if (s > best) { best = s; p = j; }
    }
    if (p != k) {
      for (int i = 0; i < m; ++i) std::swap(A[i * n + k], A[i * n + p]);
      std::swap(perm[k], perm[p]);
    }
    double alpha = 0;
    for (int i = k; i < m; ++i) alpha += A[i * n + k] * A[i * n + k];
    alpha = std::sqrt(alpha);
    if (k == 0) first_pivot = alpha;
    if (alpha == 0) { rank = k; break; }
    if (A[k * n + k] > 0) alpha = -alpha;
    // v = a_k - alpha e_k, stored in place
    std::vector<double> v(m - k);
    for (int i = k; i < m; ++i) v[i - k] = A[i * n + k];
    v[0] -= alpha;
    double vnorm2 = 0;
    for (double t : v) vnorm2 += t * t;
    if (vnorm2 > 0) {
      for (int j = k; j < n; ++j) {
        double s = 0;
        for (int i = k; i < m; ++i) s += v[i - k] * A[i * n + j];
        const double f = 2 * s / vnorm2;
        for (int i = k; i < m; ++i) A[i * n + j] -= f * v[i - k];
      }
      double s = 0;
      for (int i = k; i < m; ++i) s += v[i - k] * b[i];
      const double f = 2 * s / vnorm2;
      for (int i = k; i < m; ++i) b[i] -= f * v[i - k];
    }
  }
  std::vector<double> y(n, 0.0);
  for (int i = rank - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < rank; ++j) s -= A[i * n + j] * y[j];
    y[i] = s / A[i * n + i];
  }
  for (int j = 0; j < n; ++j) x[perm[j]] = y[j];
  return true;
}

}  // namespace oracle
