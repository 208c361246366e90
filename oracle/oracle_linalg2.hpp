// Oracle (test infrastructure only): decompositions with the semantics of the
// Eigen calls the reference's fundamental/essential solvers make
// (FullPivLU::kernel, FullPivHouseholderQR::matrixQ, PolynomialSolver::realRoots,
// JacobiSVD of 3x3 matrices, LLT). Written from the textbook algorithms
// (Golub & Van Loan); they agree with Eigen to rounding.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <limits>
#include <vector>

namespace oracle {

// Kernel of an r x c matrix (row-major) by LU with complete pivoting: at step
// k the largest |entry| of the remaining block is moved to (k, k); the rank is
// the number of pivots above eps * min(r, c) * |largest pivot|. Kernel vector j
// puts 1 at the (rank + j)-th pivoted column and -U11^-1 U12 on the pivot
// columns (the basis Eigen's FullPivLU::kernel() returns). Returns the kernel
// dimension; the basis goes column-wise into K (c x dim).
inline int fullpiv_lu_kernel(std::vector<double> A, int r, int c, std::vector<double>& K) {
  std::vector<int> rp(r), cp(c);
  for (int i = 0; i < r; ++i) rp[i] = i;
  for (int j = 0; j < c; ++j) cp[j] = j;
  const int sz = std::min(r, c);
  double maxpivot = 0;
  int nonzero = sz;
  for (int k = 0; k < sz; ++k) {
    int bi = k, bj = k;
    double best = -1;
    for (int i = k; i < r; ++i)
      for (int j = k; j < c; ++j) {
        const double v = std::fabs(A[i * c + j]);
        if (v > best) { best = v; bi = i; bj = j; }
      }
    if (best == 0) {
      nonzero = k;
      break;
    }
    if (best > maxpivot) maxpivot = best;
    if (bi != k) {
      for (int j = 0; j < c; ++j) std::swap(A[k * c + j], A[bi * c + j]);
      std::swap(rp[k], rp[bi]);
    }
    if (bj != k) {
      for (int i = 0; i < r; ++i) std::swap(A[i * c + k], A[i * c + bj]);
      std::swap(cp[k], cp[bj]);
    }
    for (int i = k + 1; i < r; ++i) {
      const double f = A[i * c + k] / A[k * c + k];
      A[i * c + k] = f;
      for (int j = k + 1; j < c; ++j) A[i * c + j] -= f * A[k * c + j];
    }
  }
  const double thr = std::numeric_limits<double>::epsilon() * (double)std::min(r, c);
  int rank = 0;
  for (int i = 0; i < nonzero; ++i)
    if (std::fabs(A[i * c + i]) > thr * maxpivot) ++rank;
  const int dim = c - rank;
  K.assign((size_t)c * dim, 0.0);
  for (int j = 0; j < dim; ++j) {
    // solve U11 x = -U12[:, j] for the pivot variables
    std::vector<double> x(rank, 0.0);
    for (int i = rank - 1; i >= 0; --i) {
      double s = -A[i * c + rank + j];
      for (int q = i + 1; q < rank; ++q) s -= A[i * c + q] * x[q];
      x[i] = s / A[i * c + i];
    }
    for (int i = 0; i < rank; ++i) K[(size_t)cp[i] * dim + j] = x[i];
    K[(size_t)cp[rank + j] * dim + j] = 1.0;
  }
  return dim;
}

// Last column of Q of the complete-pivoting Householder QR of an n x n matrix
// (Eigen's FullPivHouseholderQR(M).matrixQ().rightCols<1>()): at step k the
// largest |entry| of the remaining block becomes the pivot (row and column
// swap), then a Householder reflection annihilates column k below the
// diagonal (the row swap moves the trailing part of the rows only). When the
// remaining block is negligible against the first pivot the decomposition
// stops. Q = P_0 H_0 P_1 H_1 ... with P the row transpositions.
inline void fullpiv_householder_q_lastcol(std::vector<double> A, int n, double* q_last) {
  std::vector<std::vector<double>> vs;
  std::vector<double> taus;
  std::vector<int> transp(n);
  double biggest_all = 0;
  for (int k = 0; k < n; ++k) {
    int bi = k, bj = k;
    double best = -1;
    for (int i = k; i < n; ++i)
      for (int j = k; j < n; ++j) {
        const double v = std::fabs(A[i * n + j]);
        if (v > best) { best = v; bi = i; bj = j; }
      }
    if (k == 0) biggest_all = best;
    // a negligible remaining block ends the decomposition early
    if (best <= biggest_all * std::numeric_limits<double>::epsilon() * n) break;
    transp[k] = bi;
    if (bi != k)
      for (int j = k; j < n; ++j) std::swap(A[k * n + j], A[bi * n + j]);
    if (bj != k)
      for (int i = 0; i < n; ++i) std::swap(A[i * n + k], A[i * n + bj]);
    // Householder vector for A[k:, k] (Eigen's makeHouseholder convention)
    const double c0 = A[k * n + k];
    double tail = 0;
    for (int i = k + 1; i < n; ++i) tail += A[i * n + k] * A[i * n + k];
    std::vector<double> v(n - k, 0.0);
    double tau, beta;
    if (tail <= std::numeric_limits<double>::min()) {
      tau = 0;
      beta = c0;
      v[0] = 1;
    } else {
      beta = std::sqrt(c0 * c0 + tail);
      if (c0 >= 0) beta = -beta;
      for (int i = k + 1; i < n; ++i) v[i - k] = A[i * n + k] / (c0 - beta);
      v[0] = 1;
      tau = (beta - c0) / beta;
    }
    // apply H = I - tau v v^T to the remaining columns
    for (int j = k; j < n; ++j) {
      double s = 0;
      for (int i = k; i < n; ++i) s += v[i - k] * A[i * n + j];
      s *= tau;
      for (int i = k; i < n; ++i) A[i * n + j] -= s * v[i - k];
    }
    vs.push_back(v);
    taus.push_back(tau);
  }
  // Q e_{n-1}: apply the factors from the last to the first
  std::vector<double> e(n, 0.0);
  e[n - 1] = 1;
  for (int k = (int)vs.size() - 1; k >= 0; --k) {
    const std::vector<double>& v = vs[k];
    double s = 0;
    for (int i = k; i < n; ++i) s += v[i - k] * e[i];
    s *= taus[k];
    for (int i = k; i < n; ++i) e[i] -= s * v[i - k];
    if (transp[k] != k) std::swap(e[k], e[transp[k]]);
  }
  for (int i = 0; i < n; ++i) q_last[i] = e[i];
}

// Real roots of c0 + c1 x + c2 x^2 + c3 x^3 with the convention of Eigen's
// PolynomialSolver::realRoots: every root of the companion matrix whose
// imaginary part is below 1e-12 in magnitude counts, with its real part.
// The roots are found in closed form (trigonometric / Cardano) and polished by
// Newton steps on the original polynomial.
inline std::vector<double> cubic_real_roots(const double c[4]) {
  const double a = c[2] / c[3], b = c[1] / c[3], d = c[0] / c[3];
  // x = t - a/3: t^3 + p t + q = 0
  const double p = b - a * a / 3.0;
  const double q = 2.0 * a * a * a / 27.0 - a * b / 3.0 + d;
  const double disc = q * q / 4.0 + p * p * p / 27.0;
  std::vector<double> roots;
  auto polish = [&](double x) {
    for (int it = 0; it < 3; ++it) {
      const double f = ((c[3] * x + c[2]) * x + c[1]) * x + c[0];
      const double df = (3 * c[3] * x + 2 * c[2]) * x + c[1];
      if (df == 0) break;
      const double nx = x - f / df;
      if (!std::isfinite(nx)) break;
      x = nx;
    }
    return x;
  };
  if (disc > 0) {
    const double sq = std::sqrt(disc);
    const double u = std::cbrt(-q / 2.0 + sq), v = std::cbrt(-q / 2.0 - sq);
    const double t1 = u + v;
    roots.push_back(polish(t1 - a / 3.0));
    const double re = -(u + v) / 2.0 - a / 3.0;
    const double im = std::sqrt(3.0) / 2.0 * (u - v);
    if (std::fabs(im) < 1e-12) {
      roots.push_back(re);
      roots.push_back(re);
    }
  } else {
    const double r = std::sqrt(std::max(0.0, -p / 3.0));
    double arg = r > 0 ? (3.0 * q) / (2.0 * p * r) : 0.0;
    arg = std::max(-1.0, std::min(1.0, arg));
    const double phi = std::acos(arg) / 3.0;
    for (int k = 0; k < 3; ++k) roots.push_back(polish(2 * r * std::cos(phi - 2.0 * M_PI * k / 3.0) - a / 3.0));
  }
  return roots;
}

// Symmetric 3x3 eigen decomposition by cyclic Jacobi rotations; eigenvalues
// descending, eigenvectors in the columns of V (row-major).
inline void sym3_eigen(const double S_in[9], double w[3], double V[9]) {
  double S[9];
  for (int i = 0; i < 9; ++i) S[i] = S_in[i];
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    const double off = S[1] * S[1] + S[2] * S[2] + S[5] * S[5];
    if (off < 1e-300) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        const double apq = S[p * 3 + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = S[p * 3 + p], aqq = S[q * 3 + q];
        const double theta = (aqq - app) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        const double cs = 1 / std::sqrt(t * t + 1), sn = t * cs;
        for (int k = 0; k < 3; ++k) {
          const double skp = S[k * 3 + p], skq = S[k * 3 + q];
          S[k * 3 + p] = cs * skp - sn * skq;
          S[k * 3 + q] = sn * skp + cs * skq;
        }
        for (int k = 0; k < 3; ++k) {
          const double spk = S[p * 3 + k], sqk = S[q * 3 + k];
          S[p * 3 + k] = cs * spk - sn * sqk;
          S[q * 3 + k] = sn * spk + cs * sqk;
        }
        for (int k = 0; k < 3; ++k) {
          const double vkp = V[k * 3 + p], vkq = V[k * 3 + q];
          V[k * 3 + p] = cs * vkp - sn * vkq;
          V[k * 3 + q] = sn * vkp + cs * vkq;
        }
      }
  }
  int idx[3] = {0, 1, 2};
  std::sort(idx, idx + 3, [&](int a, int b) { return S[a * 4] > S[b * 4]; });
  double Vs[9];
  for (int j = 0; j < 3; ++j) {
    w[j] = S[idx[j] * 4];
    for (int i = 0; i < 3; ++i) Vs[i * 3 + j] = V[i * 3 + idx[j]];
  }
  for (int i = 0; i < 9; ++i) V[i] = Vs[i];
}

inline void cross3(const double* a, const double* b, double* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

// SVD of a 3x3 matrix A = U diag(s) V^T (s descending, U and V rotations or
// reflections with U diag(s) V^T = A): V from the eigenvectors of A^T A,
// U columns from A V / s, the last one completed by a cross product.
inline void svd3(const double A[9], double U[9], double s[3], double V[9]) {
  double AtA[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double t = 0;
      for (int k = 0; k < 3; ++k) t += A[k * 3 + i] * A[k * 3 + j];
      AtA[i * 3 + j] = t;
    }
  double w[3];
  sym3_eigen(AtA, w, V);
  for (int j = 0; j < 3; ++j) s[j] = std::sqrt(std::max(0.0, w[j]));
  double cols[3][3];
  for (int j = 0; j < 2; ++j) {
    double u[3];
    for (int i = 0; i < 3; ++i) u[i] = A[i * 3] * V[j] + A[i * 3 + 1] * V[3 + j] + A[i * 3 + 2] * V[6 + j];
    const double nrm = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (int i = 0; i < 3; ++i) cols[j][i] = nrm > 0 ? u[i] / nrm : (i == j ? 1.0 : 0.0);
  }
  cross3(cols[0], cols[1], cols[2]);
  // sign of the third column so that U diag(s) V^T reproduces A
  double u2[3];
  for (int i = 0; i < 3; ++i) u2[i] = A[i * 3] * V[2] + A[i * 3 + 1] * V[5] + A[i * 3 + 2] * V[8];
  if (u2[0] * cols[2][0] + u2[1] * cols[2][1] + u2[2] * cols[2][2] < 0)
    for (int i = 0; i < 3; ++i) cols[2][i] = -cols[2][i];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) U[i * 3 + j] = cols[j][i];
}

// Cholesky (LLT) solve of an n x n SPD system (lower triangle used). Returns
// false if a pivot is not positive.
inline bool llt_solve(std::vector<double> A, int n, const double* b, double* x) {
  for (int j = 0; j < n; ++j) {
    double d = A[j * n + j];
    for (int k = 0; k < j; ++k) d -= A[j * n + k] * A[j * n + k];
    if (!(d > 0)) return false;
    const double l = std::sqrt(d);
    A[j * n + j] = l;
    for (int i = j + 1; i < n; ++i) {
      double s = A[i * n + j];
      for (int k = 0; k < j; ++k) s -= A[i * n + k] * A[j * n + k];
      A[i * n + j] = s / l;
    }
  }
  std::vector<double> y(n);
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= A[i * n + k] * y[k];
    y[i] = s / A[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < n; ++k) s -= A[k * n + i] * x[k];
    x[i] = s / A[i * n + i];
  }
  return true;
}

}  // namespace oracle
