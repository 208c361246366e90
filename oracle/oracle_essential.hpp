// Oracle (test infrastructure only): the essential-matrix estimator of the
// reference (src/pygcransac/include/estimators/essential_estimator.h), its
// minimal solver (solver_essential_matrix_five_point_nister.h with the Sturm
// root isolation of maths/sturm_polynomial_solver.h), its non-minimal solver
// (solver_essential_matrix_five_point_stewenius.h) and the bundle adjustment
// the driver applies to the final inliers (solver_essential_matrix_bundle_
// adjustment.h, relative_pose/essential.cpp, relative_pose/bundle.cpp,
// relative_pose/jacobian_impl.h). Eigen's decompositions are replaced by
// textbook FP64 routines written here; the results agree with Eigen to
// rounding, not bit for bit.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <limits>
#include <vector>

#include "oracle_common.hpp"
#include "oracle_linalg.hpp"
#include "oracle_linalg2.hpp"

namespace oracle {

// ---------------------------------------------------------------------------
// Residuals (essential_estimator.h:186-246). E is row-major: E(i, j) = m[3i+j].
inline double e_sampson2(const double* p, const Model& E) {
  const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
  const double rxc = E[0] * x2 + E[3] * y2 + E[6];
  const double ryc = E[1] * x2 + E[4] * y2 + E[7];
  const double rwc = E[2] * x2 + E[5] * y2 + E[8];
  const double r = (x1 * rxc + y1 * ryc + rwc);
  const double rx = E[0] * x1 + E[1] * y1 + E[2];
  const double ry = E[3] * x1 + E[4] * y1 + E[5];
  return r * r / (rxc * rxc + ryc * ryc + rx * rx + ry * ry);
}

inline double e_symepi2(const double* p, const Model& E) {
  const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
  const double rxc = E[0] * x2 + E[3] * y2 + E[6];
  const double ryc = E[1] * x2 + E[4] * y2 + E[7];
  const double rwc = E[2] * x2 + E[5] * y2 + E[8];
  const double r = (x1 * rxc + y1 * ryc + rwc);
  const double rx = E[0] * x1 + E[1] * y1 + E[2];
  const double ry = E[3] * x1 + E[4] * y1 + E[5];
  const double a = rxc * rxc + ryc * ryc;
  const double b = rx * rx + ry * ry;
  return r * r * (a + b) / (a * b);
}

// getEpipole / isOrientationValid (essential_estimator.h:338-401).
inline bool e_orientation_valid(const Model& E, const Mat& pts, const size_t* s, size_t n) {
  constexpr double epsilon = 1.9984e-15;
  const double r0[3] = {E[0], E[1], E[2]}, r1[3] = {E[3], E[4], E[5]}, r2[3] = {E[6], E[7], E[8]};
  double e[3];
  cross3(r0, r2, e);
  bool big = false;
  for (int i = 0; i < 3; ++i)
    if (e[i] > epsilon || e[i] < -epsilon) big = true;
  if (!big) cross3(r1, r2, e);
  auto sig = [&](const double* p) {
    const double s1 = E[0] * p[2] + E[3] * p[3] + E[6];
    const double s2 = e[1] - e[2] * p[1];
    return s1 * s2;
  };
  const double sg2 = sig(pts.row(s[0]));
  for (size_t i = 1; i < n; ++i)
    if (sg2 * sig(pts.row(s[i])) < 0) return false;
  return true;
}

// Epipolar design row of one correspondence: the coefficients of
// vec(E) (column-major, index 3 j + i for E(i, j)) in x2^T E x1.
inline void e_design_row(const double* p, double w, double* r) {
  const double x0 = p[0], y0 = p[1], x1 = p[2], y1 = p[3];
  const double wx0 = w * x0, wx1 = w * x1, wy0 = w * y0, wy1 = w * y1;
  r[0] = wx0 * x1;
  r[1] = wx0 * y1;
  r[2] = wx0;
  r[3] = wy0 * x1;
  r[4] = wy0 * y1;
  r[5] = wy0;
  r[6] = wx1;
  r[7] = wy1;
  r[8] = w;
}

// ---------------------------------------------------------------------------
// Polynomials in (x, y, z) of degree <= 3, stored over a fixed monomial list.
// The monomial orders are the ones the elimination templates of the two
// five-point solvers are written for.
struct MonoList {
  int n;
  int e[20][3];
  int lut[64];  // monomial index by exponents (x, y, z), each <= 3
  MonoList(int n_, const int (*ex)[3]) : n(n_) {
    for (int i = 0; i < 64; ++i) lut[i] = -1;
    for (int i = 0; i < n; ++i) {
      for (int d = 0; d < 3; ++d) e[i][d] = ex[i][d];
      lut[ex[i][0] * 16 + ex[i][1] * 4 + ex[i][2]] = i;
    }
  }
  int index(int a, int b, int c) const { return lut[a * 16 + b * 4 + c]; }
};
// [x, y, z, 1]
inline const MonoList& mono_lin() {
  static const int ex[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
  static const MonoList m(4, ex);
  return m;
}
// Nister's orders (solver_essential_matrix_five_point_nister.h:123-160)
inline const MonoList& mono_quad_nister() {
  static const int ex[10][3] = {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {1, 0, 0}, {0, 2, 0},
                                {0, 1, 1}, {0, 1, 0}, {0, 0, 2}, {0, 0, 1}, {0, 0, 0}};
  static const MonoList m(10, ex);
  return m;
}
inline const MonoList& mono_cubic_nister() {
  static const int ex[20][3] = {{3, 0, 0}, {0, 3, 0}, {2, 1, 0}, {1, 2, 0}, {2, 0, 1}, {2, 0, 0}, {0, 2, 1},
                                {0, 2, 0}, {1, 1, 1}, {1, 1, 0}, {1, 0, 2}, {1, 0, 1}, {1, 0, 0}, {0, 1, 2},
                                {0, 1, 1}, {0, 1, 0}, {0, 0, 3}, {0, 0, 2}, {0, 0, 1}, {0, 0, 0}};
  static const MonoList m(20, ex);
  return m;
}
// GrevLex orders of the Stewenius solver (solver_essential_matrix_five_point_stewenius.h:236-300)
inline const MonoList& mono_quad_grevlex() {
  static const int ex[10][3] = {{2, 0, 0}, {1, 1, 0}, {0, 2, 0}, {1, 0, 1}, {0, 1, 1},
                                {0, 0, 2}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
  static const MonoList m(10, ex);
  return m;
}
inline const MonoList& mono_cubic_grevlex() {
  static const int ex[20][3] = {{3, 0, 0}, {2, 1, 0}, {1, 2, 0}, {0, 3, 0}, {2, 0, 1}, {1, 1, 1}, {0, 2, 1},
                                {1, 0, 2}, {0, 1, 2}, {0, 0, 3}, {2, 0, 0}, {1, 1, 0}, {0, 2, 0}, {1, 0, 1},
                                {0, 1, 1}, {0, 0, 2}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
  static const MonoList m(20, ex);
  return m;
}

// c (over lc) += sign * (a (over la) * b (over lb)): the terms are added one
// by one in the order of a's monomials, then b's.
inline void poly_mul_acc(const double* a, const MonoList& la, const double* b, const MonoList& lb, double* c,
                         const MonoList& lc, double sign = 1.0) {
  for (int i = 0; i < la.n; ++i) {
    const double ai = sign * a[i];
    for (int j = 0; j < lb.n; ++j) {
      const int k = lc.index(la.e[i][0] + lb.e[j][0], la.e[i][1] + lb.e[j][1], la.e[i][2] + lb.e[j][2]);
      c[k] += ai * b[j];
    }
  }
}

// ---------------------------------------------------------------------------
// Partial-pivoting LU solve A X = B (Eigen's partialPivLu().solve): A n x n,
// B n x m, both row-major; X overwrites B.
inline void partial_piv_lu_solve(std::vector<double> A, int n, std::vector<double>& B, int m) {
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::fabs(A[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i * n + k]) > best) { best = std::fabs(A[i * n + k]); p = i; }
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
      std::swap(perm[k], perm[p]);
    }
    if (A[k * n + k] != 0.0)
      for (int i = k + 1; i < n; ++i) A[i * n + k] /= A[k * n + k];
    for (int i = k + 1; i < n; ++i)
      for (int j = k + 1; j < n; ++j) A[i * n + j] -= A[i * n + k] * A[k * n + j];
  }
  std::vector<double> X((size_t)n * m);
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < m; ++c) X[i * m + c] = B[perm[i] * m + c];
  for (int c = 0; c < m; ++c) {
    for (int i = 0; i < n; ++i) {
      double s = X[i * m + c];
      for (int q = 0; q < i; ++q) s -= A[i * n + q] * X[q * m + c];
      X[i * m + c] = s;
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = X[i * m + c];
      for (int q = i + 1; q < n; ++q) s -= A[i * n + q] * X[q * m + c];
      X[i * m + c] = s / A[i * n + i];
    }
  }
  B = X;
}

// Full-pivoting LU solve A X = B (Eigen's FullPivLU::solve): A r x c, B r x m;
// returns X c x m. Unknowns past the numerical rank are set to zero.
inline std::vector<double> full_piv_lu_solve(std::vector<double> A, int r, int c, const std::vector<double>& B,
                                             int m) {
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
  const double thr = std::numeric_limits<double>::epsilon() * (double)sz;
  int rank = 0;
  for (int i = 0; i < nonzero; ++i)
    if (std::fabs(A[i * c + i]) > thr * maxpivot) ++rank;
  std::vector<double> X((size_t)c * m, 0.0);
  for (int col = 0; col < m; ++col) {
    std::vector<double> y(r);
    for (int i = 0; i < r; ++i) y[i] = B[rp[i] * m + col];
    for (int i = 0; i < sz; ++i)
      for (int q = 0; q < i; ++q) y[i] -= A[i * c + q] * y[q];
    for (int i = rank - 1; i >= 0; --i) {
      double s = y[i];
      for (int q = i + 1; q < rank; ++q) s -= A[i * c + q] * y[q];
      y[i] = s / A[i * c + i];
    }
    for (int i = 0; i < rank; ++i) X[cp[i] * m + col] = y[i];
  }
  return X;
}

// Householder QR with column pivoting of an n x n matrix (the pivot is the
// remaining column of largest norm, recomputed at every step); returns the
// last `k` columns of Q (n x k, row-major) — the null space that
// ColPivHouseholderQR(M).matrixQ().rightCols<k>() gives.
inline std::vector<double> colpiv_qr_q_rightcols(std::vector<double> A, int n, int k) {
  std::vector<std::vector<double>> vs;
  std::vector<double> taus;
  for (int s = 0; s < n; ++s) {
    int p = s;
    double best = -1;
    for (int j = s; j < n; ++j) {
      double t = 0;
      for (int i = s; i < n; ++i) t += A[i * n + j] * A[i * n + j];
      if (t > best) { best = t; p = j; }
    }
    if (p != s)
      for (int i = 0; i < n; ++i) std::swap(A[i * n + s], A[i * n + p]);
    const double c0 = A[s * n + s];
    double tail = 0;
    for (int i = s + 1; i < n; ++i) tail += A[i * n + s] * A[i * n + s];
    std::vector<double> v(n - s, 0.0);
    double tau, beta;
    v[0] = 1;
    if (tail <= std::numeric_limits<double>::min()) {
      tau = 0;
      beta = c0;
    } else {
      beta = std::sqrt(c0 * c0 + tail);
      if (c0 >= 0) beta = -beta;
      for (int i = s + 1; i < n; ++i) v[i - s] = A[i * n + s] / (c0 - beta);
      tau = (beta - c0) / beta;
    }
    for (int j = s; j < n; ++j) {
      double t = 0;
      for (int i = s; i < n; ++i) t += v[i - s] * A[i * n + j];
      t *= tau;
      for (int i = s; i < n; ++i) A[i * n + j] -= t * v[i - s];
    }
    vs.push_back(v);
    taus.push_back(tau);
  }
  std::vector<double> Q((size_t)n * k, 0.0);
  for (int c = 0; c < k; ++c) {
    std::vector<double> e(n, 0.0);
    e[n - k + c] = 1;
    for (int s = n - 1; s >= 0; --s) {
      const std::vector<double>& v = vs[s];
      double t = 0;
      for (int i = s; i < n; ++i) t += v[i - s] * e[i];
      t *= taus[s];
      for (int i = s; i < n; ++i) e[i] -= t * v[i - s];
    }
    for (int i = 0; i < n; ++i) Q[i * k + c] = e[i];
  }
  return Q;
}

// Eigenvalues of a real n x n matrix: Householder reduction to upper
// Hessenberg form, then Francis double-shift QR iterations with
// Wilkinson-style deflation (the EISPACK hqr scheme). A pair deflated from a
// 2 x 2 block with a non-negative discriminant gives two real eigenvalues
// (imaginary part exactly zero), otherwise a complex pair. Returns false when
// an eigenvalue did not converge in 30 iterations.
inline bool real_eigenvalues(std::vector<double> a, int n, std::vector<double>& wr, std::vector<double>& wi) {
  // Hessenberg reduction
  for (int k = 0; k < n - 2; ++k) {
    double alpha = 0;
    for (int i = k + 1; i < n; ++i) alpha += a[i * n + k] * a[i * n + k];
    if (alpha == 0) continue;
    alpha = std::sqrt(alpha);
    if (a[(k + 1) * n + k] > 0) alpha = -alpha;
    std::vector<double> v(n, 0.0);
    for (int i = k + 1; i < n; ++i) v[i] = a[i * n + k];
    v[k + 1] -= alpha;
    double vn = 0;
    for (int i = k + 1; i < n; ++i) vn += v[i] * v[i];
    if (vn == 0) continue;
    // A <- (I - 2 v v^T / vn) A (I - 2 v v^T / vn)
    for (int j = 0; j < n; ++j) {
      double s = 0;
      for (int i = k + 1; i < n; ++i) s += v[i] * a[i * n + j];
      s = 2 * s / vn;
      for (int i = k + 1; i < n; ++i) a[i * n + j] -= s * v[i];
    }
    for (int i = 0; i < n; ++i) {
      double s = 0;
      for (int j = k + 1; j < n; ++j) s += a[i * n + j] * v[j];
      s = 2 * s / vn;
      for (int j = k + 1; j < n; ++j) a[i * n + j] -= s * v[j];
    }
    for (int i = k + 2; i < n; ++i) a[i * n + k] = 0;
  }
  wr.assign(n, 0.0);
  wi.assign(n, 0.0);
  auto A = [&](int i, int j) -> double& { return a[i * n + j]; };
  double anorm = 0;
  for (int i = 0; i < n; ++i)
    for (int j = std::max(i - 1, 0); j < n; ++j) anorm += std::fabs(A(i, j));
  int nn = n - 1;
  double t = 0;
  while (nn >= 0) {
    int its = 0, l;
    for (;;) {
      // look for a negligible subdiagonal element
      for (l = nn; l >= 1; --l) {
        double s = std::fabs(A(l - 1, l - 1)) + std::fabs(A(l, l));
        if (s == 0) s = anorm;
        if (std::fabs(A(l, l - 1)) + s == s) {
          A(l, l - 1) = 0;
          break;
        }
      }
      double x = A(nn, nn);
      if (l == nn) {  // one eigenvalue
        wr[nn] = x + t;
        wi[nn] = 0;
        --nn;
        break;
      }
      double y = A(nn - 1, nn - 1);
      double w = A(nn, nn - 1) * A(nn - 1, nn);
      if (l == nn - 1) {  // two eigenvalues
        const double p = 0.5 * (y - x);
        const double q = p * p + w;
        double z = std::sqrt(std::fabs(q));
        x += t;
        if (q >= 0) {
          z = p + (p >= 0 ? std::fabs(z) : -std::fabs(z));
          wr[nn - 1] = wr[nn] = x + z;
          if (z != 0) wr[nn] = x - w / z;
          wi[nn - 1] = wi[nn] = 0;
        } else {
          wr[nn - 1] = wr[nn] = x + p;
          wi[nn - 1] = -z;
          wi[nn] = z;
        }
        nn -= 2;
        break;
      }
      if (its == 30) return false;
      if (its == 10 || its == 20) {  // exceptional shift
        t += x;
        for (int i = 0; i <= nn; ++i) A(i, i) -= x;
        const double s = std::fabs(A(nn, nn - 1)) + std::fabs(A(nn - 1, nn - 2));
        x = y = 0.75 * s;
        w = -0.4375 * s * s;
      }
      ++its;
      int m;
      double p = 0, q = 0, r = 0, z;
      for (m = nn - 2; m >= l; --m) {
        z = A(m, m);
        r = x - z;
        double s = y - z;
        p = (r * s - w) / A(m + 1, m) + A(m, m + 1);
        q = A(m + 1, m + 1) - z - r - s;
        r = A(m + 2, m + 1);
        s = std::fabs(p) + std::fabs(q) + std::fabs(r);
        p /= s;
        q /= s;
        r /= s;
        if (m == l) break;
        const double u = std::fabs(A(m, m - 1)) * (std::fabs(q) + std::fabs(r));
        const double v = std::fabs(p) * (std::fabs(A(m - 1, m - 1)) + std::fabs(z) + std::fabs(A(m + 1, m + 1)));
        if (u + v == v) break;
      }
      for (int i = m + 2; i <= nn; ++i) {
        A(i, i - 2) = 0;
        if (i != m + 2) A(i, i - 3) = 0;
      }
      for (int k = m; k <= nn - 1; ++k) {
        if (k != m) {
          p = A(k, k - 1);
          q = A(k + 1, k - 1);
          r = 0;
          if (k != nn - 1) r = A(k + 2, k - 1);
          x = std::fabs(p) + std::fabs(q) + std::fabs(r);
          if (x != 0) {
            p /= x;
            q /= x;
            r /= x;
          }
        }
        double s = std::sqrt(p * p + q * q + r * r);
        if (p < 0) s = -s;
        if (s != 0) {
          if (k == m) {
            if (l != m) A(k, k - 1) = -A(k, k - 1);
          } else {
            A(k, k - 1) = -s * x;
          }
          p += s;
          x = p / s;
          y = q / s;
          z = r / s;
          q /= p;
          r /= p;
          for (int j = k; j <= nn; ++j) {  // row modification
            p = A(k, j) + q * A(k + 1, j);
            if (k != nn - 1) {
              p += r * A(k + 2, j);
              A(k + 2, j) -= p * z;
            }
            A(k + 1, j) -= p * y;
            A(k, j) -= p * x;
          }
          const int mmin = nn < k + 3 ? nn : k + 3;
          for (int i = l; i <= mmin; ++i) {  // column modification
            p = x * A(i, k) + y * A(i, k + 1);
            if (k != nn - 1) {
              p += z * A(i, k + 2);
              A(i, k + 2) -= p * r;
            }
            A(i, k + 1) -= p * q;
            A(i, k) -= p;
          }
        }
      }
    }
  }
  return true;
}

// A null vector of the n x n matrix M (rank n - 1): LU with complete pivoting
// over n - 1 steps, the last pivoted unknown set to one.
inline std::vector<double> null_vector(std::vector<double> M, int n) {
  std::vector<int> cp(n);
  for (int j = 0; j < n; ++j) cp[j] = j;
  for (int k = 0; k < n - 1; ++k) {
    int bi = k, bj = k;
    double best = -1;
    for (int i = k; i < n; ++i)
      for (int j = k; j < n; ++j) {
        const double v = std::fabs(M[i * n + j]);
        if (v > best) { best = v; bi = i; bj = j; }
      }
    if (bi != k)
      for (int j = 0; j < n; ++j) std::swap(M[k * n + j], M[bi * n + j]);
    if (bj != k) {
      for (int i = 0; i < n; ++i) std::swap(M[i * n + k], M[i * n + bj]);
      std::swap(cp[k], cp[bj]);
    }
    if (M[k * n + k] == 0) continue;
    for (int i = k + 1; i < n; ++i) {
      const double f = M[i * n + k] / M[k * n + k];
      for (int j = k + 1; j < n; ++j) M[i * n + j] -= f * M[k * n + j];
      M[i * n + k] = 0;
    }
  }
  std::vector<double> y(n, 0.0);
  y[n - 1] = 1.0;
  for (int i = n - 2; i >= 0; --i) {
    double s = -M[i * n + n - 1];
    for (int q = i + 1; q < n - 1; ++q) s -= M[i * n + q] * y[q];
    y[i] = M[i * n + i] != 0 ? s / M[i * n + i] : 0.0;
  }
  std::vector<double> x(n);
  for (int i = 0; i < n; ++i) x[cp[i]] = y[i];
  return x;
}

// ---------------------------------------------------------------------------
// Sturm-sequence root isolation of a degree-N polynomial (ascending
// coefficients) as in sturm_polynomial_solver.h:223-262: normalise by the
// leading coefficient, build the sequence with the remainder recurrence,
// bisect the Cauchy interval while more than one root lies inside, then
// Ridders' method and Newton steps on each isolated root (tolerance 1e-10).
struct Sturm {
  static constexpr int N = 10;
  double f[2 * N + 1];  // monic polynomial, then its scaled derivative
  double sv[3 * N];
  double polyval(const double* p, int deg, double x) const {  // p monic of degree deg
    double v = x + p[deg - 1];
    for (int i = deg - 2; i >= 0; --i) v = x * v + p[i];
    return v;
  }
  void build() {
    double buf[3 * N];
    double* f1 = buf;
    double* f2 = f1 + N + 1;
    double* f3 = f2 + N;
    for (int i = 0; i < 2 * N + 1; ++i) buf[i] = f[i];
    for (int i = 0; i < N - 1; ++i) {
      const double q1 = f1[N - i] * f2[N - 1 - i];
      const double q0 = f1[N - 1 - i] * f2[N - 1 - i] - f1[N - i] * f2[N - 2 - i];
      f3[0] = f1[0] - q0 * f2[0];
      for (int j = 1; j < N - 1 - i; ++j) f3[j] = f1[j] - q1 * f2[j - 1] - q0 * f2[j];
      const double c = -std::fabs(f3[N - 2 - i]);
      const double ci = 1.0 / c;
      for (int j = 0; j < N - 1 - i; ++j) f3[j] = f3[j] * ci;
      double* t = f1;
      f1 = f2;
      f2 = f3;
      f3 = t;
      sv[3 * i] = q0;
      sv[3 * i + 1] = q1;
      sv[3 * i + 2] = c;
    }
    sv[3 * N - 3] = f1[0];
    sv[3 * N - 2] = f1[1];
    sv[3 * N - 1] = f2[0];
  }
  int sign_changes(double x) const {
    double v[N + 1];
    v[N] = sv[3 * N - 1];
    v[N - 1] = sv[3 * N - 3] + x * sv[3 * N - 2];
    for (int i = N - 2; i >= 0; --i) v[i] = (sv[3 * i] + x * sv[3 * i + 1]) * v[i + 1] + sv[3 * i + 2] * v[i + 2];
    int cnt = 0;
    for (int i = 0; i < N; ++i)
      if ((v[i] < 0) != (v[i + 1] < 0)) ++cnt;
    return cnt;
  }
  void refine(double a, double b, double* roots, int& nr, double tol) const {
    double fa = polyval(f, N, a), fb = polyval(f, N, b);
    if (!((fa < 0) ^ (fb < 0))) return;
    for (int it = 0; it < 30; ++it) {
      if (std::fabs(a - b) < 1e-3) break;
      const double c = (a + b) * 0.5;
      const double fc = polyval(f, N, c);
      const double s = std::sqrt(fc * fc - fa * fb);
      if (!s) break;
      const double d = (fa < fb) ? c + (a - c) * fc / s : c + (c - a) * fc / s;
      const double fd = polyval(f, N, d);
      if (fd >= 0 ? (fc < 0) : (fc > 0)) {
        a = c; fa = fc; b = d; fb = fd;
      } else if (fd >= 0 ? (fa < 0) : (fa > 0)) {
        b = d; fb = fd;
      } else {
        a = d; fa = fd;
      }
    }
    double x = (a + b) * 0.5;
    for (int it = 0; it < 10; ++it) {
      const double fx = polyval(f, N, x);
      if (std::fabs(fx) < tol) break;
      const double fpx = (double)N * polyval(f + N + 1, N - 1, x);
      const double dx = fx / fpx;
      x = x - dx;
      if (std::fabs(dx) < tol) break;
    }
    roots[nr++] = x;
  }
  void isolate(double a, double b, int sa, int sb, double* roots, int& nr, double tol, int depth) const {
    if (depth > 30) return;
    const int n = sa - sb;
    if (n > 1) {
      const double c = (a + b) * 0.5;
      const int sc = sign_changes(c);
      isolate(a, c, sa, sc, roots, nr, tol, depth + 1);
      isolate(c, b, sc, sb, roots, nr, tol, depth + 1);
    } else if (n == 1) {
      refine(a, b, roots, nr, tol);
    }
  }
  int solve(const double* coeffs, double* roots, double tol = 1e-10) {
    if (coeffs[N] == 0.0) return 0;
    for (int i = 0; i <= N; ++i) f[i] = coeffs[i];
    const double ci = 1.0 / f[N];
    for (int i = 0; i < N; ++i) f[i] *= ci;
    f[N] = 1.0;
    for (int i = 0; i < N - 1; ++i) f[N + 1 + i] = f[i + 1] * ((i + 1) / (double)N);
    f[2 * N] = 1.0;
    build();
    double mx = 0;
    for (int i = 0; i < N; ++i) mx = std::max(mx, std::fabs(f[i]));
    const double r0 = 1.0 + mx;
    const int sa = sign_changes(-r0), sb = sign_changes(r0);
    if (sa - sb == 0) return 0;
    int nr = 0;
    isolate(-r0, r0, sa, sb, roots, nr, tol, 0);
    return nr;
  }
};

// ---------------------------------------------------------------------------
// EssentialMatrixFivePointNisterSolver::estimateModel (nister.h:263-615) on a
// minimal sample with unit weights.
inline bool e_nister5(const Mat& pts, const size_t* s, std::vector<Model>& models) {
  std::vector<double> D(5 * 9);
  for (int i = 0; i < 5; ++i) e_design_row(pts.row(s[i]), 1.0, &D[i * 9]);
  std::vector<double> K;
  if (fullpiv_lu_kernel(D, 5, 9, K) != 4) return false;
  // EE[k] = coefficients of vec(E)[k] over [x, y, z, 1]: basis vector j of the
  // kernel multiplies monomial j
  double EE[9][4];
  for (int k = 0; k < 9; ++k)
    for (int j = 0; j < 4; ++j) EE[k][j] = K[k * 4 + j];
  auto E_ = [&](int i, int j) { return EE[3 * j + i]; };
  const MonoList &L = mono_lin(), &Q = mono_quad_nister(), &C = mono_cubic_nister();
  std::vector<double> coeffs(10 * 20, 0.0);
  // determinant (row 9)
  {
    double* row = &coeffs[9 * 20];
    const int third[3] = {0, 1, 2};
    // E20 (E01 E12 - E02 E11) + E21 (E02 E10 - E00 E12) + E22 (E00 E11 - E01 E10)
    const int pr[3][8] = {{0, 1, 1, 2, 0, 2, 1, 1}, {0, 2, 1, 0, 0, 0, 1, 2}, {0, 0, 1, 1, 0, 1, 1, 0}};
    for (int t = 0; t < 3; ++t) {
      double d[10] = {0};
      poly_mul_acc(E_(pr[t][0], pr[t][1]), L, E_(pr[t][2], pr[t][3]), L, d, Q);
      poly_mul_acc(E_(pr[t][4], pr[t][5]), L, E_(pr[t][6], pr[t][7]), L, d, Q, -1.0);
      poly_mul_acc(d, Q, E_(2, third[t]), L, row, C);
    }
  }
  // EE^T - 1/2 trace(EE^T) I, then times E (rows 0..8, row 3 i + j)
  double EET[3][3][10];
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) {
      double* c = EET[i][j];
      for (int q = 0; q < 10; ++q) c[q] = 0;
      for (int k = 0; k < 3; ++k) poly_mul_acc(E_(i, k), L, E_(j, k), L, c, Q);
    }
  for (int q = 0; q < 10; ++q) {
    const double t = 0.5 * (EET[0][0][q] + EET[1][1][q] + EET[2][2][q]);
    EET[0][0][q] -= t;
    EET[1][1][q] -= t;
    EET[2][2][q] -= t;
  }
  auto eet = [&](int i, int j) -> const double* { return i <= j ? EET[i][j] : EET[j][i]; };
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double* row = &coeffs[(3 * i + j) * 20];
      for (int k = 0; k < 3; ++k) poly_mul_acc(eet(i, k), Q, E_(k, j), L, row, C);
    }
  // eliminate: right 10 x 10 block <- left^-1 right
  std::vector<double> left(100), right(100);
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) {
      left[i * 10 + j] = coeffs[i * 20 + j];
      right[i * 10 + j] = coeffs[i * 20 + 10 + j];
    }
  partial_piv_lu_solve(left, 10, right, 10);
  auto R = [&](int i, int j) { return right[i * 10 + j]; };  // coeffs(i, 10 + j)
  double A[3][13];
  for (int i = 0; i < 3; ++i) {
    const int a = 4 + 2 * i, b = 5 + 2 * i;
    A[i][0] = -R(b, 0);
    A[i][1] = R(a, 0) - R(b, 1);
    A[i][2] = R(a, 1) - R(b, 2);
    A[i][3] = R(a, 2);
    A[i][4] = -R(b, 3);
    A[i][5] = R(a, 3) - R(b, 4);
    A[i][6] = R(a, 4) - R(b, 5);
    A[i][7] = R(a, 5);
    A[i][8] = -R(b, 6);
    A[i][9] = R(a, 6) - R(b, 7);
    A[i][10] = R(a, 7) - R(b, 8);
    A[i][11] = R(a, 8) - R(b, 9);
    A[i][12] = R(a, 9);
  }
  // det of [col0 (cubic) | col1 (cubic) | col2 (quartic)] in z, ascending
  auto pmul = [](const double* a, int na, const double* b, int nb, double* c) {  // c = a * b
    for (int i = 0; i < na + nb - 1; ++i) c[i] = 0;
    for (int i = 0; i < na; ++i)
      for (int j = 0; j < nb; ++j) c[i + j] += a[i] * b[j];
  };
  double P[3][3][5];
  for (int i = 0; i < 3; ++i) {
    for (int k = 0; k < 4; ++k) {
      P[i][0][k] = A[i][3 - k];
      P[i][1][k] = A[i][7 - k];
    }
    for (int k = 0; k < 5; ++k) P[i][2][k] = A[i][12 - k];
  }
  double poly[11] = {0};
  {
    double t1[8], t2[8], m0[8], t3[8], t4[8], m1[8], t5[7], t6[7], m2[7], u[11];
    pmul(P[1][1], 4, P[2][2], 5, t1);
    pmul(P[1][2], 5, P[2][1], 4, t2);
    for (int k = 0; k < 8; ++k) m0[k] = t1[k] - t2[k];
    pmul(P[1][0], 4, P[2][2], 5, t3);
    pmul(P[1][2], 5, P[2][0], 4, t4);
    for (int k = 0; k < 8; ++k) m1[k] = t3[k] - t4[k];
    pmul(P[1][0], 4, P[2][1], 4, t5);
    pmul(P[1][1], 4, P[2][0], 4, t6);
    for (int k = 0; k < 7; ++k) m2[k] = t5[k] - t6[k];
    pmul(P[0][0], 4, m0, 8, u);
    for (int k = 0; k < 11; ++k) poly[k] += u[k];
    pmul(P[0][1], 4, m1, 8, u);
    for (int k = 0; k < 11; ++k) poly[k] -= u[k];
    pmul(P[0][2], 5, m2, 7, u);
    for (int k = 0; k < 11; ++k) poly[k] += u[k];
  }
  Sturm st;
  double roots[10];
  const int nr = st.solve(poly, roots);
  for (int r = 0; r < nr; ++r) {
    const double z = roots[r], z2 = z * z, z3 = z2 * z, z4 = z2 * z2;
    double B[3][2], b[3];
    for (int i = 0; i < 3; ++i) {
      B[i][0] = A[i][0] * z3 + A[i][1] * z2 + A[i][2] * z + A[i][3];
      B[i][1] = A[i][4] * z3 + A[i][5] * z2 + A[i][6] * z + A[i][7];
      b[i] = A[i][8] * z4 + A[i][9] * z3 + A[i][10] * z2 + A[i][11] * z + A[i][12];
    }
    const double det = B[0][0] * B[1][1] - B[1][0] * B[0][1];
    const double id = 1.0 / det;
    const double i00 = B[1][1] * id, i01 = -B[0][1] * id, i10 = -B[1][0] * id, i11 = B[0][0] * id;
    double xz0 = i00 * b[0] + i01 * b[1], xz1 = i10 * b[0] + i11 * b[1];
    if (std::fabs(B[2][0] * xz0 + B[2][1] * xz1 - b[2]) > 1e-6) {
      std::vector<double> M = {B[0][0], B[0][1], B[1][0], B[1][1], B[2][0], B[2][1]};
      std::vector<double> rhs = {b[0], b[1], b[2]};
      const std::vector<double> X = full_piv_lu_solve(M, 3, 2, rhs, 1);
      xz0 = X[0];
      xz1 = X[1];
    }
    const double x = -xz0, y = -xz1;
    const double sc = 1.0 / std::sqrt(x * x + y * y + z * z + 1.0);
    Model E;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double* c = EE[3 * j + i];
        E[3 * i + j] = (c[0] * x + c[1] * y + c[2] * z + c[3]) * sc;
      }
    models.push_back(E);
  }
  return !models.empty();
}

// ---------------------------------------------------------------------------
// EssentialMatrixFivePointSteweniusSolver::estimateModel (stewenius.h:114-234).
// Weights are read by point index, like the reference.
inline bool e_stewenius(const Mat& pts, const size_t* s, size_t n, const double* weights,
                        std::vector<Model>& models) {
  std::vector<double> D(n * 9);
  for (size_t i = 0; i < n; ++i) e_design_row(pts.row(s[i]), weights ? weights[s[i]] : 1.0, &D[i * 9]);
  // null space: 9 x 4, column j multiplies monomial j of [x, y, z, 1]
  std::vector<double> Nsp(36);
  if (n == 5) {
    std::vector<double> K;
    if (fullpiv_lu_kernel(D, 5, 9, K) != 4) return false;
    Nsp = K;
  } else {
    std::vector<double> AtA(81, 0.0);
    for (int a = 0; a < 9; ++a)
      for (int b = 0; b < 9; ++b) {
        double t = 0;
        for (size_t i = 0; i < n; ++i) t += D[i * 9 + a] * D[i * 9 + b];
        AtA[a * 9 + b] = t;
      }
    Nsp = colpiv_qr_q_rightcols(AtA, 9, 4);
  }
  auto NS = [&](int i, int j) { return &Nsp[(3 * j + i) * 4]; };  // E(i, j) over [x, y, z, 1]
  const MonoList &L = mono_lin(), &Q = mono_quad_grevlex(), &C = mono_cubic_grevlex();
  std::vector<double> cm(10 * 20, 0.0);
  // trace constraint rows 0..8: (2 E E^T) E - 1/2 trace(2 E E^T) E
  double eet[3][3][10];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double t[10] = {0};
      for (int k = 0; k < 3; ++k) poly_mul_acc(NS(i, k), L, NS(j, k), L, t, Q);
      for (int q = 0; q < 10; ++q) eet[i][j][q] = 2 * t[q];
    }
  double tr[10];
  for (int q = 0; q < 10; ++q) tr[q] = eet[0][0][q] + eet[1][1][q] + eet[2][2][q];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double row[20] = {0}, tt[20] = {0};
      for (int k = 0; k < 3; ++k) poly_mul_acc(eet[i][k], Q, NS(k, j), L, row, C);
      poly_mul_acc(tr, Q, NS(i, j), L, tt, C);
      for (int q = 0; q < 20; ++q) cm[(3 * i + j) * 20 + q] = row[q] - 0.5 * tt[q];
    }
  // determinant row 9
  {
    const int pr[3][8] = {{0, 1, 1, 2, 0, 2, 1, 1}, {0, 2, 1, 0, 0, 0, 1, 2}, {0, 0, 1, 1, 0, 1, 1, 0}};
    double row[20] = {0};
    for (int t = 0; t < 3; ++t) {
      double d[10] = {0};
      poly_mul_acc(NS(pr[t][0], pr[t][1]), L, NS(pr[t][2], pr[t][3]), L, d, Q);
      poly_mul_acc(NS(pr[t][4], pr[t][5]), L, NS(pr[t][6], pr[t][7]), L, d, Q, -1.0);
      poly_mul_acc(d, Q, NS(2, t), L, row, C);
    }
    for (int q = 0; q < 20; ++q) cm[9 * 20 + q] = row[q];
  }
  std::vector<double> left(100), right(100);
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) {
      left[i * 10 + j] = cm[i * 20 + j];
      right[i * 10 + j] = cm[i * 20 + 10 + j];
    }
  const std::vector<double> el = full_piv_lu_solve(left, 10, 10, right, 10);
  std::vector<double> act(100, 0.0);
  const int src[6] = {0, 1, 2, 4, 5, 7};
  for (int r = 0; r < 6; ++r)
    for (int j = 0; j < 10; ++j) act[r * 10 + j] = el[src[r] * 10 + j];
  act[6 * 10 + 0] = -1.0;
  act[7 * 10 + 1] = -1.0;
  act[8 * 10 + 3] = -1.0;
  act[9 * 10 + 6] = -1.0;
  std::vector<double> wr, wi;
  if (!real_eigenvalues(act, 10, wr, wi)) return false;
  for (int i = 0; i < 10; ++i) {
    if (wi[i] != 0) continue;
    std::vector<double> M = act;
    for (int d = 0; d < 10; ++d) M[d * 10 + d] -= wr[i];
    const std::vector<double> v = null_vector(M, 10);
    Model E;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        const double* ns = NS(r, c);
        E[3 * r + c] = ns[0] * v[6] + ns[1] * v[7] + ns[2] * v[8] + ns[3] * v[9];
      }
    models.push_back(E);
  }
  return !models.empty();
}

// ---------------------------------------------------------------------------
// Relative pose and its bundle adjustment (relative_pose/*).
struct Pose {
  double q[4];  // w, x, y, z
  double t[3];
};

inline void quat_to_R(const double* q, double* R) {
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  const double twx = tx * w, twy = ty * w, twz = tz * w;
  const double txx = tx * x, txy = ty * x, txz = tz * x;
  const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
  R[0] = 1 - (tyy + tzz); R[1] = txy - twz;       R[2] = txz + twy;
  R[3] = txy + twz;       R[4] = 1 - (txx + tzz); R[5] = tyz - twx;
  R[6] = txz - twy;       R[7] = tyz + twx;       R[8] = 1 - (txx + tyy);
}

// rotation matrix to unit quaternion (Shepperd's method), then normalised
inline void R_to_quat(const double* R, double* q) {
  const double tr = R[0] + R[4] + R[8];
  double w, v[3];
  if (tr > 0) {
    double t = std::sqrt(tr + 1.0);
    w = 0.5 * t;
    t = 0.5 / t;
    v[0] = (R[7] - R[5]) * t;
    v[1] = (R[2] - R[6]) * t;
    v[2] = (R[3] - R[1]) * t;
  } else {
    int i = 0;
    if (R[4] > R[0]) i = 1;
    if (R[8] > R[i * 4]) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    double t = std::sqrt(R[i * 4] - R[j * 4] - R[k * 4] + 1.0);
    v[i] = 0.5 * t;
    t = 0.5 / t;
    w = (R[k * 3 + j] - R[j * 3 + k]) * t;
    v[j] = (R[j * 3 + i] + R[i * 3 + j]) * t;
    v[k] = (R[k * 3 + i] + R[i * 3 + k]) * t;
  }
  const double n = std::sqrt(w * w + v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  q[0] = w / n;
  q[1] = v[0] / n;
  q[2] = v[1] / n;
  q[3] = v[2] / n;
}

// essential_from_motion (essential.cpp:34-39): E = [t]x R
inline Model essential_from_pose(const Pose& P) {
  double R[9];
  quat_to_R(P.q, R);
  const double S[9] = {0.0, -P.t[2], P.t[1], P.t[2], 0.0, -P.t[0], -P.t[1], P.t[0], 0.0};
  Model E;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) E[3 * i + j] = S[3 * i] * R[j] + S[3 * i + 1] * R[3 + j] + S[3 * i + 2] * R[6 + j];
  return E;
}

// check_cheirality (essential.cpp:42-57) with unit bearing vectors, depth 0
inline bool cheirality_ok(const Pose& P, const double* x1, const double* x2) {
  double R[9];
  quat_to_R(P.q, R);
  double Rx1[3];
  for (int i = 0; i < 3; ++i) Rx1[i] = R[3 * i] * x1[0] + R[3 * i + 1] * x1[1] + R[3 * i + 2] * x1[2];
  const double a = -(Rx1[0] * x2[0] + Rx1[1] * x2[1] + Rx1[2] * x2[2]);
  const double b1 = -(Rx1[0] * P.t[0] + Rx1[1] * P.t[1] + Rx1[2] * P.t[2]);
  const double b2 = x2[0] * P.t[0] + x2[1] * P.t[1] + x2[2] * P.t[2];
  const double l1 = b1 - a * b2;
  const double l2 = -a * b1 + b2;
  const double md = 0.0 * (1 - a * a);
  return l1 > md && l2 > md;
}

// motion_from_essential (essential.cpp:59-132): the four (R, t) candidates of
// E, kept when the correspondence (x1, x2) lies in front of both cameras.
inline void poses_from_essential(const Model& E, const double* x1, const double* x2, std::vector<Pose>& out) {
  auto col = [&](int j, double* c) { c[0] = E[j]; c[1] = E[3 + j]; c[2] = E[6 + j]; };
  double c0[3], c1[3], c2[3];
  col(0, c0);
  col(1, c1);
  col(2, c2);
  double u12[3], u13[3], u23[3];
  cross3(c0, c1, u12);
  cross3(c0, c2, u13);
  cross3(c1, c2, u23);
  auto sq = [](const double* v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; };
  const double n12 = sq(u12), n13 = sq(u13), n23 = sq(u23);
  double UW[3][3];  // UW[col][row]
  auto set_cols = [&](const double* a, const double* u, double nu) {
    const double na = std::sqrt(sq(a));
    for (int i = 0; i < 3; ++i) {
      UW[1][i] = a[i] / na;
      UW[2][i] = u[i] / std::sqrt(nu);
    }
  };
  if (n12 > n13) {
    if (n12 > n23) set_cols(c0, u12, n12);
    else set_cols(c1, u23, n23);
  } else {
    if (n13 > n23) set_cols(c0, u13, n13);
    else set_cols(c1, u23, n23);
  }
  double t0[3];
  cross3(UW[2], UW[1], t0);
  for (int i = 0; i < 3; ++i) UW[0][i] = -t0[i];
  double Vt[3][3];
  for (int j = 0; j < 3; ++j) {
    Vt[0][j] = UW[1][0] * E[j] + UW[1][1] * E[3 + j] + UW[1][2] * E[6 + j];
    Vt[1][j] = -UW[0][0] * E[j] + -UW[0][1] * E[3 + j] + -UW[0][2] * E[6 + j];
  }
  {
    const double n0 = std::sqrt(sq(Vt[0]));
    for (int j = 0; j < 3; ++j) Vt[0][j] /= n0;
    const double d = Vt[0][0] * Vt[1][0] + Vt[0][1] * Vt[1][1] + Vt[0][2] * Vt[1][2];
    for (int j = 0; j < 3; ++j) Vt[1][j] -= d * Vt[0][j];
    const double n1 = std::sqrt(sq(Vt[1]));
    for (int j = 0; j < 3; ++j) Vt[1][j] /= n1;
    cross3(Vt[0], Vt[1], Vt[2]);
  }
  auto rot = [&](double* q) {
    double R[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) R[3 * i + j] = UW[0][i] * Vt[0][j] + UW[1][i] * Vt[1][j] + UW[2][i] * Vt[2][j];
    R_to_quat(R, q);
  };
  Pose P;
  rot(P.q);
  for (int i = 0; i < 3; ++i) P.t[i] = UW[2][i];
  if (cheirality_ok(P, x1, x2)) out.push_back(P);
  for (int i = 0; i < 3; ++i) P.t[i] = -P.t[i];
  if (cheirality_ok(P, x1, x2)) out.push_back(P);
  for (int c = 0; c < 2; ++c)
    for (int i = 0; i < 3; ++i) UW[c][i] = -UW[c][i];
  rot(P.q);
  if (cheirality_ok(P, x1, x2)) out.push_back(P);
  for (int i = 0; i < 3; ++i) P.t[i] = -P.t[i];
  if (cheirality_ok(P, x1, x2)) out.push_back(P);
}

// RelativePoseJacobianAccumulator (jacobian_impl.h:307-467) with the
// truncated loss of scale 1 and per-position weights, and lm_5dof_impl
// (bundle.cpp:176-250): 25 iterations, lambda 1e-3, gradient and step
// tolerances 1e-8. A Cholesky failure gives a zero step (the loop ends).
inline void refine_relpose(const Mat& pts, const size_t* s, size_t n, const double* w, Pose& P) {
  auto residual = [&](const Pose& Q) {
    const Model E = essential_from_pose(Q);
    double cost = 0;
    for (size_t k = 0; k < n; ++k) {
      const double* p = pts.row(s[k]);
      const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
      const double Ex0 = E[0] * x1 + E[1] * y1 + E[2], Ex1 = E[3] * x1 + E[4] * y1 + E[5],
                   Ex2 = E[6] * x1 + E[7] * y1 + E[8];
      const double C = x2 * Ex0 + y2 * Ex1 + Ex2;
      const double a0 = E[0] * x2 + E[3] * y2 + E[6], a1 = E[1] * x2 + E[4] * y2 + E[7];
      const double nJ = (Ex0 * Ex0 + Ex1 * Ex1) + (a0 * a0 + a1 * a1);
      const double r2 = (C * C) / nJ;
      const double l = std::min(r2, 1.0);
      cost += w ? w[k] * l : l;
    }
    return cost;
  };
  double JtJ[5][5] = {{0}}, Jtr[5] = {0}, tb[3][2] = {{0}};
  double lambda = 1e-3;
  double cost = residual(P);
  bool recompute = true;
  for (int iter = 0; iter < 25; ++iter) {
    if (recompute) {
      for (int a = 0; a < 5; ++a) {
        Jtr[a] = 0;
        for (int b = 0; b < 5; ++b) JtJ[a][b] = 0;
      }
      // tangent basis of the translation
      const double* t = P.t;
      double e[3] = {0, 0, 0};
      if (std::fabs(t[0]) < std::fabs(t[1])) {
        if (std::fabs(t[0]) < std::fabs(t[2])) e[0] = 1;
        else e[2] = 1;
      } else {
        if (std::fabs(t[1]) < std::fabs(t[2])) e[1] = 1;
        else e[2] = 1;
      }
      double b0[3], b1[3];
      cross3(t, e, b0);
      double nb = std::sqrt(b0[0] * b0[0] + b0[1] * b0[1] + b0[2] * b0[2]);
      for (int i = 0; i < 3; ++i) b0[i] /= nb;
      cross3(b0, t, b1);
      nb = std::sqrt(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
      for (int i = 0; i < 3; ++i) b1[i] /= nb;
      for (int i = 0; i < 3; ++i) {
        tb[i][0] = b0[i];
        tb[i][1] = b1[i];
      }
      const Model E = essential_from_pose(P);
      double R[9];
      quat_to_R(P.q, R);
      // dR (9 x 3) and dt (9 x 2) over column-major vec(E)
      double dR[9][3] = {{0}}, dt[9][2];
      for (int i = 0; i < 3; ++i) {
        const double Ec0 = E[3 * i], Ec1 = E[3 * i + 1], Ec2 = E[3 * i + 2];
        dR[i][0] = 0;       dR[i][1] = -Ec2;     dR[i][2] = Ec1;
        dR[3 + i][0] = Ec2; dR[3 + i][1] = 0;    dR[3 + i][2] = -Ec0;
        dR[6 + i][0] = -Ec1; dR[6 + i][1] = Ec0; dR[6 + i][2] = 0;
      }
      for (int j = 0; j < 3; ++j) {
        const double Rc[3] = {R[j], R[3 + j], R[6 + j]};
        double c0v[3], c1v[3];
        cross3(b0, Rc, c0v);
        cross3(b1, Rc, c1v);
        for (int i = 0; i < 3; ++i) {
          dt[3 * j + i][0] = c0v[i];
          dt[3 * j + i][1] = c1v[i];
        }
      }
      for (size_t k = 0; k < n; ++k) {
        const double* p = pts.row(s[k]);
        const double p0 = p[0], p1 = p[1], q0 = p[2], q1 = p[3];
        const double Ex0 = E[0] * p0 + E[1] * p1 + E[2], Ex1 = E[3] * p0 + E[4] * p1 + E[5],
                     Ex2 = E[6] * p0 + E[7] * p1 + E[8];
        const double C = q0 * Ex0 + q1 * Ex1 + Ex2;
        const double J0 = E[0] * q0 + E[3] * q1 + E[6], J1 = E[1] * q0 + E[4] * q1 + E[7];
        const double J2 = Ex0, J3 = Ex1;
        const double nJ = std::sqrt(J0 * J0 + J1 * J1 + J2 * J2 + J3 * J3);
        const double inv = 1.0 / nJ;
        const double r = C * inv;
        double weight = ((r * r) < 1.0 ? 1.0 : 0.0) / (double)n;
        if (w) weight = w[k] * weight;
        if (weight == 0.0) continue;
        double dF[9] = {p0 * q0, p0 * q1, p0, p1 * q0, p1 * q1, p1, q0, q1, 1.0};
        const double sc = C * inv * inv;
        dF[0] -= sc * (J2 * p0 + J0 * q0);
        dF[1] -= sc * (J3 * p0 + J0 * q1);
        dF[2] -= sc * (J0);
        dF[3] -= sc * (J2 * p1 + J1 * q0);
        dF[4] -= sc * (J3 * p1 + J1 * q1);
        dF[5] -= sc * (J1);
        dF[6] -= sc * (J2);
        dF[7] -= sc * (J3);
        for (int i = 0; i < 9; ++i) dF[i] *= inv;
        double J[5];
        for (int c = 0; c < 3; ++c) {
          double a = 0;
          for (int rr = 0; rr < 9; ++rr) a += dF[rr] * dR[rr][c];
          J[c] = a;
        }
        for (int c = 0; c < 2; ++c) {
          double a = 0;
          for (int rr = 0; rr < 9; ++rr) a += dF[rr] * dt[rr][c];
          J[3 + c] = a;
        }
        const double f = weight * C * inv;
        for (int a = 0; a < 5; ++a) Jtr[a] += f * J[a];
        for (int a = 0; a < 5; ++a)
          for (int b = 0; b <= a; ++b) JtJ[a][b] += weight * (J[a] * J[b]);
      }
      double gn = 0;
      for (int a = 0; a < 5; ++a) gn += Jtr[a] * Jtr[a];
      if (std::sqrt(gn) < 1e-8) break;
    }
    for (int a = 0; a < 5; ++a) JtJ[a][a] += lambda;
    std::vector<double> A(25);
    for (int a = 0; a < 5; ++a)
      for (int b = 0; b < 5; ++b) A[a * 5 + b] = a >= b ? JtJ[a][b] : JtJ[b][a];
    double sol[5];
    if (llt_solve(A, 5, Jtr, sol)) {
      for (int a = 0; a < 5; ++a) sol[a] = -sol[a];
    } else {
      for (int a = 0; a < 5; ++a) sol[a] = 0;
    }
    double sn = 0;
    for (int a = 0; a < 5; ++a) sn += sol[a] * sol[a];
    if (std::sqrt(sn) < 1e-8) break;
    double wv[3] = {sol[0], sol[1], sol[2]};
    const double th = std::sqrt(wv[0] * wv[0] + wv[1] * wv[1] + wv[2] * wv[2]);
    for (int i = 0; i < 3; ++i) wv[i] /= th;
    const double a = std::sin(th), b = std::cos(th);
    const double S[9] = {0, -wv[2], wv[1], wv[2], 0, -wv[0], -wv[1], wv[0], 0};
    double S2[9], R[9], M[9], RM[9];
    matmul3(S, S, S2);
    for (int i = 0; i < 9; ++i) M[i] = a * S[i] + (1 - b) * S2[i];
    quat_to_R(P.q, R);
    matmul3(R, M, RM);
    for (int i = 0; i < 9; ++i) RM[i] = R[i] + RM[i];
    Pose Pn;
    R_to_quat(RM, Pn.q);
    for (int i = 0; i < 3; ++i) Pn.t[i] = P.t[i] + (tb[i][0] * sol[3] + tb[i][1] * sol[4]);
    const double cn = residual(Pn);
    if (cn < cost) {
      P = Pn;
      lambda /= 10;
      cost = cn;
      recompute = true;
    } else {
      for (int q = 0; q < 5; ++q) JtJ[q][q] -= lambda;
      lambda *= 10;
      recompute = false;
    }
  }
}

// EssentialMatrixBundleAdjustmentSolver::estimateModel with no initial model
// (solver_essential_matrix_bundle_adjustment.h:114-188): Stewenius on the
// sample, every cheirality-consistent pose of each solution refined.
// `w_point` is indexed by point, `w_pos` by sample position.
inline void e_bundle_adjust(const Mat& pts, const size_t* s, size_t n, const double* w_point, const double* w_pos,
                            std::vector<Model>& out) {
  std::vector<Model> init;
  e_stewenius(pts, s, n, w_point, init);
  const double* p = pts.row(s[0]);
  double x1[3] = {p[0], p[1], 1.0}, x2[3] = {p[2], p[3], 1.0};
  const double n1 = std::sqrt(x1[0] * x1[0] + x1[1] * x1[1] + 1.0);
  const double n2 = std::sqrt(x2[0] * x2[0] + x2[1] * x2[1] + 1.0);
  for (int i = 0; i < 3; ++i) {
    x1[i] /= n1;
    x2[i] /= n2;
  }
  for (const Model& E : init) {
    std::vector<Pose> poses;
    poses_from_essential(E, x1, x2, poses);
    for (Pose& P : poses) {
      refine_relpose(pts, s, n, w_pos, P);
      out.push_back(essential_from_pose(P));
    }
  }
}

// ---------------------------------------------------------------------------
// EssentialMatrixEstimator<Nister, Stewenius> (essential_estimator.h:57-402).
struct EssentialEstimator {
  static constexpr size_t sample_size() { return 5; }
  static constexpr bool space_partitioning = false;  // SpacePartitioningRANSAC applies
  static constexpr size_t max_solutions() { return 10; }  // maximumMinimalSolutions
  size_t sample_size_rt() const { return 5; }
  size_t inlier_limit() const { return 7 * sample_size(); }
  double squared_residual(const double* p, const Model& E) const { return e_sampson2(p, E); }
  bool is_valid_sample(const Mat&, const size_t*) const { return true; }
  bool estimate_minimal(const Mat& pts, const size_t* s, std::vector<Model>& models) const {
    models.clear();
    if (!e_nister5(pts, s, models)) return false;
    for (int k = (int)models.size() - 1; k >= 0; --k)
      if (!e_orientation_valid(models[k], pts, s, 5)) models.erase(models.begin() + k);
    return !models.empty();
  }
  bool estimate_nonminimal(const Mat& pts, const size_t* s, size_t n, std::vector<Model>& models,
                           const double* weights) const {
    if (n < 5) return false;
    if (!e_stewenius(pts, s, n, weights, models)) return false;
    for (Model& E : models) {
      double nr = 0;
      for (double v : E) nr += v * v;
      nr = std::sqrt(nr);
      for (double& v : E) v /= nr;
      if (E[8] < 0)
        for (double& v : E) v = -v;
    }
    return true;
  }
  // isValidModel (essential_estimator.h:279-305)
  bool is_valid_model(Model& model, const Mat& pts, const std::vector<size_t>& inliers, const size_t*,
                      double threshold, bool& updated) const {
    updated = false;
    const double mn = std::max((double)sample_size(), (double)inliers.size() * 0.1);
    const size_t min_n = (size_t)mn;
    const double sq = threshold * threshold;
    size_t c = 0;
    for (size_t idx : inliers)
      if (e_symepi2(pts.row(idx), model) < sq)
        if (++c >= min_n) return true;
    return false;
  }
};

// EssentialMatrixEstimator<EssentialMatrixTwoPointsPlanar,
// EssentialMatrixBundleAdjustmentSolver> (types.h:121-126): planar camera
// motion, rotation about the camera's y axis and translation in its x-z
// plane.
struct EssentialPlanarEstimator : EssentialEstimator {
  static constexpr size_t sample_size() { return 2; }
  static constexpr size_t max_solutions() { return 1; }  // SolverEngine::maximumSolutions (solver_engine.h:73-76)
  size_t sample_size_rt() const { return 2; }
  static constexpr size_t non_minimal_sample_size() { return 6; }
  size_t inlier_limit() const { return 7 * sample_size(); }

  // EssentialMatrixTwoPointsPlanar::estimateModel
  // (solver_essential_matrix_two_points_planar.h:92-175): C = -A2^+ A1 from
  // the rows A1 = (y1, -y1 x2), A2 = (-y2, x1 y2); the quadratic in cos 2a
  // from C^T C; angles +-acos(root) / 2; the direction of C (cos a, sin a)
  // gives a - b. Models with non-finite entries are dropped (the reference
  // keeps them; they score nothing); the rest pass the orientation test on
  // the two points (essential_estimator.h:166-172).
  bool estimate_minimal(const Mat& pts, const size_t* s, std::vector<Model>& models) const {
    models.clear();
    double A1[2][2], A2[2][2];
    for (int i = 0; i < 2; ++i) {
      const double* p = pts.row(s[i]);
      const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
      A1[i][0] = y1;
      A1[i][1] = -y1 * x2;
      A2[i][0] = -y2;
      A2[i][1] = x1 * y2;
    }
    const double g00 = A2[0][0] * A2[0][0] + A2[1][0] * A2[1][0];
    const double g01 = A2[0][0] * A2[0][1] + A2[1][0] * A2[1][1];
    const double g11 = A2[0][1] * A2[0][1] + A2[1][1] * A2[1][1];
    const double det = g00 * g11 - g01 * g01;
    const double i00 = g11 / det, i01 = -g01 / det, i11 = g00 / det;
    double P[2][2];
    for (int j = 0; j < 2; ++j) {
      P[0][j] = i00 * A2[j][0] + i01 * A2[j][1];
      P[1][j] = i01 * A2[j][0] + i11 * A2[j][1];
    }
    double C[2][2];
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c) C[r][c] = -(P[r][0] * A1[0][c] + P[r][1] * A1[1][c]);
    const double a = C[0][0] * C[0][0] + C[1][0] * C[1][0];
    const double b = C[0][1] * C[0][0] + C[1][1] * C[1][0];
    const double c = C[0][1] * C[0][1] + C[1][1] * C[1][1];
    const double cf1 = 4 * b * b + (a - c) * (a - c);
    const double cf2 = -2 * (a - c) * (2 - a - c);
    const double cf3 = (2 - a - c) * (2 - a - c) - 4 * b * b;
    const double disc = std::sqrt(cf2 * cf2 - 4 * cf1 * cf3);
    const double c2a1 = (-cf2 + disc) / (2 * cf1), c2a2 = (-cf2 - disc) / (2 * cf1);
    const double alphas[4] = {std::acos(c2a1) / 2, std::acos(c2a2) / 2, -std::acos(c2a1) / 2, -std::acos(c2a2) / 2};
    for (int q = 0; q < 4; ++q) {
      const double sa = std::sin(alphas[q]), ca = std::cos(alphas[q]);
      double w0 = C[0][0] * ca + C[0][1] * sa, w1 = C[1][0] * ca + C[1][1] * sa;
      const double nw = std::sqrt(w0 * w0 + w1 * w1);
      w0 /= nw;
      w1 /= nw;
      const double al = std::atan2(sa, ca), amb = std::atan2(w1, w0);
      const Model E = {0.0, -std::sin(al), 0.0, std::sin(amb), 0.0, -std::cos(amb), 0.0, std::cos(al), 0.0};
      bool fin = true;
      for (double v : E) fin = fin && std::isfinite(v);
      if (fin && e_orientation_valid(E, pts, s, 2)) models.push_back(E);
    }
    return !models.empty();
  }

  // EssentialMatrixBundleAdjustmentSolver::estimateModel with no initial
  // model (solver_essential_matrix_bundle_adjustment.h:114-188) through
  // estimateModelNonminimal (essential_estimator.h:307-333): the weight
  // pointer goes to both the Stewenius start (read by point) and the pose
  // refinement (read by sample position, jacobian_impl.h:327-342); at most
  // ten models are kept; each is normalised with E33 >= 0.
  bool estimate_nonminimal(const Mat& pts, const size_t* s, size_t n, std::vector<Model>& models,
                           const double* weights) const {
    if (n < non_minimal_sample_size()) return false;
    std::vector<Model> out;
    e_bundle_adjust(pts, s, n, weights, weights, out);
    if (out.size() > 10) out.resize(10);
    if (out.empty()) return false;
    for (Model& E : out) {
      double nr = 0;
      for (double v : E) nr += v * v;
      nr = std::sqrt(nr);
      for (double& v : E) v /= nr;
      if (E[8] < 0)
        for (double& v : E) v = -v;
      models.push_back(E);
    }
    return true;
  }
};

}  // namespace oracle
