// Essential-matrix model on the device: the five-point minimal solver
// (Nister's trace constraints, Sturm-bracketed degree-10 polynomial), the
// non-minimal five-point solver (Stewenius' action matrix and its real
// eigenvalues), the relative-pose decomposition and the 5-dof
// Levenberg-Marquardt refinement used by the driver's final bundle adjustment.
//
// Behaviour follows src/pygcransac/include/estimators/essential_estimator.h
// (estimateModel 161-184, Sampson 186-213, symmetric distance 215-246,
// isValidModel 279-305, estimateModelNonminimal 308-335, orientation 338-401),
// solver_essential_matrix_five_point_nister.h:204-615,
// maths/sturm_polynomial_solver.h:38-262,
// solver_essential_matrix_five_point_stewenius.h:114-340,
// solver_essential_matrix_bundle_adjustment.h:114-188,
// relative_pose/essential.cpp:34-132, relative_pose/bundle.cpp:176-250,412-452
// and relative_pose/jacobian_impl.h:307-467. Every routine is written for one
// thread; the engine runs minimal solves one per thread, local-optimisation
// fits one per thread and the refits of the final model on one thread after a
// CTA-wide reduction of their sums.
#pragma once

#include "gcr_fundamental.cuh"

namespace gcr {
namespace ess {

// ---------------------------------------------------------------------------
// Polynomials in (x, y, z) over fixed monomial lists, the orders the two
// solvers' elimination templates are written for:
//   linear            [x, y, z, 1]
//   Nister quadratic  [x^2, xy, xz, x, y^2, yz, y, z^2, z, 1]
//   Nister cubic      [x^3, y^3, x^2y, xy^2, x^2z, x^2, y^2z, y^2, xyz, xy,
//                      xz^2, xz, x, yz^2, yz, y, z^3, z^2, z, 1]
//   GrevLex quadratic [x^2, xy, y^2, xz, yz, z^2, x, y, z, 1]
//   GrevLex cubic     [x^3, x^2y, xy^2, y^3, x^2z, xyz, y^2z, xz^2, yz^2, z^3,
//                      x^2, xy, y^2, xz, yz, z^2, x, y, z, 1]
// A product table gives, for term i of the first factor and term j of the
// second, the index of their product monomial in the result list.
static __constant__ unsigned char kLinLinQuadN[16] = {0, 1, 2, 3, 1, 4, 5, 6, 2, 5, 7, 8, 3, 6, 8, 9};
static __constant__ unsigned char kQuadNLinCubN[40] = {0,  2,  4,  5,  2,  3,  8,  9,  4,  8,  10, 11, 5,  9,
                                                       11, 12, 3,  1,  6,  7,  8,  6,  13, 14, 9,  7,  14, 15,
                                                       10, 13, 16, 17, 11, 14, 17, 18, 12, 15, 18, 19};
static __constant__ unsigned char kLinLinQuadG[16] = {0, 1, 3, 6, 1, 2, 4, 7, 3, 4, 5, 8, 6, 7, 8, 9};
static __constant__ unsigned char kQuadGLinCubG[40] = {0,  1,  4,  10, 1,  2,  5,  11, 2,  3,  6,  12, 4,  5,
                                                       7,  13, 5,  6,  8,  14, 7,  8,  9,  15, 10, 11, 13, 16,
                                                       11, 12, 14, 17, 13, 14, 15, 18, 16, 17, 18, 19};

// c += sign * (a * b): terms added one by one in the order of a's monomials,
// then b's.
template <int NA>
__device__ __forceinline__ void pmul_acc(const double* a, const double* b, double* c, const unsigned char* tab,
                                         double sign) {
  for (int i = 0; i < NA; ++i) {
    const double ai = sign * a[i];
#pragma unroll
    for (int j = 0; j < 4; ++j) c[tab[i * 4 + j]] += ai * b[j];
  }
}

// Epipolar design row: coefficients of column-major vec(E) in x2^T E x1.
__device__ __forceinline__ void design_row(const double* p, double w, double* r) {
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

// Kernel of the 5x9 design matrix by LU with complete pivoting in the basis of
// Eigen's FullPivLU::kernel() (pivot search in row-major order, rank threshold
// eps * 5 * max pivot). K[k][j] is entry k of basis vector j. Returns the
// kernel dimension (the solvers need 4).
__device__ inline int lu_kernel_5x9(double A[5][9], double K[9][4]) {
  int cp[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) cp[j] = j;
  long long maxpivot = 0;
  int nonzero = 5;
  bool stopped = false;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    int bi = k, bj = k;
    long long best = -1;
#pragma unroll
    for (int i = k; i < 5; ++i)
#pragma unroll
      for (int j = k; j < 9; ++j) {
        const long long v = dabs_bits(A[i][j]);
        if (v > best) { best = v; bi = i; bj = j; }
      }
    if (!stopped && best == 0) {
      nonzero = k;
      stopped = true;
    }
    if (!stopped) {
      if (best > maxpivot) maxpivot = best;
#pragma unroll
      for (int i = k + 1; i < 5; ++i) {
        const bool s = (i == bi);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const double t = A[k][j], u = A[i][j];
          A[k][j] = s ? u : t;
          A[i][j] = s ? t : u;
        }
      }
#pragma unroll
      for (int j = k + 1; j < 9; ++j) {
        const bool s = (j == bj);
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          const double t = A[i][k], u = A[i][j];
          A[i][k] = s ? u : t;
          A[i][j] = s ? t : u;
        }
        const int t = cp[k], u = cp[j];
        cp[k] = s ? u : t;
        cp[j] = s ? t : u;
      }
#pragma unroll
      for (int i = k + 1; i < 5; ++i) {
        const double f = A[i][k] / A[k][k];
        A[i][k] = f;
#pragma unroll
        for (int j = k + 1; j < 9; ++j) A[i][j] -= f * A[k][j];
      }
    }
  }
  const double thr = 2.220446049250313e-16 * 5.0 * __longlong_as_double(maxpivot);
  int rank = 0;
#pragma unroll
  for (int i = 0; i < 5; ++i)
    if (i < nonzero && fabs(A[i][i]) > thr) ++rank;
  if (rank != 5) return 9 - rank;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    double x[5];
#pragma unroll
    for (int i = 4; i >= 0; --i) {
      double s = -A[i][5 + j];
#pragma unroll
      for (int q = i + 1; q < 5; ++q) s -= A[i][q] * x[q];
      x[i] = s / A[i][i];
    }
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      double v = 0.0;
#pragma unroll
      for (int i = 0; i < 5; ++i) v = (cp[i] == t) ? x[i] : v;
      v = (cp[5 + j] == t) ? 1.0 : v;
      K[t][j] = v;
    }
  }
  return 4;
}

// ---------------------------------------------------------------------------
// Sturm-sequence root isolation of a degree-10 polynomial (ascending
// coefficients): monic normalisation, the remainder-recurrence sequence,
// bisection of the Cauchy interval (depth <= 30, left half first) and
// Ridders' method + Newton steps on each isolated root (tolerance 1e-10).
struct Sturm10 {
  static constexpr int N = 10;
  double f[2 * N + 1];
  double sv[3 * N];

  __device__ static double polyval(const double* p, int deg, double x) {
    double v = x + p[deg - 1];
    for (int i = deg - 2; i >= 0; --i) v = x * v + p[i];
    return v;
  }
  __device__ void build() {
    double buf[3 * N];
    for (int i = 0; i < 2 * N + 1; ++i) buf[i] = f[i];
    int o1 = 0, o2 = N + 1, o3 = 2 * N + 1;
    for (int i = 0; i < N - 1; ++i) {
      double* f1 = buf + o1;
      double* f2 = buf + o2;
      double* f3 = buf + o3;
      const double q1 = f1[N - i] * f2[N - 1 - i];
      const double q0 = f1[N - 1 - i] * f2[N - 1 - i] - f1[N - i] * f2[N - 2 - i];
      f3[0] = f1[0] - q0 * f2[0];
      for (int j = 1; j < N - 1 - i; ++j) f3[j] = f1[j] - q1 * f2[j - 1] - q0 * f2[j];
      const double c = -fabs(f3[N - 2 - i]);
      const double ci = 1.0 / c;
      for (int j = 0; j < N - 1 - i; ++j) f3[j] = f3[j] * ci;
      const int t = o1;
      o1 = o2;
      o2 = o3;
      o3 = t;
      sv[3 * i] = q0;
      sv[3 * i + 1] = q1;
      sv[3 * i + 2] = c;
    }
    sv[3 * N - 3] = buf[o1];
    sv[3 * N - 2] = buf[o1 + 1];
    sv[3 * N - 1] = buf[o2];
  }
  __device__ int sign_changes(double x) const {
    double v1 = sv[3 * N - 1];                     // v[i + 1] as i descends
    double v0 = sv[3 * N - 3] + x * sv[3 * N - 2];  // v[i]
    int cnt = (v0 < 0) != (v1 < 0) ? 1 : 0;
    for (int i = N - 2; i >= 0; --i) {
      const double v = (sv[3 * i] + x * sv[3 * i + 1]) * v0 + sv[3 * i + 2] * v1;
      if ((v < 0) != (v0 < 0)) ++cnt;
      v1 = v0;
      v0 = v;
    }
    return cnt;
  }
  __device__ void refine(double a, double b, double* roots, int& nr, double tol) const {
    double fa = polyval(f, N, a), fb = polyval(f, N, b);
    if (!((fa < 0) ^ (fb < 0))) return;
    for (int it = 0; it < 30; ++it) {
      if (fabs(a - b) < 1e-3) break;
      const double c = (a + b) * 0.5;
      const double fc = polyval(f, N, c);
      const double s = sqrt(fc * fc - fa * fb);
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
      if (fabs(fx) < tol) break;
      const double fpx = (double)N * polyval(f + N + 1, N - 1, x);
      const double dx = fx / fpx;
      x = x - dx;
      if (fabs(dx) < tol) break;
    }
    if (nr < N) roots[nr++] = x;
  }
  // Returns the number of real roots written to `roots` (<= 10).
  __device__ int solve(const double* coeffs, double* roots, double tol = 1e-10) {
    if (coeffs[N] == 0.0) return 0;
    for (int i = 0; i <= N; ++i) f[i] = coeffs[i];
    const double ci = 1.0 / f[N];
    for (int i = 0; i < N; ++i) f[i] *= ci;
    f[N] = 1.0;
    for (int i = 0; i < N - 1; ++i) f[N + 1 + i] = f[i + 1] * ((i + 1) / (double)N);
    f[2 * N] = 1.0;
    build();
    double mx = 0;
    for (int i = 0; i < N; ++i) mx = fmax(mx, fabs(f[i]));
    const double r0 = 1.0 + mx;
    const int sa0 = sign_changes(-r0), sb0 = sign_changes(r0);
    if (sa0 - sb0 == 0) return 0;
    // depth-first, left half first: the order of the recursive bisection
    double sa_[64], sb_[64];
    int ca[64], cb[64], dep[64];
    int top = 0, nr = 0;
    sa_[0] = -r0; sb_[0] = r0; ca[0] = sa0; cb[0] = sb0; dep[0] = 0;
    top = 1;
    while (top > 0) {
      --top;
      const double a = sa_[top], b = sb_[top];
      const int sa = ca[top], sb = cb[top], d = dep[top];
      if (d > 30) continue;
      const int n = sa - sb;
      if (n > 1) {
        if (top + 2 > 64) continue;  // cannot happen: depth <= 31 keeps the stack below 33
        const double c = (a + b) * 0.5;
        const int sc = sign_changes(c);
        sa_[top] = c; sb_[top] = b; ca[top] = sc; cb[top] = sb; dep[top] = d + 1; ++top;
        sa_[top] = a; sb_[top] = c; ca[top] = sa; cb[top] = sc; dep[top] = d + 1; ++top;
      } else if (n == 1) {
        refine(a, b, roots, nr, tol);
      }
    }
    return nr;
  }
};

// ---------------------------------------------------------------------------
// Dense helpers on small row-major arrays (one thread).

// Partial-pivoting LU solve of the 10 x 10 system L X = R in place (R holds the
// right-hand sides and receives X): the coeffs.block<10,10>(0,0).partialPivLu()
// .solve(coeffs.block<10,10>(0,10)) step.
__device__ inline void partial_piv_solve10(double* L, double* R) {
  int perm[10];
  for (int i = 0; i < 10; ++i) perm[i] = i;
  for (int k = 0; k < 10; ++k) {
    int p = k;
    double best = fabs(L[k * 10 + k]);
    for (int i = k + 1; i < 10; ++i)
      if (fabs(L[i * 10 + k]) > best) { best = fabs(L[i * 10 + k]); p = i; }
    if (p != k) {
      for (int j = 0; j < 10; ++j) { const double t = L[k * 10 + j]; L[k * 10 + j] = L[p * 10 + j]; L[p * 10 + j] = t; }
      const int t = perm[k]; perm[k] = perm[p]; perm[p] = t;
    }
    if (L[k * 10 + k] != 0.0)
      for (int i = k + 1; i < 10; ++i) L[i * 10 + k] /= L[k * 10 + k];
    for (int i = k + 1; i < 10; ++i)
      for (int j = k + 1; j < 10; ++j) L[i * 10 + j] -= L[i * 10 + k] * L[k * 10 + j];
  }
  double X[100];
  for (int i = 0; i < 10; ++i)
    for (int c = 0; c < 10; ++c) X[i * 10 + c] = R[perm[i] * 10 + c];
  for (int c = 0; c < 10; ++c) {
    for (int i = 0; i < 10; ++i) {
      double s = X[i * 10 + c];
      for (int q = 0; q < i; ++q) s -= L[i * 10 + q] * X[q * 10 + c];
      X[i * 10 + c] = s;
    }
    for (int i = 9; i >= 0; --i) {
      double s = X[i * 10 + c];
      for (int q = i + 1; q < 10; ++q) s -= L[i * 10 + q] * X[q * 10 + c];
      X[i * 10 + c] = s / L[i * 10 + i];
    }
  }
  for (int i = 0; i < 100; ++i) R[i] = X[i];
}

// Full-pivoting LU solve A X = B (FullPivLU::solve semantics): A is r x c
// (r >= c), B is r x m; X (c x m) is written to X. Unknowns past the numerical
// rank are zero. A and B are overwritten.
__device__ inline void full_piv_solve(double* A, int r, int c, double* B, int m, double* X) {
  int rp[10], cp[10];
  for (int i = 0; i < r; ++i) rp[i] = i;
  for (int j = 0; j < c; ++j) cp[j] = j;
  const int sz = r < c ? r : c;
  double maxpivot = 0;
  int nonzero = sz;
  for (int k = 0; k < sz; ++k) {
    int bi = k, bj = k;
    double best = -1;
    for (int i = k; i < r; ++i)
      for (int j = k; j < c; ++j) {
        const double v = fabs(A[i * c + j]);
        if (v > best) { best = v; bi = i; bj = j; }
      }
    if (best == 0) {
      nonzero = k;
      break;
    }
    if (best > maxpivot) maxpivot = best;
    if (bi != k) {
      for (int j = 0; j < c; ++j) { const double t = A[k * c + j]; A[k * c + j] = A[bi * c + j]; A[bi * c + j] = t; }
      const int t = rp[k]; rp[k] = rp[bi]; rp[bi] = t;
    }
    if (bj != k) {
      for (int i = 0; i < r; ++i) { const double t = A[i * c + k]; A[i * c + k] = A[i * c + bj]; A[i * c + bj] = t; }
      const int t = cp[k]; cp[k] = cp[bj]; cp[bj] = t;
    }
    for (int i = k + 1; i < r; ++i) {
      const double f = A[i * c + k] / A[k * c + k];
      A[i * c + k] = f;
      for (int j = k + 1; j < c; ++j) A[i * c + j] -= f * A[k * c + j];
    }
  }
  const double thr = 2.220446049250313e-16 * (double)sz;
  int rank = 0;
  for (int i = 0; i < nonzero; ++i)
    if (fabs(A[i * c + i]) > thr * maxpivot) ++rank;
  for (int i = 0; i < c * m; ++i) X[i] = 0.0;
  for (int col = 0; col < m; ++col) {
    double y[10];
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
}

// Last four columns of Q of the column-pivoting Householder QR of a 9 x 9
// matrix (pivot: remaining column of largest norm, recomputed every step;
// Householder vectors in Eigen's convention). Q4[k][j] = Q(k, 5 + j). M is
// overwritten.
__device__ inline void colpiv_q_last4(double* M, double Q4[9][4]) {
  double tau[9];
  for (int s = 0; s < 9; ++s) {
    int p = s;
    double best = -1;
    for (int j = s; j < 9; ++j) {
      double t = 0;
      for (int i = s; i < 9; ++i) t += M[i * 9 + j] * M[i * 9 + j];
      if (t > best) { best = t; p = j; }
    }
    if (p != s)
      for (int i = 0; i < 9; ++i) { const double t = M[i * 9 + s]; M[i * 9 + s] = M[i * 9 + p]; M[i * 9 + p] = t; }
    const double c0 = M[s * 9 + s];
    double tail = 0;
    for (int i = s + 1; i < 9; ++i) tail += M[i * 9 + s] * M[i * 9 + s];
    double t, beta;
    if (tail <= 2.2250738585072014e-308) {
      t = 0;
      beta = c0;
      for (int i = s + 1; i < 9; ++i) M[i * 9 + s] = 0;
    } else {
      beta = sqrt(c0 * c0 + tail);
      if (c0 >= 0) beta = -beta;
      for (int i = s + 1; i < 9; ++i) M[i * 9 + s] = M[i * 9 + s] / (c0 - beta);
      t = (beta - c0) / beta;
    }
    tau[s] = t;
    M[s * 9 + s] = beta;
    for (int j = s + 1; j < 9; ++j) {
      double a = M[s * 9 + j];
      for (int i = s + 1; i < 9; ++i) a += M[i * 9 + s] * M[i * 9 + j];
      a *= t;
      M[s * 9 + j] -= a;
      for (int i = s + 1; i < 9; ++i) M[i * 9 + j] -= a * M[i * 9 + s];
    }
  }
  for (int c = 0; c < 4; ++c) {
    double e[9];
    for (int i = 0; i < 9; ++i) e[i] = (i == 5 + c) ? 1.0 : 0.0;
    for (int s = 8; s >= 0; --s) {
      double a = e[s];
      for (int i = s + 1; i < 9; ++i) a += M[i * 9 + s] * e[i];
      a *= tau[s];
      e[s] -= a;
      for (int i = s + 1; i < 9; ++i) e[i] -= a * M[i * 9 + s];
    }
    for (int i = 0; i < 9; ++i) Q4[i][c] = e[i];
  }
}

// Eigenvalues of a real 10 x 10 matrix (overwritten): Householder reduction to
// Hessenberg form, then Francis double-shift QR with the EISPACK hqr deflation
// and exceptional shifts at 10 and 20 iterations. A 2 x 2 block with a
// non-negative discriminant gives two real eigenvalues (wi exactly 0).
// Returns false when an eigenvalue took more than 30 iterations.
__device__ inline bool real_eigenvalues10(double* a, double* wr, double* wi) {
  const int n = 10;
  for (int k = 0; k < n - 2; ++k) {
    double alpha = 0;
    for (int i = k + 1; i < n; ++i) alpha += a[i * n + k] * a[i * n + k];
    if (alpha == 0) continue;
    alpha = sqrt(alpha);
    if (a[(k + 1) * n + k] > 0) alpha = -alpha;
    double v[10];
    for (int i = 0; i < n; ++i) v[i] = i > k ? a[i * n + k] : 0.0;
    v[k + 1] -= alpha;
    double vn = 0;
    for (int i = k + 1; i < n; ++i) vn += v[i] * v[i];
    if (vn == 0) continue;
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
  for (int i = 0; i < n; ++i) wr[i] = wi[i] = 0.0;
  double anorm = 0;
  for (int i = 0; i < n; ++i)
    for (int j = (i > 0 ? i - 1 : 0); j < n; ++j) anorm += fabs(a[i * n + j]);
  int nn = n - 1;
  double t = 0;
  while (nn >= 0) {
    int its = 0, l;
    for (;;) {
      for (l = nn; l >= 1; --l) {
        double s = fabs(a[(l - 1) * n + l - 1]) + fabs(a[l * n + l]);
        if (s == 0) s = anorm;
        if (fabs(a[l * n + l - 1]) + s == s) {
          a[l * n + l - 1] = 0;
          break;
        }
      }
      double x = a[nn * n + nn];
      if (l == nn) {
        wr[nn] = x + t;
        wi[nn] = 0;
        --nn;
        break;
      }
      double y = a[(nn - 1) * n + nn - 1];
      double w = a[nn * n + nn - 1] * a[(nn - 1) * n + nn];
      if (l == nn - 1) {
        const double p = 0.5 * (y - x);
        const double q = p * p + w;
        double z = sqrt(fabs(q));
        x += t;
        if (q >= 0) {
          z = p + (p >= 0 ? fabs(z) : -fabs(z));
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
      if (its == 10 || its == 20) {
        t += x;
        for (int i = 0; i <= nn; ++i) a[i * n + i] -= x;
        const double s = fabs(a[nn * n + nn - 1]) + fabs(a[(nn - 1) * n + nn - 2]);
        x = y = 0.75 * s;
        w = -0.4375 * s * s;
      }
      ++its;
      int m;
      double p = 0, q = 0, r = 0, z;
      for (m = nn - 2; m >= l; --m) {
        z = a[m * n + m];
        r = x - z;
        double s = y - z;
        p = (r * s - w) / a[(m + 1) * n + m] + a[m * n + m + 1];
        q = a[(m + 1) * n + m + 1] - z - r - s;
        r = a[(m + 2) * n + m + 1];
        s = fabs(p) + fabs(q) + fabs(r);
        p /= s;
        q /= s;
        r /= s;
        if (m == l) break;
        const double u = fabs(a[m * n + m - 1]) * (fabs(q) + fabs(r));
        const double v = fabs(p) * (fabs(a[(m - 1) * n + m - 1]) + fabs(z) + fabs(a[(m + 1) * n + m + 1]));
        if (u + v == v) break;
      }
      for (int i = m + 2; i <= nn; ++i) {
        a[i * n + i - 2] = 0;
        if (i != m + 2) a[i * n + i - 3] = 0;
      }
      for (int k = m; k <= nn - 1; ++k) {
        if (k != m) {
          p = a[k * n + k - 1];
          q = a[(k + 1) * n + k - 1];
          r = 0;
          if (k != nn - 1) r = a[(k + 2) * n + k - 1];
          x = fabs(p) + fabs(q) + fabs(r);
          if (x != 0) {
            p /= x;
            q /= x;
            r /= x;
          }
        }
        double s = sqrt(p * p + q * q + r * r);
        if (p < 0) s = -s;
        if (s != 0) {
          if (k == m) {
            if (l != m) a[k * n + k - 1] = -a[k * n + k - 1];
          } else {
            a[k * n + k - 1] = -s * x;
          }
          p += s;
          x = p / s;
          y = q / s;
          z = r / s;
          q /= p;
          r /= p;
          for (int j = k; j <= nn; ++j) {
            p = a[k * n + j] + q * a[(k + 1) * n + j];
            if (k != nn - 1) {
              p += r * a[(k + 2) * n + j];
              a[(k + 2) * n + j] -= p * z;
            }
            a[(k + 1) * n + j] -= p * y;
            a[k * n + j] -= p * x;
          }
          const int mmin = nn < k + 3 ? nn : k + 3;
          for (int i = l; i <= mmin; ++i) {
            p = x * a[i * n + k] + y * a[i * n + k + 1];
            if (k != nn - 1) {
              p += z * a[i * n + k + 2];
              a[i * n + k + 2] -= p * r;
            }
            a[i * n + k + 1] -= p * q;
            a[i * n + k] -= p;
          }
        }
      }
    }
  }
  return true;
}

// Null vector of a 10 x 10 matrix of rank 9 (overwritten): complete-pivoting
// elimination over 9 steps, the last pivoted unknown set to one.
__device__ inline void null_vector10(double* M, double* x) {
  const int n = 10;
  int cp[10];
  for (int j = 0; j < n; ++j) cp[j] = j;
  for (int k = 0; k < n - 1; ++k) {
    int bi = k, bj = k;
    double best = -1;
    for (int i = k; i < n; ++i)
      for (int j = k; j < n; ++j) {
        const double v = fabs(M[i * n + j]);
        if (v > best) { best = v; bi = i; bj = j; }
      }
    if (bi != k)
      for (int j = 0; j < n; ++j) { const double t = M[k * n + j]; M[k * n + j] = M[bi * n + j]; M[bi * n + j] = t; }
    if (bj != k) {
      for (int i = 0; i < n; ++i) { const double t = M[i * n + k]; M[i * n + k] = M[i * n + bj]; M[i * n + bj] = t; }
      const int t = cp[k]; cp[k] = cp[bj]; cp[bj] = t;
    }
    if (M[k * n + k] == 0) continue;
    for (int i = k + 1; i < n; ++i) {
      const double f = M[i * n + k] / M[k * n + k];
      for (int j = k + 1; j < n; ++j) M[i * n + j] -= f * M[k * n + j];
      M[i * n + k] = 0;
    }
  }
  double y[10];
  y[n - 1] = 1.0;
  for (int i = n - 2; i >= 0; --i) {
    double s = -M[i * n + n - 1];
    for (int q = i + 1; q < n - 1; ++q) s -= M[i * n + q] * y[q];
    y[i] = M[i * n + i] != 0 ? s / M[i * n + i] : 0.0;
  }
  for (int i = 0; i < n; ++i) x[cp[i]] = y[i];
}

// ---------------------------------------------------------------------------
// Nister's five-point solver on a minimal sample (unit weights). Writes up to
// 10 row-major models to out; returns their number.
__device__ inline int nister5(const double* pts, const int* s, double* out) {
  double K[9][4];
  {
    double A[5][9];
#pragma unroll
    for (int i = 0; i < 5; ++i) design_row(pts + 4 * s[i], 1.0, A[i]);
    if (lu_kernel_5x9(A, K) != 4) return 0;
  }
  // E(i, j) = vec index 3 j + i, coefficients over [x, y, z, 1] = K[3 j + i][0..3]
  double coeffs[10][20];
#pragma unroll
  for (int r = 0; r < 10; ++r)
#pragma unroll
    for (int c = 0; c < 20; ++c) coeffs[r][c] = 0.0;
  {
    // determinant row: E20 (E01 E12 - E02 E11) + E21 (E02 E10 - E00 E12) + E22 (E00 E11 - E01 E10)
    constexpr int pr[3][8] = {{0, 1, 1, 2, 0, 2, 1, 1}, {0, 2, 1, 0, 0, 0, 1, 2}, {0, 0, 1, 1, 0, 1, 1, 0}};
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      double d[10];
#pragma unroll
      for (int q = 0; q < 10; ++q) d[q] = 0.0;
      pmul_acc<4>(K[3 * pr[t][1] + pr[t][0]], K[3 * pr[t][3] + pr[t][2]], d, kLinLinQuadN, 1.0);
      pmul_acc<4>(K[3 * pr[t][5] + pr[t][4]], K[3 * pr[t][7] + pr[t][6]], d, kLinLinQuadN, -1.0);
      pmul_acc<10>(d, K[3 * t + 2], coeffs[9], kQuadNLinCubN, 1.0);
    }
  }
  {
    double EET[6][10];  // (0,0) (0,1) (0,2) (1,1) (1,2) (2,2)
    constexpr int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int u = 0; u < 6; ++u) {
#pragma unroll
      for (int q = 0; q < 10; ++q) EET[u][q] = 0.0;
#pragma unroll
      for (int k = 0; k < 3; ++k) pmul_acc<4>(K[3 * k + ii[u]], K[3 * k + jj[u]], EET[u], kLinLinQuadN, 1.0);
    }
#pragma unroll
    for (int q = 0; q < 10; ++q) {
      const double t = 0.5 * (EET[0][q] + EET[3][q] + EET[5][q]);
      EET[0][q] -= t;
      EET[3][q] -= t;
      EET[5][q] -= t;
    }
    constexpr int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) pmul_acc<10>(EET[sym[i][k]], K[3 * j + k], coeffs[3 * i + j], kQuadNLinCubN, 1.0);
  }
  double L[100], R[100];
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) {
      L[i * 10 + j] = coeffs[i][j];
      R[i * 10 + j] = coeffs[i][10 + j];
    }
  partial_piv_solve10(L, R);
  double A[3][13];
  for (int i = 0; i < 3; ++i) {
    const double* a = R + (4 + 2 * i) * 10;
    const double* b = R + (5 + 2 * i) * 10;
    A[i][0] = -b[0];
    A[i][1] = a[0] - b[1];
    A[i][2] = a[1] - b[2];
    A[i][3] = a[2];
    A[i][4] = -b[3];
    A[i][5] = a[3] - b[4];
    A[i][6] = a[4] - b[5];
    A[i][7] = a[5];
    A[i][8] = -b[6];
    A[i][9] = a[6] - b[7];
    A[i][10] = a[7] - b[8];
    A[i][11] = a[8] - b[9];
    A[i][12] = a[9];
  }
  // determinant of [cubic | cubic | quartic] columns, ascending in z
  double poly[11];
  {
    double P[3][3][5];
    for (int i = 0; i < 3; ++i) {
      for (int k = 0; k < 4; ++k) {
        P[i][0][k] = A[i][3 - k];
        P[i][1][k] = A[i][7 - k];
      }
      for (int k = 0; k < 5; ++k) P[i][2][k] = A[i][12 - k];
    }
    auto pmul = [](const double* a, int na, const double* b, int nb, double* c) {
      for (int i = 0; i < na + nb - 1; ++i) c[i] = 0;
      for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) c[i + j] += a[i] * b[j];
    };
    double t1[8], t2[8], m0[8], m1[8], m2[7], u[11];
    pmul(P[1][1], 4, P[2][2], 5, t1);
    pmul(P[1][2], 5, P[2][1], 4, t2);
    for (int k = 0; k < 8; ++k) m0[k] = t1[k] - t2[k];
    pmul(P[1][0], 4, P[2][2], 5, t1);
    pmul(P[1][2], 5, P[2][0], 4, t2);
    for (int k = 0; k < 8; ++k) m1[k] = t1[k] - t2[k];
    pmul(P[1][0], 4, P[2][1], 4, t1);
    pmul(P[1][1], 4, P[2][0], 4, t2);
    for (int k = 0; k < 7; ++k) m2[k] = t1[k] - t2[k];
    for (int k = 0; k < 11; ++k) poly[k] = 0;
    pmul(P[0][0], 4, m0, 8, u);
    for (int k = 0; k < 11; ++k) poly[k] += u[k];
    pmul(P[0][1], 4, m1, 8, u);
    for (int k = 0; k < 11; ++k) poly[k] -= u[k];
    pmul(P[0][2], 5, m2, 7, u);
    for (int k = 0; k < 11; ++k) poly[k] += u[k];
  }
  Sturm10 st;
  double roots[10];
  const int nr = st.solve(poly, roots);
  int nm = 0;
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
    if (fabs(B[2][0] * xz0 + B[2][1] * xz1 - b[2]) > 1e-6) {
      double M[6] = {B[0][0], B[0][1], B[1][0], B[1][1], B[2][0], B[2][1]};
      double rhs[3] = {b[0], b[1], b[2]};
      double X[2];
      full_piv_solve(M, 3, 2, rhs, 1, X);
      xz0 = X[0];
      xz1 = X[1];
    }
    const double x = -xz0, y = -xz1;
    const double sc = 1.0 / sqrt(x * x + y * y + z * z + 1.0);
    double* E = out + 9 * nm;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double* c = K[3 * j + i];
        E[3 * i + j] = (c[0] * x + c[1] * y + c[2] * z + c[3]) * sc;
      }
    ++nm;
  }
  return nm;
}

// Stewenius' solver from the null space N (N[k][j]: entry k of vec(E), basis
// vector j). Writes up to 10 row-major models (not normalised); returns their
// number.
__device__ inline int stewenius_from_null(const double N[9][4], double* out) {
  double cm[10][20];
#pragma unroll
  for (int r = 0; r < 10; ++r)
#pragma unroll
    for (int c = 0; c < 20; ++c) cm[r][c] = 0.0;
  {
    double eet[9][10];  // 2 E E^T, all (i, j)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double t[10];
#pragma unroll
        for (int q = 0; q < 10; ++q) t[q] = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) pmul_acc<4>(N[3 * k + i], N[3 * k + j], t, kLinLinQuadG, 1.0);
#pragma unroll
        for (int q = 0; q < 10; ++q) eet[3 * i + j][q] = 2 * t[q];
      }
    double tr[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) tr[q] = eet[0][q] + eet[4][q] + eet[8][q];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double row[20], tt[20];
#pragma unroll
        for (int q = 0; q < 20; ++q) row[q] = tt[q] = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) pmul_acc<10>(eet[3 * i + k], N[3 * j + k], row, kQuadGLinCubG, 1.0);
        pmul_acc<10>(tr, N[3 * j + i], tt, kQuadGLinCubG, 1.0);
#pragma unroll
        for (int q = 0; q < 20; ++q) cm[3 * i + j][q] = row[q] - 0.5 * tt[q];
      }
    constexpr int pr[3][8] = {{0, 1, 1, 2, 0, 2, 1, 1}, {0, 2, 1, 0, 0, 0, 1, 2}, {0, 0, 1, 1, 0, 1, 1, 0}};
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      double d[10];
#pragma unroll
      for (int q = 0; q < 10; ++q) d[q] = 0.0;
      pmul_acc<4>(N[3 * pr[t][1] + pr[t][0]], N[3 * pr[t][3] + pr[t][2]], d, kLinLinQuadG, 1.0);
      pmul_acc<4>(N[3 * pr[t][5] + pr[t][4]], N[3 * pr[t][7] + pr[t][6]], d, kLinLinQuadG, -1.0);
      pmul_acc<10>(d, N[3 * t + 2], cm[9], kQuadGLinCubG, 1.0);
    }
  }
  double L[100], R[100], El[100];
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) {
      L[i * 10 + j] = cm[i][j];
      R[i * 10 + j] = cm[i][10 + j];
    }
  full_piv_solve(L, 10, 10, R, 10, El);
  double act[100];
  for (int i = 0; i < 100; ++i) act[i] = 0.0;
  constexpr int src[6] = {0, 1, 2, 4, 5, 7};
  for (int r = 0; r < 6; ++r)
    for (int j = 0; j < 10; ++j) act[r * 10 + j] = El[src[r] * 10 + j];
  act[6 * 10 + 0] = -1.0;
  act[7 * 10 + 1] = -1.0;
  act[8 * 10 + 3] = -1.0;
  act[9 * 10 + 6] = -1.0;
  double wr[10], wi[10];
  {
    double H[100];
    for (int i = 0; i < 100; ++i) H[i] = act[i];
    if (!real_eigenvalues10(H, wr, wi)) return 0;
  }
  int nm = 0;
  for (int i = 0; i < 10; ++i) {
    if (wi[i] != 0) continue;
    double M[100], v[10];
    for (int q = 0; q < 100; ++q) M[q] = act[q];
    for (int d = 0; d < 10; ++d) M[d * 10 + d] -= wr[i];
    null_vector10(M, v);
    double* E = out + 9 * nm;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        const double* ns = N[3 * c + r];
        E[3 * r + c] = ns[0] * v[6] + ns[1] * v[7] + ns[2] * v[8] + ns[3] * v[9];
      }
    ++nm;
  }
  return nm;
}

// Stewenius from the (weighted) 9 x 9 normal matrix of more than five rows:
// null space = last four columns of Q of its column-pivoting QR.
__device__ inline int stewenius_from_ata(const double* ata81, double* out) {
  double M[81];
  for (int i = 0; i < 81; ++i) M[i] = ata81[i];
  double N[9][4];
  colpiv_q_last4(M, N);
  return stewenius_from_null(N, out);
}

// Stewenius on exactly five rows: null space from the LU kernel.
__device__ inline int stewenius_five(const double rows[5][9], double* out) {
  double A[5][9], N[9][4];
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 9; ++j) A[i][j] = rows[i][j];
  if (lu_kernel_5x9(A, N) != 4) return 0;
  return stewenius_from_null(N, out);
}

// estimateModelNonminimal's post-processing: unit Frobenius norm, E33 >= 0.
__device__ __forceinline__ void normalise_sign(double* E) {
  double nr = 0;
  for (int i = 0; i < 9; ++i) nr += E[i] * E[i];
  nr = sqrt(nr);
  for (int i = 0; i < 9; ++i) E[i] /= nr;
  if (E[8] < 0)
    for (int i = 0; i < 9; ++i) E[i] = -E[i];
}

// ---------------------------------------------------------------------------
// Relative pose: unit quaternion (w, x, y, z) and translation.
struct Pose {
  double q[4];
  double t[3];
};

__device__ __forceinline__ void quat_to_R(const double* q, double* R) {
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
__device__ inline void R_to_quat(const double* R, double* q) {
  const double tr = R[0] + R[4] + R[8];
  double w, v[3];
  if (tr > 0) {
    double t = sqrt(tr + 1.0);
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
    double t = sqrt(R[i * 4] - R[j * 4] - R[k * 4] + 1.0);
    double vi = 0.5 * t;
    t = 0.5 / t;
    w = (R[k * 3 + j] - R[j * 3 + k]) * t;
    const double vj = (R[j * 3 + i] + R[i * 3 + j]) * t;
    const double vk = (R[k * 3 + i] + R[i * 3 + k]) * t;
    v[0] = i == 0 ? vi : (j == 0 ? vj : vk);
    v[1] = i == 1 ? vi : (j == 1 ? vj : vk);
    v[2] = i == 2 ? vi : (j == 2 ? vj : vk);
  }
  const double n = sqrt(w * w + v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  q[0] = w / n;
  q[1] = v[0] / n;
  q[2] = v[1] / n;
  q[3] = v[2] / n;
}

// E = [t]x R
__device__ inline void essential_from_pose(const Pose& P, double* E) {
  double R[9];
  quat_to_R(P.q, R);
  const double S[9] = {0.0, -P.t[2], P.t[1], P.t[2], 0.0, -P.t[0], -P.t[1], P.t[0], 0.0};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) E[3 * i + j] = S[3 * i] * R[j] + S[3 * i + 1] * R[3 + j] + S[3 * i + 2] * R[6 + j];
}

__device__ inline bool cheirality_ok(const Pose& P, const double* x1, const double* x2) {
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

// The four (R, t) of E kept when (x1, x2) lies in front of both cameras;
// returns their number.
__device__ inline int poses_from_essential(const double* E, const double* x1, const double* x2, Pose* out) {
  const double c0[3] = {E[0], E[3], E[6]}, c1[3] = {E[1], E[4], E[7]}, c2[3] = {E[2], E[5], E[8]};
  double u12[3], u13[3], u23[3];
  dcross3(c0, c1, u12);
  dcross3(c0, c2, u13);
  dcross3(c1, c2, u23);
  auto sq = [](const double* v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; };
  const double n12 = sq(u12), n13 = sq(u13), n23 = sq(u23);
  double UW[3][3];  // UW[col][row]
  const double* a;
  const double* u;
  double nu;
  if (n12 > n13) {
    if (n12 > n23) { a = c0; u = u12; nu = n12; }
    else { a = c1; u = u23; nu = n23; }
  } else {
    if (n13 > n23) { a = c0; u = u13; nu = n13; }
    else { a = c1; u = u23; nu = n23; }
  }
  {
    const double na = sqrt(sq(a)), snu = sqrt(nu);
    for (int i = 0; i < 3; ++i) {
      UW[1][i] = a[i] / na;
      UW[2][i] = u[i] / snu;
    }
  }
  double t0[3];
  dcross3(UW[2], UW[1], t0);
  for (int i = 0; i < 3; ++i) UW[0][i] = -t0[i];
  double Vt[3][3];
  for (int j = 0; j < 3; ++j) {
    Vt[0][j] = UW[1][0] * E[j] + UW[1][1] * E[3 + j] + UW[1][2] * E[6 + j];
    Vt[1][j] = -UW[0][0] * E[j] + -UW[0][1] * E[3 + j] + -UW[0][2] * E[6 + j];
  }
  {
    const double n0 = sqrt(sq(Vt[0]));
    for (int j = 0; j < 3; ++j) Vt[0][j] /= n0;
    const double d = Vt[0][0] * Vt[1][0] + Vt[0][1] * Vt[1][1] + Vt[0][2] * Vt[1][2];
    for (int j = 0; j < 3; ++j) Vt[1][j] -= d * Vt[0][j];
    const double n1 = sqrt(sq(Vt[1]));
    for (int j = 0; j < 3; ++j) Vt[1][j] /= n1;
    dcross3(Vt[0], Vt[1], Vt[2]);
  }
  auto rot = [&](double* q) {
    double R[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) R[3 * i + j] = UW[0][i] * Vt[0][j] + UW[1][i] * Vt[1][j] + UW[2][i] * Vt[2][j];
    R_to_quat(R, q);
  };
  int np = 0;
  Pose P;
  rot(P.q);
  for (int i = 0; i < 3; ++i) P.t[i] = UW[2][i];
  if (cheirality_ok(P, x1, x2)) out[np++] = P;
  for (int i = 0; i < 3; ++i) P.t[i] = -P.t[i];
  if (cheirality_ok(P, x1, x2)) out[np++] = P;
  for (int c = 0; c < 2; ++c)
    for (int i = 0; i < 3; ++i) UW[c][i] = -UW[c][i];
  rot(P.q);
  if (cheirality_ok(P, x1, x2)) out[np++] = P;
  for (int i = 0; i < 3; ++i) P.t[i] = -P.t[i];
  if (cheirality_ok(P, x1, x2)) out[np++] = P;
  return np;
}

// Tangent basis of the translation update (jacobian_impl.h:351-367) and the
// Jacobians of vec(E) with respect to the rotation (dR, 9 x 3) and the
// translation (dt, 9 x 2) at pose P; E receives [t]x R.
struct PoseJac {
  double E[9];
  double tb[3][2];
  double dR[9][3];
  double dt[9][2];
};

__device__ inline void pose_jacobians(const Pose& P, PoseJac& J) {
  const double* t = P.t;
  double e[3] = {0, 0, 0};
  if (fabs(t[0]) < fabs(t[1])) {
    if (fabs(t[0]) < fabs(t[2])) e[0] = 1;
    else e[2] = 1;
  } else {
    if (fabs(t[1]) < fabs(t[2])) e[1] = 1;
    else e[2] = 1;
  }
  double b0[3], b1[3];
  dcross3(t, e, b0);
  double nb = sqrt(b0[0] * b0[0] + b0[1] * b0[1] + b0[2] * b0[2]);
  for (int i = 0; i < 3; ++i) b0[i] /= nb;
  dcross3(b0, t, b1);
  nb = sqrt(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
  for (int i = 0; i < 3; ++i) b1[i] /= nb;
  for (int i = 0; i < 3; ++i) {
    J.tb[i][0] = b0[i];
    J.tb[i][1] = b1[i];
  }
  essential_from_pose(P, J.E);
  double R[9];
  quat_to_R(P.q, R);
  const double* E = J.E;
  for (int i = 0; i < 3; ++i) {
    const double Ec0 = E[3 * i], Ec1 = E[3 * i + 1], Ec2 = E[3 * i + 2];
    J.dR[i][0] = 0;        J.dR[i][1] = -Ec2;     J.dR[i][2] = Ec1;
    J.dR[3 + i][0] = Ec2;  J.dR[3 + i][1] = 0;    J.dR[3 + i][2] = -Ec0;
    J.dR[6 + i][0] = -Ec1; J.dR[6 + i][1] = Ec0;  J.dR[6 + i][2] = 0;
  }
  for (int j = 0; j < 3; ++j) {
    const double Rc[3] = {R[j], R[3 + j], R[6 + j]};
    double c0v[3], c1v[3];
    dcross3(b0, Rc, c0v);
    dcross3(b1, Rc, c1v);
    for (int i = 0; i < 3; ++i) {
      J.dt[3 * j + i][0] = c0v[i];
      J.dt[3 * j + i][1] = c1v[i];
    }
  }
}

// Truncated (scale 1) Sampson loss of one correspondence under E.
__device__ __forceinline__ double relpose_loss(const double* E, const double* p) {
  const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
  const double Ex0 = E[0] * x1 + E[1] * y1 + E[2], Ex1 = E[3] * x1 + E[4] * y1 + E[5],
               Ex2 = E[6] * x1 + E[7] * y1 + E[8];
  const double C = x2 * Ex0 + y2 * Ex1 + Ex2;
  const double a0 = E[0] * x2 + E[3] * y2 + E[6], a1 = E[1] * x2 + E[4] * y2 + E[7];
  const double nJ = (Ex0 * Ex0 + Ex1 * Ex1) + (a0 * a0 + a1 * a1);
  const double r2 = (C * C) / nJ;
  return fmin(r2, 1.0);
}

// Contribution of one correspondence (weight w, n rows) to J^T J (lower, 15)
// and J^T r (5): acc[0..14] row-major lower triangle, acc[15..19].
__device__ __forceinline__ void relpose_accumulate(const PoseJac& J, const double* p, double w, int n, double* acc) {
  const double* E = J.E;
  const double p0 = p[0], p1 = p[1], q0 = p[2], q1 = p[3];
  const double Ex0 = E[0] * p0 + E[1] * p1 + E[2], Ex1 = E[3] * p0 + E[4] * p1 + E[5],
               Ex2 = E[6] * p0 + E[7] * p1 + E[8];
  const double C = q0 * Ex0 + q1 * Ex1 + Ex2;
  const double J0 = E[0] * q0 + E[3] * q1 + E[6], J1 = E[1] * q0 + E[4] * q1 + E[7];
  const double J2 = Ex0, J3 = Ex1;
  const double nJ = sqrt(J0 * J0 + J1 * J1 + J2 * J2 + J3 * J3);
  const double inv = 1.0 / nJ;
  const double r = C * inv;
  double weight = ((r * r) < 1.0 ? 1.0 : 0.0) / (double)n;
  weight = w * weight;
  if (weight == 0.0) return;
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
#pragma unroll
  for (int i = 0; i < 9; ++i) dF[i] *= inv;
  double Jv[5];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double a = 0;
#pragma unroll
    for (int rr = 0; rr < 9; ++rr) a += dF[rr] * J.dR[rr][c];
    Jv[c] = a;
  }
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    double a = 0;
#pragma unroll
    for (int rr = 0; rr < 9; ++rr) a += dF[rr] * J.dt[rr][c];
    Jv[3 + c] = a;
  }
  const double f = weight * C * inv;
  int k = 0;
#pragma unroll
  for (int a = 0; a < 5; ++a)
#pragma unroll
    for (int b = 0; b <= a; ++b) acc[k++] += weight * (Jv[a] * Jv[b]);
#pragma unroll
  for (int a = 0; a < 5; ++a) acc[15 + a] += f * Jv[a];
}

// One damped step: solves (JtJ) sol = -Jtr (JtJ already damped, lower 15),
// returns false when the step is below 1e-8 (a failed factorisation gives a
// zero step). Pn receives the updated pose.
__device__ inline bool relpose_step(const double* JtJ15, const double* Jtr, const PoseJac& J, const Pose& P,
                                    Pose& Pn) {
  double A[5][5], x[5];
  int k = 0;
  for (int a = 0; a < 5; ++a)
    for (int b = 0; b <= a; ++b) {
      A[a][b] = JtJ15[k];
      A[b][a] = JtJ15[k];
      ++k;
    }
  for (int a = 0; a < 5; ++a) x[a] = Jtr[a];
  if (cholesky_solve<5>(A, x)) {
    for (int a = 0; a < 5; ++a) x[a] = -x[a];
  } else {
    for (int a = 0; a < 5; ++a) x[a] = 0;
  }
  double sn = 0;
  for (int a = 0; a < 5; ++a) sn += x[a] * x[a];
  if (sqrt(sn) < 1e-8) return false;
  double wv[3] = {x[0], x[1], x[2]};
  const double th = sqrt(wv[0] * wv[0] + wv[1] * wv[1] + wv[2] * wv[2]);
  for (int i = 0; i < 3; ++i) wv[i] /= th;
  const double a = sin(th), b = cos(th);
  const double S[9] = {0, -wv[2], wv[1], wv[2], 0, -wv[0], -wv[1], wv[0], 0};
  double S2[9], R[9], M[9], RM[9];
  matmul3(S, S, S2);
  for (int i = 0; i < 9; ++i) M[i] = a * S[i] + (1 - b) * S2[i];
  quat_to_R(P.q, R);
  matmul3(R, M, RM);
  for (int i = 0; i < 9; ++i) RM[i] = R[i] + RM[i];
  R_to_quat(RM, Pn.q);
  for (int i = 0; i < 3; ++i) Pn.t[i] = P.t[i] + (J.tb[i][0] * x[3] + J.tb[i][1] * x[4]);
  return true;
}

}  // namespace ess

// EssentialMatrixEstimator<Nister, Stewenius> on K^-1-normalised coordinates.
struct EssentialModel {
  static constexpr int KIND = 3;
  static constexpr int M = 5;
  static constexpr int MAXSOL = 10;
  static constexpr int LO_MAXSOL = 10;
  static constexpr int NONMIN = 5;
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;
  static constexpr bool AFFINE = false;
  static constexpr bool CTA_VALIDITY = true;
  // maximumSolutions of the minimal solver (the count SPRT uses)
  static constexpr int DECLARED_SOLUTIONS = 10;
  // the non-minimal solver is EssentialMatrixBundleAdjustmentSolver
  // (Stewenius, then every cheirality-consistent pose refined)
  static constexpr bool NONMIN_BA = false;

  __device__ static bool valid_sample(const double*, const int*) { return true; }

  __device__ static int minimal(const double* pts, const int* s, double* out, const double* = nullptr) {
    double tmp[90];
    const int n = ess::nister5(pts, s, tmp);
    // the reference erases failing models from the back; the survivors keep
    // their order
    int k = 0;
    for (int q = 0; q < n; ++q)
      if (FundamentalModel::orientation_valid(tmp + 9 * q, pts, s, 5)) {
        for (int i = 0; i < 9; ++i) out[9 * k + i] = tmp[9 * q + i];
        ++k;
      }
    return k;
  }

  __device__ __forceinline__ static double r2_f64(const double* p, const double* E) {
    return FundamentalModel::r2_f64(p, E);
  }
  __device__ __forceinline__ static double symepi2_f64(const double* p, const double* E) {
    return FundamentalModel::symepi2_f64(p, E);
  }
  __device__ __forceinline__ static float r2_f32(const float4 p, const float* E, float& it) {
    return FundamentalModel::r2_f32(p, E, it);
  }
  __device__ static void prepare_f32(const double* E, const double* c, double S, float* out) {
    FundamentalModel::prepare_f32(E, c, S, out);
  }

  // Per-thread non-minimal fit with unit weights (local-optimisation trials):
  // Stewenius on the rows, each model normalised. Returns the model count.
  __device__ static int fit_thread_multi(const double* pts, const int* idx, int n, double* out) {
    if (n < NONMIN) return 0;
    const int nm = stewenius_thread(pts, idx, n, out);
    for (int q = 0; q < nm; ++q) ess::normalise_sign(out + 9 * q);
    return nm;
  }

  // Stewenius on the rows idx[0..n) (n >= 5) with unit weights, by one
  // thread; the models as the solver returns them.
  __device__ static int stewenius_thread(const double* pts, const int* idx, int n, double* out) {
    int nm;
    if (n == 5) {
      double rows[5][9];
      for (int i = 0; i < 5; ++i) ess::design_row(pts + 4 * idx[i], 1.0, rows[i]);
      nm = ess::stewenius_five(rows, out);
    } else {
      double ata[45];
#pragma unroll
      for (int k = 0; k < 45; ++k) ata[k] = 0;
      for (int i = 0; i < n; ++i) {
        double r[9];
        ess::design_row(pts + 4 * idx[i], 1.0, r);
        int k = 0;
#pragma unroll
        for (int a = 0; a < 9; ++a)
#pragma unroll
          for (int b = 0; b <= a; ++b) ata[k++] += r[a] * r[b];
      }
      double full[81];
      int k = 0;
      for (int a = 0; a < 9; ++a)
        for (int b = 0; b <= a; ++b) {
          full[a * 9 + b] = ata[k];
          full[b * 9 + a] = ata[k];
          ++k;
        }
      nm = ess::stewenius_from_ata(full, out);
    }
    return nm;
  }
};

// Planar-motion essential matrix (findPlanarEssentialMatrix_,
// gcransac_python.cpp:3531-3870): EssentialMatrixEstimator<
// EssentialMatrixTwoPointsPlanar, EssentialMatrixBundleAdjustmentSolver>
// (types.h:121-126) on K^-1-normalised coordinates.
struct EssentialPlanarModel : EssentialModel {
  static constexpr int M = 2;
  static constexpr int MAXSOL = 4;
  static constexpr int NONMIN = 6;  // EssentialMatrixBundleAdjustmentSolver::sampleSize
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;
  static constexpr int DECLARED_SOLUTIONS = 1;  // the solver declares none (SolverEngine's 1)
  static constexpr bool NONMIN_BA = true;

  // EssentialMatrixTwoPointsPlanar::estimateModel
  // (solver_essential_matrix_two_points_planar.h:92-175): rotation about the
  // camera's y axis and translation in its x-z plane. With rows
  // A1 = (y1, -y1 x2) and A2 = (-y2, x1 y2) of the two points, C = -A2^+ A1
  // maps the rotation direction v1 = (cos a, sin a) onto the direction of
  // (a - b); |C v1| = 1 gives a quadratic in cos 2a (coefficients from
  // C^T C), and each root gives the angles +-acos / 2. Models whose entries
  // are not finite (no real root, or |cos 2a| > 1) are dropped here (the
  // reference keeps and scores them; they cannot win); the rest pass the
  // estimator's orientation test on the two points (essential_estimator.h:
  // 166-172).
  __device__ static int minimal(const double* pts, const int* s, double* out, const double* = nullptr) {
    double A1[2][2], A2[2][2];
    for (int i = 0; i < 2; ++i) {
      const double* p = pts + 4 * s[i];
      const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
      A1[i][0] = y1;
      A1[i][1] = -y1 * x2;
      A2[i][0] = -y2;
      A2[i][1] = x1 * y2;
    }
    // (A2^T A2)^-1 A2^T
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
    const double disc = sqrt(cf2 * cf2 - 4 * cf1 * cf3);
    const double c2a1 = (-cf2 + disc) / (2 * cf1), c2a2 = (-cf2 - disc) / (2 * cf1);
    const double alphas[4] = {acos(c2a1) / 2, acos(c2a2) / 2, -acos(c2a1) / 2, -acos(c2a2) / 2};
    int k = 0;
    for (int q = 0; q < 4; ++q) {
      double sa, ca;
      sincos(alphas[q], &sa, &ca);
      double w0 = C[0][0] * ca + C[0][1] * sa, w1 = C[1][0] * ca + C[1][1] * sa;
      const double nw = sqrt(w0 * w0 + w1 * w1);
      w0 /= nw;
      w1 /= nw;
      const double al = atan2(sa, ca), amb = atan2(w1, w0);
      double* E = out + 9 * k;
      E[0] = 0.0; E[1] = -sin(al); E[2] = 0.0;
      E[3] = sin(amb); E[4] = 0.0; E[5] = -cos(amb);
      E[6] = 0.0; E[7] = cos(al); E[8] = 0.0;
      bool fin = true;
      for (int e = 0; e < 9; ++e) fin = fin && isfinite(E[e]);
      if (fin && FundamentalModel::orientation_valid(E, pts, s, 2)) ++k;
    }
    return k;
  }

  // refine_relpose (bundle.cpp:412-452; lm_5dof_impl 176-250) of P over the
  // rows idx[0..n) with unit weights, by one thread: the same LM as the
  // CTA-wide refinement, with sequential sums.
  __device__ static void refine_relpose_thread(const double* pts, const int* idx, int n, ess::Pose& P) {
    auto residual = [&](const ess::Pose& Q) {
      double E[9];
      ess::essential_from_pose(Q, E);
      double c = 0;
      for (int k = 0; k < n; ++k) c += ess::relpose_loss(E, pts + 4 * idx[k]);
      return c;
    };
    double lambda = 1e-3;
    double cost = residual(P);
    bool recompute = true;
    double tot[20];
    ess::PoseJac J;
    for (int iter = 0; iter < 25; ++iter) {
      if (recompute) {
        ess::pose_jacobians(P, J);
        for (int q = 0; q < 20; ++q) tot[q] = 0;
        for (int k = 0; k < n; ++k) ess::relpose_accumulate(J, pts + 4 * idx[k], 1.0, n, tot);
        double gn = 0;
        for (int a = 0; a < 5; ++a) gn += tot[15 + a] * tot[15 + a];
        if (sqrt(gn) < 1e-8) break;
      }
      constexpr int diag[5] = {0, 2, 5, 9, 14};
      for (int a = 0; a < 5; ++a) tot[diag[a]] += lambda;
      ess::Pose Pn;
      if (!ess::relpose_step(tot, tot + 15, J, P, Pn)) break;
      const double cn = residual(Pn);
      if (cn < cost) {
        P = Pn;
        lambda /= 10;
        cost = cn;
        recompute = true;
      } else {
        for (int a = 0; a < 5; ++a) tot[diag[a]] -= lambda;
        lambda *= 10;
        recompute = false;
      }
    }
  }

  // Per-thread non-minimal fit of the local-optimisation trials (unit
  // weights): EssentialMatrixBundleAdjustmentSolver::estimateModel
  // (solver_essential_matrix_bundle_adjustment.h:114-188), Stewenius, then
  // every cheirality-consistent pose (checked on the first row) refined, at
  // most LO_MAXSOL models, each normalised with E33 >= 0.
  __device__ static int fit_thread_multi(const double* pts, const int* idx, int n, double* out) {
    if (n < NONMIN) return 0;
    double init[9 * LO_MAXSOL];
    const int ni = stewenius_thread(pts, idx, n, init);
    double x1[3], x2[3];
    {
      const double* p0 = pts + 4 * idx[0];
      x1[0] = p0[0]; x1[1] = p0[1]; x1[2] = 1.0;
      x2[0] = p0[2]; x2[1] = p0[3]; x2[2] = 1.0;
      const double n1 = sqrt(x1[0] * x1[0] + x1[1] * x1[1] + 1.0);
      const double n2 = sqrt(x2[0] * x2[0] + x2[1] * x2[1] + 1.0);
      for (int i = 0; i < 3; ++i) {
        x1[i] /= n1;
        x2[i] /= n2;
      }
    }
    int nout = 0;
    for (int q = 0; q < ni; ++q) {
      ess::Pose poses[4];
      const int np = ess::poses_from_essential(init + 9 * q, x1, x2, poses);
      for (int v = 0; v < np && nout < LO_MAXSOL; ++v) {
        ess::Pose P = poses[v];
        refine_relpose_thread(pts, idx, n, P);
        ess::essential_from_pose(P, out + 9 * nout);
        ess::normalise_sign(out + 9 * nout);
        ++nout;
      }
    }
    return nout;
  }
};

}  // namespace gcr
