// Oracle (test infrastructure only): fundamental-matrix estimator restated
// from src/pygcransac/include/estimators/fundamental_estimator.h:65-801 with
// its solvers (solver_fundamental_matrix_seven_point.h:91-291,
// solver_fundamental_matrix_eight_point.h:93-182,
// solver_fundamental_matrix_bundle_adjustment.h:114-178,
// solver_fundamental_matrix_plane_and_parallax.h:102-165), the factorised-F
// Levenberg-Marquardt of relative_pose/bundle.cpp:252-339 with
// relative_pose/jacobian_impl.h:470-615, and the findFundamentalMatrix_
// driver (src/pygcransac/src/gcransac_python.cpp:1600-1923).
#pragma once

#include "oracle_common.hpp"
#include "oracle_gcransac.hpp"
#include "oracle_homography.hpp"
#include "oracle_linalg.hpp"
#include "oracle_linalg2.hpp"

namespace oracle {

// Sampson distance (fundamental_estimator.h:195-222)
inline double f_sampson2(const double* p, const Model& F) {
  const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
  const double rxc = F[0] * x2 + F[3] * y2 + F[6];
  const double ryc = F[1] * x2 + F[4] * y2 + F[7];
  const double rwc = F[2] * x2 + F[5] * y2 + F[8];
  const double r = x1 * rxc + y1 * ryc + rwc;
  const double rx = F[0] * x1 + F[1] * y1 + F[2];
  const double ry = F[3] * x1 + F[4] * y1 + F[5];
  return r * r / (rxc * rxc + ryc * ryc + rx * rx + ry * ry);
}

// squaredSymmetricEpipolarDistance (fundamental_estimator.h:224-259)
inline double f_symepi2(const double* p, const Model& F) {
  const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
  const double rxc = F[0] * x2 + F[3] * y2 + F[6];
  const double ryc = F[1] * x2 + F[4] * y2 + F[7];
  const double rwc = F[2] * x2 + F[5] * y2 + F[8];
  const double r = x1 * rxc + y1 * ryc + rwc;
  const double rx = F[0] * x1 + F[1] * y1 + F[2];
  const double ry = F[3] * x1 + F[4] * y1 + F[5];
  const double a = rxc * rxc + ryc * ryc;
  const double b = rx * rx + ry * ry;
  return r * r * (a + b) / (a * b);
}

// Row of the epipolar design matrix (x2 x1, x2 y1, x2, y2 x1, y2 y1, y2, x1, y1, 1) * w.
inline void f_design_row(const double* p, double w, double* r) {
  const double x0 = p[0], y0 = p[1], x1 = p[2], y1 = p[3];
  const double wx0 = w * x0, wy0 = w * y0, wx1 = w * x1, wy1 = w * y1;
  r[0] = wx1 * x0; r[1] = wx1 * y0; r[2] = wx1;
  r[3] = wy1 * x0; r[4] = wy1 * y0; r[5] = wy1;
  r[6] = wx0; r[7] = wy0; r[8] = w;
}

inline bool f_models_from_rows7(std::vector<double>& A, bool guards, std::vector<Model>& models);

// Three-affine-correspondence solver (solver_fundamental_matrix_three_affine.h:84-250):
// rows of eight values (x1, y1, x2, y2, a11, a12, a21, a22); the epipolar row
// of each of the three correspondences and the two affine rows of the first
// two make a 7 x 9 system. Its null space is taken as the seven-point
// solver's LU kernel (the reference takes the two last right singular vectors
// of A^T A: another basis of the same plane, so the same matrices in possibly
// another order); no coefficient checks, as in the reference.
inline bool f_three_affine(const double* const rows[3], std::vector<Model>& models) {
  std::vector<double> A(7 * 9);
  int r = 0;
  for (int i = 0; i < 3; ++i) {
    const double* p = rows[i];
    const double x0 = p[0], y0 = p[1], x1 = p[2], y1 = p[3];
    const double a11 = p[4], a12 = p[5], a21 = p[6], a22 = p[7];
    const double e[9] = {x1 * x0, x1 * y0, x1, y1 * x0, y1 * y0, y1, x0, y0, 1.0};
    for (int k = 0; k < 9; ++k) A[9 * r + k] = e[k];
    ++r;
    if (i < 2) {
      const double u[9] = {x1 + a11 * x0, a11 * y0, a11, y1 + a21 * x0, a21 * y0, a21, 1.0, 0.0, 0.0};
      const double v[9] = {a12 * x0, x1 + a12 * y0, a12, a22 * x0, y1 + a22 * y0, a22, 0.0, 1.0, 0.0};
      for (int k = 0; k < 9; ++k) {
        A[9 * r + k] = u[k];
        A[9 * (r + 1) + k] = v[k];
      }
      r += 2;
    }
  }
  return f_models_from_rows7(A, false, models);
}

// Four-SIFT-correspondence solver (solver_fundamental_matrix_four_sift.h:89-250):
// rows (u1, v1, u2, v2, q1, q2, o1, o2) with feature scales q and orientations
// o; the epipolar row of each of the four correspondences and the
// orientation-scale row of the first three make a 7 x 9 system, whose null
// space is taken as the seven-point solver's LU kernel (the reference takes
// the FullPivLU kernel of A^T A: another basis of the same plane); no
// coefficient checks, as in the reference.
inline bool f_four_sift(const double* const rows[4], std::vector<Model>& models) {
  std::vector<double> A(7 * 9);
  int r = 0;
  for (int i = 0; i < 4; ++i) {
    const double* p = rows[i];
    const double u1 = p[0], v1 = p[1], u2 = p[2], v2 = p[3], q1 = p[4], q2 = p[5], o1 = p[6], o2 = p[7];
    const double s1 = std::sin(o1), c1 = std::cos(o1), s2 = std::sin(o2), c2 = std::cos(o2);
    const double e[9] = {u2 * u1, u2 * v1, u2, v2 * u1, v2 * v1, v2, u1, v1, 1.0};
    for (int k = 0; k < 9; ++k) A[9 * r + k] = e[k];
    ++r;
    if (i == 3) break;
    const double o[9] = {s2 * s2 * q2 * u1 - c1 * c2 * q1 * u2 - q2 * u1,
                         s2 * s2 * q2 * v1 - s1 * c2 * q1 * u2 - q2 * v1,
                         s2 * s2 * q2 - q2,
                         -c2 * s2 * q2 * u1 - c1 * c2 * q1 * v2,
                         -c2 * s2 * q2 * v1 - s1 * c2 * q1 * v2,
                         -c2 * s2 * q2,
                         -c1 * c2 * q1,
                         -s1 * c2 * q1,
                         0.0};
    for (int k = 0; k < 9; ++k) A[9 * r + k] = o[k];
    ++r;
  }
  return f_models_from_rows7(A, false, models);
}

// Seven-point solver (solver_fundamental_matrix_seven_point.h:91-291) on the
// rows `rows`, weights w[i] per row (nullptr: none).
inline bool f_seven_point(const double* const* rows, const double* w, std::vector<Model>& models) {
  std::vector<double> A(7 * 9);
  for (int i = 0; i < 7; ++i) {
    if (w) f_design_row(rows[i], w[i], &A[i * 9]);
    else {
      const double x0 = rows[i][0], y0 = rows[i][1], x1 = rows[i][2], y1 = rows[i][3];
      double* r = &A[i * 9];
      r[0] = x1 * x0; r[1] = x1 * y0; r[2] = x1; r[3] = y1 * x0; r[4] = y1 * y0; r[5] = y1;
      r[6] = x0; r[7] = y0; r[8] = 1;
    }
  }
  return f_models_from_rows7(A, true, models);
}

// The models of a 7 x 9 epipolar system A (row-major): the two-dimensional
// null space (FullPivLU kernel), the cubic det(l f1 + (1 - l) f2) = 0 and each
// real root's matrix normalised to F33 = 1. `guards`: the seven-point
// solver's checks of the cubic's coefficients
// (solver_fundamental_matrix_seven_point.h:240-251).
inline bool f_models_from_rows7(std::vector<double>& A, bool guards, std::vector<Model>& models) {
  std::vector<double> K;
  if (fullpiv_lu_kernel(A, 7, 9, K) != 2) return false;
  double f1[9], f2[9];
  for (int i = 0; i < 9; ++i) {
    f1[i] = K[i * 2 + 0];
    f2[i] = K[i * 2 + 1];
  }
  for (int i = 0; i < 9; ++i) f1[i] -= f2[i];
  double c[4], t0, t1, t2;
  t0 = f2[4] * f2[8] - f2[5] * f2[7];
  t1 = f2[3] * f2[8] - f2[5] * f2[6];
  t2 = f2[3] * f2[7] - f2[4] * f2[6];
  c[0] = f2[0] * t0 - f2[1] * t1 + f2[2] * t2;
  c[1] = f1[0] * t0 - f1[1] * t1 + f1[2] * t2 - f1[3] * (f2[1] * f2[8] - f2[2] * f2[7]) +
         f1[4] * (f2[0] * f2[8] - f2[2] * f2[6]) - f1[5] * (f2[0] * f2[7] - f2[1] * f2[6]) +
         f1[6] * (f2[1] * f2[5] - f2[2] * f2[4]) - f1[7] * (f2[0] * f2[5] - f2[2] * f2[3]) +
         f1[8] * (f2[0] * f2[4] - f2[1] * f2[3]);
  t0 = f1[4] * f1[8] - f1[5] * f1[7];
  t1 = f1[3] * f1[8] - f1[5] * f1[6];
  t2 = f1[3] * f1[7] - f1[4] * f1[6];
  c[2] = f2[0] * t0 - f2[1] * t1 + f2[2] * t2 - f2[3] * (f1[1] * f1[8] - f1[2] * f1[7]) +
         f2[4] * (f1[0] * f1[8] - f1[2] * f1[6]) - f2[5] * (f1[0] * f1[7] - f1[1] * f1[6]) +
         f2[6] * (f1[1] * f1[5] - f1[2] * f1[4]) - f2[7] * (f1[0] * f1[5] - f1[2] * f1[3]) +
         f2[8] * (f1[0] * f1[4] - f1[1] * f1[3]);
  c[3] = f1[0] * t0 - f1[1] * t1 + f1[2] * t2;
  const double eps = std::numeric_limits<double>::epsilon();
  if (guards && (std::fabs(c[0] + c[1] + c[2] + c[3]) < 1e-9 || std::fabs(c[0]) < eps || std::fabs(c[1]) < eps ||
                 std::fabs(c[2]) < eps || std::fabs(c[3]) < eps))
    return false;
  if (!(c[3] != 0.0)) return false;  // no cubic (the polynomial solver needs a leading coefficient)
  const std::vector<double> roots = cubic_real_roots(c);
  const int n = (int)roots.size();
  if (n < 1 || n > 3) return false;
  for (double root : roots) {
    double lambda = root, mu = 1.;
    const double s = f1[8] * root + f2[8];
    if (std::fabs(s) > eps) {
      mu = 1.0 / s;
      lambda *= mu;
      Model F;
      for (int i = 0; i < 8; ++i) F[i] = f1[i] * lambda + f2[i] * mu;
      F[8] = 1.0;
      models.push_back(F);
    }
  }
  return true;
}

// Eight-point solver (solver_fundamental_matrix_eight_point.h:93-182): the last
// column of Q of the complete-pivoting QR of A^T A.
inline void f_eight_point(const double* const* rows, int n, const double* w, std::vector<Model>& models) {
  double AtA[81] = {0};
  for (int i = 0; i < n; ++i) {
    double r[9];
    f_design_row(rows[i], w ? w[i] : 1.0, r);
    for (int a = 0; a < 9; ++a)
      for (int b = 0; b < 9; ++b) AtA[a * 9 + b] += r[a] * r[b];
  }
  std::vector<double> M(AtA, AtA + 81);
  double q[9];
  fullpiv_householder_q_lastcol(M, 9, q);
  Model F;
  for (int i = 0; i < 9; ++i) F[i] = q[i];
  models.push_back(F);
}

// FactorizedFundamentalMatrix (jacobian_impl.h:472-490): F = u0 v0^T + sigma u1 v1^T.
struct FactF {
  double U[9], V[9], sigma;
  void from(const Model& F) {
    double s[3];
    svd3(F.data(), U, s, V);
    sigma = s[1] / s[0];
  }
  Model F() const {
    Model f;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) f[i * 3 + j] = U[i * 3] * V[j * 3] + sigma * U[i * 3 + 1] * V[j * 3 + 1];
    return f;
  }
};

// FundamentalJacobianAccumulator with TRUNCATED loss (robust_loss.h:19-31) and
// the LM of lm_F_impl (bundle.cpp:252-339), options of the BA solver
// (25 iterations, loss scale 1, tolerances 1e-8, lambda0 1e-3). Row k uses
// weights[k] when weights is given.
inline void f_refine_lm(const double* const* rows, int n, const double* weights, Model& Fio) {
  const double sq_thr = 1.0;
  auto cost_of = [&](const FactF& FF) {
    const Model F = FF.F();
    double cost = 0;
    for (int k = 0; k < n; ++k) {
      const double x1 = rows[k][0], y1 = rows[k][1], x2 = rows[k][2], y2 = rows[k][3];
      const double Fx0 = F[0] * x1 + F[1] * y1 + F[2], Fx1 = F[3] * x1 + F[4] * y1 + F[5],
                   Fx2 = F[6] * x1 + F[7] * y1 + F[8];
      const double C = x2 * Fx0 + y2 * Fx1 + Fx2;
      const double a0 = F[0] * x2 + F[3] * y2 + F[6], a1 = F[1] * x2 + F[4] * y2 + F[7];
      const double nJc = Fx0 * Fx0 + Fx1 * Fx1 + a0 * a0 + a1 * a1;
      const double r2 = C * C / nJc;
      const double l = std::min(r2, sq_thr);
      cost += weights ? weights[k] * l : l;
    }
    return cost;
  };
  double lambda = 1e-3;
  FactF F;
  F.from(Fio);
  double cost = cost_of(F);
  bool recompute = true;
  std::vector<double> JtJ(49, 0.0);
  double Jtr[7] = {0};
  for (int iter = 0; iter < 25; ++iter) {
    if (recompute) {
      std::fill(JtJ.begin(), JtJ.end(), 0.0);
      for (double& v : Jtr) v = 0;
      const Model Fm = F.F();
      double ds[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) ds[i * 3 + j] = F.U[i * 3 + 1] * F.V[j * 3 + 1];
      // dF/dparams (9 x 7), rows in column-major order of F as in the reference
      const double* f = Fm.data();
      auto FF = [&](int i, int j) { return f[i * 3 + j]; };
      const double D[9][7] = {
          {0, FF(2, 0), -FF(1, 0), 0, FF(0, 2), -FF(0, 1), ds[0]},
          {-FF(2, 0), 0, FF(0, 0), 0, FF(1, 2), -FF(1, 1), ds[3]},
          {FF(1, 0), -FF(0, 0), 0, 0, FF(2, 2), -FF(2, 1), ds[6]},
          {0, FF(2, 1), -FF(1, 1), -FF(0, 2), 0, FF(0, 0), ds[1]},
          {-FF(2, 1), 0, FF(0, 1), -FF(1, 2), 0, FF(1, 0), ds[4]},
          {FF(1, 1), -FF(0, 1), 0, -FF(2, 2), 0, FF(2, 0), ds[7]},
          {0, FF(2, 2), -FF(1, 2), FF(0, 1), -FF(0, 0), 0, ds[2]},
          {-FF(2, 2), 0, FF(0, 2), FF(1, 1), -FF(1, 0), 0, ds[5]},
          {FF(1, 2), -FF(0, 2), 0, FF(2, 1), -FF(2, 0), 0, ds[8]}};
      for (int k = 0; k < n; ++k) {
        const double p0 = rows[k][0], p1 = rows[k][1], q0 = rows[k][2], q1 = rows[k][3];
        const double Fx0 = f[0] * p0 + f[1] * p1 + f[2], Fx1 = f[3] * p0 + f[4] * p1 + f[5],
                     Fx2 = f[6] * p0 + f[7] * p1 + f[8];
        const double C = q0 * Fx0 + q1 * Fx1 + Fx2;
        const double J0 = f[0] * q0 + f[3] * q1 + f[6], J1 = f[1] * q0 + f[4] * q1 + f[7];
        const double J2 = Fx0, J3 = Fx1;
        const double nJ = std::sqrt(J0 * J0 + J1 * J1 + J2 * J2 + J3 * J3);
        const double inv = 1.0 / nJ;
        const double r = C * inv;
        double weight = ((r * r) < sq_thr ? 1.0 : 0.0) / n;
        if (weights) weight = weights[k] * weight;
        if (weight == 0.0) continue;
        double dF[9] = {p0 * q0, p0 * q1, p0, p1 * q0, p1 * q1, p1, q0, q1, 1.0};
        const double s = C * inv * inv;
        dF[0] -= s * (J2 * p0 + J0 * q0);
        dF[1] -= s * (J3 * p0 + J0 * q1);
        dF[2] -= s * (J0);
        dF[3] -= s * (J2 * p1 + J1 * q0);
        dF[4] -= s * (J3 * p1 + J1 * q1);
        dF[5] -= s * (J1);
        dF[6] -= s * (J2);
        dF[7] -= s * (J3);
        for (double& v : dF) v *= inv;
        double J[7];
        for (int c = 0; c < 7; ++c) {
          double t = 0;
          for (int rr = 0; rr < 9; ++rr) t += dF[rr] * D[rr][c];
          J[c] = t;
        }
        for (int a = 0; a < 7; ++a) {
          Jtr[a] += weight * C * inv * J[a];
          for (int b = 0; b <= a; ++b) JtJ[a * 7 + b] += weight * (J[a] * J[b]);
        }
      }
      double gn = 0;
      for (double v : Jtr) gn += v * v;
      if (std::sqrt(gn) < 1e-8) break;
    }
    for (int k = 0; k < 7; ++k) JtJ[k * 7 + k] += lambda;
    double sol[7] = {0, 0, 0, 0, 0, 0, 0}, mJtr[7];
    for (int k = 0; k < 7; ++k) mJtr[k] = -Jtr[k];
    if (!llt_solve(JtJ, 7, mJtr, sol))
      for (double& v : sol) v = 0;
    double sn = 0;
    for (double v : sol) sn += v * v;
    if (std::sqrt(sn) < 1e-8) break;
    double w1[3] = {sol[0], sol[1], sol[2]}, w2[3] = {sol[3], sol[4], sol[5]};
    const double th1 = std::sqrt(w1[0] * w1[0] + w1[1] * w1[1] + w1[2] * w1[2]);
    const double th2 = std::sqrt(w2[0] * w2[0] + w2[1] * w2[1] + w2[2] * w2[2]);
    for (int i = 0; i < 3; ++i) { w1[i] /= th1; w2[i] /= th2; }
    const double a1 = std::sin(th1), b1 = std::cos(th1), a2 = std::sin(th2), b2 = std::cos(th2);
    auto rot = [](const double* w, double a, double b, const double* M, double* out) {
      // out = M + (a [w]x + (1 - b) [w]x^2) M
      const double S[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
      double S2[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) S2[i * 3 + j] = S[i * 3] * S[j] + S[i * 3 + 1] * S[3 + j] + S[i * 3 + 2] * S[6 + j];
      double R[9];
      for (int i = 0; i < 9; ++i) R[i] = a * S[i] + (1 - b) * S2[i];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          out[i * 3 + j] = M[i * 3 + j] + R[i * 3] * M[j] + R[i * 3 + 1] * M[3 + j] + R[i * 3 + 2] * M[6 + j];
    };
    FactF Fn;
    rot(w1, a1, b1, F.U, Fn.U);
    rot(w2, a2, b2, F.V, Fn.V);
    Fn.sigma = F.sigma + sol[6];
    const double cost_new = cost_of(Fn);
    if (cost_new < cost) {
      F = Fn;
      lambda /= 10;
      cost = cost_new;
      recompute = true;
    } else {
      for (int k = 0; k < 7; ++k) JtJ[k * 7 + k] -= lambda;
      lambda *= 10;
      recompute = false;
    }
  }
  Fio = F.F();
}

// The two fundamental-matrix estimator configurations the reference uses:
// the default (7-point minimal, bundle-adjustment non-minimal, DEGENSAC on)
// and the one inside DEGENSAC (plane-and-parallax minimal with a fixed
// homography, 8-point non-minimal, validity ratio 0, DEGENSAC off).
struct FundamentalEstimator {
  bool plane_parallax = false;
  Model homography{};           // plane-and-parallax only
  double min_ratio = 0.5;
  bool use_degensac = true;
  mutable uint32_t degensac_calls = 0;
  uint64_t seed = 0;            // stream key of the DEGENSAC samplers
  mutable bool degensac_ran = false;

  bool affine = false;           // three affine correspondences per minimal sample (rows of 8)
  bool sift = false;             // four SIFT correspondences per minimal sample (rows of 8)
  static constexpr size_t kSample = 7;
  size_t sample_size_rt() const { return plane_parallax ? 2 : (sift ? 4 : (affine ? 3 : 7)); }
  static constexpr size_t sample_size() { return 7; }
  static constexpr bool space_partitioning = false;  // SpacePartitioningRANSAC applies
  static constexpr size_t max_solutions() { return 3; }  // maximumMinimalSolutions
  size_t inlier_limit() const { return 7 * sample_size_rt(); }
  // FundamentalMatrixEightPointSolver (plane-and-parallax inner runs and the
  // affine-correspondence estimator, types.h:83-86) or the bundle adjustment
  size_t non_minimal_sample_size() const { return plane_parallax || affine ? 8 : 7; }

  double squared_residual(const double* p, const Model& F) const { return f_sampson2(p, F); }

  // getEpipole / isOrientationValid (fundamental_estimator.h:737-800)
  static bool orientation_valid(const Model& F, const Mat& pts, const size_t* s, size_t n) {
    constexpr double epsilon = 1.9984e-15;
    double e[3];
    const double r0[3] = {F[0], F[1], F[2]}, r1[3] = {F[3], F[4], F[5]}, r2[3] = {F[6], F[7], F[8]};
    cross3(r0, r2, e);
    bool big = false;
    for (int i = 0; i < 3; ++i)
      if (e[i] > epsilon || e[i] < -epsilon) big = true;
    if (!big) cross3(r1, r2, e);
    auto sig = [&](const double* p) {
      const double s1 = F[0] * p[2] + F[3] * p[3] + F[6];
      const double s2 = e[1] - e[2] * p[1];
      return s1 * s2;
    };
    const double sg2 = sig(pts.row(s[0]));
    for (size_t i = 1; i < n; ++i)
      if (sg2 * sig(pts.row(s[i])) < 0) return false;
    return true;
  }

  bool is_valid_sample(const Mat&, const size_t*) const { return true; }

  bool estimate_minimal(const Mat& pts, const size_t* s, std::vector<Model>& models) const {
    std::vector<Model> tmp;
    if (sift) {
      const double* rows[4] = {pts.row(s[0]), pts.row(s[1]), pts.row(s[2]), pts.row(s[3])};
      f_four_sift(rows, tmp);
    } else if (affine) {
      const double* rows[3] = {pts.row(s[0]), pts.row(s[1]), pts.row(s[2])};
      f_three_affine(rows, tmp);
    } else if (!plane_parallax) {
      const double* rows[7];
      for (int i = 0; i < 7; ++i) rows[i] = pts.row(s[i]);
      f_seven_point(rows, nullptr, tmp);
    } else {
      const double *p1 = pts.row(s[0]), *p2 = pts.row(s[1]);
      const Model& H = homography;
      auto proj = [&](const double* p, double* o) {
        for (int i = 0; i < 3; ++i) o[i] = H[i * 3] * p[0] + H[i * 3 + 1] * p[1] + H[i * 3 + 2];
      };
      double q1[3], q2[3], d1[3] = {p1[2], p1[3], 1}, d2[3] = {p2[2], p2[3], 1}, l1[3], l2[3], e[3];
      proj(p1, q1);
      proj(p2, q2);
      cross3(q1, d1, l1);
      cross3(q2, d2, l2);
      cross3(l1, l2, e);
      if (std::fabs(e[2]) >= std::numeric_limits<double>::epsilon()) {
        const double ex[9] = {0, -e[2], e[1], e[2], 0, -e[0], -e[1], e[0], 0};
        Model F;
        matmul3(ex, H.data(), F.data());
        tmp.push_back(F);
      }
    }
    // estimateModel keeps the models passing the oriented epipolar constraint
    const size_t m = sample_size_rt();
    for (const Model& F : tmp)
      if (orientation_valid(F, pts, s, m)) models.push_back(F);
    return !models.empty();
  }

  // estimateModelNonminimal (fundamental_estimator.h:574-618)
  bool estimate_nonminimal(const Mat& pts, const size_t* s, size_t n, std::vector<Model>& models,
                           const double* weights) const {
    if (n < non_minimal_sample_size()) return false;
    double ms[2] = {0, 0}, md[2] = {0, 0};
    for (size_t i = 0; i < n; ++i) {
      const double* p = pts.row(s[i]);
      ms[0] += p[0]; ms[1] += p[1]; md[0] += p[2]; md[1] += p[3];
    }
    ms[0] /= n; ms[1] /= n; md[0] /= n; md[1] /= n;
    double ads = 0, add = 0;
    for (size_t i = 0; i < n; ++i) {
      const double* p = pts.row(s[i]);
      const double dx1 = ms[0] - p[0], dy1 = ms[1] - p[1], dx2 = md[0] - p[2], dy2 = md[1] - p[3];
      ads += std::sqrt(dx1 * dx1 + dy1 * dy1);
      add += std::sqrt(dx2 * dx2 + dy2 * dy2);
    }
    ads /= n; add /= n;
    const double rs = M_SQRT2 / ads, rd = M_SQRT2 / add;
    std::vector<double> np(n * 4);
    std::vector<const double*> rows(n);
    for (size_t i = 0; i < n; ++i) {
      const double* p = pts.row(s[i]);
      np[i * 4 + 0] = (p[0] - ms[0]) * rs;
      np[i * 4 + 1] = (p[1] - ms[1]) * rs;
      np[i * 4 + 2] = (p[2] - md[0]) * rd;
      np[i * 4 + 3] = (p[3] - md[1]) * rd;
      rows[i] = &np[i * 4];
    }
    // packed row i carries weights[i] (point index i), as in the reference
    std::vector<Model> out;
    if (plane_parallax || affine) {
      f_eight_point(rows.data(), (int)n, weights, out);
    } else {
      // FundamentalMatrixBundleAdjustmentSolver: 8-point (7-point below 8 rows) then LM
      if (n >= 8) f_eight_point(rows.data(), (int)n, weights, out);
      else f_seven_point(rows.data(), weights, out);
      for (Model& F : out) f_refine_lm(rows.data(), (int)n, weights, F);
    }
    const double Ts[9] = {rs, 0, -rs * ms[0], 0, rs, -rs * ms[1], 0, 0, 1};
    const double TdT[9] = {rd, 0, 0, 0, rd, 0, -rd * md[0], -rd * md[1], 1};
    for (Model& F : out) {
      double t[9];
      matmul3(TdT, F.data(), t);
      Model G;
      matmul3(t, Ts, G.data());
      double nrm = 0;
      for (double v : G) nrm += v * v;
      nrm = std::sqrt(nrm);
      for (double& v : G) v /= nrm;
      if (G[8] < 0)
        for (double& v : G) v = -v;
      models.push_back(G);
    }
    return true;
  }

  bool is_valid_model(Model& model, const Mat& pts, const std::vector<size_t>& inliers, const size_t* sample,
                      double threshold, bool& updated) const;
};

// applyDegensac (fundamental_estimator.h:341-572).
inline bool degensac(const FundamentalEstimator& est, Model& model, const Mat& pts, const std::vector<size_t>& inliers,
                     const size_t* sample, double threshold, bool& updated) {
  updated = false;
  static const int triplets[15] = {0, 1, 2, 3, 4, 5, 0, 1, 6, 3, 4, 6, 2, 5, 6};
  double U[9], s[3], V[9];
  svd3(model.data(), U, s, V);
  const double ep[3] = {U[2] / U[8], U[5] / U[8], 1.0};
  const double ex[9] = {0, -ep[2], ep[1], ep[2], 0, -ep[0], -ep[1], ep[0], 0};
  double A[9];
  matmul3(ex, model.data(), A);
  bool degenerate = false;
  Model bestH{};
  const double sq_h_thr = 4.0;
  for (int t = 0; t < 5; ++t) {
    const size_t i1 = sample[triplets[3 * t]], i2 = sample[triplets[3 * t + 1]], i3 = sample[triplets[3 * t + 2]];
    const double* P[3] = {pts.row(i1), pts.row(i2), pts.row(i3)};
    double b[3], M[9];
    for (int k = 0; k < 3; ++k) {
      const double x1[3] = {P[k][0], P[k][1], 1}, x2[3] = {P[k][2], P[k][3], 1};
      double pe[3], Ax[3], c[3];
      cross3(x2, ep, pe);
      for (int r = 0; r < 3; ++r) Ax[r] = A[r * 3] * x1[0] + A[r * 3 + 1] * x1[1] + A[r * 3 + 2] * x1[2];
      cross3(x2, Ax, c);
      b[k] = (c[0] * pe[0] + c[1] * pe[1] + c[2] * pe[2]) / (pe[0] * pe[0] + pe[1] * pe[1] + pe[2] * pe[2]);
      M[k * 3] = x1[0]; M[k * 3 + 1] = x1[1]; M[k * 3 + 2] = x1[2];
    }
    double Mi[9];
    inverse3(M, Mi);
    double mb[3];
    for (int r = 0; r < 3; ++r) mb[r] = Mi[r * 3] * b[0] + Mi[r * 3 + 1] * b[1] + Mi[r * 3 + 2] * b[2];
    Model H;
    for (int r = 0; r < 3; ++r)
      for (int c2 = 0; c2 < 3; ++c2) H[r * 3 + c2] = A[r * 3 + c2] - ep[r] * mb[c2];
    size_t cnt = 3;
    for (int i = 0; i < 7; ++i) {
      const size_t idx = sample[i];
      if (idx == i1 || idx == i2 || idx == i3) continue;
      if (HomographyEstimator().squared_residual(pts.row(idx), H) < sq_h_thr) ++cnt;
    }
    if (cnt >= 5) {
      bestH = H;
      degenerate = true;
      break;
    }
  }
  if (!degenerate) return true;
  est.degensac_ran = true;
  HomographyEstimator hest;
  std::vector<size_t> h_inl;
  for (size_t i : inliers)
    if (hest.squared_residual(pts.row(i), bestH) < sq_h_thr) h_inl.push_back(i);
  if (h_inl.size() < 4) return false;
  std::vector<Model> hs;
  hest.estimate_nonminimal(pts, h_inl.data(), h_inl.size(), hs, nullptr);
  if (hs.size() != 1) return false;
  FundamentalEstimator pp;
  pp.plane_parallax = true;
  pp.homography = hs[0];
  pp.min_ratio = 0.0;
  pp.use_degensac = false;
  GCRansac<FundamentalEstimator, MSACScoring<FundamentalEstimator>> g;
  g.settings.threshold = threshold;
  g.settings.spatial_coherence_weight = 0;
  g.settings.confidence = 0.99;
  const uint32_t stream = 16u + est.degensac_calls++;
  UniformSampler sampler(est.seed, stream);
  Model m2{};
  g.run(pts, pp, &sampler, &sampler, nullptr, m2);
  if (g.statistics.inliers.size() > inliers.size()) {
    updated = true;
    model = m2;
  }
  return true;
}

inline bool FundamentalEstimator::is_valid_model(Model& model, const Mat& pts, const std::vector<size_t>& inliers,
                                                 const size_t* sample, double threshold, bool& updated) const {
  const size_t m = sample_size_rt();
  const size_t min_n = std::max(m, (size_t)((double)inliers.size() * min_ratio));
  const double sq = threshold * threshold;
  size_t cnt = 0;
  bool passed = false;
  for (size_t i : inliers)
    if (f_symepi2(pts.row(i), model) < sq)
      if (++cnt >= min_n) {
        passed = true;
        break;
      }
  if (!passed) return false;
  if (!plane_parallax && use_degensac) return degensac(*this, model, pts, inliers, sample, threshold, updated);
  return true;
}

// The affine-correspondence fundamental-matrix estimator of
// findFundamentalMatrixAC_ (gcransac_python.cpp:1924-2221):
// FundamentalMatrixEstimator<FundamentalMatrixThreeAffineSolver,
// FundamentalMatrixEightPointSolver> (types.h:83-86) — three correspondences
// per minimal sample, an inner sample of 7 x 3 in the local optimisation, the
// plain 8-point solver as its non-minimal solver, and no DEGENSAC
// (fundamental_estimator.h:326 runs it for samples of 7 or more).
struct FundamentalAffineEstimator : FundamentalEstimator {
  FundamentalAffineEstimator() {
    affine = true;
    use_degensac = false;
  }
  static constexpr size_t sample_size() { return 3; }
};

// The SIFT-correspondence fundamental-matrix estimator of
// findFundamentalMatrixSIFT_ (gcransac_python.cpp:2222-2518):
// FundamentalMatrixEstimator<FundamentalMatrixFourSIFTSolver,
// FundamentalMatrixEightPointSolver> (types.h:88-90) — four correspondences
// per minimal sample, an inner sample of 7 x 4, the plain 8-point solver as
// its non-minimal solver, no DEGENSAC.
struct FundamentalSiftEstimator : FundamentalEstimator {
  FundamentalSiftEstimator() {
    affine = true;  // rows of 8, the 8-point non-minimal solver
    sift = true;
    use_degensac = false;
  }
  static constexpr size_t sample_size() { return 4; }
};

}  // namespace oracle
