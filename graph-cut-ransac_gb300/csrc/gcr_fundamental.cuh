// Fundamental-matrix model on the device: 7-point minimal solver with the
// oriented epipolar constraint, Sampson residuals, the symmetric epipolar
// validity test and the DEGENSAC degeneracy test, the normalised 8-point +
// Levenberg-Marquardt non-minimal solver, and the plane-and-parallax model of
// the DEGENSAC inner run.
//
// Behaviour follows src/pygcransac/include/estimators/fundamental_estimator.h
// (estimateModel 161-184, Sampson 195-222, symmetric distance 224-259,
// isValidModel 287-338, applyDegensac 341-572, estimateModelNonminimal
// 574-618, orientation 737-800) and the solvers
// solver_fundamental_matrix_seven_point.h:91-291,
// solver_fundamental_matrix_eight_point.h:93-182,
// solver_fundamental_matrix_bundle_adjustment.h:114-178,
// solver_fundamental_matrix_plane_and_parallax.h:102-165 and
// relative_pose/bundle.cpp:252-339 + jacobian_impl.h:470-615.
#pragma once

#include "gcr_device.cuh"
#include "gcr_homography.cuh"
#include "gcr_linalg.cuh"

namespace gcr {

__device__ __forceinline__ void dcross3(const double* a, const double* b, double* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

// |x| compared through the bit pattern (keeps pivot searches off the FP64 pipe)
__device__ __forceinline__ long long dabs_bits(double x) { return __double_as_longlong(x) & 0x7fffffffffffffffLL; }

// Kernel basis of the 7x9 design matrix by LU with complete pivoting, in the
// basis Eigen's FullPivLU::kernel() returns (free pivoted columns set to 1).
// Returns the kernel dimension (the solver needs 2).
__device__ inline int lu_kernel_7x9(double A[7][9], double f1[9], double f2[9]) {
  // Every index is a compile-time constant after unrolling (row and column
  // swaps are selects), so the 7x9 system stays in registers.
  int cp[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) cp[j] = j;
  long long maxpivot = 0;
  int nonzero = 7;
  bool stopped = false;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    int bi = k, bj = k;
    long long best = -1;
#pragma unroll
    for (int i = k; i < 7; ++i)
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
      for (int i = k + 1; i < 7; ++i) {
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
        for (int i = 0; i < 7; ++i) {
          const double t = A[i][k], u = A[i][j];
          A[i][k] = s ? u : t;
          A[i][j] = s ? t : u;
        }
        const int t = cp[k], u = cp[j];
        cp[k] = s ? u : t;
        cp[j] = s ? t : u;
      }
      const double inv = 1.0 / A[k][k];
#pragma unroll
      for (int i = k + 1; i < 7; ++i) {
        const double f = A[i][k] * inv;
        A[i][k] = f;
#pragma unroll
        for (int j = k + 1; j < 9; ++j) A[i][j] -= f * A[k][j];
      }
    }
  }
  const double thr = 2.220446049250313e-16 * 7.0 * __longlong_as_double(maxpivot);
  int rank = 0;
#pragma unroll
  for (int i = 0; i < 7; ++i)
    if (i < nonzero && fabs(A[i][i]) > thr) ++rank;
  if (rank != 7) return 9 - rank;
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    double x[7];
#pragma unroll
    for (int i = 6; i >= 0; --i) {
      double s = -A[i][7 + j];
#pragma unroll
      for (int q = i + 1; q < 7; ++q) s -= A[i][q] * x[q];
      x[i] = s / A[i][i];
    }
    double* o = j == 0 ? f1 : f2;
    // o[cp[i]] = x[i] (i < 7), o[cp[7 + j]] = 1, others 0: selects over the
    // static output index
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      double v = 0.0;
#pragma unroll
      for (int i = 0; i < 7; ++i) v = (cp[i] == t) ? x[i] : v;
      v = (cp[7 + j] == t) ? 1.0 : v;
      o[t] = v;
    }
  }
  return 2;
}

// Real roots of c0 + c1 x + c2 x^2 + c3 x^3: closed form (trigonometric or
// Cardano), Newton-polished; a complex pair with |imaginary part| < 1e-12
// contributes its real part twice (the PolynomialSolver::realRoots rule).
__device__ inline int cubic_real_roots(const double c[4], double r[3]) {
  const double a = c[2] / c[3], b = c[1] / c[3], d = c[0] / c[3];
  const double p = b - a * a / 3.0;
  const double q = 2.0 * a * a * a / 27.0 - a * b / 3.0 + d;
  const double disc = q * q / 4.0 + p * p * p / 27.0;
  auto polish = [&](double x) {
    for (int it = 0; it < 3; ++it) {
      const double f = ((c[3] * x + c[2]) * x + c[1]) * x + c[0];
      const double df = (3 * c[3] * x + 2 * c[2]) * x + c[1];
      if (df == 0) break;
      const double nx = x - f / df;
      if (!isfinite(nx)) break;
      x = nx;
    }
    return x;
  };
  int n = 0;
  if (disc > 0) {
    const double sq = sqrt(disc);
    const double u = cbrt(-q / 2.0 + sq), v = cbrt(-q / 2.0 - sq);
    r[n++] = polish(u + v - a / 3.0);
    const double re = -(u + v) / 2.0 - a / 3.0;
    const double im = 0.8660254037844386 * (u - v);
    if (fabs(im) < 1e-12) {
      r[n++] = re;
      r[n++] = re;
    }
  } else {
    const double rr = sqrt(fmax(0.0, -p / 3.0));
    double arg = rr > 0 ? (3.0 * q) / (2.0 * p * rr) : 0.0;
    arg = fmax(-1.0, fmin(1.0, arg));
    const double phi = acos(arg) / 3.0;
    for (int k = 0; k < 3; ++k) r[n++] = polish(2 * rr * cos(phi - 2.0943951023931957 * k) - a / 3.0);
  }
  return n;
}

struct FundamentalModel {
  static constexpr int KIND = 1;
  static constexpr int M = 7;
  static constexpr int MAXSOL = 3;
  static constexpr int LO_MAXSOL = 1;
  static constexpr int NONMIN = 7;
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;
  static constexpr bool AFFINE = false;
  static constexpr bool DEGENSAC = true;          // isValidModel's plane check (samples of 7)
  static constexpr bool EPILOGUE_WEIGHTED = true;  // findFundamentalMatrix_'s bundle adjustment weights
  static constexpr bool NONMIN_LM = true;          // non-minimal solver: bundle adjustment (8-point + LM)
  static constexpr bool CTA_VALIDITY = true;

  // oriented epipolar constraint of a sample (getEpipole + isOrientationValid)
  __device__ static bool orientation_valid(const double* F, const double* pts, const int* s, int n) {
    const double eps = 1.9984e-15;
    double e[3];
    const double r0[3] = {F[0], F[1], F[2]}, r1[3] = {F[3], F[4], F[5]}, r2[3] = {F[6], F[7], F[8]};
    dcross3(r0, r2, e);
    if (!(e[0] > eps || e[0] < -eps || e[1] > eps || e[1] < -eps || e[2] > eps || e[2] < -eps)) dcross3(r1, r2, e);
    auto sig = [&](const double* p) { return (F[0] * p[2] + F[3] * p[3] + F[6]) * (e[1] - e[2] * p[1]); };
    const double s0 = sig(pts + 4 * s[0]);
    for (int i = 1; i < n; ++i)
      if (s0 * sig(pts + 4 * s[i]) < 0) return false;
    return true;
  }

  __device__ static bool valid_sample(const double*, const int*) { return true; }

  // seven-point solver on the given rows (weights: none); up to three models
  __device__ static int seven_point(const double* const rows[7], double* out) {
    double A[7][9];
    for (int i = 0; i < 7; ++i) {
      const double x0 = rows[i][0], y0 = rows[i][1], x1 = rows[i][2], y1 = rows[i][3];
      A[i][0] = x1 * x0; A[i][1] = x1 * y0; A[i][2] = x1;
      A[i][3] = y1 * x0; A[i][4] = y1 * y0; A[i][5] = y1;
      A[i][6] = x0; A[i][7] = y0; A[i][8] = 1;
    }
    return models_from_rows7(A, true, out);
  }

  // The models of a 7 x 9 epipolar system: its two-dimensional null space (LU
  // kernel), the cubic det(l f1 + (1 - l) f2) = 0, each real root's matrix
  // normalised to F33 = 1 (up to three). `guards`: the seven-point solver's
  // checks of the cubic's coefficients (solver_fundamental_matrix_seven_point.h:240-251).
  __device__ static int models_from_rows7(double A[7][9], bool guards, double* out) {
    double f1[9], f2[9];
    if (lu_kernel_7x9(A, f1, f2) != 2) return 0;
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
    const double eps = 2.220446049250313e-16;
    if (guards && (fabs(c[0] + c[1] + c[2] + c[3]) < 1e-9 || fabs(c[0]) < eps || fabs(c[1]) < eps ||
                   fabs(c[2]) < eps || fabs(c[3]) < eps))
      return 0;
    if (!(c[3] != 0.0)) return 0;  // no cubic (the polynomial solver needs a leading coefficient)
    double roots[3];
    const int nr = cubic_real_roots(c, roots);
    int nm = 0;
    for (int k = 0; k < nr; ++k) {
      double lambda = roots[k], mu = 1.;
      const double s = f1[8] * roots[k] + f2[8];
      if (fabs(s) > eps) {
        mu = 1.0 / s;
        lambda *= mu;
        double* F = out + 9 * nm;
        for (int i = 0; i < 8; ++i) F[i] = f1[i] * lambda + f2[i] * mu;
        F[8] = 1.0;
        ++nm;
      }
    }
    return nm;
  }

  __device__ static int minimal(const double* pts, const int* s, double* out, const double* = nullptr) {
    const double* rows[7];
    for (int i = 0; i < 7; ++i) rows[i] = pts + 4 * s[i];
    double tmp[27];
    const int n = seven_point(rows, tmp);
    int k = 0;
    for (int q = 0; q < n; ++q)
      if (orientation_valid(tmp + 9 * q, pts, s, 7)) {
        for (int i = 0; i < 9; ++i) out[9 * k + i] = tmp[9 * q + i];
        ++k;
      }
    return k;
  }

  __device__ __forceinline__ static double r2_f64(const double* p, const double* F) {
    const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
    const double rxc = F[0] * x2 + F[3] * y2 + F[6];
    const double ryc = F[1] * x2 + F[4] * y2 + F[7];
    const double rwc = F[2] * x2 + F[5] * y2 + F[8];
    const double r = x1 * rxc + y1 * ryc + rwc;
    const double rx = F[0] * x1 + F[1] * y1 + F[2];
    const double ry = F[3] * x1 + F[4] * y1 + F[5];
    return r * r / (rxc * rxc + ryc * ryc + rx * rx + ry * ry);
  }

  __device__ __forceinline__ static double symepi2_f64(const double* p, const double* F) {
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

  // FP32 Sampson distance on centred coordinates; `it` = 1/sqrt(denominator)
  // for the error bound.
  __device__ __forceinline__ static float r2_f32(const float4 p, const float* F, float& it) {
    const float rxc = fmaf(F[0], p.z, fmaf(F[3], p.w, F[6]));
    const float ryc = fmaf(F[1], p.z, fmaf(F[4], p.w, F[7]));
    const float rwc = fmaf(F[2], p.z, fmaf(F[5], p.w, F[8]));
    const float r = fmaf(p.x, rxc, fmaf(p.y, ryc, rwc));
    const float rx = fmaf(F[0], p.x, fmaf(F[1], p.y, F[2]));
    const float ry = fmaf(F[3], p.x, fmaf(F[4], p.y, F[5]));
    const float den = fmaf(rxc, rxc, fmaf(ryc, ryc, fmaf(rx, rx, ry * ry)));
    it = rsqrtf(den);
    const float rn = r * it;
    return rn * rn;
  }

  // F' = T(c2)^T F T(c1) acts on centred coordinates with the same Sampson
  // distance; scaled to unit max entry. out[9]: error scale of the epipolar
  // term (8 eps times the absolute sum of its terms), so that the FP32
  // distance differs from the FP64 one by at most out[9] * (it + 1) + 1e-5 r.
  __device__ static void prepare_f32(const double* F, const double* c, double S, float* out) {
    double g[9];
    // F T(c1): column 2 += c1x col0 + c1y col1
    for (int r = 0; r < 3; ++r) {
      g[3 * r + 0] = F[3 * r + 0];
      g[3 * r + 1] = F[3 * r + 1];
      g[3 * r + 2] = F[3 * r + 0] * c[0] + F[3 * r + 1] * c[1] + F[3 * r + 2];
    }
    // T(c2)^T (.): row 2 += c2x row0 + c2y row1
    for (int k = 0; k < 3; ++k) g[6 + k] += c[2] * g[k] + c[3] * g[3 + k];
    double mx = 0;
    for (int k = 0; k < 9; ++k) mx = fmax(mx, fabs(g[k]));
    const double s = mx > 0 ? 1.0 / mx : 1.0;
    for (int k = 0; k < 9; ++k) g[k] *= s;
    for (int k = 0; k < 9; ++k) out[k] = (float)g[k];
    const double Sx = fmax(S, 1.0);
    double kC = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) kC += fabs(g[3 * i + j]) * (i < 2 ? Sx : 1.0) * (j < 2 ? Sx : 1.0);
    const double cm = 8.0 * 5.9604644775390625e-08 * kC;
    out[9] = isfinite(cm) ? (float)cm : 3.0e38f;
    out[10] = 0.f;
    out[11] = 0.f;
  }

  // Degeneracy test of DEGENSAC (applyDegensac, fundamental_estimator.h:357-459):
  // the homographies implied by F and five triplets of the sample; returns
  // true and the first homography that 5 of the 7 points fit within 2 px.
  __device__ static bool degenerate_sample(const double* F, const double* pts, const int* s, double* H_out) {
    // left epipole (null vector of F^T, the last left singular vector)
    const double c0[3] = {F[0], F[3], F[6]}, c1[3] = {F[1], F[4], F[7]}, c2[3] = {F[2], F[5], F[8]};
    double e01[3], e02[3], e12[3];
    dcross3(c0, c1, e01);
    dcross3(c0, c2, e02);
    dcross3(c1, c2, e12);
    const double n01 = e01[0] * e01[0] + e01[1] * e01[1] + e01[2] * e01[2];
    const double n02 = e02[0] * e02[0] + e02[1] * e02[1] + e02[2] * e02[2];
    const double n12 = e12[0] * e12[0] + e12[1] * e12[1] + e12[2] * e12[2];
    const double* eb = n01 >= n02 ? (n01 >= n12 ? e01 : e12) : (n02 >= n12 ? e02 : e12);
    const double ep[3] = {eb[0] / eb[2], eb[1] / eb[2], 1.0};
    const double ex[9] = {0, -ep[2], ep[1], ep[2], 0, -ep[0], -ep[1], ep[0], 0};
    double A[9];
    matmul3(ex, F, A);
    const int trip[15] = {0, 1, 2, 3, 4, 5, 0, 1, 6, 3, 4, 6, 2, 5, 6};
    for (int t = 0; t < 5; ++t) {
      const int i1 = s[trip[3 * t]], i2 = s[trip[3 * t + 1]], i3 = s[trip[3 * t + 2]];
      const double* P[3] = {pts + 4 * i1, pts + 4 * i2, pts + 4 * i3};
      double b[3], M[9];
      for (int k = 0; k < 3; ++k) {
        const double x1[3] = {P[k][0], P[k][1], 1}, x2[3] = {P[k][2], P[k][3], 1};
        double pe[3], Ax[3], cc[3];
        dcross3(x2, ep, pe);
        for (int r = 0; r < 3; ++r) Ax[r] = A[r * 3] * x1[0] + A[r * 3 + 1] * x1[1] + A[r * 3 + 2] * x1[2];
        dcross3(x2, Ax, cc);
        b[k] = (cc[0] * pe[0] + cc[1] * pe[1] + cc[2] * pe[2]) / (pe[0] * pe[0] + pe[1] * pe[1] + pe[2] * pe[2]);
        M[k * 3] = x1[0]; M[k * 3 + 1] = x1[1]; M[k * 3 + 2] = x1[2];
      }
      double Mi[9];
      inverse3(M, Mi);
      double mb[3];
      for (int r = 0; r < 3; ++r) mb[r] = Mi[r * 3] * b[0] + Mi[r * 3 + 1] * b[1] + Mi[r * 3 + 2] * b[2];
      double H[9];
      for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) H[r * 3 + q] = A[r * 3 + q] - ep[r] * mb[q];
      int cnt = 3;
      for (int i = 0; i < 7; ++i) {
        const int idx = s[i];
        if (idx == i1 || idx == i2 || idx == i3) continue;
        if (HomographyModel::r2_f64(pts + 4 * idx, H) < 4.0) ++cnt;
      }
      if (cnt >= 5) {
        for (int k = 0; k < 9; ++k) H_out[k] = H[k];
        return true;
      }
    }
    return false;
  }

  // ---------------------------------------------------------------------------
  // Non-minimal solver: Hartley normalisation, 8-point start, LM refinement,
  // denormalisation F = Td^T F Ts, unit Frobenius norm, F33 >= 0.
  using Norm = HomographyModel::Norm;

  // packed lower triangle (45) of A^T A plus nothing else: the 8-point system
  __device__ __forceinline__ static void design_row(const Norm& N, const double* p, double w, double* r) {
    const double x0 = (p[0] - N.ms0) * N.rs, y0 = (p[1] - N.ms1) * N.rs;
    const double x1 = (p[2] - N.md0) * N.rd, y1 = (p[3] - N.md1) * N.rd;
    const double wx0 = w * x0, wy0 = w * y0, wx1 = w * x1, wy1 = w * y1;
    r[0] = wx1 * x0; r[1] = wx1 * y0; r[2] = wx1;
    r[3] = wy1 * x0; r[4] = wy1 * y0; r[5] = wy1;
    r[6] = wx0; r[7] = wy0; r[8] = w;
  }
  static constexpr int NATA = 45;
  __device__ __forceinline__ static void accumulate_ata(const Norm& N, const double* p, double w, double* acc) {
    double r[9];
    design_row(N, p, w, r);
    int k = 0;
#pragma unroll
    for (int a = 0; a < 9; ++a)
#pragma unroll
      for (int b = 0; b <= a; ++b) acc[k++] += r[a] * r[b];
  }
  __device__ static void eight_point_from_ata(const double* acc, double* F) {
    double M[81];
    int k = 0;
    for (int a = 0; a < 9; ++a)
      for (int b = 0; b <= a; ++b) {
        M[a * 9 + b] = acc[k];
        M[b * 9 + a] = acc[k];
        ++k;
      }
    fullpiv_qr_lastcol9(M, F);
  }

  // FactorizedFundamentalMatrix: F = u0 v0^T + sigma u1 v1^T
  struct FactF {
    double U[9], V[9], sigma;
  };
  __device__ static void factf_from(const double* F, FactF& f) {
    double s[3];
    svd3(F, f.U, s, f.V);
    f.sigma = s[1] / s[0];
  }
  __device__ static void factf_F(const FactF& f, double* F) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) F[i * 3 + j] = f.U[i * 3] * f.V[j * 3] + f.sigma * f.U[i * 3 + 1] * f.V[j * 3 + 1];
  }

  // truncated Sampson cost of one normalised correspondence (loss scale 1)
  __device__ __forceinline__ static double lm_cost_point(const double* F, double p0, double p1, double q0, double q1) {
    const double Fx0 = F[0] * p0 + F[1] * p1 + F[2], Fx1 = F[3] * p0 + F[4] * p1 + F[5],
                 Fx2 = F[6] * p0 + F[7] * p1 + F[8];
    const double C = q0 * Fx0 + q1 * Fx1 + Fx2;
    const double a0 = F[0] * q0 + F[3] * q1 + F[6], a1 = F[1] * q0 + F[4] * q1 + F[7];
    const double r2 = C * C / (Fx0 * Fx0 + Fx1 * Fx1 + a0 * a0 + a1 * a1);
    return r2 < 1.0 ? r2 : 1.0;
  }

  // d F / d (rotation of U, rotation of V, sigma) in the column-major order of
  // the entries of F (jacobian_impl.h:541-550)
  __device__ static void lm_dparams(const FactF& f, const double* F, double D[9][7]) {
    double ds[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) ds[i * 3 + j] = f.U[i * 3 + 1] * f.V[j * 3 + 1];
    const double v[9][7] = {{0, F[6], -F[3], 0, F[2], -F[1], ds[0]},
                            {-F[6], 0, F[0], 0, F[5], -F[4], ds[3]},
                            {F[3], -F[0], 0, 0, F[8], -F[7], ds[6]},
                            {0, F[7], -F[4], -F[2], 0, F[0], ds[1]},
                            {-F[7], 0, F[1], -F[5], 0, F[3], ds[4]},
                            {F[4], -F[1], 0, -F[8], 0, F[6], ds[7]},
                            {0, F[8], -F[5], F[1], -F[0], 0, ds[2]},
                            {-F[8], 0, F[2], F[4], -F[3], 0, ds[5]},
                            {F[5], -F[2], 0, F[7], -F[6], 0, ds[8]}};
    for (int r = 0; r < 9; ++r)
      for (int c = 0; c < 7; ++c) D[r][c] = v[r][c];
  }

  // J^T J (lower, 28) and J^T r (7) contribution of one correspondence with
  // row weight w (FundamentalJacobianAccumulator::accumulate)
  static constexpr int NLM = 35;
  __device__ __forceinline__ static void lm_accumulate_point(const double* F, const double D[9][7], double p0,
                                                             double p1, double q0, double q1, double w, int n,
                                                             double* acc) {
    const double Fx0 = F[0] * p0 + F[1] * p1 + F[2], Fx1 = F[3] * p0 + F[4] * p1 + F[5],
                 Fx2 = F[6] * p0 + F[7] * p1 + F[8];
    const double C = q0 * Fx0 + q1 * Fx1 + Fx2;
    const double J0 = F[0] * q0 + F[3] * q1 + F[6], J1 = F[1] * q0 + F[4] * q1 + F[7];
    const double J2 = Fx0, J3 = Fx1;
    const double nJ = sqrt(J0 * J0 + J1 * J1 + J2 * J2 + J3 * J3);
    const double inv = 1.0 / nJ;
    const double r = C * inv;
    double weight = ((r * r) < 1.0 ? 1.0 : 0.0) / n;
    weight = w * weight;
    if (weight == 0.0) return;
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
#pragma unroll
    for (int k = 0; k < 9; ++k) dF[k] *= inv;
    double J[7];
#pragma unroll
    for (int c = 0; c < 7; ++c) {
      double t = 0;
#pragma unroll
      for (int rr = 0; rr < 9; ++rr) t += dF[rr] * D[rr][c];
      J[c] = t;
    }
    int k = 0;
#pragma unroll
    for (int a = 0; a < 7; ++a) {
#pragma unroll
      for (int b = 0; b <= a; ++b) acc[k++] += weight * (J[a] * J[b]);
    }
#pragma unroll
    for (int a = 0; a < 7; ++a) acc[28 + a] += weight * C * inv * J[a];
  }

  // lm_accumulate_point with J = dF^T D formed from the structure of D
  // (lm_dparams): the six rotation columns hold signed entries of F, the
  // sigma column the products ds = U[:,1] V[:,1]^T; the nonzero terms are
  // summed in row order like the dense product. kDcode[r][c] = +-(k + 1)
  // for the entry +-F[k], 0 for a structural zero.
  __device__ __forceinline__ static void lm_accumulate_point_s(const double* F, const double* ds, double p0,
                                                               double p1, double q0, double q1, int n, double* acc) {
    constexpr signed char kDcode[9][6] = {{0, 7, -4, 0, 3, -2}, {-7, 0, 1, 0, 6, -5}, {4, -1, 0, 0, 9, -8},
                                          {0, 8, -5, -3, 0, 1},  {-8, 0, 2, -6, 0, 4}, {5, -2, 0, -9, 0, 7},
                                          {0, 9, -6, 2, -1, 0},  {-9, 0, 3, 5, -4, 0}, {6, -3, 0, 8, -7, 0}};
    constexpr int kDs[9] = {0, 3, 6, 1, 4, 7, 2, 5, 8};
    const double Fx0 = F[0] * p0 + F[1] * p1 + F[2], Fx1 = F[3] * p0 + F[4] * p1 + F[5],
                 Fx2 = F[6] * p0 + F[7] * p1 + F[8];
    const double C = q0 * Fx0 + q1 * Fx1 + Fx2;
    const double J0 = F[0] * q0 + F[3] * q1 + F[6], J1 = F[1] * q0 + F[4] * q1 + F[7];
    const double J2 = Fx0, J3 = Fx1;
    const double nJ = sqrt(J0 * J0 + J1 * J1 + J2 * J2 + J3 * J3);
    const double inv = 1.0 / nJ;
    const double r = C * inv;
    if (!((r * r) < 1.0)) return;
    const double weight = 1.0 / n;
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
#pragma unroll
    for (int k = 0; k < 9; ++k) dF[k] *= inv;
    double J[7];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      double t = 0;
#pragma unroll
      for (int rr = 0; rr < 9; ++rr) {
        const int code = kDcode[rr][c];
        if (code > 0) t += dF[rr] * F[code - 1];
        if (code < 0) t += dF[rr] * (-F[-code - 1]);
      }
      J[c] = t;
    }
    {
      double t = 0;
#pragma unroll
      for (int rr = 0; rr < 9; ++rr) t += dF[rr] * ds[kDs[rr]];
      J[6] = t;
    }
    int k = 0;
#pragma unroll
    for (int a = 0; a < 7; ++a) {
#pragma unroll
      for (int b = 0; b <= a; ++b) acc[k++] += weight * (J[a] * J[b]);
    }
#pragma unroll
    for (int a = 0; a < 7; ++a) acc[28 + a] += weight * C * inv * J[a];
  }

  // one LM step from the accumulated system: sol = -(JtJ + lambda I)^-1 Jtr,
  // then the rotated factorisation (bundle.cpp:285-320). Returns false when
  // the step is below the tolerance.
  __device__ static bool lm_step(const double* acc, double lambda, const FactF& f, FactF& fn) {
    double A[7][7], x[7];
    int k = 0;
#pragma unroll
    for (int a = 0; a < 7; ++a)
#pragma unroll
      for (int b = 0; b <= a; ++b) {
        A[a][b] = acc[k];
        A[b][a] = acc[k];
        ++k;
      }
#pragma unroll
    for (int a = 0; a < 7; ++a) {
      A[a][a] += lambda;
      x[a] = -acc[28 + a];
    }
    if (!cholesky_solve<7>(A, x))
      for (int a = 0; a < 7; ++a) x[a] = 0;
    double sn = 0;
    for (int a = 0; a < 7; ++a) sn += x[a] * x[a];
    if (sqrt(sn) < 1e-8) return false;
    double w1[3] = {x[0], x[1], x[2]}, w2[3] = {x[3], x[4], x[5]};
    const double th1 = sqrt(w1[0] * w1[0] + w1[1] * w1[1] + w1[2] * w1[2]);
    const double th2 = sqrt(w2[0] * w2[0] + w2[1] * w2[1] + w2[2] * w2[2]);
    for (int i = 0; i < 3; ++i) {
      w1[i] /= th1;
      w2[i] /= th2;
    }
    auto rot = [](const double* w, double th, const double* M, double* out) {
      const double a = sin(th), b = cos(th);
      const double S[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
      double S2[9], R[9];
      matmul3(S, S, S2);
      for (int i = 0; i < 9; ++i) R[i] = a * S[i] + (1 - b) * S2[i];
      double RM[9];
      matmul3(R, M, RM);
      for (int i = 0; i < 9; ++i) out[i] = M[i] + RM[i];
    };
    rot(w1, th1, f.U, fn.U);
    rot(w2, th2, f.V, fn.V);
    fn.sigma = f.sigma + x[6];
    return true;
  }

  __device__ static void denormalise(const Norm& N, const double* Fn, double* out) {
    const double Ts[9] = {N.rs, 0, -N.rs * N.ms0, 0, N.rs, -N.rs * N.ms1, 0, 0, 1};
    const double TdT[9] = {N.rd, 0, 0, 0, N.rd, 0, -N.rd * N.md0, -N.rd * N.md1, 1};
    double t[9], G[9];
    matmul3(TdT, Fn, t);
    matmul3(t, Ts, G);
    double nrm = 0;
    for (int i = 0; i < 9; ++i) nrm += G[i] * G[i];
    nrm = sqrt(nrm);
    const double sgn = (G[8] / nrm) < 0 ? -1.0 : 1.0;
    for (int i = 0; i < 9; ++i) out[i] = sgn * (G[i] / nrm);
  }

  // The same fit by a group of four lanes of one warp (lane q of the group
  // takes rows q, q + 4, ...; `mask` selects the group's lanes): every sum
  // over the rows is formed per lane and combined by two butterfly steps,
  // ((s0 + s1) + (s2 + s3)) in every lane, and the small solves run in all
  // four lanes in lockstep. The rows' work per lane is a quarter of the
  // one-thread fit, which shortens the dependent chain of each LM iteration.
  __device__ static double sum4(double v, unsigned mask) {
    v += __shfl_xor_sync(mask, v, 1);
    v += __shfl_xor_sync(mask, v, 2);
    return v;
  }
  __device__ static bool fit_group(const double* pts, const int* idx, int n, double* out, int q, unsigned mask) {
    if (n < 8) return false;
    Norm N;
    {
      double a = 0, b = 0, c = 0, d = 0;
      for (int i = q; i < n; i += 4) {
        const double* p = pts + 4 * idx[i];
        a += p[0]; b += p[1]; c += p[2]; d += p[3];
      }
      a = sum4(a, mask); b = sum4(b, mask); c = sum4(c, mask); d = sum4(d, mask);
      N.ms0 = a / n; N.ms1 = b / n; N.md0 = c / n; N.md1 = d / n;
      double ads = 0, add = 0;
      for (int i = q; i < n; i += 4) {
        const double* p = pts + 4 * idx[i];
        const double dx1 = N.ms0 - p[0], dy1 = N.ms1 - p[1], dx2 = N.md0 - p[2], dy2 = N.md1 - p[3];
        ads += sqrt(dx1 * dx1 + dy1 * dy1);
        add += sqrt(dx2 * dx2 + dy2 * dy2);
      }
      ads = sum4(ads, mask);
      add = sum4(add, mask);
      N.rs = M_SQRT2 / (ads / n);
      N.rd = M_SQRT2 / (add / n);
    }
    double F[9];
    {
      double ata[NATA];
#pragma unroll
      for (int k = 0; k < NATA; ++k) ata[k] = 0;
      for (int i = q; i < n; i += 4) accumulate_ata(N, pts + 4 * idx[i], 1.0, ata);
#pragma unroll
      for (int k = 0; k < NATA; ++k) ata[k] = sum4(ata[k], mask);
      eight_point_from_ata(ata, F);
    }
    FactF f;
    factf_from(F, f);
    auto cost_of = [&](const double* G) {
      double c = 0;
      for (int i = q; i < n; i += 4) {
        const double* p = pts + 4 * idx[i];
        c += lm_cost_point(G, (p[0] - N.ms0) * N.rs, (p[1] - N.ms1) * N.rs, (p[2] - N.md0) * N.rd,
                           (p[3] - N.md1) * N.rd);
      }
      return sum4(c, mask);
    };
    double G[9];
    factf_F(f, G);
    double lambda = 1e-3;
    double cost = cost_of(G);
    bool recompute = true;
    double acc[NLM];
    for (int iter = 0; iter < 25; ++iter) {
      if (recompute) {
#pragma unroll
        for (int k = 0; k < NLM; ++k) acc[k] = 0;
        double ds[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) ds[i * 3 + j] = f.U[i * 3 + 1] * f.V[j * 3 + 1];
        for (int i = q; i < n; i += 4) {
          const double* p = pts + 4 * idx[i];
          lm_accumulate_point_s(G, ds, (p[0] - N.ms0) * N.rs, (p[1] - N.ms1) * N.rs, (p[2] - N.md0) * N.rd,
                                (p[3] - N.md1) * N.rd, n, acc);
        }
#pragma unroll
        for (int k = 0; k < NLM; ++k) acc[k] = sum4(acc[k], mask);
        double gn = 0;
#pragma unroll
        for (int a = 0; a < 7; ++a) gn += acc[28 + a] * acc[28 + a];
        if (sqrt(gn) < 1e-8) break;
      }
      FactF fn;
      if (!lm_step(acc, lambda, f, fn)) break;
      double Gn[9];
      factf_F(fn, Gn);
      const double cn = cost_of(Gn);
      if (cn < cost) {
        f = fn;
#pragma unroll
        for (int k = 0; k < 9; ++k) G[k] = Gn[k];
        lambda /= 10;
        cost = cn;
        recompute = true;
      } else {
        lambda *= 10;
        recompute = false;
      }
    }
    if (q == 0) denormalise(N, G, out);
    return true;
  }

  // Per-thread non-minimal fit with unit weights (the local-optimisation
  // trials run one per thread): normalisation, 8-point start, 25 LM
  // iterations on the factorised F, denormalisation. The model of the
  // current factorisation and its cost are carried between iterations; the
  // Jacobian uses the structure of dF/dparams instead of a dense 9x7 matrix.
  __device__ static bool fit_thread(const double* pts, const int* idx, int n, double* out) {
    if (n < 8) return false;  // the 7-row case cannot occur in the loop (see the engine)
    Norm N;
    HomographyModel::normalise(pts, idx, n, N);
    double F[9];
    {
      double ata[NATA];
#pragma unroll
      for (int k = 0; k < NATA; ++k) ata[k] = 0;
      for (int i = 0; i < n; ++i) accumulate_ata(N, pts + 4 * idx[i], 1.0, ata);
      eight_point_from_ata(ata, F);
    }
    FactF f;
    factf_from(F, f);
    auto cost_of = [&](const double* G) {
      double c = 0;
      for (int i = 0; i < n; ++i) {
        const double* p = pts + 4 * idx[i];
        c += lm_cost_point(G, (p[0] - N.ms0) * N.rs, (p[1] - N.ms1) * N.rs, (p[2] - N.md0) * N.rd,
                           (p[3] - N.md1) * N.rd);
      }
      return c;
    };
    double G[9];
    factf_F(f, G);
    double lambda = 1e-3;
    double cost = cost_of(G);
    bool recompute = true;
    double acc[NLM];
    for (int iter = 0; iter < 25; ++iter) {
      if (recompute) {
#pragma unroll
        for (int k = 0; k < NLM; ++k) acc[k] = 0;
        double ds[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) ds[i * 3 + j] = f.U[i * 3 + 1] * f.V[j * 3 + 1];
        for (int i = 0; i < n; ++i) {
          const double* p = pts + 4 * idx[i];
          lm_accumulate_point_s(G, ds, (p[0] - N.ms0) * N.rs, (p[1] - N.ms1) * N.rs, (p[2] - N.md0) * N.rd,
                                (p[3] - N.md1) * N.rd, n, acc);
        }
        double gn = 0;
#pragma unroll
        for (int a = 0; a < 7; ++a) gn += acc[28 + a] * acc[28 + a];
        if (sqrt(gn) < 1e-8) break;
      }
      FactF fn;
      if (!lm_step(acc, lambda, f, fn)) break;
      double Gn[9];
      factf_F(fn, Gn);
      const double cn = cost_of(Gn);
      if (cn < cost) {
        f = fn;
#pragma unroll
        for (int k = 0; k < 9; ++k) G[k] = Gn[k];
        lambda /= 10;
        cost = cn;
        recompute = true;
      } else {
        lambda *= 10;
        recompute = false;
      }
    }
    denormalise(N, G, out);
    return true;
  }
};

// The estimator of DEGENSAC's inner run: FundamentalMatrixEstimator with the
// plane-and-parallax minimal solver (2 points and a fixed homography,
// solver_fundamental_matrix_plane_and_parallax.h:102-165), the 8-point
// non-minimal solver, validity ratio 0 and no DEGENSAC
// (fundamental_estimator.h:519-553).
struct PlaneParallaxModel {
  static constexpr int KIND = 2;
  static constexpr int M = 2;
  static constexpr int MAXSOL = 1;
  static constexpr int LO_MAXSOL = 1;
  static constexpr int NONMIN = 8;
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;
  static constexpr bool AFFINE = false;
  static constexpr bool CTA_VALIDITY = true;
  using Norm = HomographyModel::Norm;

  __device__ static bool valid_sample(const double*, const int*) { return true; }

  __device__ static int minimal(const double* pts, const int* s, double* out, const double* H) {
    const double* p1 = pts + 4 * s[0];
    const double* p2 = pts + 4 * s[1];
    double q1[3], q2[3];
    for (int i = 0; i < 3; ++i) {
      q1[i] = H[i * 3] * p1[0] + H[i * 3 + 1] * p1[1] + H[i * 3 + 2];
      q2[i] = H[i * 3] * p2[0] + H[i * 3 + 1] * p2[1] + H[i * 3 + 2];
    }
    const double d1[3] = {p1[2], p1[3], 1}, d2[3] = {p2[2], p2[3], 1};
    double l1[3], l2[3], e[3];
    dcross3(q1, d1, l1);
    dcross3(q2, d2, l2);
    dcross3(l1, l2, e);
    if (fabs(e[2]) < 2.220446049250313e-16) return 0;
    const double ex[9] = {0, -e[2], e[1], e[2], 0, -e[0], -e[1], e[0], 0};
    double F[9];
    matmul3(ex, H, F);
    if (!FundamentalModel::orientation_valid(F, pts, s, 2)) return 0;
    for (int i = 0; i < 9; ++i) out[i] = F[i];
    return 1;
  }

  __device__ __forceinline__ static double r2_f64(const double* p, const double* F) {
    return FundamentalModel::r2_f64(p, F);
  }
  __device__ __forceinline__ static float r2_f32(const float4 p, const float* F, float& it) {
    return FundamentalModel::r2_f32(p, F, it);
  }
  __device__ static void prepare_f32(const double* F, const double* c, double S, float* out) {
    FundamentalModel::prepare_f32(F, c, S, out);
  }

  // normalised 8-point fit, unit weights, one thread
  __device__ static bool fit_thread(const double* pts, const int* idx, int n, double* out) {
    if (n < NONMIN) return false;
    Norm N;
    HomographyModel::normalise(pts, idx, n, N);
    double ata[FundamentalModel::NATA];
#pragma unroll
    for (int k = 0; k < FundamentalModel::NATA; ++k) ata[k] = 0;
    for (int i = 0; i < n; ++i) FundamentalModel::accumulate_ata(N, pts + 4 * idx[i], 1.0, ata);
    double F[9];
    FundamentalModel::eight_point_from_ata(ata, F);
    FundamentalModel::denormalise(N, F, out);
    return true;
  }
};

// Affine-correspondence fundamental matrix (findFundamentalMatrixAC_,
// gcransac_python.cpp:1924-2221; FundamentalMatrixEstimator with
// FundamentalMatrixThreeAffineSolver, solver_fundamental_matrix_three_affine.h:84-250).
// Three correspondences per minimal sample, whose local affine maps
// (a11, a12, a21, a22) sit in the engine's aux array: the epipolar row of
// each and the two affine rows of the first two make a 7 x 9 system, solved
// like the seven-point one (LU kernel, cubic; the reference takes the null
// space from an SVD of A^T A, another basis of the same plane, and applies no
// coefficient checks). No DEGENSAC (the estimator runs it for samples of 7 or
// more), the plain normalised 8-point solver as the non-minimal solver (local
// optimisation, iteratively reweighted fits, final fit; no
// Levenberg-Marquardt), an inner sample of 7 x 3 in the local optimisation,
// and a driver bundle adjustment without weights.
struct FundamentalAffineModel : FundamentalModel {
  static constexpr int M = 3;
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;
  static constexpr bool AFFINE = true;
  static constexpr bool DEGENSAC = false;
  static constexpr bool EPILOGUE_WEIGHTED = false;
  static constexpr bool NONMIN_LM = false;  // FundamentalMatrixEightPointSolver (types.h:83-86)
  static constexpr int NONMIN = 8;

  __device__ static bool valid_sample_affine(const double*, const double*, const int*) { return true; }

  // Non-minimal fit of the local optimisation's trials, one per thread: the
  // normalised 8-point solver (solver_fundamental_matrix_eight_point.h:93-182)
  // with unit weights, denormalised.
  __device__ static bool fit_thread(const double* pts, const int* idx, int n, double* out) {
    if (n < NONMIN) return false;
    Norm N;
    HomographyModel::normalise(pts, idx, n, N);
    double ata[NATA];
#pragma unroll
    for (int k = 0; k < NATA; ++k) ata[k] = 0;
    for (int i = 0; i < n; ++i) accumulate_ata(N, pts + 4 * idx[i], 1.0, ata);
    double F[9];
    eight_point_from_ata(ata, F);
    denormalise(N, F, out);
    return true;
  }

  __device__ static int minimal_affine(const double* pts, const double* aff, const int* s, double* out) {
    double A[7][9];
    int r = 0;
    for (int i = 0; i < 3; ++i) {
      const double* p = pts + 4 * s[i];
      const double x0 = p[0], y0 = p[1], x1 = p[2], y1 = p[3];
      A[r][0] = x1 * x0; A[r][1] = x1 * y0; A[r][2] = x1;
      A[r][3] = y1 * x0; A[r][4] = y1 * y0; A[r][5] = y1;
      A[r][6] = x0; A[r][7] = y0; A[r][8] = 1.0;
      ++r;
      if (i < 2) {
        const double* m = aff + 4 * s[i];
        const double a11 = m[0], a12 = m[1], a21 = m[2], a22 = m[3];
        A[r][0] = x1 + a11 * x0; A[r][1] = a11 * y0; A[r][2] = a11;
        A[r][3] = y1 + a21 * x0; A[r][4] = a21 * y0; A[r][5] = a21;
        A[r][6] = 1.0; A[r][7] = 0.0; A[r][8] = 0.0;
        ++r;
        A[r][0] = a12 * x0; A[r][1] = x1 + a12 * y0; A[r][2] = a12;
        A[r][3] = a22 * x0; A[r][4] = y1 + a22 * y0; A[r][5] = a22;
        A[r][6] = 0.0; A[r][7] = 1.0; A[r][8] = 0.0;
        ++r;
      }
    }
    double tmp[27];
    const int n = models_from_rows7(A, false, tmp);
    // the estimator keeps the models that pass the oriented epipolar
    // constraint on the sample (fundamental_estimator.h:161-184)
    int k = 0;
    for (int q = 0; q < n; ++q)
      if (orientation_valid(tmp + 9 * q, pts, s, 3)) {
        for (int i = 0; i < 9; ++i) out[9 * k + i] = tmp[9 * q + i];
        ++k;
      }
    return k;
  }
};

// SIFT-correspondence fundamental matrix (findFundamentalMatrixSIFT_,
// gcransac_python.cpp:2222-2518; FundamentalMatrixEstimator with
// FundamentalMatrixFourSIFTSolver, solver_fundamental_matrix_four_sift.h:89-250):
// the aux array holds each correspondence's feature scales and orientations
// (q1, q2, o1, o2); four correspondences per minimal sample, the epipolar
// row of each and the orientation-scale row of the first three. Everything
// else as the affine-correspondence kind (the reference's two drivers differ
// only in the estimator), with an inner sample of 7 x 4.
struct FundamentalSiftModel : FundamentalAffineModel {
  static constexpr int M = 4;
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;

  __device__ static int minimal_affine(const double* pts, const double* aux, const int* s, double* out) {
    double A[7][9];
    int r = 0;
    for (int i = 0; i < 4; ++i) {
      const double* p = pts + 4 * s[i];
      const double u1 = p[0], v1 = p[1], u2 = p[2], v2 = p[3];
      A[r][0] = u2 * u1; A[r][1] = u2 * v1; A[r][2] = u2;
      A[r][3] = v2 * u1; A[r][4] = v2 * v1; A[r][5] = v2;
      A[r][6] = u1; A[r][7] = v1; A[r][8] = 1.0;
      ++r;
      if (i == 3) break;
      const double* f = aux + 4 * s[i];
      const double q1 = f[0], q2 = f[1], o1 = f[2], o2 = f[3];
      double s1, c1, s2, c2;
      sincos(o1, &s1, &c1);
      sincos(o2, &s2, &c2);
      A[r][0] = s2 * s2 * q2 * u1 - c1 * c2 * q1 * u2 - q2 * u1;
      A[r][1] = s2 * s2 * q2 * v1 - s1 * c2 * q1 * u2 - q2 * v1;
      A[r][2] = s2 * s2 * q2 - q2;
      A[r][3] = -c2 * s2 * q2 * u1 - c1 * c2 * q1 * v2;
      A[r][4] = -c2 * s2 * q2 * v1 - s1 * c2 * q1 * v2;
      A[r][5] = -c2 * s2 * q2;
      A[r][6] = -c1 * c2 * q1;
      A[r][7] = -s1 * c2 * q1;
      A[r][8] = 0.0;
      ++r;
    }
    double tmp[27];
    const int n = models_from_rows7(A, false, tmp);
    int k = 0;
    for (int q = 0; q < n; ++q)
      if (orientation_valid(tmp + 9 * q, pts, s, 4)) {
        for (int i = 0; i < 9; ++i) out[9 * k + i] = tmp[9 * q + i];
        ++k;
      }
    return k;
  }
};

}  // namespace gcr
