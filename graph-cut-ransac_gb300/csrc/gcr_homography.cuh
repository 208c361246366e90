// Homography model on the device: sample check, 4-point minimal solver,
// residuals and the normalised weighted least-squares fit.
//
// Behaviour follows src/pygcransac/include/estimators/homography_estimator.h
// (isValidSample 346-381, squaredResidual 181-199, isValidModel 326-342,
// normalizePoints 213-310) and solver_homography_four_point.h (minimal
// 109-190, non-minimal 192-264) of the reference.
#pragma once

#include "gcr_device.cuh"
#include "gcr_linalg.cuh"

namespace gcr {

struct HomographyModel {
  static constexpr int KIND = 0;
  static constexpr bool CTA_VALIDITY = false;
  static constexpr int M = 4;          // minimal sample size
  static constexpr int MAXSOL = 1;     // models per minimal sample
  static constexpr int LO_MAXSOL = 1;  // models per non-minimal fit
  static constexpr int NONMIN = 4;     // smallest non-minimal sample
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr bool WEIGHTED = true;
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;
  static constexpr bool AFFINE = false;  // minimal samples need no local affine maps

  // orientation test: the four points keep the same side of the lines through
  // two of them in both images
  __device__ static bool valid_sample(const double* pts, const int* s) {
    const double *a = pts + 4 * s[0], *b = pts + 4 * s[1], *c = pts + 4 * s[2], *d = pts + 4 * s[3];
    double p[3], q[3];
    auto cross = [](double r[3], const double* u, const double* v) {
      r[0] = u[1] - v[1];
      r[1] = v[0] - u[0];
      r[2] = u[0] * v[1] - u[1] * v[0];
    };
    cross(p, a, b);
    cross(q, a + 2, b + 2);
    if ((p[0] * c[0] + p[1] * c[1] + p[2]) * (q[0] * c[2] + q[1] * c[3] + q[2]) < 0) return false;
    if ((p[0] * d[0] + p[1] * d[1] + p[2]) * (q[0] * d[2] + q[1] * d[3] + q[2]) < 0) return false;
    cross(p, c, d);
    cross(q, c + 2, d + 2);
    if ((p[0] * a[0] + p[1] * a[1] + p[2]) * (q[0] * a[2] + q[1] * a[3] + q[2]) < 0) return false;
    if ((p[0] * b[0] + p[1] * b[1] + p[2]) * (q[0] * b[2] + q[1] * b[3] + q[2]) < 0) return false;
    return true;
  }

  // 8x9 system in raw pixel coordinates with h33 = 1, solved by the
  // reference's Gauss elimination (bubble pivot pre-pass, no further pivoting).
  __device__ static bool solve_four(const double* const rows[4], const double* w4, double* out) {
    double a[8][9];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const double* p = rows[i];
      const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
      const double w = w4 ? w4[i] : 1.0;
      const double mwx1 = -w * x1, mwy1 = -w * y1, wx2 = w * x2, wy2 = w * y2;
      a[2 * i][0] = mwx1; a[2 * i][1] = mwy1; a[2 * i][2] = -w;
      a[2 * i][3] = 0; a[2 * i][4] = 0; a[2 * i][5] = 0;
      a[2 * i][6] = wx2 * x1; a[2 * i][7] = wx2 * y1; a[2 * i][8] = -wx2;
      a[2 * i + 1][0] = 0; a[2 * i + 1][1] = 0; a[2 * i + 1][2] = 0;
      a[2 * i + 1][3] = mwx1; a[2 * i + 1][4] = mwy1; a[2 * i + 1][5] = -w;
      a[2 * i + 1][6] = wy2 * x1; a[2 * i + 1][7] = wy2 * y1; a[2 * i + 1][8] = -wy2;
    }
    double h[8];
    gauss_elimination8(a, h);
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (isnan(h[i])) return false;
    for (int i = 0; i < 8; ++i) out[i] = h[i];
    out[8] = 1.0;
    return true;
  }

  __device__ static int minimal(const double* pts, const int* s, double* out, const double* = nullptr) {
    const double* rows[4] = {pts + 4 * s[0], pts + 4 * s[1], pts + 4 * s[2], pts + 4 * s[3]};
    return solve_four(rows, nullptr, out) ? 1 : 0;
  }

  __device__ static bool valid_model(const double* m) { return fabs(det3(m)) >= 1e-2; }

  __device__ __forceinline__ static double r2_f64(const double* p, const double* h) {
    const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
    const double t1 = h[0] * x1 + h[1] * y1 + h[2];
    const double t2 = h[3] * x1 + h[4] * y1 + h[5];
    const double t3 = h[6] * x1 + h[7] * y1 + h[8];
    const double d1 = x2 - (t1 / t3);
    const double d2 = y2 - (t2 / t3);
    return d1 * d1 + d2 * d2;
  }

  // FP32 filter residual on centred coordinates; `it` returns 1/t3 for the
  // error bound.
  __device__ __forceinline__ static float r2_f32(const float4 p, const float* h, float& it) {
    const float t1 = fmaf(h[0], p.x, fmaf(h[1], p.y, h[2]));
    const float t2 = fmaf(h[3], p.x, fmaf(h[4], p.y, h[5]));
    const float t3 = fmaf(h[6], p.x, fmaf(h[7], p.y, h[8]));
    it = __frcp_rn(t3);
    const float d1 = fmaf(-t1, it, p.z);
    const float d2 = fmaf(-t2, it, p.w);
    return fmaf(d1, d1, d2 * d2);
  }

  // FP32 copy of the model acting on coordinates shifted by -c1 (image 1) and
  // -c2 (image 2): H' = T(-c2) H T(c1), scaled so that h'33 = 1 when possible.
  // out[9] receives the error scale cm: the FP32 residual differs from the
  // FP64 one by at most cm * (|1/t3| + 1) (first-order bound on the rounding
  // of the model, the coordinates and the arithmetic, with a factor 8 margin).
  __device__ static void prepare_f32(const double* h, const double* c, double S, float* out) {
    const double c1x = c[0], c1y = c[1], c2x = c[2], c2y = c[3];
    double g[9];
    for (int r = 0; r < 3; ++r) {
      g[3 * r + 0] = h[3 * r + 0];
      g[3 * r + 1] = h[3 * r + 1];
      g[3 * r + 2] = h[3 * r + 0] * c1x + h[3 * r + 1] * c1y + h[3 * r + 2];
    }
    for (int k = 0; k < 3; ++k) {
      g[k] -= c2x * g[6 + k];
      g[3 + k] -= c2y * g[6 + k];
    }
    const double s = fabs(g[8]) > 1e-300 ? 1.0 / g[8] : 1.0;
    for (int k = 0; k < 9; ++k) g[k] *= s;
    for (int k = 0; k < 9; ++k) out[k] = (float)g[k];
    const double k1 = fmax((fabs(g[0]) + fabs(g[1])) * S + fabs(g[2]), (fabs(g[3]) + fabs(g[4])) * S + fabs(g[5]));
    const double k3 = (fabs(g[6]) + fabs(g[7])) * S + fabs(g[8]);
    const double cm = 8.0 * 5.9604644775390625e-08 * (k1 + S * k3 + S);
    out[9] = isfinite(cm) ? (float)cm : 3.0e38f;
    out[10] = 0.f;
    out[11] = 0.f;
  }

  // Hartley normalisation of the selected rows (normalizePoints semantics):
  // mass points and sqrt(2) / mean distance ratios of both images.
  struct Norm {
    double ms0, ms1, md0, md1, rs, rd;
  };

  // The weighted least-squares system of the non-minimal solver (rows
  // w[-x,-y,-1,0,0,0,Xx,Xy] = -wX and w[0,0,0,-x,-y,-1,Yx,Yy] = -wY in
  // normalised coordinates) has the normal matrix
  //   [S 0 -B_X; 0 S -B_Y; -B_X^T -B_Y^T C]  with  S = sum w^2 u u^T, u = (x, y, 1),
  //   B_X = sum w^2 X u v^T, B_Y = sum w^2 Y u v^T, C = sum w^2 (X^2+Y^2) v v^T, v = (x, y),
  // so 23 sums describe it completely (instead of 44 entries of the dense form).
  static constexpr int NACC = 23;
  // acc layout: 0..5 S (xx xy x yy y 1) | 6..10 X (xx xy x yy y) | 11..15 Y (same)
  //             16..18 R (xx xy yy) | 19 X | 20 Y | 21..22 R (x y)
  __device__ __forceinline__ static void accumulate(const Norm& N, const double* p, double w, double* acc) {
    const double x = (p[0] - N.ms0) * N.rs, y = (p[1] - N.ms1) * N.rs;
    const double X = (p[2] - N.md0) * N.rd, Y = (p[3] - N.md1) * N.rd;
    const double w2 = w * w;
    const double wx = w2 * x, wy = w2 * y;
    acc[0] += wx * x; acc[1] += wx * y; acc[2] += wx; acc[3] += wy * y; acc[4] += wy; acc[5] += w2;
    const double Xwx = X * wx, Xwy = X * wy;
    acc[6] += Xwx * x; acc[7] += Xwx * y; acc[8] += Xwx; acc[9] += Xwy * y; acc[10] += Xwy;
    const double Ywx = Y * wx, Ywy = Y * wy;
    acc[11] += Ywx * x; acc[12] += Ywx * y; acc[13] += Ywx; acc[14] += Ywy * y; acc[15] += Ywy;
    const double R = X * X + Y * Y;
    const double Rwx = R * wx, Rwy = R * wy;
    acc[16] += Rwx * x; acc[17] += Rwx * y; acc[18] += Rwy * y;
    acc[19] += X * w2; acc[20] += Y * w2; acc[21] += Rwx; acc[22] += Rwy;
  }

  // Solves the normal equations by block elimination (one 3x3 LDL^T of S
  // shared by both 3x3 blocks, then the 2x2 Schur complement) and
  // denormalises: H = Td^-1 Hn Ts.
  __device__ static bool solve_normal(const Norm& N, const double* a, double* out) {
    // S (symmetric 3x3): s00 s01 s02 / s11 s12 / s22
    const double s00 = a[0], s01 = a[1], s02 = a[2], s11 = a[3], s12 = a[4], s22 = a[5];
    // LDL^T. Like the reference's least-squares solver, a degenerate system
    // still yields a (possibly non-finite) model rather than a failure.
    const double d0 = s00;
    const double l10 = s01 / d0, l20 = s02 / d0;
    const double d1 = s11 - l10 * s01;
    const double l21 = (s12 - l20 * s01) / d1;
    const double d2 = s22 - l20 * s02 - l21 * (s12 - l20 * s01);
    auto solveS = [&](double b0, double b1, double b2, double* z) {
      const double y0 = b0, y1 = b1 - l10 * y0, y2 = b2 - l20 * y0 - l21 * y1;
      const double z2 = y2 / d2, z1 = y1 / d1 - l21 * z2, z0 = y0 / d0 - l10 * z1 - l20 * z2;
      z[0] = z0; z[1] = z1; z[2] = z2;
    };
    // B_X columns (u * x, u * y) and B_Y; the off-diagonal blocks are -B
    const double BX0[3] = {a[6], a[7], a[8]};   // u * x : (xx, yx, x)
    const double BX1[3] = {a[7], a[9], a[10]};  // u * y : (xy, yy, y)
    const double BY0[3] = {a[11], a[12], a[13]};
    const double BY1[3] = {a[12], a[14], a[15]};
    // right-hand sides: (S_X u, S_Y u, -S_R v)
    const double b1x[3] = {a[8], a[10], a[19]};
    const double b1y[3] = {a[13], a[15], a[20]};
    double ZX0[3], ZX1[3], ZY0[3], ZY1[3], zx[3], zy[3];
    solveS(BX0[0], BX0[1], BX0[2], ZX0);
    solveS(BX1[0], BX1[1], BX1[2], ZX1);
    solveS(BY0[0], BY0[1], BY0[2], ZY0);
    solveS(BY1[0], BY1[1], BY1[2], ZY1);
    solveS(b1x[0], b1x[1], b1x[2], zx);
    solveS(b1y[0], b1y[1], b1y[2], zy);
    auto dot3 = [](const double* p, const double* q) { return p[0] * q[0] + p[1] * q[1] + p[2] * q[2]; };
    // Schur complement M = C - B_X^T S^-1 B_X - B_Y^T S^-1 B_Y (the signs of -B cancel)
    const double m00 = a[16] - dot3(BX0, ZX0) - dot3(BY0, ZY0);
    const double m01 = a[17] - dot3(BX0, ZX1) - dot3(BY0, ZY1);
    const double m11 = a[18] - dot3(BX1, ZX1) - dot3(BY1, ZY1);
    // right side: -S_R v - (-B_X)^T S^-1 b1x - (-B_Y)^T S^-1 b1y
    const double r0 = -a[21] + dot3(BX0, zx) + dot3(BY0, zy);
    const double r1 = -a[22] + dot3(BX1, zx) + dot3(BY1, zy);
    const double det = m00 * m11 - m01 * m01;
    const double h6 = (r0 * m11 - r1 * m01) / det;
    const double h7 = (m00 * r1 - m01 * r0) / det;
    // h1 = S^-1 (b1x + B_X h3), h2 = S^-1 (b1y + B_Y h3)
    double hn[9];
    hn[0] = zx[0] + ZX0[0] * h6 + ZX1[0] * h7;
    hn[1] = zx[1] + ZX0[1] * h6 + ZX1[1] * h7;
    hn[2] = zx[2] + ZX0[2] * h6 + ZX1[2] * h7;
    hn[3] = zy[0] + ZY0[0] * h6 + ZY1[0] * h7;
    hn[4] = zy[1] + ZY0[1] * h6 + ZY1[1] * h7;
    hn[5] = zy[2] + ZY0[2] * h6 + ZY1[2] * h7;
    hn[6] = h6;
    hn[7] = h7;
    hn[8] = 1.0;
    const double Ts[9] = {N.rs, 0, -N.rs * N.ms0, 0, N.rs, -N.rs * N.ms1, 0, 0, 1};
    const double Tdi[9] = {1.0 / N.rd, 0, N.md0, 0, 1.0 / N.rd, N.md1, 0, 0, 1};
    double t[9];
    matmul3(Tdi, hn, t);
    matmul3(t, Ts, out);
    return true;
  }

  __device__ static void normalise(const double* pts, const int* idx, int n, Norm& N) {
    double a = 0, b = 0, c = 0, d = 0;
    for (int i = 0; i < n; ++i) {
      const double* p = pts + 4 * idx[i];
      a += p[0]; b += p[1]; c += p[2]; d += p[3];
    }
    N.ms0 = a / n; N.ms1 = b / n; N.md0 = c / n; N.md1 = d / n;
    double ads = 0, add = 0;
    for (int i = 0; i < n; ++i) {
      const double* p = pts + 4 * idx[i];
      const double dx1 = N.ms0 - p[0], dy1 = N.ms1 - p[1], dx2 = N.md0 - p[2], dy2 = N.md1 - p[3];
      ads += sqrt(dx1 * dx1 + dy1 * dy1);
      add += sqrt(dx2 * dx2 + dy2 * dy2);
    }
    N.rs = M_SQRT2 / (ads / n);
    N.rd = M_SQRT2 / (add / n);
  }

  // Normalised least squares over the n rows idx[] with unit weights by one
  // thread (the local-optimisation trials run one per lane).
  __device__ static bool fit_thread(const double* pts, const int* idx, int n, double* out) {
    if (n < NONMIN) return false;
    Norm N;
    normalise(pts, idx, n, N);
    double acc[NACC];
#pragma unroll
    for (int k = 0; k < NACC; ++k) acc[k] = 0;
    for (int i = 0; i < n; ++i) accumulate(N, pts + 4 * idx[i], 1.0, acc);
    return solve_normal(N, acc, out);
  }
};

// Affine-correspondence homography (findHomographyAC_, solver = 2 of the
// python entry; src/pygcransac/include/estimators/homography_affine_correspondence_estimator.h:58-403
// with the minimal solver of solver_homography_two_affine.h:88-237). The
// minimal sample is two correspondences whose local affine maps (a11, a12,
// a21, a22) sit in the engine's aux array; residuals, the non-minimal fit and
// the model check are the point estimator's, the inner sample of the local
// optimisation is 7 x 2 correspondences.
struct HomographyAffineModel : HomographyModel {
  static constexpr int M = 2;
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;
  static constexpr bool AFFINE = true;

  // isValidSample (:346-400): the point estimator's oriented test on the two
  // points and two points built from the first affine map,
  // c = (1, 0, A (1, 0)^T), d = (1, 0, A (0, 1)^T).
  __device__ static bool valid_sample_affine(const double* pts, const double* aff, const int* s) {
    const double *a = pts + 4 * s[0], *b = pts + 4 * s[1];
    const double* A = aff + 4 * s[0];
    const double c[4] = {1.0, 0.0, A[0], A[2]};
    const double d[4] = {1.0, 0.0, A[1], A[3]};
    auto cross = [](double r[3], const double* u, const double* v) {
      r[0] = u[1] - v[1];
      r[1] = v[0] - u[0];
      r[2] = u[0] * v[1] - u[1] * v[0];
    };
    double p[3], q[3];
    cross(p, a, b);
    cross(q, a + 2, b + 2);
    if ((p[0] * c[0] + p[1] * c[1] + p[2]) * (q[0] * c[2] + q[1] * c[3] + q[2]) < 0) return false;
    if ((p[0] * d[0] + p[1] * d[1] + p[2]) * (q[0] * d[2] + q[1] * d[3] + q[2]) < 0) return false;
    cross(p, c, d);
    cross(q, c + 2, d + 2);
    if ((p[0] * a[0] + p[1] * a[1] + p[2]) * (q[0] * a[2] + q[1] * a[3] + q[2]) < 0) return false;
    if ((p[0] * b[0] + p[1] * b[1] + p[2]) * (q[0] * b[2] + q[1] * b[3] + q[2]) < 0) return false;
    return true;
  }

  // The minimal case's 8 x 9 system (both correspondences' point rows, the
  // first one's four affine rows) has a one-dimensional null space; the
  // reference takes it from an SVD and divides by h33. With h33 = 1 the first
  // eight columns form a square system, solved here by Gaussian elimination
  // with partial pivoting. A singular system gives no model.
  __device__ static int minimal_affine(const double* pts, const double* aff, const int* s, double* out) {
    double A[8][9];
    auto point_rows = [](double (*r)[9], const double* p) {
      const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
      r[0][0] = -x1; r[0][1] = -y1; r[0][2] = -1.0; r[0][3] = 0.0; r[0][4] = 0.0; r[0][5] = 0.0;
      r[0][6] = x2 * x1; r[0][7] = x2 * y1; r[0][8] = -x2;
      r[1][0] = 0.0; r[1][1] = 0.0; r[1][2] = 0.0; r[1][3] = -x1; r[1][4] = -y1; r[1][5] = -1.0;
      r[1][6] = y2 * x1; r[1][7] = y2 * y1; r[1][8] = -y2;
    };
    const double* a = pts + 4 * s[0];
    const double* m = aff + 4 * s[0];
    point_rows(A, a);
    {
      const double x1 = a[0], y1 = a[1], x2 = a[2], y2 = a[3];
      const double a11 = m[0], a12 = m[1], a21 = m[2], a22 = m[3];
      double* r = A[2];
      r[0] = -1.0; r[1] = 0.0; r[2] = 0.0; r[3] = 0.0; r[4] = 0.0; r[5] = 0.0;
      r[6] = x2 + a11 * x1; r[7] = a11 * y1; r[8] = -a11;
      r = A[3];
      r[0] = 0.0; r[1] = -1.0; r[2] = 0.0; r[3] = 0.0; r[4] = 0.0; r[5] = 0.0;
      r[6] = a12 * x1; r[7] = x2 + a12 * y1; r[8] = -a12;
      r = A[4];
      r[0] = 0.0; r[1] = 0.0; r[2] = 0.0; r[3] = -1.0; r[4] = 0.0; r[5] = 0.0;
      r[6] = y2 + a21 * x1; r[7] = a21 * y1; r[8] = -a21;
      r = A[5];
      r[0] = 0.0; r[1] = 0.0; r[2] = 0.0; r[3] = 0.0; r[4] = -1.0; r[5] = 0.0;
      r[6] = a22 * x1; r[7] = y2 + a22 * y1; r[8] = -a22;
    }
    point_rows(A + 6, pts + 4 * s[1]);
    // column 8 holds the right-hand side -A[:, 8] (negated above)
    for (int col = 0; col < 8; ++col) {
      int piv = col;
      for (int r = col + 1; r < 8; ++r)
        if (fabs(A[r][col]) > fabs(A[piv][col])) piv = r;
      if (!(fabs(A[piv][col]) > 0.0)) return 0;
      if (piv != col)
        for (int k = 0; k < 9; ++k) {
          const double t = A[piv][k];
          A[piv][k] = A[col][k];
          A[col][k] = t;
        }
      for (int r = col + 1; r < 8; ++r) {
        const double f = A[r][col] / A[col][col];
        for (int k = col; k < 9; ++k) A[r][k] -= f * A[col][k];
      }
    }
    double h[8];
    for (int i = 7; i >= 0; --i) {
      double acc = A[i][8];
      for (int k = i + 1; k < 8; ++k) acc -= A[i][k] * h[k];
      h[i] = acc / A[i][i];
    }
    for (int i = 0; i < 8; ++i) {
      if (!isfinite(h[i])) return 0;
      out[i] = h[i];
    }
    out[8] = 1.0;
    return 1;
  }
};

// Real roots, in ascending order, of c[0] + c[1] x + ... + c[deg] x^deg
// (deg <= 4). The roots of the quadratic derivative come in closed form; the
// roots of each higher derivative, and of the polynomial itself, are then
// isolated between consecutive roots of the next derivative and the Cauchy
// bound and bisected to the last representable midpoint. Leading
// coefficients that are exactly zero lower the degree. Returns the count.
__device__ inline int poly_quadratic_roots(const double* c, double* roots) {
  const double disc = c[1] * c[1] - 4.0 * c[2] * c[0];
  if (disc < 0.0) return 0;
  const double q = -0.5 * (c[1] + copysign(sqrt(disc), c[1]));
  double r0 = q / c[2], r1 = q != 0.0 ? c[0] / q : r0;
  if (r1 < r0) {
    const double t = r0;
    r0 = r1;
    r1 = t;
  }
  roots[0] = r0;
  roots[1] = r1;
  return 2;
}

// roots of c (degree deg, c[deg] != 0) given the ascending real roots cp of
// its derivative
__device__ inline int poly_bracketed_roots(const double* c, int deg, const double* cp, int ncp, double* roots) {
  double bound = 0.0;
  for (int i = 0; i < deg; ++i) bound = fmax(bound, fabs(c[i] / c[deg]));
  bound += 1.0;
  auto f = [&](double x) {
    double v = c[deg];
    for (int i = deg - 1; i >= 0; --i) v = v * x + c[i];
    return v;
  };
  double edges[6];
  int ne = 0;
  edges[ne++] = -bound;
  for (int i = 0; i < ncp; ++i)
    if (cp[i] > -bound && cp[i] < bound) edges[ne++] = cp[i];
  edges[ne++] = bound;
  int nr = 0;
  for (int k = 0; k + 1 < ne; ++k) {
    double lo = edges[k], hi = edges[k + 1];
    double flo = f(lo);
    const double fhi = f(hi);
    if (flo == 0.0) {
      if (nr == 0 || roots[nr - 1] != lo) roots[nr++] = lo;
      continue;
    }
    if ((flo < 0.0) == (fhi < 0.0)) continue;
    for (int it = 0; it < 200; ++it) {
      const double mid = 0.5 * (lo + hi);
      if (mid <= lo || mid >= hi) break;
      const double fm = f(mid);
      if (fm == 0.0) {
        lo = hi = mid;
        break;
      }
      if ((fm < 0.0) == (flo < 0.0)) {
        lo = mid;
        flo = fm;
      } else {
        hi = mid;
      }
    }
    roots[nr++] = 0.5 * (lo + hi);
  }
  return nr;
}

__device__ inline int poly_real_roots(const double* c_in, int deg, double* roots) {
  while (deg > 0 && c_in[deg] == 0.0) --deg;
  if (deg <= 0) return 0;
  if (deg == 1) {
    roots[0] = -c_in[0] / c_in[1];
    return isfinite(roots[0]) ? 1 : 0;
  }
  // lv[j]: the (deg - j)-th derivative, of degree j
  double lv[5][5];
  for (int i = 0; i <= deg; ++i) lv[deg][i] = c_in[i];
  for (int j = deg - 1; j >= 2; --j)
    for (int i = 0; i <= j; ++i) lv[j][i] = (i + 1) * lv[j + 1][i + 1];
  double cur[4], nxt[4];
  int n = poly_quadratic_roots(lv[2], cur);
  for (int j = 3; j <= deg; ++j) {
    n = poly_bracketed_roots(lv[j], j, cur, n, nxt);
    for (int i = 0; i < n; ++i) cur[i] = nxt[i];
  }
  for (int i = 0; i < n; ++i) roots[i] = cur[i];
  return n;
}

// SIFT-correspondence homography (findHomographySIFT_,
// gcransac_python.cpp:4813-5069): rows (x1, y1, x2, y2, q1, q2, o1, o2) with
// the features' scales q and orientations o; the point estimator
// (RobustHomographyEstimator: residual, validity, the 4-point non-minimal
// fit) with the two-correspondence minimal solver HomographyTwoSIFTSolver
// (solver_homography_two_sift.h:113-480).
struct HomographySiftModel : HomographyModel {
  static constexpr int M = 2;
  static constexpr int MAXSOL = 4;  // conic intersections
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;
  static constexpr bool AFFINE = true;

  // isValidSample (homography_estimator.h:350-351): samples of fewer than
  // four correspondences are not tested
  __device__ static bool valid_sample_affine(const double*, const double*, const int*) { return true; }

  // Each correspondence gives its two point rows and one orientation row
  // (J o1 parallel to o2 for the homography's Jacobian J at x1): a 6 x 9
  // system with a three-dimensional null space. Each correspondence's scale
  // ratio then gives a quadratic form in the null-space coordinates,
  // q2 w(h)^2 - q1 D(h) = 0 with w = h7 x1 + h8 y1 + h9 and
  // D = (h1 h5 - h2 h4) + x2 (h4 h8 - h5 h7) + y2 (h2 h7 - h1 h8)
  // (w^2 det J); the two conics meet in up to four points. The reference
  // takes the null space from an SVD and intersects the conics by an
  // elimination template and a 4 x 4 eigenproblem; here the null space comes
  // from Gaussian elimination with full pivoting over h1..h8 (h9 stays free,
  // so its basis vector carries h9 = 1 and the others h9 = 0), and the
  // intersections from the resultant quartic in the second coordinate, whose
  // real roots are isolated by bisection; the first coordinate follows
  // linearly. Models come in ascending order of that root, each with h9 = 1.
  __device__ static int minimal_affine(const double* pts, const double* aux, const int* s, double* out) {
    double A[6][9];
    double u1[2], v1[2], u2[2], v2[2], q1[2], q2[2];
    for (int c = 0; c < 2; ++c) {
      const double* p = pts + 4 * s[c];
      const double* f = aux + 4 * s[c];
      u1[c] = p[0]; v1[c] = p[1]; u2[c] = p[2]; v2[c] = p[3];
      q1[c] = f[0]; q2[c] = f[1];
      double s1, c1, s2, c2;
      sincos(f[2], &s1, &c1);
      sincos(f[3], &s2, &c2);
      double* r = A[3 * c];
      r[0] = 0.0; r[1] = 0.0; r[2] = 0.0; r[3] = u1[c]; r[4] = v1[c]; r[5] = 1.0;
      r[6] = -u1[c] * v2[c]; r[7] = -v1[c] * v2[c]; r[8] = -v2[c];
      r = A[3 * c + 1];
      r[0] = u1[c]; r[1] = v1[c]; r[2] = 1.0; r[3] = 0.0; r[4] = 0.0; r[5] = 0.0;
      r[6] = -u1[c] * u2[c]; r[7] = -v1[c] * u2[c]; r[8] = -u2[c];
      r = A[3 * c + 2];
      r[0] = -c1 * s2; r[1] = -s1 * s2; r[2] = 0.0; r[3] = c1 * c2; r[4] = s1 * c2; r[5] = 0.0;
      r[6] = u2[c] * c1 * s2 - v2[c] * c1 * c2; r[7] = u2[c] * s1 * s2 - v2[c] * s1 * c2; r[8] = 0.0;
    }
    // elimination with full pivoting over columns 0..7
    int col_of[6];
    bool used[8] = {false, false, false, false, false, false, false, false};
    for (int k = 0; k < 6; ++k) {
      int pr = -1, pc = -1;
      double best = 0.0;
      for (int r = k; r < 6; ++r)
        for (int c = 0; c < 8; ++c)
          if (!used[c] && fabs(A[r][c]) > best) { best = fabs(A[r][c]); pr = r; pc = c; }
      if (!(best > 0.0)) return 0;
      if (pr != k)
        for (int j = 0; j < 9; ++j) { const double t = A[pr][j]; A[pr][j] = A[k][j]; A[k][j] = t; }
      used[pc] = true;
      col_of[k] = pc;
      const double inv = 1.0 / A[k][pc];
      for (int j = 0; j < 9; ++j) A[k][j] *= inv;
      for (int r = 0; r < 6; ++r) {
        if (r == k) continue;
        const double fct = A[r][pc];
        if (fct != 0.0)
          for (int j = 0; j < 9; ++j) A[r][j] -= fct * A[k][j];
      }
    }
    int fr[3];
    int nf = 0;
    for (int c = 0; c < 8; ++c)
      if (!used[c]) fr[nf++] = c;
    fr[2] = 8;
    // basis vectors: N[b] has 1 at free column fr[b], 0 at the other free
    // columns, and -A[k][fr[b]] at pivot column col_of[k]
    double N[3][9];
    for (int b = 0; b < 3; ++b) {
      for (int j = 0; j < 9; ++j) N[b][j] = 0.0;
      N[b][fr[b]] = 1.0;
      for (int k = 0; k < 6; ++k) N[b][col_of[k]] = -A[k][fr[b]];
    }
    // conic of each correspondence in (a, b) for h = a N0 + b N1 + N2:
    // k[0] a^2 + k[1] a b + k[2] b^2 + k[3] a + k[4] b + k[5]
    double K[2][6];
    for (int c = 0; c < 2; ++c) {
      auto form = [&](const double* x, const double* y) {
        const double wx = x[6] * u1[c] + x[7] * v1[c] + x[8];
        const double wy = y[6] * u1[c] + y[7] * v1[c] + y[8];
        const double dxy = 0.5 * ((x[0] * y[4] + y[0] * x[4] - x[1] * y[3] - y[1] * x[3]) +
                                  u2[c] * (x[3] * y[7] + y[3] * x[7] - x[4] * y[6] - y[4] * x[6]) +
                                  v2[c] * (x[1] * y[6] + y[1] * x[6] - x[0] * y[7] - y[0] * x[7]));
        return q2[c] * wx * wy - q1[c] * dxy;
      };
      K[c][0] = form(N[0], N[0]);
      K[c][1] = 2.0 * form(N[0], N[1]);
      K[c][2] = form(N[1], N[1]);
      K[c][3] = 2.0 * form(N[0], N[2]);
      K[c][4] = 2.0 * form(N[1], N[2]);
      K[c][5] = form(N[2], N[2]);
    }
    // as quadratics in a: A_c a^2 + (K1 b + K3) a + (K2 b^2 + K4 b + K5);
    // resultant (A1 C2 - A2 C1)^2 - (A1 B2 - A2 B1)(B1 C2 - B2 C1)
    const double a1 = K[0][0], a2 = K[1][0];
    const double p2 = a1 * K[1][2] - a2 * K[0][2], p1 = a1 * K[1][4] - a2 * K[0][4], p0 = a1 * K[1][5] - a2 * K[0][5];
    const double l1 = a1 * K[1][1] - a2 * K[0][1], l0 = a1 * K[1][3] - a2 * K[0][3];
    const double k3 = K[0][1] * K[1][2] - K[1][1] * K[0][2];
    const double k2 = K[0][1] * K[1][4] + K[0][3] * K[1][2] - K[1][1] * K[0][4] - K[1][3] * K[0][2];
    const double k1 = K[0][1] * K[1][5] + K[0][3] * K[1][4] - K[1][1] * K[0][5] - K[1][3] * K[0][4];
    const double k0 = K[0][3] * K[1][5] - K[1][3] * K[0][5];
    const double r[5] = {p0 * p0 - l0 * k0, 2.0 * p1 * p0 - (l1 * k0 + l0 * k1),
                         p1 * p1 + 2.0 * p2 * p0 - (l1 * k1 + l0 * k2), 2.0 * p2 * p1 - (l1 * k2 + l0 * k3),
                         p2 * p2 - l1 * k3};
    double roots[4];
    const int nr = poly_real_roots(r, 4, roots);
    int nm = 0;
    for (int i = 0; i < nr; ++i) {
      const double b = roots[i];
      // A2 Q1 - A1 Q2 = -(L(b) a + P(b)) = 0
      const double L = l1 * b + l0, P = (p2 * b + p1) * b + p0;
      const double a = -P / L;
      double* h = out + 9 * nm;
      bool fin = true;
      for (int j = 0; j < 9; ++j) {
        h[j] = a * N[0][j] + b * N[1][j] + N[2][j];
        fin = fin && isfinite(h[j]);
      }
      if (fin) ++nm;
    }
    return nm;
  }
};

}  // namespace gcr
