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
  static constexpr int M = 4;          // minimal sample size
  static constexpr int MAXSOL = 1;     // models per minimal sample
  static constexpr int NONMIN = 4;     // smallest non-minimal sample
  static constexpr int INLIER_LIMIT = 7 * M;
  static constexpr bool WEIGHTED = true;
  static constexpr int NACC = 44;          // packed upper 8x8 normal matrix + right side
  static constexpr int SAMPLE_CAP = INLIER_LIMIT;

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

  __device__ static int minimal(const double* pts, const int* s, double* out) {
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

  // Hartley normalisation of the selected rows (normalizePoints semantics).
  // Returns the similarity parameters (mass points and ratios).
  struct Norm {
    double ms0, ms1, md0, md1, rs, rd;
  };

  // Normalised least squares over n rows given by idx[] with optional per-row
  // weights (row k uses wrow[k]), single thread. Denormalised result in out.
  __device__ static bool fit_thread(const double* pts, const int* idx, int n, const double* wrow, double* out) {
    if (n < NONMIN) return false;
    Norm N;
    {
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
    double acc[NACC];
    for (int k = 0; k < NACC; ++k) acc[k] = 0;
    for (int i = 0; i < n; ++i) {
      const double* p = pts + 4 * idx[i];
      const double w = wrow ? wrow[i] : 1.0;
      accumulate(N, p, w, acc);
    }
    return solve_normal(N, acc, out);
  }

  // Adds the two weighted equations of one correspondence to the packed
  // normal equations (upper triangle of the 8x8 A^T A, row-major packed).
  __device__ __forceinline__ static void accumulate(const Norm& N, const double* p, double w, double* acc) {
    double* ata = acc;
    double* atb = acc + 36;
    const double x1 = (p[0] - N.ms0) * N.rs, y1 = (p[1] - N.ms1) * N.rs;
    const double x2 = (p[2] - N.md0) * N.rd, y2 = (p[3] - N.md1) * N.rd;
    const double mwx1 = -w * x1, mwy1 = -w * y1, wx2 = w * x2, wy2 = w * y2;
    const double r0[8] = {mwx1, mwy1, -w, 0, 0, 0, wx2 * x1, wx2 * y1};
    const double r1[8] = {0, 0, 0, mwx1, mwy1, -w, wy2 * x1, wy2 * y1};
    const double b0 = -wx2, b1 = -wy2;
    int k = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
#pragma unroll
      for (int j = i; j < 8; ++j) ata[k++] += r0[i] * r0[j] + r1[i] * r1[j];
      atb[i] += r0[i] * b0 + r1[i] * b1;
    }
  }

  __device__ static bool solve_normal(const Norm& N, const double* acc, double* out) {
    const double* ata = acc;
    const double* atb = acc + 36;
    double A[8][8], x[8];
    int k = 0;
    for (int i = 0; i < 8; ++i)
      for (int j = i; j < 8; ++j) { A[i][j] = ata[k]; A[j][i] = ata[k]; ++k; }
    for (int i = 0; i < 8; ++i) x[i] = atb[i];
    if (!cholesky_solve<8>(A, x)) return false;
    const double hn[9] = {x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7], 1.0};
    // H = Td^-1 * Hn * Ts with Ts = [rs 0 -rs ms0; 0 rs -rs ms1; 0 0 1]
    const double Ts[9] = {N.rs, 0, -N.rs * N.ms0, 0, N.rs, -N.rs * N.ms1, 0, 0, 1};
    const double Tdi[9] = {1.0 / N.rd, 0, N.md0, 0, 1.0 / N.rd, N.md1, 0, 0, 1};
    double t[9];
    matmul3(Tdi, hn, t);
    matmul3(t, Ts, out);
    return true;
  }
};

}  // namespace gcr
