// FP32 local-optimisation fit of a fundamental matrix: the non-minimal fit
// of FundamentalMatrixBundleAdjustmentSolver (normalised 8-point start, then
// 25 Levenberg-Marquardt iterations on the factorised F = u0 v0^T + sigma u1
// v1^T with the truncated Sampson loss; solver_fundamental_matrix_bundle_
// adjustment.h:114-178, relative_pose/bundle.cpp:252-339,
// relative_pose/jacobian_impl.h:470-615) computed entirely in FP32 from the
// centred FP32 correspondence tile, by a group of lanes.
//
// This is the fast local optimisation of the learned form: GB300 issues FP64
// at about 1/64 of its FP32 rate, and the graph-cut local optimisation (50
// such fits per labelling) is where the learned form spends most of its FP64
// work. A fit's model is only a candidate: it is scored exactly (FP64 inlier
// decisions) like every other model. The same solver pieces (pivoted-QR null
// vector, 3x3 SVD, damped Cholesky step) serve the CTA-wide iteratively
// reweighted fits, the final refit and the drivers' bundle adjustment of the
// fast mode. Masks can differ from the FP64 fits' in the last bits of a
// candidate, so parity runs keep the FP64 fits (the engine's default).
#pragma once

#include "gcr_fundamental.cuh"

namespace gcr {
namespace lo32 {

// sum over the `width` lanes of a group (width a power of two, lanes of a
// group contiguous): every lane gets ((s0 + s1) + (s2 + s3)) ...
__device__ __forceinline__ float gsum(float v, unsigned mask, int width) {
  for (int o = 1; o < width; o <<= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}

// Symmetric 3x3 eigen decomposition by cyclic Jacobi rotations (descending
// eigenvalues, eigenvectors in the columns of V, row-major).
__device__ inline void sym3_eigen(const float* S_in, float* w, float* V) {
  float S[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) S[i] = S_in[i];
#pragma unroll
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.f : 0.f;
  for (int sweep = 0; sweep < 12; ++sweep) {
    const float off = S[1] * S[1] + S[2] * S[2] + S[5] * S[5];
    const float diag = S[0] * S[0] + S[4] * S[4] + S[8] * S[8];
    if (!(off > 1e-14f * diag) || off < 1e-36f) break;
#pragma unroll
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0;
      const int q = pq == 0 ? 1 : 2;
      const float apq = S[p * 3 + q];
      if (fabsf(apq) > 1e-36f) {
        const float app = S[p * 3 + p], aqq = S[q * 3 + q];
        const float theta = (aqq - app) / (2.f * apq);
        const float t = (theta >= 0.f ? 1.f : -1.f) / (fabsf(theta) + sqrtf(theta * theta + 1.f));
        const float cs = rsqrtf(t * t + 1.f), sn = t * cs;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float skp = S[k * 3 + p], skq = S[k * 3 + q];
          S[k * 3 + p] = cs * skp - sn * skq;
          S[k * 3 + q] = sn * skp + cs * skq;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float spk = S[p * 3 + k], sqk = S[q * 3 + k];
          S[p * 3 + k] = cs * spk - sn * sqk;
          S[q * 3 + k] = sn * spk + cs * sqk;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float vkp = V[k * 3 + p], vkq = V[k * 3 + q];
          V[k * 3 + p] = cs * vkp - sn * vkq;
          V[k * 3 + q] = sn * vkp + cs * vkq;
        }
      }
    }
  }
  float d[3] = {S[0], S[4], S[8]};
  auto cswap = [&](int a, int b) {
    const bool sw = d[a] < d[b];
    const float da = d[a], db = d[b];
    d[a] = sw ? db : da;
    d[b] = sw ? da : db;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float va = V[i * 3 + a], vb = V[i * 3 + b];
      V[i * 3 + a] = sw ? vb : va;
      V[i * 3 + b] = sw ? va : vb;
    }
  };
  cswap(0, 1);
  cswap(1, 2);
  cswap(0, 1);
#pragma unroll
  for (int j = 0; j < 3; ++j) w[j] = d[j];
}

// SVD of a 3x3 matrix (singular values descending): V from the eigenvectors of
// A^T A, the first two columns of U from A V / s, the third by a cross product
// with the sign that reproduces A.
__device__ inline void svd3(const float* A, float* U, float* s, float* V) {
  float AtA[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) AtA[i * 3 + j] = A[i] * A[j] + A[3 + i] * A[3 + j] + A[6 + i] * A[6 + j];
  float w[3];
  sym3_eigen(AtA, w, V);
#pragma unroll
  for (int j = 0; j < 3; ++j) s[j] = sqrtf(fmaxf(0.f, w[j]));
  float c[3][3];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    float u[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) u[i] = A[i * 3] * V[j] + A[i * 3 + 1] * V[3 + j] + A[i * 3 + 2] * V[6 + j];
    const float nrm = sqrtf(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) c[j][i] = nrm > 0.f ? u[i] / nrm : (i == j ? 1.f : 0.f);
  }
  c[2][0] = c[0][1] * c[1][2] - c[0][2] * c[1][1];
  c[2][1] = c[0][2] * c[1][0] - c[0][0] * c[1][2];
  c[2][2] = c[0][0] * c[1][1] - c[0][1] * c[1][0];
  float u2[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) u2[i] = A[i * 3] * V[2] + A[i * 3 + 1] * V[5] + A[i * 3 + 2] * V[8];
  if (u2[0] * c[2][0] + u2[1] * c[2][1] + u2[2] * c[2][2] < 0.f)
#pragma unroll
    for (int i = 0; i < 3; ++i) c[2][i] = -c[2][i];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) U[i * 3 + j] = c[j][i];
}

// Null vector of the 9x9 symmetric normal matrix M of the 8-point system: the
// last column of Q of its complete-pivoting Householder QR (M is overwritten).
__device__ inline void qr9_null(float* M, float* q) {
  int transp[9];
  float tau[9];
  float biggest_all = 0.f;
  int steps = 9;
  for (int k = 0; k < 9; ++k) {
    int bi = k, bj = k;
    float best = -1.f;
    for (int i = k; i < 9; ++i)
      for (int j = k; j < 9; ++j) {
        const float v = fabsf(M[i * 9 + j]);
        if (v > best) { best = v; bi = i; bj = j; }
      }
    if (k == 0) biggest_all = best;
    if (best <= biggest_all * (1.1920929e-07f * 9.f)) {
      steps = k;
      break;
    }
    transp[k] = bi;
    if (bi != k)
      for (int j = k; j < 9; ++j) { const float t = M[k * 9 + j]; M[k * 9 + j] = M[bi * 9 + j]; M[bi * 9 + j] = t; }
    if (bj != k)
      for (int i = 0; i < 9; ++i) { const float t = M[i * 9 + k]; M[i * 9 + k] = M[i * 9 + bj]; M[i * 9 + bj] = t; }
    const float c0 = M[k * 9 + k];
    float tail = 0.f;
    for (int i = k + 1; i < 9; ++i) tail += M[i * 9 + k] * M[i * 9 + k];
    float t, beta;
    if (tail <= 1.17549435e-38f) {
      t = 0.f;
      beta = c0;
      for (int i = k + 1; i < 9; ++i) M[i * 9 + k] = 0.f;
    } else {
      beta = sqrtf(c0 * c0 + tail);
      if (c0 >= 0.f) beta = -beta;
      const float inv = 1.f / (c0 - beta);
      for (int i = k + 1; i < 9; ++i) M[i * 9 + k] *= inv;
      t = (beta - c0) / beta;
    }
    tau[k] = t;
    M[k * 9 + k] = beta;
    for (int j = k + 1; j < 9; ++j) {
      float s = M[k * 9 + j];
      for (int i = k + 1; i < 9; ++i) s += M[i * 9 + k] * M[i * 9 + j];
      s *= t;
      M[k * 9 + j] -= s;
      for (int i = k + 1; i < 9; ++i) M[i * 9 + j] -= s * M[i * 9 + k];
    }
  }
  for (int i = 0; i < 9; ++i) q[i] = 0.f;
  q[8] = 1.f;
  for (int k = steps - 1; k >= 0; --k) {
    float s = q[k];
    for (int i = k + 1; i < 9; ++i) s += M[i * 9 + k] * q[i];
    s *= tau[k];
    q[k] -= s;
    for (int i = k + 1; i < 9; ++i) q[i] -= s * M[i * 9 + k];
    if (transp[k] != k) { const float tt = q[k]; q[k] = q[transp[k]]; q[transp[k]] = tt; }
  }
}

// Cholesky solve of the 7x7 damped normal equations (x holds b on entry).
__device__ __forceinline__ bool chol7(float A[7][7], float* x) {
  bool ok = true;
#pragma unroll
  for (int j = 0; j < 7; ++j) {
    float d = A[j][j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= A[j][k] * A[j][k];
    ok = ok && (d > 0.f);
    const float l = sqrtf(fmaxf(d, 1e-30f));
    A[j][j] = l;
    const float il = 1.f / l;
#pragma unroll
    for (int i = j + 1; i < 7; ++i) {
      float s = A[i][j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= A[i][k] * A[j][k];
      A[i][j] = s * il;
    }
  }
#pragma unroll
  for (int i = 0; i < 7; ++i) {
    float s = x[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s -= A[i][k] * x[k];
    x[i] = s / A[i][i];
  }
#pragma unroll
  for (int i = 6; i >= 0; --i) {
    float s = x[i];
#pragma unroll
    for (int k = i + 1; k < 7; ++k) s -= A[k][i] * x[k];
    x[i] = s / A[i][i];
  }
  return ok;
}

struct FactF {
  float U[9], V[9], sigma;
};

__device__ __forceinline__ void fact_to_F(const FactF& f, float* F) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) F[i * 3 + j] = f.U[i * 3] * f.V[j * 3] + f.sigma * f.U[i * 3 + 1] * f.V[j * 3 + 1];
}

// truncated Sampson cost of one normalised correspondence (loss scale 1)
// (truncated at trunc2: 1 in the solver's coordinates; s^2 for coordinates
// scaled by s from a loss truncated at 1 in the original ones)
__device__ __forceinline__ float cost_point(const float* F, float p0, float p1, float q0, float q1,
                                           float trunc2 = 1.f) {
  const float Fx0 = F[0] * p0 + F[1] * p1 + F[2], Fx1 = F[3] * p0 + F[4] * p1 + F[5],
              Fx2 = F[6] * p0 + F[7] * p1 + F[8];
  const float C = q0 * Fx0 + q1 * Fx1 + Fx2;
  const float a0 = F[0] * q0 + F[3] * q1 + F[6], a1 = F[1] * q0 + F[4] * q1 + F[7];
  const float r2 = C * C / (Fx0 * Fx0 + Fx1 * Fx1 + a0 * a0 + a1 * a1);
  return r2 < trunc2 ? r2 : trunc2;
}

// J^T J (lower, 28) and J^T r (7) of one correspondence, weight 1/n for the
// points inside the loss (FundamentalJacobianAccumulator::accumulate) with
// J = dC/dF^T dF/d(rotation of U, rotation of V, sigma) formed from the
// structure of dF/dparams (rotation columns: signed entries of F; sigma column:
// U[:,1] V[:,1]^T).
__device__ __forceinline__ void accumulate_point(const float* F, const float* ds, float p0, float p1, float q0,
                                                 float q1, float inv_n, float* acc, float trunc2 = 1.f) {
  const float Fx0 = F[0] * p0 + F[1] * p1 + F[2], Fx1 = F[3] * p0 + F[4] * p1 + F[5],
              Fx2 = F[6] * p0 + F[7] * p1 + F[8];
  const float C = q0 * Fx0 + q1 * Fx1 + Fx2;
  const float J0 = F[0] * q0 + F[3] * q1 + F[6], J1 = F[1] * q0 + F[4] * q1 + F[7];
  const float J2 = Fx0, J3 = Fx1;
  const float inv = rsqrtf(J0 * J0 + J1 * J1 + J2 * J2 + J3 * J3);
  const float r = C * inv;
  if (!(r * r < trunc2)) return;
  float dF[9] = {p0 * q0, p0 * q1, p0, p1 * q0, p1 * q1, p1, q0, q1, 1.f};
  const float s = C * inv * inv;
  dF[0] -= s * (J2 * p0 + J0 * q0);
  dF[1] -= s * (J3 * p0 + J0 * q1);
  dF[2] -= s * J0;
  dF[3] -= s * (J2 * p1 + J1 * q0);
  dF[4] -= s * (J3 * p1 + J1 * q1);
  dF[5] -= s * J1;
  dF[6] -= s * J2;
  dF[7] -= s * J3;
#pragma unroll
  for (int k = 0; k < 9; ++k) dF[k] *= inv;
  // columns of dF/dparams (jacobian_impl.h:541-550), F row-major
  float J[7];
  J[0] = -dF[1] * F[6] + dF[2] * F[3] - dF[4] * F[7] + dF[5] * F[4] - dF[7] * F[8] + dF[8] * F[5];
  J[1] = dF[0] * F[6] - dF[2] * F[0] + dF[3] * F[7] - dF[5] * F[1] + dF[6] * F[8] - dF[8] * F[2];
  J[2] = -dF[0] * F[3] + dF[1] * F[0] - dF[3] * F[4] + dF[4] * F[1] - dF[6] * F[5] + dF[7] * F[2];
  J[3] = -dF[3] * F[2] - dF[4] * F[5] - dF[5] * F[8] + dF[6] * F[1] + dF[7] * F[4] + dF[8] * F[7];
  J[4] = dF[0] * F[2] + dF[1] * F[5] + dF[2] * F[8] - dF[6] * F[0] - dF[7] * F[3] - dF[8] * F[6];
  J[5] = -dF[0] * F[1] - dF[1] * F[4] - dF[2] * F[7] + dF[3] * F[0] + dF[4] * F[3] + dF[5] * F[6];
  J[6] = dF[0] * ds[0] + dF[1] * ds[3] + dF[2] * ds[6] + dF[3] * ds[1] + dF[4] * ds[4] + dF[5] * ds[7] +
         dF[6] * ds[2] + dF[7] * ds[5] + dF[8] * ds[8];
  int k = 0;
#pragma unroll
  for (int a = 0; a < 7; ++a)
#pragma unroll
    for (int b = 0; b <= a; ++b) acc[k++] += inv_n * (J[a] * J[b]);
#pragma unroll
  for (int a = 0; a < 7; ++a) acc[28 + a] += inv_n * r * J[a];
}

// One damped step (bundle.cpp:285-320): sol = -(J^T J + lambda I)^-1 J^T r,
// U and V rotated by exp([w]x), sigma += dsigma. False when the step is below
// the FP32 tolerance.
__device__ __forceinline__ bool step(const float* acc, float lambda, const FactF& f, FactF& fn) {
  float A[7][7], x[7];
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
  if (!chol7(A, x))
#pragma unroll
    for (int a = 0; a < 7; ++a) x[a] = 0.f;
  float sn = 0.f;
#pragma unroll
  for (int a = 0; a < 7; ++a) sn += x[a] * x[a];
  if (!(sqrtf(sn) >= 1e-7f)) return false;
  auto rot = [](const float* w, const float* M, float* out) {
    const float th = sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
#pragma unroll
    for (int i = 0; i < 9; ++i) out[i] = M[i];
    if (!(th > 1e-30f)) return;
    const float u0 = w[0] / th, u1 = w[1] / th, u2 = w[2] / th;
    float a, c;
    sincosf(th, &a, &c);
    const float b = 1.f - c;
    const float S[9] = {0.f, -u2, u1, u2, 0.f, -u0, -u1, u0, 0.f};
    float R[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float s2 = S[i * 3] * S[j] + S[i * 3 + 1] * S[3 + j] + S[i * 3 + 2] * S[6 + j];
        R[i * 3 + j] = a * S[i * 3 + j] + b * s2;
      }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        out[i * 3 + j] += R[i * 3] * M[j] + R[i * 3 + 1] * M[3 + j] + R[i * 3 + 2] * M[6 + j];
  };
  rot(x, f.U, fn.U);
  rot(x + 3, f.V, fn.V);
  fn.sigma = f.sigma + x[6];
  return true;
}

// Fit of the rows idx[0..n) (indices into the pair's centred FP32 tile pts32;
// centre = the pair's centring) by the `width` lanes of the group `mask`, lane
// q taking rows q, q + width, ...; every lane returns the same verdict and
// lane 0 writes the model (original pixel coordinates, unit Frobenius norm,
// F33 >= 0) in FP64 to out.
__device__ inline bool fit_fundamental(const float4* pts32, const double* centre, const int* idx, int n, double* out,
                                       int q, unsigned mask, int width) {
  if (n < 8) return false;
  const float inv_n = 1.f / (float)n;
  float m0 = 0.f, m1 = 0.f, m2 = 0.f, m3 = 0.f;
  for (int i = q; i < n; i += width) {
    const float4 p = pts32[idx[i]];
    m0 += p.x; m1 += p.y; m2 += p.z; m3 += p.w;
  }
  m0 = gsum(m0, mask, width) * inv_n;
  m1 = gsum(m1, mask, width) * inv_n;
  m2 = gsum(m2, mask, width) * inv_n;
  m3 = gsum(m3, mask, width) * inv_n;
  float ds1 = 0.f, ds2 = 0.f;
  for (int i = q; i < n; i += width) {
    const float4 p = pts32[idx[i]];
    ds1 += sqrtf((p.x - m0) * (p.x - m0) + (p.y - m1) * (p.y - m1));
    ds2 += sqrtf((p.z - m2) * (p.z - m2) + (p.w - m3) * (p.w - m3));
  }
  ds1 = gsum(ds1, mask, width);
  ds2 = gsum(ds2, mask, width);
  if (!(ds1 > 0.f && ds2 > 0.f)) return false;
  const float rs = 1.41421356f / (ds1 * inv_n), rd = 1.41421356f / (ds2 * inv_n);
  // the 8-point start: null vector of A^T A (45 sums)
  float F[9];
  {
    float ata[45];
#pragma unroll
    for (int k = 0; k < 45; ++k) ata[k] = 0.f;
    for (int i = q; i < n; i += width) {
      const float4 p = pts32[idx[i]];
      const float x0 = (p.x - m0) * rs, y0 = (p.y - m1) * rs, x1 = (p.z - m2) * rd, y1 = (p.w - m3) * rd;
      const float r[9] = {x1 * x0, x1 * y0, x1, y1 * x0, y1 * y0, y1, x0, y0, 1.f};
      int k = 0;
#pragma unroll
      for (int a = 0; a < 9; ++a)
#pragma unroll
        for (int b = 0; b <= a; ++b) ata[k++] += r[a] * r[b];
    }
    float M[81];
    int k = 0;
#pragma unroll
    for (int a = 0; a < 9; ++a)
#pragma unroll
      for (int b = 0; b <= a; ++b) {
        const float v = gsum(ata[k++], mask, width);
        M[a * 9 + b] = v;
        M[b * 9 + a] = v;
      }
    qr9_null(M, F);
  }
  FactF f;
  {
    float s[3];
    svd3(F, f.U, s, f.V);
    f.sigma = s[0] > 0.f ? s[1] / s[0] : 0.f;
  }
  auto cost_of = [&](const float* G) {
    float c = 0.f;
    for (int i = q; i < n; i += width) {
      const float4 p = pts32[idx[i]];
      c += cost_point(G, (p.x - m0) * rs, (p.y - m1) * rs, (p.z - m2) * rd, (p.w - m3) * rd);
    }
    return gsum(c, mask, width);
  };
  float G[9];
  fact_to_F(f, G);
  float lambda = 1e-3f;
  float cost = cost_of(G);
  bool recompute = true;
  float acc[35];
  for (int iter = 0; iter < 25; ++iter) {
    if (recompute) {
#pragma unroll
      for (int k = 0; k < 35; ++k) acc[k] = 0.f;
      float ds[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) ds[i * 3 + j] = f.U[i * 3 + 1] * f.V[j * 3 + 1];
      for (int i = q; i < n; i += width) {
        const float4 p = pts32[idx[i]];
        accumulate_point(G, ds, (p.x - m0) * rs, (p.y - m1) * rs, (p.z - m2) * rd, (p.w - m3) * rd, inv_n, acc);
      }
#pragma unroll
      for (int k = 0; k < 35; ++k) acc[k] = gsum(acc[k], mask, width);
      float gn = 0.f;
#pragma unroll
      for (int a = 0; a < 7; ++a) gn += acc[28 + a] * acc[28 + a];
      if (!(sqrtf(gn) >= 1e-7f)) break;
    }
    FactF fn;
    if (!step(acc, lambda, f, fn)) break;
    float Gn[9];
    fact_to_F(fn, Gn);
    const float cn = cost_of(Gn);
    if (cn < cost) {
      f = fn;
#pragma unroll
      for (int k = 0; k < 9; ++k) G[k] = Gn[k];
      lambda *= 0.1f;
      cost = cn;
      recompute = true;
    } else {
      lambda *= 10.f;
      recompute = false;
    }
  }
  bool finite = true;
#pragma unroll
  for (int k = 0; k < 9; ++k) finite = finite && isfinite(G[k]);
  if (!finite) return false;
  if (q == 0) {
    // back to pixels in FP64: the normalisation's means are relative to the
    // centring of the tile
    HomographyModel::Norm N;
    N.ms0 = (double)m0 + centre[0];
    N.ms1 = (double)m1 + centre[1];
    N.md0 = (double)m2 + centre[2];
    N.md1 = (double)m3 + centre[3];
    N.rs = (double)rs;
    N.rd = (double)rd;
    double Gd[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Gd[k] = (double)G[k];
    FundamentalModel::denormalise(N, Gd, out);
  }
  return true;
}

}  // namespace lo32
}  // namespace gcr
