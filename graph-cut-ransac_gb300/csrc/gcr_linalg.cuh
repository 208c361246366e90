// Small dense FP64 linear algebra for per-thread use on the device.
#pragma once

#include <cuda_runtime.h>

namespace gcr {

__host__ __device__ __forceinline__ double det3(const double* m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

__host__ __device__ __forceinline__ void matmul3(const double* a, const double* b, double* c) {
  double t[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
#pragma unroll
  for (int k = 0; k < 9; ++k) c[k] = t[k];
}

__host__ __device__ __forceinline__ bool inverse3(const double* m, double* out) {
  const double c00 = m[4] * m[8] - m[5] * m[7];
  const double c01 = m[5] * m[6] - m[3] * m[8];
  const double c02 = m[3] * m[7] - m[4] * m[6];
  const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
  const double id = 1.0 / det;
  out[0] = c00 * id;
  out[1] = (m[2] * m[7] - m[1] * m[8]) * id;
  out[2] = (m[1] * m[5] - m[2] * m[4]) * id;
  out[3] = c01 * id;
  out[4] = (m[0] * m[8] - m[2] * m[6]) * id;
  out[5] = (m[2] * m[3] - m[0] * m[5]) * id;
  out[6] = c02 * id;
  out[7] = (m[1] * m[6] - m[0] * m[7]) * id;
  out[8] = (m[0] * m[4] - m[1] * m[3]) * id;
  return det != 0;
}

// Symmetric 3x3 eigen decomposition by cyclic Jacobi rotations; eigenvalues
// in descending order, eigenvectors in the columns of V (row-major). Every
// index is a compile-time constant so that the matrices stay in registers.
__device__ inline void sym3_eigen(const double* S_in, double* w, double* V) {
  double S[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) S[i] = S_in[i];
#pragma unroll
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    const double off = S[1] * S[1] + S[2] * S[2] + S[5] * S[5];
    if (off < 1e-300) break;
#pragma unroll
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0;
      const int q = pq == 0 ? 1 : 2;
      const double apq = S[p * 3 + q];
      if (!(fabs(apq) < 1e-300)) {
        const double app = S[p * 3 + p], aqq = S[q * 3 + q];
        const double theta = (aqq - app) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
        const double cs = 1 / sqrt(t * t + 1), sn = t * cs;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const double skp = S[k * 3 + p], skq = S[k * 3 + q];
          S[k * 3 + p] = cs * skp - sn * skq;
          S[k * 3 + q] = sn * skp + cs * skq;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const double spk = S[p * 3 + k], sqk = S[q * 3 + k];
          S[p * 3 + k] = cs * spk - sn * sqk;
          S[q * 3 + k] = sn * spk + cs * sqk;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const double vkp = V[k * 3 + p], vkq = V[k * 3 + q];
          V[k * 3 + p] = cs * vkp - sn * vkq;
          V[k * 3 + q] = sn * vkp + cs * vkq;
        }
      }
    }
  }
  // descending order by three compare-and-swap steps on (eigenvalue, column)
  double d[3] = {S[0], S[4], S[8]};
  auto cswap = [&](int a, int b) {
    const bool sw = d[a] < d[b];
    const double da = d[a], db = d[b];
    d[a] = sw ? db : da;
    d[b] = sw ? da : db;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double va = V[i * 3 + a], vb = V[i * 3 + b];
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

// SVD A = U diag(s) V^T of a 3x3 matrix (s descending): V from the
// eigenvectors of A^T A, U columns from A V / s, the last completed by a
// cross product with the sign that reproduces A.
__device__ inline void svd3(const double* A, double* U, double* s, double* V) {
  double AtA[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) AtA[i * 3 + j] = A[i] * A[j] + A[3 + i] * A[3 + j] + A[6 + i] * A[6 + j];
  double w[3];
  sym3_eigen(AtA, w, V);
  for (int j = 0; j < 3; ++j) s[j] = sqrt(fmax(0.0, w[j]));
  double c[3][3];
  for (int j = 0; j < 2; ++j) {
    double u[3];
    for (int i = 0; i < 3; ++i) u[i] = A[i * 3] * V[j] + A[i * 3 + 1] * V[3 + j] + A[i * 3 + 2] * V[6 + j];
    const double nrm = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (int i = 0; i < 3; ++i) c[j][i] = nrm > 0 ? u[i] / nrm : (i == j ? 1.0 : 0.0);
  }
  c[2][0] = c[0][1] * c[1][2] - c[0][2] * c[1][1];
  c[2][1] = c[0][2] * c[1][0] - c[0][0] * c[1][2];
  c[2][2] = c[0][0] * c[1][1] - c[0][1] * c[1][0];
  double u2[3];
  for (int i = 0; i < 3; ++i) u2[i] = A[i * 3] * V[2] + A[i * 3 + 1] * V[5] + A[i * 3 + 2] * V[8];
  if (u2[0] * c[2][0] + u2[1] * c[2][1] + u2[2] * c[2][2] < 0)
    for (int i = 0; i < 3; ++i) c[2][i] = -c[2][i];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) U[i * 3 + j] = c[j][i];
}

// Last column of Q of the complete-pivoting Householder QR of a 9x9 matrix
// (the 8-point solver's FullPivHouseholderQR(A^T A).matrixQ().rightCols<1>()).
// M is overwritten; Householder vectors are kept below the diagonal.
__device__ inline void fullpiv_qr_lastcol9(double* M, double* q) {
  int transp[9];
  double tau[9];
  long long biggest_all = 0;
  int steps = 9;
  for (int k = 0; k < 9; ++k) {
    int bi = k, bj = k;
    long long best = -1;
    for (int i = k; i < 9; ++i)
      for (int j = k; j < 9; ++j) {
        const long long v = __double_as_longlong(M[i * 9 + j]) & 0x7fffffffffffffffLL;
        if (v > best) { best = v; bi = i; bj = j; }
      }
    if (k == 0) biggest_all = best;
    // a negligible remaining block ends the decomposition (remaining
    // reflections are the identity)
    if (__longlong_as_double(best) <= __longlong_as_double(biggest_all) * (2.220446049250313e-16 * 9.0)) {
      steps = k;
      break;
    }
    transp[k] = bi;
    // row swap of the trailing part only: columns < k hold earlier reflectors
    if (bi != k)
      for (int j = k; j < 9; ++j) { const double t = M[k * 9 + j]; M[k * 9 + j] = M[bi * 9 + j]; M[bi * 9 + j] = t; }
    if (bj != k)
      for (int i = 0; i < 9; ++i) { const double t = M[i * 9 + k]; M[i * 9 + k] = M[i * 9 + bj]; M[i * 9 + bj] = t; }
    const double c0 = M[k * 9 + k];
    double tail = 0;
    for (int i = k + 1; i < 9; ++i) tail += M[i * 9 + k] * M[i * 9 + k];
    double t, beta;
    if (tail <= 2.2250738585072014e-308) {
      t = 0;
      beta = c0;
      for (int i = k + 1; i < 9; ++i) M[i * 9 + k] = 0;
    } else {
      beta = sqrt(c0 * c0 + tail);
      if (c0 >= 0) beta = -beta;
      const double inv = 1.0 / (c0 - beta);
      for (int i = k + 1; i < 9; ++i) M[i * 9 + k] *= inv;
      t = (beta - c0) / beta;
    }
    tau[k] = t;
    M[k * 9 + k] = beta;
    // apply H_k = I - t v v^T (v = [1; M[k+1.., k]]) to columns k+1..
    for (int j = k + 1; j < 9; ++j) {
      double s = M[k * 9 + j];
      for (int i = k + 1; i < 9; ++i) s += M[i * 9 + k] * M[i * 9 + j];
      s *= t;
      M[k * 9 + j] -= s;
      for (int i = k + 1; i < 9; ++i) M[i * 9 + j] -= s * M[i * 9 + k];
    }
  }
  for (int i = 0; i < 9; ++i) q[i] = 0;
  q[8] = 1;
  for (int k = steps - 1; k >= 0; --k) {
    double s = q[k];
    for (int i = k + 1; i < 9; ++i) s += M[i * 9 + k] * q[i];
    s *= tau[k];
    q[k] -= s;
    for (int i = k + 1; i < 9; ++i) q[i] -= s * M[i * 9 + k];
    if (transp[k] != k) { const double tt = q[k]; q[k] = q[transp[k]]; q[transp[k]] = tt; }
  }
}

// Gauss elimination of an 8x9 augmented system with the pivoting scheme of
// the reference's utils::gaussElimination<8> (src/pygcransac/include/math_utils.h:45-87):
// a bubble pre-pass that swaps rows on the diagonal column entries, then
// elimination without pivoting and back substitution.
__device__ __forceinline__ void gauss_elimination8(double a[8][9], double x[8]) {
  // every loop is unrolled so that the system stays in registers
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int k = i + 1; k < 8; k++) {
      const bool sw = fabs(a[i][i]) < fabs(a[k][i]);
#pragma unroll
      for (int j = 0; j <= 8; j++) {
        const double t = a[i][j], u = a[k][j];
        a[i][j] = sw ? u : t;
        a[k][j] = sw ? t : u;
      }
    }
#pragma unroll
  for (int i = 0; i < 7; i++)
#pragma unroll
    for (int k = i + 1; k < 8; k++) {
      const double t = a[k][i] / a[i][i];
#pragma unroll
      for (int j = 0; j <= 8; j++) a[k][j] = a[k][j] - t * a[i][j];
    }
#pragma unroll
  for (int i = 7; i >= 0; i--) {
    double s = a[i][8];
#pragma unroll
    for (int j = i + 1; j < 8; j++) s = s - a[i][j] * x[j];
    x[i] = s / a[i][i];
  }
}

// Solves the symmetric positive definite system A x = b in place (x holds b on
// entry). Returns false when A is not numerically positive definite.
template <int N>
__device__ __forceinline__ bool cholesky_solve(double A[N][N], double* x) {
  bool ok = true;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    double d = A[j][j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= A[j][k] * A[j][k];
    ok = ok && (d > 0);
    const double l = sqrt(d);
    A[j][j] = l;
    const double il = 1.0 / l;
#pragma unroll
    for (int i = j + 1; i < N; ++i) {
      double s = A[i][j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= A[i][k] * A[j][k];
      A[i][j] = s * il;
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    double s = x[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s -= A[i][k] * x[k];
    x[i] = s / A[i][i];
  }
#pragma unroll
  for (int i = N - 1; i >= 0; --i) {
    double s = x[i];
#pragma unroll
    for (int k = i + 1; k < N; ++k) s -= A[k][i] * x[k];
    x[i] = s / A[i][i];
  }
  return ok;
}

}  // namespace gcr
