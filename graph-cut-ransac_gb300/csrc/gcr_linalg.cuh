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
