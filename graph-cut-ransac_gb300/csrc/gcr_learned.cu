// Learned inlier-probability proposal: per-correspondence features, a small
// MLP (BF16 weights, FP32 accumulation) and its training kernels. The
// predicted probabilities order the correspondences for the PROSAC sampler.
//
// Features of correspondence i of a pair (kFeat = 20 values, padded to 32):
//   (x1/w1 - 0.5, y1/h1 - 0.5, x2/w2 - 0.5, y2/h2 - 0.5) and, for each of the
//   k = 8 nearest neighbours j of i in the first image (FP32 squared
//   distance, ties by index), the pair
//     (|d_j - d_i|^(1/2) / 4, |x1_j - x1_i|^(1/2) / 4)
//   with d = x2 - x1 the displacement in pixels, the k pairs ordered by the
//   first value (a missing neighbour gives (4, 4) and sorts last). Inliers of
//   a coherent motion have near neighbours that move alike; a random match
//   does not.
// Network: 32 -> 128 -> 128 -> 128 -> 1, ReLU between layers, the last output
// is a logit; the inputs of the first three layers are rounded to BF16 and
// multiplied on the tensor cores with FP32 accumulation. Parameters are kept
// as FP32 master copies (Adam) and BF16 copies used by the forward and
// backward passes.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>

#include "../../include/gcr.h"

namespace gcr {
void set_last_error(const char* msg);
}

namespace {

constexpr int kK = 8;          // neighbours
constexpr int kFeat = 20;      // real features
constexpr int kIn = 32;        // padded input width
constexpr int kH = 128;        // hidden width
constexpr int kRows = 16;      // rows (correspondences) per CTA of the MLP passes
constexpr int kTile = 128;     // query rows per CTA of the neighbour search and the ordering
constexpr int kCand = 2048;    // candidates staged in shared memory per round
constexpr double kMissing = 65536.0;  // squared length standing in for a missing neighbour (feature 4.0)
constexpr int kGridMax = 8192;      // pairs up to this size use the shared-memory grid search
constexpr int kGridMaxSide = 64;    // at most 64 x 64 cells (G^2 <= kGridMax / 2)
constexpr int kGridThreads = 256;
// parameter layout (floats): W1 [kIn][kH], b1 [kH], W2 [kH][kH], b2, W3, b3, W4 [kH], b4 [1]
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kIn * kH;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;
constexpr int kOffB3 = kOffW3 + kH * kH;
constexpr int kOffW4 = kOffB3 + kH;
constexpr int kOffB4 = kOffW4 + kH;
constexpr int kParams = kOffB4 + 1;

gcr_status fail(gcr_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  gcr::set_last_error(buf);
  return s;
}

#define CUDA_TRY(expr)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess) return fail(GCR_DEVICE_ERROR, "%s failed: %s", #expr, cudaGetErrorString(e_)); \
  } while (0)

// k nearest neighbours in registers, ascending by (squared distance, index);
// a candidate enters when it precedes the current k-th. The order is the same
// whatever the order the candidates arrive in.
struct Knn {
  float d[kK];
  int j[kK];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      d[k] = INFINITY;
      j[k] = -1;
    }
  }
  __device__ __forceinline__ void offer(float dist, int idx) {
    if (dist < d[kK - 1] || (dist == d[kK - 1] && idx < j[kK - 1])) {
      d[kK - 1] = dist;
      j[kK - 1] = idx;
#pragma unroll
      for (int k = kK - 1; k > 0; --k) {
        if (d[k] < d[k - 1] || (d[k] == d[k - 1] && j[k] < j[k - 1])) {
          const float tf = d[k];
          d[k] = d[k - 1];
          d[k - 1] = tf;
          const int ti = j[k];
          j[k] = j[k - 1];
          j[k - 1] = ti;
        }
      }
    }
  }
};

// FP32 squared distance, each operation rounded on its own (reproducible on
// any IEEE host)
__device__ __forceinline__ float sqdist(float qx, float qy, float px, float py) {
  const float ex = __fsub_rn(qx, px), ey = __fsub_rn(qy, py);
  return __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
}

// Features of row i of a pair from its neighbours (local indices, -1 missing)
__device__ void write_features(const double* corr, int64_t o0, int i, const int* nb, const gcr_image_size& z,
                               float* feat) {
  const double* p = corr + 4 * (o0 + i);
  float* f = feat + (int64_t)kIn * (o0 + i);
  f[0] = (float)(p[0] / z.w1 - 0.5);
  f[1] = (float)(p[1] / z.h1 - 0.5);
  f[2] = (float)(p[2] / z.w2 - 0.5);
  f[3] = (float)(p[3] / z.h2 - 0.5);
  // per neighbour: squared length of the displacement difference (pixels)
  // and squared first-image distance, ordered by the former (ascending,
  // stable), so the first entry is the best-agreeing neighbour; missing
  // neighbours sort last
  const double dx = p[2] - p[0], dy = p[3] - p[1];
  double dm[kK], dd[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    double mag = kMissing, dist = kMissing;
    if (nb[k] >= 0) {
      const double* q = corr + 4 * (o0 + nb[k]);
      const double a = (q[2] - q[0]) - dx, b = (q[3] - q[1]) - dy;
      const double ex = q[0] - p[0], ey = q[1] - p[1];
      mag = __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b));
      dist = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
    }
    dm[k] = mag;
    dd[k] = dist;
#pragma unroll
    for (int t = k; t > 0; --t) {
      if (dm[t] < dm[t - 1]) {
        double x = dm[t]; dm[t] = dm[t - 1]; dm[t - 1] = x;
        x = dd[t]; dd[t] = dd[t - 1]; dd[t - 1] = x;
      }
    }
  }
  // fourth roots (square roots of lengths) compress the pixel range: an
  // agreeing inlier neighbour gives about 1, a random one about 17
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    f[4 + 2 * k] = (float)(0.25 * sqrt(sqrt(dm[k])));
    f[5 + 2 * k] = (float)(0.25 * sqrt(sqrt(dd[k])));
  }
#pragma unroll
  for (int c = kFeat; c < kIn; ++c) f[c] = 0.f;
}

// Features of the pairs with more than kGridMax correspondences: grid (tile of
// kTile rows, pair). Each thread holds one query; the pair's first-image
// points stream through shared memory in rounds of kCand.
__global__ void __launch_bounds__(kTile) features_scan_kernel(const double* corr, const int64_t* offsets,
                                                              const gcr_image_size* sizes, float* feat) {
  __shared__ float2 cand[kCand];
  const int pair = blockIdx.y;
  const int64_t o0 = offsets[pair];
  const int n = (int)(offsets[pair + 1] - o0);
  if (n <= kGridMax || (int)blockIdx.x * kTile >= n) return;  // uniform over the CTA
  const int i = (int)blockIdx.x * kTile + threadIdx.x;
  const bool active = i < n;
  float px = 0.f, py = 0.f;
  if (active) {
    px = (float)corr[4 * (o0 + i)];
    py = (float)corr[4 * (o0 + i) + 1];
  }
  Knn nn;
  nn.init();
  for (int c0 = 0; c0 < n; c0 += kCand) {
    const int m = min(kCand, n - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < m; t += kTile) {
      const double* q = corr + 4 * (o0 + c0 + t);
      cand[t] = make_float2((float)q[0], (float)q[1]);
    }
    __syncthreads();
    if (!active) continue;
    for (int t = 0; t < m; ++t)
      if (c0 + t != i) nn.offer(sqdist(cand[t].x, cand[t].y, px, py), c0 + t);
  }
  if (active) write_features(corr, o0, i, nn.j, sizes[pair], feat);
}

// Features of the pairs with at most kGridMax correspondences: one CTA per
// pair. The first-image points are bucketed into a G x G grid over their
// bounding box (G^2 about n / 2 cells) by a counting sort in shared memory;
// each query then visits rings of cells around its own until its k-th
// distance lies below the distance to every unvisited cell (with a margin of
// 1e-3 cell for the rounding of cell boundaries). Exact: the same neighbours
// as the all-pairs scan.
__host__ __device__ constexpr size_t grid_smem_bytes(int max_n) {
  return sizeof(float2) * (size_t)max_n + sizeof(int) * (size_t)max_n + 2 * sizeof(int) * (size_t)(max_n / 2 + 2);
}

__global__ void __launch_bounds__(kGridThreads) features_grid_kernel(const double* corr, const int64_t* offsets,
                                                                     const gcr_image_size* sizes, float* feat) {
  extern __shared__ __align__(16) unsigned char gsm[];
  __shared__ float bbox[4];
  __shared__ float red[4][kGridThreads / 32];
  const int pair = blockIdx.x;
  const int64_t o0 = offsets[pair];
  const int n = (int)(offsets[pair + 1] - o0);
  if (n > kGridMax || n <= 0) return;  // uniform over the CTA
  float2* pts = reinterpret_cast<float2*>(gsm);
  int* sorted = reinterpret_cast<int*>(pts + n);
  const int G = max(1, min(kGridMaxSide, (int)sqrtf(0.5f * (float)n)));
  const int cells = G * G;
  int* start = sorted + n;        // [cells + 1]
  int* cursor = start + cells + 1;  // [cells]
  float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
  for (int i = threadIdx.x; i < n; i += kGridThreads) {
    const double* q = corr + 4 * (o0 + i);
    const float2 v = make_float2((float)q[0], (float)q[1]);
    pts[i] = v;
    mnx = fminf(mnx, v.x);
    mny = fminf(mny, v.y);
    mxx = fmaxf(mxx, v.x);
    mxy = fmaxf(mxy, v.y);
  }
  for (int c = threadIdx.x; c < cells; c += kGridThreads) cursor[c] = 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = mnx;
    red[1][warp] = mny;
    red[2][warp] = mxx;
    red[3][warp] = mxy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = INFINITY, b = INFINITY, c = -INFINITY, d = -INFINITY;
    for (int w = 0; w < kGridThreads / 32; ++w) {
      a = fminf(a, red[0][w]);
      b = fminf(b, red[1][w]);
      c = fmaxf(c, red[2][w]);
      d = fmaxf(d, red[3][w]);
    }
    bbox[0] = a;
    bbox[1] = b;
    bbox[2] = (c - a) > 0.f ? (c - a) / (float)G : 1.f;  // cell width
    bbox[3] = (d - b) > 0.f ? (d - b) / (float)G : 1.f;  // cell height
  }
  __syncthreads();
  const float x0 = bbox[0], y0 = bbox[1], cw = bbox[2], ch = bbox[3];
  auto cell_of = [&](float2 v, int& cx, int& cy) {
    cx = min(G - 1, max(0, (int)((v.x - x0) / cw)));
    cy = min(G - 1, max(0, (int)((v.y - y0) / ch)));
  };
  for (int i = threadIdx.x; i < n; i += kGridThreads) {
    int cx, cy;
    cell_of(pts[i], cx, cy);
    atomicAdd(&cursor[cy * G + cx], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int c = 0; c < cells; ++c) {
      start[c] = acc;
      acc += cursor[c];
      cursor[c] = start[c];
    }
    start[cells] = acc;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += kGridThreads) {
    int cx, cy;
    cell_of(pts[i], cx, cy);
    sorted[atomicAdd(&cursor[cy * G + cx], 1)] = i;
  }
  __syncthreads();
  const float mx = 1e-3f * cw, my = 1e-3f * ch;
  for (int i = threadIdx.x; i < n; i += kGridThreads) {
    const float2 q = pts[i];
    int cx, cy;
    cell_of(q, cx, cy);
    Knn nn;
    nn.init();
    for (int r = 0;; ++r) {
      for (int dy = -r; dy <= r; ++dy) {
        const int y = cy + dy;
        if (y < 0 || y >= G) continue;
        const int step = (dy == -r || dy == r) ? 1 : 2 * r;
        for (int dx = -r; dx <= r; dx += max(step, 1)) {
          const int x = cx + dx;
          if (x < 0 || x >= G) continue;
          const int c = y * G + x;
          for (int s = start[c]; s < start[c + 1]; ++s) {
            const int j = sorted[s];
            if (j != i) nn.offer(sqdist(pts[j].x, pts[j].y, q.x, q.y), j);
          }
        }
      }
      // distance to the nearest unvisited cell (sides still inside the grid)
      float lb = INFINITY;
      if (cx - r > 0) lb = fminf(lb, q.x - (x0 + (float)(cx - r) * cw) - mx);
      if (cx + r < G - 1) lb = fminf(lb, (x0 + (float)(cx + r + 1) * cw) - q.x - mx);
      if (cy - r > 0) lb = fminf(lb, q.y - (y0 + (float)(cy - r) * ch) - my);
      if (cy + r < G - 1) lb = fminf(lb, (y0 + (float)(cy + r + 1) * ch) - q.y - my);
      if (lb == INFINITY) break;  // the rings cover the grid
      if (lb > 0.f && nn.d[kK - 1] < lb * lb) break;
    }
    write_features(corr, o0, i, nn.j, sizes[pair], feat);
  }
}

__device__ __forceinline__ float bf(const __nv_bfloat16* w, int i) { return __bfloat162float(w[i]); }

__device__ __forceinline__ float4 bf4(const __nv_bfloat16* w, int i) {
  const uint2 u = *reinterpret_cast<const uint2*>(w + i);
  const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.x));
  const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.y));
  return make_float4(a.x, a.y, b.x, b.y);
}

// ---- Forward pass on the tensor cores: mma.sync m16n8k16, BF16 x BF16 ->
// FP32. Each warp owns 16 rows; a layer is 16 n-tiles of 8 columns x K/16
// k-steps. The FP32 accumulator fragment of n-tiles (2j, 2j+1) has exactly
// the layout of the next layer's A fragment for k-step j (rows g and g + 8,
// columns 2t, 2t + 1 and 8 + 2t, 9 + 2t of the 16), so activations stay in
// registers between layers: bias, ReLU, rounding to BF16, next layer. The
// weights sit in shared memory transposed ([n][k], rows padded by 8 so the
// warp's B-fragment loads hit 32 distinct banks) and are loaded once per
// persistent CTA. The output layer (128 -> 1) is an FP32 dot product of the
// third layer's FP32 activations, reduced over the four lanes of each row.
// Activations: layer inputs are rounded to BF16 (the features included); A1
// and A2 are stored rounded (what the next layer read), A3 in FP32.
constexpr int kMmaWarps = 4;
constexpr int kTileRows = 16 * kMmaWarps;
constexpr int kLd1 = kIn + 8;
constexpr int kLdH = kH + 8;
constexpr size_t kForwardSmem =
    sizeof(__nv_bfloat16) * (size_t)(kH * kLd1 + 2 * kH * kLdH) + sizeof(float) * (size_t)(4 * kH + 4);

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ float round_bf16(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// c = bias + A W for one warp's 16 rows; Wt is [kH][ld] (n-major), K the layer width
template <int K>
__device__ __forceinline__ void mma_layer(const uint32_t (&a)[K / 16][4], const __nv_bfloat16* Wt, int ld,
                                          const float* bias, float (&c)[kH / 8][4], int g, int t) {
#pragma unroll
  for (int nt = 0; nt < kH / 8; ++nt) {
    const float b0 = bias[8 * nt + 2 * t], b1 = bias[8 * nt + 2 * t + 1];
    c[nt][0] = b0;
    c[nt][1] = b1;
    c[nt][2] = b0;
    c[nt][3] = b1;
    const __nv_bfloat16* w = Wt + (8 * nt + g) * ld + 2 * t;
#pragma unroll
    for (int ks = 0; ks < K / 16; ++ks) {
      const uint32_t w0 = *reinterpret_cast<const uint32_t*>(w + 16 * ks);
      const uint32_t w1 = *reinterpret_cast<const uint32_t*>(w + 16 * ks + 8);
      mma_bf16(c[nt], a[ks], w0, w1);
    }
  }
}

// ReLU of the accumulators, packed as the next layer's A fragments; the
// rounded activations are stored to out (when not NULL) for rows ra, rb
__device__ __forceinline__ void relu_pack(float (&c)[kH / 8][4], uint32_t (&a)[kH / 16][4], float* out, int64_t ra,
                                          int64_t rb, int64_t n, int t) {
#pragma unroll
  for (int nt = 0; nt < kH / 8; ++nt) {
#pragma unroll
    for (int q = 0; q < 4; ++q) c[nt][q] = round_bf16(fmaxf(c[nt][q], 0.f));
    if (out) {
      const int col = 8 * nt + 2 * t;
      if (ra < n) *reinterpret_cast<float2*>(out + ra * kH + col) = make_float2(c[nt][0], c[nt][1]);
      if (rb < n) *reinterpret_cast<float2*>(out + rb * kH + col) = make_float2(c[nt][2], c[nt][3]);
    }
  }
#pragma unroll
  for (int j = 0; j < kH / 16; ++j) {
    a[j][0] = pack_bf16(c[2 * j][0], c[2 * j][1]);
    a[j][1] = pack_bf16(c[2 * j][2], c[2 * j][3]);
    a[j][2] = pack_bf16(c[2 * j + 1][0], c[2 * j + 1][1]);
    a[j][3] = pack_bf16(c[2 * j + 1][2], c[2 * j + 1][3]);
  }
}

__global__ void __launch_bounds__(32 * kMmaWarps, 2) forward_kernel(const float* feat, int64_t n,
                                                                    const __nv_bfloat16* P, float* A1, float* A2,
                                                                    float* A3, float* logits) {
  extern __shared__ __align__(16) unsigned char fsm[];
  __nv_bfloat16* W1t = reinterpret_cast<__nv_bfloat16*>(fsm);
  __nv_bfloat16* W2t = W1t + kH * kLd1;
  __nv_bfloat16* W3t = W2t + kH * kLdH;
  float* vec = reinterpret_cast<float*>(W3t + kH * kLdH);  // b1, b2, b3, w4, b4
  for (int i = threadIdx.x; i < kIn * kH; i += blockDim.x) W1t[(i % kH) * kLd1 + i / kH] = P[kOffW1 + i];
  for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) {
    W2t[(i % kH) * kLdH + i / kH] = P[kOffW2 + i];
    W3t[(i % kH) * kLdH + i / kH] = P[kOffW3 + i];
  }
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    vec[i] = __bfloat162float(P[kOffB1 + i]);
    vec[kH + i] = __bfloat162float(P[kOffB2 + i]);
    vec[2 * kH + i] = __bfloat162float(P[kOffB3 + i]);
    vec[3 * kH + i] = __bfloat162float(P[kOffW4 + i]);
  }
  if (threadIdx.x == 0) vec[4 * kH] = __bfloat162float(P[kOffB4]);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int64_t tiles = (n + kTileRows - 1) / kTileRows;
  for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int64_t ra = tile * kTileRows + 16 * warp + g, rb = ra + 8;
    uint32_t a1[kIn / 16][4];
#pragma unroll
    for (int ks = 0; ks < kIn / 16; ++ks) {
      const int c0 = 16 * ks + 2 * t;
      float2 x00 = make_float2(0.f, 0.f), x01 = x00, x10 = x00, x11 = x00;
      if (ra < n) {
        x00 = *reinterpret_cast<const float2*>(feat + ra * kIn + c0);
        x01 = *reinterpret_cast<const float2*>(feat + ra * kIn + c0 + 8);
      }
      if (rb < n) {
        x10 = *reinterpret_cast<const float2*>(feat + rb * kIn + c0);
        x11 = *reinterpret_cast<const float2*>(feat + rb * kIn + c0 + 8);
      }
      a1[ks][0] = pack_bf16(x00.x, x00.y);
      a1[ks][1] = pack_bf16(x10.x, x10.y);
      a1[ks][2] = pack_bf16(x01.x, x01.y);
      a1[ks][3] = pack_bf16(x11.x, x11.y);
    }
    float c[kH / 8][4];
    uint32_t a[kH / 16][4];
    mma_layer<kIn>(a1, W1t, kLd1, vec, c, g, t);
    relu_pack(c, a, A1, ra, rb, n, t);
    mma_layer<kH>(a, W2t, kLdH, vec + kH, c, g, t);
    relu_pack(c, a, A2, ra, rb, n, t);
    mma_layer<kH>(a, W3t, kLdH, vec + 2 * kH, c, g, t);
    float sa = 0.f, sb = 0.f;
#pragma unroll
    for (int nt = 0; nt < kH / 8; ++nt) {
      const int col = 8 * nt + 2 * t;
      const float h0 = fmaxf(c[nt][0], 0.f), h1 = fmaxf(c[nt][1], 0.f);
      const float h2 = fmaxf(c[nt][2], 0.f), h3 = fmaxf(c[nt][3], 0.f);
      sa = fmaf(h0, vec[3 * kH + col], fmaf(h1, vec[3 * kH + col + 1], sa));
      sb = fmaf(h2, vec[3 * kH + col], fmaf(h3, vec[3 * kH + col + 1], sb));
      if (A3) {
        if (ra < n) *reinterpret_cast<float2*>(A3 + ra * kH + col) = make_float2(h0, h1);
        if (rb < n) *reinterpret_cast<float2*>(A3 + rb * kH + col) = make_float2(h2, h3);
      }
    }
    sa += __shfl_xor_sync(0xffffffffu, sa, 1);
    sa += __shfl_xor_sync(0xffffffffu, sa, 2);
    sb += __shfl_xor_sync(0xffffffffu, sb, 1);
    sb += __shfl_xor_sync(0xffffffffu, sb, 2);
    if (t == 0) {
      if (ra < n) logits[ra] = sa + vec[4 * kH];
      if (rb < n) logits[rb] = sb + vec[4 * kH];
    }
  }
}

// Backward pass of the weighted binary cross-entropy with logits,
// loss = sum_i w_i [max(z,0) - z y + log(1 + exp(-|z|))] / sum_i w_i.
// Persistent: each CTA walks chunks of kRows rows and accumulates the
// parameter gradient in shared memory (thread j owns column j of every weight
// matrix, so the accumulation needs no atomics); at the end each CTA adds its
// partial gradient to G once.
constexpr int kParamsPad = (kParams + 3) & ~3;
constexpr size_t kBackwardSmem = sizeof(float) * (kParamsPad + 2 * kRows * kH + kRows);

__global__ void __launch_bounds__(kH) backward_kernel(const float* feat, int64_t n, const __nv_bfloat16* P,
                                                      const float* A1, const float* A2, const float* A3,
                                                      const float* logits, const float* labels,
                                                      const float* weights, float inv_wsum, float* G) {
  extern __shared__ __align__(16) float smem[];
  float* acc = smem;                // kParamsPad, parameter layout
  float* dz = acc + kParamsPad;     // [kRows][kH] gradient w.r.t. the current pre-activation
  float* act = dz + kRows * kH;     // [kRows][width] the current layer's input
  float* g4 = act + kRows * kH;     // [kRows] gradient w.r.t. the logits
  const int j = threadIdx.x;
  for (int t = j; t < kParamsPad; t += kH) acc[t] = 0.f;
  const int64_t chunks = (n + kRows - 1) / kRows;
  const float* prevs[3] = {A2, A1, feat};
  const int widths[3] = {kH, kH, kIn};
  const int offW[3] = {kOffW3, kOffW2, kOffW1};
  const int offB[3] = {kOffB3, kOffB2, kOffB1};
  for (int64_t chunk = blockIdx.x; chunk < chunks; chunk += gridDim.x) {
    const int64_t r0 = chunk * kRows;
    const int rows = (int)min((int64_t)kRows, n - r0);
    __syncthreads();
    if (j < kRows) {
      float g = 0.f;
      if (j < rows) {
        const float z = logits[r0 + j];
        const float s = 1.f / (1.f + expf(-z));
        g = (s - labels[r0 + j]) * weights[r0 + j] * inv_wsum;
      }
      g4[j] = g;
    }
    for (int t = j; t < kRows * kH; t += kH) act[t] = t / kH < rows ? A3[r0 * kH + t] : 0.f;
    __syncthreads();
    // layer 4: dW4[k] = sum_r A3[r][k] g4[r], db4 = sum_r g4[r], dz3 = g4 W4^T relu'(A3)
    {
      float s = 0.f;
#pragma unroll
      for (int r = 0; r < kRows; ++r) s = fmaf(act[r * kH + j], g4[r], s);
      acc[kOffW4 + j] += s;
      if (j == 0) {
        float sb = 0.f;
        for (int r = 0; r < kRows; ++r) sb += g4[r];
        acc[kOffB4] += sb;
      }
      const float w4 = bf(P, kOffW4 + j);
#pragma unroll
      for (int r = 0; r < kRows; ++r) dz[r * kH + j] = act[r * kH + j] > 0.f ? g4[r] * w4 : 0.f;
    }
    // layers 3, 2, 1: dW[k][j] += sum_r in[r][k] dz[r][j], db[j] += sum_r dz[r][j],
    // then dz_prev[r][k] = (sum_j dz[r][j] W[k][j]) relu'(in[r][k])
#pragma unroll
    for (int L = 0; L < 3; ++L) {
      const int width = widths[L];
      __syncthreads();
      // the first layer read the features rounded to BF16
      for (int t = j; t < kRows * width; t += kH)
        act[t] = t / width < rows ? (L == 2 ? round_bf16(prevs[L][r0 * width + t]) : prevs[L][r0 * width + t]) : 0.f;
      __syncthreads();
      float dzr[kRows];
      float sb = 0.f;
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        dzr[r] = dz[r * kH + j];
        sb += dzr[r];
      }
      acc[offB[L] + j] += sb;
      float* aw = acc + offW[L];
      for (int k = 0; k < width; k += 4) {
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
          const float4 a = *reinterpret_cast<const float4*>(act + r * width + k);
          s0 = fmaf(a.x, dzr[r], s0);
          s1 = fmaf(a.y, dzr[r], s1);
          s2 = fmaf(a.z, dzr[r], s2);
          s3 = fmaf(a.w, dzr[r], s3);
        }
        aw[k * kH + j] += s0;
        aw[(k + 1) * kH + j] += s1;
        aw[(k + 2) * kH + j] += s2;
        aw[(k + 3) * kH + j] += s3;
      }
      if (L < 2) {
        const __nv_bfloat16* W = P + offW[L];
        float dp[kRows];
#pragma unroll
        for (int r = 0; r < kRows; ++r) dp[r] = 0.f;
        for (int c = 0; c < kH; c += 4) {
          const float4 w = bf4(W, j * kH + c);
#pragma unroll
          for (int r = 0; r < kRows; ++r) {
            const float4 d = *reinterpret_cast<const float4*>(dz + r * kH + c);
            dp[r] = fmaf(d.x, w.x, dp[r]);
            dp[r] = fmaf(d.y, w.y, dp[r]);
            dp[r] = fmaf(d.z, w.z, dp[r]);
            dp[r] = fmaf(d.w, w.w, dp[r]);
          }
        }
        __syncthreads();  // every thread has read dz
#pragma unroll
        for (int r = 0; r < kRows; ++r) dz[r * kH + j] = act[r * kH + j] > 0.f ? dp[r] : 0.f;
      }
    }
  }
  __syncthreads();
  for (int t = j; t < kParams; t += kH)
    if (acc[t] != 0.f) atomicAdd(G + t, acc[t]);
}

// Descending order of the logits within each pair (ties by index, NaN last),
// for pairs of more than kGridMax rows: grid (tile of kTile rows, pair). Row i's rank is the number of rows of its
// pair that precede it; the row is copied to that position of the sorted
// correspondences and its local index recorded in perm.
__device__ __forceinline__ float order_key(float z) { return isnan(z) ? -INFINITY : z; }

__global__ void __launch_bounds__(kTile) order_kernel(const double* corr, const int64_t* offsets, const float* logits,
                                                      double* sorted, int* perm) {
  __shared__ float cz[kCand];
  const int pair = blockIdx.y;
  const int64_t o0 = offsets[pair];
  const int n = (int)(offsets[pair + 1] - o0);
  if (n <= kGridMax || (int)blockIdx.x * kTile >= n) return;  // uniform over the CTA
  const int i = (int)blockIdx.x * kTile + threadIdx.x;
  const bool active = i < n;
  const float zi = active ? order_key(logits[o0 + i]) : 0.f;
  int rank = 0;
  for (int c0 = 0; c0 < n; c0 += kCand) {
    const int m = min(kCand, n - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < m; t += kTile) cz[t] = order_key(logits[o0 + c0 + t]);
    __syncthreads();
    if (!active) continue;
    for (int t = 0; t < m; ++t) {
      const float zt = cz[t];
      rank += (zt > zi) | ((zt == zi) & (c0 + t < i));
    }
  }
  if (!active) return;
  const int64_t dst = o0 + rank;
  const double4_32a v = *reinterpret_cast<const double4_32a*>(corr + 4 * (o0 + i));
  *reinterpret_cast<double4_32a*>(sorted + 4 * dst) = v;
  perm[dst] = i;
}

// The same order for pairs of at most kGridMax rows: one CTA per pair sorts
// 64-bit keys (the logit mapped to an unsigned integer whose ascending order
// is the logits' descending order, NaN last and -0 equal to +0, then the row)
// with a bitonic network in shared memory.
__device__ __forceinline__ uint64_t order_key64(float z, int i) {
  float k = order_key(z);
  if (k == 0.f) k = 0.f;  // -0 sorts with +0
  const uint32_t u = __float_as_uint(-k);
  const uint32_t asc = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  return ((uint64_t)asc << 32) | (uint32_t)i;
}

constexpr int kSortThreads = 512;

__global__ void __launch_bounds__(kSortThreads) order_sort_kernel(const double* corr, const int64_t* offsets,
                                                                  const float* logits, double* sorted, int* perm) {
  extern __shared__ __align__(16) unsigned long long keys[];
  const int pair = blockIdx.x;
  const int64_t o0 = offsets[pair];
  const int n = (int)(offsets[pair + 1] - o0);
  if (n > kGridMax || n <= 0) return;  // uniform over the CTA
  int npad = 1;
  while (npad < n) npad <<= 1;
  for (int i = threadIdx.x; i < npad; i += kSortThreads)
    keys[i] = i < n ? order_key64(logits[o0 + i], i) : ~0ull;
  __syncthreads();
  for (int k = 2; k <= npad; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < npad; i += kSortThreads) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long a = keys[i], b = keys[l];
          if ((a > b) == ((i & k) == 0)) {
            keys[i] = b;
            keys[l] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int s = threadIdx.x; s < n; s += kSortThreads) {
    const int i = (int)(keys[s] & 0xffffffffull);
    const double4_32a v = *reinterpret_cast<const double4_32a*>(corr + 4 * (o0 + i));
    *reinterpret_cast<double4_32a*>(sorted + 4 * (o0 + s)) = v;
    perm[o0 + s] = i;
  }
}

// mask[offsets[pair] + perm[r]] = sorted_mask[r]
__global__ void unpermute_kernel(const uint8_t* sorted_mask, const int* perm, const int64_t* offsets,
                                 const int* pair_of_row, int64_t total, uint8_t* mask) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= total) return;
  mask[offsets[pair_of_row[r]] + perm[r]] = sorted_mask[r];
}

// Adam step on the FP32 master parameters; refreshes the BF16 copies.
__global__ void adam_kernel(float* M, float* V, float* Pm, __nv_bfloat16* P, const float* G, int count, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float g = G[i];
  const float m = b1 * M[i] + (1.f - b1) * g;
  const float v = b2 * V[i] + (1.f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  const float p = Pm[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
  Pm[i] = p;
  P[i] = __float2bfloat16(p);
}

__global__ void to_bf16_kernel(const float* Pm, __nv_bfloat16* P, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) P[i] = __float2bfloat16(Pm[i]);
}

}  // namespace

extern "C" {

int64_t gcr_learned_param_count(void) { return kParams; }
int32_t gcr_learned_feature_width(void) { return kIn; }

static gcr_status check_pairs(int64_t num_pairs, int64_t max_n) {
  if (num_pairs < 0 || num_pairs > 65535) return fail(GCR_INVALID_ARG, "num_pairs %lld outside [0, 65535]", (long long)num_pairs);
  if (max_n < 0 || max_n > (int64_t)1 << 30) return fail(GCR_INVALID_ARG, "max_n %lld outside [0, 2^30]", (long long)max_n);
  return GCR_OK;
}

gcr_status gcr_learned_features(const double* d_corr, const int64_t* d_offsets, const gcr_image_size* d_sizes,
                                int64_t num_pairs, int64_t max_n, float* d_feat, void* stream) {
  if (!d_corr || !d_offsets || !d_sizes || !d_feat) return fail(GCR_INVALID_ARG, "NULL buffer");
  const gcr_status st = check_pairs(num_pairs, max_n);
  if (st != GCR_OK) return st;
  if (num_pairs == 0 || max_n == 0) return GCR_OK;
  const int small_n = (int)(max_n < kGridMax ? max_n : kGridMax);
  const size_t smem = grid_smem_bytes(small_n);
  CUDA_TRY(cudaFuncSetAttribute(features_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  features_grid_kernel<<<(unsigned)num_pairs, kGridThreads, smem, (cudaStream_t)stream>>>(d_corr, d_offsets,
                                                                                            d_sizes, d_feat);
  CUDA_TRY(cudaGetLastError());
  if (max_n > kGridMax) {
    const dim3 grid((unsigned)((max_n + kTile - 1) / kTile), (unsigned)num_pairs);
    features_scan_kernel<<<grid, kTile, 0, (cudaStream_t)stream>>>(d_corr, d_offsets, d_sizes, d_feat);
    CUDA_TRY(cudaGetLastError());
  }
  return GCR_OK;
}

gcr_status gcr_learned_params_to_bf16(const float* d_master, void* d_bf16, void* stream) {
  if (!d_master || !d_bf16) return fail(GCR_INVALID_ARG, "NULL buffer");
  to_bf16_kernel<<<(kParams + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_master, (__nv_bfloat16*)d_bf16, kParams);
  CUDA_TRY(cudaGetLastError());
  return GCR_OK;
}

gcr_status gcr_learned_forward(const float* d_feat, int64_t n, const void* d_bf16, float* d_a1, float* d_a2,
                               float* d_a3, float* d_logits, void* stream) {
  if (!d_feat || !d_bf16 || !d_logits) return fail(GCR_INVALID_ARG, "NULL buffer");
  if (n <= 0) return GCR_OK;
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CUDA_TRY(cudaFuncSetAttribute(forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kForwardSmem));
  const int64_t tiles = (n + kTileRows - 1) / kTileRows;
  const unsigned grid = (unsigned)(tiles < 2 * sms ? tiles : 2 * sms);
  forward_kernel<<<grid, 32 * kMmaWarps, kForwardSmem, (cudaStream_t)stream>>>(
      d_feat, n, (const __nv_bfloat16*)d_bf16, d_a1, d_a2, d_a3, d_logits);
  CUDA_TRY(cudaGetLastError());
  return GCR_OK;
}

gcr_status gcr_learned_backward(const float* d_feat, int64_t n, const void* d_bf16, const float* d_a1,
                                const float* d_a2, const float* d_a3, const float* d_logits, const float* d_labels,
                                const float* d_weights, float inv_weight_sum, float* d_grad, void* stream) {
  if (!d_feat || !d_bf16 || !d_a1 || !d_a2 || !d_a3 || !d_logits || !d_labels || !d_weights || !d_grad)
    return fail(GCR_INVALID_ARG, "NULL buffer");
  if (n <= 0) return GCR_OK;
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CUDA_TRY(cudaFuncSetAttribute(backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBackwardSmem));
  const int64_t chunks = (n + kRows - 1) / kRows;
  const unsigned grid = (unsigned)(chunks < sms ? chunks : sms);
  backward_kernel<<<grid, kH, kBackwardSmem, (cudaStream_t)stream>>>(
      d_feat, n, (const __nv_bfloat16*)d_bf16, d_a1, d_a2, d_a3, d_logits, d_labels, d_weights, inv_weight_sum,
      d_grad);
  CUDA_TRY(cudaGetLastError());
  return GCR_OK;
}

gcr_status gcr_learned_adam(float* d_m, float* d_v, float* d_master, void* d_bf16, const float* d_grad, float lr,
                            int64_t step, void* stream) {
  if (!d_m || !d_v || !d_master || !d_bf16 || !d_grad) return fail(GCR_INVALID_ARG, "NULL buffer");
  if (step < 1) return fail(GCR_INVALID_ARG, "Adam step counts from 1");
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<(kParams + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_m, d_v, d_master, (__nv_bfloat16*)d_bf16,
                                                                      d_grad, kParams, lr, b1, b2, eps, c1, c2);
  CUDA_TRY(cudaGetLastError());
  return GCR_OK;
}

gcr_status gcr_learned_order(const double* d_corr, const int64_t* d_offsets, int64_t num_pairs, int64_t max_n,
                             const float* d_logits, double* d_sorted_corr, int32_t* d_perm, void* stream) {
  if (!d_corr || !d_offsets || !d_logits || !d_sorted_corr || !d_perm) return fail(GCR_INVALID_ARG, "NULL buffer");
  if (((uintptr_t)d_corr | (uintptr_t)d_sorted_corr) & 31)
    return fail(GCR_INVALID_ARG, "correspondence buffers must be 32-byte aligned");
  const gcr_status st = check_pairs(num_pairs, max_n);
  if (st != GCR_OK) return st;
  if (num_pairs == 0 || max_n == 0) return GCR_OK;
  int npad = 1;
  while (npad < (max_n < kGridMax ? max_n : kGridMax)) npad <<= 1;
  const size_t smem = sizeof(unsigned long long) * (size_t)npad;
  CUDA_TRY(cudaFuncSetAttribute(order_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  order_sort_kernel<<<(unsigned)num_pairs, kSortThreads, smem, (cudaStream_t)stream>>>(d_corr, d_offsets, d_logits,
                                                                                       d_sorted_corr, d_perm);
  CUDA_TRY(cudaGetLastError());
  if (max_n > kGridMax) {
    const dim3 grid((unsigned)((max_n + kTile - 1) / kTile), (unsigned)num_pairs);
    order_kernel<<<grid, kTile, 0, (cudaStream_t)stream>>>(d_corr, d_offsets, d_logits, d_sorted_corr, d_perm);
    CUDA_TRY(cudaGetLastError());
  }
  return GCR_OK;
}

gcr_status gcr_learned_propose(const double* d_corr, const int64_t* d_offsets, const gcr_image_size* d_sizes,
                               int64_t num_pairs, int64_t max_n, int64_t total, const void* d_bf16, float* d_feat,
                               float* d_logits, double* d_sorted_corr, int32_t* d_perm, void* stream) {
  gcr_status st = gcr_learned_features(d_corr, d_offsets, d_sizes, num_pairs, max_n, d_feat, stream);
  if (st == GCR_OK) st = gcr_learned_forward(d_feat, total, d_bf16, nullptr, nullptr, nullptr, d_logits, stream);
  if (st == GCR_OK) st = gcr_learned_order(d_corr, d_offsets, num_pairs, max_n, d_logits, d_sorted_corr, d_perm, stream);
  return st;
}

gcr_status gcr_learned_unpermute_mask(const uint8_t* d_sorted_mask, const int32_t* d_perm, const int64_t* d_offsets,
                                      const int32_t* d_pair_of_row, int64_t total, uint8_t* d_mask, void* stream) {
  if (!d_sorted_mask || !d_perm || !d_offsets || !d_pair_of_row || !d_mask) return fail(GCR_INVALID_ARG, "NULL buffer");
  if (total <= 0) return GCR_OK;
  unpermute_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_sorted_mask, d_perm, d_offsets,
                                                                                    d_pair_of_row, total, d_mask);
  CUDA_TRY(cudaGetLastError());
  return GCR_OK;
}

}  // extern "C"
