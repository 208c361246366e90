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

// ---- Forward pass on the fifth-generation tensor cores (tcgen05) ----------
// A persistent CTA of four warps takes tiles of 128 rows (correspondences).
// Each layer is one chain of K/16 tcgen05.mma instructions (kind::f16: BF16
// operands read from shared memory through matrix descriptors, M = N = 128,
// FP32 accumulator in tensor memory), issued by one thread; its completion
// arrives on an mbarrier through tcgen05.commit. The epilogue reads the
// accumulator back with tcgen05.ld (thread i of warp w owns TMEM lane
// 32w + i, which holds row 32w + i of the tile), adds the bias, applies ReLU,
// rounds to BF16 and writes the next layer's A operand into shared memory.
// The output layer (128 -> 1) is each thread's FP32 dot product over its row.
// Activations: layer inputs are rounded to BF16 (the features included); A1
// and A2 are stored rounded (what the next layer read), A3 in FP32.
//
// Operand layout in shared memory: no swizzle, K-major, 8 x 8 BF16 core
// matrices of 128 contiguous bytes (8 rows x 16 bytes). For an operand of
// 128 rows (the activations' M or the weights' N), element (row, k) sits at
// (k / 8) * 2048 + (row / 8) * 128 + (row % 8) * 16 + (k % 8) * 2: the
// descriptors' leading byte offset (next core matrix along K) is 2048 and the
// stride byte offset (next group of 8 rows) is 128. Weights are stored as
// W^T ([n][k]); the features' 32 columns use the first 8 KB of the
// activation buffer in the same layout.
constexpr int kUmmaRows = 128;  // rows per tile = MMA M = TMEM lanes
constexpr int kUmmaThreads = 128;
constexpr uint32_t kUmmaLbo = 2048, kUmmaSbo = 128;
constexpr uint32_t kTmemCols = 128;  // one FP32 accumulator of 128 x 128
constexpr size_t kSmW1 = 0;
constexpr size_t kSmW2 = kSmW1 + sizeof(__nv_bfloat16) * kH * kIn;
constexpr size_t kSmW3 = kSmW2 + sizeof(__nv_bfloat16) * kH * kH;
constexpr size_t kSmAct = kSmW3 + sizeof(__nv_bfloat16) * kH * kH;
constexpr size_t kSmVec = kSmAct + sizeof(__nv_bfloat16) * kUmmaRows * kH;
constexpr size_t kSmBar = kSmVec + ((sizeof(float) * (4 * kH + 1) + 15) & ~size_t(15));
constexpr size_t kForwardSmem = kSmBar + 16;  // mbarrier + TMEM address
// instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N / 8 at bit 17,
// M / 16 at bit 24
constexpr uint32_t kUmmaIdesc =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kH >> 3) << 17) | ((uint32_t)(kUmmaRows >> 4) << 24);

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ float round_bf16(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// byte offset of element (row, k) of a 128-row operand (layout above)
__device__ __forceinline__ uint32_t core_offset(int row, int k) {
  return (uint32_t)((k >> 3) * kUmmaLbo + (row >> 3) * kUmmaSbo + (row & 7) * 16 + (k & 7) * 2);
}
// shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all >> 4), descriptor version 1 at bit 46, no swizzle (bits 61-63)
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(kUmmaLbo >> 4) << 16) |
         ((uint64_t)(kUmmaSbo >> 4) << 32) | (1ull << 46);
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(tmem_d), "l"(a), "l"(b), "r"(kUmmaIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// orders this thread's generic-proxy writes of shared memory before the
// tensor cores' (async-proxy) reads
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_init1(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// waits for the phase of the given parity with a bounded number of polls
__device__ __forceinline__ bool mbar_wait_parity(unsigned long long* bar, unsigned parity) {
  constexpr int kPolls = 1 << 22;
  for (int it = 0; it < kPolls; ++it) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
// 32 consecutive FP32 accumulator columns of this thread's TMEM lane; the
// wait for the load is part of the same statement, so no use of the
// registers can move before it
__device__ __forceinline__ void tmem_load32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// One layer: the A operand (this tile's activations) and B (the layer's W^T)
// in shared memory, K / 16 MMAs into the TMEM accumulator, then every thread
// waits for their completion. Returns false when the bounded wait ran out.
template <int K>
__device__ __forceinline__ bool umma_layer(uint32_t tmem, uint32_t a_base, uint32_t b_base, unsigned long long* bar,
                                           unsigned& phase) {
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
#pragma unroll
    for (int ks = 0; ks < K / 16; ++ks)
      umma_bf16(tmem, umma_desc(a_base + 2 * ks * kUmmaLbo), umma_desc(b_base + 2 * ks * kUmmaLbo), ks > 0);
    umma_commit(bar);
  }
  const bool done = mbar_wait_parity(bar, phase);
  phase ^= 1u;
  tc_fence_after();
  return done;
}

// bias + ReLU + BF16 rounding of one hidden layer's accumulator row; the
// rounded values become the next layer's A operand (row r of the tile) and
// are stored to out when given
__device__ __forceinline__ void umma_hidden_epilogue(uint32_t t_row, const float* bias, unsigned char* act, int r,
                                                     float* out, int64_t row, int64_t n) {
#pragma unroll 1
  for (int c0 = 0; c0 < kH; c0 += 32) {
    float v[32];
    tmem_load32(t_row + (uint32_t)c0, v);
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = round_bf16(fmaxf(v[j] + bias[c0 + j], 0.f));
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint4 u;
      u.x = pack_bf16(v[8 * q], v[8 * q + 1]);
      u.y = pack_bf16(v[8 * q + 2], v[8 * q + 3]);
      u.z = pack_bf16(v[8 * q + 4], v[8 * q + 5]);
      u.w = pack_bf16(v[8 * q + 6], v[8 * q + 7]);
      *reinterpret_cast<uint4*>(act + core_offset(r, c0 + 8 * q)) = u;
    }
    if (out && row < n) {
      float4* o = reinterpret_cast<float4*>(out + row * kH + c0);
#pragma unroll
      for (int q = 0; q < 8; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
  }
}

__global__ void __launch_bounds__(kUmmaThreads, 2) forward_kernel(const float* feat, int64_t n,
                                                                  const __nv_bfloat16* P, float* A1, float* A2,
                                                                  float* A3, float* logits) {
  extern __shared__ __align__(1024) unsigned char fsm[];
  unsigned char* act = fsm + kSmAct;
  float* vec = reinterpret_cast<float*>(fsm + kSmVec);  // b1, b2, b3, w4, b4
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(fsm + kSmBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(fsm + kSmBar + 8);
  const int tid = threadIdx.x, warp = tid >> 5;
  // W^T in the core-matrix layout; P holds W as [k][n]
  for (int i = tid; i < kIn * kH; i += kUmmaThreads)
    *reinterpret_cast<__nv_bfloat16*>(fsm + kSmW1 + core_offset(i % kH, i / kH)) = P[kOffW1 + i];
  for (int i = tid; i < kH * kH; i += kUmmaThreads) {
    *reinterpret_cast<__nv_bfloat16*>(fsm + kSmW2 + core_offset(i % kH, i / kH)) = P[kOffW2 + i];
    *reinterpret_cast<__nv_bfloat16*>(fsm + kSmW3 + core_offset(i % kH, i / kH)) = P[kOffW3 + i];
  }
  for (int i = tid; i < kH; i += kUmmaThreads) {
    vec[i] = __bfloat162float(P[kOffB1 + i]);
    vec[kH + i] = __bfloat162float(P[kOffB2 + i]);
    vec[2 * kH + i] = __bfloat162float(P[kOffB3 + i]);
    vec[3 * kH + i] = __bfloat162float(P[kOffW4 + i]);
  }
  if (tid == 0) {
    vec[4 * kH] = __bfloat162float(P[kOffB4]);
    mbar_init1(bar);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t t_row = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's 32 TMEM lanes
  const uint32_t s_w1 = smem_u32(fsm + kSmW1), s_w2 = smem_u32(fsm + kSmW2), s_w3 = smem_u32(fsm + kSmW3);
  const uint32_t s_act = smem_u32(act);
  unsigned phase = 0;
  int64_t failed_tile = -1;
  const int64_t tiles = (n + kUmmaRows - 1) / kUmmaRows;
  for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int64_t row = tile * kUmmaRows + tid;
    // layer 1's A operand: this row's 32 features rounded to BF16
    {
      float4 x[kIn / 4];
      if (row < n) {
        const float4* src = reinterpret_cast<const float4*>(feat + row * kIn);
#pragma unroll
        for (int j = 0; j < kIn / 4; ++j) x[j] = src[j];
      } else {
#pragma unroll
        for (int j = 0; j < kIn / 4; ++j) x[j] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int kg = 0; kg < kIn / 8; ++kg) {
        uint4 u;
        u.x = pack_bf16(x[2 * kg].x, x[2 * kg].y);
        u.y = pack_bf16(x[2 * kg].z, x[2 * kg].w);
        u.z = pack_bf16(x[2 * kg + 1].x, x[2 * kg + 1].y);
        u.w = pack_bf16(x[2 * kg + 1].z, x[2 * kg + 1].w);
        *reinterpret_cast<uint4*>(act + core_offset(tid, 8 * kg)) = u;
      }
    }
    bool ok = umma_layer<kIn>(tmem, s_act, s_w1, bar, phase);
    if (__syncthreads_or(!ok)) { failed_tile = tile; break; }
    umma_hidden_epilogue(t_row, vec, act, tid, A1, row, n);
    ok = umma_layer<kH>(tmem, s_act, s_w2, bar, phase);
    if (__syncthreads_or(!ok)) { failed_tile = tile; break; }
    umma_hidden_epilogue(t_row, vec + kH, act, tid, A2, row, n);
    ok = umma_layer<kH>(tmem, s_act, s_w3, bar, phase);
    if (__syncthreads_or(!ok)) { failed_tile = tile; break; }
    float s = 0.f;
#pragma unroll 1
    for (int c0 = 0; c0 < kH; c0 += 32) {
      float v[32];
      tmem_load32(t_row + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        v[j] = fmaxf(v[j] + vec[2 * kH + c0 + j], 0.f);
        s = fmaf(v[j], vec[3 * kH + c0 + j], s);
      }
      if (A3 && row < n) {
        float4* o = reinterpret_cast<float4*>(A3 + row * kH + c0);
#pragma unroll
        for (int q = 0; q < 8; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
    }
    if (row < n) logits[row] = s + vec[4 * kH];
  }
  if (failed_tile >= 0) {
    // a commit that never arrived: give the MMAs in flight one more bounded
    // wait and set this CTA's remaining logits to NaN (they sort last)
    mbar_wait_parity(bar, phase ^ 1u);
    for (int64_t tile = failed_tile; tile < tiles; tile += gridDim.x) {
      const int64_t row = tile * kUmmaRows + tid;
      if (row < n) logits[row] = __int_as_float(0x7fc00000);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
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
  if (((uintptr_t)d_feat | (uintptr_t)d_a1 | (uintptr_t)d_a2 | (uintptr_t)d_a3) & 15)
    return fail(GCR_INVALID_ARG, "feature and activation buffers must be 16-byte aligned");
  if (n <= 0) return GCR_OK;
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CUDA_TRY(cudaFuncSetAttribute(forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kForwardSmem));
  const int64_t tiles = (n + kUmmaRows - 1) / kUmmaRows;
  const unsigned grid = (unsigned)(tiles < 2 * sms ? tiles : 2 * sms);
  forward_kernel<<<grid, kUmmaThreads, kForwardSmem, (cudaStream_t)stream>>>(
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
