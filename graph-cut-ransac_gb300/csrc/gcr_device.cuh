// Device utilities of the GB300 Graph-Cut RANSAC engine: the counter-based
// sampler streams, CTA-wide reductions and sorting, bounded waits.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#ifndef GCR_BLOCK
#define GCR_BLOCK 256
#endif
#define GCR_WARPS (GCR_BLOCK / 32)

namespace gcr {

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). The d-th 32-bit draw of
// call c of stream s under seed k is word (d & 3) of
// Philox(counter = {d >> 2, c_lo, c_hi, s}, key = {k_lo, k_hi}).
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0;
    const uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

enum : uint32_t {
  STREAM_MAIN = 1,
  STREAM_LO = 2,
  STREAM_NAPSAC_LOCAL = 3,
  STREAM_NAPSAC_CENTER = 4,
  STREAM_NAPSAC_GLOBAL = 5,
};

// Sequential reader of one call of one stream: caches the 4-word block.
struct DrawStream {
  uint64_t seed;
  uint32_t stream;
  uint64_t call;
  uint32_t d = 0;
  uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;  // current 4-word block (kept in registers)
  uint32_t block_id = 0xffffffffu;
  __device__ DrawStream(uint64_t s, uint32_t st, uint64_t c) : seed(s), stream(st), call(c) {}
  __device__ __forceinline__ uint32_t next_u32() {
    const uint32_t b = d >> 2;
    if (b != block_id) {
      uint32_t blk[4] = {b, (uint32_t)call, (uint32_t)(call >> 32), stream};
      philox4x32_10(blk, (uint32_t)seed, (uint32_t)(seed >> 32));
      w0 = blk[0]; w1 = blk[1]; w2 = blk[2]; w3 = blk[3];
      block_id = b;
    }
    const uint32_t q = (d++) & 3;
    return q == 0 ? w0 : (q == 1 ? w1 : (q == 2 ? w2 : w3));
  }
  // uniform integer in [lo, hi] (inclusive)
  __device__ __forceinline__ uint32_t next_in(uint32_t lo, uint32_t hi) {
    const uint64_t range = (uint64_t)hi - lo + 1;
    return lo + (uint32_t)(((uint64_t)next_u32() * range) >> 32);
  }
};

// Unique set of k indices from [lo, hi] by rejection, in draw order
// (utils::UniformRandomGenerator::generateUniqueRandomSet semantics).
__device__ __forceinline__ bool unique_set(DrawStream& ds, int* s, int k, uint32_t lo, uint32_t hi) {
  for (int i = 0; i < k; ++i) {
    s[i] = (int)ds.next_in(lo, hi);
    for (int j = i - 1; j >= 0; --j)
      if (s[i] == s[j]) { --i; break; }
    if (ds.d > (1u << 20)) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// CTA-wide helpers (blockDim.x == GCR_BLOCK). Every helper ends with a barrier
// so its result may be read by all threads.

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <class T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T u = __shfl_xor_sync(0xffffffffu, v, o);
    v = u < v ? u : v;
  }
  return v;
}

// Deterministic block sum: warp trees, then warp 0 sums the warp partials.
template <class T>
__device__ T block_sum(T v, T* red /* >= GCR_WARPS */) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  T r = 0;
#pragma unroll
  for (int i = 0; i < GCR_WARPS; ++i) r += red[i];
  __syncthreads();
  return r;
}

// Exclusive prefix of one int per thread; returns the total in *total.
__device__ inline int block_exclusive_scan(int v, int* red /* >= GCR_WARPS + 1 */, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) red[w] = x;
  __syncthreads();
  int base = 0;
  for (int i = 0; i < w; ++i) base += red[i];
  int tot = 0;
#pragma unroll
  for (int i = 0; i < GCR_WARPS; ++i) tot += red[i];
  __syncthreads();
  *total = tot;
  return base + x - v;
}

// In-place ascending bitonic sort of n (power of two) keys by the whole CTA.
__device__ inline void block_bitonic_sort(unsigned long long* a, int n) {
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += GCR_BLOCK) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const unsigned long long x = a[i], y = a[ixj];
          const bool up = (i & k) == 0;
          if ((x > y) == up) { a[i] = y; a[ixj] = x; }
        }
      }
      __syncthreads();
    }
  }
}

}  // namespace gcr
