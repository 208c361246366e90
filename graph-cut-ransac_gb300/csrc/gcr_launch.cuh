// Kernel entry and host-side launcher of the pair engine for one model kind.
#pragma once

#include <cstdio>
#include <cstring>
#include <vector>

#include "gcr_engine.cuh"

// Resident CTAs per SM the kernel is compiled for (registers <= 64K / (256 * 2)).
#ifndef GCR_MIN_BLOCKS
#define GCR_MIN_BLOCKS 2
#endif

namespace gcr {

__device__ inline double block_max_abs(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double r = 0;
  for (int i = 0; i < GCR_WARPS; ++i) r = fmax(r, red[i]);
  __syncthreads();
  return r;
}

// The GPU's global nanosecond timer (per-pair service times).
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Dynamic shared memory: the FP32 correspondence tile, the engine state and,
// for fundamental matrices, the state of DEGENSAC's inner run.
constexpr size_t kTileBytes = sizeof(float4) * kSmemPoints;
__host__ __device__ constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

template <class Est>
__host__ __device__ constexpr size_t nested_bytes() {
  return has_degensac<Est>() ? align256(sizeof(Shared<PlaneParallaxModel>)) : 0;
}

template <class Est>
__host__ __device__ constexpr size_t shared_total() {
  return kTileBytes + align256(sizeof(Shared<Est>)) + nested_bytes<Est>();
}

// Centred FP32 copy of a pair's correspondences into dst (shared memory or
// global), the largest centred magnitude into mx (per thread); returns
// nonzero when this thread saw a coordinate (fitting or pixel) that is not
// finite.
__device__ inline int load_pair_tile(const Workspace& ws, const PairDesc& pd, const double* p64, float4* dst,
                                     double& mx) {
  int bad = 0;
  for (int i = threadIdx.x; i < pd.n; i += GCR_BLOCK) {
    const double a = p64[4 * i] - pd.centre[0], b = p64[4 * i + 1] - pd.centre[1];
    const double c = p64[4 * i + 2] - pd.centre[2], d = p64[4 * i + 3] - pd.centre[3];
    dst[i] = make_float4((float)a, (float)b, (float)c, (float)d);
    mx = fmax(mx, fmax(fmax(fabs(a), fabs(b)), fmax(fabs(c), fabs(d))));
    bad |= !(isfinite(a) && isfinite(b) && isfinite(c) && isfinite(d));
  }
  if (ws.pix64 != ws.pts64) {
    const double* px = ws.pix64 + 4 * pd.offset;
    for (int i = threadIdx.x; i < 4 * pd.n; i += GCR_BLOCK) bad |= !isfinite(px[i]);
  }
  return bad;
}

// Persistent kernel: each CTA takes pairs from a global ticket until none is
// left; blockIdx.x selects the CTA's scratch slot.
template <class Est>
__global__ void __launch_bounds__(GCR_BLOCK, GCR_MIN_BLOCKS) pair_kernel(Workspace ws, EngineParams prm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* tile = reinterpret_cast<float4*>(smem_raw);
  Shared<Est>& sh = *reinterpret_cast<Shared<Est>*>(smem_raw + kTileBytes);
  __shared__ int s_pair;
  const Slot slot = ws.slots[blockIdx.x];
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_pair = atomicAdd(ws.ticket, 1);
    __syncthreads();
    const int ticket = s_pair;
    if (ticket >= prm.num_pairs) break;
    const int pair = ws.order ? ws.order[ticket] : ticket;
    if (ws.times && threadIdx.x == 0) ws.times[2 * pair] = global_ns();
    const PairDesc pd = ws.pairs[pair];
    Engine<Est> eng(sh, ws, prm, pd, slot, pair);
    if constexpr (has_degensac<Est>()) {
      eng.nsh = reinterpret_cast<Shared<PlaneParallaxModel>*>(smem_raw + kTileBytes + align256(sizeof(Shared<Est>)));
      eng.nslot = ws.nested_slots[blockIdx.x];
    }
    // the centred FP32 copy (written by centre_kernel): copied into shared
    // memory by coalesced 16-byte loads when it fits, read from global memory
    // otherwise. (A bulk copy by the tensor memory accelerator on an mbarrier
    // staged the same bytes, but the essential-matrix engine's per-thread
    // solvers then ran 4.3 times the cycles: 545 against 1256 pairs/s on 1024
    // pairs; the other kinds measured equal or faster with these loads.)
    const PairAux aux = ws.aux[pair];
    const bool in_smem = pd.n <= kSmemPoints;
    const float4* src = ws.pts32 + pd.offset;
    if (in_smem) {
      for (int i = threadIdx.x; i < pd.n; i += GCR_BLOCK) tile[i] = src[i];
      __syncthreads();
    }
    eng.scale = aux.scale;
    eng.pts32 = in_smem ? tile : src;
    // a pair with a coordinate that is not finite is not run (status
    // GCR_INVALID_ARG, no model, empty mask)
    if (aux.bad) eng.reject(ST_INVALID_ARG);
    else eng.run();
    if (ws.times) {
      __syncthreads();
      if (threadIdx.x == 0) ws.times[2 * pair + 1] = global_ns();
    }
  }
}

template <class Est>
size_t shared_bytes() {
  return shared_total<Est>();
}

// Scratch bytes of one slot for pairs of at most max_n correspondences.
// Light slots (DEGENSAC's inner run) have no graph-cut or sampler-grid scratch.
template <class Est>
size_t slot_bytes(int max_n, int sort_cap, bool light = false) {
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t s = 0;
  s += al(sizeof(double) * 9 * (Shared<Est>::kModels + Shared<Est>::kStage));
  s += al(sizeof(float) * 12 * Shared<Est>::kModels);
  s += al(sizeof(int) * GCR_BLOCK * Est::SAMPLE_CAP);
  s += al(sizeof(int) * GCR_BLOCK * Est::M);
  s += al(sizeof(double) * (GCR_WARPS * 64 + 64));
  s += 3 * al(sizeof(int) * max_n);
  s += al((size_t)max_n);
  s += 2 * al(sizeof(double) * max_n);
  if (!light) {
    s += al(sizeof(int) * 16 * (size_t)max_n);
    s += al(sizeof(int) * (size_t)max_n);
    s += al(sizeof(double) * GCR_BLOCK);
    s += 3 * al(sizeof(int) * (size_t)max_n);
    s += al(sizeof(unsigned long long) * sort_cap);
    s += al(sizeof(int) * max_n);
    s += al(sizeof(int) * (max_n + 1));
    s += al(sizeof(double) * GCR_WARPS * kMaxFlowCap * kMaxFlowCap);
    s += al(sizeof(double) * GCR_WARPS * 3 * kMaxFlowCap);
    s += al(sizeof(int) * GCR_WARPS * 3 * kMaxFlowCap);
  }
  return s;
}

template <class Est>
Slot carve_slot(unsigned char* base, int max_n, int sort_cap, bool light = false) {
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  Slot s{};
  unsigned char* p = base;
  auto take = [&](size_t b) { unsigned char* r = p; p += al(b); return r; };
  s.models64 = (double*)take(sizeof(double) * 9 * (Shared<Est>::kModels + Shared<Est>::kStage));
  s.models32 = (float*)take(sizeof(float) * 12 * Shared<Est>::kModels);
  s.samples = (int*)take(sizeof(int) * GCR_BLOCK * Est::SAMPLE_CAP);
  s.bsamples = (int*)take(sizeof(int) * GCR_BLOCK * Est::M);
  s.red = (double*)take(sizeof(double) * (GCR_WARPS * 64 + 64));
  s.list0 = (int*)take(sizeof(int) * max_n);
  s.list1 = (int*)take(sizeof(int) * max_n);
  s.list2 = (int*)take(sizeof(int) * max_n);
  s.flag = (uint8_t*)take((size_t)max_n);
  s.dres = (double*)take(sizeof(double) * max_n);
  s.tr = (double*)take(sizeof(double) * max_n);
  if (!light) {
    s.napsac = (int*)take(sizeof(int) * 16 * (size_t)max_n);
    s.sprt_pool = (int*)take(sizeof(int) * (size_t)max_n);
    s.sprt_buf = (double*)take(sizeof(double) * GCR_BLOCK);
    s.sp_cell = (int*)take(sizeof(int) * (size_t)max_n);
    s.sp_flag = (int*)take(sizeof(int) * (size_t)max_n);
    s.sp_sel = (int*)take(sizeof(int) * (size_t)max_n);
    s.sortbuf = (unsigned long long*)take(sizeof(unsigned long long) * sort_cap);
    s.cell_pts = (int*)take(sizeof(int) * max_n);
    s.cell_start = (int*)take(sizeof(int) * (max_n + 1));
    s.flow = (double*)take(sizeof(double) * GCR_WARPS * kMaxFlowCap * kMaxFlowCap);
    s.node_d = (double*)take(sizeof(double) * GCR_WARPS * 3 * kMaxFlowCap);
    s.node_i = (int*)take(sizeof(int) * GCR_WARPS * 3 * kMaxFlowCap);
  }
  return s;
}

}  // namespace gcr
