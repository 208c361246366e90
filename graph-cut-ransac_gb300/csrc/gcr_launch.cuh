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

// Persistent kernel: each CTA takes pairs from a global ticket until none is
// left; blockIdx.x selects the CTA's scratch slot.
// Dynamic shared memory: the FP32 correspondence tile, the engine state and,
// for fundamental matrices, the state of DEGENSAC's inner run.
constexpr size_t kTileBytes = sizeof(float4) * kSmemPoints;
__host__ __device__ constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

template <class Est>
__host__ __device__ constexpr size_t nested_bytes() {
  return Est::KIND == 1 ? align256(sizeof(Shared<PlaneParallaxModel>)) : 0;
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

// ---- Staging of a pair's FP32 tile into shared memory by the tensor memory
// accelerator: one bulk copy (cp.async.bulk, global -> shared) per pair,
// completing on an mbarrier. Both addresses are 16-byte aligned and the size
// (16 bytes per correspondence) is a multiple of 16.
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier generic-proxy accesses of shared memory before
// later async-proxy (bulk copy) writes
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_copy_to_smem(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits (every thread) for the phase of the given parity; false when the
// bounded number of polls ran out.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  constexpr long long kPolls = 1ll << 22;
  for (long long it = 0; it < kPolls; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Persistent kernel: each CTA takes pairs from a global ticket until none is
// left; blockIdx.x selects the CTA's scratch slot.
template <class Est>
__global__ void __launch_bounds__(GCR_BLOCK, GCR_MIN_BLOCKS) pair_kernel(Workspace ws, EngineParams prm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* tile = reinterpret_cast<float4*>(smem_raw);
  Shared<Est>& sh = *reinterpret_cast<Shared<Est>*>(smem_raw + kTileBytes);
  __shared__ int s_pair;
  __shared__ __align__(8) unsigned long long tile_bar;
  const Slot slot = ws.slots[blockIdx.x];
  unsigned tile_phase = 0;
  if (threadIdx.x == 0) mbar_init(&tile_bar);
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
    if constexpr (Est::KIND == 1) {
      eng.nsh = reinterpret_cast<Shared<PlaneParallaxModel>*>(smem_raw + kTileBytes + align256(sizeof(Shared<Est>)));
      eng.nslot = ws.nested_slots[blockIdx.x];
    }
    // the centred FP32 copy (written by centre_kernel): staged into shared
    // memory by one bulk copy when it fits, read from global memory otherwise
    const PairAux aux = ws.aux[pair];
    const bool in_smem = pd.n <= kSmemPoints;
    float4* src = ws.pts32 + pd.offset;
    bool staged = true;
    if (in_smem && pd.n > 0) {
      // every thread is past its last access of the tile (the barrier at the
      // top of the loop); the copy's writes come after them
      if (threadIdx.x == 0) {
        fence_proxy_async_smem();
        bulk_copy_to_smem(tile, src, (unsigned)(sizeof(float4) * pd.n), &tile_bar);
      }
      bool done = mbar_wait_bounded(&tile_bar, tile_phase);
      if (!__syncthreads_and(done)) done = mbar_wait_bounded(&tile_bar, tile_phase);
      staged = __syncthreads_and(done);
      tile_phase ^= 1u;
    }
    eng.scale = aux.scale;
    eng.pts32 = in_smem ? tile : src;
    if (!staged) {
      // the copy did not complete within the bounded wait: report the pair and
      // stop this CTA (its tile may still be written)
      eng.reject(ST_DEVICE_ERROR);
      break;
    }
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
