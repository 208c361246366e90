// gcr_find_homography_device_noalloc: the homography search on one image pair
// with every byte of device scratch taken from a fixed array compiled into
// this library, so that a call allocates no device memory at all.
//
// Who needs this: callers that may not allocate while they run — a process
// whose device memory is reserved up front by another allocator and must not
// grow, a real-time loop where the implicit device synchronisation of
// cudaMalloc/cudaFree would stall other streams, or code that queues work
// with nothing but plain kernel launches. gcr_batch_run_device grows its
// scratch with cudaMalloc on demand; this entry point never does.
//
// Limits: one image pair per call, at most kNoAllocMaxPoints correspondences
// (the FP32 copy of the pair then always stays in shared memory), and one
// scratch array per device: calls that overlap in time on the same device —
// from two host threads, or queued on two streams that run concurrently —
// use the same scratch and race. Queue them on one stream, or serialise them.
//
// The first call on a device does a one-time set-up with that device current
// (it looks up the scratch array's device address and raises the kernel's
// shared-memory limit); make that first call before any stream capture
// begins.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <limits>
#include <mutex>

#include "../../include/gcr.h"
#include "gcr_homography.cuh"
#include "gcr_launch.cuh"

namespace gcr {
// Records the message returned by gcr_last_error_string (gcr_api.cu).
void set_last_error(const char* msg);
// The argument checks of every gcr_params entry point (gcr_api.cu).
gcr_status check_params(gcr_model_kind kind, const gcr_params* p);
// Grid divisions per axis for neighborhood_size (gcr_api.cu).
int32_t grid_divisions(double neighborhood_size, bool radius_graph);
}  // namespace gcr

namespace {

using Est = gcr::HomographyModel;

constexpr int kNoAllocMaxPoints = gcr::kSmemPoints;  // 4096 correspondences
constexpr size_t kNoAllocScratchBytes = size_t(5) << 20;  // 5 MiB: one engine slot for 4096 points
constexpr int kMaxDevices = 64;

// The scratch of every call on a device. Nothing in it has to start at zero:
// the engine writes each array of its slot before it reads it, for every pair.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct DeviceSetup {
  bool done = false;
  gcr::Slot slot{};
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mutex;

gcr_status fail(gcr_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  gcr::set_last_error(buf);
  return s;
}

// One engine CTA on the single pair of the call: the per-pair body of the
// persistent pair kernel, with the pair descriptor and the scratch slot passed
// by value instead of read from device arrays, and no work ticket.
__global__ void __launch_bounds__(GCR_BLOCK, 1)
    single_pair_kernel(gcr::Workspace ws, gcr::EngineParams prm, gcr::PairDesc pd, gcr::Slot slot) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* tile = reinterpret_cast<float4*>(smem_raw);
  gcr::Shared<Est>& sh = *reinterpret_cast<gcr::Shared<Est>*>(smem_raw + gcr::kTileBytes);
  gcr::Engine<Est> eng(sh, ws, prm, pd, slot, 0);
  double mx = 0.0;
  const int bad = gcr::load_pair_tile(ws, pd, ws.pts64, tile, mx);
  eng.scale = gcr::block_max_abs(mx, sh.red_d);
  eng.pts32 = tile;
  if (__syncthreads_or(bad)) eng.reject(gcr::ST_INVALID_ARG);
  else eng.run();
}

// One-time set-up of the current device; returns its scratch slot. A device
// counts as set up only once both steps succeeded, so a call that failed here
// (for instance one made during a stream capture) leaves the next call to try
// again.
gcr_status setup_device(int dev, gcr::Slot* out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceSetup& s = g_setup[dev];
  if (!s.done) {
    unsigned char* base = nullptr;
    cudaError_t err = cudaGetSymbolAddress((void**)&base, g_noalloc_scratch);
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(single_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)gcr::shared_bytes<Est>());
    if (err == cudaSuccess && gcr::slot_bytes<Est>(kNoAllocMaxPoints, kNoAllocMaxPoints) > kNoAllocScratchBytes)
      err = cudaErrorInvalidValue;  // cannot happen for the sizes above
    if (err != cudaSuccess)
      return fail(GCR_DEVICE_ERROR, "set-up of the allocation-free scratch on device %d failed: %s", dev,
                  cudaGetErrorString(err));
    s.slot = gcr::carve_slot<Est>(base, kNoAllocMaxPoints, kNoAllocMaxPoints);
    s.done = true;
  }
  *out = s.slot;
  return GCR_OK;
}

}  // namespace

extern "C" gcr_status gcr_find_homography_device_noalloc(const double* d_corr, int64_t n,
                                                         const gcr_image_size* size, const gcr_params* params,
                                                         uint64_t seed, double* d_model_out9,
                                                         uint8_t* d_mask_out, gcr_stats* d_stats_out,
                                                         void* stream) {
  if (!d_corr || !size || !params || !d_model_out9 || !d_mask_out || !d_stats_out)
    return fail(GCR_INVALID_ARG, "NULL argument");
  if (n < Est::M) return fail(GCR_TOO_FEW_POINTS, "%lld correspondences, needs >= %d", (long long)n, Est::M);
  if (n > kNoAllocMaxPoints)
    return fail(GCR_CAPACITY,
                "%lld correspondences exceed the %d that the fixed scratch of the allocation-free entry point "
                "holds; use gcr_batch_run_device for larger pairs",
                (long long)n, kNoAllocMaxPoints);
  if (size->h1 <= 0 || size->w1 <= 0 || size->h2 <= 0 || size->w2 <= 0)
    return fail(GCR_INVALID_ARG, "image sizes must be positive");
  gcr_status chk = gcr::check_params(GCR_HOMOGRAPHY, params);
  if (chk != GCR_OK) return chk;
  // the limits of this entry point beyond the shared checks
  const gcr_params& p = *params;
  if (p.sampler != GCR_SAMPLER_UNIFORM && p.sampler != GCR_SAMPLER_PROSAC && p.sampler != GCR_SAMPLER_PNAPSAC)
    return fail(GCR_UNSUPPORTED, "sampler %d is not provided here (0 uniform, 1 PROSAC, 2 P-NAPSAC)", p.sampler);
  if (p.scoring != GCR_SCORING_MSAC) return fail(GCR_UNSUPPORTED, "scoring %d is not provided here", p.scoring);
  if (p.spatial_coherence_weight > 0 && p.neighborhood != GCR_NEIGHBORHOOD_GRID)
    return fail(GCR_UNSUPPORTED, "only the grid neighbourhood (0) is provided here with a spatial coherence term");

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(GCR_DEVICE_ERROR, "cudaGetDevice failed: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(GCR_DEVICE_ERROR, "device %d out of range", dev);
  gcr::Slot slot;
  gcr_status st = setup_device(dev, &slot);
  if (st != GCR_OK) return st;

  // the same descriptor and engine parameters as gcr_batch_run_device builds
  // for a batch of one homography pair
  gcr::PairDesc pd{};
  pd.offset = 0;
  pd.n = (int32_t)n;
  // the grid's divisions, as gcr_batch_run_device sets them (the radius
  // graph is not taken here, so the size is a division count)
  pd.n_div = gcr::grid_divisions(p.neighborhood_size, false);
  const double nd = (double)pd.n_div;
  const double eps = std::numeric_limits<double>::epsilon();
  pd.cell[0] = (size->w1 + eps) / nd;
  pd.cell[1] = (size->h1 + eps) / nd;
  pd.cell[2] = (size->w2 + eps) / nd;
  pd.cell[3] = (size->h2 + eps) / nd;
  pd.threshold = p.threshold;
  pd.centre[0] = 0.5 * size->w1;
  pd.centre[1] = 0.5 * size->h1;
  pd.centre[2] = 0.5 * size->w2;
  pd.centre[3] = 0.5 * size->h2;
  pd.img[0] = size->w1;
  pd.img[1] = size->h1;
  pd.img[2] = size->w2;
  pd.img[3] = size->h2;
  pd.seed = seed;

  gcr::Workspace ws{};
  ws.pts64 = d_corr;
  ws.pix64 = d_corr;
  ws.pts32 = nullptr;  // the pair always fits the shared-memory tile
  ws.pairs = nullptr;
  ws.slots = nullptr;
  ws.nested_slots = nullptr;
  ws.ticket = nullptr;
  ws.models_out = d_model_out9;
  ws.masks_out = d_mask_out;
  ws.stats_out = (gcr::StatsOut*)d_stats_out;
  ws.phase = nullptr;
  ws.times = nullptr;

  gcr::EngineParams prm{};
  prm.confidence = p.confidence;
  prm.lambda = p.spatial_coherence_weight;
  prm.max_iters = p.max_iterations;
  prm.min_iters = p.min_iterations;
  prm.lo_number = p.lo_number;
  prm.sampler = p.sampler;
  prm.scoring = p.scoring;
  prm.num_pairs = 1;
  prm.max_n = (int32_t)n;
  prm.nested = 0;
  prm.stream_main = 1;
  prm.stream_lo = 2;
  prm.pp_h = nullptr;
  prm.use_sprt = p.use_sprt ? 1 : 0;
  prm.use_sp = p.use_space_partitioning ? 1 : 0;
  prm.gc_max = 10;      // GCRANSAC's default max_graph_cut_number
  prm.final_irls = 1;   // and do_final_iterated_least_squares
  prm.epilogue = 1;
  prm.batch_calls = GCR_BLOCK;
  prm.lo_fp32 = 0;
  // the homography driver's SPRT starts from the inlier ratio 0.01 whatever
  // min_inlier_ratio_for_sprt holds (gcransac_python.cpp:4394-4396)
  prm.sprt_min_ratio = 0.01;

  single_pair_kernel<<<1, GCR_BLOCK, gcr::shared_bytes<Est>(), (cudaStream_t)stream>>>(ws, prm, pd, slot);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GCR_DEVICE_ERROR, "engine launch failed: %s", cudaGetErrorString(e));
  return GCR_OK;
}
