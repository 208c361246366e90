// C-ABI of libgcr.so (include/gcr.h): argument checks, device buffers of a
// gcr_context, per-pair descriptors and the engine launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/gcr.h"
#include "gcr_engine.cuh"
#include "gcr_kinds.h"
#include "gcr_launch.cuh"

namespace {

thread_local std::string g_last_error;
thread_local long long g_last_launches = 0;
thread_local long long* g_last_phase = nullptr;
// host probabilities of the single-pair entries, staged by gcr_find_batch
thread_local const double* g_batch_probs = nullptr;
// host sample tape of the host-buffer entries (gcr_set_sample_tape)
thread_local const int32_t* g_host_tape = nullptr;
thread_local long long g_host_tape_calls = 0;

gcr_status fail(gcr_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}

#define CUDA_TRY(expr)                                                                        \
  do {                                                                                        \
    cudaError_t e_ = (expr);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail(GCR_DEVICE_ERROR, "%s failed: %s", #expr, cudaGetErrorString(e_));          \
  } while (0)

// Growable device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t b = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) cap = b;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

const gcr::KindOps* ops_for(gcr_model_kind kind) {
  switch (kind) {
    case GCR_HOMOGRAPHY: return gcr::homography_ops();
    case GCR_FUNDAMENTAL: return gcr::fundamental_ops();
    case GCR_ESSENTIAL: return gcr::essential_ops();
    case GCR_HOMOGRAPHY_AFFINE: return gcr::homography_affine_ops();
    case GCR_FUNDAMENTAL_AFFINE: return gcr::fundamental_affine_ops();
    case GCR_FUNDAMENTAL_SIFT: return gcr::fundamental_sift_ops();
    case GCR_HOMOGRAPHY_SIFT: return gcr::homography_sift_ops();
    case GCR_ESSENTIAL_PLANAR: return gcr::essential_planar_ops();
  }
  return nullptr;
}

// Kinds with rows of 8 doubles (points, then the local affine map or the
// features' scales and orientations), split into point rows and the four
// extra values before the engine runs.
bool affine_kind(gcr_model_kind kind) {
  return kind == GCR_HOMOGRAPHY_AFFINE || kind == GCR_FUNDAMENTAL_AFFINE || kind == GCR_FUNDAMENTAL_SIFT ||
         kind == GCR_HOMOGRAPHY_SIFT;
}

// Essential-matrix kinds: K^-1 normalisation of the rows, thresholds divided
// by the mean focal length, the pose epilogue.
bool essential_kind(gcr_model_kind kind) { return kind == GCR_ESSENTIAL || kind == GCR_ESSENTIAL_PLANAR; }

// Doubles per correspondence row of a model kind (gcr_model_kind).
int kind_columns(gcr_model_kind kind) { return affine_kind(kind) ? 8 : 4; }

// The homography drivers construct their SPRT test without the
// min_inlier_ratio_for_sprt argument (gcransac_python.cpp:4394-4396,
// 4719-4721, 4979-4981), so it starts from the constructor's default inlier ratio 0.01
// (preemption_sprt.h:141-143); the other drivers pass the argument.
bool homography_driver(gcr_model_kind kind) {
  return kind == GCR_HOMOGRAPHY || kind == GCR_HOMOGRAPHY_AFFINE || kind == GCR_HOMOGRAPHY_SIFT;
}

}  // namespace

namespace gcr {
void set_last_error(const char* msg) { g_last_error = msg; }
}  // namespace gcr

struct gcr_context {
  int device = 0;
  int num_sms = 0;
  DevBuf pairs, slots_meta, slot_mem, pts32, ticket, norm_pts, kinv, row_pair, phase, aux;
  DevBuf affine;  // affine correspondences: the point columns, then the affine maps ([total][4] each)
  // staging of the host-buffer entry points
  DevBuf corr, models, masks, stats;
  DevBuf magsac;  // the MAGSAC++ weight table, uploaded on first use
  // the device work of the last prepared batch (see gcr_batch_prepare)
  struct Pending {
    bool valid = false;
    const gcr::KindOps* ops = nullptr;
    int grid = 0;
    gcr::Workspace ws{};
    gcr::EngineParams prm{};
    bool normalise = false;
    bool split_affine = false;      // affine correspondences: split the rows of 8 before the engine runs
    int64_t total = 0;
    const double* probs = nullptr;  // importance sampler: probabilities to tabulate
    const double* d_corr = nullptr;
    int num_pairs = 0;
  } pending;
  int slot_kind = -1, slot_max_n = 0, slot_count = 0;
  bool prepared[8] = {false, false, false, false, false, false, false, false};
  unsigned long long* pair_times = nullptr;  // see gcr_context_set_pair_times
  DevBuf rg_int, rg_dbl, rg_px;              // radius-graph scratch (one region per resident CTA)
  DevBuf ar_p, ar_i, ar_ab, ar_cnt;          // AR sampler heaps and per-point state (per resident CTA)
  const double* probs = nullptr;             // see gcr_context_set_probabilities
  DevBuf cdf, probs_stage;                   // importance sampler tables, staged probabilities
  long long flow_cap = 0;                    // see gcr_context_set_flow_step_limit
  const int32_t* tape = nullptr;             // see gcr_context_set_sample_tape
  long long tape_calls = 0;
  DevBuf tape_stage;                         // the host tape of the host-buffer entries, staged
  std::vector<gcr_tuning> tuning;            // see gcr_context_set_tuning
  DevBuf order;                              // pair of each work ticket (largest first)
  gcr_tuning last_tuning{};                  // the entry the last prepared batch used
  int32_t lo_fp32 = 0;                       // see gcr_context_set_lo_precision
};

namespace gcr {

// Argument checks shared by every entry point that takes gcr_params.
gcr_status check_params(gcr_model_kind kind, const gcr_params* p) {
  if (!p) return fail(GCR_INVALID_ARG, "params is NULL");
  if (!(p->threshold > 0)) return fail(GCR_INVALID_ARG, "threshold must be > 0");
  if (!(p->confidence > 0 && p->confidence < 1)) return fail(GCR_INVALID_ARG, "confidence must be in (0, 1)");
  if (!(p->spatial_coherence_weight >= 0 && p->spatial_coherence_weight <= 1))
    return fail(GCR_INVALID_ARG, "spatial_coherence_weight must be in [0, 1]");
  if (p->max_iterations < 0 || p->min_iterations < 0) return fail(GCR_INVALID_ARG, "negative iteration limit");
  if (p->lo_number < 0 || p->lo_number > GCR_BLOCK)
    return fail(GCR_UNSUPPORTED, "lo_number must be in [0, %d]", GCR_BLOCK);
  if (p->sampler < GCR_SAMPLER_UNIFORM || p->sampler > GCR_SAMPLER_AR)
    return fail(GCR_UNSUPPORTED,
                "sampler %d is not provided (0 uniform, 1 PROSAC, 2 P-NAPSAC, 3 importance, 4 AR)", p->sampler);
  if (p->sampler == GCR_SAMPLER_AR && !(p->sampler_variance > 0))
    return fail(GCR_INVALID_ARG, "the AR sampler needs sampler_variance > 0");
  if (p->scoring != GCR_SCORING_MSAC && p->scoring != GCR_SCORING_MAGSAC)
    return fail(GCR_UNSUPPORTED, "scoring %d is not provided (0 MSAC, 1 MAGSAC++)", p->scoring);
  if (p->use_sprt && !(p->min_inlier_ratio_for_sprt > 0 && p->min_inlier_ratio_for_sprt < 1))
    return fail(GCR_INVALID_ARG, "min_inlier_ratio_for_sprt must be in (0, 1) when use_sprt is set");
  if (p->neighborhood != GCR_NEIGHBORHOOD_GRID && p->neighborhood != GCR_NEIGHBORHOOD_FLANN)
    return fail(GCR_UNSUPPORTED, "neighbourhood %d is not provided (0 grid, 1 radius graph)", p->neighborhood);
  if (p->neighborhood == GCR_NEIGHBORHOOD_GRID && !(p->neighborhood_size >= 1))
    return fail(GCR_INVALID_ARG, "neighborhood_size must be >= 1 for the grid");
  // cell keys hold 10 bits per axis (40 bits for the four axes)
  if (p->neighborhood == GCR_NEIGHBORHOOD_GRID && !(p->neighborhood_size < 1025))
    return fail(GCR_UNSUPPORTED, "neighborhood_size must be at most 1024 grid divisions");
  if (p->neighborhood == GCR_NEIGHBORHOOD_FLANN && !(p->neighborhood_size > 0 && std::isfinite(p->neighborhood_size)))
    return fail(GCR_INVALID_ARG, "neighborhood_size (the radius) must be > 0 and finite for the radius graph");
  if (kind == GCR_ESSENTIAL_PLANAR && p->scoring != GCR_SCORING_MSAC)
    return fail(GCR_UNSUPPORTED, "the planar essential-matrix driver scores with MSAC only");
  if (affine_kind(kind)) {
    // findHomographyAC_ / findFundamentalMatrixAC_ / findFundamentalMatrixSIFT_ /
    // findHomographySIFT_ (gcransac_python.cpp:4553, 1924, 2222, 4813): MSAC,
    // and no P-NAPSAC
    if (p->sampler == GCR_SAMPLER_PNAPSAC)
      return fail(GCR_UNSUPPORTED, "the affine-correspondence drivers provide samplers 0, 1, 3 and 4");
    if (p->scoring != GCR_SCORING_MSAC)
      return fail(GCR_UNSUPPORTED, "the affine-correspondence drivers score with MSAC only");
  }
  return GCR_OK;
}

// Grid divisions per axis: neighborhood_size truncated (as the drivers'
// size_t conversion does), within [1, 1024]; one cell when the radius graph
// replaces the grid.
int32_t grid_divisions(double neighborhood_size, bool radius_graph) {
  if (radius_graph || !(neighborhood_size >= 1)) return 1;
  return neighborhood_size >= 1024 ? 1024 : (int32_t)neighborhood_size;
}

}  // namespace gcr

namespace {

using gcr::check_params;

// MAGSAC++ weight table (MAGSACScoringFunction, scoring_function.h:263-334):
// the upper incomplete gamma function Gamma(1.5, x / 1000) for x = 0..36000,
// which equals sqrt(pi)/2 erfc(sqrt(x/1000)) + sqrt(x/1000) exp(-x/1000).
const std::vector<double>& magsac_table() {
  static const std::vector<double> g = [] {
    std::vector<double> t(36001);
    for (int i = 0; i <= 36000; ++i) {
      const double x = i / 1000.0;
      t[i] = std::sqrt(M_PI) * 0.5 * std::erfc(std::sqrt(x)) + std::sqrt(x) * std::exp(-x);
    }
    return t;
  }();
  return g;
}

// radius graph: edges kept per correspondence (beyond this a pair reports
// GCR_CAPACITY)
constexpr int64_t kRadiusEdgesPerPoint = 32;

int pow2_at_least(int n) {
  int s = 1;
  while (s < n) s <<= 1;
  return s;
}

}  // namespace

extern "C" {

void gcr_default_params(gcr_model_kind kind, gcr_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->threshold = 1.0;
  p->confidence = 0.99;
  p->max_iterations = 10000;
  p->min_iterations = 50;
  p->sampler = GCR_SAMPLER_PROSAC;
  p->lo_number = 50;
  p->scoring = GCR_SCORING_MSAC;
  p->use_sprt = 1;
  p->seed = 0;
  p->min_inlier_ratio_for_sprt = kind == GCR_ESSENTIAL ? 0.01 : 0.00001;
  p->sampler_variance = 0.1;
  switch (kind) {
    case GCR_HOMOGRAPHY:  // bindings.cpp:1158-1178
    case GCR_HOMOGRAPHY_AFFINE:  // the same python entry with solver = 2
    case GCR_HOMOGRAPHY_SIFT:    // and with solver = 1
      p->spatial_coherence_weight = 0.975;
      p->neighborhood = GCR_NEIGHBORHOOD_GRID;
      p->neighborhood_size = 4.0;
      p->use_space_partitioning = kind == GCR_HOMOGRAPHY ? 1 : 0;
      break;
    case GCR_FUNDAMENTAL:  // bindings.cpp:1003-1022
    case GCR_FUNDAMENTAL_AFFINE:  // the same python entry with solver = 2
    case GCR_FUNDAMENTAL_SIFT:    // and with solver = 1
      p->spatial_coherence_weight = 0.0;
      p->neighborhood = GCR_NEIGHBORHOOD_FLANN;
      p->neighborhood_size = 20.0;
      break;
    case GCR_ESSENTIAL:  // bindings.cpp:1091-1112
      p->spatial_coherence_weight = 0.1;
      p->neighborhood = GCR_NEIGHBORHOOD_FLANN;
      p->neighborhood_size = 20.0;
      break;
    case GCR_ESSENTIAL_PLANAR:  // bindings.cpp:1114-1133
      p->spatial_coherence_weight = 0.975;
      p->neighborhood = GCR_NEIGHBORHOOD_FLANN;
      p->neighborhood_size = 20.0;
      break;
  }
}

const char* gcr_last_error_string(void) { return g_last_error.c_str(); }

int64_t gcr_last_launch_count(void) { return g_last_launches; }

#ifdef GCR_PHASE_PROFILE
// Device pointer of the [P][16] phase counters of the last launch (profiling builds only).
void* gcr_debug_phase_counters(void) { return g_last_phase; }
#endif

gcr_status gcr_context_create(gcr_context** ctx) {
  if (!ctx) return fail(GCR_INVALID_ARG, "ctx is NULL");
  gcr_context* c = new gcr_context();
  if (cudaGetDevice(&c->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) {
    delete c;
    return fail(GCR_DEVICE_ERROR, "no CUDA device available");
  }
  *ctx = c;
  return GCR_OK;
}

gcr_status gcr_context_destroy(gcr_context* c) {
  if (!c) return GCR_OK;
  for (DevBuf* b : {&c->pairs, &c->slots_meta, &c->slot_mem, &c->pts32, &c->aux, &c->affine, &c->ticket, &c->norm_pts, &c->kinv,
                    &c->row_pair, &c->phase, &c->corr, &c->models, &c->masks, &c->stats, &c->magsac, &c->rg_int,
                    &c->rg_dbl, &c->rg_px, &c->ar_p, &c->ar_i, &c->ar_ab, &c->ar_cnt, &c->cdf, &c->probs_stage, &c->tape_stage, &c->order})
    b->release();
  delete c;
  return GCR_OK;
}

// Device-resident batch: bulk arrays are device pointers, per-pair metadata
// (offsets, intrinsics, image sizes, seeds) are host arrays.
}  // extern "C"

// Host side of a batch: argument checks, scratch growth, descriptor and
// intrinsics uploads (queued on s). The device work it describes (ticket
// reset, K^-1 normalisation, engine launch) is recorded in *L and queued by
// launch_batch.
// GCRANSAC::run without the drivers (gcr_run): the caller's grid, the
// neighbourhood coordinates apart from the fitting ones, the threshold in the
// fitting coordinates' units, no epilogue.
struct RunOnly {
  const double* d_pixels;
  double cell[4];
  int divisions;
};

static gcr_status prepare_batch(gcr_context* c, gcr_model_kind kind, int64_t num_pairs, const double* d_corr,
                                const int64_t* h_offsets, const double* h_K, const gcr_image_size* h_sizes,
                                const gcr_params* params, const uint64_t* h_seeds, double* d_models_out,
                                uint8_t* d_masks_out, gcr_stats* d_stats_out, cudaStream_t s,
                                gcr_context::Pending* L, const RunOnly* run_only = nullptr) {
  L->valid = false;
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  const gcr::KindOps* ops = ops_for(kind);
  if (!ops) return fail(GCR_UNSUPPORTED, "model kind %d is not provided by this build", (int)kind);
  gcr_status st = check_params(kind, params);
  if (st != GCR_OK) return st;
  if (num_pairs <= 0) return GCR_OK;
  if (num_pairs > (1 << 30)) return fail(GCR_CAPACITY, "too many pairs");
  if (!d_corr || !h_offsets || !h_sizes || !d_models_out || !d_masks_out || !d_stats_out)
    return fail(GCR_INVALID_ARG, "NULL buffer");
  if (essential_kind(kind) && !h_K && !run_only) return fail(GCR_INVALID_ARG, "essential matrices need intrinsics");
  if (kind == GCR_ESSENTIAL_PLANAR && run_only)
    return fail(GCR_UNSUPPORTED, "gcr_run provides the homography, fundamental and essential estimators");
  if (affine_kind(kind) && run_only)
    return fail(GCR_UNSUPPORTED, "gcr_run takes point correspondences; affine ones run through gcr_find_batch");
  const int m = ops->sample_size;
  int max_n = 0;
  for (int64_t i = 0; i < num_pairs; ++i) {
    const int64_t n = h_offsets[i + 1] - h_offsets[i];
    if (n < 0) return fail(GCR_INVALID_ARG, "offsets are not non-decreasing at pair %lld", (long long)i);
    if (n < m) return fail(GCR_TOO_FEW_POINTS, "pair %lld has %lld correspondences, needs >= %d", (long long)i,
                           (long long)n, m);
    if (n >= (1 << 24)) return fail(GCR_CAPACITY, "pair %lld exceeds 2^24 correspondences", (long long)i);
    max_n = std::max<int>(max_n, (int)n);
  }
  const int64_t total = h_offsets[num_pairs] - h_offsets[0];
  if (h_offsets[0] != 0) return fail(GCR_INVALID_ARG, "offsets[0] must be 0");
  // image sizes set the grid's cell sizes and the centring of the FP32 copies
  for (int64_t i = 0; i < num_pairs; ++i) {
    const gcr_image_size& z = h_sizes[i];
    if (z.h1 <= 0 || z.w1 <= 0 || z.h2 <= 0 || z.w2 <= 0)
      return fail(GCR_INVALID_ARG, "pair %lld: image sizes must be positive (got %d x %d, %d x %d)", (long long)i,
                  z.h1, z.w1, z.h2, z.w2);
  }
  // the radius graph replaces the grid when asked for with a spatial term; the
  // fundamental / essential drivers build no neighbourhood for a weight at or
  // below machine epsilon, and the homography driver keeps the grid under space
  // partitioning (gcransac_python.cpp:1658-1687, 4282-4286)
  const double eps0 = std::numeric_limits<double>::epsilon();
  const bool radius = params->neighborhood == GCR_NEIGHBORHOOD_FLANN &&
                      (kind == GCR_HOMOGRAPHY ? params->spatial_coherence_weight > 0
                                              : params->spatial_coherence_weight > eps0) &&
                      !(kind == GCR_HOMOGRAPHY && params->use_space_partitioning);

  if (!c->prepared[kind]) {
    CUDA_TRY(ops->prepare());
    c->prepared[kind] = true;
  }
  int per_sm = 0;
  CUDA_TRY(ops->occupancy(&per_sm));
  if (per_sm < 1) return fail(GCR_DEVICE_ERROR, "engine kernel does not fit on an SM");
  // launch shape from the context's tuning table: the entry of this kind
  // with the smallest max_n that covers the batch's largest pair
  gcr_tuning tune{};
  tune.kind = (int32_t)kind;
  tune.max_n = max_n;
  tune.batch_calls = GCR_BLOCK;
  tune.ctas_per_sm = per_sm;
  tune.order = 0;
  {
    const gcr_tuning* best = nullptr;
    for (const gcr_tuning& e : c->tuning)
      if (e.kind == (int32_t)kind && e.max_n >= max_n && (!best || e.max_n < best->max_n)) best = &e;
    if (best) {
      if (best->batch_calls > 0) tune.batch_calls = std::min(best->batch_calls, (int32_t)GCR_BLOCK);
      if (best->ctas_per_sm > 0) tune.ctas_per_sm = std::min(best->ctas_per_sm, (int32_t)per_sm);
      tune.order = best->order;
      tune.max_n = best->max_n;
    }
  }
  c->last_tuning = tune;
  const int resident = tune.ctas_per_sm * c->num_sms;
  const int grid = (int)std::min<int64_t>(num_pairs, resident);
  const int sort_cap = pow2_at_least(max_n);

  // scratch slots (one per resident CTA), grown on demand
  if (c->slot_kind != (int)kind || c->slot_max_n < max_n || c->slot_count < grid) {
    const int want_n = std::max(max_n, c->slot_kind == (int)kind ? c->slot_max_n : 0);
    const int want_cnt = std::max(grid, c->slot_kind == (int)kind ? c->slot_count : 0);
    const int want_sort = pow2_at_least(want_n);
    const size_t per = ops->slot_bytes(want_n, want_sort);
    const size_t per_nested = ops->nested_slot_bytes ? ops->nested_slot_bytes(want_n) : 0;
    CUDA_TRY(cudaStreamSynchronize(s));
    CUDA_TRY(c->slot_mem.ensure((per + per_nested) * (size_t)want_cnt));
    CUDA_TRY(c->slots_meta.ensure(sizeof(gcr::Slot) * 2 * want_cnt));
    std::vector<gcr::Slot> meta(2 * (size_t)want_cnt);
    for (int i = 0; i < want_cnt; ++i) {
      unsigned char* b = (unsigned char*)c->slot_mem.p + (per + per_nested) * (size_t)i;
      ops->carve(b, want_n, want_sort, &meta[i]);
      if (ops->carve_nested) ops->carve_nested(b + per, want_n, &meta[want_cnt + i]);
    }
    CUDA_TRY(cudaMemcpy(c->slots_meta.p, meta.data(), sizeof(gcr::Slot) * 2 * want_cnt, cudaMemcpyHostToDevice));
    c->slot_kind = (int)kind;
    c->slot_max_n = want_n;
    c->slot_count = want_cnt;
  }
  (void)sort_cap;

  // per-pair descriptors
  std::vector<gcr::PairDesc> pd((size_t)num_pairs);
  const double eps = std::numeric_limits<double>::epsilon();
  for (int64_t i = 0; i < num_pairs; ++i) {
    gcr::PairDesc& d = pd[i];
    const gcr_image_size& z = h_sizes[i];
    d.offset = h_offsets[i];
    d.n = (int32_t)(h_offsets[i + 1] - h_offsets[i]);
    d.n_div = gcr::grid_divisions(params->neighborhood_size, radius);
    const double nd = (double)d.n_div;
    // the homography driver pads the image size by machine epsilon
    // (gcransac_python.cpp:4290-4297), the fundamental/essential ones do not
    // (1670-1677)
    const double pad = kind == GCR_HOMOGRAPHY ? eps : 0.0;
    const bool essential = essential_kind(kind);
    d.cell[0] = (z.w1 + pad) / nd;
    d.cell[1] = (z.h1 + pad) / nd;
    d.cell[2] = (z.w2 + pad) / nd;
    d.cell[3] = (z.h2 + pad) / nd;
    d.threshold = params->threshold;
    d.centre[0] = 0.5 * z.w1;
    d.centre[1] = 0.5 * z.h1;
    d.centre[2] = 0.5 * z.w2;
    d.centre[3] = 0.5 * z.h2;
    if (essential && !run_only) {
      // findEssentialMatrix_ (gcransac_python.cpp:2598-2603, 2655): the run
      // works on K^-1-normalised coordinates with the threshold divided by
      // the mean focal length; those coordinates need no centring
      const double* K1 = h_K + 18 * i;
      const double* K2 = K1 + 9;
      const double normalizer = 0.25 * (K1[0] + K1[4] + K2[0] + K2[4]);
      d.threshold = params->threshold / normalizer;
      for (int q = 0; q < 4; ++q) d.centre[q] = 0.0;
    }
    if (run_only) {
      d.n_div = run_only->divisions;
      for (int q = 0; q < 4; ++q) d.cell[q] = run_only->cell[q];
      d.threshold = params->threshold;
      if (essential)
        for (int q = 0; q < 4; ++q) d.centre[q] = 0.0;
    }
    d.img[0] = z.w1;
    d.img[1] = z.h1;
    d.img[2] = z.w2;
    d.img[3] = z.h2;
    d.seed = h_seeds ? h_seeds[i] : params->seed + (uint64_t)i;
  }
  CUDA_TRY(c->pairs.ensure(sizeof(gcr::PairDesc) * num_pairs));
  CUDA_TRY(cudaMemcpyAsync(c->pairs.p, pd.data(), sizeof(gcr::PairDesc) * num_pairs, cudaMemcpyHostToDevice, s));
  const double* run_pts = d_corr;
  if (essential_kind(kind) && !run_only) {
    // K^-1 of both cameras per pair (a singular K is rejected)
    std::vector<double> kinv(18 * (size_t)num_pairs);
    for (int64_t i = 0; i < num_pairs; ++i)
      for (int cam = 0; cam < 2; ++cam)
        if (!gcr::inverse3(h_K + 18 * i + 9 * cam, kinv.data() + 18 * i + 9 * cam))
          return fail(GCR_INVALID_ARG, "intrinsics of pair %lld camera %d are singular", (long long)i, cam + 1);
    CUDA_TRY(c->kinv.ensure(sizeof(double) * kinv.size()));
    // (a copy from pageable memory is staged before the call returns)
    CUDA_TRY(cudaMemcpyAsync(c->kinv.p, kinv.data(), sizeof(double) * kinv.size(), cudaMemcpyHostToDevice, s));
    CUDA_TRY(c->norm_pts.ensure(sizeof(double) * 4 * (size_t)std::max<int64_t>(total, 1)));
    run_pts = (const double*)c->norm_pts.p;
  }
  const double* affine_maps = nullptr;
  if (affine_kind(kind)) {
    // rows of 8 are split into the point columns (what every step but the
    // minimal solver reads) and the affine maps
    CUDA_TRY(c->affine.ensure(sizeof(double) * 8 * (size_t)std::max<int64_t>(total, 1)));
    run_pts = (const double*)c->affine.p;
    affine_maps = run_pts + 4 * (size_t)std::max<int64_t>(total, 1);
  }
  // the centred FP32 copy of every pair (staging kernel) and its per-pair results
  CUDA_TRY(c->pts32.ensure(sizeof(float4) * (size_t)std::max<int64_t>(total, 1)));
  CUDA_TRY(c->aux.ensure(sizeof(gcr::PairAux) * (size_t)num_pairs));
  CUDA_TRY(c->ticket.ensure(sizeof(int)));
  // largest pairs first: a persistent CTA that takes a big pair late would
  // otherwise finish long after the others (stable order among equal sizes)
  const int* d_order = nullptr;
  if (tune.order == 1 && num_pairs > 1) {
    std::vector<int> ord((size_t)num_pairs);
    for (int64_t i = 0; i < num_pairs; ++i) ord[i] = (int)i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
      return h_offsets[a + 1] - h_offsets[a] > h_offsets[b + 1] - h_offsets[b];
    });
    CUDA_TRY(c->order.ensure(sizeof(int) * (size_t)num_pairs));
    CUDA_TRY(cudaMemcpy(c->order.p, ord.data(), sizeof(int) * (size_t)num_pairs, cudaMemcpyHostToDevice));
    d_order = (const int*)c->order.p;
  }

  gcr::Workspace ws;
  ws.pts64 = run_pts;
  ws.pix64 = run_only ? run_only->d_pixels : (affine_kind(kind) ? run_pts : d_corr);
  ws.affine64 = affine_maps;
  ws.pts32 = (float4*)c->pts32.p;
  ws.pairs = (const gcr::PairDesc*)c->pairs.p;
  ws.slots = (gcr::Slot*)c->slots_meta.p;
  ws.nested_slots = (gcr::Slot*)c->slots_meta.p + c->slot_count;
  ws.ticket = (int*)c->ticket.p;
  ws.models_out = d_models_out;
  ws.masks_out = d_masks_out;
  ws.stats_out = (gcr::StatsOut*)d_stats_out;
  ws.phase = nullptr;
  ws.times = c->pair_times;
  ws.order = d_order;
  ws.aux = (const gcr::PairAux*)c->aux.p;
#ifdef GCR_PHASE_PROFILE
  CUDA_TRY(c->phase.ensure(sizeof(long long) * 16 * num_pairs));
  CUDA_TRY(cudaMemsetAsync(c->phase.p, 0, sizeof(long long) * 16 * num_pairs, s));
  ws.phase = (long long*)c->phase.p;
  g_last_phase = (long long*)c->phase.p;
#endif

  gcr::EngineParams prm;
  prm.confidence = params->confidence;
  prm.lambda = params->spatial_coherence_weight;
  // the fundamental/essential drivers build no neighbourhood for a weight at
  // or below machine epsilon (gcransac_python.cpp:1658-1667)
  if (kind != GCR_HOMOGRAPHY && prm.lambda <= eps && !run_only) prm.lambda = 0.0;
  prm.max_iters = params->max_iterations;
  prm.min_iters = params->min_iterations;
  prm.lo_number = params->lo_number;
  prm.sampler = params->sampler;
  prm.scoring = params->scoring;
  prm.num_pairs = (int32_t)num_pairs;
  prm.max_n = max_n;
  prm.nested = 0;
  prm.stream_main = 1;  // STREAM_MAIN
  prm.stream_lo = 2;    // STREAM_LO
  prm.pp_h = nullptr;
  prm.use_sprt = params->use_sprt ? 1 : 0;
  prm.use_sp = (kind == GCR_HOMOGRAPHY && params->use_space_partitioning) ? 1 : 0;
  // the planar driver's SPRT branch sets max_graph_cut_number = 100 and
  // do_final_iterated_least_squares = false (gcransac_python.cpp:3741-3742);
  // its other branch and the other drivers keep the defaults (10, true)
  const bool planar_sprt = kind == GCR_ESSENTIAL_PLANAR && params->use_sprt && !run_only;
  prm.gc_max = planar_sprt ? 100 : 10;
  prm.final_irls = planar_sprt ? 0 : 1;
  prm.sprt_min_ratio = homography_driver(kind) && !run_only ? 0.01 : params->min_inlier_ratio_for_sprt;
  prm.epilogue = run_only ? 0 : 1;
  prm.flow_cap = c->flow_cap;
  prm.tape = c->tape;
  prm.tape_calls = c->tape ? c->tape_calls : 0;
  prm.batch_calls = tune.batch_calls;
  prm.lo_fp32 = c->lo_fp32;
  prm.cdf = nullptr;
  prm.neighborhood = 0;
  prm.radius2 = 0.0;
  prm.rg_cap = 0;
  prm.rg_stride_n = 0;
  prm.rg_int = nullptr;
  prm.rg_dbl = nullptr;
  prm.rg_px = nullptr;
  if (radius) {
    // the homography driver with space partitioning keeps the grid
    // (gcransac_python.cpp:4282-4286); otherwise the radius graph, with room
    // for kRadiusEdgesPerPoint edges per correspondence
    const int64_t stride = (int64_t)max_n + 1;
    const int64_t cap = (int64_t)max_n * kRadiusEdgesPerPoint;
    if (cap > 0x7fffffffLL) return fail(GCR_CAPACITY, "radius graph capacity");
    CUDA_TRY(c->rg_int.ensure(sizeof(int) * (size_t)grid * (size_t)(5 * stride + 3 * cap)));
    CUDA_TRY(c->rg_dbl.ensure(sizeof(double) * (size_t)grid * (size_t)(2 * cap + 3 * stride)));
    CUDA_TRY(c->rg_px.ensure(sizeof(float4) * (size_t)grid * (size_t)stride));
    prm.neighborhood = 1;
    prm.radius2 = params->neighborhood_size * params->neighborhood_size;
    prm.rg_cap = (int32_t)cap;
    prm.rg_stride_n = (int32_t)stride;
    prm.rg_int = (int*)c->rg_int.p;
    prm.rg_dbl = (double*)c->rg_dbl.p;
    prm.rg_px = (float4*)c->rg_px.p;
  }
  prm.probs = nullptr;
  // the planar driver's AR sampler takes the variance 0.1 whatever the
  // argument holds (gcransac_python.cpp:3675)
  prm.sampler_variance = kind == GCR_ESSENTIAL_PLANAR && !run_only ? 0.1 : params->sampler_variance;
  prm.ar_p = nullptr;
  prm.ar_i = nullptr;
  prm.ar_ab = nullptr;
  prm.ar_cnt = nullptr;
  prm.ar_cap = 0;
  prm.ar_stride_n = 0;
  if (params->sampler == GCR_SAMPLER_AR) {
    if (!c->probs) return fail(GCR_INVALID_ARG, "the AR sampler (4) needs per-correspondence probabilities");
    // a heap entry per point plus m per sampler call, for the iteration limit
    // (at most 2^20) and two batches of calls beyond it
    const int64_t calls = std::min<int64_t>(params->max_iterations, 1 << 20) + 2 * GCR_BLOCK;
    const int64_t cap = (int64_t)max_n + (int64_t)ops->sample_size * calls;
    if (cap > 0x7fffffffLL) return fail(GCR_CAPACITY, "AR sampler heap");
    const int64_t stride = (int64_t)max_n + 1;
    CUDA_TRY(c->ar_p.ensure(sizeof(double) * (size_t)grid * (size_t)cap));
    CUDA_TRY(c->ar_i.ensure(sizeof(int) * (size_t)grid * (size_t)cap));
    CUDA_TRY(c->ar_ab.ensure(sizeof(double) * 2 * (size_t)grid * (size_t)stride));
    CUDA_TRY(c->ar_cnt.ensure(sizeof(int) * (size_t)grid * (size_t)stride));
    prm.probs = c->probs;
    prm.ar_p = (double*)c->ar_p.p;
    prm.ar_i = (int*)c->ar_i.p;
    prm.ar_ab = (double*)c->ar_ab.p;
    prm.ar_cnt = (int*)c->ar_cnt.p;
    prm.ar_cap = (int32_t)cap;
    prm.ar_stride_n = (int32_t)stride;
  }
  if (params->sampler == GCR_SAMPLER_IMPORTANCE) {
    if (!c->probs) return fail(GCR_INVALID_ARG, "the importance sampler (3) needs per-correspondence probabilities");
    CUDA_TRY(c->cdf.ensure(sizeof(double) * (size_t)std::max<int64_t>(total, 1)));
    prm.cdf = (const double*)c->cdf.p;
  }
  prm.mag_table = nullptr;
  prm.mag_c2dof = 0.25 * std::pow(2.0, 1.5);
  prm.mag_gamma_k = 0.0036572608340910764;
  prm.mag_gamma_diff = std::tgamma(1.5) - prm.mag_gamma_k;
  if (params->scoring == GCR_SCORING_MAGSAC) {
    if (c->magsac.cap == 0) {
      const std::vector<double>& g = magsac_table();
      CUDA_TRY(c->magsac.ensure(sizeof(double) * g.size()));
      CUDA_TRY(cudaMemcpy(c->magsac.p, g.data(), sizeof(double) * g.size(), cudaMemcpyHostToDevice));
    }
    prm.mag_table = (const double*)c->magsac.p;
  }
  L->ops = ops;
  L->grid = grid;
  L->ws = ws;
  L->prm = prm;
  L->normalise = essential_kind(kind) && !run_only;
  L->split_affine = affine_kind(kind);
  L->total = total;
  L->probs = params->sampler == GCR_SAMPLER_IMPORTANCE ? c->probs : nullptr;
  L->d_corr = d_corr;
  L->num_pairs = (int)num_pairs;
  L->valid = true;
  return GCR_OK;
}

// Device side of a prepared batch: only stream work (a memset and kernel
// launches), so it can be recorded into a CUDA graph.
static gcr_status launch_batch(gcr_context* c, const gcr_context::Pending& L, cudaStream_t s) {
  CUDA_TRY(cudaMemsetAsync(c->ticket.p, 0, sizeof(int), s));
  int launches = 1;
  if (L.normalise) {
    CUDA_TRY(gcr::launch_normalise_essential(L.d_corr, (const double*)c->kinv.p, (const gcr::PairDesc*)c->pairs.p,
                                             L.num_pairs, (double*)c->norm_pts.p, s));
    ++launches;
  }
  if (L.split_affine) {
    double* pts = (double*)c->affine.p;
    CUDA_TRY(gcr::launch_split_affine(L.d_corr, L.total, pts, pts + 4 * std::max<int64_t>(L.total, 1), s));
    ++launches;
  }
  if (L.probs) {
    CUDA_TRY(gcr::launch_importance_cdf(L.probs, (const gcr::PairDesc*)c->pairs.p, L.num_pairs, (double*)c->cdf.p, s));
    ++launches;
  }
  CUDA_TRY(gcr::launch_centre(L.ws, (gcr::PairAux*)c->aux.p, L.num_pairs, s));
  ++launches;
  CUDA_TRY(L.ops->launch(L.grid, s, L.ws, L.prm));
  g_last_launches = launches;
  return GCR_OK;
}

namespace gcr {

// std::discrete_distribution's table (the reference's ImportanceSampler,
// samplers/importance_sampler.h:67-81): p_i / sum p, running sums, the last
// entry 1. One thread per pair, sums in row order (the oracle's order).
__global__ void importance_cdf_kernel(const double* probs, const PairDesc* pairs, int num_pairs, double* cdf) {
  const int pair = blockIdx.x * blockDim.x + threadIdx.x;
  if (pair >= num_pairs) return;
  const PairDesc pd = pairs[pair];
  const double* p = probs + pd.offset;
  double* c = cdf + pd.offset;
  double sum = 0.0;
  for (int i = 0; i < pd.n; ++i) sum += p[i];
  double acc = 0.0;
  for (int i = 0; i < pd.n; ++i) {
    acc += p[i] / sum;
    c[i] = acc;
  }
  if (pd.n > 0) c[pd.n - 1] = 1.0;
}

// Affine correspondences: rows of 8 (x1, y1, x2, y2, a11, a12, a21, a22) into
// the point rows [total][4] and the affine maps [total][4] (grid-stride, two
// 16-byte loads and stores per row when the input is 16-byte aligned).
__global__ void split_affine_kernel(const double* corr8, int64_t total, double* pts, double* aff) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const double* r = corr8 + 8 * i;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      pts[4 * i + k] = r[k];
      aff[4 * i + k] = r[4 + k];
    }
  }
}

cudaError_t launch_split_affine(const double* corr8, int64_t total, double* pts, double* aff, cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((total + 255) / 256, 4096);
  split_affine_kernel<<<(unsigned)blocks, 256, 0, s>>>(corr8, total, pts, aff);
  return cudaGetLastError();
}

// Staging kernel, one CTA per pair (grid-stride over pairs): the centred FP32
// copy of the pair's fitting coordinates into ws.pts32, its largest centred
// magnitude and its non-finite flag into aux.
__global__ void __launch_bounds__(GCR_BLOCK) centre_kernel(Workspace ws, PairAux* aux, int num_pairs) {
  __shared__ double red[GCR_WARPS];
  for (int pair = blockIdx.x; pair < num_pairs; pair += gridDim.x) {
    const PairDesc pd = ws.pairs[pair];
    double mx = 0.0;
    const int bad = load_pair_tile(ws, pd, ws.pts64 + 4 * pd.offset, ws.pts32 + pd.offset, mx);
    const double scale = block_max_abs(mx, red);
    const int any_bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
      PairAux a;
      a.scale = scale;
      a.bad = any_bad ? 1 : 0;
      a.pad = 0;
      aux[pair] = a;
    }
  }
}

cudaError_t launch_centre(const Workspace& ws, PairAux* aux, int num_pairs, cudaStream_t s) {
  const int grid = std::min(num_pairs, 65535);
  centre_kernel<<<grid, GCR_BLOCK, 0, s>>>(ws, aux, num_pairs);
  return cudaGetLastError();
}

cudaError_t launch_importance_cdf(const double* probs, const PairDesc* pairs, int num_pairs, double* cdf,
                                  cudaStream_t s) {
  importance_cdf_kernel<<<(num_pairs + 127) / 128, 128, 0, s>>>(probs, pairs, num_pairs, cdf);
  return cudaGetLastError();
}

}  // namespace gcr

extern "C" {

gcr_status gcr_batch_run_device(gcr_context* c, gcr_model_kind kind, int64_t num_pairs, const double* d_corr,
                                const int64_t* h_offsets, const double* h_K,
                                const gcr_image_size* h_sizes, const gcr_params* params, const uint64_t* h_seeds,
                                double* d_models_out, uint8_t* d_masks_out, gcr_stats* d_stats_out, void* stream) {
  g_last_launches = 0;
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  if (num_pairs <= 0) return GCR_OK;
  cudaStream_t s = (cudaStream_t)stream;
  c->pending.valid = false;  // the scratch a prepared batch refers to may move
  gcr_context::Pending L;
  gcr_status st = prepare_batch(c, kind, num_pairs, d_corr, h_offsets, h_K, h_sizes, params, h_seeds, d_models_out,
                                d_masks_out, d_stats_out, s, &L);
  if (st != GCR_OK || !L.valid) return st;
  return launch_batch(c, L, s);
}

gcr_status gcr_batch_prepare(gcr_context* c, gcr_model_kind kind, int64_t num_pairs, const double* d_corr,
                             const int64_t* h_offsets, const double* h_K, const gcr_image_size* h_sizes,
                             const gcr_params* params, const uint64_t* h_seeds, double* d_models_out,
                             uint8_t* d_masks_out, gcr_stats* d_stats_out) {
  g_last_launches = 0;
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  c->pending.valid = false;
  if (num_pairs <= 0) return fail(GCR_INVALID_ARG, "num_pairs must be positive");
  gcr_status st = prepare_batch(c, kind, num_pairs, d_corr, h_offsets, h_K, h_sizes, params, h_seeds, d_models_out,
                                d_masks_out, d_stats_out, 0, &c->pending);
  if (st != GCR_OK) return st;
  CUDA_TRY(cudaStreamSynchronize(0));
  return GCR_OK;
}

gcr_status gcr_context_set_probabilities(gcr_context* c, const double* d_probabilities) {
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  c->probs = d_probabilities;
  c->pending.valid = false;
  return GCR_OK;
}

gcr_status gcr_context_set_pair_times(gcr_context* c, unsigned long long* d_times) {
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  c->pair_times = d_times;
  return GCR_OK;
}

gcr_status gcr_context_set_flow_step_limit(gcr_context* c, int64_t steps) {
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  if (steps < 0) return fail(GCR_INVALID_ARG, "the step limit must be >= 0 (0 restores the defaults)");
  c->flow_cap = steps;
  c->pending.valid = false;
  return GCR_OK;
}

gcr_status gcr_context_set_sample_tape(gcr_context* c, const int32_t* d_tape, int64_t calls_per_pair) {
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  if (calls_per_pair < 0) return fail(GCR_INVALID_ARG, "calls_per_pair must be >= 0");
  c->tape = calls_per_pair > 0 ? d_tape : nullptr;
  c->tape_calls = c->tape ? calls_per_pair : 0;
  c->pending.valid = false;
  return GCR_OK;
}

gcr_status gcr_context_set_tuning(gcr_context* c, const gcr_tuning* entries, int32_t count) {
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  if (count < 0 || (count > 0 && !entries)) return fail(GCR_INVALID_ARG, "bad tuning table");
  for (int32_t i = 0; i < count; ++i) {
    const gcr_tuning& e = entries[i];
    if (!ops_for((gcr_model_kind)e.kind)) return fail(GCR_INVALID_ARG, "tuning entry %d: unknown kind %d", i, e.kind);
    if (e.batch_calls < 0 || e.batch_calls > GCR_BLOCK)
      return fail(GCR_INVALID_ARG, "tuning entry %d: batch_calls must be in [0, %d]", i, GCR_BLOCK);
    if (e.ctas_per_sm < 0 || e.order < 0 || e.order > 1 || e.max_n < 0)
      return fail(GCR_INVALID_ARG, "tuning entry %d: bad ctas_per_sm, order or max_n", i);
  }
  c->tuning.assign(entries, entries + count);
  c->pending.valid = false;
  return GCR_OK;
}

gcr_status gcr_context_set_lo_precision(gcr_context* c, int32_t precision) {
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  if (precision != GCR_LO_FP64 && precision != GCR_LO_FP32)
    return fail(GCR_INVALID_ARG, "precision must be GCR_LO_FP64 (0) or GCR_LO_FP32 (1)");
  c->lo_fp32 = precision == GCR_LO_FP32 ? 1 : 0;
  c->pending.valid = false;
  return GCR_OK;
}

gcr_status gcr_context_last_tuning(const gcr_context* c, gcr_tuning* out) {
  if (!c || !out) return fail(GCR_INVALID_ARG, "NULL argument");
  *out = c->last_tuning;
  return GCR_OK;
}

gcr_status gcr_set_sample_tape(const int32_t* h_tape, int64_t calls_per_pair) {
  if (calls_per_pair < 0) return fail(GCR_INVALID_ARG, "calls_per_pair must be >= 0");
  g_host_tape = calls_per_pair > 0 ? h_tape : nullptr;
  g_host_tape_calls = g_host_tape ? calls_per_pair : 0;
  return GCR_OK;
}

gcr_status gcr_batch_launch(gcr_context* c, void* stream) {
  g_last_launches = 0;
  if (!c) return fail(GCR_INVALID_ARG, "context is NULL");
  if (!c->pending.valid) return fail(GCR_INVALID_ARG, "no prepared batch on this context (call gcr_batch_prepare)");
  return launch_batch(c, c->pending, (cudaStream_t)stream);
}

gcr_status gcr_find_batch(gcr_model_kind kind, int64_t num_pairs, const double* corr, const int64_t* offsets,
                          const double* K, const gcr_image_size* sizes, const gcr_params* params,
                          const uint64_t* seeds, double* models_out, uint8_t* masks_out, gcr_stats* stats_out) {
  static thread_local gcr_context* ctx = nullptr;
  // arguments first: a bad call returns its status before any device work
  if (!ops_for(kind)) return fail(GCR_UNSUPPORTED, "model kind %d is not provided by this build", (int)kind);
  gcr_status chk = check_params(kind, params);
  if (chk != GCR_OK) return chk;
  if (num_pairs <= 0) return GCR_OK;
  if (!corr || !offsets || !sizes || !models_out || !masks_out || !stats_out)
    return fail(GCR_INVALID_ARG, "NULL buffer");
  if (!ctx) {
    gcr_status s = gcr_context_create(&ctx);
    if (s != GCR_OK) return s;
  }
  const int64_t total = offsets[num_pairs];
  const int cols = kind_columns(kind);
  CUDA_TRY(ctx->corr.ensure(sizeof(double) * cols * (size_t)std::max<int64_t>(total, 1)));
  CUDA_TRY(ctx->models.ensure(sizeof(double) * 9 * num_pairs));
  CUDA_TRY(ctx->masks.ensure((size_t)std::max<int64_t>(total, 1)));
  CUDA_TRY(ctx->stats.ensure(sizeof(gcr_stats) * num_pairs));
  cudaStream_t s = 0;
  CUDA_TRY(cudaMemcpyAsync(ctx->corr.p, corr, sizeof(double) * cols * total, cudaMemcpyHostToDevice, s));
  ctx->probs = nullptr;
  if (g_batch_probs) {
    CUDA_TRY(ctx->probs_stage.ensure(sizeof(double) * (size_t)std::max<int64_t>(total, 1)));
    CUDA_TRY(cudaMemcpyAsync(ctx->probs_stage.p, g_batch_probs, sizeof(double) * total, cudaMemcpyHostToDevice, s));
    ctx->probs = (const double*)ctx->probs_stage.p;
  }
  ctx->tape = nullptr;
  ctx->tape_calls = 0;
  if (g_host_tape) {
    const int m = ops_for(kind)->sample_size;
    const size_t tb = sizeof(int32_t) * (size_t)m * (size_t)g_host_tape_calls * (size_t)num_pairs;
    CUDA_TRY(ctx->tape_stage.ensure(tb));
    CUDA_TRY(cudaMemcpyAsync(ctx->tape_stage.p, g_host_tape, tb, cudaMemcpyHostToDevice, s));
    ctx->tape = (const int32_t*)ctx->tape_stage.p;
    ctx->tape_calls = g_host_tape_calls;
  }
  gcr_status st = gcr_batch_run_device(ctx, kind, num_pairs, (const double*)ctx->corr.p, offsets, K, sizes,
                                       params, seeds, (double*)ctx->models.p, (uint8_t*)ctx->masks.p,
                                       (gcr_stats*)ctx->stats.p, s);
  ctx->tape = nullptr;
  ctx->tape_calls = 0;
  if (st != GCR_OK) return st;
  CUDA_TRY(cudaMemcpyAsync(models_out, ctx->models.p, sizeof(double) * 9 * num_pairs, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(masks_out, ctx->masks.p, (size_t)total, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(stats_out, ctx->stats.p, sizeof(gcr_stats) * num_pairs, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return GCR_OK;
}

static gcr_status find_one(gcr_model_kind kind, const double* corr, int64_t n, const double* K1, const double* K2,
                           const gcr_image_size* size, const double* probabilities, const gcr_params* params,
                           double* model_out9, uint8_t* mask_out, gcr_stats* stats_out) {
  if (!corr || !size || !params || !model_out9 || !mask_out) return fail(GCR_INVALID_ARG, "NULL argument");
  if (!ops_for(kind)) return fail(GCR_UNSUPPORTED, "model kind %d is not provided by this build", (int)kind);
  const int m = ops_for(kind)->sample_size;
  if (n < m) return fail(GCR_TOO_FEW_POINTS, "%lld correspondences, needs >= %d", (long long)n, m);
  const int64_t offsets[2] = {0, n};
  double K[18];
  if (essential_kind(kind)) {
    if (!K1 || !K2) return fail(GCR_INVALID_ARG, "essential matrices need K1 and K2");
    std::memcpy(K, K1, 9 * sizeof(double));
    std::memcpy(K + 9, K2, 9 * sizeof(double));
  }
  gcr_stats st{};
  const uint64_t seed = params->seed;
  const bool weighted = params->sampler == GCR_SAMPLER_IMPORTANCE || params->sampler == GCR_SAMPLER_AR;
  if (weighted && !probabilities)
    return fail(GCR_INVALID_ARG, "samplers 3 and 4 need per-correspondence probabilities");
  g_batch_probs = weighted ? probabilities : nullptr;
  gcr_status rc = gcr_find_batch(kind, 1, corr, offsets, essential_kind(kind) ? K : nullptr, size, params, &seed,
                                 model_out9, mask_out, &st);
  g_batch_probs = nullptr;
  if (rc != GCR_OK) return rc;
  if (stats_out) *stats_out = st;
  if (st.status != GCR_OK) {
    if (st.status == GCR_NO_MODEL) return fail(GCR_NO_MODEL, "no model with more than %d inliers", m);
    return fail((gcr_status)st.status, "device engine reported status %d", st.status);
  }
  return GCR_OK;
}

gcr_status gcr_find_homography(const double* corr, int64_t n, const gcr_image_size* size, const double* probabilities,
                               const gcr_params* params, double* model_out9, uint8_t* mask_out,
                               gcr_stats* stats_out) {
  return find_one(GCR_HOMOGRAPHY, corr, n, nullptr, nullptr, size, probabilities, params, model_out9, mask_out,
                  stats_out);
}

gcr_status gcr_find_fundamental(const double* corr, int64_t n, const gcr_image_size* size,
                                const double* probabilities, const gcr_params* params, double* model_out9,
                                uint8_t* mask_out, gcr_stats* stats_out) {
  return find_one(GCR_FUNDAMENTAL, corr, n, nullptr, nullptr, size, probabilities, params, model_out9, mask_out,
                  stats_out);
}

gcr_status gcr_find_essential(const double* corr, int64_t n, const double* K1, const double* K2,
                              const gcr_image_size* size, const double* probabilities, const gcr_params* params,
                              double* model_out9, uint8_t* mask_out, gcr_stats* stats_out) {
  return find_one(GCR_ESSENTIAL, corr, n, K1, K2, size, probabilities, params, model_out9, mask_out, stats_out);
}

gcr_status gcr_find_homography_affine(const double* corr, int64_t n, const gcr_image_size* size,
                                      const double* probabilities, const gcr_params* params, double* model_out9,
                                      uint8_t* mask_out, gcr_stats* stats_out) {
  return find_one(GCR_HOMOGRAPHY_AFFINE, corr, n, nullptr, nullptr, size, probabilities, params, model_out9,
                  mask_out, stats_out);
}

gcr_status gcr_find_fundamental_affine(const double* corr, int64_t n, const gcr_image_size* size,
                                       const double* probabilities, const gcr_params* params, double* model_out9,
                                       uint8_t* mask_out, gcr_stats* stats_out) {
  return find_one(GCR_FUNDAMENTAL_AFFINE, corr, n, nullptr, nullptr, size, probabilities, params, model_out9,
                  mask_out, stats_out);
}

gcr_status gcr_find_fundamental_sift(const double* corr, int64_t n, const gcr_image_size* size,
                                     const double* probabilities, const gcr_params* params, double* model_out9,
                                     uint8_t* mask_out, gcr_stats* stats_out) {
  return find_one(GCR_FUNDAMENTAL_SIFT, corr, n, nullptr, nullptr, size, probabilities, params, model_out9,
                  mask_out, stats_out);
}

gcr_status gcr_find_essential_planar(const double* corr, int64_t n, const double* K1, const double* K2,
                                     const gcr_image_size* size, const double* probabilities, const gcr_params* params,
                                     double* model_out9, uint8_t* mask_out, gcr_stats* stats_out) {
  return find_one(GCR_ESSENTIAL_PLANAR, corr, n, K1, K2, size, probabilities, params, model_out9, mask_out,
                  stats_out);
}

gcr_status gcr_find_homography_sift(const double* corr, int64_t n, const gcr_image_size* size,
                                    const double* probabilities, const gcr_params* params, double* model_out9,
                                    uint8_t* mask_out, gcr_stats* stats_out) {
  return find_one(GCR_HOMOGRAPHY_SIFT, corr, n, nullptr, nullptr, size, probabilities, params, model_out9,
                  mask_out, stats_out);
}

}  // extern "C"

// GCRANSAC::run on one pair (gcr_run and gcr_run_with_probabilities):
// `probabilities` [n] (host) or NULL feed the importance and AR samplers.
static gcr_status run_single(gcr_model_kind kind, const double* points, const double* pixels, int64_t n,
                             const double* cell_sizes, int32_t divisions, const gcr_image_size* size,
                             const double* probabilities, const gcr_params* params, double* model_out9,
                             uint8_t* mask_out, gcr_stats* stats_out) {
  static thread_local gcr_context* ctx = nullptr;
  g_last_launches = 0;
  if (!points || !cell_sizes || !size || !params || !model_out9 || !mask_out)
    return fail(GCR_INVALID_ARG, "NULL argument");
  if (!ops_for(kind)) return fail(GCR_UNSUPPORTED, "model kind %d is not provided by this build", (int)kind);
  const int m = ops_for(kind)->sample_size;
  if (n < m) return fail(GCR_TOO_FEW_POINTS, "%lld points, needs >= %d", (long long)n, m);
  if (divisions < 1) return fail(GCR_INVALID_ARG, "the grid needs at least one division per axis");
  for (int q = 0; q < 4; ++q)
    if (!(cell_sizes[q] > 0)) return fail(GCR_INVALID_ARG, "grid cell sizes must be positive");
  if (!ctx) {
    gcr_status s0 = gcr_context_create(&ctx);
    if (s0 != GCR_OK) return s0;
  }
  cudaStream_t s = 0;
  const size_t bytes = sizeof(double) * 4 * (size_t)n;
  // points and pixels share one staging buffer: [points | pixels]
  CUDA_TRY(ctx->corr.ensure(2 * bytes));
  CUDA_TRY(ctx->models.ensure(sizeof(double) * 9));
  CUDA_TRY(ctx->masks.ensure((size_t)n));
  CUDA_TRY(ctx->stats.ensure(sizeof(gcr_stats)));
  double* d_pts = (double*)ctx->corr.p;
  double* d_pix = d_pts + 4 * n;
  CUDA_TRY(cudaMemcpyAsync(d_pts, points, bytes, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(d_pix, pixels ? pixels : points, bytes, cudaMemcpyHostToDevice, s));
  ctx->probs = nullptr;
  if (probabilities) {
    CUDA_TRY(ctx->probs_stage.ensure(sizeof(double) * (size_t)n));
    CUDA_TRY(cudaMemcpyAsync(ctx->probs_stage.p, probabilities, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    ctx->probs = (const double*)ctx->probs_stage.p;
  }
  ctx->tape = nullptr;
  ctx->tape_calls = 0;
  if (g_host_tape) {
    const size_t tb = sizeof(int32_t) * (size_t)m * (size_t)g_host_tape_calls;
    CUDA_TRY(ctx->tape_stage.ensure(tb));
    CUDA_TRY(cudaMemcpyAsync(ctx->tape_stage.p, g_host_tape, tb, cudaMemcpyHostToDevice, s));
    ctx->tape = (const int32_t*)ctx->tape_stage.p;
    ctx->tape_calls = g_host_tape_calls;
  }
  RunOnly ro;
  ro.d_pixels = d_pix;
  for (int q = 0; q < 4; ++q) ro.cell[q] = cell_sizes[q];
  ro.divisions = divisions;
  const int64_t offsets[2] = {0, n};
  const uint64_t seed = params->seed;
  ctx->pending.valid = false;
  gcr_context::Pending L;
  gcr_status st = prepare_batch(ctx, kind, 1, d_pts, offsets, nullptr, size, params, &seed, (double*)ctx->models.p,
                                (uint8_t*)ctx->masks.p, (gcr_stats*)ctx->stats.p, s, &L, &ro);
  if (st != GCR_OK) return st;
  ctx->tape = nullptr;
  ctx->tape_calls = 0;
  st = launch_batch(ctx, L, s);
  if (st != GCR_OK) return st;
  gcr_stats so{};
  CUDA_TRY(cudaMemcpyAsync(model_out9, ctx->models.p, sizeof(double) * 9, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(mask_out, ctx->masks.p, (size_t)n, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(&so, ctx->stats.p, sizeof(gcr_stats), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (stats_out) *stats_out = so;
  if (so.status != GCR_OK) {
    if (so.status == GCR_NO_MODEL) return fail(GCR_NO_MODEL, "no model with more than %d inliers", m);
    return fail((gcr_status)so.status, "device engine reported status %d", so.status);
  }
  return GCR_OK;
}

extern "C" {

gcr_status gcr_run(gcr_model_kind kind, const double* points, const double* pixels, int64_t n,
                   const double* cell_sizes, int32_t divisions, const gcr_image_size* size,
                   const gcr_params* params, double* model_out9, uint8_t* mask_out, gcr_stats* stats_out) {
  if (params && (params->sampler == GCR_SAMPLER_IMPORTANCE || params->sampler == GCR_SAMPLER_AR))
    return fail(GCR_INVALID_ARG, "samplers 3 and 4 need probabilities: use gcr_run_with_probabilities");
  return run_single(kind, points, pixels, n, cell_sizes, divisions, size, nullptr, params, model_out9, mask_out,
                    stats_out);
}

gcr_status gcr_run_with_probabilities(gcr_model_kind kind, const double* points, const double* pixels, int64_t n,
                                      const double* cell_sizes, int32_t divisions, const gcr_image_size* size,
                                      const double* probabilities, const gcr_params* params, double* model_out9,
                                      uint8_t* mask_out, gcr_stats* stats_out) {
  if (!probabilities) return fail(GCR_INVALID_ARG, "probabilities is NULL");
  for (int64_t i = 0; i < n; ++i)
    if (!(probabilities[i] >= 0.0) || !std::isfinite(probabilities[i]))
      return fail(GCR_INVALID_ARG, "probability %lld is negative or not finite", (long long)i);
  return run_single(kind, points, pixels, n, cell_sizes, divisions, size, probabilities, params, model_out9,
                    mask_out, stats_out);
}

}  // extern "C"

namespace gcr {
// Kinds not compiled into this build.
__attribute__((weak)) const KindOps* fundamental_ops() { return nullptr; }
__attribute__((weak)) const KindOps* essential_ops() { return nullptr; }
__attribute__((weak)) const KindOps* homography_affine_ops() { return nullptr; }
__attribute__((weak)) const KindOps* fundamental_affine_ops() { return nullptr; }
__attribute__((weak)) const KindOps* fundamental_sift_ops() { return nullptr; }
__attribute__((weak)) const KindOps* homography_sift_ops() { return nullptr; }
__attribute__((weak)) const KindOps* essential_planar_ops() { return nullptr; }
}  // namespace gcr
