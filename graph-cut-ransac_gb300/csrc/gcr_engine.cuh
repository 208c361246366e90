// Persistent CTA-per-pair Graph-Cut RANSAC engine.
//
// One CTA owns one image pair at a time and runs the whole
// hypothesize-and-verify loop of GCRANSAC::run (src/pygcransac/include/GCRANSAC.h:200-627)
// for it:
//   * batched sampling + minimal solves, one sampler call per thread;
//   * an FP32 scoring pass of every hypothesis against every correspondence
//     held in shared memory, with an FP64 re-check of points inside the FP32
//     error band so that inlier counts are exact;
//   * an ordered commit that replays the reference's sequential decisions
//     (strict score comparison, validity, adaptive iteration count, LO trigger)
//     with FP64 scores for every hypothesis that may beat the best one;
//   * graph-cut local optimisation (GCRANSAC.h:779-1021): the labelling graph of
//     the grid neighbourhood is a disjoint union of one clique per grid cell, so
//     every cell is an independent s-t min-cut solved by one warp with
//     push-relabel;
//   * the final iterated least squares (GCRANSAC.h:629-758).
//
// Control flow: every thread executes the sequential decision logic on
// thread-private copies of the scalar state; every input of a decision is
// CTA-uniform, so all threads take the same branches and meet at the same
// barriers inside the CTA-collective operations.
#pragma once

#include "gcr_device.cuh"
#include "gcr_essential.cuh"
#include "gcr_fundamental.cuh"
#include "gcr_homography.cuh"
#include "gcr_linalg.cuh"
#include "gcr_lo_f32.cuh"

namespace gcr {

constexpr int kMaxFlowCap = 256;        // largest grid cell solved by one warp
constexpr long long kFlowOpsCap = 20000000;  // push/relabel steps per cell before TIMEOUT
constexpr double kResidualEps = 1e-12;  // residual capacity treated as saturated
#ifndef GCR_TILE_POINTS
#define GCR_TILE_POINTS 4096
#endif
constexpr int kSmemPoints = GCR_TILE_POINTS;  // correspondences kept resident in shared memory
constexpr int kLoRegion = GCR_BLOCK;    // model slots reserved for local optimisation

enum PairStatus {
  ST_OK = 0,
  ST_INVALID_ARG = 1,   // a coordinate of the pair is not finite
  ST_NO_MODEL = 3,
  ST_DEVICE_ERROR = 4,  // an internal consistency check failed (a row index outside the pair)
  ST_TIMEOUT = 5,
  ST_CAPACITY = 6,
  ST_UNSUPPORTED = 7
};

enum { SAMPLER_UNIFORM = 0, SAMPLER_PROSAC = 1, SAMPLER_PNAPSAC = 2, SAMPLER_IMPORTANCE = 3, SAMPLER_AR = 4 };
constexpr uint32_t kStreamAr = 6;  // jitter draws of the AR sampler
enum { SCORING_MSAC = 0, SCORING_MAGSAC = 1 };

struct EngineParams {
  double confidence;
  double lambda;        // spatial coherence weight
  int64_t max_iters;
  int64_t min_iters;
  int32_t lo_number;
  int32_t sampler;
  int32_t scoring;
  int32_t num_pairs;
  int32_t max_n;
  // nested runs (DEGENSAC's plane-and-parallax GC-RANSAC): one sampler stream
  // shared by the main loop and the local optimisation, results kept in
  // shared memory instead of the outputs
  int32_t nested;
  uint32_t stream_main;
  uint32_t stream_lo;
  const double* pp_h;   // homography of the plane-and-parallax solver (nested runs)
  // MAGSAC++ scoring (scoring == 1): the weight table Gamma(1.5, x / 1000),
  // x = 0..36000, and the constants C 2^1.5, Gamma(1.5) - gamma_k, gamma_k,
  // all evaluated on the host
  const double* mag_table;
  // importance sampler: per-pair cumulative normalised probabilities [total]
  const double* cdf;
  // neighbourhood: 0 the grid; 1 the radius graph (FlannNeighborhoodGraph's
  // ball of radius sqrt(radius2) in the four pixel coordinates), whose
  // per-CTA scratch follows
  int32_t neighborhood;
  double radius2;
  int32_t rg_cap;        // edge capacity per CTA
  int32_t rg_stride_n;   // max_n + 1
  int* rg_int;           // per CTA: nb_start, rev_start [rg_stride_n]; nb_idx, rev_edge, edge_src [rg_cap];
                         // height, queue, mark [rg_stride_n]
  double* rg_dbl;        // per CTA: cap_f, cap_b [rg_cap]; excess, cap_t, back_s [rg_stride_n]
  float4* rg_px;         // per CTA: FP32 copy of the pixel coordinates [rg_stride_n]
  // AR sampler: the caller's probabilities [total], the estimator variance
  // and per CTA a max-heap of (probability, point) [ar_cap] plus the
  // per-point a, b [2 * ar_stride_n] and appearance counts [ar_stride_n]
  const double* probs;
  double sampler_variance;
  double* ar_p;
  int* ar_i;
  double* ar_ab;
  int* ar_cnt;
  int32_t ar_cap;
  int32_t ar_stride_n;
  double mag_c2dof;
  double mag_gamma_diff;
  double mag_gamma_k;
  // SPRT preemptive verification of main-loop models
  int32_t use_sprt;
  double sprt_min_ratio;
  // space-partitioning pre-selection of homography models
  int32_t use_sp;
  // graph cuts per run (GCRANSAC::settings.max_graph_cut_number) and the
  // final iteratively reweighted fit (do_final_iterated_least_squares)
  int32_t gc_max;
  int32_t final_irls;
  // 1: the Python drivers' epilogue after the run (bundle adjustment of the
  // final inliers for F and E); 0: GCRANSAC::run alone
  int32_t epilogue;
  // push / relabel steps of one labelling flow problem before the pair
  // reports ST_TIMEOUT; 0 for the defaults (kFlowOpsCap per grid cell, 2^24
  // on the radius graph)
  long long flow_cap;
  // recorded main-sampler samples replacing the sampler's draws (null: the
  // sampler draws): [num_pairs][tape_calls][M] point indices
  const int32_t* tape;
  long long tape_calls;
  // sampler calls (hypotheses) drawn, solved and scored per batch, 1..GCR_BLOCK;
  // calls are counter-based and replayed in call order, so any batch size
  // gives the same results (a tuning knob)
  int32_t batch_calls;
  // 1: the local optimisation's fundamental-matrix fits in FP32 (lo32::
  // fit_fundamental); 0: in FP64, the oracle's arithmetic (parity)
  int32_t lo_fp32;
};

// Per-pair inputs prepared on the device.
struct PairDesc {
  int64_t offset;       // first row in the concatenated arrays
  int32_t n;
  int32_t n_div;        // grid divisions along every axis
  double threshold;     // threshold in the coordinates the model is fitted in
  double cell[4];       // grid cell sizes (pixel coordinates)
  double centre[4];     // centring of the FP32 copy
  double img[4];        // image sizes w1, h1, w2, h2 (P-NAPSAC grids)
  uint64_t seed;
};

// Device mirror of gcr_stats (include/gcr.h).
struct StatsOut {
  int64_t iteration_number;
  int64_t graph_cut_number;
  int64_t local_optimization_number;
  int64_t inlier_number;
  double score;
  int32_t status;
  int32_t flags;
  int64_t models_scored;
};

// Per-CTA scratch in global memory (one slot per resident CTA).
struct Slot {
  double* models64;     // [kModels][9]
  float* models32;      // [kModels][12]
  int* samples;         // [GCR_BLOCK][SAMPLE_CAP] local-optimisation samples
  int* bsamples;        // [GCR_BLOCK][M] minimal samples of the current batch
  int* list0;           // [max_n]
  int* list1;           // [max_n]
  int* list2;           // [max_n]
  uint8_t* flag;        // [max_n]
  double* dres;         // [max_n]
  double* tr;           // [max_n]
  unsigned long long* sortbuf;  // [pow2 >= max_n]
  int* cell_pts;        // [max_n]
  int* cell_start;      // [max_n + 1]
  double* flow;         // [GCR_WARPS][kMaxFlowCap^2]
  double* node_d;       // [GCR_WARPS][3 * kMaxFlowCap]  excess, sink residual, scratch
  int* node_i;          // [GCR_WARPS][3 * kMaxFlowCap]  height, queue, mark
  double* red;          // [GCR_WARPS * 64 + 64] reduction partials
  int* napsac;          // [16][max_n] P-NAPSAC layers (sorted points, cell start, cell size per point)
  int* sprt_pool;       // [max_n] SPRT's point order
  double* sprt_buf;     // [GCR_BLOCK] squared residual of a chunk's inliers, -1 for outliers
  int* sp_cell;         // [max_n] grid cell of each sorted position
  int* sp_flag;         // [max_n] cell kept by the space partitioning of the current model
  int* sp_sel;          // [max_n] points of the kept cells, cell by cell
                        // x4, hits, subset sizes, layers, growth table
};

// Per-pair results of the staging kernel (centre_kernel): the largest
// centred magnitude of the pair's coordinates (the FP32 error bounds scale
// with it) and whether a coordinate is not finite.
struct PairAux {
  double scale;
  int32_t bad;
  int32_t pad;
};

struct Workspace {
  const double* pts64;  // [total][4] coordinates the model is fitted in
  const double* pix64;  // [total][4] pixel coordinates for the grid
  float4* pts32;        // [total] centred FP32 copy of pts64, written by centre_kernel before the engine runs
  const PairDesc* pairs;
  Slot* slots;
  Slot* nested_slots;   // light slots of DEGENSAC's inner run (fundamental matrices)
  int* ticket;
  double* models_out;   // [P][9]
  uint8_t* masks_out;   // [total]
  StatsOut* stats_out;  // [P]
  long long* phase;     // [P][16] phase cycle counters (GCR_PHASE_PROFILE builds), else null
  unsigned long long* times;  // [P][2] global timer (ns) when a CTA takes the pair and when it is done, or null
  const int* order;     // [P] pair of each work ticket (largest pairs first), or null for ticket order
  const PairAux* aux;   // [P] staging results (centre_kernel)
  const double* affine64;  // [total][4] local affine maps (a11, a12, a21, a22) of affine correspondences, or null
};

struct Score {
  int count;
  double value;
};

// A container of the reference's temp_inner_inliers: the inlier set of one
// model, kept as (pointer to that model, inlier count).
struct Container {
  const double* model;
  int count;
  // SPRT containers list the inliers among SPRT-pool positions
  // [start, start + len) in pool order; start < 0: all points, index order
  int start = -1;
  int len = 0;
};

template <class Est>
struct Shared {
  // local-optimisation region: one model per trial, or the models of 25
  // trials when a non-minimal fit returns up to ten (a larger region would
  // leave room for only one CTA per SM)
  static constexpr int kLo = kLoRegion;
  static constexpr int kModels = GCR_BLOCK * Est::MAXSOL + kLo;
  // staging of per-trial model lists of multi-model non-minimal fits (global only)
  static constexpr int kStage = Est::LO_MAXSOL > 1 ? GCR_BLOCK : 0;
  static constexpr int kMulti = Est::LO_MAXSOL;
  double best_model[9];
  double cont_model[2][9];
  double lo_best_model[9];
  double work_model[9];
  double fit_model[9];
  float mf32[12];                 // FP32 form of the model being scored exactly
  double red_d[GCR_WARPS * 48];
  int red_i[GCR_WARPS + 2];
  int n_ok[GCR_BLOCK];
  int mbase[GCR_BLOCK];
  int mcount[kModels];
  float mscore[kModels];
  float mbound[kModels];
  int s_cnt[GCR_BLOCK];
  float s_sum[GCR_BLOCK];
  float s_err[GCR_BLOCK];
  int lo_ok[GCR_BLOCK];
  int lo_base[GCR_BLOCK];
  double multi_models[9 * kMulti];  // models of the last CTA-wide multi-model fit
  int multi_count;
  double lm_f[19];                // factorised F (U, V, sigma) of the CTA-wide LM
  double lm_fn[19];
  double lm_G[9];
  double lm_D[63];
  double lm_acc[35];
  double degen_H[9];
  double pp_H[9];                 // homography of the plane-and-parallax solver
  double result_model[9];         // model of a nested run
  int result_count;               // inlier count of a nested run
  int lm_flag;
  int fit_ok;
  int flow_status;
  int bad_row;                    // a row index read from a list fell outside the pair
  int ar_size;                    // entries in the AR sampler's heap
  int ar_overflow;
  int big_cells;                  // grid cells of the current labelling above kMaxFlowCap points
  int out_tmax[33];               // source-set size of a cell of n <= 32 points all beyond the threshold
};

// Whether a model kind runs DEGENSAC's plane check in its validity test:
// the fundamental-matrix estimator does for minimal samples of 7 or more
// (fundamental_estimator.h:326), so not for three affine correspondences.
template <class Est>
__host__ __device__ constexpr bool has_degensac() {
  if constexpr (Est::KIND == 1) return Est::DEGENSAC;
  else return false;
}

// Whether a fundamental-matrix kind's non-minimal solver is the bundle
// adjustment (8-point start, then Levenberg-Marquardt) or the plain 8-point
// solver (the affine-correspondence estimator, types.h:83-86).
template <class Est>
__host__ __device__ constexpr bool nonminimal_lm() {
  if constexpr (Est::KIND == 1) return Est::NONMIN_LM;
  else return false;
}

// Models per minimal sample in SPRT's cost model: the minimal solver's
// declared maximumSolutions (preemption_sprt.h:134). Every homography solver
// declares one, the two-SIFT solver although its two conics meet in up to
// four points (solver_homography_two_sift.h:83-86).
template <class Est>
__host__ __device__ constexpr int sprt_solutions() {
  if constexpr (Est::KIND == 0) return 1;
  else if constexpr (Est::KIND == 3) return Est::DECLARED_SOLUTIONS;
  else return Est::MAXSOL;
}

// Whether an essential-matrix kind's non-minimal solver is the bundle
// adjustment solver (the planar-motion estimator, types.h:121-126).
template <class Est>
__host__ __device__ constexpr bool nonmin_ba() {
  if constexpr (Est::KIND == 3) return Est::NONMIN_BA;
  else return false;
}

// GCRANSAC::getIterationNumber (GCRANSAC.h:156-172)
__device__ __forceinline__ long long iteration_number_for(long long inliers, long long points, int m,
                                                          double log_prob) {
  const double q = pow((double)inliers / (double)points, (double)m);
  const double l2 = log(1 - q);
  if (fabs(l2) < 2.220446049250313e-16) return 0x7fffffffffffffffLL;
  const double iter = log_prob / l2;
  if (!(iter < 9.2e18)) return 0x7fffffffffffffffLL;
  return (long long)iter + 1;
}

template <class Est>
struct Engine {
  static constexpr int m = Est::M;
  static constexpr int kModels = Shared<Est>::kModels;
  static constexpr int kBatchModels = GCR_BLOCK * Est::MAXSOL;

  Shared<Est>& sh;
  const Workspace& ws;
  const EngineParams& prm;
  const PairDesc& pd;
  const Slot& slot;
  int pair;
  const double* pts64;
  const double* affine64;  // this pair's local affine maps (affine correspondences), or null
  const float4* pts32;   // shared-memory or global FP32 copy of this pair
  double scale = 1.0;    // max |centred coordinate| of this pair
  int N;
  double t2;
  double log_prob;
  // MAGSAC++ scoring (MAGSACScoringFunction::getScore, scoring_function.h:
  // 237-348): inlier iff r <= threshold, weight from the gamma table
  bool mag = false;
  double mag_thr = 0, mag_thr2 = 0, mag_sq2 = 0, mag_oos = 0, mag_w0 = 0;
  // space partitioning (homographies): cells of the grid kept for a model
  bool sp = false;
  int sp_ncells = 0;
  int sp_count = 0;  // points in the kept cells of the last selection
  // SPRT state (identical in every thread)
  bool sprt = false;
  int sprt_cursor = 0;
  double sprt_eps = 0, sprt_delta = 0, sprt_A = 0, sprt_tM = 1, sprt_mS = 1;
  int status = ST_OK;
  int flags = 0;

  // sequential state (identical in every thread)
  long long iter = 0, max_iter = 0, gc_number = 0, lo_number = 0, lo_calls = 0;
  long long models_scored = 0;  // models the sequential algorithm scores in full
  long long degensac_calls = 0;  // DEGENSAC inner runs so far (their sampler streams)
  Shared<PlaneParallaxModel>* nsh = nullptr;  // state of DEGENSAC's inner run
  Slot nslot{};
  Score best{0, 0.0};
  Container cont[2];
  int off = 0;

  __device__ Engine(Shared<Est>& s, const Workspace& w, const EngineParams& p, const PairDesc& d, const Slot& sl,
                    int pair_)
      : sh(s), ws(w), prm(p), pd(d), slot(sl), pair(pair_) {
    N = pd.n;
    pts64 = ws.pts64 + 4 * pd.offset;
    affine64 = ws.affine64 ? ws.affine64 + 4 * pd.offset : nullptr;
    const double tt = 1.5 * pd.threshold;
    t2 = tt * tt;
    log_prob = log(1.0 - prm.confidence);
    if (prm.scoring == SCORING_MAGSAC && prm.mag_table != nullptr) {
      mag = true;
      mag_thr = pd.threshold;
      mag_thr2 = mag_thr * mag_thr;
      mag_sq2 = mag_thr * mag_thr * 2.0;
      mag_oos = prm.mag_c2dof / mag_thr;
      mag_w0 = mag_oos * prm.mag_gamma_diff;
    }
    cont[0] = {nullptr, 0};
    cont[1] = {nullptr, 0};
  }

  __device__ __forceinline__ void sync() { __syncthreads(); }

  // Optional per-phase cycle counters (built with -DGCR_PHASE_PROFILE).
  __device__ __forceinline__ long long tick() const {
#ifdef GCR_PHASE_PROFILE
    return clock64();
#else
    return 0;
#endif
  }
  __device__ __forceinline__ void tock(int id, long long t0, long long count = -1) const {
#ifdef GCR_PHASE_PROFILE
    if (threadIdx.x == 0 && ws.phase) ws.phase[pair * 16 + id] += count >= 0 ? count : clock64() - t0;
#else
    (void)id; (void)t0; (void)count;
#endif
  }

  // Row `idx` of the pair's fitting coordinates, for indices read from lists:
  // an index outside [0, N) is recorded (the pair then reports
  // ST_DEVICE_ERROR) and row 0 is read instead of memory beyond the pair.
  __device__ __forceinline__ const double* row64(int idx) const {
    if ((unsigned)idx >= (unsigned)N) {
      sh.bad_row = 1;
      idx = 0;
    }
    return pts64 + 4 * idx;
  }
  __device__ __forceinline__ bool row_ok(int idx) const {
    if ((unsigned)idx < (unsigned)N) return true;
    sh.bad_row = 1;
    return false;
  }

  // thread 0 copies 9 doubles; everyone waits
  __device__ void copy_model(double* dst, const double* src) {
    sync();
    if (threadIdx.x < 9) dst[threadIdx.x] = src[threadIdx.x];
    sync();
  }

  // ------------------------------------------------------------------
  // FP32 scoring of models [k0, k0 + K) of the slot table. Writes exact inlier
  // counts (points inside the FP32 error band are re-decided in FP64) and an
  // FP32 MSAC score with an upper bound of its error.
  __device__ void score_models_f32(int k0, int K) {
    const float tf = (float)sqrt(t2);
    const float t2f = (float)t2;
    // the FP32 thresholds are rounded: widen every band by their rounding
    const float slack = 1.2e-7f * (mag ? (float)mag_thr2 : t2f);
    const int tid = threadIdx.x;
    for (int base = 0; base < K; base += GCR_BLOCK) {
      const int Kb = min(GCR_BLOCK, K - base);
      const int KP = (Kb + 31) & ~31;
      const int S = GCR_BLOCK / KP;
      const int slice = tid / KP, mi = tid % KP;
      int cnt = 0;
      float sum = 0.f, err = 0.f;
      if (slice < S && mi < Kb) {
        const int k = k0 + base + mi;
        float h[9];
        const float* src = slot.models32 + 12 * k;
#pragma unroll
        for (int q = 0; q < 9; ++q) h[q] = src[q];
        const float cm = src[9];
        const double* m64 = slot.models64 + 9 * k;
        const int chunk = (N + S - 1) / S;
        const int i0 = slice * chunk, i1 = min(N, i0 + chunk);
        float inner = 0.f;
        int inner_n = 0;
        if (!mag) {
          for (int i = i0; i < i1; ++i) {
            const float4 p = pts32[i];
            float it;
            const float r2 = Est::r2_f32(p, h, it);
            const float e = fmaf(cm, fabsf(it), cm);
            const float eb = fmaf(e, e, 2.f * tf * e) + slack;
            const float dlt = r2 - t2f;
            if (dlt < -eb) {
              ++cnt;
              inner += r2;
              err += eb;
            } else if (!(dlt > eb)) {  // inside the band, or NaN
              const double r2d = Est::r2_f64(pts64 + 4 * i, m64);
              if (r2d < t2) {
                ++cnt;
                inner += (float)r2d;
              }
            }
            if (++inner_n == 64) {
              sum += inner;
              inner = 0.f;
              inner_n = 0;
            }
          }
          sum += inner;
        } else {
          // MAGSAC++: sum of normalised weights; the FP32 residual may move the
          // table index by 1e4 eb / (2 thr^2) + 1 bins, each worth at most
          // 5e-4 of normalised weight
          const float mt = (float)mag_thr, mt2 = (float)mag_thr2;
          const float xs = (float)(1e4 / mag_sq2);
          const float gk = (float)prm.mag_gamma_k, gdi = (float)(1.0 / prm.mag_gamma_diff);
          for (int i = i0; i < i1; ++i) {
            const float4 p = pts32[i];
            float it;
            const float r2 = Est::r2_f32(p, h, it);
            const float e = fmaf(cm, fabsf(it), cm);
            const float eb = fmaf(e, e, 2.f * mt * e) + slack;
            const float dlt = r2 - mt2;
            if (dlt < -eb) {
              ++cnt;
              const int x = min(36000, (int)roundf(r2 * xs));
              inner += ((float)prm.mag_table[x] - gk) * gdi;
              err += fmaf(eb, xs, 1.f) * 5e-4f;
            } else if (!(dlt > eb)) {
              const double r2d = Est::r2_f64(pts64 + 4 * i, m64);
              const double r = sqrt(r2d);
              if (!(r > mag_thr)) {
                ++cnt;
                inner += (float)mag_weight(r);
              }
            }
            if (++inner_n == 64) {
              sum += inner;
              inner = 0.f;
              inner_n = 0;
            }
          }
          sum += inner;
        }
      }
      sh.s_cnt[tid] = cnt;
      sh.s_sum[tid] = sum;
      sh.s_err[tid] = err;
      sync();
      if (tid < Kb) {
        int c = 0;
        float s = 0.f, e = 0.f;
        for (int q = 0; q < S; ++q) {
          c += sh.s_cnt[q * KP + tid];
          s += sh.s_sum[q * KP + tid];
          e += sh.s_err[q * KP + tid];
        }
        const int k = k0 + base + tid;
        sh.mcount[k] = c;
        if (!mag) {
          sh.mscore[k] = c == 0 ? 0.f : (c * t2f - s) / t2f;
          // per-point residual error + FP32 summation error + the final division
          sh.mbound[k] = (e + 2.f * s * (64.f + (float)N / 64.f) * 5.97e-8f) / t2f + 4e-7f * c + 1e-6f;
        } else {
          sh.mscore[k] = s;
          sh.mbound[k] = e + 2.f * s * (64.f + (float)N / 64.f) * 5.97e-8f + 1e-5f * c + 1e-6f;
        }
      }
      sync();
    }
  }

  // FP32 form of `model` in sh.mf32 (thread 0, then everyone waits).
  __device__ void prepare_shared_f32(const double* model) {
    sync();
    if (threadIdx.x == 0) Est::prepare_f32(model, pd.centre, scale, sh.mf32);
    sync();
  }

  // Exact FP64 MSAC score (scoring_function.h:137-233) of a model; optionally
  // writes the inlier list in index order. Points whose FP32 residual lies
  // above the threshold by more than its error bound are outliers without an
  // FP64 evaluation; all others are decided and summed in FP64.
  // MAGSAC++ weight of a correspondence at residual r <= threshold, divided by
  // the weight at zero residual.
  __device__ __forceinline__ double mag_weight(double r) const {
    double w;
    if (r < 2.220446049250313e-16) {
      w = mag_w0;
    } else {
      long long x = (long long)round(1e4 * (r * r) / mag_sq2);
      if (36000 < x) x = 36000;
      w = mag_oos * (prm.mag_table[x] - prm.mag_gamma_k);
    }
    return w / mag_w0;
  }

  __device__ Score exact_score(const double* model, int* list, const float* m32 = nullptr, bool msac = false) {
    if (mag && !msac) return exact_score_magsac(model, list, m32);
    if (m32 == nullptr) {
      prepare_shared_f32(model);
      m32 = sh.mf32;
    }
    double h[9];
    float hf[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      h[q] = model[q];
      hf[q] = m32[q];
    }
    const float cm = m32[9];
    const float tf = (float)sqrt(t2), t2f = (float)t2;
    double acc = 0.0;
    int total = 0;
    for (int base = 0; base < N; base += GCR_BLOCK) {
      const int i = base + threadIdx.x;
      int f = 0;
      if (i < N) {
        float it;
        const float r2f = Est::r2_f32(pts32[i], hf, it);
        const float e = fmaf(cm, fabsf(it), cm);
        const float eb = fmaf(e, e, 2.f * tf * e) + 1.2e-7f * t2f;
        if (!(r2f - t2f > eb)) {
          const double r2 = Est::r2_f64(pts64 + 4 * i, h);
          if (r2 < t2) {
            f = 1;
            acc -= r2;
          }
        }
      }
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (list && f) list[total + pos] = i;
      total += tot;
    }
    const double s = block_sum(acc, sh.red_d);
    Score sc;
    sc.count = total;
    sc.value = total == 0 ? 0.0 : (s + total * t2) / t2;
    return sc;
  }

  // MAGSACScoringFunction::getScore: inlier iff r <= threshold, value = sum
  // of normalised weights (points whose FP32 residual lies above the
  // threshold by more than its error bound are skipped).
  __device__ Score exact_score_magsac(const double* model, int* list, const float* m32) {
    if (m32 == nullptr) {
      prepare_shared_f32(model);
      m32 = sh.mf32;
    }
    double h[9];
    float hf[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      h[q] = model[q];
      hf[q] = m32[q];
    }
    const float cm = m32[9];
    const float mt = (float)mag_thr, mt2 = (float)mag_thr2;
    double acc = 0.0;
    int total = 0;
    for (int base = 0; base < N; base += GCR_BLOCK) {
      const int i = base + threadIdx.x;
      int f = 0;
      if (i < N) {
        float it;
        const float r2f = Est::r2_f32(pts32[i], hf, it);
        const float e = fmaf(cm, fabsf(it), cm);
        const float eb = fmaf(e, e, 2.f * mt * e) + 1.2e-7f * mt2;
        if (!(r2f - mt2 > eb)) {
          const double r = sqrt(Est::r2_f64(pts64 + 4 * i, h));
          if (!(r > mag_thr)) {
            f = 1;
            acc += mag_weight(r);
          }
        }
      }
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (list && f) list[total + pos] = i;
      total += tot;
    }
    Score sc;
    sc.count = total;
    sc.value = block_sum(acc, sh.red_d);
    return sc;
  }

  __device__ void put_f32(int k) {
    Est::prepare_f32(slot.models64 + 9 * k, pd.centre, scale, slot.models32 + 12 * k);
  }

  // Is `cand` (FP32 score + bound of model k) possibly better than `ref`?
  __device__ __forceinline__ bool maybe_better(int k, double ref) const {
    return (double)sh.mscore[k] + (double)sh.mbound[k] >= ref;
  }

  // ------------------------------------------------------------------
  // Grid neighbourhood: points sorted by (cell key, index); cell_start holds
  // the cell boundaries. Returns the number of cells.
  // Points sorted by (cell key, index) for a grid of the given cell sizes and
  // radix (GridNeighborhoodGraph<4>::initialize, grid_neighborhood_graph.h:230-292:
  // idx_d = floor(coord_d / cell_d), key = sum_d idx_d * nd^d). Writes the
  // sorted point list and the cell boundaries; returns the number of cells.
  __device__ int sort_cells(const double* cell, uint64_t nd, int* sorted, int* starts) {
    unsigned long long* a = slot.sortbuf;
    const double* pix = ws.pix64 + 4 * pd.offset;
    int sort_n = 1;
    while (sort_n < N) sort_n <<= 1;
    for (int i = threadIdx.x; i < sort_n; i += GCR_BLOCK) {
      if (i < N) {
        const double* p = pix + 4 * i;
        uint64_t key = 0, o = 1;
        for (int d = 0; d < 4; ++d) {
          const uint64_t idx = (uint64_t)(int64_t)floor(p[d] / cell[d]);
          key += o * idx;
          o *= nd;
        }
        a[i] = ((key & 0xFFFFFFFFFFull) << 24) | (unsigned long long)i;
      } else {
        a[i] = ~0ull;
      }
    }
    sync();
    block_bitonic_sort(a, sort_n);
    int ncells = 0;
    for (int base = 0; base < N; base += GCR_BLOCK) {
      const int i = base + threadIdx.x;
      int f = 0;
      if (i < N) {
        sorted[i] = (int)(a[i] & 0xFFFFFFull);
        f = (i == 0) || ((a[i] >> 24) != (a[i - 1] >> 24));
      }
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (f) starts[ncells + pos] = i;
      ncells += tot;
    }
    if (threadIdx.x == 0) starts[ncells] = N;
    sync();
    return ncells;
  }

  __device__ int build_grid() { return sort_cells(pd.cell, (uint64_t)pd.n_div, slot.cell_pts, slot.cell_start); }

  // ------------------------------------------------------------------
  // ProgressiveNapsacSampler<4> (samplers/progressive_napsac_sampler.h:50-326)
  // with the driver's layers {16, 8, 4, 2} and length 0.5 N
  // (gcransac_python.cpp:4333-4343). Its state evolves call by call (hit
  // counters of the points), so thread 0 draws a batch sequentially.
  struct Napsac {
    long long kth = 0, max_iters = 0;
    long long local_calls = 0, global_calls = 0;
    // lazily extended P-NAPSAC growth table
    int growth_n = 0;
    double T_n = 0;
    unsigned int T_prime = 1;
    // global PROSAC (sample size m, convergence N)
    long long g_kth = 1, g_subset = 0, g_hi = 0, g_growth = 1;
    double g_Tn = 0;
    // one-point PROSAC of the centre points (sample size 1, convergence N):
    // call index, subset size, growth[subset - 1] and T_n of the recurrence
    long long op_kth = 1, op_subset = 1, op_growth = 1;
    double op_Tn = 0;
  };
  Napsac ns;

  __device__ int* nl_sorted(int l) const { return slot.napsac + (size_t)(3 * l) * N; }
  __device__ int* nl_start(int l) const { return slot.napsac + (size_t)(3 * l + 1) * N; }
  __device__ int* nl_size(int l) const { return slot.napsac + (size_t)(3 * l + 2) * N; }
  __device__ int* n_hits() const { return slot.napsac + (size_t)12 * N; }
  __device__ int* n_subset() const { return slot.napsac + (size_t)13 * N; }
  __device__ int* n_layer() const { return slot.napsac + (size_t)14 * N; }
  __device__ unsigned int* n_growth() const { return (unsigned int*)(slot.napsac + (size_t)15 * N); }

  __device__ void napsac_setup() {
    const int divs[4] = {16, 8, 4, 2};
    for (int l = 0; l < 4; ++l) {
      double cs[4];
      for (int d = 0; d < 4; ++d) cs[d] = pd.img[d] / (double)divs[l];
      const int nc = sort_cells(cs, (uint64_t)divs[l], nl_sorted(l), slot.cell_start);
      // per point: start and size of its cell in the sorted list
      for (int c = threadIdx.x; c < nc; c += GCR_BLOCK) {
        const int s0 = slot.cell_start[c], s1 = slot.cell_start[c + 1];
        for (int i = s0; i < s1; ++i) {
          const int p = nl_sorted(l)[i];
          nl_start(l)[p] = s0;
          nl_size(l)[p] = s1 - s0;
        }
      }
      sync();
    }
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) {
      n_hits()[i] = 0;
      n_subset()[i] = m;
      n_layer()[i] = 0;
    }
    ns.kth = 0;
    ns.max_iters = (long long)(0.5 * (double)N);
    ns.local_calls = ns.global_calls = 0;
    // P-NAPSAC growth function: local sample size m - 1
    const int ls = m - 1;
    double T = (double)ns.max_iters;
    for (int i = 0; i < ls; ++i) T *= (double)(ls - i) / (double)(N - i);
    ns.T_n = T;
    ns.T_prime = 1;
    ns.growth_n = 0;
    // global PROSAC
    ns.g_kth = 1;
    ns.g_subset = m;
    ns.g_hi = m - 1;
    ns.g_growth = 1;
    double Tg = (double)N;
    for (int i = 0; i < m; ++i) Tg *= (double)(m - i) / (double)(N - i);
    ns.g_Tn = Tg;
    // the centre sampler's growth recurrence starts from N * (1 / N), which
    // rounds below 1 for many N: its growth function then steps by 2 once and
    // a centre point is returned twice, so it is followed exactly
    ns.op_kth = 1;
    ns.op_subset = 1;
    ns.op_growth = 1;
    double To = (double)N;
    To *= 1.0 / (double)N;
    ns.op_Tn = To;
    sync();
  }

  // growth_function_progressive_napsac[i], extended on demand (thread 0)
  __device__ unsigned int napsac_growth(int i) {
    const int ls = m - 1;
    unsigned int* g = n_growth();
    while (ns.growth_n <= i) {
      const int k = ns.growth_n;
      if (k + 1 <= ls) {
        g[k] = ns.T_prime;
      } else {
        const double Tn1 = (double)(k + 1) * ns.T_n / (double)(k + 1 - ls);
        g[k] = ns.T_prime + (unsigned int)(size_t)ceil(Tn1 - ns.T_n);
        ns.T_n = Tn1;
        ns.T_prime = g[k];
      }
      ++ns.growth_n;
    }
    return g[i];
  }

  // global ProsacSampler(sample size m, convergence N): setSampleNumber(k)
  // then sample (prosac_sampler.h:177-236); thread 0
  __device__ bool napsac_global(long long k, int* s) {
    // growth[subset - 1] of this sampler is tracked in g_growth
    auto grow = [&]() {
      const long long before = ns.g_subset;
      ++ns.g_subset;
      if (ns.g_subset > N) ns.g_subset = N;
      ns.g_hi = ns.g_subset - 2;
      if (ns.g_subset != before) {
        const long long i = ns.g_subset - 1;
        if (i + 1 > m) {
          const double Tn1 = (double)(i + 1) * ns.g_Tn / (double)(i + 1 - m);
          ns.g_growth = ns.g_growth + (long long)(unsigned int)ceil(Tn1 - ns.g_Tn);
          ns.g_Tn = Tn1;
        }
      }
    };
    ns.g_kth = k;
    bool global = false;
    if (ns.g_kth > N) {
      global = true;
    } else {
      while (ns.g_kth > ns.g_growth && ns.g_subset != N) grow();
    }
    DrawStream ds(pd.seed, STREAM_NAPSAC_GLOBAL, (uint64_t)(ns.global_calls++));
    bool ok;
    if (global) {
      ok = unique_set(ds, s, m, 0, (uint32_t)(N - 1));
    } else {
      ok = unique_set(ds, s, m - 1, 0, (uint32_t)ns.g_hi);
      s[m - 1] = (int)(ns.g_subset - 1);
      // incrementIterationNumber
      ++ns.g_kth;
      if (!(ns.g_kth > N) && ns.g_kth > ns.g_growth) grow();
    }
    return ok;
  }

  // One P-NAPSAC call (thread 0). Returns false when the sampler fails.
  __device__ bool napsac_call(int* s) {
    ++ns.kth;
    if (ns.kth > ns.max_iters) return napsac_global(ns.kth, s);
    // one-point PROSAC of sample size 1 and convergence N
    // (prosac_sampler.h:65-87, 199-236; its random range is empty before
    // convergence, which the local phase never reaches): the call returns
    // point subset - 1, then the subset grows past growth[subset - 1]
    const int initial = (int)(ns.op_subset - 1);
    ++ns.op_kth;
    if (ns.op_kth > ns.op_growth && ns.op_subset < N) {
      ++ns.op_subset;
      const long long i = ns.op_subset - 1;  // >= 1: past the sample size
      const double Tn1 = (double)(i + 1) * ns.op_Tn / (double)i;
      ns.op_growth = ns.op_growth + (long long)(unsigned int)ceil(Tn1 - ns.op_Tn);
      ns.op_Tn = Tn1;
    }
    int* hits = n_hits();
    const int h = ++hits[initial];
    int ss = n_subset()[initial];
    while ((unsigned int)h > napsac_growth(ss - 1) && ss < N) ss = min(ss + 1, N);
    n_subset()[initial] = ss;
    int layer = n_layer()[initial];
    bool last = false;
    for (;;) {
      if (layer >= 4) {
        last = true;
        break;
      }
      if (nl_size(layer)[initial] < ss) {
        ++layer;
        continue;
      }
      break;
    }
    n_layer()[initial] = layer;
    if (last) {
      const bool ok = napsac_global(ns.kth, s);
      s[m - 1] = initial;
      return ok;
    }
    const int* nb = nl_sorted(layer) + nl_start(layer)[initial];
    s[m - 1] = initial;
    s[m - 2] = nb[ss - 1];
    // generateUniqueRandomSet(subset, m - 2, ss - 2, initial): the local
    // index is compared with the point index `initial`, as in the reference
    DrawStream ds(pd.seed, STREAM_NAPSAC_LOCAL, (uint64_t)(ns.local_calls++));
    const uint32_t hi = (uint32_t)(ss - 2);
    for (int i = 0; i < m - 2; ++i) {
      s[i] = (int)ds.next_in(0, hi);
      if (s[i] == initial) { --i; continue; }
      for (int j = i - 1; j >= 0; --j)
        if (s[i] == s[j]) { --i; break; }
      if (ds.d > (1u << 20)) return false;
    }
    for (int i = 0; i < m - 2; ++i) {
      s[i] = nb[s[i]];
      ++hits[s[i]];
    }
    ++hits[s[m - 2]];
    return true;
  }

  // ------------------------------------------------------------------
  // s-t min cut of one grid cell (a clique plus terminal arcs) by one warp.
  // The labelling graph is built as in GCRANSAC::labeling (GCRANSAC.h:945-1007)
  // with Energy::add_term1/add_term2 (energy.h:203-253): node i of the cell
  // gets the terminal capacity tr_i = unary_i - sum_{j>i} lambda (d_i + d_j)/2,
  // the arc i->j (i < j) lambda - lambda (d_i + d_j)/2 and the arc j->i lambda.
  // FIFO push-relabel with exact initial distance labels computes a maximum
  // preflow; then a backward search from the sink over residuals above
  // kResidualEps marks the SINK side (what_segment == SINK, graph.h:478-483).
  // Writes slot.flag[point] for the cell's points. Returns false on the step cap.
  // Comparisons of non-negative doubles through their bit patterns (IEEE order
  // equals integer order for non-negative values) keep the residual tests off
  // the FP64 pipe.
  __device__ __forceinline__ static bool dpos(double x) { return __double_as_longlong(x) > 0; }
  __device__ __forceinline__ static bool dgt(double x, double y) {
    return __double_as_longlong(x) > __double_as_longlong(y);
  }
  __device__ __forceinline__ static bool dlt(double x, double y) {
    return __double_as_longlong(x) < __double_as_longlong(y);
  }

  __device__ bool mincut_cell(int c0, int n, int warp) {
    const int lane = threadIdx.x & 31;
    const double lam = prm.lambda;
    double* R = slot.flow + (size_t)warp * kMaxFlowCap * kMaxFlowCap;
    double* ex = slot.node_d + (size_t)warp * 3 * kMaxFlowCap;
    double* sr = ex + kMaxFlowCap;
    int* h = slot.node_i + (size_t)warp * 3 * kMaxFlowCap;
    int* q = h + kMaxFlowCap;
    int* mark = q + kMaxFlowCap;
    const int* gp = slot.cell_pts + c0;
    const double* d = slot.dres;
    for (int e = lane; e < n * n; e += 32) {
      const int i = e / n, j = e - i * n;
      double v = 0.0;
      if (i < j) v = lam - (0.5 * (d[gp[i]] + d[gp[j]])) * lam;
      else if (i > j) v = lam;
      R[e] = v;
    }
    for (int i = lane; i < n; i += 32) {
      double t = slot.tr[gp[i]];
      const double di = d[gp[i]];
      for (int j = i + 1; j < n; ++j) t = t - (0.5 * (di + d[gp[j]])) * lam;
      ex[i] = t > 0 ? t : 0.0;
      sr[i] = t < 0 ? -t : 0.0;
      mark[i] = 0;
    }
    __syncwarp();
    const int dead = n + 2;
    // exact distance labels: backward BFS from the sink over residual arcs
    for (int i = lane; i < n; i += 32) h[i] = dpos(sr[i]) ? 1 : dead;
    __syncwarp();
    for (int level = 1; level <= n; ++level) {
      bool grew = false;
      for (int u = lane; u < n; u += 32) {
        if (h[u] != dead) continue;
        for (int v = 0; v < n; ++v)
          if (h[v] == level && dpos(R[u * n + v])) {
            h[u] = -(level + 1);
            break;
          }
      }
      __syncwarp();
      for (int u = lane; u < n; u += 32)
        if (h[u] < 0) {
          h[u] = -h[u];
          grew = true;
        }
      __syncwarp();
      if (!__any_sync(0xffffffffu, grew)) break;
    }
    // FIFO of active nodes (positive excess and a finite label)
    int qh = 0, qt = 0;
    for (int base = 0; base < n; base += 32) {
      const int u = base + lane;
      const bool act = u < n && dpos(ex[u]) && h[u] < dead;
      const unsigned b = __ballot_sync(0xffffffffu, act);
      if (act) {
        q[(qt + __popc(b & ((1u << lane) - 1))) % kMaxFlowCap] = u;
        mark[u] = 1;
      }
      qt += __popc(b);
    }
    __syncwarp();
    long long ops = 0;
    const long long ops_cap = prm.flow_cap > 0 ? prm.flow_cap : kFlowOpsCap;
    bool ok = true;
    while (qh != qt) {
      const int u = q[qh % kMaxFlowCap];
      ++qh;
      __syncwarp();
      if (lane == 0) mark[u] = 0;
      __syncwarp();
      for (;;) {
        if (++ops > ops_cap) { ok = false; break; }
        double e = ex[u];
        const int hu = h[u];
        if (!dpos(e) || hu >= dead) break;
        if (hu == 1 && dpos(sr[u])) {
          __syncwarp();
          if (lane == 0) {
            const double s = sr[u];
            const double dl = dlt(e, s) ? e : s;
            ex[u] = e - dl;
            sr[u] = s - dl;
          }
          __syncwarp();
          e = ex[u];
          if (!dpos(e)) break;
        }
        for (int base = 0; base < n && dpos(e); base += 32) {
          const int v = base + lane;
          const bool adm = v < n && v != u && h[v] == hu - 1 && dpos(R[u * n + v]);
          unsigned b = __ballot_sync(0xffffffffu, adm);
          while (b != 0u && dpos(e)) {
            const int vv = base + __ffs(b) - 1;
            b &= b - 1;
            int enq = 0;
            __syncwarp();
            if (lane == 0) {
              const double r = R[u * n + vv];
              const double dl = dlt(e, r) ? e : r;
              R[u * n + vv] = r - dl;
              R[vv * n + u] = R[vv * n + u] + dl;
              ex[u] = e - dl;
              ex[vv] = ex[vv] + dl;
              if (!mark[vv] && h[vv] < dead) {
                mark[vv] = 1;
                q[qt % kMaxFlowCap] = vv;
                enq = 1;
              }
            }
            enq = __shfl_sync(0xffffffffu, enq, 0);
            qt += enq;
            __syncwarp();
            e = ex[u];
          }
        }
        if (!dpos(e)) break;
        // relabel: 1 + min label over residual arcs (the sink has label 0)
        int mn = dpos(sr[u]) ? 0 : 0x7fffffff;
        for (int v = lane; v < n; v += 32)
          if (v != u && dpos(R[u * n + v]) && h[v] < mn) mn = h[v];
        mn = warp_min(mn);
        __syncwarp();
        if (lane == 0) h[u] = (mn == 0x7fffffff || mn + 1 >= dead) ? dead : mn + 1;
        __syncwarp();
      }
      if (!ok) break;
    }
    __syncwarp();
    // SINK side: backward search from the sink over residuals > kResidualEps
    for (int i = lane; i < n; i += 32) mark[i] = dgt(sr[i], kResidualEps) ? 1 : 0;
    __syncwarp();
    for (int round = 0; round < n; ++round) {
      bool grew = false;
      for (int u = lane; u < n; u += 32) {
        if (mark[u]) continue;
        for (int v = 0; v < n; ++v)
          if (mark[v] == 1 && dgt(R[u * n + v], kResidualEps)) {
            mark[u] = 2;
            break;
          }
      }
      __syncwarp();
      for (int u = lane; u < n; u += 32)
        if (mark[u] == 2) {
          mark[u] = 1;
          grew = true;
        }
      __syncwarp();
      if (!__any_sync(0xffffffffu, grew)) break;
    }
    for (int i = lane; i < n; i += 32) slot.flag[gp[i]] = (uint8_t)mark[i];
    __syncwarp();
    return ok;
  }

  // GCRANSAC::labeling (GCRANSAC.h:912-1021): writes the SINK points in index
  // order into `list` and returns their number.
  // ------------------------------------------------------------------
  // Radius neighbourhood (FlannNeighborhoodGraph, neighborhood/
  // flann_neighborhood_graph.h:100-139, with an exact search): the edges
  // {i, j}, j > i, whose squared 4-D pixel distance ((a^2 + b^2) + c^2) + d^2,
  // every operation rounded, is at most radius2. An FP32 pass with a margin
  // picks the candidates, FP64 decides. Edges are stored by i (ascending j) and
  // indexed by j for the flow. Returns false when they exceed the capacity.
  __device__ __forceinline__ int* rg_i(int k) const {
    return prm.rg_int + (size_t)blockIdx.x * (2 * (size_t)prm.rg_stride_n * 1 + 3 * (size_t)prm.rg_cap +
                                              3 * (size_t)prm.rg_stride_n) + k;
  }
  __device__ __forceinline__ int* rg_nb_start() const { return rg_i(0); }
  __device__ __forceinline__ int* rg_rev_start() const { return rg_i(prm.rg_stride_n); }
  __device__ __forceinline__ int* rg_nb_idx() const { return rg_i(2 * prm.rg_stride_n); }
  __device__ __forceinline__ int* rg_rev_edge() const { return rg_i(2 * prm.rg_stride_n + prm.rg_cap); }
  __device__ __forceinline__ int* rg_edge_src() const { return rg_i(2 * prm.rg_stride_n + 2 * prm.rg_cap); }
  __device__ __forceinline__ int* rg_height() const { return rg_i(2 * prm.rg_stride_n + 3 * prm.rg_cap); }
  __device__ __forceinline__ int* rg_queue() const { return rg_i(3 * prm.rg_stride_n + 3 * prm.rg_cap); }
  __device__ __forceinline__ int* rg_mark() const { return rg_i(4 * prm.rg_stride_n + 3 * prm.rg_cap); }
  __device__ __forceinline__ double* rg_d(int k) const {
    return prm.rg_dbl + (size_t)blockIdx.x * (2 * (size_t)prm.rg_cap + 3 * (size_t)prm.rg_stride_n) + k;
  }
  __device__ __forceinline__ double* rg_cap_f() const { return rg_d(0); }
  __device__ __forceinline__ double* rg_cap_b() const { return rg_d(prm.rg_cap); }
  __device__ __forceinline__ double* rg_excess() const { return rg_d(2 * prm.rg_cap); }
  __device__ __forceinline__ double* rg_cap_t() const { return rg_d(2 * prm.rg_cap + prm.rg_stride_n); }
  __device__ __forceinline__ double* rg_back_s() const { return rg_d(2 * prm.rg_cap + 2 * prm.rg_stride_n); }

  __device__ __forceinline__ bool rg_within(int i, int j, const float4& pi, const float4& pj, float r2f) const {
    const float a = pj.x - pi.x, b = pj.y - pi.y, c = pj.z - pi.z, d = pj.w - pi.w;
    const float d2f = a * a + b * b + c * c + d * d;
    if (d2f > r2f) return false;
    const double* pix = ws.pix64 + 4 * pd.offset;
    const double* p = pix + 4 * i;
    const double* q = pix + 4 * j;
    const double da = q[0] - p[0], db = q[1] - p[1], dc = q[2] - p[2], dd = q[3] - p[3];
    const double d2 =
        __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(da, da), __dmul_rn(db, db)), __dmul_rn(dc, dc)), __dmul_rn(dd, dd));
    return d2 <= prm.radius2;
  }

  bool rg_ok = false;  // the radius graph of this pair is built
  __device__ bool build_radius_graph() {
    float4* px = prm.rg_px + (size_t)blockIdx.x * prm.rg_stride_n;
    const double* pix = ws.pix64 + 4 * pd.offset;
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) {
      const double* p = pix + 4 * i;
      px[i] = make_float4((float)p[0], (float)p[1], (float)p[2], (float)p[3]);
    }
    sync();
    // FP32 candidates: the FP32 distance of a pair within the radius is at
    // most radius2 (1 + 1e-5) + 1e-3 (coordinates below 1e6 px)
    const float r2f = (float)(prm.radius2 * (1.0 + 1e-5) + 1e-3);
    int* start = rg_nb_start();
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) {
      const float4 pi = px[i];
      int cnt = 0;
      for (int j = i + 1; j < N; ++j)
        if (rg_within(i, j, pi, px[j], r2f)) ++cnt;
      start[i + 1] = cnt;
    }
    sync();
    if (threadIdx.x == 0) {
      start[0] = 0;
      long long acc = 0;
      for (int i = 1; i <= N; ++i) {
        acc += start[i];
        start[i] = acc > 0x7fffffff ? 0x7fffffff : (int)acc;
      }
      sh.flow_status = acc > prm.rg_cap ? 1 : 0;
    }
    sync();
    if (sh.flow_status) return false;
    const int E = start[N];
    int* nb = rg_nb_idx();
    int* src = rg_edge_src();
    int* rstart = rg_rev_start();
    for (int i = threadIdx.x; i <= N; i += GCR_BLOCK) rstart[i] = 0;
    sync();
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) {
      const float4 pi = px[i];
      int pos = start[i];
      for (int j = i + 1; j < N; ++j)
        if (rg_within(i, j, pi, px[j], r2f)) {
          nb[pos] = j;
          src[pos] = i;
          ++pos;
          atomicAdd(&rstart[j + 1], 1);
        }
    }
    sync();
    if (threadIdx.x == 0)
      for (int i = 1; i <= N; ++i) rstart[i] += rstart[i - 1];
    sync();
    // edges by their second endpoint (order within a list does not matter)
    int* cursor = rg_queue();
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) cursor[i] = rstart[i];
    sync();
    int* rev = rg_rev_edge();
    for (int e = threadIdx.x; e < E; e += GCR_BLOCK) rev[atomicAdd(&cursor[nb[e]], 1)] = e;
    sync();
    return true;
  }

  // Labelling on the radius graph (GCRANSAC.h:912-1021): the pairwise terms of
  // the edges (capacities lambda - A forward, lambda backward, A taken from the
  // first endpoint's terminal weight, in ascending neighbour order), then a
  // FIFO push-relabel maximum flow on one thread and the nodes that still
  // reach the sink through residuals above kResidualEps (the minimal sink
  // side). Bounded: past 2^24 push / relabel steps the pair reports a timeout.
  __device__ void radius_mincut() {
    const int* start = rg_nb_start();
    const int* nb = rg_nb_idx();
    double* cf = rg_cap_f();
    double* cb = rg_cap_b();
    double* ex = rg_excess();
    double* ct = rg_cap_t();
    double* bs = rg_back_s();
    const double lam = prm.lambda;
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) {
      double tri = slot.tr[i];
      const double di = slot.dres[i];
      for (int e = start[i]; e < start[i + 1]; ++e) {
        const double A = 0.5 * (di + slot.dres[nb[e]]) * lam;
        tri = tri - A;
        cf[e] = lam - A;
        cb[e] = lam;
      }
      ex[i] = tri > 0 ? tri : 0.0;   // source arc saturated by the preflow
      bs[i] = ex[i];                 // residual back to the source
      ct[i] = tri < 0 ? -tri : 0.0;  // sink arc
    }
    sync();
    if (threadIdx.x == 0) {
      const int* rstart = rg_rev_start();
      const int* rev = rg_rev_edge();
      const int* src = rg_edge_src();
      int* h = rg_height();
      int* q = rg_queue();
      int* inq = rg_mark();
      const int hs = N + 1;  // height of the source (nodes 0..N-1, sink at 0)
      int qh = 0, qt = 0, qn = 0;
      for (int i = 0; i < N; ++i) {
        h[i] = 0;
        inq[i] = 0;
        if (ex[i] > 0) {
          q[qt] = i;
          qt = qt + 1 == N ? 0 : qt + 1;
          ++qn;
          inq[i] = 1;
        }
      }
      long long steps = 0;
      const long long steps_cap = prm.flow_cap > 0 ? prm.flow_cap : (1ll << 24);
      bool ok = true;
      while (qn > 0) {
        const int u = q[qh];
        qh = qh + 1 == N ? 0 : qh + 1;
        --qn;
        inq[u] = 0;
        while (ex[u] > 0) {
          if (++steps > steps_cap || h[u] > 2 * N + 2) {
            ok = false;
            break;
          }
          int hmin = 0x7fffffff;
          // to the sink
          if (ct[u] > 0) {
            if (h[u] == 1) {
              const double d = fmin(ex[u], ct[u]);
              ct[u] -= d;
              ex[u] -= d;
              if (ex[u] <= 0) break;
            } else hmin = min(hmin, 0);
          }
          // forward edges u -> v
          for (int e = start[u]; e < start[u + 1] && ex[u] > 0; ++e) {
            if (!(cf[e] > 0)) continue;
            const int v = nb[e];
            if (h[u] == h[v] + 1) {
              const double d = fmin(ex[u], cf[e]);
              cf[e] -= d;
              cb[e] += d;
              ex[u] -= d;
              ex[v] += d;
              if (!inq[v]) {
                q[qt] = v;
                qt = qt + 1 == N ? 0 : qt + 1;
                ++qn;
                inq[v] = 1;
              }
            } else hmin = min(hmin, h[v]);
          }
          // backward edges u -> w (edges (w, u), residual cap_b)
          for (int k = rstart[u]; k < rstart[u + 1] && ex[u] > 0; ++k) {
            const int e = rev[k];
            if (!(cb[e] > 0)) continue;
            const int w = src[e];
            if (h[u] == h[w] + 1) {
              const double d = fmin(ex[u], cb[e]);
              cb[e] -= d;
              cf[e] += d;
              ex[u] -= d;
              ex[w] += d;
              if (!inq[w]) {
                q[qt] = w;
                qt = qt + 1 == N ? 0 : qt + 1;
                ++qn;
                inq[w] = 1;
              }
            } else hmin = min(hmin, h[w]);
          }
          // back to the source
          if (ex[u] > 0 && bs[u] > 0) {
            if (h[u] == hs + 1) {
              const double d = fmin(ex[u], bs[u]);
              bs[u] -= d;
              ex[u] -= d;
            } else hmin = min(hmin, hs);
          }
          if (ex[u] > 0) {
            if (hmin == 0x7fffffff) {  // no residual arc: cannot happen for a preflow
              ok = false;
              break;
            }
            h[u] = hmin + 1;
          }
        }
        if (!ok) break;
      }
      // minimal sink side: reverse search from the sink over residuals
      for (int i = 0; i < N; ++i) inq[i] = 0;
      qt = 0;
      for (int i = 0; i < N; ++i)
        if (ct[i] > kResidualEps) {
          inq[i] = 1;
          q[qt++] = i;
        }
      for (int k = 0; k < qt; ++k) {
        const int v = q[k];
        // u -> v residuals: forward edges (u, v) [cap_f], backward of (v, u) [cap_b]
        for (int r = rstart[v]; r < rstart[v + 1]; ++r) {
          const int e = rev[r];
          const int u = src[e];
          if (!inq[u] && cf[e] > kResidualEps) {
            inq[u] = 1;
            q[qt++] = u;
          }
        }
        for (int e = start[v]; e < start[v + 1]; ++e) {
          const int u = nb[e];
          if (!inq[u] && cb[e] > kResidualEps) {
            inq[u] = 1;
            q[qt++] = u;
          }
        }
      }
      for (int i = 0; i < N; ++i) slot.flag[i] = (uint8_t)inq[i];
      if (!ok) sh.flow_status = ST_TIMEOUT;
    }
  }

  // ------------------------------------------------------------------
  // Minimum cut of one grid cell of 2..32 points by the closed form of
  // clique_cut_cta (below, where the energy is derived), one warp and one
  // point per lane, everything in registers: the inliers' keys sorted by a
  // warp bitonic network, the prefix sums of d by a warp scan, the energy of
  // every source-set size t on lane t. The arithmetic follows clique_cut_cta
  // step for step, so both give the same cut. Writes slot.flag for the
  // cell's points.
  // The largest minimising source-set size of a clique of n points that all
  // lie beyond the threshold (d = 1, a = -(1 - lambda)): the energies of
  // clique_cut_warp with no inliers, E(t) = t c' + lambda t (n - t) with
  // c' = lambda (t - 1) / 2 - (1 - lambda). One thread per n.
  __device__ int outlier_clique_tmax(int n) const {
    if (n < 2) return 0;
    const double lam = prm.lambda;
    const double oml = 1.0 - lam;
    double e[33];
    double fmin = 0.0;
    for (int t = 0; t <= n; ++t) {
      const double c = 0.5 * lam * (double)(t - 1);
      const double ko = c - oml;
      const double S = 0.0 + (double)t * ko;
      e[t] = t == 0 ? 0.0 : S + lam * (double)t * (double)(n - t);
      fmin = e[t] < fmin ? e[t] : fmin;
    }
    const double tol = 1e-12 * (1.0 + oml * n + 0.5 * lam * (double)(n - 1) * 0.0 + 0.25 * lam * (double)n * n);
    int tmax = 0;
    for (int t = 0; t <= n; ++t)
      if (e[t] <= fmin + tol) tmax = t;
    return tmax;
  }

  __device__ void clique_cut_warp(int c0, int n) {
    constexpr unsigned kAll = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const double lam = prm.lambda;
    const double oml = 1.0 - lam;
    const int* gp = slot.cell_pts + c0;
    const bool live = lane < n;
    const int p = live ? gp[lane] : 0;
    const double trv = live ? slot.tr[p] : 1.0;
    const double dv = live ? slot.dres[p] : 0.0;
    const bool inl = live && !(trv > 0);
    const unsigned b_in = __ballot_sync(kAll, inl);
    const unsigned b_out = __ballot_sync(kAll, live && trv > 0);
    const int m = __popc(b_in);
    const int n_out = n - m;
    if (m == 0) {
      // every point beyond the threshold: one shared key, the cut depends on n
      // only (sh.out_tmax, the same energies with no inliers)
      if (live) slot.flag[p] = lane < sh.out_tmax[n] ? 0 : 1;
      return;
    }
    const int ib = 32 - __clz(n);
    const unsigned long long low = (1ull << ib) - 1ull;
    unsigned long long key =
        inl ? ((((unsigned long long)__double_as_longlong(dv)) << 2) & ~low) | (unsigned long long)lane : ~0ull;
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
      for (int j = k >> 1; j > 0; j >>= 1) {
        const unsigned long long o = __shfl_xor_sync(kAll, key, j);
        const bool keep_min = ((lane & k) == 0) == ((lane & j) == 0);
        key = keep_min ? (o < key ? o : key) : (o > key ? o : key);
      }
    // lane r: the inlier of rank r (ascending d), its d and the exclusive
    // prefix sum of d over the ranks
    const int owner = (int)(key & low) & 31;
    const double dsh = __shfl_sync(kAll, dv, owner);
    const double v = lane < m ? dsh : 0.0;
    double x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(kAll, x, o);
      if (lane >= o) x += y;
    }
    const double Dex = 0.0 + (x - v);
    const double Dm = __shfl_sync(kAll, x, 31);
    auto pref = [&](int j) {  // every lane calls it (shuffle)
      const double s = __shfl_sync(kAll, Dex, j & 31);
      return j >= m ? Dm : s;
    };
    auto inl_sum = [&](int j, double sl) {
      const double a = pref(j), b = pref(m - j);
      return sl >= 0 ? oml * j + sl * a : oml * j + sl * (Dm - b);
    };
    auto count_le = [&](double sl, double ko) {  // inliers with key <= ko
      int lo = 0, hi = m;
#pragma unroll
      for (int it = 0; it < 6; ++it) {
        const int mid = (lo + hi) >> 1;
        const double d = __shfl_sync(kAll, v, (sl >= 0 ? mid : m - 1 - mid) & 31);
        if (lo < hi) {
          if (oml + sl * d <= ko) lo = mid + 1;
          else hi = mid;
        }
      }
      return lo;
    };
    auto energy = [&](int t) -> double {  // every lane calls it; t may exceed n (ignored)
      const double c = 0.5 * lam * (double)(t - 1);
      const double sl = c - oml, ko = c - oml;
      const int J = count_le(sl, ko);
      const double s1 = inl_sum(t, sl);
      const double s2 = inl_sum(J, sl) + (double)(t - J) * ko;
      const double s3 = inl_sum(t - n_out, sl) + (double)n_out * ko;
      const double S = t <= J ? s1 : (t <= J + n_out ? s2 : s3);
      return t == 0 ? 0.0 : S + lam * (double)t * (double)(n - t);
    };
    const double e0 = energy(lane);
    const double e1 = n == 32 ? energy(32) : 0.0;  // t = 32, a full cell
    double fmin = 0.0;
    if (lane <= n) fmin = e0 < fmin ? e0 : fmin;
    if (n == 32) fmin = e1 < fmin ? e1 : fmin;
    fmin = warp_min(fmin);
    const double tol = 1e-12 * (1.0 + oml * n + 0.5 * lam * (double)(n - 1) * Dm + 0.25 * lam * (double)n * n);
    int tmax = 0;
    if (lane <= n && e0 <= fmin + tol) tmax = lane;
    if (n == 32 && e1 <= fmin + tol) tmax = 32;
    tmax = -warp_min(-tmax);
    const double c = 0.5 * lam * (double)(tmax - 1);
    const double sl = c - oml;
    const int J = count_le(sl, sl);
    const int in_T = tmax == 0 ? 0 : (tmax <= J ? tmax : (tmax <= J + n_out ? J : tmax - n_out));
    const int out_T = tmax - in_T;
    if (lane < m) {
      const int r = sl >= 0 ? lane : m - 1 - lane;
      slot.flag[gp[owner]] = r < in_T ? 0 : 1;
    }
    if (live && trv > 0) {
      const int pos = __popc(b_out & ((1u << lane) - 1u));
      slot.flag[p] = pos < out_T ? 0 : 1;
    }
  }

  // ------------------------------------------------------------------
  // Minimum cut of one grid cell of n > kMaxFlowCap points by its closed form
  // (the whole CTA; `scratch` holds n ints and is free during the cut).
  //
  // A cell is a clique. With label 1 = SINK (inlier), 0 = SOURCE, the unary
  // energies of GCRANSAC::labeling (GCRANSAC.h:945-961; a point's terminal
  // capacity tr_i = E1_i - E0_i) and the pairwise terms of every pair of the
  // cell (add_term2(i, j, lambda (d_i + d_j) / 2, lambda, lambda, 0),
  // GCRANSAC.h:965-1007), the energy of a source set T of t points is
  //   E(T) = sum_i E1_i + sum_{i in T} (a_i + c_t d_i) + lambda t (n - t),
  //   a_i = -tr_i,  c_t = lambda (t - 1) / 2,
  // because the pairs inside T cost lambda (d_i + d_j) / 2 each and the
  // mixed pairs lambda. For a fixed t the best T is the t points of smallest
  // key a_i + c_t d_i, and the keys have a simple order: every point beyond the
  // threshold has d = 1 and a = -(1 - lambda) (one shared key), and every
  // point within it has a = (1 - lambda)(1 - d), a key monotone in d. So after
  // one sort of the inliers by d, the minimum over all T of each size t is a
  // prefix sum, and the cut is the size of lowest energy. The maximum flow's
  // SINK side (what_segment, graph.h:478-483) is the smallest minimising sink
  // set, i.e. the largest minimising T: the largest t whose energy is within
  // rounding of the minimum. Writes slot.flag for the cell's points.
  __device__ void clique_cut_cta(int c0, int n, int* scratch) {
    const double lam = prm.lambda;
    const double oml = 1.0 - lam;
    const int* gp = slot.cell_pts + c0;
    const int tid = threadIdx.x;
    // inliers (tr <= 0) of the cell: keys = (d bits, cell position); the d
    // bits of d in [0, 1] order like d, their two top bits are zero, and the
    // low bits the position needs are dropped
    const int ib = 32 - __clz(n);
    const unsigned long long low = (1ull << ib) - 1ull;
    unsigned long long* keys = slot.sortbuf;
    int m = 0;
    for (int base = 0; base < n; base += GCR_BLOCK) {
      const int k = base + tid;
      int f = 0;
      if (k < n) f = slot.tr[gp[k]] > 0 ? 0 : 1;
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (f) {
        const unsigned long long db = (unsigned long long)__double_as_longlong(slot.dres[gp[k]]);
        keys[m + pos] = ((db << 2) & ~low) | (unsigned long long)k;
      }
      m += tot;
    }
    const int n_out = n - m;
    int sn = 1;
    while (sn < m) sn <<= 1;
    for (int i = m + tid; i < sn; i += GCR_BLOCK) keys[i] = ~0ull;
    sync();
    if (m > 1) block_bitonic_sort(keys, sn);
    // sorted inliers: the point of each rank (ascending d) into scratch, then
    // the exclusive prefix sums of d over that order into the key array
    for (int j = tid; j < m; j += GCR_BLOCK) scratch[j] = gp[(int)(keys[j] & low)];
    sync();
    double* D = reinterpret_cast<double*>(keys);
    double carry = 0.0;
    for (int base = 0; base < m; base += GCR_BLOCK) {
      const int j = base + tid;
      const double v = j < m ? slot.dres[scratch[j]] : 0.0;
      double x = v;
      const int lane = tid & 31, w = tid >> 5;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      sync();
      if (lane == 31) sh.red_d[w] = x;
      sync();
      double wb = 0.0, tot = 0.0;
      for (int q = 0; q < GCR_WARPS; ++q) {
        if (q < w) wb += sh.red_d[q];
        tot += sh.red_d[q];
      }
      if (j < m) D[j] = carry + wb + (x - v);
      carry += tot;
      sync();
    }
    const double Dm = carry;
    // r-th smallest inlier key at slope s = c - (1 - lambda): ascending d for
    // s >= 0, descending d otherwise
    auto d_at = [&](int j) { return slot.dres[scratch[j]]; };
    auto pref = [&](int j) { return j >= m ? Dm : D[j]; };
    auto inl_sum = [&](int j, double sl) {  // the j smallest inlier keys
      return sl >= 0 ? oml * j + sl * pref(j) : oml * j + sl * (Dm - pref(m - j));
    };
    auto count_le = [&](double sl, double ko) {  // inliers with key <= ko
      int lo = 0, hi = m;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const double d = d_at(sl >= 0 ? mid : m - 1 - mid);
        if (oml + sl * d <= ko) lo = mid + 1;
        else hi = mid;
      }
      return lo;
    };
    auto energy = [&](int t) -> double {  // E(T) - sum_i E1_i of the best T of size t
      if (t == 0) return 0.0;
      const double c = 0.5 * lam * (double)(t - 1);
      const double sl = c - oml, ko = c - oml;
      const int J = count_le(sl, ko);
      double S;
      if (t <= J) S = inl_sum(t, sl);
      else if (t <= J + n_out) S = inl_sum(J, sl) + (double)(t - J) * ko;
      else S = inl_sum(t - n_out, sl) + (double)n_out * ko;
      return S + lam * (double)t * (double)(n - t);
    };
    double fmin = 0.0;
    for (int t = tid; t <= n; t += GCR_BLOCK) {
      const double e = energy(t);
      fmin = e < fmin ? e : fmin;
    }
    fmin = warp_min(fmin);
    sync();
    if ((tid & 31) == 0) sh.red_d[tid >> 5] = fmin;
    sync();
    for (int q = 0; q < GCR_WARPS; ++q) fmin = sh.red_d[q] < fmin ? sh.red_d[q] : fmin;
    // rounding bound of the energies: |terms| <= (1 - lambda) n + lambda (n - 1) / 2 Dm + lambda n^2 / 4
    const double tol = 1e-12 * (1.0 + oml * n + 0.5 * lam * (double)(n - 1) * Dm + 0.25 * lam * (double)n * n);
    int tmax = 0;
    for (int t = tid; t <= n; t += GCR_BLOCK)
      if (energy(t) <= fmin + tol) tmax = t > tmax ? t : tmax;
    tmax = -warp_min(-tmax);
    sync();
    if ((tid & 31) == 0) sh.red_i[tid >> 5] = tmax;
    sync();
    for (int q = 0; q < GCR_WARPS; ++q) tmax = sh.red_i[q] > tmax ? sh.red_i[q] : tmax;
    sync();
    // the source set of size tmax: its inliers by key rank, its outliers by index
    const double c = 0.5 * lam * (double)(tmax - 1);
    const double sl = c - oml;
    int in_T = 0;
    if (tmax > 0) {
      const int J = count_le(sl, sl);
      in_T = tmax <= J ? tmax : (tmax <= J + n_out ? J : tmax - n_out);
    }
    const int out_T = tmax - in_T;
    for (int j = tid; j < m; j += GCR_BLOCK) {
      const int r = sl >= 0 ? j : m - 1 - j;
      slot.flag[scratch[j]] = r < in_T ? 0 : 1;
    }
    int seen = 0;
    for (int base = 0; base < n; base += GCR_BLOCK) {
      const int k = base + tid;
      const int f = (k < n && slot.tr[gp[k]] > 0) ? 1 : 0;
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (f) slot.flag[gp[k]] = seen + pos < out_T ? 0 : 1;
      seen += tot;
    }
    sync();
  }

  __device__ int labeling(const double* model, int ncells, int* list) {
    const double sq = t2;  // thr^2 * 9 / 4
    const double oml = 1.0 - prm.lambda;
    prepare_shared_f32(model);
    double h[9];
    float hf[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      h[k] = model[k];
      hf[k] = sh.mf32[k];
    }
    const float cm = sh.mf32[9];
    const float tf = (float)sqrt(t2), t2f = (float)t2;
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) {
      float it;
      const float r2f = Est::r2_f32(pts32[i], hf, it);
      const float ee = fmaf(cm, fabsf(it), cm);
      const float eb = fmaf(ee, ee, 2.f * tf * ee);
      if (r2f - t2f > eb) {
        // certainly beyond the threshold: d = 1 and the unary term is (1 - lambda)
        slot.dres[i] = 1.0;
        slot.tr[i] = oml * (1 - 0.0) - 0;
        continue;
      }
      const double r2 = Est::r2_f64(pts64 + 4 * i, h);
      double di = r2 / sq;
      di = di < 0.0 ? 0.0 : (di > 1.0 ? 1.0 : di);
      const double e = 1 - di;
      slot.dres[i] = di;
      slot.tr[i] = r2 <= sq ? 0 - oml * e : oml * (1 - e) - 0;
    }
    sync();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) sh.flow_status = 0;
    sync();
    const bool pairwise = prm.lambda > 0;
    // Every point starts with its unary decision (SINK iff the sink capacity
    // is positive). That is the labelling without pairwise terms, and on the
    // grid it stays the label of the points of single-point cells and of
    // cells the flow solver does not take (more than kMaxFlowCap points, or an
    // inconsistent cell table: status ST_CAPACITY), so no flag of this pair
    // keeps a value from an earlier pair or from other uses of the slot.
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) slot.flag[i] = (uint8_t)(slot.tr[i] < -kResidualEps ? 1 : 0);
    sync();
    if (pairwise && prm.neighborhood == 1) {
      // without a graph (capacity exceeded, reported) the unary labels stand
      if (rg_ok) radius_mincut();
      sync();
    }
    if (threadIdx.x == 0) sh.big_cells = 0;
    if (pairwise && prm.neighborhood == 0 && threadIdx.x <= 32) sh.out_tmax[threadIdx.x] = outlier_clique_tmax(threadIdx.x);
    sync();
    for (int c = warp; pairwise && prm.neighborhood == 0 && c < ncells; c += GCR_WARPS) {
      const int c0 = slot.cell_start[c], n = slot.cell_start[c + 1] - c0;
      if (c0 < 0 || n < 1 || c0 + n > N) {  // inconsistent cell table: skip, report
        if (lane == 0) atomicMax(&sh.flow_status, ST_CAPACITY);
        continue;
      }
      if (n == 1) continue;  // unary label, set above
      if (n <= 32) {
        clique_cut_warp(c0, n);
      } else if (n > kMaxFlowCap) {
        if (lane == 0) atomicAdd(&sh.big_cells, 1);  // cut below by the whole CTA
      } else if (!mincut_cell(c0, n, warp)) {
        if (lane == 0) atomicMax(&sh.flow_status, ST_TIMEOUT);
      }
    }
    sync();
    // cells above the warp solver's capacity: one at a time by the CTA, in
    // cell order, with the list scratch that the labelled inliers fill later
    if (sh.big_cells > 0) {
      for (int base = 0; base < ncells; base += GCR_BLOCK) {
        const int c = base + threadIdx.x;
        int f = 0;
        if (c < ncells) {
          const int c0 = slot.cell_start[c], n = slot.cell_start[c + 1] - c0;
          f = (c0 >= 0 && n > kMaxFlowCap && c0 + n <= N) ? 1 : 0;
        }
        int tot;
        const int pos = block_exclusive_scan(f, sh.red_i, &tot);
        if (f) sh.s_cnt[pos] = c;
        sync();
        for (int q = 0; q < tot; ++q) {
          const int cc = sh.s_cnt[q];
          const int c0 = slot.cell_start[cc];
          clique_cut_cta(c0, slot.cell_start[cc + 1] - c0, list);
        }
        sync();
      }
    }
    if (sh.flow_status != 0 && status == ST_OK) status = sh.flow_status;
    // flags are read as booleans, so the list never holds more than N points
    int total = 0;
    for (int base = 0; base < N; base += GCR_BLOCK) {
      const int i = base + threadIdx.x;
      const int f = (i < N && slot.flag[i] != 0) ? 1 : 0;
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (f) list[total + pos] = i;
      total += tot;
    }
    sync();  // callers read entries other threads wrote after the last scan
    return total;
  }

  // ------------------------------------------------------------------
  // CTA-wide non-minimal fits over the rows list[0..n).
  // Row weights (weight_mode): 0 unit; 1 the iterated-least-squares weights of
  // the reference, where packed row k gets weights[k] of the point INDEX k
  // (GCRANSAC.h:657-675 with the solvers reading weights_[i] for packed row i,
  // e.g. solver_homography_four_point.h:211-224): Tukey^2 of point k under
  // sh.work_model when point k is in the set (slot.flag), else 0; 2 explicit
  // weights slot.dres[k]. Result in sh.fit_model; returns success (uniform).
  __device__ __forceinline__ double row_weight(int k, int weight_mode, const double* wm) const {
    if (weight_mode == 0) return 1.0;
    if (weight_mode == 2) return slot.dres[k];
    if (k < N && slot.flag[k]) {
      const double r2 = Est::r2_f64(pts64 + 4 * k, wm);
      const double wt = fmax(0.0, 1.0 - r2 / t2);
      return wt * wt;
    }
    return 0.0;
  }

  // Hartley normalisation of the rows (normalizePoints semantics), CTA-wide.
  __device__ void cta_norm(const int* list, int n, HomographyModel::Norm& nm) {
    double s[4] = {0, 0, 0, 0};
    for (int k = threadIdx.x; k < n; k += GCR_BLOCK) {
      const double* p = row64(list[k]);
      s[0] += p[0]; s[1] += p[1]; s[2] += p[2]; s[3] += p[3];
    }
    nm.ms0 = block_sum(s[0], sh.red_d) / n;
    nm.ms1 = block_sum(s[1], sh.red_d) / n;
    nm.md0 = block_sum(s[2], sh.red_d) / n;
    nm.md1 = block_sum(s[3], sh.red_d) / n;
    double a = 0, b = 0;
    for (int k = threadIdx.x; k < n; k += GCR_BLOCK) {
      const double* p = row64(list[k]);
      const double dx1 = nm.ms0 - p[0], dy1 = nm.ms1 - p[1], dx2 = nm.md0 - p[2], dy2 = nm.md1 - p[3];
      a += sqrt(dx1 * dx1 + dy1 * dy1);
      b += sqrt(dx2 * dx2 + dy2 * dy2);
    }
    nm.rs = M_SQRT2 / (block_sum(a, sh.red_d) / n);
    nm.rd = M_SQRT2 / (block_sum(b, sh.red_d) / n);
  }

  // Deterministic CTA reduction of NA per-thread partial sums into tot (thread 0).
  template <int NA>
  __device__ void cta_reduce(const double* acc, double* tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NA; ++q) {
      const double v = warp_sum(acc[q]);
      if (lane == 0) slot.red[warp * 64 + q] = v;
    }
    sync();
    if (threadIdx.x < NA) {
      double t = 0;
      for (int w = 0; w < GCR_WARPS; ++w) t += slot.red[w * 64 + threadIdx.x];
      tot[threadIdx.x] = t;
    }
    sync();
  }

  // Homography least squares (normalised, 23-sum normal equations).
  __device__ bool fit_cta_h(const int* list, int n, int weight_mode) {
    using H = HomographyModel;
    if (n < H::NONMIN) return false;
    H::Norm nm;
    cta_norm(list, n, nm);
    double acc[H::NACC];
#pragma unroll
    for (int q = 0; q < H::NACC; ++q) acc[q] = 0;
    double wm[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) wm[q] = sh.work_model[q];
    for (int k = threadIdx.x; k < n; k += GCR_BLOCK) H::accumulate(nm, row64(list[k]), row_weight(k, weight_mode, wm), acc);
    cta_reduce<H::NACC>(acc, sh.lm_acc);
    if (threadIdx.x == 0) sh.fit_ok = H::solve_normal(nm, sh.lm_acc, sh.fit_model) ? 1 : 0;
    sync();
    return sh.fit_ok != 0;
  }

  // Fundamental matrix: FundamentalMatrixBundleAdjustmentSolver on the rows
  // (8-point start, 25 LM iterations on the factorised F), optionally inside
  // the estimator's normalisation (estimateModelNonminimal) or on the raw rows
  // (the driver's final bundle adjustment).
  __device__ double fit_f_cost(const double* f19, int n, int weight_mode, const HomographyModel::Norm& nm,
                               const double* wm) {
    using F = FundamentalModel;
    double G[9];
    if (threadIdx.x == 0) {
      F::FactF ff;
      for (int q = 0; q < 9; ++q) { ff.U[q] = f19[q]; ff.V[q] = f19[9 + q]; }
      ff.sigma = f19[18];
      F::factf_F(ff, sh.lm_G);
    }
    sync();
#pragma unroll
    for (int q = 0; q < 9; ++q) G[q] = sh.lm_G[q];
    double c = 0;
    for (int k = threadIdx.x; k < n; k += GCR_BLOCK) {
      const double* p = row64(slot_list_[k]);
      const double w = row_weight(k, weight_mode, wm);
      const double l = F::lm_cost_point(G, (p[0] - nm.ms0) * nm.rs, (p[1] - nm.ms1) * nm.rs, (p[2] - nm.md0) * nm.rd,
                                        (p[3] - nm.md1) * nm.rd);
      c += weight_mode == 0 ? l : w * l;
    }
    return block_sum(c, sh.red_d);
  }

  const int* slot_list_ = nullptr;

  // fit_cta_f in FP32 (the fast precision mode, prm.lo_fp32): each thread
  // forms its rows' 8-point products, weights, Jacobian terms and costs in
  // FP32 from the FP32 tile; the partial sums are reduced across the CTA in
  // FP64; thread 0 runs the small solves in FP32 like the local-optimisation
  // trials (the 8-point null vector by pivoted QR, the 3x3 SVD of the
  // factorisation, the damped 7x7 Cholesky steps). Normalised fits use the
  // estimator's normalisation (FP64, cta_norm). A fit on raw pixel
  // coordinates (`raw`, the drivers' bundle adjustment) runs on the pair's
  // centred coordinates scaled by s = 1 / (largest centred coordinate): the
  // Sampson distance scales by s under a common similarity of both images,
  // so the loss truncated at 1 px^2 is truncated at s^2 there and the
  // minimiser is the same; FP32 products of raw pixel coordinates would span
  // ten decades. The model is mapped back in FP64.
  __device__ bool fit_cta_f_fast(const int* list, int n, int weight_mode, bool raw, const double* init) {
    using F = FundamentalModel;
    HomographyModel::Norm nm;
    float trunc2 = 1.f;
    if (raw) {
      const double s = scale > 0.0 ? 1.0 / scale : 1.0;
      nm.ms0 = pd.centre[0]; nm.ms1 = pd.centre[1];
      nm.md0 = pd.centre[2]; nm.md1 = pd.centre[3];
      nm.rs = nm.rd = s;
      trunc2 = (float)(s * s);
    } else {
      cta_norm(list, n, nm);
    }
    // the tile is centred: x_n = (x_c - (ms - c)) rs
    const float a0 = (float)(nm.ms0 - pd.centre[0]), a1 = (float)(nm.ms1 - pd.centre[1]);
    const float b0 = (float)(nm.md0 - pd.centre[2]), b1 = (float)(nm.md1 - pd.centre[3]);
    const float rs = (float)nm.rs, rd = (float)nm.rd;
    // row weights: 0 unit; 1 Tukey^2 of point k (the row index, as the
    // reference's weights array) under sh.work_model when k is in the set; 2 slot.dres[k]
    float wf[10];
    if (weight_mode == 1) {
      prepare_shared_f32(sh.work_model);
#pragma unroll
      for (int q = 0; q < 10; ++q) wf[q] = sh.mf32[q];
    }
    const float t2f = (float)t2;
    auto weight = [&](int k) -> float {
      if (weight_mode == 0) return 1.f;
      if (weight_mode == 2) return (float)slot.dres[k];
      if (k < N && slot.flag[k]) {
        float it;
        const float r2 = Est::r2_f32(pts32[k], wf, it);
        const float w = fmaxf(0.f, 1.f - r2 / t2f);
        return w * w;
      }
      return 0.f;
    };
    auto row = [&](int k, float& p0, float& p1, float& q0, float& q1) {
      const float4 p = pts32[row_ok(list[k]) ? list[k] : 0];
      p0 = (p.x - a0) * rs;
      p1 = (p.y - a1) * rs;
      q0 = (p.z - b0) * rd;
      q1 = (p.w - b1) * rd;
    };
    // the factorisation lives in sh.lm_f / sh.lm_fn as FP32 values
    auto load_fact = [&](const double* f19, lo32::FactF& f) {
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        f.U[q] = (float)f19[q];
        f.V[q] = (float)f19[9 + q];
      }
      f.sigma = (float)f19[18];
    };
    auto store_fact = [&](const lo32::FactF& f, double* f19) {
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        f19[q] = f.U[q];
        f19[9 + q] = f.V[q];
      }
      f19[18] = f.sigma;
    };
    if (init != nullptr) {
      // warm start: the given model in this fit's normalised coordinates,
      // Fn = Td^-T F Ts^-1, unit norm, factorised
      if (threadIdx.x == 0) {
        const double A[9] = {1.0 / nm.rd, 0, 0, 0, 1.0 / nm.rd, 0, nm.md0, nm.md1, 1};
        const double B[9] = {1.0 / nm.rs, 0, nm.ms0, 0, 1.0 / nm.rs, nm.ms1, 0, 0, 1};
        double t[9], G[9];
        matmul3(A, init, t);
        matmul3(t, B, G);
        double nrm = 0;
        for (int q = 0; q < 9; ++q) nrm += G[q] * G[q];
        nrm = sqrt(nrm);
        float F0[9], sv[3];
        for (int q = 0; q < 9; ++q) F0[q] = (float)(G[q] / nrm);
        lo32::FactF ff;
        lo32::svd3(F0, ff.U, sv, ff.V);
        ff.sigma = sv[0] > 0.f ? sv[1] / sv[0] : 0.f;
        store_fact(ff, sh.lm_f);
      }
    } else {
      // the 8-point start: null vector of the CTA-reduced A^T A
      float af[F::NATA];
#pragma unroll
      for (int q = 0; q < F::NATA; ++q) af[q] = 0.f;
      for (int k = threadIdx.x; k < n; k += GCR_BLOCK) {
        float x0, y0, x1, y1;
        row(k, x0, y0, x1, y1);
        const float w = weight(k);
        const float r[9] = {w * x1 * x0, w * x1 * y0, w * x1, w * y1 * x0, w * y1 * y0, w * y1, w * x0, w * y0, w};
        int q = 0;
#pragma unroll
        for (int a = 0; a < 9; ++a)
#pragma unroll
          for (int c = 0; c <= a; ++c) af[q++] += r[a] * r[c];
      }
      double acc[F::NATA];
#pragma unroll
      for (int q = 0; q < F::NATA; ++q) acc[q] = (double)af[q];
      cta_reduce<F::NATA>(acc, slot.red + GCR_WARPS * 64);
      if (threadIdx.x == 0) {
        const double* ata = slot.red + GCR_WARPS * 64;
        float M[81], F0[9], sv[3];
        int k = 0;
        for (int r = 0; r < 9; ++r)
          for (int c = 0; c <= r; ++c) {
            const float v = (float)ata[k++];
            M[r * 9 + c] = v;
            M[c * 9 + r] = v;
          }
        lo32::qr9_null(M, F0);
        lo32::FactF ff;
        lo32::svd3(F0, ff.U, sv, ff.V);
        ff.sigma = sv[0] > 0.f ? sv[1] / sv[0] : 0.f;
        store_fact(ff, sh.lm_f);
      }
    }
    sync();
    const float inv_n = 1.f / (float)n;
    // truncated Sampson cost of the factorisation f19 (thread 0 forms F)
    auto cost_of = [&](const double* f19) {
      if (threadIdx.x == 0) {
        lo32::FactF ff;
        float Gf[9];
        load_fact(f19, ff);
        lo32::fact_to_F(ff, Gf);
        for (int q = 0; q < 9; ++q) sh.lm_G[q] = Gf[q];
      }
      sync();
      float G[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) G[q] = (float)sh.lm_G[q];
      float c = 0.f;
      for (int k = threadIdx.x; k < n; k += GCR_BLOCK) {
        float p0, p1, q0, q1;
        row(k, p0, p1, q0, q1);
        const float l = lo32::cost_point(G, p0, p1, q0, q1, trunc2);
        c += weight_mode == 0 ? l : weight(k) * l;
      }
      return block_sum((double)c, sh.red_d);
    };
    double lambda = 1e-3;
    double cost = cost_of(sh.lm_f);
    bool recompute = true;
    for (int iter = 0; iter < 25; ++iter) {
      if (recompute) {
        if (threadIdx.x == 0) {
          lo32::FactF ff;
          float Gf[9];
          load_fact(sh.lm_f, ff);
          lo32::fact_to_F(ff, Gf);
          for (int q = 0; q < 9; ++q) sh.lm_G[q] = Gf[q];
        }
        sync();
        float G[9], ds[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) G[q] = (float)sh.lm_G[q];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) ds[i * 3 + j] = (float)(sh.lm_f[i * 3 + 1] * sh.lm_f[9 + j * 3 + 1]);
        float af[F::NLM];
#pragma unroll
        for (int q = 0; q < F::NLM; ++q) af[q] = 0.f;
        for (int k = threadIdx.x; k < n; k += GCR_BLOCK) {
          float p0, p1, q0, q1;
          row(k, p0, p1, q0, q1);
          lo32::accumulate_point(G, ds, p0, p1, q0, q1, weight(k) * inv_n, af, trunc2);
        }
        double acc[F::NLM];
#pragma unroll
        for (int q = 0; q < F::NLM; ++q) acc[q] = (double)af[q];
        cta_reduce<F::NLM>(acc, sh.lm_acc);
        float gn = 0.f;
        for (int a = 0; a < 7; ++a) gn += (float)sh.lm_acc[28 + a] * (float)sh.lm_acc[28 + a];
        if (!(sqrtf(gn) >= 1e-7f)) break;  // the FP32 tolerance of the trials' fits
      }
      if (threadIdx.x == 0) {
        lo32::FactF ff, fn;
        float a35[F::NLM];
        for (int q = 0; q < F::NLM; ++q) a35[q] = (float)sh.lm_acc[q];
        load_fact(sh.lm_f, ff);
        const bool ok = lo32::step(a35, (float)lambda, ff, fn);
        sh.lm_flag = ok ? 1 : 0;
        store_fact(ok ? fn : ff, sh.lm_fn);
      }
      sync();
      if (!sh.lm_flag) break;
      const double cn = cost_of(sh.lm_fn);
      if (cn < cost) {
        sync();
        if (threadIdx.x < 19) sh.lm_f[threadIdx.x] = sh.lm_fn[threadIdx.x];
        sync();
        lambda /= 10;
        cost = cn;
        recompute = true;
      } else {
        lambda *= 10;
        recompute = false;
      }
    }
    if (threadIdx.x == 0) {
      lo32::FactF ff;
      float Ff[9];
      load_fact(sh.lm_f, ff);
      lo32::fact_to_F(ff, Ff);
      double Fn[9];
      for (int q = 0; q < 9; ++q) Fn[q] = Ff[q];
      F::denormalise(nm, Fn, sh.fit_model);
    }
    sync();
    return true;
  }

  // `init`: the warm start of the FP32 mode's fits (ignored by the FP64 fits,
  // which start from the 8-point solution like the reference's solver)
  __device__ bool fit_cta_f(const int* list, int n, int weight_mode, bool normalise, bool lm = true,
                            const double* init = nullptr) {
    using F = FundamentalModel;
    if (n < 8) return false;  // 7 rows never reach the non-minimal solver in the loop
    if (prm.lo_fp32 && lm) return fit_cta_f_fast(list, n, weight_mode, !normalise, init);
    slot_list_ = list;
    HomographyModel::Norm nm;
    if (normalise) cta_norm(list, n, nm);
    else { nm.ms0 = nm.ms1 = nm.md0 = nm.md1 = 0.0; nm.rs = nm.rd = 1.0; }
    double wm[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) wm[q] = sh.work_model[q];
    {
      double acc[F::NATA];
#pragma unroll
      for (int q = 0; q < F::NATA; ++q) acc[q] = 0;
      for (int k = threadIdx.x; k < n; k += GCR_BLOCK)
        F::accumulate_ata(nm, row64(list[k]), row_weight(k, weight_mode, wm), acc);
      cta_reduce<F::NATA>(acc, slot.red + GCR_WARPS * 64);
    }
    if (threadIdx.x == 0) {
      double F0[9];
      F::eight_point_from_ata(slot.red + GCR_WARPS * 64, F0);
      F::FactF ff;
      F::factf_from(F0, ff);
      for (int q = 0; q < 9; ++q) { sh.lm_f[q] = ff.U[q]; sh.lm_f[9 + q] = ff.V[q]; }
      sh.lm_f[18] = ff.sigma;
    }
    sync();
    if (!lm) {
      // plain normalised 8-point solver (the inner DEGENSAC estimator)
      if (threadIdx.x == 0) {
        double F0[9];
        F::eight_point_from_ata(slot.red + GCR_WARPS * 64, F0);
        F::denormalise(nm, F0, sh.fit_model);
      }
      sync();
      return true;
    }
    double lambda = 1e-3;
    double cost = fit_f_cost(sh.lm_f, n, weight_mode, nm, wm);
    bool recompute = true;
    for (int iter = 0; iter < 25; ++iter) {
      if (recompute) {
        if (threadIdx.x == 0) {
          F::FactF ff;
          for (int q = 0; q < 9; ++q) { ff.U[q] = sh.lm_f[q]; ff.V[q] = sh.lm_f[9 + q]; }
          ff.sigma = sh.lm_f[18];
          F::factf_F(ff, sh.lm_G);
          double D[9][7];
          F::lm_dparams(ff, sh.lm_G, D);
          for (int r = 0; r < 9; ++r)
            for (int c = 0; c < 7; ++c) sh.lm_D[r * 7 + c] = D[r][c];
        }
        sync();
        double G[9], D[9][7];
#pragma unroll
        for (int q = 0; q < 9; ++q) G[q] = sh.lm_G[q];
#pragma unroll
        for (int r = 0; r < 9; ++r)
#pragma unroll
          for (int c = 0; c < 7; ++c) D[r][c] = sh.lm_D[r * 7 + c];
        double acc[F::NLM];
#pragma unroll
        for (int q = 0; q < F::NLM; ++q) acc[q] = 0;
        for (int k = threadIdx.x; k < n; k += GCR_BLOCK) {
          const double* p = row64(list[k]);
          F::lm_accumulate_point(G, D, (p[0] - nm.ms0) * nm.rs, (p[1] - nm.ms1) * nm.rs, (p[2] - nm.md0) * nm.rd,
                                 (p[3] - nm.md1) * nm.rd, row_weight(k, weight_mode, wm), n, acc);
        }
        cta_reduce<F::NLM>(acc, sh.lm_acc);
        double gn = 0;
        for (int a = 0; a < 7; ++a) gn += sh.lm_acc[28 + a] * sh.lm_acc[28 + a];
        if (sqrt(gn) < 1e-8) break;
      }
      if (threadIdx.x == 0) {
        F::FactF ff, fn;
        for (int q = 0; q < 9; ++q) { ff.U[q] = sh.lm_f[q]; ff.V[q] = sh.lm_f[9 + q]; }
        ff.sigma = sh.lm_f[18];
        sh.lm_flag = F::lm_step(sh.lm_acc, lambda, ff, fn) ? 1 : 0;
        for (int q = 0; q < 9; ++q) { sh.lm_fn[q] = fn.U[q]; sh.lm_fn[9 + q] = fn.V[q]; }
        sh.lm_fn[18] = fn.sigma;
      }
      sync();
      if (!sh.lm_flag) break;
      const double cn = fit_f_cost(sh.lm_fn, n, weight_mode, nm, wm);
      if (cn < cost) {
        sync();
        if (threadIdx.x < 19) sh.lm_f[threadIdx.x] = sh.lm_fn[threadIdx.x];
        sync();
        lambda /= 10;
        cost = cn;
        recompute = true;
      } else {
        lambda *= 10;
        recompute = false;
      }
    }
    if (threadIdx.x == 0) {
      F::FactF ff;
      for (int q = 0; q < 9; ++q) { ff.U[q] = sh.lm_f[q]; ff.V[q] = sh.lm_f[9 + q]; }
      ff.sigma = sh.lm_f[18];
      double Fn[9];
      F::factf_F(ff, Fn);
      if (normalise) F::denormalise(nm, Fn, sh.fit_model);
      else
        for (int q = 0; q < 9; ++q) sh.fit_model[q] = Fn[q];
    }
    sync();
    return true;
  }

  __device__ bool fit_cta(const int* list, int n, int weight_mode, const double* init = nullptr) {
    if constexpr (Est::LO_MAXSOL > 1) return false;  // multi-model estimators use fit_cta_multi
    if constexpr (Est::KIND == 1) return fit_cta_f(list, n, weight_mode, true, nonminimal_lm<Est>(), init);
    if constexpr (Est::KIND == 2) return fit_cta_f(list, n, weight_mode, true, false);
    return fit_cta_h(list, n, weight_mode);
  }

  // ------------------------------------------------------------------
  // Essential matrices: the non-minimal solver returns up to ten models.

  // Weighted Stewenius fit of the rows list[0..n) by the CTA: the weighted
  // normal matrix is reduced across the CTA, thread 0 solves. weight_mode 0:
  // unit weights; 2: slot.dres[k] by row position; 3: the squared Tukey
  // weight of point list[k] under sh.work_model (weights by point index, as
  // the Stewenius solver reads them). With `normalise` each model gets unit
  // norm and E33 >= 0 (estimateModelNonminimal). Models go to
  // sh.multi_models; returns their number.
  __device__ int fit_cta_multi(const int* list, int n, int weight_mode, bool normalise) {
    if constexpr (Est::LO_MAXSOL > 1) {
      if (n < Est::NONMIN) return 0;
      double wm[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) wm[q] = sh.work_model[q];
      auto weight = [&](int k) -> double {
        if (weight_mode == 0) return 1.0;
        if (weight_mode == 2) return slot.dres[k];
        const double r2 = Est::r2_f64(row64(list[k]), wm);
        const double w = fmax(0.0, 1.0 - r2 / t2);
        return w * w;
      };
      if (n == 5) {
        if (threadIdx.x == 0) {
          double rows[5][9];
          for (int k = 0; k < 5; ++k) ess::design_row(row64(list[k]), weight(k), rows[k]);
          sh.multi_count = ess::stewenius_five(rows, sh.multi_models);
        }
      } else {
        double acc[45];
#pragma unroll
        for (int q = 0; q < 45; ++q) acc[q] = 0;
        for (int k = threadIdx.x; k < n; k += GCR_BLOCK) {
          double r[9];
          ess::design_row(row64(list[k]), weight(k), r);
          int q = 0;
#pragma unroll
          for (int a = 0; a < 9; ++a)
#pragma unroll
            for (int b = 0; b <= a; ++b) acc[q++] += r[a] * r[b];
        }
        cta_reduce<45>(acc, slot.red + GCR_WARPS * 64);
        if (threadIdx.x == 0) {
          const double* t = slot.red + GCR_WARPS * 64;
          double full[81];
          int q = 0;
          for (int a = 0; a < 9; ++a)
            for (int b = 0; b <= a; ++b) {
              full[a * 9 + b] = t[q];
              full[b * 9 + a] = t[q];
              ++q;
            }
          sh.multi_count = ess::stewenius_from_ata(full, sh.multi_models);
        }
      }
      if constexpr (nonmin_ba<Est>()) {
        sync();
        bundle_adjust_models(list, n, weight_mode);
      }
      if (threadIdx.x == 0 && normalise)
        for (int q = 0; q < sh.multi_count; ++q) ess::normalise_sign(sh.multi_models + 9 * q);
      sync();
      return sh.multi_count;
    } else {
      return 0;
    }
  }

  // EssentialMatrixBundleAdjustmentSolver::estimateModel after its Stewenius
  // start (solver_essential_matrix_bundle_adjustment.h:141-183): the models
  // in sh.multi_models are replaced by every cheirality-consistent pose of
  // each (checked on the first row of the list) refined over the rows, at
  // most kMulti of them. The refinement reads its weights by row position
  // (jacobian_impl.h:327-342) from the array the Stewenius start reads by
  // point: unit weights for weight_mode 0, slot.dres for 2, and for 3 the
  // weight array of the iteratively reweighted fit, which holds the squared
  // Tukey weight of each listed point and 0 elsewhere, read at index k for
  // row k (slot.sp_flag marks the listed points; space partitioning, its
  // other user, runs for homographies only).
  __device__ void bundle_adjust_models(const int* list, int n, int weight_mode) {
    if constexpr (nonmin_ba<Est>()) {
      if (weight_mode == 0) {
        for (int k = threadIdx.x; k < n; k += GCR_BLOCK) slot.dres[k] = 1.0;
      } else if (weight_mode == 3) {
        for (int p = threadIdx.x; p < N; p += GCR_BLOCK) slot.sp_flag[p] = 0;
        sync();
        for (int k = threadIdx.x; k < n; k += GCR_BLOCK) slot.sp_flag[list[k]] = 1;
        sync();
        double wm[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) wm[q] = sh.work_model[q];
        for (int k = threadIdx.x; k < n; k += GCR_BLOCK) {
          double w = 0.0;
          if (slot.sp_flag[k]) {
            const double r2 = Est::r2_f64(row64(k), wm);
            const double t = fmax(0.0, 1.0 - r2 / t2);
            w = t * t;
          }
          slot.dres[k] = w;
        }
      }
      sync();
      double x1[3], x2[3];
      {
        const double* p0 = row64(list[0]);
        x1[0] = p0[0]; x1[1] = p0[1]; x1[2] = 1.0;
        x2[0] = p0[2]; x2[1] = p0[3]; x2[2] = 1.0;
        const double n1 = sqrt(x1[0] * x1[0] + x1[1] * x1[1] + 1.0);
        const double n2 = sqrt(x2[0] * x2[0] + x2[1] * x2[1] + 1.0);
        for (int i = 0; i < 3; ++i) {
          x1[i] /= n1;
          x2[i] /= n2;
        }
      }
      const int nin = sh.multi_count;
      double Em[9 * Shared<Est>::kMulti];
      for (int q = 0; q < 9 * nin; ++q) Em[q] = sh.multi_models[q];
      sync();
      int nout = 0;
      for (int q = 0; q < nin; ++q) {
        double Eq[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) Eq[e] = Em[9 * q + e];
        ess::Pose poses[4];
        const int np = ess::poses_from_essential(Eq, x1, x2, poses);
        for (int v = 0; v < np && nout < Shared<Est>::kMulti; ++v) {
          ess::Pose P = poses[v];
          refine_relpose_cta(list, n, P);
          double Eo[9];
          ess::essential_from_pose(P, Eo);
          if (threadIdx.x == 0)
            for (int e = 0; e < 9; ++e) sh.multi_models[9 * nout + e] = Eo[e];
          ++nout;
        }
      }
      if (threadIdx.x == 0) sh.multi_count = nout;
      sync();
    }
  }

  // Local-optimisation trials whose fits return several models: trials run
  // one per thread (trial u on thread u), in chunks of kLo / LO_MAXSOL; each
  // chunk's models are
  // compacted in trial order into the local-optimisation region, scored in
  // FP32 and replayed in order.
  __device__ void lo_trials_multi(int nL, int ss, const int* L, int trials, Score& max_score, bool& updated) {
    if constexpr (Est::LO_MAXSOL > 1) {
      constexpr int chunk_cap = Shared<Est>::kLo / Est::LO_MAXSOL;
      constexpr int kstage = kBatchModels + Shared<Est>::kLo;
      const int kb = kBatchModels;
      const int u = threadIdx.x;  // this thread's trial within the chunk
      for (int t0 = 0; t0 < trials; t0 += chunk_cap) {
        const int nt = min(chunk_cap, trials - t0);
        int cnt = 0;
        if (u < nt) {
          int* smp = slot.samples + u * Est::SAMPLE_CAP;
          DrawStream ds(pd.seed, prm.stream_lo, (uint64_t)(lo_calls + t0 + u));
          if (unique_set(ds, smp, ss, 0, (uint32_t)(nL - 1))) {
            for (int q = 0; q < ss; ++q) smp[q] = L[smp[q]];
            cnt = Est::fit_thread_multi(pts64, smp, ss, slot.models64 + 9 * (kstage + u * Est::LO_MAXSOL));
          }
          sh.lo_ok[u] = cnt;
        }
        sync();
        if (threadIdx.x == 0) {
          int acc = 0;
          for (int v = 0; v < nt; ++v) {
            sh.lo_base[v] = acc;
            acc += sh.lo_ok[v];
          }
          sh.multi_count = acc;
        }
        sync();
        const int total = sh.multi_count;
        if (u < nt) {
          const int base = sh.lo_base[u];
          for (int q = 0; q < cnt; ++q) {
            const double* src = slot.models64 + 9 * (kstage + u * Est::LO_MAXSOL + q);
            double* dst = slot.models64 + 9 * (kb + base + q);
#pragma unroll
            for (int e = 0; e < 9; ++e) dst[e] = src[e];
            put_f32(kb + base + q);
          }
        }
        sync();
        score_models_f32(kb, total);
        for (int v = 0; v < nt; ++v) {
          const int nm = sh.lo_ok[v], b0 = sh.lo_base[v];
          for (int q = 0; q < nm; ++q) {
            ++models_scored;
            const int k = kb + b0 + q;
            if (sh.mcount[k] == 0 || !maybe_better(k, max_score.value)) continue;
            const Score sc = exact_score(slot.models64 + 9 * k, nullptr, slot.models32 + 12 * k);
            if (max_score.value < sc.value) {
              updated = true;
              max_score = sc;
              copy_model(sh.lo_best_model, slot.models64 + 9 * k);
            }
          }
        }
        sync();
      }
      lo_calls += trials;
    }
  }

  // iteratedLeastSquaresFitting (GCRANSAC.h:629-758) with several models per
  // fit: one model replaces the current set when it has more inliers; with
  // several, every model with more inliers than the current set and at least
  // as many as the best so far does, in order.
  __device__ bool irls_multi(int*& list, int& n, int*& spare) {
    if (n <= m) return false;
    int iterations = 0;
    int best_count = 0;
    while (++iterations < 10) {
      const int nm = fit_cta_multi(list, n, 3, true);
      if (nm == 0) break;
      if (nm == 1) {
        const Score sc = exact_score(sh.multi_models, spare);
        ++models_scored;
        if (sc.count < m) break;
        if (sc.count <= n) break;
        copy_model(sh.work_model, sh.multi_models);
        int* t = list;
        list = spare;
        spare = t;
        n = sc.count;
      } else {
        bool upd = false;
        for (int q = 0; q < nm; ++q) {
          const Score sc = exact_score(sh.multi_models + 9 * q, spare);
          ++models_scored;
          if (sc.count < m) continue;
          if (sc.count <= n) continue;
          if (sc.count >= best_count) {
            upd = true;
            best_count = sc.count;
            copy_model(sh.work_model, sh.multi_models + 9 * q);
            int* t = list;
            list = spare;
            spare = t;
            n = sc.count;
          }
        }
        if (!upd) break;
      }
    }
    return iterations > 1;
  }

  // refine_relpose (bundle.cpp:412-452 + 176-250) of the pose in sh over the
  // rows list[0..n) with the position weights in slot.dres; every thread
  // carries the same LM state, the sums are CTA reductions.
  __device__ void refine_relpose_cta(const int* list, int n, ess::Pose& P) {
    auto residual = [&](const ess::Pose& Q) {
      double E[9];
      ess::essential_from_pose(Q, E);
      double c = 0;
      for (int k = threadIdx.x; k < n; k += GCR_BLOCK) c += slot.dres[k] * ess::relpose_loss(E, row64(list[k]));
      return block_sum(c, sh.red_d);
    };
    double lambda = 1e-3;
    double cost = residual(P);
    bool recompute = true;
    double tot[20];
    ess::PoseJac J;
    for (int iter = 0; iter < 25; ++iter) {
      if (recompute) {
        ess::pose_jacobians(P, J);
        double acc[20];
#pragma unroll
        for (int q = 0; q < 20; ++q) acc[q] = 0;
        for (int k = threadIdx.x; k < n; k += GCR_BLOCK)
          ess::relpose_accumulate(J, row64(list[k]), slot.dres[k], n, acc);
        cta_reduce<20>(acc, slot.red + GCR_WARPS * 64);
#pragma unroll
        for (int q = 0; q < 20; ++q) tot[q] = slot.red[GCR_WARPS * 64 + q];
        sync();
        double gn = 0;
        for (int a = 0; a < 5; ++a) gn += tot[15 + a] * tot[15 + a];
        if (sqrt(gn) < 1e-8) break;
      }
      constexpr int diag[5] = {0, 2, 5, 9, 14};
      for (int a = 0; a < 5; ++a) tot[diag[a]] += lambda;
      ess::Pose Pn;
      if (!ess::relpose_step(tot, tot + 15, J, P, Pn)) break;
      const double cn = residual(Pn);
      if (cn < cost) {
        P = Pn;
        lambda /= 10;
        cost = cn;
        recompute = true;
      } else {
        for (int a = 0; a < 5; ++a) tot[diag[a]] -= lambda;
        lambda *= 10;
        recompute = false;
      }
    }
  }

  // ------------------------------------------------------------------
  // GCRANSAC::graphCutLocalOptimization (GCRANSAC.h:779-910).
  __device__ void local_optimization(int ncells) {
    Score max_score = best;
    copy_model(sh.lo_best_model, sh.best_model);
    const int inlier_limit = Est::INLIER_LIMIT;
    int* L = slot.list0;
    const int trials = prm.lo_number;
    ++lo_number;
    while (++gc_number < prm.gc_max) {
      bool updated = false;
      long long t0 = tick();
      const int nL = labeling(sh.lo_best_model, ncells, L);
      tock(4, t0);
      t0 = tick();
      const int ss = min(inlier_limit, nL);
      if constexpr (Est::LO_MAXSOL > 1) {
        if (ss < nL) {
          lo_trials_multi(nL, ss, L, trials, max_score, updated);
          tock(5, t0);
        } else if (m < nL) {
          // every trial fits all labelled inliers: the same models each time, so
          // only the first trial can improve; the rest are counted
          const int nm = fit_cta_multi(L, nL, 0, true);
          if (nm > 0) {
            models_scored += (long long)trials * nm;
            for (int q = 0; q < nm && trials > 0; ++q) {
              const Score sc = exact_score(sh.multi_models + 9 * q, nullptr);
              if (max_score.value < sc.value) {
                updated = true;
                max_score = sc;
                copy_model(sh.lo_best_model, sh.multi_models + 9 * q);
              }
            }
          }
        }
      } else {
        if (nonminimal_lm<Est>() && ss < nL) {
          // fundamental matrices: each trial on a group of four lanes; lane 0
          // of the group draws the sample with the LO sampler stream
          const int kb = kBatchModels;
          const int q = threadIdx.x & 3;
          const unsigned gmask = 0xFu << (threadIdx.x & 28);
          for (int u0 = 0; u0 < trials; u0 += GCR_BLOCK / 4) {
            const int u = u0 + (threadIdx.x >> 2);
            if (u < trials) {
              int* smp = slot.samples + u * Est::SAMPLE_CAP;
              if (q == 0) {
                DrawStream ds(pd.seed, prm.stream_lo, (uint64_t)(lo_calls + u));
                const bool ok = unique_set(ds, smp, ss, 0, (uint32_t)(nL - 1));
                if (ok)
                  for (int k = 0; k < ss; ++k) smp[k] = L[smp[k]];
                sh.lo_ok[u] = ok ? 1 : 0;
              }
              __syncwarp(gmask);
              bool ok = sh.lo_ok[u] != 0;
              if (ok)
                ok = prm.lo_fp32 ? lo32::fit_fundamental(pts32, pd.centre, smp, ss, slot.models64 + 9 * (kb + u), q,
                                                         gmask, 4)
                                 : FundamentalModel::fit_group(pts64, smp, ss, slot.models64 + 9 * (kb + u), q, gmask);
              __syncwarp(gmask);
              if (q == 0) {
                sh.lo_ok[u] = ok ? 1 : 0;
                if (ok) put_f32(kb + u);
              }
            }
          }
          sync();
          tock(5, t0);
          lo_calls += trials;
          t0 = tick();
          score_lo_trials(kb, trials, max_score, updated);
          tock(6, t0);
        } else if (ss < nL) {
          // one thread per trial draws the sample from the labelled inliers with
          // the LO sampler stream and fits it
          const int kb = kBatchModels;
          if (threadIdx.x < trials) {
            long long c0 = tick();
            int* smp = slot.samples + threadIdx.x * Est::SAMPLE_CAP;
            DrawStream ds(pd.seed, prm.stream_lo, (uint64_t)(lo_calls + threadIdx.x));
            bool ok = unique_set(ds, smp, ss, 0, (uint32_t)(nL - 1));
            tock(12, c0);
            c0 = tick();
            if (ok) {
              for (int q = 0; q < ss; ++q) smp[q] = L[smp[q]];
              ok = Est::fit_thread(pts64, smp, ss, slot.models64 + 9 * (kb + threadIdx.x));
            }
            tock(13, c0);
            c0 = tick();
            sh.lo_ok[threadIdx.x] = ok ? 1 : 0;
            if (ok) put_f32(kb + threadIdx.x);
            tock(14, c0);
          }
          sync();
          tock(5, t0);
          lo_calls += trials;
          t0 = tick();
          score_lo_trials(kb, trials, max_score, updated);
          tock(6, t0);
        } else if (m < nL) {
          if (!fit_cta(L, nL, 0)) {
            // the reference breaks out of the trial loop; nothing was updated
          } else {
            const Score sc = exact_score(sh.fit_model, nullptr);
            models_scored += trials;
            if (max_score.value < sc.value) {
              updated = true;
              max_score = sc;
              copy_model(sh.lo_best_model, sh.fit_model);
            }
          }
        }
      }
      if (!updated) break;
    }
    if (best.value < max_score.value) {
      best = max_score;
      copy_model(sh.best_model, sh.lo_best_model);
      copy_model(sh.cont_model[off], sh.lo_best_model);
      cont[off] = {sh.cont_model[off], max_score.count};
    }
  }

  // Scores the LO trial models kb..kb+trials (their success flags in the
  // trial-flag array) and replays the sequential best-model update.
  __device__ void score_lo_trials(int kb, int trials, Score& max_score, bool& updated) {
    score_models_f32(kb, trials);
    for (int t = 0; t < trials; ++t) {
      if (!sh.lo_ok[t]) continue;
      ++models_scored;
      const int k = kb + t;
      if (sh.mcount[k] == 0 || !maybe_better(k, max_score.value)) continue;
      tock(10, 0, 1);
      const Score sc = exact_score(slot.models64 + 9 * k, nullptr, slot.models32 + 12 * k);
      if (max_score.value < sc.value) {
        updated = true;
        max_score = sc;
        copy_model(sh.lo_best_model, slot.models64 + 9 * k);
      }
    }
  }

  // ------------------------------------------------------------------
  // FundamentalMatrixEstimator::isValidModel (fundamental_estimator.h:287-338)
  // on the model's inlier list: at least max(7, 0.5 |I|) inliers under the
  // symmetric epipolar distance, then DEGENSAC (341-572). Returns validity;
  // `updated` reports a model replaced by the DEGENSAC inner run.
  __device__ bool valid_model_cta(const double* model, const int* sample, const int* list, int cnt, bool& updated) {
    updated = false;
    double F[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) F[q] = model[q];
    const double ratio = Est::KIND == 1 ? 0.5 : (Est::KIND == 3 ? 0.1 : 0.0);
    const int min_n = max(Est::M, (int)((double)cnt * ratio));
    int c = 0;
    for (int k = threadIdx.x; k < cnt; k += GCR_BLOCK)
      if (FundamentalModel::symepi2_f64(row64(list[k]), F) < t2) ++c;
    c = block_sum(c, sh.red_i);
    if (c < min_n) return false;
    if constexpr (!has_degensac<Est>()) return true;
    if (threadIdx.x == 0) sh.lm_flag = FundamentalModel::degenerate_sample(F, pts64, sample, sh.degen_H) ? 1 : 0;
    sync();
    if (!sh.lm_flag) return true;
    // H-degenerate sample: the plane's inliers among the model's inliers
    double H[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) H[q] = sh.degen_H[q];
    int total = 0;
    for (int base = 0; base < cnt; base += GCR_BLOCK) {
      const int k = base + threadIdx.x;
      const int f = (k < cnt && HomographyModel::r2_f64(row64(list[k]), H) < 4.0) ? 1 : 0;
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (f) slot.list2[total + pos] = list[k];
      total += tot;
    }
    sync();  // the fit reads entries other threads wrote after the last scan
    if (total < HomographyModel::NONMIN) return false;
    // plane homography from its inliers, then the plane-and-parallax GC-RANSAC
    if (!fit_cta_h(slot.list2, total, 0)) return false;
    if constexpr (Est::KIND == 1) {
      if (nsh == nullptr) {
        flags |= 4;
        return true;
      }
      flags |= 8;
      Shared<PlaneParallaxModel>& ish = *nsh;
      sync();
      if (threadIdx.x < 9) ish.pp_H[threadIdx.x] = sh.fit_model[threadIdx.x];
      sync();
      EngineParams p2 = prm;
      p2.confidence = 0.99;
      p2.lambda = 0.0;
      p2.max_iters = 1LL << 40;
      p2.min_iters = 20;
      p2.lo_number = 10;
      p2.sampler = SAMPLER_UNIFORM;
      p2.scoring = SCORING_MSAC;
      p2.use_sprt = 0;
      p2.nested = 1;
      p2.stream_main = p2.stream_lo = 16u + (uint32_t)(degensac_calls++);
      p2.pp_h = ish.pp_H;
      PairDesc pd2 = pd;
      pd2.threshold = 1.5 * pd.threshold;  // the run's truncated threshold
      Engine<PlaneParallaxModel> inner(ish, ws, p2, pd2, nslot, pair);
      inner.pts32 = pts32;
      inner.scale = scale;
      inner.run();
      if (ish.result_count > cnt) {
        updated = true;
        sync();
        if (threadIdx.x < 9) sh.degen_H[threadIdx.x] = ish.result_model[threadIdx.x];
        sync();
      }
    }
    return true;
  }

  // ------------------------------------------------------------------
  // SPRTPreemptiveVerfication (preemption/preemption_sprt.h:50-380): models
  // are tested on the points in a fixed random order, continuing from where
  // the previous model stopped, and rejected as soon as the likelihood ratio
  // exceeds the decision threshold A. Two inputs of the reference are not
  // reproducible and are replaced: the point order is a Fisher-Yates
  // permutation with the reference's loop structure whose draws come from
  // Philox stream 3 instead of rand(), and t_M is 1/m (what the reference gets
  // whenever its first-sample estimate returns a model).

  // estimateThresholdA (preemption_sprt.h:361-379)
  __device__ double sprt_threshold_A(double eps, double del) const {
    const double C = (1 - del) * log((1 - del) / (1 - eps)) + del * (log(del / eps));
    const double K = (sprt_tM * C) / sprt_mS + 1;
    double An_1 = K, An = K;
    for (int i = 0; i < 10; ++i) {
      An = K + log(An_1);
      if (fabs(An - An_1) < 1.5e-8) break;
      An_1 = An;
    }
    return An;
  }

  __device__ void sprt_init() {
    if (threadIdx.x == 0) {
      int* pool = slot.sprt_pool;
      for (int i = 0; i < N; ++i) pool[i] = i;
      DrawStream ds(pd.seed, 3u, 0);
      int max = N;
      for (int i = 0; i < N; ++i) {
        const int idx = (int)(ds.next_u32() % (uint32_t)max);
        const int t = pool[idx];
        --max;
        pool[idx] = pool[max];
        pool[max] = t;
      }
    }
    sync();
    sprt = true;
    sprt_cursor = 0;
    sprt_tM = 1.0 / (double)m;
    sprt_mS = (double)sprt_solutions<Est>();
    sprt_delta = prm.sprt_min_ratio / 10.0;
    sprt_eps = prm.sprt_min_ratio;
    sprt_A = sprt_threshold_A(sprt_eps, sprt_delta);
  }

  // Inlier decisions (r^2 < t^2, FP32 filter + FP64 decision) of the points at
  // SPRT-pool positions pos0 .. pos0 + cnt - 1 (mod N): sprt_buf[j] receives
  // the squared residual of an inlier, -1 otherwise.
  __device__ void sprt_flags(const double* h, const float* hf, float cm, int pos0, int cnt) {
    const float tf = (float)sqrt(t2), t2f = (float)t2;
    const int j = threadIdx.x;
    if (j < cnt) {
      int pos = pos0 + j;
      if (pos >= N) pos -= N;
      const int p = slot.sprt_pool[pos];
      float it;
      const float r2f = Est::r2_f32(pts32[p], hf, it);
      const float e = fmaf(cm, fabsf(it), cm);
      const float eb = fmaf(e, e, 2.f * tf * e) + 1.2e-7f * t2f;
      double v = -1.0;
      if (!(r2f - t2f > eb)) {
        const double r2 = Est::r2_f64(pts64 + 4 * p, h);
        if (r2 < t2) v = r2;
      }
      slot.sprt_buf[j] = v;
    }
    sync();
  }

  // verifyModel (preemption_sprt.h:232-347): returns whether the model
  // passed; sc is its truncated-quadratic score over the tested points, list
  // (optional) receives their inliers in pool order, [start, start + len) are
  // the pool positions tested.
  __device__ bool sprt_verify(const double* model, const float* m32, Score& sc, int* list, int& start, int& len) {
    double h[9];
    float hf[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      h[q] = model[q];
      hf[q] = m32[q];
    }
    const float cm = m32[9];
    start = sprt_cursor;
    const double eps = sprt_eps, del = sprt_delta, A = sprt_A;
    double lambda = 1.0, val = 0.0;
    int cnt = 0, tested = 0;
    bool valid = true;
    while (valid && tested < N) {
      const int chunk = min(GCR_BLOCK, N - tested);
      sprt_flags(h, hf, cm, sprt_cursor, chunk);
      if (threadIdx.x == 0) {
        double lam = lambda, vl = val;
        int c = cnt, used = 0;
        bool ok = true;
        for (int j = 0; j < chunk; ++j) {
          const double r2 = slot.sprt_buf[j];
          double ln;
          if (r2 >= 0) {
            ln = lam * (del / eps);
            ++c;
            vl += 1.0 - r2 / t2;
          } else {
            ln = lam * ((1 - del) / (1 - eps));
          }
          ++used;
          if (ln > A * 1.0) {
            ok = false;
            break;
          }
          lam = ln;
        }
        sh.red_d[0] = lam;
        sh.red_d[1] = vl;
        sh.red_i[0] = c;
        sh.red_i[1] = used;
        sh.red_i[2] = ok ? 1 : 0;
      }
      sync();
      lambda = sh.red_d[0];
      val = sh.red_d[1];
      const int cnew = sh.red_i[0], used = sh.red_i[1];
      valid = sh.red_i[2] != 0;
      sync();
      const int j = threadIdx.x;
      const int f = (j < used && slot.sprt_buf[j] >= 0) ? 1 : 0;
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (list && f) {
        int pp = sprt_cursor + j;
        if (pp >= N) pp -= N;
        list[cnt + pos] = slot.sprt_pool[pp];
      }
      cnt = cnew;
      tested += used;
      sprt_cursor += used;
      if (sprt_cursor >= N) sprt_cursor -= N;
      sync();
    }
    len = tested;
    sc.count = cnt;
    sc.value = val;
    if (valid) {
      if (val > best.value) {
        sprt_eps = (double)cnt / N;
        sprt_A = sprt_threshold_A(sprt_eps, sprt_delta);
      }
    } else {
      const double de = (double)cnt / N;
      if (de > 0 && fabs(del - de) / del > 0.05) {
        sprt_delta = de;
        sprt_A = sprt_threshold_A(sprt_eps, de);
      }
    }
    return valid;
  }

  // ------------------------------------------------------------------
  // SpacePartitioningRANSAC::runHomography (inlier_selectors/
  // space_partitioning_ransac.h:341-505) on the neighbourhood grid: a cell with
  // fewer than four points is always kept; otherwise its four source-image
  // corners are mapped by H and the cell is kept when one lands in the cell's
  // destination indices, or when the threshold-grown box of the mapped corners
  // 00 and 11 overlaps the destination cell. Cells are visited by ascending
  // key (the reference visits them in std::unordered_map order, which is
  // library-specific). A mapped coordinate outside the int range (or NaN)
  // converts to INT_MIN.
  __device__ static int sp_trunc_int(double v) {
    if (!(v > -2147483649.0 && v < 2147483648.0)) return (int)0x80000000;
    return (int)v;
  }

  __device__ void sp_init(int ncells) {
    sp = true;
    sp_ncells = ncells;
    for (int c = threadIdx.x; c < ncells; c += GCR_BLOCK)
      for (int j = slot.cell_start[c]; j < slot.cell_start[c + 1]; ++j) slot.sp_cell[j] = c;
    sync();
  }

  // Keeps the cells of `model`: sp_flag per cell, sp_sel the points of the
  // kept cells in cell order, sp_count their number.
  __device__ void sp_select(const double* model) {
    double H[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) H[q] = model[q];
    const bool degenerate = fabs(det3(H)) < 1e-3;
    const double cs1 = pd.cell[0], cs2 = pd.cell[1], cs3 = pd.cell[2], cs4 = pd.cell[3];
    const uint64_t n = (uint64_t)pd.n_div;
    const double thr = 1.5 * pd.threshold;
    const double* pix = ws.pix64 + 4 * pd.offset;
    auto proj = [&](uint64_t hx, uint64_t vy, double& x, double& y) {
      const double X1 = (double)hx * cs1, Y1 = (double)vy * cs2;
      double x2p = X1 * H[0] + Y1 * H[1] + H[2], y2p = X1 * H[3] + Y1 * H[4] + H[5],
             h2p = X1 * H[6] + Y1 * H[7] + H[8];
      x2p /= h2p;
      y2p /= h2p;
      x = x2p;
      y = y2p;
    };
    for (int c = threadIdx.x; c < sp_ncells; c += GCR_BLOCK) {
      int keep = 0;
      const int c0 = slot.cell_start[c], sz = slot.cell_start[c + 1] - c0;
      if (!degenerate) {
        if (sz < 4) {
          keep = 1;
        } else {
          const double* p = pix + 4 * slot.cell_pts[c0];
          uint64_t ci[4];
          for (int d = 0; d < 4; ++d) ci[d] = (uint64_t)(int64_t)floor(p[d] / pd.cell[d]);
          double c00x = 0, c00y = 0, c11x = 0, c11y = 0;
          for (int st = 0; st < 4 && !keep; ++st) {
            const uint64_t hx = ci[0] + (uint64_t)(st >> 1);
            if (hx >= n) continue;
            const uint64_t vy = ci[1] + (uint64_t)(st & 1);
            if (vy >= n) continue;
            double x, y;
            proj(hx, vy, x, y);
            if (st == 0) { c00x = x; c00y = y; }
            if (st == 3) { c11x = x; c11y = y; }
            const int ix = sp_trunc_int(x / cs3), iy = sp_trunc_int(y / cs4);
            if ((uint64_t)(int64_t)ix == ci[2] && (uint64_t)(int64_t)iy == ci[3]) keep = 1;
          }
          if (!keep) {
            const uint64_t hx11 = ci[0] + 1, vy11 = ci[1] + 1;
            if (vy11 >= n || hx11 >= n) proj(hx11, vy11, c11x, c11y);
            const double l1x = c00x - thr, l1y = c00y - thr, r1x = c11x + thr, r1y = c11y + thr;
            const double l2x = cs3 * (double)ci[2], l2y = cs4 * (double)ci[3];
            const double r2x = l2x + cs3, r2y = l2y + cs4;
            if ((l1x <= r2x && l2x <= r1x) || (r1y <= l2y && r2y <= l1y)) keep = 1;
          }
        }
      }
      slot.sp_flag[c] = keep;
    }
    sync();
    int total = 0;
    for (int base = 0; base < N; base += GCR_BLOCK) {
      const int j = base + threadIdx.x;
      const int f = (j < N && slot.sp_flag[slot.sp_cell[j]]) ? 1 : 0;
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (f) slot.sp_sel[total + pos] = slot.cell_pts[j];
      total += tot;
    }
    sp_count = total;
    sync();
  }

  // getScore over the kept points (scoring_function.h:186-230): MSAC in cell
  // order; the first `len` kept points when len >= 0.
  __device__ Score exact_score_sp(const double* model, int* list, int len = -1) {
    prepare_shared_f32(model);
    double h[9];
    float hf[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      h[q] = model[q];
      hf[q] = sh.mf32[q];
    }
    const float cm = sh.mf32[9];
    const float tf = (float)sqrt(t2), t2f = (float)t2;
    const int S = len >= 0 ? len : sp_count;
    double acc = 0.0;
    int total = 0;
    for (int base = 0; base < S; base += GCR_BLOCK) {
      const int j = base + threadIdx.x;
      int f = 0, p = 0;
      if (j < S) {
        p = slot.sp_sel[j];
        float it;
        const float r2f = Est::r2_f32(pts32[p], hf, it);
        const float e = fmaf(cm, fabsf(it), cm);
        const float eb = fmaf(e, e, 2.f * tf * e) + 1.2e-7f * t2f;
        if (!(r2f - t2f > eb)) {
          const double r2 = Est::r2_f64(pts64 + 4 * p, h);
          if (r2 < t2) {
            f = 1;
            acc -= r2;
          }
        }
      }
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (list && f) list[total + pos] = p;
      total += tot;
    }
    const double s = block_sum(acc, sh.red_d);
    Score sc;
    sc.count = total;
    sc.value = total == 0 ? 0.0 : (s + total * t2) / t2;
    return sc;
  }

  // verifyModel with index sets (preemption_sprt.h:268-296): the kept points
  // in cell order, the pool cursor untouched.
  __device__ bool sprt_verify_sp(const double* model, const float* m32, Score& sc, int* list, int& len) {
    double h[9];
    float hf[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      h[q] = model[q];
      hf[q] = m32[q];
    }
    const float cm = m32[9];
    const float tf = (float)sqrt(t2), t2f = (float)t2;
    const double eps = sprt_eps, del = sprt_delta, A = sprt_A;
    double lambda = 1.0, val = 0.0;
    int cnt = 0, tested = 0;
    bool valid = true;
    const int S = sp_count;
    while (valid && tested < S) {
      const int chunk = min(GCR_BLOCK, S - tested);
      const int j = threadIdx.x;
      if (j < chunk) {
        const int p = slot.sp_sel[tested + j];
        float it;
        const float r2f = Est::r2_f32(pts32[p], hf, it);
        const float e = fmaf(cm, fabsf(it), cm);
        const float eb = fmaf(e, e, 2.f * tf * e) + 1.2e-7f * t2f;
        double v = -1.0;
        if (!(r2f - t2f > eb)) {
          const double r2 = Est::r2_f64(pts64 + 4 * p, h);
          if (r2 < t2) v = r2;
        }
        slot.sprt_buf[j] = v;
      }
      sync();
      if (threadIdx.x == 0) {
        double lam = lambda, vl = val;
        int c = cnt, used = 0;
        bool ok = true;
        for (int q = 0; q < chunk; ++q) {
          const double r2 = slot.sprt_buf[q];
          double ln;
          if (r2 >= 0) {
            ln = lam * (del / eps);
            ++c;
            vl += 1.0 - r2 / t2;
          } else {
            ln = lam * ((1 - del) / (1 - eps));
          }
          ++used;
          if (ln > A * 1.0) {
            ok = false;
            break;
          }
          lam = ln;
        }
        sh.red_d[0] = lam;
        sh.red_d[1] = vl;
        sh.red_i[0] = c;
        sh.red_i[1] = used;
        sh.red_i[2] = ok ? 1 : 0;
      }
      sync();
      lambda = sh.red_d[0];
      val = sh.red_d[1];
      const int cnew = sh.red_i[0], used = sh.red_i[1];
      valid = sh.red_i[2] != 0;
      sync();
      const int f = (j < used && slot.sprt_buf[j] >= 0) ? 1 : 0;
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (list && f) list[cnt + pos] = slot.sp_sel[tested + j];
      cnt = cnew;
      tested += used;
      sync();
    }
    len = tested;
    sc.count = cnt;
    sc.value = val;
    if (valid) {
      if (val > best.value) {
        sprt_eps = (double)cnt / N;
        sprt_A = sprt_threshold_A(sprt_eps, sprt_delta);
      }
    } else {
      const double de = (double)cnt / N;
      if (de > 0 && fabs(del - de) / del > 0.05) {
        sprt_delta = de;
        sprt_A = sprt_threshold_A(sprt_eps, de);
      }
    }
    return valid;
  }

  // Inliers of `model` at pool positions [start, start + len), in pool order.
  __device__ int sprt_list(const double* model, int start, int len, int* list) {
    prepare_shared_f32(model);
    double h[9];
    float hf[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      h[q] = model[q];
      hf[q] = sh.mf32[q];
    }
    const float cm = sh.mf32[9];
    int total = 0;
    for (int done = 0; done < len; done += GCR_BLOCK) {
      const int chunk = min(GCR_BLOCK, len - done);
      int p0 = start + done;
      if (p0 >= N) p0 -= N;
      sprt_flags(h, hf, cm, p0, chunk);
      const int j = threadIdx.x;
      const int f = (j < chunk && slot.sprt_buf[j] >= 0) ? 1 : 0;
      int tot;
      const int pos = block_exclusive_scan(f, sh.red_i, &tot);
      if (list && f) {
        int pp = p0 + j;
        if (pp >= N) pp -= N;
        list[total + pos] = slot.sprt_pool[pp];
      }
      total += tot;
      sync();
    }
    return total;
  }

  // ------------------------------------------------------------------
  // Materialises the inlier list of a container's model into `list`.
  __device__ int materialise(const Container& c, int* list) {
    if (c.model == nullptr) return 0;
    if (c.start == -2) {
      // the first `len` kept points of the model's space partitioning
      sp_select(c.model);
      return exact_score_sp(c.model, list, c.len).count;
    }
    if (c.start >= 0) return sprt_list(c.model, c.start, c.len, list);
    return exact_score(c.model, list).count;
  }

  // GCRANSAC::iteratedLeastSquaresFitting (GCRANSAC.h:629-758) for estimators
  // with one model per fit. `list`/`n` is the container being refined in
  // place (its model is tracked through sh.work_model). Returns iterations > 1.
  __device__ bool irls(int*& list, int& n, int*& spare) {
    if (n <= m) return false;
    int iterations = 0;
    while (++iterations < 10) {
      // membership flags of the current set (the weights array of the reference)
      for (int i = threadIdx.x; i < N; i += GCR_BLOCK) slot.flag[i] = 0;
      sync();
      for (int k = threadIdx.x; k < n; k += GCR_BLOCK)
        if (row_ok(list[k])) slot.flag[list[k]] = 1;
      sync();
      // the FP32 mode starts each refit from the current model
      if (!fit_cta(list, n, 1, prm.lo_fp32 ? sh.work_model : nullptr)) break;
      const Score sc = exact_score(sh.fit_model, spare);
      ++models_scored;
      if (sc.count < m) break;
      if (sc.count <= n) break;
      copy_model(sh.work_model, sh.fit_model);
      int* t = list;
      list = spare;
      spare = t;
      n = sc.count;
    }
    return iterations > 1;
  }

  // ------------------------------------------------------------------
  // One batch of main-sampler calls [a0, a0 + GCR_BLOCK): thread j draws call
  // a0 + j, checks the sample, runs the minimal solver and writes its models
  // compacted into the slot table; sh.n_ok[j] / sh.mbase[j] describe them.
  // ------------------------------------------------------------------
  // AR sampler (samplers/adaptive_reordering_sampler.h:46-166). The driver
  // divides the probabilities by their maximum (gcransac_python.cpp:1731-1736);
  // each point enters a max-heap of (probability, index) with the estimator's
  // a, b; a sample pops the m largest entries (stale ones included) and the
  // update that follows every sample (GCRANSAC.h:304-335, 474-478) pushes each
  // sampled point back with |a / (a + b + appearances)| + jitter, clamped to
  // [0, 0.999]. The jitter, rand() in the reference, is
  // 0.01 u / (2^32 - 1) - 0.005 with u word q of the call's kStreamAr stream.
  // Probabilities that are not positive start at 1e-12 (the reference divides
  // by zero there). The state depends only on the calls, so thread 0 replays
  // a batch of calls ahead.
  __device__ __forceinline__ bool ar_greater(double pa, int ia, double pb, int ib) const {
    return pa > pb || (pa == pb && ia > ib);
  }
  __device__ void ar_sift_down(double* hp, int* hi, int n, int k) const {
    for (int it = 0; it < 64; ++it) {
      const int l = 2 * k + 1, r = l + 1;
      int best = k;
      if (l < n && ar_greater(hp[l], hi[l], hp[best], hi[best])) best = l;
      if (r < n && ar_greater(hp[r], hi[r], hp[best], hi[best])) best = r;
      if (best == k) return;
      const double tp = hp[k]; hp[k] = hp[best]; hp[best] = tp;
      const int ti = hi[k]; hi[k] = hi[best]; hi[best] = ti;
      k = best;
    }
  }
  __device__ void ar_push(double* hp, int* hi, int& n, double p, int i) const {
    int k = n++;
    hp[k] = p;
    hi[k] = i;
    for (int it = 0; it < 64 && k > 0; ++it) {
      const int parent = (k - 1) >> 1;
      if (!ar_greater(hp[k], hi[k], hp[parent], hi[parent])) break;
      const double tp = hp[k]; hp[k] = hp[parent]; hp[parent] = tp;
      const int ti = hi[k]; hi[k] = hi[parent]; hi[parent] = ti;
      k = parent;
    }
  }
  __device__ double* ar_hp() const { return prm.ar_p + (size_t)blockIdx.x * prm.ar_cap; }
  __device__ int* ar_hi() const { return prm.ar_i + (size_t)blockIdx.x * prm.ar_cap; }
  __device__ double* ar_a() const { return prm.ar_ab + (size_t)blockIdx.x * 2 * prm.ar_stride_n; }
  __device__ double* ar_b() const { return ar_a() + prm.ar_stride_n; }
  __device__ int* ar_c() const { return prm.ar_cnt + (size_t)blockIdx.x * prm.ar_stride_n; }

  __device__ void ar_init() {
    if (threadIdx.x == 0) {
      const double* pr = prm.probs + pd.offset;
      double mx = 0.0;
      for (int i = 0; i < N; ++i) mx = pr[i] > mx ? pr[i] : mx;
      double* hp = ar_hp();
      int* hi = ar_hi();
      double* A = ar_a();
      double* B = ar_b();
      int* C = ar_c();
      const double var = prm.sampler_variance;
      for (int i = 0; i < N; ++i) {
        double p = pr[i] / mx;
        if (p == 1.0) p -= 1e-6;
        if (!(p > 1e-12)) p = 1e-12;
        const double omp = 1.0 - p;
        const double a = __dsub_rn(__ddiv_rn(__dmul_rn(__dmul_rn(p, p), omp), var), p);
        A[i] = a;
        B[i] = __ddiv_rn(__dmul_rn(a, omp), p);
        C[i] = 0;
        hp[i] = p;
        hi[i] = i;
      }
      for (int k = N / 2 - 1; k >= 0; --k) ar_sift_down(hp, hi, N, k);
      sh.ar_size = N;
      sh.ar_overflow = 0;
    }
    sync();
  }

  // thread 0: the samples of calls a0 .. a0 + calls - 1 into slot.bsamples
  __device__ void ar_batch(long long a0, int calls) {
    if (threadIdx.x == 0) {
      double* hp = ar_hp();
      int* hi = ar_hi();
      const double* A = ar_a();
      const double* B = ar_b();
      int* C = ar_c();
      int n = sh.ar_size;
      for (int c = 0; c < calls; ++c) {
        if (sh.ar_overflow || n + m > prm.ar_cap || n < m) {
          sh.ar_overflow = 1;
          sh.s_cnt[c] = 0;
          continue;
        }
        int* smp = slot.bsamples + c * Est::M;
        for (int q = 0; q < m; ++q) {
          smp[q] = hi[0];
          --n;
          hp[0] = hp[n];
          hi[0] = hi[n];
          ar_sift_down(hp, hi, n, 0);
        }
        DrawStream ds(pd.seed, kStreamAr, (uint64_t)(a0 + c));
        for (int q = 0; q < m; ++q) {
          const int idx = smp[q];
          const int k = ++C[idx];
          const double r = fabs(__ddiv_rn(A[idx], __dadd_rn(__dadd_rn(A[idx], B[idx]), (double)k)));
          const double u = (double)ds.next_u32();
          double v = __dsub_rn(__dadd_rn(r, __dmul_rn(0.01, __ddiv_rn(u, 4294967295.0))), 0.005);
          v = v < 0.999 ? v : 0.999;
          v = v > 0.0 ? v : 0.0;
          ar_push(hp, hi, n, v, idx);
        }
        sh.s_cnt[c] = 1;
      }
      sh.ar_size = n;
    }
    sync();
  }

  // sampler calls per batch, within [1, GCR_BLOCK] whatever the parameter holds
  __device__ __forceinline__ int calls_per_batch() const { return max(1, min(GCR_BLOCK, prm.batch_calls)); }

  __device__ int generate_batch(long long a0, long long& p_kth, long long& p_subset, long long& p_hi,
                                double& p_Tn, long long& p_Tprime) {
    const int j = threadIdx.x;
    const int B = calls_per_batch();  // calls of this batch: a0 .. a0 + B - 1, one per thread j < B
    int s[Est::M];
#pragma unroll
    for (int q = 0; q < Est::M; ++q) s[q] = 0;
    bool ok = false;
    if (prm.tape != nullptr && !prm.nested) {
      // a recorded sample sequence replaces the sampler (the reference's
      // Sampler* plugin of GCRANSAC::run, GCRANSAC.h:69-76): call c reads row
      // c of the pair's tape; a call past its end or a row with an index
      // outside [0, N) is an unsuccessful sampler call
      const long long c = a0 + j;
      ok = j < B && c < prm.tape_calls;
      const int32_t* row = prm.tape + ((size_t)pair * (size_t)prm.tape_calls + (size_t)(ok ? c : 0)) * Est::M;
#pragma unroll
      for (int q = 0; q < Est::M; ++q) {
        const int v = ok ? row[q] : 0;
        if ((unsigned)v >= (unsigned)N) ok = false;
        s[q] = (unsigned)v < (unsigned)N ? v : 0;
      }
    } else if (prm.sampler == SAMPLER_PNAPSAC) {
      if (threadIdx.x == 0)
        for (int c = 0; c < B; ++c) {
          int t[Est::M];
          const bool o = napsac_call(t);
          for (int q = 0; q < Est::M; ++q) slot.bsamples[c * Est::M + q] = t[q];
          sh.s_cnt[c] = o ? 1 : 0;
        }
      sync();
      ok = j < B && sh.s_cnt[j] != 0;
#pragma unroll
      for (int q = 0; q < Est::M; ++q) s[q] = slot.bsamples[j * Est::M + q];
      sync();
    } else if (prm.sampler == SAMPLER_UNIFORM) {
      if (j < B) {
        DrawStream ds(pd.seed, prm.stream_main, (uint64_t)(a0 + j));
        ok = unique_set(ds, s, m, 0, (uint32_t)(N - 1));
      }
    } else if (prm.sampler == SAMPLER_AR) {
      ar_batch(a0, B);
      if (sh.ar_overflow && status == ST_OK) status = ST_CAPACITY;
      ok = j < B && sh.s_cnt[j] != 0;
#pragma unroll
      for (int q = 0; q < Est::M; ++q) s[q] = slot.bsamples[j * Est::M + q];
      sync();
    } else if (prm.sampler == SAMPLER_IMPORTANCE) {
      // ImportanceSampler::sample (samplers/importance_sampler.h:120-133):
      // m independent multinomial draws (repeats allowed), each a 53-bit
      // uniform u from two stream words and the first row whose cumulative
      // probability is not below u
      DrawStream ds(pd.seed, prm.stream_main, (uint64_t)(a0 + j));
      const double* cdf = prm.cdf + pd.offset;
      for (int q = 0; q < m && j < B; ++q) {
        const uint32_t w0 = ds.next_u32(), w1 = ds.next_u32();
        const double u = ((double)(w0 >> 5) * 67108864.0 + (double)(w1 >> 6)) * (1.0 / 9007199254740992.0);
        int lo = 0, hi = N - 1;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (cdf[mid] < u) lo = mid + 1;
          else hi = mid;
        }
        s[q] = lo;
      }
      ok = j < B;
    } else {
      // PROSAC (samplers/prosac_sampler.h:51-237): every thread replays the
      // state machine for the whole batch and keeps its own call's draw range.
      const long long conv = 100000;
      long long my_hi = 0, my_last = 0;
      bool my_global = false;
      for (int c = 0; c < B; ++c) {
        if (c == j) {
          my_global = p_kth > conv;
          my_hi = p_hi;
          my_last = p_subset - 1;
        }
        if (p_kth > conv) continue;
        ++p_kth;
        if (p_kth > conv) {
          p_hi = N - 1;
        } else {
          // growth[subset - 1] is kept in p_Tprime; compute the next one lazily
          if (p_kth > p_Tprime) {
            const long long before = p_subset;
            ++p_subset;
            if (p_subset > N) p_subset = N;
            p_hi = p_subset - 2;
            // advance the growth function to index p_subset - 1
            const long long i = p_subset - 1;
            if (p_subset != before && i + 1 > m) {
              const double Tn1 = (double)(i + 1) * p_Tn / (double)(i + 1 - m);
              p_Tprime = p_Tprime + (long long)(unsigned int)ceil(Tn1 - p_Tn);
              p_Tn = Tn1;
            }
          }
        }
      }
      DrawStream ds(pd.seed, prm.stream_main, (uint64_t)(a0 + j));
      if (j >= B) {
        ok = false;
      } else if (my_global) {
        ok = unique_set(ds, s, m, 0, (uint32_t)(N - 1));
      } else {
        ok = unique_set(ds, s, m - 1, 0, (uint32_t)my_hi);
        s[m - 1] = (int)my_last;
      }
    }
    double mloc[9 * Est::MAXSOL];
    int nm = 0;
    if constexpr (Est::AFFINE) {
      if (ok && Est::valid_sample_affine(pts64, affine64, s)) nm = Est::minimal_affine(pts64, affine64, s, mloc);
    } else {
      if (ok && Est::valid_sample(pts64, s)) nm = Est::minimal(pts64, s, mloc, prm.pp_h);
    }
#pragma unroll
    for (int q = 0; q < Est::M; ++q) slot.bsamples[j * Est::M + q] = s[q];
    int total;
    const int base = block_exclusive_scan(nm, sh.red_i, &total);
    sh.n_ok[j] = nm;
    sh.mbase[j] = base;
    for (int q = 0; q < nm; ++q) {
      double* dst = slot.models64 + 9 * (base + q);
#pragma unroll
      for (int k = 0; k < 9; ++k) dst[k] = mloc[9 * q + k];
      put_f32(base + q);
    }
    sync();
    return total;
  }

  // ------------------------------------------------------------------
  __device__ void run() {
    if (threadIdx.x == 0) sh.bad_row = 0;
    sync();
    long long t0 = tick();
    // the sampler's layer grids use cell_start as scratch, so they come
    // before the neighbourhood grid that keeps it
    if (prm.sampler == SAMPLER_PNAPSAC) napsac_setup();
    if (prm.sampler == SAMPLER_AR) ar_init();
    const int ncells = prm.nested ? 0 : build_grid();
    if (prm.neighborhood == 1 && prm.lambda > 0 && !prm.nested) {
      rg_ok = build_radius_graph();
      if (!rg_ok && status == ST_OK) status = ST_CAPACITY;
    }
    if (prm.use_sprt && !prm.nested) sprt_init();
    if constexpr (Est::KIND == 0)
      if (prm.use_sp && !prm.nested && ncells > 0) sp_init(ncells);
    tock(0, t0);
    max_iter = iteration_number_for(1, N, m, log_prob);
    const long long max_iters = prm.max_iters, min_iters = prm.min_iters;
    // PROSAC state: kth, subset size, draw range, T_n, growth[subset-1]
    long long p_kth = 1, p_subset = m, p_hi = m - 1, p_Tprime = 1;
    double p_Tn = 100000.0;
    for (int i = 0; i < m; ++i) p_Tn *= (double)(m - i) / (double)(N - i);
    long long attempt = 0;
    bool done = false, in_iter = false;
    int nfail = 0;
    const long long attempt_cap = (max_iters < 0x7fffffffLL ? max_iters : 0x7fffffffLL) * 101 + 101;
    while (!done) {
      t0 = tick();
      generate_batch(attempt, p_kth, p_subset, p_hi, p_Tn, p_Tprime);
      tock(1, t0);
      t0 = tick();
      const int K = sh.mbase[GCR_BLOCK - 1] + sh.n_ok[GCR_BLOCK - 1];
      if (!sprt && !(sp && !mag)) score_models_f32(0, K);
      tock(2, t0);
      bool restart = false;
      long long next_attempt = attempt + calls_per_batch();
      for (int j = 0; j < calls_per_batch(); ++j) {
        if (!in_iter) {
          const long long lim = max_iter < max_iters ? max_iter : max_iters;
          if (!(min_iters > iter || iter < lim)) {
            done = true;
            if (prm.nested) lo_calls = attempt + j;  // one stream: the next call follows
            break;
          }
          ++iter;
          in_iter = true;
          nfail = 0;
        }
        const int nm = sh.n_ok[j];
        if (nm == 0) {
          if (++nfail == 100) {
            iter += 100;
            in_iter = false;
          }
          continue;
        }
        iter += nfail;
        in_iter = false;
        bool do_lo = false;
        for (int q = 0; q < nm; ++q) {
          const int k = sh.mbase[j] + q;
          const double* mk = slot.models64 + 9 * k;
          ++models_scored;
          Score sc;
          if (sp) {
            // GCRANSAC.h:343-366: rejected when the kept cells hold fewer
            // points than the best model has inliers
            sp_select(mk);
            if (sp_count < best.count) continue;
          }
          if (sprt) {
            // SPRT provides the score (GCRANSAC.h:370-431)
            int st0 = 0, ln = 0;
            t0 = tick();
            bool passed;
            if (sp) {
              passed = sprt_verify_sp(mk, slot.models32 + 12 * k, sc, Est::CTA_VALIDITY ? slot.list1 : nullptr, ln);
              st0 = -2;
            } else {
              passed = sprt_verify(mk, slot.models32 + 12 * k, sc, Est::CTA_VALIDITY ? slot.list1 : nullptr, st0, ln);
            }
            tock(3, t0);
            Container ct;
            ct.model = mk;
            ct.count = sc.count;
            ct.start = st0;
            ct.len = ln;
            cont[off] = ct;
            if (!passed) continue;
          } else if (sp && !mag) {
            // MSAC over the kept points, cell by cell
            sc = exact_score_sp(mk, Est::CTA_VALIDITY ? slot.list1 : nullptr);
            Container ct;
            ct.model = mk;
            ct.count = sc.count;
            ct.start = -2;
            ct.len = sp_count;
            cont[off] = ct;
            if (sc.count == 0) continue;
          } else {
            cont[off] = {mk, sh.mcount[k]};
            if (sh.mcount[k] == 0 || !maybe_better(k, best.value)) continue;
            t0 = tick();
            sc = exact_score(mk, Est::CTA_VALIDITY ? slot.list1 : nullptr, slot.models32 + 12 * k);
            tock(3, t0);
            tock(9, 0, 1);
          }
          bool updated = false;
          bool valid = false;
          if (best.value < sc.value) {
            if constexpr (Est::CTA_VALIDITY)
              valid = valid_model_cta(mk, slot.bsamples + j * Est::M, slot.list1, sc.count, updated);
            else
              valid = Est::valid_model(mk);
          }
          if (valid) {
            Score scb = sc;
            const double* mb = mk;
            if (updated) {
              // DEGENSAC replaced the model: rescore it into the container
              copy_model(sh.cont_model[off], sh.degen_H);
              scb = exact_score(sh.cont_model[off], nullptr);
              cont[off] = {sh.cont_model[off], scb.count};
              mb = sh.cont_model[off];
            }
            off ^= 1;
            copy_model(sh.best_model, mb);
            best = scb;
            do_lo = iter > 20 && best.count > m;
            max_iter = iteration_number_for(best.count, N, m, log_prob);
          }
        }
        if (do_lo) {
          ++lo_number;
          if (prm.nested) lo_calls = attempt + j + 1;  // one stream: LO draws follow this attempt
          t0 = tick();
          local_optimization(ncells);
          tock(11, t0);
          max_iter = iteration_number_for(best.count, N, m, log_prob);
          if (prm.nested) {
            // later attempts of this batch used call indices the LO consumed
            next_attempt = lo_calls;
            restart = true;
            break;
          }
        }
      }
      attempt = next_attempt;
      (void)restart;
      // containers that point into the batch table are copied out before reuse
      for (int c = 0; c < 2; ++c) {
        if (cont[c].model != nullptr && cont[c].model >= slot.models64 &&
            cont[c].model < slot.models64 + 9 * kBatchModels) {
          copy_model(sh.cont_model[c], cont[c].model);
          cont[c].model = sh.cont_model[c];
        }
      }
      if (attempt > attempt_cap) {
        if (status == ST_OK) status = ST_TIMEOUT;
        done = true;
      }
    }
    t0 = tick();
    finish(ncells);
    tock(8, t0);
  }

  // A pair the engine does not run: status st, a zero model, an empty mask
  // and zero counts.
  __device__ void reject(int st) {
    StatsOut* so = ws.stats_out + pair;
    uint8_t* mask = ws.masks_out + pd.offset;
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) mask[i] = 0;
    if (threadIdx.x < 9) ws.models_out[9 * pair + threadIdx.x] = 0.0;
    if (threadIdx.x == 0) {
      so->iteration_number = 0;
      so->graph_cut_number = 0;
      so->local_optimization_number = 0;
      so->inlier_number = 0;
      so->score = 0.0;
      so->status = st;
      so->flags = 0;
      so->models_scored = 0;
    }
    sync();
  }

  __device__ void finish(int ncells) {
    StatsOut* so = ws.stats_out + pair;
    uint8_t* mask = ws.masks_out + pd.offset;
    if (prm.nested && best.count <= m) {
      if (threadIdx.x == 0) sh.result_count = 0;
      sync();
      return;
    }
    if (best.count <= m) {
      for (int i = threadIdx.x; i < N; i += GCR_BLOCK) mask[i] = 0;
      if (threadIdx.x < 9) ws.models_out[9 * pair + threadIdx.x] = 0.0;
      if (threadIdx.x == 0) {
        so->iteration_number = iter;
        so->graph_cut_number = gc_number;
        so->local_optimization_number = lo_number;
        so->inlier_number = 0;
        so->score = best.value;
        so->status = status == ST_OK ? ST_NO_MODEL : status;
        so->flags = flags;
        so->models_scored = models_scored;
      }
      return;
    }
    if (lo_number == 0) {
      ++lo_number;
      local_optimization(ncells);
    }
    if (cont[off].count != best.count) off ^= 1;
    if (cont[off].count != best.count) {
      copy_model(sh.cont_model[off], sh.best_model);
      best = exact_score(sh.best_model, nullptr);
      cont[off] = {sh.cont_model[off], best.count};
    }
    // materialise the container; the IRLS refines it in place
    int* list = slot.list1;
    int* spare = slot.list2;
    int n = materialise(cont[off], list);
    copy_model(sh.work_model, sh.best_model);
    bool irls_applied = false;
    bool ok = false;
    if (prm.final_irls) {
      if constexpr (Est::LO_MAXSOL > 1) ok = irls_multi(list, n, spare);
      else ok = irls(list, n, spare);
    }
    if (ok) {
      // the container now holds the inliers of the IRLS model
      copy_model(sh.cont_model[off], sh.work_model);
      cont[off] = {sh.cont_model[off], n};
      const int idx = off ^ 1;
      const Score sc = exact_score(sh.work_model, nullptr);
      copy_model(sh.cont_model[idx], sh.work_model);
      cont[idx] = {sh.cont_model[idx], sc.count};
      if (best.value < sc.value) {
        irls_applied = true;
        copy_model(sh.best_model, sh.work_model);
        off = idx;
      }
    }
    if (Est::LO_MAXSOL > 1 && !irls_applied) {
      // one fit on the first best.count points of the container; every model
      // better than the run's best takes the other container
      const int nm = fit_cta_multi(list, best.count < n ? best.count : n, 0, true);
      for (int q = 0; q < nm; ++q) {
        const int idx = off ^ 1;
        const Score sc = exact_score(sh.multi_models + 9 * q, nullptr);
        copy_model(sh.cont_model[idx], sh.multi_models + 9 * q);
        cont[idx] = {sh.cont_model[idx], sc.count};
        if (best.value < sc.value) {
          copy_model(sh.best_model, sh.multi_models + 9 * q);
          off = idx;
        }
      }
    } else if (!irls_applied) {
      // one least-squares fit on the first best.count points of the container
      if (fit_cta(list, best.count < n ? best.count : n, 0, prm.lo_fp32 ? sh.best_model : nullptr)) {
        const int idx = off ^ 1;
        const Score sc = exact_score(sh.fit_model, nullptr);
        copy_model(sh.cont_model[idx], sh.fit_model);
        cont[idx] = {sh.cont_model[idx], sc.count};
        if (best.value < sc.value) {
          copy_model(sh.best_model, sh.fit_model);
          off = idx;
        }
      }
    }
    if (irls_applied) flags |= 2;
    if (lo_number > 0) flags |= 1;
    // output: model and the inliers of the final container
    int cnt = materialise(cont[off], list);
    double final_score = best.value;
    if constexpr (Est::KIND == 1) if (prm.epilogue) {
      // findFundamentalMatrix_ epilogue (gcransac_python.cpp:1833-1889):
      // weighted bundle adjustment of the final inliers on the raw
      // coordinates, kept when its MSAC score beats the run's score; at most 7
      // inliers give the identity.
      if (cnt > 7) {
        double Fb[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) Fb[q] = sh.best_model[q];
        // the affine-correspondence driver runs it without weights
        // (gcransac_python.cpp:2157-2163)
        constexpr int wmode = Est::EPILOGUE_WEIGHTED ? 2 : 0;
        if constexpr (Est::EPILOGUE_WEIGHTED) {
          for (int k = threadIdx.x; k < cnt; k += GCR_BLOCK)
            slot.dres[k] = fmax(0.0, 1.0 - Est::r2_f64(row64(list[k]), Fb) / t2);
        }
        sync();
        if (fit_cta_f(list, cnt, wmode, false, true, prm.lo_fp32 ? sh.best_model : nullptr)) {
          const Score sc = exact_score(sh.fit_model, spare, nullptr, true);
          if (final_score < sc.value) {
            final_score = sc.value;
            copy_model(sh.best_model, sh.fit_model);
            int* t = list;
            list = spare;
            spare = t;
            cnt = sc.count;
          }
        }
      } else {
        sync();
        if (threadIdx.x < 9) sh.best_model[threadIdx.x] = (threadIdx.x % 4 == 0) ? 1.0 : 0.0;
        sync();
      }
    }
    if constexpr (Est::KIND == 3) if (prm.epilogue) {
      // findEssentialMatrix_ epilogue (gcransac_python.cpp:2770-2828): the
      // essential-matrix bundle adjustment of the final inliers (Stewenius
      // start, every cheirality-consistent pose refined), each result kept
      // when its MSAC score beats the best so far; at most 5 inliers give
      // the identity. Weights by inlier position.
      if (cnt > 5) {
        double Eb[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) Eb[q] = sh.best_model[q];
        for (int k = threadIdx.x; k < cnt; k += GCR_BLOCK)
          slot.dres[k] = fmax(0.0, 1.0 - Est::r2_f64(row64(list[k]), Eb) / t2);
        sync();
        const int nm = fit_cta_multi(list, cnt, 2, false);
        double x1[3], x2[3];
        {
          const double* p0 = row64(list[0]);
          x1[0] = p0[0]; x1[1] = p0[1]; x1[2] = 1.0;
          x2[0] = p0[2]; x2[1] = p0[3]; x2[2] = 1.0;
          const double n1 = sqrt(x1[0] * x1[0] + x1[1] * x1[1] + 1.0);
          const double n2 = sqrt(x2[0] * x2[0] + x2[1] * x2[1] + 1.0);
          for (int i = 0; i < 3; ++i) {
            x1[i] /= n1;
            x2[i] /= n2;
          }
        }
        // the bundle adjustment reads the original inliers (ba, ba_n) while
        // accepted results go to the two other lists
        const int* ba = list;
        const int ba_n = cnt;
        int* cur = list;
        int* tmp = spare;
        double Em[9 * Shared<Est>::kMulti];
        for (int q = 0; q < 9 * nm; ++q) Em[q] = sh.multi_models[q];
        auto consider = [&](const double* Eq) {
          sync();
          if (threadIdx.x < 9) sh.fit_model[threadIdx.x] = Eq[threadIdx.x];
          sync();
          const Score sc = exact_score(sh.fit_model, tmp, nullptr, true);
          if (final_score < sc.value) {
            final_score = sc.value;
            copy_model(sh.best_model, sh.fit_model);
            cur = tmp;
            tmp = (tmp == spare) ? slot.list0 : spare;
            cnt = sc.count;
          }
        };
        for (int q = 0; q < nm; ++q) {
          double Eq[9];
#pragma unroll
          for (int e = 0; e < 9; ++e) Eq[e] = Em[9 * q + e];
          if constexpr (nonmin_ba<Est>()) {
            // the non-minimal solver is the bundle adjustment itself: its
            // models are already the refined poses
            consider(Eq);
          } else {
            ess::Pose poses[4];
            const int np = ess::poses_from_essential(Eq, x1, x2, poses);
            for (int v = 0; v < np; ++v) {
              ess::Pose P = poses[v];
              refine_relpose_cta(ba, ba_n, P);
              ess::essential_from_pose(P, Eq);
              consider(Eq);
            }
          }
        }
        list = cur;
      } else {
        sync();
        if (threadIdx.x < 9) sh.best_model[threadIdx.x] = (threadIdx.x % 4 == 0) ? 1.0 : 0.0;
        sync();
      }
    }
    if (prm.nested) {
      sync();
      if (threadIdx.x < 9) sh.result_model[threadIdx.x] = sh.best_model[threadIdx.x];
      if (threadIdx.x == 0) sh.result_count = cnt;
      sync();
      return;
    }
    for (int i = threadIdx.x; i < N; i += GCR_BLOCK) mask[i] = 0;
    sync();
    for (int k = threadIdx.x; k < cnt; k += GCR_BLOCK)
      if (row_ok(list[k])) mask[list[k]] = 1;
    if (threadIdx.x < 9) ws.models_out[9 * pair + threadIdx.x] = sh.best_model[threadIdx.x];
    sync();
    if (sh.bad_row && status == ST_OK) status = ST_DEVICE_ERROR;
    if (threadIdx.x == 0) {
      so->iteration_number = iter;
      so->graph_cut_number = gc_number;
      so->local_optimization_number = lo_number;
      so->inlier_number = cnt;
      so->score = final_score;
      so->status = status;
      so->flags = flags;
      so->models_scored = models_scored;
    }
    sync();
  }
};

}  // namespace gcr
