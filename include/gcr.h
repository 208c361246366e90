/*
 * gcr.h — C-ABI of the GB300 Graph-Cut RANSAC engine (libgcr.so).
 *
 * This is the drop-in boundary for the hypothesize-and-verify path of
 * danini/graph-cut-ransac. Every entry point takes plain pointers and sizes,
 * never throws, and reports failures through gcr_status plus
 * gcr_last_error_string(). The caller owns every buffer.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   gcr_find_homography   <- findHomography_        src/pygcransac/src/gcransac_python.cpp:4221
 *                            (python: findHomography src/pygcransac/src/bindings.cpp:859-983)
 *   gcr_find_fundamental  <- findFundamentalMatrix_ src/pygcransac/src/gcransac_python.cpp:1600
 *                            (python: findFundamentalMatrix src/pygcransac/src/bindings.cpp:279-401)
 *   gcr_find_essential    <- findEssentialMatrix_   src/pygcransac/src/gcransac_python.cpp:2519
 *                            (python: findEssentialMatrix src/pygcransac/src/bindings.cpp:710-857)
 *   gcr_find_batch / gcr_batch_run_device
 *                         <- a loop of the three calls above, one per image pair
 *                            (the reference has no batched form)
 *   gcr_params            <- gcransac::utils::Settings src/pygcransac/include/settings.h:44-87
 *                            plus the driver arguments of the find*_ functions
 *   gcr_stats             <- gcransac::utils::RANSACStatistics src/pygcransac/include/statistics.h:43-72
 */
#ifndef GCR_H_
#define GCR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gcr_status {
  GCR_OK = 0,
  GCR_INVALID_ARG = 1,     /* bad pointer, shape or parameter value; per pair: a
                              coordinate that is not finite (the pair is not run) */
  GCR_TOO_FEW_POINTS = 2,  /* fewer correspondences than the minimal sample */
  GCR_NO_MODEL = 3,        /* the run ended without a model of more than m inliers */
  GCR_DEVICE_ERROR = 4,    /* a CUDA call failed, or (per pair) the engine's
                              row-index check caught an index outside the pair */
  GCR_TIMEOUT = 5,         /* a device loop reached its iteration cap */
  GCR_CAPACITY = 6,        /* an input exceeds a documented size limit */
  GCR_UNSUPPORTED = 7      /* option combination not provided by this build */
} gcr_status;

/* Correspondence rows hold 4 doubles (x1, y1, x2, y2) for the point kinds and
 * 8 for the others: for the affine kinds the point pair followed by the 2x2
 * local affine map (a11, a12, a21, a22) of the affine correspondence, the
 * layout of the reference's findHomographyAC_ and findFundamentalMatrixAC_
 * (gcransac_python.cpp:4553, 1924; solver = 2 of the python findHomography and
 * findFundamentalMatrix); for the SIFT kinds the point pair followed by the
 * features' scales and orientations (q1, q2, o1, o2), the layout of
 * findFundamentalMatrixSIFT_ and findHomographySIFT_ (:2222, 4813; solver = 1
 * of findFundamentalMatrix and findHomography). */
typedef enum gcr_model_kind {
  GCR_HOMOGRAPHY = 0,
  GCR_FUNDAMENTAL = 1,
  GCR_ESSENTIAL = 2,
  GCR_HOMOGRAPHY_AFFINE = 3,
  GCR_FUNDAMENTAL_AFFINE = 4,
  GCR_FUNDAMENTAL_SIFT = 5,
  GCR_HOMOGRAPHY_SIFT = 6,
  GCR_ESSENTIAL_PLANAR = 7  /* rows of 4; planar camera motion */
} gcr_model_kind;

/* Sampler ids follow examples/gcransac_parameter_types.py:8-12 of the reference. */
enum {
  GCR_SAMPLER_UNIFORM = 0,
  GCR_SAMPLER_PROSAC = 1,
  GCR_SAMPLER_PNAPSAC = 2,
  GCR_SAMPLER_IMPORTANCE = 3,     /* needs per-correspondence probabilities */
  GCR_SAMPLER_AR = 4               /* needs per-correspondence probabilities */
};

enum { GCR_NEIGHBORHOOD_GRID = 0, GCR_NEIGHBORHOOD_FLANN = 1 };
enum { GCR_SCORING_MSAC = 0, GCR_SCORING_MAGSAC = 1 };

typedef struct gcr_image_size {
  int32_t h1, w1, h2, w2;
} gcr_image_size;

typedef struct gcr_params {
  double threshold;                /* inlier-outlier threshold in pixels */
  double confidence;               /* RANSAC confidence, e.g. 0.99 */
  double spatial_coherence_weight; /* lambda of the graph-cut energy */
  double neighborhood_size;        /* grid divisions along every axis */
  int64_t max_iterations;
  int64_t min_iterations;
  int32_t sampler;                 /* GCR_SAMPLER_* */
  int32_t neighborhood;            /* GCR_NEIGHBORHOOD_GRID only */
  int32_t lo_number;               /* inner-RANSAC trials per graph-cut */
  int32_t scoring;                 /* GCR_SCORING_* */
  int32_t use_sprt;                /* SPRT preemptive verification of main-loop models */
  int32_t use_space_partitioning;  /* homographies: space-partitioning pre-selection of models */
  uint64_t seed;                   /* seed of the counter-based sampler streams */
  double min_inlier_ratio_for_sprt; /* SPRT's initial inlier-ratio guess (epsilon); the homography
                                      drivers start from 0.01 whatever this holds, as the reference's
                                      findHomography_ / findHomographyAC_ construct their SPRT test */
  double sampler_variance;         /* AR sampler (4): variance of the inlier-probability estimator */
} gcr_params;

typedef struct gcr_stats {
  int64_t iteration_number;
  int64_t graph_cut_number;
  int64_t local_optimization_number;
  int64_t inlier_number;
  double score;
  int32_t status;                  /* gcr_status of this pair */
  int32_t flags;                   /* GCR_FLAG_* */
  int64_t models_scored;           /* models the sequential algorithm scores against all
                                      correspondences (main loop + local optimisation) */
} gcr_stats;

enum {
  GCR_FLAG_LO_APPLIED = 1,         /* at least one graph-cut local optimisation ran */
  GCR_FLAG_IRLS_APPLIED = 2,       /* the final iterated least-squares model was kept */
  GCR_FLAG_DEGENSAC_SKIPPED = 4,   /* an H-degenerate F sample kept its model without the
                                      plane-and-parallax inner run */
  GCR_FLAG_DEGENSAC_RAN = 8        /* the plane-and-parallax inner run of DEGENSAC ran */
};

/* Fills *p with the defaults of the reference python entry point of `kind`
 * (src/pygcransac/src/bindings.cpp:1003-1022, 1091-1112, 1158-1178). */
void gcr_default_params(gcr_model_kind kind, gcr_params* p);

/* Single image pair, host buffers.
 *   corr           n x 4 row-major doubles (x1, y1, x2, y2)
 *   probabilities  n doubles or NULL (read only by the importance and AR samplers, 3 and 4)
 *   model_out9     3x3 row-major model
 *   mask_out       n bytes, 1 = inlier
 *   stats_out      may be NULL
 * Returns GCR_NO_MODEL (mask all zero) when no model was found, like the
 * reference returning (None, mask). */
gcr_status gcr_find_homography(const double* corr, int64_t n, const gcr_image_size* size,
                               const double* probabilities, const gcr_params* params,
                               double* model_out9, uint8_t* mask_out, gcr_stats* stats_out);

gcr_status gcr_find_fundamental(const double* corr, int64_t n, const gcr_image_size* size,
                                const double* probabilities, const gcr_params* params,
                                double* model_out9, uint8_t* mask_out, gcr_stats* stats_out);

/* K1, K2: 3x3 row-major intrinsics of the two cameras. */
gcr_status gcr_find_essential(const double* corr, int64_t n, const double* K1, const double* K2,
                              const gcr_image_size* size, const double* probabilities,
                              const gcr_params* params, double* model_out9, uint8_t* mask_out,
                              gcr_stats* stats_out);

/* Affine-correspondence homography on one image pair (findHomographyAC_,
 * gcransac_python.cpp:4553-4811; python findHomography with solver = 2).
 *   corr  n x 8 row-major doubles (x1, y1, x2, y2, a11, a12, a21, a22); the
 *         minimal sample is two correspondences: the point rows of both and
 *         the affine rows of the first (solver_homography_two_affine.h:88-237)
 * Samplers 0, 1, 3, 4 (the reference's driver refuses P-NAPSAC), MSAC; the
 * grid is built on the point columns with cells w / n only when the spatial
 * weight is above machine epsilon; SPRT starts from the inlier ratio 0.01, as
 * the reference's driver constructs it; no space partitioning. Other
 * arguments as for gcr_find_homography. */
gcr_status gcr_find_homography_affine(const double* corr, int64_t n, const gcr_image_size* size,
                                      const double* probabilities, const gcr_params* params,
                                      double* model_out9, uint8_t* mask_out, gcr_stats* stats_out);

/* Affine-correspondence fundamental matrix on one image pair
 * (findFundamentalMatrixAC_, gcransac_python.cpp:1924-2221; python
 * findFundamentalMatrix with solver = 2): rows of 8 as above; three
 * correspondences per minimal sample (the epipolar row of each and the affine
 * rows of the first two, solver_fundamental_matrix_three_affine.h:84-250); no
 * DEGENSAC; samplers 0, 1, 3, 4, MSAC; the driver's bundle adjustment of the
 * final inliers without weights. Other arguments as for gcr_find_fundamental. */
gcr_status gcr_find_fundamental_affine(const double* corr, int64_t n, const gcr_image_size* size,
                                       const double* probabilities, const gcr_params* params,
                                       double* model_out9, uint8_t* mask_out, gcr_stats* stats_out);

/* SIFT-correspondence fundamental matrix on one image pair
 * (findFundamentalMatrixSIFT_, gcransac_python.cpp:2222-2518; python
 * findFundamentalMatrix with solver = 1): rows (x1, y1, x2, y2, q1, q2, o1,
 * o2); four correspondences per minimal sample (the epipolar row of each and
 * the orientation-scale row of the first three,
 * solver_fundamental_matrix_four_sift.h:89-250); otherwise as
 * gcr_find_fundamental_affine. */
gcr_status gcr_find_fundamental_sift(const double* corr, int64_t n, const gcr_image_size* size,
                                     const double* probabilities, const gcr_params* params, double* model_out9,
                                     uint8_t* mask_out, gcr_stats* stats_out);

/* Essential matrix of a planar camera motion (rotation about the camera's y
 * axis, translation in its x-z plane) on one image pair
 * (findPlanarEssentialMatrix_, gcransac_python.cpp:3531-3870; python
 * findPlanarEssentialMatrix): rows of 4 pixels, K1 and K2 as for
 * gcr_find_essential. Two correspondences per minimal sample
 * (solver_essential_matrix_two_points_planar.h:92-175, up to four models);
 * the non-minimal solver is the essential-matrix bundle adjustment (Stewenius
 * start, every cheirality-consistent pose refined, at least 6 rows); MSAC
 * only; with use_sprt the run makes up to 100 graph cuts and skips the final
 * iteratively reweighted fit (3741-3742); the AR sampler's variance is 0.1;
 * the driver's epilogue as for gcr_find_essential. */
gcr_status gcr_find_essential_planar(const double* corr, int64_t n, const double* K1, const double* K2,
                                     const gcr_image_size* size, const double* probabilities, const gcr_params* params,
                                     double* model_out9, uint8_t* mask_out, gcr_stats* stats_out);

/* SIFT-correspondence homography on one image pair (findHomographySIFT_,
 * gcransac_python.cpp:4813-5069; python findHomography with solver = 1): rows
 * (x1, y1, x2, y2, q1, q2, o1, o2); two correspondences per minimal sample
 * (two point rows and one orientation row each, then the two scale-ratio
 * conics on the null space, solver_homography_two_sift.h:113-480, up to four
 * models); samplers 0, 1, 3, 4, MSAC, no space partitioning, SPRT from the
 * inlier ratio 0.01. Other arguments as for gcr_find_homography. */
gcr_status gcr_find_homography_sift(const double* corr, int64_t n, const gcr_image_size* size,
                                    const double* probabilities, const gcr_params* params, double* model_out9,
                                    uint8_t* mask_out, gcr_stats* stats_out);

/* Many image pairs of one model kind in one device launch, host buffers.
 *   corr        concatenated correspondences, offsets[num_pairs] rows in total
 *               (rows of 4 doubles, or of 8 for the affine kinds)
 *   offsets     num_pairs + 1 row offsets (ragged pairs)
 *   K           num_pairs * 18 doubles (K1 then K2 per pair) for GCR_ESSENTIAL, else NULL
 *   sizes       num_pairs image sizes
 *   params      one parameter set shared by all pairs
 *   seeds       num_pairs seeds, or NULL for params->seed + pair index
 *   models_out  num_pairs * 9, masks_out offsets[num_pairs] bytes, stats_out num_pairs
 * Returns GCR_OK when the launch succeeded; per-pair outcomes are in stats_out[i].status. */
gcr_status gcr_find_batch(gcr_model_kind kind, int64_t num_pairs, const double* corr,
                          const int64_t* offsets, const double* K, const gcr_image_size* sizes,
                          const gcr_params* params, const uint64_t* seeds, double* models_out,
                          uint8_t* masks_out, gcr_stats* stats_out);

/* Device-resident form of gcr_find_batch: the bulk arrays (correspondences,
 * models, masks, statistics) are device pointers of the current CUDA device,
 * the small per-pair metadata (offsets, intrinsics, image sizes, seeds) are
 * host arrays. The work is queued on `stream` (a cudaStream_t, NULL for the
 * legacy default stream) and the call returns without waiting. Scratch memory
 * is owned by `ctx`, which grows it on demand; one context per host thread. */
typedef struct gcr_context gcr_context;

gcr_status gcr_context_create(gcr_context** ctx);
gcr_status gcr_context_destroy(gcr_context* ctx);

gcr_status gcr_batch_run_device(gcr_context* ctx, gcr_model_kind kind, int64_t num_pairs,
                                const double* d_corr, const int64_t* h_offsets, const double* h_K,
                                const gcr_image_size* h_sizes, const gcr_params* params,
                                const uint64_t* h_seeds, double* d_models_out,
                                uint8_t* d_masks_out, gcr_stats* d_stats_out, void* stream);

/* Allocation-free homography search on one image pair (no counterpart in the
 * reference, whose C++ and Python entry points allocate on the host as they
 * go). For callers that must not allocate device memory while they run: a
 * process whose device memory is reserved up front by another allocator, or
 * a real-time loop where the device-wide synchronisation of cudaMalloc and
 * cudaFree would stall other streams. All scratch lives in one fixed 5 MiB
 * array per device compiled into the library; the call makes no cudaMalloc,
 * cudaFree or other allocating call and queues one kernel on `stream`.
 *   d_corr        n x 4 row-major doubles on the current device, n <= 4096
 *                 (larger n returns GCR_CAPACITY: use gcr_batch_run_device)
 *   size, params  host structs, as for gcr_find_homography
 *   seed          the pair's sampler seed
 *   d_model_out9, d_mask_out (n bytes), d_stats_out: device pointers, fully
 *                 written by the kernel; nothing needs to be cleared first
 * The first call on a device does a one-time set-up with that device current;
 * make it before any stream capture begins. Calls on the same device share
 * the scratch: calls that overlap in time (two host threads, or two streams
 * that run concurrently) race, so queue them on one stream or serialise them.
 * Returns when the kernel is queued; the per-pair outcome is d_stats_out->status. */
gcr_status gcr_find_homography_device_noalloc(const double* d_corr, int64_t n,
                                              const gcr_image_size* size, const gcr_params* params,
                                              uint64_t seed, double* d_model_out9, uint8_t* d_mask_out,
                                              gcr_stats* d_stats_out, void* stream);

/* gcr_batch_run_device split in two, for CUDA-graph capture. gcr_batch_prepare
 * does the host side (argument checks, scratch growth, per-pair descriptor and
 * intrinsics uploads; it returns after those copies complete) and records the
 * batch's device work in ctx. gcr_batch_launch queues that device work on
 * `stream`: a memset and kernel launches only, no allocation and no host
 * copies, so it can be recorded into a CUDA graph and replayed; each replay
 * re-runs the batch on the current contents of the device buffers given to
 * gcr_batch_prepare (new correspondences of the same sizes may be written there
 * between replays). The prepared batch keeps the addresses of the device
 * buffers given here: they must stay allocated for as long as a launch or a
 * captured graph of the batch may run (a caching allocator that hands a
 * released buffer back to the driver turns a later replay into writes to
 * freed memory). A prepared batch stays valid until the next
 * gcr_batch_prepare or gcr_batch_run_device on the same context. */
gcr_status gcr_batch_prepare(gcr_context* ctx, gcr_model_kind kind, int64_t num_pairs,
                             const double* d_corr, const int64_t* h_offsets, const double* h_K,
                             const gcr_image_size* h_sizes, const gcr_params* params,
                             const uint64_t* h_seeds, double* d_models_out, uint8_t* d_masks_out,
                             gcr_stats* d_stats_out);
gcr_status gcr_batch_launch(gcr_context* ctx, void* stream);

/* Probabilities of the importance sampler (sampler 3,
 * samplers/importance_sampler.h:51-136) for the batches prepared on `ctx` from
 * now on: d_probabilities [total] (device, non-negative, laid out like the
 * correspondences); NULL switches it off. The single-pair entries take the
 * same weights through their `probabilities` argument (host), which the other
 * samplers ignore, as in the reference. */
gcr_status gcr_context_set_probabilities(gcr_context* ctx, const double* d_probabilities);

/* Per-pair timing of the batches prepared on `ctx` from now on (no counterpart
 * in the reference, whose statistics hold one wall-clock time per call):
 * d_times [P][2] receives the GPU global timer in nanoseconds when a CTA takes
 * pair i and when its result is written. NULL switches it off. */
gcr_status gcr_context_set_pair_times(gcr_context* ctx, unsigned long long* d_times);

/* Step limit of the labelling's maximum-flow solvers for the batches prepared
 * on `ctx` from now on (no counterpart in the reference, whose Boykov-Kolmogorov
 * solver, maxflow.cpp:471-607, runs unbounded): a flow problem that needs more
 * than `steps` push / relabel steps stops, keeps the labels found so far and
 * the pair reports GCR_TIMEOUT; the kernel returns normally. 0 restores the
 * defaults (20,000,000 steps per grid cell, 2^24 on the radius graph). A
 * failure-detection hook: tests set a tiny limit to check that a runaway flow
 * ends with a status instead of a hung kernel. */
gcr_status gcr_context_set_flow_step_limit(gcr_context* ctx, int64_t steps);

/* Launch shape of the engine (no counterpart in the reference, which runs one
 * pair per call on one thread). None of these changes a result: sampler calls
 * are counter-based and replayed in call order, and each pair runs on one CTA
 * whatever its place in the launch.
 *   batch_calls  sampler calls (hypotheses) drawn, solved and scored together
 *                per CTA, 1..256 (0: 256)
 *   ctas_per_sm  resident engine CTAs per SM, at most what fits (0: that many)
 *   order        0: pairs in the caller's order; 1: largest pairs first
 * gcr_context_set_tuning installs a table for the batches prepared on ctx from
 * now on: gcr_batch_prepare / gcr_batch_run_device use the entry of the
 * batch's model kind with the smallest max_n at or above the batch's largest
 * pair (no entry: the defaults). The table is what pygcransac.autotune writes:
 * the fastest shape per kind and size bucket on a calibration batch, cached
 * per GPU name. gcr_context_last_tuning reports the entry the last prepared
 * batch used (max_n: the entry's bound, or the batch's largest pair). */
typedef struct gcr_tuning {
  int32_t kind;         /* gcr_model_kind */
  int32_t max_n;        /* applies to batches whose largest pair has at most max_n correspondences */
  int32_t batch_calls;
  int32_t ctas_per_sm;
  int32_t order;
  int32_t reserved;     /* 0 */
} gcr_tuning;

gcr_status gcr_context_set_tuning(gcr_context* ctx, const gcr_tuning* entries, int32_t count);
gcr_status gcr_context_last_tuning(const gcr_context* ctx, gcr_tuning* out);

/* Arithmetic of the local optimisation's fundamental-matrix fits for the
 * batches prepared on `ctx` from now on (no counterpart in the reference, which
 * computes in double throughout):
 *   GCR_LO_FP64  (default) the reference's arithmetic: masks and counts equal
 *                the FP64 oracle's
 *   GCR_LO_FP32  every fundamental-matrix fit after the minimal solver (the
 *                graph-cut local optimisation's trials, the iteratively
 *                reweighted fits, the final refit and the drivers' bundle
 *                adjustment) runs 8-point and Levenberg-Marquardt in FP32 from
 *                the FP32 tile, CTA-wide sums reduced in FP64; the bundle
 *                adjustment on raw pixel coordinates works on the pair's
 *                centred coordinates scaled into [-1, 1] with its loss
 *                truncation scaled alike. Every fit is still scored with exact
 *                inlier decisions. Models agree with the FP64 fits to model
 *                tolerance, masks can differ in borderline points. For
 *                throughput forms (the learned proposal), not for parity runs. */
enum { GCR_LO_FP64 = 0, GCR_LO_FP32 = 1 };
gcr_status gcr_context_set_lo_precision(gcr_context* ctx, int32_t precision);

/* Sample tape: recorded main-sampler samples that replace the sampler's draws,
 * so a run can replay the sample indices of another implementation — e.g. the
 * reference's own run, recorded through the Sampler* argument of
 * GCRANSAC::run (src/pygcransac/include/GCRANSAC.h:69-76, samplers/sampler.h:44-87).
 * Layout: [num_pairs][calls_per_pair][m] int32 point indices (m = 4 H, 7 F,
 * 5 E). Sampler call c of pair i (the c-th minimal sample the run asks for,
 * counting unsuccessful ones, from 0) reads row c of block i; a call past
 * calls_per_pair, or a row holding an index outside [0, n) (write -1 for a
 * call on which the recording sampler failed), is an unsuccessful sampler
 * call. Only the main sampler is replaced: the local optimisation's sampler
 * and DEGENSAC's inner run draw as before.
 *   gcr_context_set_sample_tape  device tape for the batches prepared on ctx
 *                                from now on (NULL or 0 calls: draw again)
 *   gcr_set_sample_tape          host tape read by this thread's host-buffer
 *                                entries (gcr_find_*, gcr_find_batch, gcr_run,
 *                                gcr_run_with_probabilities) from now on; the
 *                                single-pair entries read block 0 */
gcr_status gcr_context_set_sample_tape(gcr_context* ctx, const int32_t* d_tape, int64_t calls_per_pair);
gcr_status gcr_set_sample_tape(const int32_t* h_tape, int64_t calls_per_pair);

/* GCRANSAC::run on one pair (GCRANSAC.h:200-627) without the Python drivers'
 * pre- and post-processing; the entry behind the C++ plugin surface
 * include/gcransac/GCRANSAC.h. `points` [n][4] are the coordinates the model
 * is fitted in (K^-1-normalised for essential matrices, as the reference's
 * essential driver passes them to run), `pixels` [n][4] (NULL = points) the
 * coordinates of the grid neighbourhood and of the P-NAPSAC sampler;
 * `cell_sizes` [4] and `divisions` describe the grid (GridNeighborhoodGraph<4>,
 * neighborhood/grid_neighborhood_graph.h:163); `size` gives the image extents
 * P-NAPSAC uses; params->threshold is in the units of `points`. Host buffers;
 * the inlier mask and statistics are those of the run, with no bundle
 * adjustment epilogue (gcransac_python.cpp:1833-1889, 2770-2828). */
gcr_status gcr_run(gcr_model_kind kind, const double* points, const double* pixels, int64_t n,
                   const double* cell_sizes, int32_t divisions, const gcr_image_size* size,
                   const gcr_params* params, double* model_out9, uint8_t* mask_out, gcr_stats* stats_out);

/* gcr_run with a main sampler that reads per-correspondence probabilities:
 * the ImportanceSampler (samplers/importance_sampler.h:67-80, sampler 3) and
 * the AdaptiveReorderingSampler (samplers/adaptive_reordering_sampler.h:59-97,
 * sampler 4), which the reference constructs from a probability vector and
 * passes to GCRANSAC::run (GCRANSAC.h:200-627). `probabilities` [n] (host,
 * finite, non-negative; the AR sampler divides them by their maximum as the
 * reference's drivers do, gcransac_python.cpp:1730-1741). gcr_run rejects
 * samplers 3 and 4. */
gcr_status gcr_run_with_probabilities(gcr_model_kind kind, const double* points, const double* pixels, int64_t n,
                                      const double* cell_sizes, int32_t divisions, const gcr_image_size* size,
                                      const double* probabilities, const gcr_params* params, double* model_out9,
                                      uint8_t* mask_out, gcr_stats* stats_out);

/* Learned inlier-probability proposal (no counterpart in the reference, which
 * takes externally computed probabilities for its samplers 3 and 4): a
 * per-correspondence MLP whose scores order the correspondences for PROSAC
 * (sampler 1). All buffers are device pointers; work is queued on `stream`.
 * Pairs are laid out as in gcr_batch_run_device (d_offsets [num_pairs + 1],
 * max_n = the largest pair size, num_pairs <= 65535).
 *   gcr_learned_features    k = 8 nearest-neighbour displacement features,
 *                           d_feat [total][gcr_learned_feature_width()] floats
 *   gcr_learned_forward     logits [n]; the hidden activations d_a1..d_a3
 *                           ([n][128] floats) are written when not NULL
 *   gcr_learned_backward    adds the gradient of the weighted binary
 *                           cross-entropy (labels, weights [n]; the loss is
 *                           divided by the weight sum) to d_grad
 *   gcr_learned_adam        one Adam step (step counts from 1) on the FP32
 *                           master parameters, refreshing the BF16 copies
 *   gcr_learned_order       per pair, copies the correspondences in
 *                           descending logit order (ties by index) to
 *                           d_sorted_corr and records each sorted row's
 *                           original in-pair index in d_perm [total];
 *                           correspondence buffers 32-byte aligned
 *   gcr_learned_propose     features + forward + order in one call (d_feat,
 *                           d_logits: workspaces of total rows)
 *   gcr_learned_unpermute_mask
 *                           maps an inlier mask of the sorted order back to
 *                           the caller's order (d_pair_of_row [total])
 * Parameters: gcr_learned_param_count() floats (master, Adam moments,
 * gradient) or BF16 values (the copy the passes read). */
int64_t gcr_learned_param_count(void);
int32_t gcr_learned_feature_width(void);
gcr_status gcr_learned_features(const double* d_corr, const int64_t* d_offsets, const gcr_image_size* d_sizes,
                                int64_t num_pairs, int64_t max_n, float* d_feat, void* stream);
gcr_status gcr_learned_params_to_bf16(const float* d_master, void* d_bf16, void* stream);
gcr_status gcr_learned_forward(const float* d_feat, int64_t n, const void* d_bf16, float* d_a1, float* d_a2,
                               float* d_a3, float* d_logits, void* stream);
gcr_status gcr_learned_backward(const float* d_feat, int64_t n, const void* d_bf16, const float* d_a1,
                                const float* d_a2, const float* d_a3, const float* d_logits,
                                const float* d_labels, const float* d_weights, float inv_weight_sum,
                                float* d_grad, void* stream);
gcr_status gcr_learned_adam(float* d_m, float* d_v, float* d_master, void* d_bf16, const float* d_grad,
                            float lr, int64_t step, void* stream);
gcr_status gcr_learned_order(const double* d_corr, const int64_t* d_offsets, int64_t num_pairs, int64_t max_n,
                             const float* d_logits, double* d_sorted_corr, int32_t* d_perm, void* stream);
gcr_status gcr_learned_propose(const double* d_corr, const int64_t* d_offsets, const gcr_image_size* d_sizes,
                               int64_t num_pairs, int64_t max_n, int64_t total, const void* d_bf16,
                               float* d_feat, float* d_logits, double* d_sorted_corr, int32_t* d_perm,
                               void* stream);
gcr_status gcr_learned_unpermute_mask(const uint8_t* d_sorted_mask, const int32_t* d_perm,
                                      const int64_t* d_offsets, const int32_t* d_pair_of_row, int64_t total,
                                      uint8_t* d_mask, void* stream);

/* Number of kernels the last gcr_batch_run_device / gcr_batch_launch / gcr_find_* call launched. */
int64_t gcr_last_launch_count(void);

/* Message of the last failing call on this host thread. */
const char* gcr_last_error_string(void);

#ifdef __cplusplus
}
#endif

#endif /* GCR_H_ */
