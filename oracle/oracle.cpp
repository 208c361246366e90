// Oracle (test infrastructure only): C entry points of the CPU FP64
// restatement of the reference's findHomography_ / findFundamentalMatrix_ /
// findEssentialMatrix_ drivers (src/pygcransac/src/gcransac_python.cpp:4221,
// 1600, 2519). The parameter and result structs are the engine's own public
// POD types (include/gcr.h) so that tests can hand both the same inputs.
#include <atomic>
#include <chrono>
#include <thread>

#include "../include/gcr.h"
#include "oracle_essential.hpp"
#include "oracle_fundamental.hpp"
#include "oracle_gcransac.hpp"
#include "oracle_homography.hpp"

namespace oracle {

const MagsacTable& magsac_table() {
  static MagsacTable t;
  return t;
}

// Upper incomplete gamma Gamma(1.5, x) = sqrt(pi) erfc(sqrt x) + 2 sqrt(x) e^-x.
MagsacTable::MagsacTable() {
  g.resize(36001);
  for (int i = 0; i <= 36000; ++i) {
    const double x = i / 1000.0;
    g[i] = std::sqrt(M_PI) * 0.5 * std::erfc(std::sqrt(x)) + std::sqrt(x) * std::exp(-x);
  }
}

struct Common {
  const gcr_params* p;
  const gcr_image_size* sz;
  uint64_t seed;
};

static void fill_settings(Settings& s, const gcr_params& p) {
  s.threshold = p.threshold;
  s.spatial_coherence_weight = p.spatial_coherence_weight;
  s.confidence = p.confidence;
  s.max_local_optimization_number = (size_t)p.lo_number;
  s.max_iteration_number = (size_t)p.max_iterations;
  s.min_iteration_number = (size_t)p.min_iterations;
  s.use_sprt = p.use_sprt != 0;
  s.use_space_partitioning = p.use_space_partitioning != 0;
  s.sprt_min_inlier_ratio = p.min_inlier_ratio_for_sprt;
}

// point probabilities of the importance sampler for the current driver call
static thread_local const double* g_probs = nullptr;
// sample tape of the driver calls from now on ([pairs][calls][m], see
// oracle_set_sample_tape) and the current pair's rows
static const int32_t* g_tape = nullptr;
static int64_t g_tape_calls = 0;
static thread_local const int32_t* t_tape = nullptr;

static std::unique_ptr<Sampler> make_main_sampler(const gcr_params& p, const Mat& pts, size_t m,
                                                  const gcr_image_size& sz, uint64_t seed) {
  if (t_tape) return std::make_unique<TapeSampler>(t_tape, g_tape_calls, (size_t)pts.rows);
  switch (p.sampler) {
    case GCR_SAMPLER_IMPORTANCE:
      if (!g_probs) return nullptr;
      return std::make_unique<ImportanceSampler>(seed, STREAM_MAIN, g_probs, (size_t)pts.rows);
    case GCR_SAMPLER_AR:
      if (!g_probs) return nullptr;
      return std::make_unique<ARSampler>(seed, STREAM_AR, g_probs, (size_t)pts.rows, p.sampler_variance);
    case GCR_SAMPLER_UNIFORM: return std::make_unique<UniformSampler>(seed, STREAM_MAIN);
    case GCR_SAMPLER_PROSAC: return std::make_unique<ProsacSampler>(seed, STREAM_MAIN, m, (size_t)pts.rows);
    case GCR_SAMPLER_PNAPSAC: {
      const double sizes[4] = {(double)sz.w1, (double)sz.h1, (double)sz.w2, (double)sz.h2};
      return std::make_unique<ProgressiveNapsacSampler>(seed, pts, std::vector<size_t>{16, 8, 4, 2}, m, sizes, 0.5);
    }
    default: return nullptr;
  }
}

// The grid of the drivers: (w + eps) / n cells along every axis
// (gcransac_python.cpp:4290-4297).
static std::unique_ptr<Grid> make_grid(const Mat& pixel_pts, const gcr_image_size& sz, double ns) {
  const size_t n = (size_t)ns;
  const double e = std::numeric_limits<double>::epsilon();
  const double cs[4] = {(sz.w1 + e) / (double)n, (sz.h1 + e) / (double)n, (sz.w2 + e) / (double)n,
                        (sz.h2 + e) / (double)n};
  return std::make_unique<Grid>(pixel_pts, cs, n);
}

template <class Est, template <class> class Scoring>
static int run_generic(const Mat& run_pts, const Mat& pixel_pts, const Est& est, const gcr_params& p,
                       const gcr_image_size& sz, uint64_t seed, const Grid* grid, double threshold,
                       Model& model, std::vector<size_t>& inliers, gcr_stats* st, double mag_threshold,
                       size_t max_graph_cuts = 10, bool final_irls = true) {
  auto main_s = make_main_sampler(p, pixel_pts, Est::sample_size(), sz, seed);
  if (!main_s) return GCR_UNSUPPORTED;
  UniformSampler lo_s(seed, STREAM_LO);
  GCRansac<Est, Scoring<Est>> g;
  fill_settings(g.settings, p);
  g.sprt_seed = seed;
  g.settings.threshold = threshold;
  g.settings.max_graph_cut_number = max_graph_cuts;
  g.settings.do_final_iterated_least_squares = final_irls;
  if constexpr (std::is_same<Scoring<Est>, MAGSACScoring<Est>>::value) g.scoring.threshold = mag_threshold;
  const bool ok = g.run(run_pts, est, main_s.get(), &lo_s, grid, model);
  if (st) {
    st->iteration_number = (int64_t)g.statistics.iteration_number;
    st->graph_cut_number = (int64_t)g.statistics.graph_cut_number;
    st->local_optimization_number = (int64_t)g.statistics.local_optimization_number;
    st->score = g.statistics.score;
    st->flags = (g.statistics.local_optimization_number ? GCR_FLAG_LO_APPLIED : 0) |
                (g.statistics.irls_applied ? GCR_FLAG_IRLS_APPLIED : 0);
    st->models_scored = (int64_t)g.models_scored;
  }
  if (!ok) return GCR_NO_MODEL;
  inliers = g.statistics.inliers;
  return GCR_OK;
}

// findHomography_ (gcransac_python.cpp:4221-4552). Its SPRT is constructed
// without the driver's min_inlier_ratio_for_sprt (4394-4396), so the test
// starts from the constructor's default inlier ratio 0.01
// (preemption_sprt.h:141-143) whatever the argument holds.
static int find_homography(const double* corr, int64_t n, const gcr_image_size& sz, const gcr_params& p_in,
                           uint64_t seed, double* model_out, uint8_t* mask, gcr_stats* st) {
  if (n < 4) return GCR_TOO_FEW_POINTS;
  gcr_params p = p_in;
  p.min_inlier_ratio_for_sprt = 0.01;
  const Mat pts{corr, n, 4};
  // the homography driver keeps the grid under space partitioning
  // (gcransac_python.cpp:4282-4286)
  auto grid = p.neighborhood == GCR_NEIGHBORHOOD_FLANN && !p.use_space_partitioning
                  ? std::make_unique<Grid>(Grid::radius_graph(pts, p.neighborhood_size))
                  : make_grid(pts, sz, p.neighborhood_size);
  HomographyEstimator est;
  Model model{};
  std::vector<size_t> inl;
  int rc;
  if (p.scoring == GCR_SCORING_MAGSAC)
    rc = run_generic<HomographyEstimator, MAGSACScoring>(pts, pts, est, p, sz, seed, grid.get(), p.threshold,
                                                         model, inl, st, p.threshold);
  else
    rc = run_generic<HomographyEstimator, MSACScoring>(pts, pts, est, p, sz, seed, grid.get(), p.threshold,
                                                       model, inl, st, p.threshold);
  std::memset(mask, 0, (size_t)n);
  for (size_t i : inl) mask[i] = 1;
  if (st) st->inlier_number = (int64_t)inl.size();
  if (rc == GCR_OK) std::memcpy(model_out, model.data(), 9 * sizeof(double));
  else std::memset(model_out, 0, 9 * sizeof(double));
  return rc;
}

// findHomographyAC_ and findHomographySIFT_ (gcransac_python.cpp:4553-4811,
// 4813-5069): rows of eight values (points, then the local affine maps or the
// features' scales and orientations). The neighbourhood is built on the point
// columns only when the spatial weight is above machine epsilon, with cells
// w / n (no padding), or as the radius graph; samplers 0, 1, 3 and 4 (the
// drivers refuse P-NAPSAC); MSAC; SPRT from the default inlier ratio 0.01
// (4719-4721, 4979-4981); no space partitioning and no epilogue.
template <class Est>
static int find_homography_rows8(const double* corr, int64_t n, const gcr_image_size& sz, const gcr_params& p_in,
                                 uint64_t seed, double* model_out, uint8_t* mask, gcr_stats* st) {
  if (n < 2) return GCR_TOO_FEW_POINTS;
  if (p_in.sampler == GCR_SAMPLER_PNAPSAC || p_in.scoring != GCR_SCORING_MSAC) return GCR_UNSUPPORTED;
  gcr_params p = p_in;
  p.min_inlier_ratio_for_sprt = 0.01;
  p.use_space_partitioning = 0;
  const Mat pts{corr, n, 8};
  std::unique_ptr<Grid> grid;
  if (p.spatial_coherence_weight > std::numeric_limits<double>::epsilon()) {
    if (p.neighborhood == GCR_NEIGHBORHOOD_FLANN) {
      grid = std::make_unique<Grid>(Grid::radius_graph(pts, p.neighborhood_size));
    } else {
      const size_t nd = (size_t)p.neighborhood_size;
      const double cs[4] = {sz.w1 / (double)nd, sz.h1 / (double)nd, sz.w2 / (double)nd, sz.h2 / (double)nd};
      grid = std::make_unique<Grid>(pts, cs, nd);
    }
  }
  Est est;
  Model model{};
  std::vector<size_t> inl;
  const int rc = run_generic<Est, MSACScoring>(pts, pts, est, p, sz, seed, grid.get(), p.threshold, model, inl, st,
                                               p.threshold);
  std::memset(mask, 0, (size_t)n);
  for (size_t i : inl) mask[i] = 1;
  if (st) st->inlier_number = (int64_t)inl.size();
  if (rc == GCR_OK) std::memcpy(model_out, model.data(), 9 * sizeof(double));
  else std::memset(model_out, 0, 9 * sizeof(double));
  return rc;
}

// findFundamentalMatrix_ (gcransac_python.cpp:1600-1923): grid only when the
// spatial weight is positive (cells w / n, 1658-1677), the default estimator
// (0.5 validity ratio, DEGENSAC), GC-RANSAC, then a weighted bundle adjustment
// of the final inliers kept when it raises the MSAC score (1833-1887); with at
// most 7 inliers the model is the identity (1889).
static int find_fundamental(const double* corr, int64_t n, const gcr_image_size& sz, const gcr_params& p,
                            uint64_t seed, double* model_out, uint8_t* mask, gcr_stats* st) {
  if (n < 7) return GCR_TOO_FEW_POINTS;
  const Mat pts{corr, n, 4};
  std::unique_ptr<Grid> grid;
  if (p.spatial_coherence_weight > std::numeric_limits<double>::epsilon()) {
    if (p.neighborhood == GCR_NEIGHBORHOOD_FLANN) {
      grid = std::make_unique<Grid>(Grid::radius_graph(pts, p.neighborhood_size));
    } else {
      const size_t nd = (size_t)p.neighborhood_size;
      const double cs[4] = {sz.w1 / (double)nd, sz.h1 / (double)nd, sz.w2 / (double)nd, sz.h2 / (double)nd};
      grid = std::make_unique<Grid>(pts, cs, nd);
    }
  }
  FundamentalEstimator est;
  est.seed = seed;
  Model model{};
  std::vector<size_t> inl;
  int rc;
  if (p.scoring == GCR_SCORING_MAGSAC)
    rc = run_generic<FundamentalEstimator, MAGSACScoring>(pts, pts, est, p, sz, seed, grid.get(), p.threshold,
                                                          model, inl, st, p.threshold);
  else
    rc = run_generic<FundamentalEstimator, MSACScoring>(pts, pts, est, p, sz, seed, grid.get(), p.threshold, model,
                                                        inl, st, p.threshold);
  if (est.degensac_ran && st) st->flags |= 8;
  if (rc == GCR_OK) {
    if (inl.size() > 7) {
      const double tt = 1.5 * p.threshold, sq = tt * tt;
      std::vector<double> w(inl.size());
      for (size_t k = 0; k < inl.size(); ++k)
        w[k] = std::max(0.0, 1.0 - f_sampson2(pts.row(inl[k]), model) / sq);
      // FundamentalMatrixBundleAdjustmentSolver on the raw inliers: 8-point
      // start then LM; the weights are taken by inlier position for both steps
      std::vector<const double*> rows(inl.size());
      for (size_t k = 0; k < inl.size(); ++k) rows[k] = pts.row(inl[k]);
      std::vector<Model> models;
      f_eight_point(rows.data(), (int)rows.size(), w.data(), models);
      for (Model& F : models) f_refine_lm(rows.data(), (int)rows.size(), w.data(), F);
      MSACScoring<FundamentalEstimator> sc;
      sc.initialize(sq, n);
      double best = st ? st->score : 0.0;
      for (Model& F : models) {
        std::vector<size_t> cur;
        const Score s = sc.get(pts, F, est, &cur);
        if (best < s.value) {
          model = F;
          best = s.value;
          inl.swap(cur);
        }
      }
      if (st) st->score = best;
    } else {
      model = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    }
  }
  std::memset(mask, 0, (size_t)n);
  for (size_t i : inl) mask[i] = 1;
  if (st) st->inlier_number = (int64_t)inl.size();
  if (rc == GCR_OK) std::memcpy(model_out, model.data(), 9 * sizeof(double));
  else std::memset(model_out, 0, 9 * sizeof(double));
  return rc;
}

// findFundamentalMatrixAC_ and findFundamentalMatrixSIFT_
// (gcransac_python.cpp:1924-2221, 2222-2518; the two drivers differ only in
// the estimator): rows of eight values; the neighbourhood on the point columns only when the spatial weight
// is above machine epsilon (cells w / n, or the radius graph); samplers 0, 1,
// 3 and 4 (the driver refuses P-NAPSAC); MSAC; SPRT from the driver's
// min_inlier_ratio_for_sprt; then the bundle adjustment of the final inliers
// without weights (2157-2163), kept when it raises the MSAC score; with at
// most 7 inliers the model is the identity.
template <class Est>
static int find_fundamental_rows8(const double* corr, int64_t n, const gcr_image_size& sz, const gcr_params& p,
                                  uint64_t seed, double* model_out, uint8_t* mask, gcr_stats* st) {
  if (n < 3) return GCR_TOO_FEW_POINTS;
  if (p.sampler == GCR_SAMPLER_PNAPSAC || p.scoring != GCR_SCORING_MSAC) return GCR_UNSUPPORTED;
  const Mat pts{corr, n, 8};
  std::unique_ptr<Grid> grid;
  if (p.spatial_coherence_weight > std::numeric_limits<double>::epsilon()) {
    if (p.neighborhood == GCR_NEIGHBORHOOD_FLANN) {
      grid = std::make_unique<Grid>(Grid::radius_graph(pts, p.neighborhood_size));
    } else {
      const size_t nd = (size_t)p.neighborhood_size;
      const double cs[4] = {sz.w1 / (double)nd, sz.h1 / (double)nd, sz.w2 / (double)nd, sz.h2 / (double)nd};
      grid = std::make_unique<Grid>(pts, cs, nd);
    }
  }
  Est est;
  est.seed = seed;
  Model model{};
  std::vector<size_t> inl;
  const int rc = run_generic<Est, MSACScoring>(pts, pts, est, p, sz, seed, grid.get(), p.threshold, model, inl, st,
                                               p.threshold);
  if (rc == GCR_OK) {
    if (inl.size() > 7) {
      const double tt = 1.5 * p.threshold, sq = tt * tt;
      std::vector<const double*> rows(inl.size());
      for (size_t k = 0; k < inl.size(); ++k) rows[k] = pts.row(inl[k]);
      std::vector<Model> models;
      f_eight_point(rows.data(), (int)rows.size(), nullptr, models);
      for (Model& F : models) f_refine_lm(rows.data(), (int)rows.size(), nullptr, F);
      MSACScoring<Est> sc;
      sc.initialize(sq, n);
      double best = st ? st->score : 0.0;
      for (Model& F : models) {
        std::vector<size_t> cur;
        const Score s = sc.get(pts, F, est, &cur);
        if (best < s.value) {
          model = F;
          best = s.value;
          inl.swap(cur);
        }
      }
      if (st) st->score = best;
    } else {
      model = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    }
  }
  std::memset(mask, 0, (size_t)n);
  for (size_t i : inl) mask[i] = 1;
  if (st) st->inlier_number = (int64_t)inl.size();
  if (rc == GCR_OK) std::memcpy(model_out, model.data(), 9 * sizeof(double));
  else std::memset(model_out, 0, 9 * sizeof(double));
  return rc;
}

// findEssentialMatrix_ (gcransac_python.cpp:2519-2856): correspondences
// normalised by the inverse intrinsics (utils.h:65-103), threshold divided by
// the mean focal length (2601-2603), grid and P-NAPSAC on the pixel
// coordinates (cells w / n), GC-RANSAC on the normalised ones, then the
// weighted essential-matrix bundle adjustment of the final inliers kept when
// it raises the MSAC score (2770-2826); with at most 5 inliers the model is
// the identity (2828). The bundle adjustment's Stewenius start reads the
// weights by point index (the reference indexes an inlier-sized array by
// point index there); the weights are placed at the inliers' point indices,
// so both steps see the weight of each inlier.
//
// findPlanarEssentialMatrix_ (gcransac_python.cpp:3531-3870) is the same
// driver with the planar estimator: MSAC only, the AR sampler's variance
// fixed at 0.1 (3675), and with SPRT up to 100 graph cuts and no final
// iteratively reweighted fit (3741-3742).
template <class Est>
static int find_essential_kind(const double* corr, int64_t n, const double* K1, const double* K2,
                               const gcr_image_size& sz, const gcr_params& p_in, uint64_t seed, double* model_out,
                               uint8_t* mask, gcr_stats* st) {
  constexpr bool planar = std::is_same<Est, EssentialPlanarEstimator>::value;
  if (n < (int64_t)Est::sample_size()) return GCR_TOO_FEW_POINTS;
  if (!K1 || !K2) return GCR_INVALID_ARG;
  gcr_params p = p_in;
  if (planar) {
    if (p.scoring != GCR_SCORING_MSAC) return GCR_UNSUPPORTED;
    p.sampler_variance = 0.1;
  }
  const size_t gc_max = planar && p.use_sprt ? 100 : 10;
  const bool final_irls = !(planar && p.use_sprt);
  const Mat pix{corr, n, 4};
  double Ki1[9], Ki2[9];
  inverse3(K1, Ki1);
  inverse3(K2, Ki2);
  std::vector<double> nrm((size_t)n * 4);
  for (int64_t i = 0; i < n; ++i) {
    const double* q = corr + 4 * i;
    nrm[4 * i] = Ki1[0] * q[0] + Ki1[1] * q[1] + Ki1[2];
    nrm[4 * i + 1] = Ki1[3] * q[0] + Ki1[4] * q[1] + Ki1[5];
    nrm[4 * i + 2] = Ki2[0] * q[2] + Ki2[1] * q[3] + Ki2[2];
    nrm[4 * i + 3] = Ki2[3] * q[2] + Ki2[4] * q[3] + Ki2[5];
  }
  const Mat pts{nrm.data(), n, 4};
  const double normalizer = 0.25 * (K1[0] + K1[4] + K2[0] + K2[4]);
  const double thr = p.threshold / normalizer;
  std::unique_ptr<Grid> grid;
  if (p.spatial_coherence_weight > std::numeric_limits<double>::epsilon()) {
    if (p.neighborhood == GCR_NEIGHBORHOOD_FLANN) {
      grid = std::make_unique<Grid>(Grid::radius_graph(pix, p.neighborhood_size));
    } else {
      const size_t nd = (size_t)p.neighborhood_size;
      const double cs[4] = {sz.w1 / (double)nd, sz.h1 / (double)nd, sz.w2 / (double)nd, sz.h2 / (double)nd};
      grid = std::make_unique<Grid>(pix, cs, nd);
    }
  }
  Est est;
  Model model{};
  std::vector<size_t> inl;
  int rc;
  if (p.scoring == GCR_SCORING_MAGSAC)
    rc = run_generic<Est, MAGSACScoring>(pts, pix, est, p, sz, seed, grid.get(), thr, model, inl, st, thr, gc_max,
                                         final_irls);
  else
    rc = run_generic<Est, MSACScoring>(pts, pix, est, p, sz, seed, grid.get(), thr, model, inl, st, thr, gc_max,
                                       final_irls);
  if (rc == GCR_OK) {
    if (inl.size() > 5) {
      const double tt = 1.5 * thr, sq = tt * tt;
      std::vector<double> w_pos(inl.size()), w_pt((size_t)n, 0.0);
      for (size_t k = 0; k < inl.size(); ++k) {
        w_pos[k] = std::max(0.0, 1.0 - e_sampson2(pts.row(inl[k]), model) / sq);
        w_pt[inl[k]] = w_pos[k];
      }
      std::vector<Model> models;
      e_bundle_adjust(pts, inl.data(), inl.size(), w_pt.data(), w_pos.data(), models);
      MSACScoring<Est> sc;
      sc.initialize(sq, n);
      double best = st ? st->score : 0.0;
      for (Model& E : models) {
        std::vector<size_t> cur;
        const Score s = sc.get(pts, E, est, &cur);
        if (best < s.value) {
          model = E;
          best = s.value;
          inl.swap(cur);
        }
      }
      if (st) st->score = best;
    } else {
      model = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    }
  }
  std::memset(mask, 0, (size_t)n);
  for (size_t i : inl) mask[i] = 1;
  if (st) st->inlier_number = (int64_t)inl.size();
  if (rc == GCR_OK) std::memcpy(model_out, model.data(), 9 * sizeof(double));
  else std::memset(model_out, 0, 9 * sizeof(double));
  return rc;
}

// Values per correspondence row and minimal sample size of a model kind.
static int kind_columns(int kind) {
  return kind == GCR_HOMOGRAPHY_AFFINE || kind == GCR_FUNDAMENTAL_AFFINE || kind == GCR_FUNDAMENTAL_SIFT ||
                 kind == GCR_HOMOGRAPHY_SIFT
             ? 8
             : 4;
}
static int kind_sample_size(int kind) {
  switch (kind) {
    case GCR_HOMOGRAPHY: return 4;
    case GCR_FUNDAMENTAL: return 7;
    case GCR_ESSENTIAL: return 5;
    case GCR_HOMOGRAPHY_AFFINE: return 2;
    case GCR_FUNDAMENTAL_AFFINE: return 3;
    case GCR_FUNDAMENTAL_SIFT: return 4;
    case GCR_HOMOGRAPHY_SIFT: return 2;
    case GCR_ESSENTIAL_PLANAR: return 2;
    default: return 0;
  }
}

// One driver call; `tape` (or NULL) holds this pair's rows of the sample tape.
static int find_pair(int kind, const double* corr, int64_t n, const double* K1, const double* K2,
                     const gcr_image_size* sz, const gcr_params* p, uint64_t seed, double* model_out,
                     uint8_t* mask_out, gcr_stats* st, const int32_t* tape) {
  gcr_stats local{};
  gcr_stats* s = st ? st : &local;
  std::memset(s, 0, sizeof(*s));
  t_tape = tape;
  int rc;
  switch (kind) {
    case GCR_HOMOGRAPHY: rc = find_homography(corr, n, *sz, *p, seed, model_out, mask_out, s); break;
    case GCR_FUNDAMENTAL: rc = find_fundamental(corr, n, *sz, *p, seed, model_out, mask_out, s); break;
    case GCR_ESSENTIAL:
      rc = find_essential_kind<EssentialEstimator>(corr, n, K1, K2, *sz, *p, seed, model_out, mask_out, s);
      break;
    case GCR_ESSENTIAL_PLANAR:
      rc = find_essential_kind<EssentialPlanarEstimator>(corr, n, K1, K2, *sz, *p, seed, model_out, mask_out, s);
      break;
    case GCR_HOMOGRAPHY_AFFINE:
      rc = find_homography_rows8<HomographyAffineEstimator>(corr, n, *sz, *p, seed, model_out, mask_out, s);
      break;
    case GCR_HOMOGRAPHY_SIFT:
      rc = find_homography_rows8<HomographySiftEstimator>(corr, n, *sz, *p, seed, model_out, mask_out, s);
      break;
    case GCR_FUNDAMENTAL_AFFINE:
      rc = find_fundamental_rows8<FundamentalAffineEstimator>(corr, n, *sz, *p, seed, model_out, mask_out, s);
      break;
    case GCR_FUNDAMENTAL_SIFT:
      rc = find_fundamental_rows8<FundamentalSiftEstimator>(corr, n, *sz, *p, seed, model_out, mask_out, s);
      break;
    default: rc = GCR_INVALID_ARG;
  }
  t_tape = nullptr;
  s->status = rc;
  return rc;
}

}  // namespace oracle

using namespace oracle;

extern "C" {

int oracle_find(int kind, const double* corr, int64_t n, const double* K1, const double* K2,
                const gcr_image_size* sz, const gcr_params* p, uint64_t seed, double* model_out,
                uint8_t* mask_out, gcr_stats* st);

// oracle_find with the importance sampler's point probabilities
int oracle_find_prob(int kind, const double* corr, int64_t n, const double* K1, const double* K2,
                     const double* probabilities, const gcr_image_size* sz, const gcr_params* p, uint64_t seed,
                     double* model_out, uint8_t* mask_out, gcr_stats* st) {
  g_probs = probabilities;
  const int rc = oracle_find(kind, corr, n, K1, K2, sz, p, seed, model_out, mask_out, st);
  g_probs = nullptr;
  return rc;
}

int oracle_find(int kind, const double* corr, int64_t n, const double* K1, const double* K2,
                const gcr_image_size* sz, const gcr_params* p, uint64_t seed, double* model_out,
                uint8_t* mask_out, gcr_stats* st) {
  return find_pair(kind, corr, n, K1, K2, sz, p, seed, model_out, mask_out, st, g_tape);
}

// GCRANSAC::run alone (GCRANSAC.h:200-627) on caller-given fitting
// coordinates `points`, neighbourhood coordinates `pixels` and grid cells:
// the counterpart of gcr_run; no driver epilogue, threshold in the units of
// `points`.
int oracle_run(int kind, const double* points, const double* pixels, int64_t n, const double* cell_sizes,
               int32_t divisions, const gcr_image_size* sz, const gcr_params* p, uint64_t seed, double* model_out,
               uint8_t* mask, gcr_stats* st) {
  gcr_stats local{};
  gcr_stats* s = st ? st : &local;
  std::memset(s, 0, sizeof(*s));
  t_tape = g_tape;
  const Mat pts{points, n, 4};
  const Mat pix{pixels ? pixels : points, n, 4};
  const Grid grid = p->neighborhood == GCR_NEIGHBORHOOD_FLANN ? Grid::radius_graph(pix, p->neighborhood_size)
                                                              : Grid(pix, cell_sizes, (size_t)divisions);
  Model model{};
  std::vector<size_t> inl;
  int rc = GCR_INVALID_ARG;
  const bool mag = p->scoring == GCR_SCORING_MAGSAC;
  const double t = p->threshold;
  if (kind == GCR_HOMOGRAPHY) {
    if (n < 4) rc = GCR_TOO_FEW_POINTS;
    else {
      HomographyEstimator est;
      rc = mag ? run_generic<HomographyEstimator, MAGSACScoring>(pts, pix, est, *p, *sz, seed, &grid, t, model, inl, s, t)
               : run_generic<HomographyEstimator, MSACScoring>(pts, pix, est, *p, *sz, seed, &grid, t, model, inl, s, t);
    }
  } else if (kind == GCR_FUNDAMENTAL) {
    if (n < 7) rc = GCR_TOO_FEW_POINTS;
    else {
      FundamentalEstimator est;
      est.seed = seed;
      rc = mag ? run_generic<FundamentalEstimator, MAGSACScoring>(pts, pix, est, *p, *sz, seed, &grid, t, model, inl, s, t)
               : run_generic<FundamentalEstimator, MSACScoring>(pts, pix, est, *p, *sz, seed, &grid, t, model, inl, s, t);
      if (est.degensac_ran) s->flags |= 8;
    }
  } else if (kind == GCR_ESSENTIAL) {
    if (n < 5) rc = GCR_TOO_FEW_POINTS;
    else {
      EssentialEstimator est;
      rc = mag ? run_generic<EssentialEstimator, MAGSACScoring>(pts, pix, est, *p, *sz, seed, &grid, t, model, inl, s, t)
               : run_generic<EssentialEstimator, MSACScoring>(pts, pix, est, *p, *sz, seed, &grid, t, model, inl, s, t);
    }
  }
  t_tape = nullptr;
  std::memset(mask, 0, (size_t)n);
  for (size_t i : inl) mask[i] = 1;
  s->inlier_number = (int64_t)inl.size();
  if (rc == GCR_OK) std::memcpy(model_out, model.data(), 9 * sizeof(double));
  else std::memset(model_out, 0, 9 * sizeof(double));
  s->status = rc;
  return rc;
}

// oracle_run with the importance / AR samplers' point probabilities (the
// probability vector the reference's ImportanceSampler and
// AdaptiveReorderingSampler are constructed from,
// samplers/importance_sampler.h:67-80, adaptive_reordering_sampler.h:59-97)
int oracle_run_prob(int kind, const double* points, const double* pixels, int64_t n, const double* cell_sizes,
                    int32_t divisions, const gcr_image_size* sz, const double* probabilities, const gcr_params* p,
                    uint64_t seed, double* model_out, uint8_t* mask, gcr_stats* st) {
  g_probs = probabilities;
  const int rc = oracle_run(kind, points, pixels, n, cell_sizes, divisions, sz, p, seed, model_out, mask, st);
  g_probs = nullptr;
  return rc;
}

// Neighbour counts of the radius graph (Grid::radius_graph) of n points.
void oracle_radius_counts(const double* corr, int64_t n, double radius, int64_t* counts) {
  const Mat pts{corr, n, 4};
  const Grid g = Grid::radius_graph(pts, radius);
  for (int64_t i = 0; i < n; ++i) counts[i] = (int64_t)g.neighbors((size_t)i).size();
}

// Pair-parallel batch over `threads` host threads (one pair per thread at a
// time, each pair single-threaded like the reference). Returns wall seconds.
// The main sampler of the driver calls from now on reads `tape` ([pairs]
// [calls][m] point indices, m the kind's sample size; -1 marks a failed call)
// instead of drawing: pair i of oracle_find_batch reads block i, oracle_find
// and oracle_run block 0. NULL switches it off.
void oracle_set_sample_tape(const int32_t* tape, int64_t calls) {
  g_tape = calls > 0 ? tape : nullptr;
  g_tape_calls = g_tape ? calls : 0;
}

double oracle_find_batch(int kind, int64_t num_pairs, const double* corr, const int64_t* offsets, const double* K,
                         const gcr_image_size* sizes, const gcr_params* p, const uint64_t* seeds,
                         double* models_out, uint8_t* masks_out, gcr_stats* stats_out, int threads) {
  std::atomic<int64_t> next{0};
  auto worker = [&]() {
    for (;;) {
      const int64_t i = next.fetch_add(1);
      if (i >= num_pairs) return;
      const int64_t o = offsets[i], n = offsets[i + 1] - offsets[i];
      const uint64_t seed = seeds ? seeds[i] : p->seed + (uint64_t)i;
      const int m = kind_sample_size(kind);
      const int32_t* tape = g_tape ? g_tape + (size_t)i * (size_t)g_tape_calls * m : nullptr;
      find_pair(kind, corr + o * kind_columns(kind), n, K ? K + 18 * i : nullptr, K ? K + 18 * i + 9 : nullptr, &sizes[i], p,
                seed, models_out + 9 * i, masks_out + o, stats_out ? stats_out + i : nullptr, tape);
    }
  };
  const auto t0 = std::chrono::steady_clock::now();
  if (threads <= 1) worker();
  else {
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
  }
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Test hooks.
double oracle_magsac_gamma(int i) { return magsac_table().g[i]; }

// Labelling of a given model: writes 1 for SINK (inlier) nodes.
int oracle_labeling(int kind, const double* corr, int64_t n, const gcr_image_size* sz, const gcr_params* p,
                    const double* model, uint8_t* labels) {
  const Mat pts{corr, n, 4};
  auto grid = make_grid(pts, *sz, p->neighborhood_size);
  Model m;
  std::memcpy(m.data(), model, sizeof(m));
  std::vector<size_t> inl;
  if (kind == GCR_HOMOGRAPHY) {
    GCRansac<HomographyEstimator, MSACScoring<HomographyEstimator>> g;
    g.graph = grid.get();
    g.labeling(pts, m, HomographyEstimator(), p->spatial_coherence_weight, p->threshold, inl);
  } else if (kind == GCR_FUNDAMENTAL) {
    GCRansac<FundamentalEstimator, MSACScoring<FundamentalEstimator>> g;
    g.graph = grid.get();
    g.labeling(pts, m, FundamentalEstimator(), p->spatial_coherence_weight, p->threshold, inl);
  } else
    return GCR_UNSUPPORTED;
  std::memset(labels, 0, (size_t)n);
  for (size_t i : inl) labels[i] = 1;
  return 0;
}

// Scores a given model with MSAC: returns the value, writes the inlier count.
double oracle_msac_score(int kind, const double* corr, int64_t n, const double* model, double threshold,
                         int64_t* count) {
  const Mat pts{corr, n, 4};
  Model m;
  std::memcpy(m.data(), model, sizeof(m));
  Score s;
  const double sq = 2.25 * threshold * threshold;
  if (kind == GCR_HOMOGRAPHY) {
    MSACScoring<HomographyEstimator> sc;
    sc.initialize(sq, n);
    s = sc.get(pts, m, HomographyEstimator(), nullptr);
  } else if (kind == GCR_FUNDAMENTAL) {
    MSACScoring<FundamentalEstimator> sc;
    sc.initialize(sq, n);
    s = sc.get(pts, m, FundamentalEstimator(), nullptr);
  } else {
    MSACScoring<EssentialEstimator> sc;
    sc.initialize(sq, n);
    s = sc.get(pts, m, EssentialEstimator(), nullptr);
  }
  *count = (int64_t)s.inlier_number;
  return s.value;
}

// Minimal-sample solve for tests: writes up to 10 models, returns their count (-1 invalid sample);
// rows of 8 for the SIFT and affine kinds, of 4 otherwise.
int oracle_minimal(int kind, const double* corr, int64_t n, const int64_t* sample, double* models_out) {
  const Mat pts{corr, n, 4};
  std::vector<size_t> s;
  std::vector<Model> models;
  if (kind == GCR_HOMOGRAPHY_SIFT) {
    const Mat rows8{corr, n, 8};
    HomographySiftEstimator e;
    s.assign(sample, sample + 2);
    e.estimate_minimal(rows8, s.data(), models);
  } else if (kind == GCR_FUNDAMENTAL_AFFINE || kind == GCR_FUNDAMENTAL_SIFT) {
    const Mat rows8{corr, n, 8};
    if (kind == GCR_FUNDAMENTAL_AFFINE) {
      FundamentalAffineEstimator e;
      s.assign(sample, sample + 3);
      e.estimate_minimal(rows8, s.data(), models);
    } else {
      FundamentalSiftEstimator e;
      s.assign(sample, sample + 4);
      e.estimate_minimal(rows8, s.data(), models);
    }
  } else if (kind == GCR_ESSENTIAL_PLANAR) {
    EssentialPlanarEstimator e;
    s.assign(sample, sample + 2);
    e.estimate_minimal(pts, s.data(), models);
  } else if (kind == GCR_HOMOGRAPHY) {
    HomographyEstimator e;
    s.assign(sample, sample + 4);
    if (!e.is_valid_sample(pts, s.data())) return -1;
    e.estimate_minimal(pts, s.data(), models);
  } else if (kind == GCR_FUNDAMENTAL) {
    FundamentalEstimator e;
    s.assign(sample, sample + 7);
    e.estimate_minimal(pts, s.data(), models);
  } else {
    EssentialEstimator e;
    s.assign(sample, sample + 5);
    if (!e.is_valid_sample(pts, s.data())) return -1;
    e.estimate_minimal(pts, s.data(), models);
  }
  for (size_t i = 0; i < models.size() && i < 10; ++i) std::memcpy(models_out + 9 * i, models[i].data(), 72);
  return (int)models.size();
}

// Non-minimal essential-matrix solve (Stewenius) for tests: weights by point
// index or NULL; writes up to 10 normalised models, returns their count.
int oracle_nonminimal_essential(const double* corr, int64_t n, const int64_t* sample, int64_t ns,
                                const double* weights, double* models_out) {
  const Mat pts{corr, n, 4};
  std::vector<size_t> s(sample, sample + ns);
  std::vector<Model> models;
  EssentialEstimator e;
  if (!e.estimate_nonminimal(pts, s.data(), s.size(), models, weights)) return 0;
  for (size_t i = 0; i < models.size() && i < 10; ++i) std::memcpy(models_out + 9 * i, models[i].data(), 72);
  return (int)models.size();
}

// Real roots of a degree-10 polynomial (ascending coefficients) by the Sturm
// bracketing of the five-point solver; returns their count.
int oracle_sturm10(const double* coeffs, double* roots) {
  Sturm st;
  return st.solve(coeffs, roots);
}

// Draw sequence of the main sampler for tests of the device sampler.
int oracle_sample_sequence(int sampler, int64_t n, int m, uint64_t seed, int64_t calls, const double* corr,
                           const gcr_image_size* sz, int64_t* out, uint8_t* ok) {
  gcr_params p{};
  p.sampler = sampler;
  const Mat pts{corr, n, 4};
  auto s = make_main_sampler(p, pts, (size_t)m, *sz, seed);
  if (!s) return -1;
  std::vector<size_t> pool(n), sample(m);
  for (int64_t i = 0; i < n; ++i) pool[i] = (size_t)i;
  for (int64_t c = 0; c < calls; ++c) {
    ok[c] = s->sample(pool, sample.data(), (size_t)m);
    for (int j = 0; j < m; ++j) out[c * m + j] = (int64_t)sample[j];
  }
  return 0;
}

void oracle_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  philox4x32_10(c, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = c[i];
}

uint32_t oracle_draw_u32(uint64_t seed, uint32_t stream, uint64_t call, uint32_t draw) {
  return draw_u32(seed, stream, call, draw);
}

}  // extern "C"
