/* C++ plugin surface of the GB300 engine: the class and member names of the
 * reference's template interface, gcransac::GCRANSAC<ModelEstimator,
 * NeighborhoodGraph, ScoringFunction, PreemptiveModelVerification,
 * FastInlierSelector> (src/pygcransac/include/GCRANSAC.h:47-99), with the
 * library's own estimators, samplers, neighbourhood graph, scoring functions,
 * preemptive verification and inlier selector, so that code written against
 * that interface compiles against this header and runs on the device.
 *
 * Correspondences are a gcransac::MatView (row-major doubles, 4 columns:
 * x1 y1 x2 y2) instead of cv::Mat. run() forwards to gcr_run (include/gcr.h;
 * gcr_run_with_probabilities for the importance and AR samplers):
 * one pair, GCRANSAC::run semantics (no Python-driver pre- or post-processing),
 * the samplers' and graph's data points as the neighbourhood coordinates, the
 * points given to run() as the fitting coordinates (K^-1-normalised ones for
 * essential matrices, as the reference's essential driver passes them), the
 * threshold in the fitting coordinates' units.
 *
 * Header-only; link with libgcr.so. Plugin types outside this header, and
 * settings the device engine does not provide, are compile-time or run-time
 * errors (std::invalid_argument); nothing falls back to a CPU path.
 *
 * Reference counterparts:
 *   MatView                          cv::Mat (data container)
 *   Model                            model.h:43-60
 *   utils::Settings                  settings.h:44-87
 *   utils::RANSACStatistics          statistics.h:43-72
 *   utils::Default*Estimator         types.h:78-112 (7-point + bundle adjustment F,
 *                                    4-point H, Nister + Stewenius E)
 *   sampler::UniformSampler          samplers/uniform_sampler.h:45-115
 *   sampler::ProsacSampler           samplers/prosac_sampler.h:51-237
 *   sampler::ProgressiveNapsacSampler<4>  samplers/progressive_napsac_sampler.h:50-326
 *   sampler::ImportanceSampler       samplers/importance_sampler.h:51-136
 *   sampler::AdaptiveReorderingSampler  samplers/adaptive_reordering_sampler.h:46-166
 *   neighborhood::GridNeighborhoodGraph<4> neighborhood/grid_neighborhood_graph.h:132-301
 *   neighborhood::FlannNeighborhoodGraph   neighborhood/flann_neighborhood_graph.h:100-139 (exact ball)
 *   MSACScoringFunction, MAGSACScoringFunction  scoring_function.h:137-348
 *   preemption::EmptyPreemptiveVerfication, SPRTPreemptiveVerfication
 *                                    preemption/preemption_empty.h, preemption_sprt.h:50-380
 *   inlier_selector::EmptyInlierSelector, SpacePartitioningRANSAC
 *                                    inlier_selectors/empty_inlier_selector.h,
 *                                    space_partitioning_ransac.h:341-505
 */
#ifndef GCRANSAC_GB300_GCRANSAC_H_
#define GCRANSAC_GB300_GCRANSAC_H_

#include <chrono>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../gcr.h"

namespace gcransac {

/* Row-major view of n x cols doubles (cols = 4 for two-view correspondences). */
class MatView {
 public:
  MatView() = default;
  MatView(const double* data_, int rows_, int cols_) : data(data_), rows(rows_), cols(cols_) {}
  template <class T>
  const T* ptr(int r) const {
    static_assert(std::is_same<T, double>::value, "MatView holds doubles");
    return data + (size_t)r * cols;
  }
  template <class T>
  const T& at(int r, int c) const {
    static_assert(std::is_same<T, double>::value, "MatView holds doubles");
    return data[(size_t)r * cols + c];
  }
  bool empty() const { return rows == 0; }
  const double* data = nullptr;
  int rows = 0, cols = 0;
};

/* A 3 x 3 model; rows() == 0 when the run found none. */
struct Descriptor {
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int r = 0, c = 0;
  double& operator()(int i, int j) { return v[i * 3 + j]; }
  double operator()(int i, int j) const { return v[i * 3 + j]; }
  int rows() const { return r; }
  int cols() const { return c; }
};

class Model {
 public:
  Descriptor descriptor;
};

namespace utils {

struct Settings {
  bool do_final_iterated_least_squares = true, do_local_optimization = true, do_graph_cut = true,
       use_inlier_limit = false;
  double desired_fps = -1;
  size_t max_local_optimization_number = 10, min_iteration_number_before_lo = 20, min_iteration_number = 20,
         max_iteration_number = std::numeric_limits<size_t>::max(), max_unsuccessful_model_generations = 100,
         max_least_squares_iterations = 10, max_graph_cut_number = 10, core_number = 1;
  double confidence = 0.95, neighborhood_sphere_radius = 20, threshold = 2.0, spatial_coherence_weight = 0.14;
};

struct RANSACStatistics {
  size_t graph_cut_number = 0, local_optimization_number = 0, iteration_number = 0, neighbor_number = 0,
         accepted_models = 0, rejected_models = 0;
  std::string main_sampler_name, local_optimizer_sampler_name;
  double processing_time = 0.0, score = 0.0;
  std::vector<size_t> inliers;
};

/* The default estimators of the reference's drivers (types.h:78-112). */
class DefaultHomographyEstimator {
 public:
  static constexpr gcr_model_kind kind = GCR_HOMOGRAPHY;
  static constexpr size_t sampleSize() { return 4; }
  static constexpr size_t inlierLimit() { return 7 * sampleSize(); }
};
class DefaultFundamentalMatrixEstimator {
 public:
  static constexpr gcr_model_kind kind = GCR_FUNDAMENTAL;
  static constexpr size_t sampleSize() { return 7; }
  static constexpr size_t inlierLimit() { return 7 * sampleSize(); }
  /* the validity ratio (0.5) and DEGENSAC are those of the default estimator */
  explicit DefaultFundamentalMatrixEstimator(double minimum_inlier_ratio_in_validity_check_ = 0.5,
                                             bool apply_degensac_ = true) {
    if (minimum_inlier_ratio_in_validity_check_ != 0.5 || !apply_degensac_)
      throw std::invalid_argument("the device engine provides the default fundamental-matrix estimator only");
  }
};
class DefaultEssentialMatrixEstimator {
 public:
  static constexpr gcr_model_kind kind = GCR_ESSENTIAL;
  static constexpr size_t sampleSize() { return 5; }
  static constexpr size_t inlierLimit() { return 7 * sampleSize(); }
  /* intrinsics as row-major 3 x 3; the run works on points already
     normalised by their inverses */
  DefaultEssentialMatrixEstimator(const double* intrinsics_src_, const double* intrinsics_dst_,
                                  double minimum_inlier_ratio_in_validity_check_ = 0.1,
                                  double point_ratio_for_selecting_from_multiple_models_ = 0.05) {
    for (int k = 0; k < 9; ++k) {
      intrinsics_src[k] = intrinsics_src_[k];
      intrinsics_dst[k] = intrinsics_dst_[k];
    }
    if (minimum_inlier_ratio_in_validity_check_ != 0.1 || point_ratio_for_selecting_from_multiple_models_ != 0.05)
      throw std::invalid_argument("the device engine provides the default essential-matrix estimator only");
  }
  double intrinsics_src[9], intrinsics_dst[9];
};

}  // namespace utils

namespace sampler {

template <class Container, class Index>
class Sampler {
 public:
  explicit Sampler(const Container* container_) : container(container_) {}
  virtual ~Sampler() = default;
  virtual const std::string getName() const = 0;
  virtual void reset() {}
  bool isInitialized() const { return initialized; }
  /* the engine's sampler id (GCR_SAMPLER_*) */
  virtual int deviceSamplerId() const = 0;
  /* the per-point probabilities the sampler draws from (samplers 3 and 4), else NULL */
  virtual const std::vector<double>* deviceProbabilities() const { return nullptr; }
  const Container* container;

 protected:
  bool initialized = true;
};

class UniformSampler : public Sampler<MatView, size_t> {
 public:
  explicit UniformSampler(const MatView* container_) : Sampler(container_) {}
  const std::string getName() const override { return "Uniform Sampler"; }
  int deviceSamplerId() const override { return GCR_SAMPLER_UNIFORM; }
};

/* Correspondences must be ordered by decreasing quality. */
class ProsacSampler : public Sampler<MatView, size_t> {
 public:
  ProsacSampler(const MatView* container_, size_t sample_size_, size_t ransac_convergence_iterations_ = 100000)
      : Sampler(container_), sample_size(sample_size_) {
    if (ransac_convergence_iterations_ != 100000)
      throw std::invalid_argument("the device PROSAC sampler converges to uniform after 100000 samples");
  }
  const std::string getName() const override { return "PROSAC Sampler"; }
  int deviceSamplerId() const override { return GCR_SAMPLER_PROSAC; }
  size_t sample_size;
};

template <size_t _DimensionNumber>
class ProgressiveNapsacSampler : public Sampler<MatView, size_t> {
 public:
  /* layer_data_ {16, 8, 4, 2}, sizes_ {w1, h1, w2, h2} of the two images */
  ProgressiveNapsacSampler(const MatView* container_, const std::vector<size_t>& layer_data_, size_t sample_size_,
                           const std::vector<double>& sizes_, double sampler_length_ = 20)
      : Sampler(container_), sample_size(sample_size_), sizes(sizes_), sampler_length(sampler_length_) {
    static_assert(_DimensionNumber == 4, "two-view correspondences have four coordinates");
    if (layer_data_ != std::vector<size_t>{16, 8, 4, 2} || sizes_.size() != 4 || sampler_length_ != 0.5)
      throw std::invalid_argument(
          "the device P-NAPSAC sampler has layers {16, 8, 4, 2}, image sizes {w1, h1, w2, h2} and "
          "sampler length 0.5 (the drivers' configuration)");
  }
  const std::string getName() const override { return "Progressive NAPSAC Sampler"; }
  int deviceSamplerId() const override { return GCR_SAMPLER_PNAPSAC; }
  size_t sample_size;
  std::vector<double> sizes;
  double sampler_length;
};

/* ImportanceSampler (samplers/importance_sampler.h:51-136): every sample is m
   independent draws from the multinomial distribution of the given point
   probabilities (std::discrete_distribution there, the engine's counter-based
   streams here). */
class ImportanceSampler : public Sampler<MatView, size_t> {
 public:
  ImportanceSampler(const MatView* container_, const std::vector<double>& probabilities_, size_t sample_size_)
      : Sampler(container_), probabilities(probabilities_), sample_size(sample_size_) {
    initialized = probabilities_.size() == (size_t)container_->rows;
  }
  const std::string getName() const override { return "Importance Sampler"; }
  int deviceSamplerId() const override { return GCR_SAMPLER_IMPORTANCE; }
  const std::vector<double>* deviceProbabilities() const override { return &probabilities; }
  std::vector<double> probabilities;
  size_t sample_size;
};

/* AdaptiveReorderingSampler (samplers/adaptive_reordering_sampler.h:46-166):
   a max-heap of point probabilities; a sample takes the m most probable points
   and pushes each back with its updated beta-posterior estimate plus a jitter
   of +-randomness/2. The engine keeps the reference drivers' configuration:
   randomness 0.01, not ordered, and probabilities divided by their maximum
   (gcransac_python.cpp:1730-1741), so the vector given here must have maximum 1
   for the run to equal the reference's sampler on the same vector. */
class AdaptiveReorderingSampler : public Sampler<MatView, size_t> {
 public:
  AdaptiveReorderingSampler(const MatView* container_, const std::vector<double>& inlier_probabilities_,
                            size_t sample_size_, double estimator_variance_ = 0.9765, double randomness_ = 0.01,
                            bool ordered_ = false)
      : Sampler(container_), probabilities(inlier_probabilities_), sample_size(sample_size_),
        estimator_variance(estimator_variance_) {
    if (randomness_ != 0.01 || ordered_)
      throw std::invalid_argument("the device AR sampler has randomness 0.01 and no ordered mode");
    if (!(estimator_variance_ > 0)) throw std::invalid_argument("the AR sampler needs estimator_variance > 0");
    double mx = 0.0;
    for (double v : inlier_probabilities_) mx = v > mx ? v : mx;
    if (!inlier_probabilities_.empty() && mx != 1.0)
      throw std::invalid_argument(
          "the device AR sampler divides the probabilities by their maximum, as the reference's drivers do "
          "before constructing it: pass probabilities whose maximum is 1");
    initialized = inlier_probabilities_.size() == (size_t)container_->rows;
  }
  const std::string getName() const override { return "Probabilistic Reordering Sampler"; }
  int deviceSamplerId() const override { return GCR_SAMPLER_AR; }
  const std::vector<double>* deviceProbabilities() const override { return &probabilities; }
  std::vector<double> probabilities;
  size_t sample_size;
  double estimator_variance;
};

}  // namespace sampler

namespace neighborhood {

template <size_t _DimensionNumber>
class GridNeighborhoodGraph {
 public:
  GridNeighborhoodGraph(const MatView* container_, const std::vector<double>& cell_sizes_,
                        const size_t& cell_number_along_all_axes_)
      : container(container_), cell_sizes(cell_sizes_), cell_number_along_all_axes(cell_number_along_all_axes_) {
    static_assert(_DimensionNumber == 4, "two-view correspondences have four coordinates");
    if (cell_sizes_.size() != 4) throw std::invalid_argument("the grid needs four cell sizes");
  }
  const std::string getName() const { return "Grid Neighborhood Graph"; }
  const MatView* container;
  std::vector<double> cell_sizes;
  size_t cell_number_along_all_axes;
};

// The radius graph (flann_neighborhood_graph.h:100-139) as an exact ball
// search of radius matching_radius_ in the four pixel coordinates.
class FlannNeighborhoodGraph {
 public:
  FlannNeighborhoodGraph(const MatView* container_, double matching_radius_)
      : container(container_), matching_radius(matching_radius_) {
    if (!(matching_radius_ > 0)) throw std::invalid_argument("the neighbourhood radius must be positive");
  }
  const std::string getName() const { return "FLANN neighborhood (radius)"; }
  const MatView* container;
  double matching_radius;
};

}  // namespace neighborhood

template <class _ModelEstimator>
class MSACScoringFunction {
 public:
  static constexpr int device_scoring = GCR_SCORING_MSAC;
};

template <class _ModelEstimator>
class MAGSACScoringFunction {
 public:
  static constexpr int device_scoring = GCR_SCORING_MAGSAC;
};

namespace preemption {

template <class _ModelEstimator>
class EmptyPreemptiveVerfication {
 public:
  static constexpr bool device_sprt = false;
  double minimum_inlier_ratio() const { return 1e-5; }
};

template <class _ModelEstimator>
class SPRTPreemptiveVerfication {
 public:
  static constexpr bool device_sprt = true;
  SPRTPreemptiveVerfication(const MatView& points_, const _ModelEstimator& estimator_,
                            const double& minimum_inlier_ratio_ = 0.01)
      : ratio(minimum_inlier_ratio_) {
    (void)points_;
    (void)estimator_;
  }
  double minimum_inlier_ratio() const { return ratio; }

 private:
  double ratio;
};

}  // namespace preemption

namespace inlier_selector {

template <class _Estimator, class _NeighborhoodStructure>
class EmptyInlierSelector {
 public:
  static constexpr bool device_space_partitioning = false;
  explicit EmptyInlierSelector(const _NeighborhoodStructure* = nullptr) {}
};

template <class _Estimator, class _NeighborhoodStructure>
class SpacePartitioningRANSAC {
 public:
  static constexpr bool device_space_partitioning = true;
  explicit SpacePartitioningRANSAC(const _NeighborhoodStructure* kNeighborhoodGraph_) {
    (void)kNeighborhoodGraph_;
    static_assert(_Estimator::kind == GCR_HOMOGRAPHY, "space partitioning is provided for homographies");
  }
};

}  // namespace inlier_selector

template <class _ModelEstimator, class _NeighborhoodGraph,
          class _ScoringFunction = MSACScoringFunction<_ModelEstimator>,
          class _PreemptiveModelVerification = preemption::EmptyPreemptiveVerfication<_ModelEstimator>,
          class _FastInlierSelector = inlier_selector::EmptyInlierSelector<_ModelEstimator, _NeighborhoodGraph>>
class GCRANSAC {
  static constexpr bool kRadius = std::is_same<_NeighborhoodGraph, neighborhood::FlannNeighborhoodGraph>::value;
  static_assert(std::is_same<_NeighborhoodGraph, neighborhood::GridNeighborhoodGraph<4>>::value || kRadius,
                "the device engine provides the grid and the radius neighbourhood graphs");

 public:
  utils::Settings settings;
  /* seed of the engine's counter-based sampler streams (the reference seeds
     std::mt19937 from std::random_device) */
  uint64_t seed = 0;

  void run(const MatView& points_, const _ModelEstimator& estimator_,
           sampler::Sampler<MatView, size_t>* main_sampler_,
           sampler::Sampler<MatView, size_t>* local_optimization_sampler_,
           const _NeighborhoodGraph* neighborhood_graph_, Model& obtained_model_,
           _PreemptiveModelVerification& preemptive_verification_, _FastInlierSelector& fast_inlier_selector_) {
    (void)estimator_;
    (void)fast_inlier_selector_;
    gcr_params p;
    gcr_default_params(_ModelEstimator::kind, &p);
    check_settings();
    if (!main_sampler_ || !local_optimization_sampler_ || !neighborhood_graph_)
      throw std::invalid_argument("run needs both samplers and the neighbourhood graph");
    if (local_optimization_sampler_->deviceSamplerId() != GCR_SAMPLER_UNIFORM)
      throw std::invalid_argument("the local optimisation sampler must be the uniform sampler");
    if (points_.cols != 4 || neighborhood_graph_->container->rows != points_.rows ||
        neighborhood_graph_->container->cols != 4)
      throw std::invalid_argument("points and the graph's data must be the same n x 4 correspondences");
    p.threshold = settings.threshold;
    p.confidence = settings.confidence;
    p.spatial_coherence_weight = settings.spatial_coherence_weight;
    double cells_[4] = {1.0, 1.0, 1.0, 1.0};
    int32_t divisions_ = 1;
    if constexpr (kRadius) {
      p.neighborhood = GCR_NEIGHBORHOOD_FLANN;
      p.neighborhood_size = neighborhood_graph_->matching_radius;
    } else {
      p.neighborhood = GCR_NEIGHBORHOOD_GRID;
      p.neighborhood_size = (double)neighborhood_graph_->cell_number_along_all_axes;
      for (int q = 0; q < 4; ++q) cells_[q] = neighborhood_graph_->cell_sizes[q];
      divisions_ = (int32_t)neighborhood_graph_->cell_number_along_all_axes;
    }
    p.max_iterations = settings.max_iteration_number > (size_t)std::numeric_limits<int64_t>::max()
                           ? std::numeric_limits<int64_t>::max()
                           : (int64_t)settings.max_iteration_number;
    p.min_iterations = (int64_t)settings.min_iteration_number;
    p.sampler = main_sampler_->deviceSamplerId();
    const std::vector<double>* probs = main_sampler_->deviceProbabilities();
    if (probs && (!main_sampler_->isInitialized() || probs->size() != (size_t)points_.rows))
      throw std::invalid_argument("the sampler's probabilities must have one entry per correspondence");
    if (auto* ar = dynamic_cast<const sampler::AdaptiveReorderingSampler*>(main_sampler_))
      p.sampler_variance = ar->estimator_variance;
    p.lo_number = (int32_t)settings.max_local_optimization_number;
    p.scoring = _ScoringFunction::device_scoring;
    p.use_sprt = _PreemptiveModelVerification::device_sprt ? 1 : 0;
    p.min_inlier_ratio_for_sprt = preemptive_verification_.minimum_inlier_ratio();
    p.use_space_partitioning = _FastInlierSelector::device_space_partitioning ? 1 : 0;
    p.seed = seed;
    // image extents: P-NAPSAC's sizes when given, else the grid's span or the
    // points' bounding box
    gcr_image_size size;
    {
      double mx[4] = {cells_[0] * divisions_, cells_[1] * divisions_, cells_[2] * divisions_,
                      cells_[3] * divisions_};
      if constexpr (kRadius) {
        const MatView& px = *neighborhood_graph_->container;
        for (int q = 0; q < 4; ++q) mx[q] = 1.0;
        for (int r = 0; r < px.rows; ++r)
          for (int q = 0; q < 4; ++q) mx[q] = px.at<double>(r, q) > mx[q] ? px.at<double>(r, q) : mx[q];
      }
      size.w1 = (int32_t)mx[0];
      size.h1 = (int32_t)mx[1];
      size.w2 = (int32_t)mx[2];
      size.h2 = (int32_t)mx[3];
    }
    if (auto* pn = dynamic_cast<const sampler::ProgressiveNapsacSampler<4>*>(main_sampler_)) {
      size.w1 = (int32_t)pn->sizes[0];
      size.h1 = (int32_t)pn->sizes[1];
      size.w2 = (int32_t)pn->sizes[2];
      size.h2 = (int32_t)pn->sizes[3];
    }
    const int64_t n = points_.rows;
    std::vector<uint8_t> mask((size_t)n);
    gcr_stats st{};
    Model out;
    const auto t_start = std::chrono::steady_clock::now();
    const gcr_status rc =
        probs ? gcr_run_with_probabilities(_ModelEstimator::kind, points_.data, neighborhood_graph_->container->data,
                                           n, cells_, divisions_, &size, probs->data(), &p, out.descriptor.v,
                                           mask.data(), &st)
              : gcr_run(_ModelEstimator::kind, points_.data, neighborhood_graph_->container->data, n, cells_,
                        divisions_, &size, &p, out.descriptor.v, mask.data(), &st);
    if (rc != GCR_OK && rc != GCR_NO_MODEL) throw std::runtime_error(gcr_last_error_string());
    statistics = utils::RANSACStatistics();
    // wall-clock seconds of the run (GCRANSAC.h:263, 624-626); here the call
    // includes the copies of the points to the device and of the results back
    statistics.processing_time =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    statistics.main_sampler_name = main_sampler_->getName();
    statistics.local_optimizer_sampler_name = local_optimization_sampler_->getName();
    statistics.iteration_number = (size_t)st.iteration_number;
    statistics.graph_cut_number = (size_t)st.graph_cut_number;
    statistics.local_optimization_number = (size_t)st.local_optimization_number;
    statistics.score = st.score;
    for (int64_t i = 0; i < n; ++i)
      if (mask[(size_t)i]) statistics.inliers.push_back((size_t)i);
    if (rc == GCR_OK) {
      out.descriptor.r = out.descriptor.c = 3;
      obtained_model_ = out;
    } else {
      obtained_model_ = Model();
    }
  }

  void run(const MatView& points_, const _ModelEstimator& estimator_,
           sampler::Sampler<MatView, size_t>* main_sampler_,
           sampler::Sampler<MatView, size_t>* local_optimization_sampler_,
           const _NeighborhoodGraph* neighborhood_graph_, Model& obtained_model_) {
    static_assert(!_PreemptiveModelVerification::device_sprt && !_FastInlierSelector::device_space_partitioning,
                  "SPRT and space partitioning take their objects: use the eight-argument run");
    _PreemptiveModelVerification pv;
    _FastInlierSelector sel(neighborhood_graph_);
    run(points_, estimator_, main_sampler_, local_optimization_sampler_, neighborhood_graph_, obtained_model_, pv,
        sel);
  }

  void setFPS(double fps_) {
    if (fps_ > 0) throw std::invalid_argument("the device engine has no time limit");
  }
  const utils::RANSACStatistics& getRansacStatistics() const { return statistics; }
  utils::RANSACStatistics& getMutableRansacStatistics() { return statistics; }
  const _ScoringFunction& getScoringFunction() const { return scoring_function; }
  _ScoringFunction& getMutableScoringFunction() { return scoring_function; }

 protected:
  utils::RANSACStatistics statistics;
  _ScoringFunction scoring_function;

  // settings of GCRANSAC::run that the engine fixes (settings.h defaults)
  void check_settings() const {
    const utils::Settings d;
    if (!settings.do_final_iterated_least_squares || !settings.do_local_optimization ||
        settings.desired_fps > 0 || settings.min_iteration_number_before_lo != d.min_iteration_number_before_lo ||
        settings.max_unsuccessful_model_generations != d.max_unsuccessful_model_generations ||
        settings.max_least_squares_iterations != d.max_least_squares_iterations ||
        settings.max_graph_cut_number != d.max_graph_cut_number)
      throw std::invalid_argument(
          "the device engine runs GC-RANSAC with local optimisation, the final iterated least squares, no time "
          "limit, 20 iterations before LO, 100 unsuccessful generations, 10 least-squares iterations and 10 "
          "graph-cuts");
  }
};

}  // namespace gcransac

#endif  // GCRANSAC_GB300_GCRANSAC_H_
