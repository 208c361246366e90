// Oracle (test infrastructure only): fundamental-matrix estimator.
#pragma once
#include "oracle_common.hpp"
#include "oracle_linalg.hpp"

namespace oracle {

struct FundamentalEstimator {
  static constexpr size_t sample_size() { return 7; }
  size_t inlier_limit() const { return 7 * sample_size(); }
  double squared_residual(const double*, const Model&) const { return 0; }
  bool estimate_minimal(const Mat&, const size_t*, std::vector<Model>&) const { return false; }
  bool estimate_nonminimal(const Mat&, const size_t*, size_t, std::vector<Model>&, const double*) const { return false; }
  bool is_valid_model(Model&, const Mat&, const std::vector<size_t>&, const size_t*, double, bool&) const { return false; }
  bool is_valid_sample(const Mat&, const size_t*) const { return true; }
};

inline int find_fundamental(const double*, int64_t, const gcr_image_size&, const gcr_params&, uint64_t, double*,
                            uint8_t*, gcr_stats*) {
  return GCR_UNSUPPORTED;
}

}  // namespace oracle
