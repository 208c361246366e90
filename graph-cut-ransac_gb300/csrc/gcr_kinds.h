// Host-side table of the per-model-kind engine instantiations. Each kind's
// kernel lives in its own translation unit (gcr_kind_*.cu) so the three
// compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace gcr {

struct Slot;
struct Workspace;
struct EngineParams;

struct KindOps {
  int sample_size;
  size_t (*shared_bytes)();
  size_t (*slot_bytes)(int max_n, int sort_cap);
  void (*carve)(unsigned char* base, int max_n, int sort_cap, Slot* out);
  size_t (*nested_slot_bytes)(int max_n);                        // nullptr: no inner runs
  void (*carve_nested)(unsigned char* base, int max_n, Slot* out);
  cudaError_t (*prepare)();  // one-time kernel attribute setup
  cudaError_t (*occupancy)(int* blocks_per_sm);
  cudaError_t (*launch)(int grid, cudaStream_t stream, const Workspace& ws, const EngineParams& prm);
};

const KindOps* homography_ops();
const KindOps* fundamental_ops();
const KindOps* essential_ops();
const KindOps* homography_affine_ops();   // affine correspondences (gcr_kind_ha.cu)
const KindOps* fundamental_affine_ops();  // affine correspondences (gcr_kind_fa.cu)
const KindOps* fundamental_sift_ops();    // SIFT correspondences (gcr_kind_fs.cu)
const KindOps* homography_sift_ops();     // SIFT correspondences (gcr_kind_hs.cu)
const KindOps* essential_planar_ops();    // planar motion (gcr_kind_ep.cu)

struct PairDesc;
struct PairAux;

// Staging of every pair of a batch: the centred FP32 copy into ws.pts32 and
// the per-pair scale and non-finite flag into aux (one CTA per pair).
cudaError_t launch_centre(const Workspace& ws, PairAux* aux, int num_pairs, cudaStream_t stream);

// K^-1 normalisation of essential-matrix correspondences (utils.h:65-103 of
// the reference): kinv holds K1^-1 then K2^-1 (row-major) per pair; one CTA
// per pair.
cudaError_t launch_normalise_essential(const double* corr, const double* kinv, const PairDesc* pairs, int num_pairs,
                                       double* out, cudaStream_t stream);

// Affine correspondences: rows of 8 doubles into the point rows pts [total][4]
// and the local affine maps aff [total][4].
cudaError_t launch_split_affine(const double* corr8, int64_t total, double* pts, double* aff, cudaStream_t stream);

// Cumulative normalised probabilities of the importance sampler, one table per
// pair laid out like the correspondences.
cudaError_t launch_importance_cdf(const double* probs, const PairDesc* pairs, int num_pairs, double* cdf,
                                  cudaStream_t stream);

}  // namespace gcr
