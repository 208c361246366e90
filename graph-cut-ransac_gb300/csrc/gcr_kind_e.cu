// Essential-matrix instantiation of the pair engine, and the K^-1
// normalisation of the correspondences it runs on.
#include "gcr_essential.cuh"
#include "gcr_kinds.h"
#include "gcr_launch.cuh"

namespace gcr {
namespace {

using Est = EssentialModel;

size_t e_shared() { return shared_bytes<Est>(); }
size_t e_slot(int n, int s) { return slot_bytes<Est>(n, s); }
void e_carve(unsigned char* b, int n, int s, Slot* o) { *o = carve_slot<Est>(b, n, s); }
cudaError_t e_prepare() {
  return cudaFuncSetAttribute(pair_kernel<Est>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared_bytes<Est>());
}
cudaError_t e_occupancy(int* b) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, pair_kernel<Est>, GCR_BLOCK, shared_bytes<Est>());
}
cudaError_t e_launch(int grid, cudaStream_t st, const Workspace& ws, const EngineParams& prm) {
  pair_kernel<Est><<<grid, GCR_BLOCK, shared_bytes<Est>(), st>>>(ws, prm);
  return cudaGetLastError();
}

const KindOps kOps = {Est::M, e_shared, e_slot, e_carve, nullptr, nullptr, e_prepare, e_occupancy, e_launch};

// utils::normalizeCorrespondences (utils.h:65-103): (x, y, 1) times K^-1 per
// image, first two components kept. One CTA per pair; products and sums are
// rounded separately (no fused multiply-add), like a plain CPU evaluation.
__global__ void normalise_kernel(const double* corr, const double* kinv, const PairDesc* pairs, double* out) {
  const PairDesc& pd = pairs[blockIdx.x];
  const double* K1 = kinv + 18 * blockIdx.x;
  const double* K2 = K1 + 9;
  for (int i = threadIdx.x; i < pd.n; i += blockDim.x) {
    const double* p = corr + 4 * (pd.offset + i);
    double* o = out + 4 * (pd.offset + i);
    o[0] = __dadd_rn(__dadd_rn(__dmul_rn(K1[0], p[0]), __dmul_rn(K1[1], p[1])), K1[2]);
    o[1] = __dadd_rn(__dadd_rn(__dmul_rn(K1[3], p[0]), __dmul_rn(K1[4], p[1])), K1[5]);
    o[2] = __dadd_rn(__dadd_rn(__dmul_rn(K2[0], p[2]), __dmul_rn(K2[1], p[3])), K2[2]);
    o[3] = __dadd_rn(__dadd_rn(__dmul_rn(K2[3], p[2]), __dmul_rn(K2[4], p[3])), K2[5]);
  }
}

}  // namespace

const KindOps* essential_ops() { return &kOps; }

cudaError_t launch_normalise_essential(const double* corr, const double* kinv, const PairDesc* pairs, int num_pairs,
                                       double* out, cudaStream_t stream) {
  if (num_pairs <= 0) return cudaSuccess;
  normalise_kernel<<<num_pairs, 256, 0, stream>>>(corr, kinv, pairs, out);
  return cudaGetLastError();
}

}  // namespace gcr
