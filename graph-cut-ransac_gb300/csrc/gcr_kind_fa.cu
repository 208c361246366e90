// Affine-correspondence fundamental-matrix instantiation of the pair engine
// (findFundamentalMatrixAC_, gcransac_python.cpp:1924-2221): no DEGENSAC, so
// no nested slots for its inner run.
#include "gcr_fundamental.cuh"
#include "gcr_kinds.h"
#include "gcr_launch.cuh"

namespace gcr {
namespace {

using Est = FundamentalAffineModel;

size_t fa_shared() { return shared_bytes<Est>(); }
size_t fa_slot(int n, int s) { return slot_bytes<Est>(n, s); }
void fa_carve(unsigned char* b, int n, int s, Slot* o) { *o = carve_slot<Est>(b, n, s); }
cudaError_t fa_prepare() {
  return cudaFuncSetAttribute(pair_kernel<Est>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared_bytes<Est>());
}
cudaError_t fa_occupancy(int* b) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, pair_kernel<Est>, GCR_BLOCK, shared_bytes<Est>());
}
cudaError_t fa_launch(int grid, cudaStream_t st, const Workspace& ws, const EngineParams& prm) {
  pair_kernel<Est><<<grid, GCR_BLOCK, shared_bytes<Est>(), st>>>(ws, prm);
  return cudaGetLastError();
}

const KindOps kOps = {Est::M, fa_shared, fa_slot, fa_carve, nullptr, nullptr, fa_prepare, fa_occupancy, fa_launch};

}  // namespace

const KindOps* fundamental_affine_ops() { return &kOps; }

}  // namespace gcr
