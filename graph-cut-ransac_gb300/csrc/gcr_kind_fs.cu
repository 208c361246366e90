// SIFT-correspondence fundamental-matrix instantiation of the pair engine
// (findFundamentalMatrixSIFT_, gcransac_python.cpp:2222-2518): no DEGENSAC,
// so no nested slots for its inner run.
#include "gcr_fundamental.cuh"
#include "gcr_kinds.h"
#include "gcr_launch.cuh"

namespace gcr {
namespace {

using Est = FundamentalSiftModel;

size_t fs_shared() { return shared_bytes<Est>(); }
size_t fs_slot(int n, int s) { return slot_bytes<Est>(n, s); }
void fs_carve(unsigned char* b, int n, int s, Slot* o) { *o = carve_slot<Est>(b, n, s); }
cudaError_t fs_prepare() {
  return cudaFuncSetAttribute(pair_kernel<Est>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared_bytes<Est>());
}
cudaError_t fs_occupancy(int* b) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, pair_kernel<Est>, GCR_BLOCK, shared_bytes<Est>());
}
cudaError_t fs_launch(int grid, cudaStream_t st, const Workspace& ws, const EngineParams& prm) {
  pair_kernel<Est><<<grid, GCR_BLOCK, shared_bytes<Est>(), st>>>(ws, prm);
  return cudaGetLastError();
}

const KindOps kOps = {Est::M, fs_shared, fs_slot, fs_carve, nullptr, nullptr, fs_prepare, fs_occupancy, fs_launch};

}  // namespace

const KindOps* fundamental_sift_ops() { return &kOps; }

}  // namespace gcr
