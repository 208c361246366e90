// SIFT-correspondence homography instantiation of the pair engine
// (findHomographySIFT_, gcransac_python.cpp:4813-5069).
#include "gcr_homography.cuh"
#include "gcr_kinds.h"
#include "gcr_launch.cuh"

namespace gcr {
namespace {

using Est = HomographySiftModel;

size_t h_shared() { return shared_bytes<Est>(); }
size_t h_slot(int n, int s) { return slot_bytes<Est>(n, s); }
void h_carve(unsigned char* b, int n, int s, Slot* o) { *o = carve_slot<Est>(b, n, s); }
cudaError_t h_prepare() {
  return cudaFuncSetAttribute(pair_kernel<Est>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared_bytes<Est>());
}
cudaError_t h_occupancy(int* b) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, pair_kernel<Est>, GCR_BLOCK, shared_bytes<Est>());
}
cudaError_t h_launch(int grid, cudaStream_t st, const Workspace& ws, const EngineParams& prm) {
  pair_kernel<Est><<<grid, GCR_BLOCK, shared_bytes<Est>(), st>>>(ws, prm);
  return cudaGetLastError();
}

const KindOps kOps = {Est::M, h_shared, h_slot, h_carve, nullptr, nullptr, h_prepare, h_occupancy, h_launch};

}  // namespace

const KindOps* homography_sift_ops() { return &kOps; }

}  // namespace gcr
