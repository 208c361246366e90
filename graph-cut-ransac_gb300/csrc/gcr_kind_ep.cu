// Planar-motion essential-matrix instantiation of the pair engine
// (findPlanarEssentialMatrix_, gcransac_python.cpp:3531-3870); the K^-1
// normalisation is the essential kind's (gcr_kind_e.cu).
#include "gcr_essential.cuh"
#include "gcr_kinds.h"
#include "gcr_launch.cuh"

namespace gcr {
namespace {

using Est = EssentialPlanarModel;

size_t ep_shared() { return shared_bytes<Est>(); }
size_t ep_slot(int n, int s) { return slot_bytes<Est>(n, s); }
void ep_carve(unsigned char* b, int n, int s, Slot* o) { *o = carve_slot<Est>(b, n, s); }
cudaError_t ep_prepare() {
  return cudaFuncSetAttribute(pair_kernel<Est>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared_bytes<Est>());
}
cudaError_t ep_occupancy(int* b) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, pair_kernel<Est>, GCR_BLOCK, shared_bytes<Est>());
}
cudaError_t ep_launch(int grid, cudaStream_t st, const Workspace& ws, const EngineParams& prm) {
  pair_kernel<Est><<<grid, GCR_BLOCK, shared_bytes<Est>(), st>>>(ws, prm);
  return cudaGetLastError();
}

const KindOps kOps = {Est::M, ep_shared, ep_slot, ep_carve, nullptr, nullptr, ep_prepare, ep_occupancy, ep_launch};

}  // namespace

const KindOps* essential_planar_ops() { return &kOps; }

}  // namespace gcr
