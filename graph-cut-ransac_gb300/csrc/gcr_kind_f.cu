// Fundamental-matrix instantiation of the pair engine.
#include "gcr_fundamental.cuh"
#include "gcr_kinds.h"
#include "gcr_launch.cuh"

namespace gcr {
namespace {

using Est = FundamentalModel;

size_t f_shared() { return shared_bytes<Est>(); }
size_t f_slot(int n, int s) { return slot_bytes<Est>(n, s); }
void f_carve(unsigned char* b, int n, int s, Slot* o) { *o = carve_slot<Est>(b, n, s); }
size_t f_nested_slot(int n) { return slot_bytes<PlaneParallaxModel>(n, 1, true); }
void f_carve_nested(unsigned char* b, int n, Slot* o) { *o = carve_slot<PlaneParallaxModel>(b, n, 1, true); }
cudaError_t f_prepare() {
  return cudaFuncSetAttribute(pair_kernel<Est>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared_bytes<Est>());
}
cudaError_t f_occupancy(int* b) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(b, pair_kernel<Est>, GCR_BLOCK, shared_bytes<Est>());
}
cudaError_t f_launch(int grid, cudaStream_t st, const Workspace& ws, const EngineParams& prm) {
  pair_kernel<Est><<<grid, GCR_BLOCK, shared_bytes<Est>(), st>>>(ws, prm);
  return cudaGetLastError();
}

const KindOps kOps = {Est::M, f_shared, f_slot, f_carve, f_nested_slot, f_carve_nested, f_prepare, f_occupancy, f_launch};

}  // namespace

const KindOps* fundamental_ops() { return &kOps; }

}  // namespace gcr
