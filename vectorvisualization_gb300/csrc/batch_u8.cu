// Batched ray-cast instantiations for field storage VVLIC_STORAGE_UNORM8.
#include "batch.cuh"

namespace vvlic {

cudaError_t launch_batch_u8(const BatchLaunch& b, int sampler, int integ, bool grad, cudaStream_t s) {
  return launch_batch_storage<VVLIC_STORAGE_UNORM8>(b, sampler, integ, grad, s);
}

}  // namespace vvlic
