// Batched ray-cast instantiations for field storage VVLIC_STORAGE_BF16.
#include "batch.cuh"

namespace vvlic {

cudaError_t launch_batch_bf16(const BatchLaunch& b, int sampler, int integ, bool grad, cudaStream_t s) {
  return launch_batch_storage<VVLIC_STORAGE_BF16>(b, sampler, integ, grad, s);
}

}  // namespace vvlic
