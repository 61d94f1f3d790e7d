// Forward ray-cast instantiations for field storage VVLIC_STORAGE_BF16.
#include "render_fwd.cuh"

namespace vvlic {

cudaError_t launch_raycast_bf16(const RenderArgs& a, int sampler, int integ, bool grad, const Schedule& sch,
                               cudaStream_t s) {
  return launch_storage<VVLIC_STORAGE_BF16>(a, sampler, integ, grad, sch, s);
}

}  // namespace vvlic
