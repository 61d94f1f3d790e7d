// Forward ray-cast instantiations for field storage VVLIC_STORAGE_F16.
#include "render_fwd.cuh"

namespace vvlic {

cudaError_t launch_raycast_f16(const RenderArgs& a, int sampler, int integ, bool grad, const Schedule& sch,
                               cudaStream_t s) {
  return launch_storage<VVLIC_STORAGE_F16>(a, sampler, integ, grad, sch, s);
}

}  // namespace vvlic
