// Slicing / vector-field DVR / LIC-volume instantiations for field storage VVLIC_STORAGE_UNORM8.
#include "techniques.cuh"

namespace vvlic {

cudaError_t launch_technique_u8(const RenderArgs& a, const TechArgs& t, int sampler, int integ, bool grad,
                                 cudaStream_t s) {
  return launch_tech_storage<VVLIC_STORAGE_UNORM8>(a, t, sampler, integ, grad, s);
}

}  // namespace vvlic
