// Adjoint instantiations for field storage VVLIC_STORAGE_UNORM8.
#include "adjoint.cuh"

namespace vvlic {

cudaError_t launch_adjoint_u8(const RenderArgs& a, int sampler, int integ, bool lit, const float4* g_img,
                              long long* acc, const Schedule& sch, cudaStream_t s) {
  return launch_adjoint_storage<VVLIC_STORAGE_UNORM8>(a, sampler, integ, lit, g_img, acc, sch, s);
}

}  // namespace vvlic
