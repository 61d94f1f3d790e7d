// Forward ray-cast instantiations for field storage VVLIC_STORAGE_F16.
#include "render_fwd.cuh"

namespace vvlic {

cudaError_t launch_raycast_f16(const RenderArgs& a, int layout, int integ, bool grad, cudaStream_t s) {
  switch (layout) {
    case kGather: return launch_layout<VVLIC_STORAGE_F16, kGather>(a, integ, grad, s);
    case kCell: return launch_layout<VVLIC_STORAGE_F16, kCell>(a, integ, grad, s);
    case kTexture: return launch_layout<VVLIC_STORAGE_F16, kTexture>(a, integ, grad, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vvlic
