// Forward ray-cast instantiations for field storage VVLIC_STORAGE_BF16.
#include "render_fwd.cuh"

namespace vvlic {

cudaError_t launch_raycast_bf16(const RenderArgs& a, int layout, int integ, bool grad, cudaStream_t s) {
  switch (layout) {
    case kGather: return launch_layout<VVLIC_STORAGE_BF16, kGather>(a, integ, grad, s);
    case kCell: return launch_layout<VVLIC_STORAGE_BF16, kCell>(a, integ, grad, s);
    case kTexture: return cudaErrorNotSupported;
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vvlic
