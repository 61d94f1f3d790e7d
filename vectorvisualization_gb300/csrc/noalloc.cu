// Noise-gradient precompute that allocates nothing.
//
// vvlic_noise_gradients_device needs a temporary buffer of four floats per voxel (the raw
// gradients before smoothing, padded to 16 bytes) and gets it from the CUDA allocator.  Some callers cannot
// allocate device memory at that point: a host application that reserves its whole GPU memory
// budget up front and forbids allocations afterwards (a render or simulation host embedding
// this library as a plugin), or a frame loop where cudaMalloc / cudaFree would add allocator
// latency and cudaFree's device-wide synchronisation to every frame.  For them this file keeps
// the temporary buffer in a fixed device array that is part of the library's module, so the
// call itself performs no allocation.
//
// The array is VVLIC_NOALLOC_MAX_VOXELS * 4 floats (16 MiB).  Every GPU that loads the library
// holds it until the process exits.  All calls share it: two calls that run on the GPU at the
// same time (different streams or threads) race on it, so callers must order them.  Nothing in
// it needs to start at zero — the first kernel writes every element the second one reads — and
// it keeps the last call's contents.
//
// Compiled with -fmad=false like preprocess.cu; the kernels are the same ones, so the output is
// bit-identical to vvlic_noise_gradients_device.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/vvlic.h"
#include "vvlic_host.hpp"
#include "vvlic_launch.hpp"

namespace {

// Fixed scratch: raw gradients (x, y, z, padding) of up to VVLIC_NOALLOC_MAX_VOXELS voxels.
static __device__ __align__(256) float g_noalloc_gradients[vvlic::kNoiseGradBytes / sizeof(float) *
                                                           (size_t)VVLIC_NOALLOC_MAX_VOXELS];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
float* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code the array's name
// is only a host-side stand-in for the symbol, so the address is looked up once per device
// with that device current, and the result is cached.  The cache belongs to the device's
// primary context: cudaDeviceReset unloads the module, so a process that resets a device must
// not call the entry point on it again.  A launch that fails drops the cached address
// (forget_scratch_address), and the next call looks it up again.
vvlic_status scratch_address(int* dev_out, float** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return VVLIC_ERR_NO_DEVICE;
  *dev_out = dev;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_gradients);
    if (e != cudaSuccess || p == nullptr) return VVLIC_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<float*>(p);
  }
  *out = g_scratch_ptr[dev];
  return VVLIC_OK;
}

void forget_scratch_address(int dev) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  g_scratch_ptr[dev] = nullptr;
}

}  // namespace

extern "C" vvlic_status vvlic_noise_gradients_device_noalloc(const uint8_t* d_noise, int32_t mx, int32_t my,
                                                            int32_t mz, int32_t mode, const float* slice_dist,
                                                            uint8_t* d_rgba, void* stream) {
  if (!d_noise || !d_rgba) return VVLIC_ERR_INVALID_ARGUMENT;
  if (mode != VVLIC_NOISE_GRAD_SOBEL && mode != VVLIC_NOISE_GRAD_CENTRAL) return VVLIC_ERR_INVALID_ARGUMENT;
  // two voxels per axis (the border differences read the +1 neighbour) and the fixed maximum
  if (mx < 2 || my < 2 || mz < 2) return VVLIC_ERR_INVALID_ARGUMENT;
  if ((uint64_t)mx * (uint64_t)my * (uint64_t)mz > (uint64_t)VVLIC_NOALLOC_MAX_VOXELS) return VVLIC_ERR_INVALID_ARGUMENT;
  float sd[3] = {1.f, 1.f, 1.f};
  if (slice_dist)
    for (int i = 0; i < 3; ++i) sd[i] = slice_dist[i];
  float* scratch = nullptr;
  int dev = 0;
  vvlic_status st = scratch_address(&dev, &scratch);
  if (st != VVLIC_OK) return st;
  float w27[27];
  vvlic::noise_filter_weights(w27);
  const int m[3] = {mx, my, mz};
  cudaError_t e = vvlic::launch_noise_gradients(d_noise, m, mode, sd, scratch, d_rgba, w27, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    forget_scratch_address(dev);
    return VVLIC_ERR_CUDA;
  }
  return VVLIC_OK;
}
