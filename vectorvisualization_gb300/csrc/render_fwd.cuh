// Forward LIC ray-cast kernel: one thread per pixel, the whole lic3d_fragment.glsl main()
// (lic3d_fragment.glsl:5-99) per thread.  Instantiated per field storage in render_f32.cu,
// render_f16.cu and render_bf16.cu so the three compile in parallel.
#pragma once

#include "vvlic_device.cuh"
#include "vvlic_launch.hpp"

namespace vvlic {

constexpr int kTileW = 16, kTileH = 8;  // 128 threads; a warp covers a 16x2 pixel patch

template <int ST, int LAYOUT, int INTEG, bool GRAD>
__global__ void __launch_bounds__(kTileW* kTileH) raycast_kernel(const __grid_constant__ RenderArgs a) {
  __shared__ __align__(16) float s_tf[5 * VVLIC_TF_ENTRIES];
  for (int i = threadIdx.x; i < 5 * VVLIC_TF_ENTRIES; i += blockDim.x) s_tf[i] = __ldg(a.tf + i);
  __syncthreads();

  const int px = blockIdx.x * kTileW + (threadIdx.x % kTileW);
  const int py = blockIdx.y * kTileH + (threadIdx.x / kTileW);
  const bool active = px < a.W && py < a.H;
  uint32_t samples = 0, hit = 0;
  float4 dest = make_float4(0.f, 0.f, 0.f, 0.f);
  float3 pos, dir;
  if (active && ray_setup(a, px, py, pos, dir)) {
    hit = 1;
    float4 src = make_float4(0.f, 0.f, 0.f, 0.f);
    bool outside = false;
    for (int j = 0; !outside && j < a.num_iter; ++j) {
      for (int i = 0; i < a.num_iter; ++i) {
        const float4 f = Field<ST, LAYOUT>::sample(a, pos);
        const float4 tf = tf_rgba(s_tf, a.tf_index == VVLIC_TF_INDEX_MAGNITUDE ? f.w : f.z);
        float4 il = compute_lic<ST, LAYOUT, INTEG, GRAD>(a, pos, f);
        ++samples;
        il.w *= a.intensity_scale;
        src = shade(a, s_tf, il, tf, pos, dir);
        dest = blend(dest, src);
        pos = add3(pos, scl3(dir, a.step_size));
        outside = outside_box(a, pos) || src.w > a.alpha_thr;
        if (outside) break;
      }
    }
  }
  if (active) {
    const size_t pix = (size_t)py * a.W + px;
    reinterpret_cast<float4*>(a.out)[pix] = dest;
    if (a.samples) a.samples[pix] = samples;
  }
  // per-warp reduction of the counters
  unsigned s = __reduce_add_sync(0xffffffffu, samples);
  unsigned h = __reduce_add_sync(0xffffffffu, hit);
  if ((threadIdx.x & 31) == 0) {
    if (s) atomicAdd(a.counters + 0, (unsigned long long)s);
    if (h) atomicAdd(a.counters + 1, (unsigned long long)h);
  }
}

template <int ST, int LAYOUT, int INTEG, bool GRAD>
static cudaError_t launch_one(const RenderArgs& a, cudaStream_t stream) {
  dim3 grid((a.W + kTileW - 1) / kTileW, (a.H + kTileH - 1) / kTileH);
  raycast_kernel<ST, LAYOUT, INTEG, GRAD><<<grid, kTileW * kTileH, 0, stream>>>(a);
  return cudaGetLastError();
}

template <int ST, int LAYOUT>
static cudaError_t launch_layout(const RenderArgs& a, int integ, bool grad, cudaStream_t s) {
  if (grad) {
    if (integ == VVLIC_EULER) return launch_one<ST, LAYOUT, VVLIC_EULER, true>(a, s);
    if (integ == VVLIC_HEUN) return launch_one<ST, LAYOUT, VVLIC_HEUN, true>(a, s);
    return launch_one<ST, LAYOUT, VVLIC_RK4, true>(a, s);
  }
  if (integ == VVLIC_EULER) return launch_one<ST, LAYOUT, VVLIC_EULER, false>(a, s);
  if (integ == VVLIC_HEUN) return launch_one<ST, LAYOUT, VVLIC_HEUN, false>(a, s);
  return launch_one<ST, LAYOUT, VVLIC_RK4, false>(a, s);
}

}  // namespace vvlic
