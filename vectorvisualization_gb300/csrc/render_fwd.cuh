// Forward LIC ray-cast kernels: one thread per pixel runs the whole lic3d_fragment.glsl main()
// (lic3d_fragment.glsl:5-99).  Two work distributions:
//   * static: one CTA per 16x8 pixel tile in raster order;
//   * queue:  persistent CTAs whose warps pull 8x4 pixel tiles from a device work queue, the
//             tiles pre-ordered longest ray chord first (one atomicAdd per tile, no waiting).
// Instantiated per field storage in render_f32.cu / render_f16.cu / render_bf16.cu /
// render_u8.cu so the translation units compile in parallel.
#pragma once

#include "vvlic_device.cuh"
#include "vvlic_launch.hpp"

namespace vvlic {

constexpr int kTileW = 16, kTileH = 8;  // static schedule: 128 threads, a warp covers 16x2 pixels
constexpr int kWarpTileW = 8, kWarpTileH = 4;  // queue schedule: one warp per 8x4 pixel tile
constexpr int kThreads = 128;
// Minimum resident CTAs per SM requested from the compiler for the render kernels, i.e. a cap
// of 65536 / (kThreads * VVLIC_MIN_BLOCKS) registers per thread.  6 (80 registers, no spills)
// measured 155 Gsample-steps/s on the lit 1024^2 frame against 142 with the compiler's own
// choice; 7 (73 registers, ~60 B spilled) beat 6 on the same GPU by 2 % (lit 1024^2 frame),
// 5 % (the 64-volume batch) and 1 % (the 512^3 RK4 frame); 8 (64 registers) measured as 6.
#ifndef VVLIC_MIN_BLOCKS
#define VVLIC_MIN_BLOCKS 7
#endif
// The same for the RK4 kernels, which hold four slopes per step and trace two samples per pass
// (trace_ray): 4 CTAs, 128 registers.  With one sample per pass, 6 CTAs (80 registers) was
// best: 7 and 8 CTAs spilled and ran 1.5-3 % slower on the 512^3 RK4 orbit frames.
#ifndef VVLIC_RK4_MIN_BLOCKS
#define VVLIC_RK4_MIN_BLOCKS 4
#endif
// Unlit (and line-lit) Euler / Heun kernels: no noise gradients to carry.
#ifndef VVLIC_UNLIT_MIN_BLOCKS
#define VVLIC_UNLIT_MIN_BLOCKS VVLIC_MIN_BLOCKS
#endif
template <int INTEG, bool GRAD> constexpr int min_blocks() {
  return INTEG == VVLIC_RK4 ? VVLIC_RK4_MIN_BLOCKS : (GRAD ? VVLIC_MIN_BLOCKS : VVLIC_UNLIT_MIN_BLOCKS);
}

__device__ __forceinline__ void load_tf(const RenderArgs& a, float* s_tf) {
  for (int i = threadIdx.x; i < 5 * VVLIC_TF_ENTRIES; i += blockDim.x) s_tf[i] = __ldg(a.tf + i);
  __syncthreads();
}

__device__ __forceinline__ void store_pixel(const RenderArgs& a, int px, int py, float4 dest, uint32_t samples) {
  const size_t pix = (size_t)py * a.W + px;
  if (!in_range(a, (long long)pix, (long long)a.W * a.H, VVLIC_CHECK_IMAGE)) return;
  reinterpret_cast<float4*>(a.out)[pix] = dest;
  if (a.samples) a.samples[pix] = samples;
  if (a.tape_n) {
    a.tape_n[pix] = samples;
    if (samples > (uint32_t)a.tape_stride) atomicAdd(a.tape_overflow, 1ull);  // tape too short
  }
}

__device__ __forceinline__ void flush_counters(const RenderArgs& a, uint32_t samples, uint32_t hits) {
  unsigned s = __reduce_add_sync(0xffffffffu, samples);
  unsigned h = __reduce_add_sync(0xffffffffu, hits);
  if ((threadIdx.x & 31) == 0) {
    if (s) atomicAdd(a.counters + 0, (unsigned long long)s);
    if (h) atomicAdd(a.counters + 1, (unsigned long long)h);
  }
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
__global__ void __launch_bounds__(kThreads, min_blocks<INTEG, GRAD>()) raycast_kernel(const __grid_constant__ RenderArgs a) {
  __shared__ __align__(16) float s_tf[5 * VVLIC_TF_ENTRIES];
  load_tf(a, s_tf);
  const int px = blockIdx.x * kTileW + (threadIdx.x % kTileW);
  const int py = blockIdx.y * kTileH + (threadIdx.x / kTileW);
  uint32_t samples = 0, hit = 0;
  if (px < a.W && py < a.H) {
    float4 dest = trace_ray<ST, FL, NL, INTEG, GRAD>(a, s_tf, px, py, samples, hit);
    store_pixel(a, px, py, dest, samples);
  }
  flush_counters(a, samples, hit);
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
__global__ void __launch_bounds__(kThreads, min_blocks<INTEG, GRAD>()) raycast_queue_kernel(const __grid_constant__ RenderArgs a,
                                                                 const uint32_t* __restrict__ order, int ntiles,
                                                                 unsigned* __restrict__ next) {
  __shared__ __align__(16) float s_tf[5 * VVLIC_TF_ENTRIES];
  load_tf(a, s_tf);
  const int lane = threadIdx.x & 31;
  const int tiles_x = (a.W + kWarpTileW - 1) / kWarpTileW;
  uint32_t samples_acc = 0, hits_acc = 0;
  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(next, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= (unsigned)ntiles) break;
    const unsigned tile = __ldg(order + t);
    const int px = (int)(tile % tiles_x) * kWarpTileW + (lane & (kWarpTileW - 1));
    const int py = (int)(tile / tiles_x) * kWarpTileH + (lane / kWarpTileW);
    if (px < a.W && py < a.H) {
      uint32_t samples, hit;
      float4 dest = trace_ray<ST, FL, NL, INTEG, GRAD>(a, s_tf, px, py, samples, hit);
      store_pixel(a, px, py, dest, samples);
      samples_acc += samples;
      hits_acc += hit;
    }
  }
  flush_counters(a, samples_acc, hits_acc);
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
static cudaError_t launch_one(const RenderArgs& a, const Schedule& sch, cudaStream_t stream) {
  if (!sch.order) {
    dim3 grid((a.W + kTileW - 1) / kTileW, (a.H + kTileH - 1) / kTileH);
    raycast_kernel<ST, FL, NL, INTEG, GRAD><<<grid, kThreads, 0, stream>>>(a);
    return cudaGetLastError();
  }
  auto kern = raycast_queue_kernel<ST, FL, NL, INTEG, GRAD>;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, 0);
  if (e != cudaSuccess) return e;
  const int grid = std::max(1, per_sm) * sch.num_sms;
  kern<<<grid, kThreads, 0, stream>>>(a, sch.order, sch.ntiles, sch.next);
  return cudaGetLastError();
}

template <int ST, int FL, int NL>
static cudaError_t launch_layout(const RenderArgs& a, int integ, bool grad, const Schedule& sch, cudaStream_t s) {
  if (grad) {
    if (integ == VVLIC_EULER) return launch_one<ST, FL, NL, VVLIC_EULER, true>(a, sch, s);
    if (integ == VVLIC_HEUN) return launch_one<ST, FL, NL, VVLIC_HEUN, true>(a, sch, s);
    return launch_one<ST, FL, NL, VVLIC_RK4, true>(a, sch, s);
  }
  if (integ == VVLIC_EULER) return launch_one<ST, FL, NL, VVLIC_EULER, false>(a, sch, s);
  if (integ == VVLIC_HEUN) return launch_one<ST, FL, NL, VVLIC_HEUN, false>(a, sch, s);
  return launch_one<ST, FL, NL, VVLIC_RK4, false>(a, sch, s);
}

// Sampler (VVLIC_SAMPLER_*) -> (field layout, noise layout).
template <int ST>
static cudaError_t launch_storage(const RenderArgs& a, int sampler, int integ, bool grad, const Schedule& sch,
                                  cudaStream_t s) {
  switch (sampler) {
    case VVLIC_SAMPLER_GATHER: return launch_layout<ST, kGather, kGather>(a, integ, grad, sch, s);
    case VVLIC_SAMPLER_CELL: return launch_layout<ST, kCell, kCell>(a, integ, grad, sch, s);
    case VVLIC_SAMPLER_TEXTURE:
      if constexpr (ST == VVLIC_STORAGE_BF16) return cudaErrorNotSupported;  // runs as F16 (kernel_storage)
      else return launch_layout<ST, kTexture, kTexture>(a, integ, grad, sch, s);
    case VVLIC_SAMPLER_HYBRID:
      if constexpr (ST == VVLIC_STORAGE_BF16) return cudaErrorNotSupported;
      else return launch_layout<ST, kTexture, kCellFast>(a, integ, grad, sch, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vvlic
