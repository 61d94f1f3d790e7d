// Batched LIC ray-cast: many render jobs (volume x view x image, each with its own LIC
// parameters and filter) in one persistent launch.  Warps pull (job, tile) items from one
// device work queue in job-major order (batch.cu); on a job switch a warp copies that
// job's argument block into its own shared-memory slot and traces the tile from there.  The
// transfer function is the context's and is shared by every job.
#pragma once

#include "render_fwd.cuh"

namespace vvlic {

constexpr int kWarpsPerCta = kThreads / 32;

// Register cap of the unlit Euler / Heun batch kernels, whose arguments come from shared memory
// rather than the constant bank.  On the 64-volume unlit batch: 8 CTAs/SM (64 registers) 1253 ms,
// 7 1283 ms, 6 1326 ms.  (The single-render unlit kernels measured best at 7: 27.5 ms against
// 29.7 at 8 and 33.5 at 9 on the 128^3 4-view forward.)
#ifndef VVLIC_BATCH_UNLIT_MIN_BLOCKS
#define VVLIC_BATCH_UNLIT_MIN_BLOCKS 8
#endif
template <int INTEG, bool GRAD> constexpr int batch_min_blocks() {
  return (!GRAD && INTEG != VVLIC_RK4) ? VVLIC_BATCH_UNLIT_MIN_BLOCKS : min_blocks<INTEG, GRAD>();
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
__global__ void __launch_bounds__(kThreads, batch_min_blocks<INTEG, GRAD>())
    raycast_batch_kernel(const RenderArgs* __restrict__ jobs, const uint2* __restrict__ order, int nitems,
                         unsigned* __restrict__ next, const float* __restrict__ tf, unsigned long long* counters,
                         int tw) {
  __shared__ __align__(16) float s_tf[5 * VVLIC_TF_ENTRIES];
  __shared__ __align__(16) RenderArgs s_args[kWarpsPerCta];
  for (int i = threadIdx.x; i < 5 * VVLIC_TF_ENTRIES; i += blockDim.x) s_tf[i] = __ldg(tf + i);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  RenderArgs& a = s_args[warp];
  const int th = 32 / tw;
  unsigned cur = 0xffffffffu;
  uint32_t samples_acc = 0, hits_acc = 0;
  unsigned long long steps_acc = 0;
  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(next, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= (unsigned)nitems) break;
    const uint2 item = __ldg(order + t);
    if (item.x != cur) {  // load the job's argument block into this warp's slot
      const uint32_t* src = reinterpret_cast<const uint32_t*>(jobs + item.x);
      uint32_t* dst = reinterpret_cast<uint32_t*>(&a);
      for (int i = lane; i < (int)(sizeof(RenderArgs) / 4); i += 32) dst[i] = __ldg(src + i);
      __syncwarp();
      cur = item.x;
    }
    const int tiles_x = (a.W + tw - 1) / tw;
    const int px = (int)(item.y % tiles_x) * tw + lane % tw;
    const int py = (int)(item.y / tiles_x) * th + lane / tw;
    if (px < a.W && py < a.H) {
      uint32_t samples, hit;
      float4 dest = trace_ray<ST, FL, NL, INTEG, GRAD>(a, s_tf, px, py, samples, hit);
      store_pixel(a, px, py, dest, samples);
      samples_acc += samples;
      hits_acc += hit;
      steps_acc += (unsigned long long)samples * (a.lb + a.lf);
    }
  }
  unsigned s = __reduce_add_sync(0xffffffffu, samples_acc);
  unsigned h = __reduce_add_sync(0xffffffffu, hits_acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) steps_acc += __shfl_xor_sync(0xffffffffu, steps_acc, o);
  if (lane == 0) {
    if (s) atomicAdd(counters + 0, (unsigned long long)s);
    if (h) atomicAdd(counters + 1, (unsigned long long)h);
    if (steps_acc) atomicAdd(counters + 2, steps_acc);
  }
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
static cudaError_t launch_batch_one(const BatchLaunch& b, cudaStream_t s) {
  auto kern = raycast_batch_kernel<ST, FL, NL, INTEG, GRAD>;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, 0);
  if (e != cudaSuccess) return e;
  kern<<<std::max(1, per_sm) * b.num_sms, kThreads, 0, s>>>(b.jobs, b.order, b.nitems, b.next, b.tf, b.counters, b.tw);
  return cudaGetLastError();
}

template <int ST, int FL, int NL>
static cudaError_t launch_batch_layout(const BatchLaunch& b, int integ, bool grad, cudaStream_t s) {
  if (grad) {
    if (integ == VVLIC_EULER) return launch_batch_one<ST, FL, NL, VVLIC_EULER, true>(b, s);
    if (integ == VVLIC_HEUN) return launch_batch_one<ST, FL, NL, VVLIC_HEUN, true>(b, s);
    return launch_batch_one<ST, FL, NL, VVLIC_RK4, true>(b, s);
  }
  if (integ == VVLIC_EULER) return launch_batch_one<ST, FL, NL, VVLIC_EULER, false>(b, s);
  if (integ == VVLIC_HEUN) return launch_batch_one<ST, FL, NL, VVLIC_HEUN, false>(b, s);
  return launch_batch_one<ST, FL, NL, VVLIC_RK4, false>(b, s);
}

template <int ST>
static cudaError_t launch_batch_storage(const BatchLaunch& b, int sampler, int integ, bool grad, cudaStream_t s) {
  switch (sampler) {
    case VVLIC_SAMPLER_GATHER: return launch_batch_layout<ST, kGather, kGather>(b, integ, grad, s);
    case VVLIC_SAMPLER_CELL: return launch_batch_layout<ST, kCell, kCell>(b, integ, grad, s);
    case VVLIC_SAMPLER_TEXTURE:
      if constexpr (ST == VVLIC_STORAGE_BF16) return cudaErrorNotSupported;  // runs as F16 (kernel_storage)
      else return launch_batch_layout<ST, kTexture, kTexture>(b, integ, grad, s);
    case VVLIC_SAMPLER_HYBRID:
      if constexpr (ST == VVLIC_STORAGE_BF16) return cudaErrorNotSupported;
      else return launch_batch_layout<ST, kTexture, kCellFast>(b, integ, grad, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vvlic
