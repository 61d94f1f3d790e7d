// Host-visible launch entry points shared between the translation units of libvvlic.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/vvlic.h"

namespace vvlic {

struct RenderArgs;
struct TechArgs;

// Slicing, vector-field DVR, LIC-volume precompute and DVR (techniques_<storage>.cu).
cudaError_t launch_technique_f32(const RenderArgs& a, const TechArgs& t, int sampler, int integ, bool grad,
                                 cudaStream_t s);
cudaError_t launch_technique_f16(const RenderArgs& a, const TechArgs& t, int sampler, int integ, bool grad,
                                 cudaStream_t s);
cudaError_t launch_technique_bf16(const RenderArgs& a, const TechArgs& t, int sampler, int integ, bool grad,
                                  cudaStream_t s);
cudaError_t launch_technique_u8(const RenderArgs& a, const TechArgs& t, int sampler, int integ, bool grad,
                                cudaStream_t s);

// Work distribution of one render launch: `order` == nullptr selects the static raster grid;
// otherwise persistent CTAs pull `ntiles` 8x4 tiles in `order` through the counter `next`.
struct Schedule {
  const uint32_t* order = nullptr;
  int ntiles = 0;
  unsigned* next = nullptr;
  int num_sms = 1;
};

// Forward ray-cast, one launcher per field storage (render_<storage>.cu).
cudaError_t launch_raycast_f32(const RenderArgs& a, int sampler, int integ, bool grad, const Schedule& sch,
                               cudaStream_t s);
cudaError_t launch_raycast_f16(const RenderArgs& a, int sampler, int integ, bool grad, const Schedule& sch,
                               cudaStream_t s);
cudaError_t launch_raycast_bf16(const RenderArgs& a, int sampler, int integ, bool grad, const Schedule& sch,
                                cudaStream_t s);
cudaError_t launch_raycast_u8(const RenderArgs& a, int sampler, int integ, bool grad, const Schedule& sch,
                              cudaStream_t s);

// Adjoint of the unlit (lit == false) or gradient-lit render (adjoint_<storage>.cu):
// accumulates 64-bit fixed-point gradients into acc (TF 1024, opacity 256, taps).
cudaError_t launch_adjoint_f32(const RenderArgs& a, int sampler, int integ, bool lit, const float4* g_img,
                               long long* acc, const Schedule& sch, cudaStream_t s);
cudaError_t launch_adjoint_f16(const RenderArgs& a, int sampler, int integ, bool lit, const float4* g_img,
                               long long* acc, const Schedule& sch, cudaStream_t s);
cudaError_t launch_adjoint_bf16(const RenderArgs& a, int sampler, int integ, bool lit, const float4* g_img,
                                long long* acc, const Schedule& sch, cudaStream_t s);
cudaError_t launch_adjoint_u8(const RenderArgs& a, int sampler, int integ, bool lit, const float4* g_img,
                              long long* acc, const Schedule& sch, cudaStream_t s);

// Batched render (batch_<storage>.cu): one persistent launch over (job, tile) items.
struct BatchLaunch {
  const RenderArgs* jobs;
  const uint2* order;
  int nitems;
  unsigned* next;
  const float* tf;
  unsigned long long* counters;  // [0] samples, [1] rays, [2] sample-steps
  int tw;                        // tile width in pixels (a warp covers tw x 32/tw)
  int num_sms;
};
cudaError_t launch_batch_f32(const BatchLaunch& b, int sampler, int integ, bool grad, cudaStream_t s);
cudaError_t launch_batch_f16(const BatchLaunch& b, int sampler, int integ, bool grad, cudaStream_t s);
cudaError_t launch_batch_bf16(const BatchLaunch& b, int sampler, int integ, bool grad, cudaStream_t s);
cudaError_t launch_batch_u8(const BatchLaunch& b, int sampler, int integ, bool grad, cudaStream_t s);
// Word layout of the batch scratch: job tile starts (njobs+1, padded to an even count), the
// (job, tile) order as 8-byte aligned uint2 pairs, the queue counter.
struct BatchScratch {
  unsigned* start;
  uint2* order;
  unsigned* next;
  size_t words;
};
inline BatchScratch batch_scratch(unsigned* base, int njobs, int ntiles) {
  BatchScratch b;
  const size_t s0 = ((size_t)njobs + 2) & ~(size_t)1;
  b.start = base;
  b.order = base ? reinterpret_cast<uint2*>(base + s0) : nullptr;
  b.next = base ? base + s0 + 2 * (size_t)ntiles : nullptr;
  b.words = s0 + 2 * (size_t)ntiles + 2;
  return b;
}
// Job-major (job, tile) order over a batch (batch.cu); start[] holds njobs+1 entries
// (exclusive prefix of tiles per job).
cudaError_t launch_batch_order(const BatchScratch& b, int njobs, int ntiles, cudaStream_t s);

// Longest-first tile order for the queue schedule (render.cu): per-tile chord cost, a
// counting sort over 1024 cost buckets, scatter.  `scratch` holds 2*ntiles + 2048 + 1 words.
cudaError_t launch_tile_order(const RenderArgs& a, int ntiles, int tiles_x, int shift, unsigned* scratch,
                              cudaStream_t s);

// BRICK sampler (brick.cu): brick shapes and TMA maps for a render of volume v, and its launch.
struct BrickArgs;
struct Volume;
vvlic_status prepare_brick(vvlic_ctx* c, Volume& v, const RenderArgs& a, bool grad, BrickArgs& b);
cudaError_t launch_brick(int storage, const RenderArgs& a, const BrickArgs& b, int integ, bool grad, cudaStream_t s);

// Preprocessing (preprocess.cu, compiled without FMA contraction so results match the
// reference's CPU arithmetic bit for bit).
// Field encoding of fillTexDataFloatInterp into `storage` texels; d_maxbits is a 4-byte
// device scratch word.
cudaError_t launch_encode_field(const void* d_xyz, int dtype, const int n[3], int storage, void* d_texels,
                                unsigned* d_maxbits, cudaStream_t s);
// Time interpolation of two raw vector fields at t = interpIndex / InterpSize.
cudaError_t launch_interp_field(const void* d_a0, const void* d_a1, int dtype, const int n[3], float t, void* d_out,
                                cudaStream_t s);
// Raw noise gradients (float xyz + padding: kNoiseGradBytes per voxel, 16-byte aligned) into
// d_grad, then smoothing + quantisation + pack.
constexpr size_t kNoiseGradBytes = 4 * sizeof(float);
cudaError_t launch_noise_gradients(const uint8_t* d_noise, const int m[3], int mode, const float sd[3],
                                   float* d_grad, uint8_t* d_rgba, const float w27[27], cudaStream_t s);
// Corner-packed cell arrays (see VVLIC_SAMPLER_CELL).
cudaError_t launch_build_field_cells(const void* d_texels, const int n[3], int storage, void* d_cells,
                                     cudaStream_t s);
cudaError_t launch_build_noise_cells(const uint8_t* d_texels, const int m[3], int ch, uint8_t* d_cells,
                                     cudaStream_t s);

// BF16 texels (count RGBA quadruples) -> half-precision RGBA, the format of a BF16 volume's
// texture copy.  Exact for every texel value in [2^-14, 65504]; smaller magnitudes round to the
// nearest half subnormal (absolute error <= 2^-25).
cudaError_t launch_bf16_to_half(const void* d_bf16, size_t count, void* d_half, cudaStream_t s);

// Bytes per texel of a field storage.
inline int texel_bytes(int storage) { return storage == 0 ? 16 : (storage == 3 ? 4 : 8); }

// Storage whose kernel instantiation a launch uses.  Texture-sampled kernels see the field only
// through the texture, whose format is float4 (F32), half4 (F16) or uchar4 (UNORM8); the texture
// of a BF16 volume holds half-precision copies of its BF16 texels, so its TEXTURE and HYBRID
// launches run the F16 instantiations.
inline int kernel_storage(int storage, int sampler) {
  const bool tex = sampler == VVLIC_SAMPLER_TEXTURE || sampler == VVLIC_SAMPLER_HYBRID;
  return (storage == VVLIC_STORAGE_BF16 && tex) ? VVLIC_STORAGE_F16 : storage;
}

}  // namespace vvlic
