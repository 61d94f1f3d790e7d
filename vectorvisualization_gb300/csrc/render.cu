// Render entry points: uniform derivation (Renderer::setRenderVolParams, renderer.cpp:925-996),
// lazy construction of the field/noise layouts the chosen sampler reads, and the launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstring>
#include <thread>

#include "../../include/vvlic.h"
#include "brick.cuh"
#include "vvlic_device.cuh"
#include "vvlic_host.hpp"
#include "vvlic_launch.hpp"

using namespace vvlic;

namespace {

vvlic_status ensure_cells(vvlic_ctx* c, Volume& v, cudaStream_t s) {
  if (v.d_cells) return VVLIC_OK;
  const size_t cells = (size_t)(v.n[0] + 1) * (v.n[1] + 1) * (v.n[2] + 1);
  const size_t bytes = cells * 8 * texel_bytes(v.storage);
  cudaError_t e = cudaMalloc(&v.d_cells, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "cell layout allocation");
  v.cell_bytes = bytes;
  e = launch_build_field_cells(v.d_texels, v.n, v.storage, v.d_cells, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "cell layout build");
  return VVLIC_OK;
}

vvlic_status ensure_noise_cells(vvlic_ctx* c, NoiseTex& n, cudaStream_t s) {
  if (n.d_cells) return VVLIC_OK;
  const size_t bytes = noise_cell_count(n.m) * 8 * n.ch;
  cudaError_t e = cudaMalloc(&n.d_cells, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise cell allocation");
  e = launch_build_noise_cells(n.d_texels, n.m, n.ch, n.d_cells, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise cell build");
  return VVLIC_OK;
}

// Copies the volume's texels into its texture array (allocated by ensure_texture).  The texture
// unit has no bf16 format: a BF16 volume's texture is a half4 array holding its BF16 texels
// converted to half (exact for the encoded texels, all in [0, 1], down to 2^-14).
vvlic_status copy_field_texture(vvlic_ctx* c, Volume& v, cudaStream_t s) {
  const bool bf16 = v.storage == VVLIC_STORAGE_BF16;
  const size_t tb = texel_bytes(v.storage);  // 8 bytes for F16, BF16 and their half4 copy alike
  const size_t count = (size_t)v.n[0] * v.n[1] * v.n[2];
  void* src = v.d_texels;
  cudaError_t e;
  if (bf16) {
    // stream-ordered scratch: freed behind the array copy that reads it
    e = cudaMallocAsync(&src, count * tb, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "BF16 texture staging allocation");
    e = launch_bf16_to_half(v.d_texels, count, src, s);
    if (e != cudaSuccess) {
      cudaFreeAsync(src, s);
      return cuda_fail(c, e, "BF16 texture conversion");
    }
  }
  cudaMemcpy3DParms cp;
  std::memset(&cp, 0, sizeof cp);
  cp.srcPtr = make_cudaPitchedPtr(src, v.n[0] * tb, v.n[0], v.n[1]);
  cp.dstArray = v.array;
  cp.extent = make_cudaExtent(v.n[0], v.n[1], v.n[2]);
  cp.kind = cudaMemcpyDeviceToDevice;
  e = cudaMemcpy3DAsync(&cp, s);
  if (bf16) {
    cudaError_t ef = cudaFreeAsync(src, s);
    if (e == cudaSuccess) e = ef;
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "texture array copy");
  return VVLIC_OK;
}

vvlic_status ensure_texture(vvlic_ctx* c, Volume& v, cudaStream_t s) {
  if (v.tex) return VVLIC_OK;
  const bool bf16 = v.storage == VVLIC_STORAGE_BF16;
  cudaChannelFormatDesc desc = v.storage == VVLIC_STORAGE_F32 ? cudaCreateChannelDesc<float4>()
                               : (v.storage == VVLIC_STORAGE_F16 || bf16) ? cudaCreateChannelDescHalf4()
                                                                          : cudaCreateChannelDesc<uchar4>();
  cudaExtent ext = make_cudaExtent(v.n[0], v.n[1], v.n[2]);
  cudaError_t e = cudaMalloc3DArray(&v.array, &desc, ext);
  if (e != cudaSuccess) return cuda_fail(c, e, "texture array allocation");
  v.array_bytes = (size_t)v.n[0] * v.n[1] * v.n[2] * texel_bytes(v.storage);
  vvlic_status st = copy_field_texture(c, v, s);
  if (st) return st;
  cudaResourceDesc rd;
  std::memset(&rd, 0, sizeof rd);
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = v.array;
  cudaTextureDesc td;
  std::memset(&td, 0, sizeof td);
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;  // CLAMP_TO_EDGE
  td.filterMode = cudaFilterModeLinear;
  td.readMode = v.storage == VVLIC_STORAGE_UNORM8 ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
  td.normalizedCoords = 1;  // GL texture coordinates
  e = cudaCreateTextureObject(&v.tex, &rd, &td, nullptr);
  if (e != cudaSuccess) return cuda_fail(c, e, "texture object");
  return VVLIC_OK;
}

// Noise as an R8 / RGBA8 texture read as normalised float with WRAP addressing (GL REPEAT).
vvlic_status copy_noise_texture(vvlic_ctx* c, NoiseTex& n, cudaStream_t s) {
  cudaMemcpy3DParms cp;
  std::memset(&cp, 0, sizeof cp);
  cp.srcPtr = make_cudaPitchedPtr(n.d_texels, (size_t)n.m[0] * n.ch, n.m[0], n.m[1]);
  cp.dstArray = n.array;
  cp.extent = make_cudaExtent(n.m[0], n.m[1], n.m[2]);
  cp.kind = cudaMemcpyDeviceToDevice;
  cudaError_t e = cudaMemcpy3DAsync(&cp, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise texture copy");
  return VVLIC_OK;
}

vvlic_status ensure_noise_texture(vvlic_ctx* c, NoiseTex& n, cudaStream_t s) {
  if (n.tex) return VVLIC_OK;
  cudaChannelFormatDesc desc =
      n.ch == 4 ? cudaCreateChannelDesc<uchar4>() : cudaCreateChannelDesc<unsigned char>();
  cudaExtent ext = make_cudaExtent(n.m[0], n.m[1], n.m[2]);
  cudaError_t e = cudaMalloc3DArray(&n.array, &desc, ext);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise texture allocation");
  vvlic_status st = copy_noise_texture(c, n, s);
  if (st) return st;
  cudaResourceDesc rd;
  std::memset(&rd, 0, sizeof rd);
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = n.array;
  cudaTextureDesc td;
  std::memset(&td, 0, sizeof td);
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeWrap;
  td.filterMode = cudaFilterModeLinear;
  td.readMode = cudaReadModeNormalizedFloat;
  td.normalizedCoords = 1;
  e = cudaCreateTextureObject(&n.tex, &rd, &td, nullptr);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise texture object");
  return VVLIC_OK;
}

}  // namespace

namespace vvlic {

vvlic_status refresh_volume_layouts(vvlic_ctx* c, Volume& v, cudaStream_t s) {
  if (v.d_cells) {
    cudaError_t e = launch_build_field_cells(v.d_texels, v.n, v.storage, v.d_cells, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "cell layout rebuild");
  }
  if (v.array) return copy_field_texture(c, v, s);
  return VVLIC_OK;
}

vvlic_status refresh_noise_layouts(vvlic_ctx* c, NoiseTex& n, cudaStream_t s) {
  if (n.d_cells) {
    cudaError_t e = launch_build_noise_cells(n.d_texels, n.m, n.ch, n.d_cells, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "noise cell rebuild");
  }
  if (n.array) return copy_noise_texture(c, n, s);
  return VVLIC_OK;
}

// Fill the kernel argument block for one volume and image size.
vvlic_status build_render_args(vvlic_ctx* c, Volume& v, int W, int H, cudaStream_t s, RenderArgs& a) {
  return build_render_args_ex(c, v, W, H, s, c->params, c->view, nullptr, a);
}

vvlic_status build_render_args_ex(vvlic_ctx* c, Volume& v, int W, int H, cudaStream_t s, const vvlic_params& p,
                                  const vvlic_view& view, const JobFilter* filter, RenderArgs& a) {
  std::memset(&a, 0, sizeof a);
  if (!c->noise.d_texels) return fail(c, VVLIC_ERR_NOT_READY, "render: no noise uploaded");
  if (p.illum == VVLIC_ILLUM_GRADIENT && c->noise.ch != 4)
    return fail(c, VVLIC_ERR_NOT_READY, "render: gradient lighting needs noise uploaded with gradients");
  if (p.scalar_gate && !c->d_scalar) return fail(c, VVLIC_ERR_NOT_READY, "render: scalar gate on, no scalar volume");
  int lb = p.low_res ? 15 : p.steps_backward, lf = p.low_res ? 15 : p.steps_forward;
  float inv_area = 0.5f;
  if (filter) {
    derive_taps_from_table(filter->table, filter->width, filter->clamp, filter->is_box, lb, lf, a.taps, &inv_area);
  } else if (derive_taps(c, lb, lf, a.taps, &inv_area)) {
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "render: explicit taps were set for L_b=%d L_f=%d, params have %d/%d",
                c->taps_lb, c->taps_lf, lb, lf);
  }
  vvlic_status st;
  a.n[0] = v.n[0];
  a.n[1] = v.n[1];
  a.n[2] = v.n[2];
  switch (p.sampler) {
    case VVLIC_SAMPLER_GATHER:
    case VVLIC_SAMPLER_BRICK:  // bricks are staged from the texel arrays; fetches outside them gather
      a.field = v.d_texels;
      a.noise = c->noise.d_texels;
      break;
    case VVLIC_SAMPLER_CELL:
      if ((st = ensure_cells(c, v, s))) return st;
      if ((st = ensure_noise_cells(c, c->noise, s))) return st;
      a.field = v.d_cells;
      a.noise = c->noise.d_cells;
      break;
    case VVLIC_SAMPLER_TEXTURE:
      if ((st = ensure_texture(c, v, s))) return st;
      if ((st = ensure_noise_texture(c, c->noise, s))) return st;
      a.tex = v.tex;
      a.noise_tex = c->noise.tex;
      break;
    default:  // HYBRID
      if ((st = ensure_texture(c, v, s))) return st;
      if ((st = ensure_noise_cells(c, c->noise, s))) return st;
      a.tex = v.tex;
      a.noise = c->noise.d_cells;
      break;
  }

  for (int i = 0; i < 3; ++i) {
    a.m[i] = c->noise.m[i];
    a.sn[i] = c->sn[i];
  }
  a.noise_ch = c->noise.ch;
  a.scalar = c->d_scalar;
  a.tf = c->d_tf;
  a.W = W;
  a.H = H;
  double rc[21];
  derive_rays(view, v.geom, W, H, rc);
  for (int i = 0; i < 3; ++i) {
    a.o0[i] = (float)rc[i];
    a.o1[i] = (float)rc[3 + i];
    a.o2[i] = (float)rc[6 + i];
    a.d0[i] = (float)rc[9 + i];
    a.d1[i] = (float)rc[12 + i];
    a.d2[i] = (float)rc[15 + i];
  }
  a.clamp0 = rc[18] != 0.0;
  // scaleVol / scaleVolInv as the shader receives them (renderer.cpp:939-944)
  const bool bug = (p.quirks & VVLIC_QUIRK_UNIFORM_SCALE_BUG) && p.illum != VVLIC_ILLUM_NONE;
  for (int i = 0; i < 3; ++i) {
    a.ext[i] = v.geom.extent[i];
    a.tex_max[i] = v.geom.tex_max[i];
    a.scale_vol[i] = bug ? v.geom.scale_inv[i] : v.geom.scale[i];
    a.scale_vol_inv[i] = bug ? 0.0f : v.geom.scale_inv[i];
  }
  const float h = p.low_res ? 1.0f / 64.0f : p.step_size_lic;
  a.step_size = p.low_res ? 2.0f * p.step_size_vol : p.step_size_vol;
  a.freq_scale = p.low_res ? 0.7f * p.freq_scale : p.freq_scale;
  const bool nofreq = (p.quirks & VVLIC_QUIRK_GRAD_NOISE_NO_FREQ) != 0;
  for (int i = 0; i < 3; ++i) {
    a.nscale[i] = (float)((double)a.freq_scale * a.m[i]);
    a.nscale_grad[i] = nofreq ? (float)a.m[i] : a.nscale[i];
  }
  a.alpha_corr = p.low_res ? 2.0f * p.step_size_vol * 128.0f : p.step_size_vol * 128.0f;
  a.h_eff = h * p.eye_dist_factor;
  a.intensity_scale = inv_area / (float)(lf + lb) * p.gradient_scale;  // licKernel.b * gradient.r
  a.illum_scale = p.illum_scale;
  a.alpha_thr = p.alpha_threshold;
  a.gate_lo = p.gate_lo;
  a.gate_hi = p.gate_hi;
  a.num_iter = p.num_iterations;
  a.lb = lb;
  a.lf = lf;
  a.illum = p.illum;
  a.tf_index = p.tf_index;
  a.sof = p.speed_of_flow;
  a.gate = p.scalar_gate;
  a.quirks = (int)p.quirks;
  a.spec_exp = p.spec_exp;
  for (int i = 0; i < 3; ++i) {
    a.light_pos[i] = p.light_pos[i];
    a.light_diff[i] = p.light_diffuse[i];
    a.light_spec[i] = p.light_specular[i];
    a.light_amb[i] = p.light_ambient[i];
  }
  if (p.illum == VVLIC_ILLUM_ZOECKLER || p.illum == VVLIC_ILLUM_MALLO) {
    if ((st = ensure_illum_luts(c)) != VVLIC_OK) return st;
    a.luts = (const uchar4*)c->d_luts;
    a.lut_w = c->lut_w;
    a.lut_h = c->lut_h;
  }
  a.counters = c->d_counters;
  return VVLIC_OK;
}

cudaError_t launch_technique(int storage, const RenderArgs& a, const TechArgs& t, int sampler, int integ, bool grad,
                             cudaStream_t s) {
  switch (kernel_storage(storage, sampler)) {
    case VVLIC_STORAGE_F32: return launch_technique_f32(a, t, sampler, integ, grad, s);
    case VVLIC_STORAGE_F16: return launch_technique_f16(a, t, sampler, integ, grad, s);
    case VVLIC_STORAGE_UNORM8: return launch_technique_u8(a, t, sampler, integ, grad, s);
    default: return launch_technique_bf16(a, t, sampler, integ, grad, s);
  }
}

cudaError_t launch_raycast(const RenderArgs& a, int storage, int sampler, int integ, bool grad, const Schedule& sch,
                           cudaStream_t s) {
  switch (kernel_storage(storage, sampler)) {
    case VVLIC_STORAGE_F32: return launch_raycast_f32(a, sampler, integ, grad, sch, s);
    case VVLIC_STORAGE_F16: return launch_raycast_f16(a, sampler, integ, grad, sch, s);
    case VVLIC_STORAGE_UNORM8: return launch_raycast_u8(a, sampler, integ, grad, sch, s);
    default: return launch_raycast_bf16(a, sampler, integ, grad, sch, s);
  }
}

// ------------------------------------------------------------------------------------------
// longest-first tile order for the queue schedule
// ------------------------------------------------------------------------------------------
namespace {

constexpr int kBuckets = 1024;

// One warp per 8x4 tile: the tile's cost is its longest ray's sample count (the warp runs until
// that ray finishes), estimated from the ray-box chord: samples ~ chord / spacing + 1.
__global__ void tile_cost_kernel(const __grid_constant__ RenderArgs a, int ntiles, int tiles_x, int shift,
                                 unsigned* bucket, unsigned* hist) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < ntiles; t += warps) {
    const int px = (t % tiles_x) * 8 + (lane & 7), py = (t / tiles_x) * 4 + (lane >> 3);
    unsigned cost = 0;
    float o[3], d[3], tn, tf;
    if (px < a.W && py < a.H && ray_interval(a, px, py, o, d, tn, tf)) {
      const float len = (tf - tn) * sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      cost = (unsigned)fminf(len / a.step_size + 1.0f, 4.0e9f);
    }
    cost = __reduce_max_sync(0xffffffffu, cost);
    if (lane == 0) {
      const unsigned b = kBuckets - 1 - min(cost >> shift, (unsigned)(kBuckets - 1));  // descending
      bucket[t] = b;
      atomicAdd(hist + b, 1u);
    }
  }
}

// Exclusive scan of the bucket histogram into start offsets (one CTA of kBuckets threads).
__global__ void bucket_scan_kernel(const unsigned* hist, unsigned* offsets) {
  __shared__ unsigned s[kBuckets];
  const int i = threadIdx.x;
  s[i] = hist[i];
  __syncthreads();
  for (int d = 1; d < kBuckets; d <<= 1) {
    unsigned v = i >= d ? s[i - d] : 0u;
    __syncthreads();
    s[i] += v;
    __syncthreads();
  }
  offsets[i] = s[i] - hist[i];
}

__global__ void tile_scatter_kernel(int ntiles, const unsigned* bucket, unsigned* offsets, unsigned* order) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x)
    order[atomicAdd(offsets + bucket[t], 1u)] = (unsigned)t;
}

}  // namespace

cudaError_t launch_tile_order(const RenderArgs& a, int ntiles, int tiles_x, int shift, unsigned* scratch,
                              cudaStream_t s) {
  unsigned* bucket = scratch;
  unsigned* order = scratch + ntiles;
  unsigned* hist = scratch + 2 * (size_t)ntiles;
  unsigned* offsets = hist + kBuckets;
  cudaError_t e = cudaMemsetAsync(hist, 0, kBuckets * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  const int warps_per_block = 8;
  const int blocks = std::min((ntiles + warps_per_block - 1) / warps_per_block, 152 * 16);
  tile_cost_kernel<<<blocks, 32 * warps_per_block, 0, s>>>(a, ntiles, tiles_x, shift, bucket, hist);
  bucket_scan_kernel<<<1, kBuckets, 0, s>>>(hist, offsets);
  tile_scatter_kernel<<<std::min((ntiles + 255) / 256, 152 * 8), 256, 0, s>>>(ntiles, bucket, offsets, order);
  return cudaGetLastError();
}

}  // namespace vvlic

namespace {

// Queue schedule for one image: longest-first tile order in the context's scratch.
vvlic_status make_schedule(vvlic_ctx* c, const RenderArgs& a, const Geometry& gm, int w, int h, cudaStream_t s,
                           Schedule& sch) {
  const int tiles_x = (w + 7) / 8, ntiles = tiles_x * ((h + 3) / 4);
  const size_t words = 2 * (size_t)ntiles + 2 * 1024 + 1;
  if (c->sched_cap < words) {
    if (c->d_sched) cudaFree(c->d_sched);
    c->d_sched = nullptr;
    c->sched_cap = 0;
    cudaError_t e = cudaMalloc(&c->d_sched, words * sizeof(unsigned));
    if (e != cudaSuccess) return cuda_fail(c, e, "schedule allocation");
    c->sched_cap = words;
  }
  // cost buckets of 2^shift samples so the longest possible chord fits 1024 buckets
  const double diag = std::sqrt((double)gm.extent[0] * gm.extent[0] + (double)gm.extent[1] * gm.extent[1] +
                                (double)gm.extent[2] * gm.extent[2]);
  const double maxcost = diag / a.step_size + 2.0;
  int shift = 0;
  while ((maxcost / (double)(1u << shift)) >= 1024.0 && shift < 31) ++shift;
  unsigned* scratch = c->d_sched;
  cudaError_t e = launch_tile_order(a, ntiles, tiles_x, shift, scratch, s);
  sch.order = scratch + ntiles;
  sch.ntiles = ntiles;
  sch.next = scratch + 2 * (size_t)ntiles + 2 * 1024;
  if (e == cudaSuccess) e = cudaMemsetAsync(sch.next, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return cuda_fail(c, e, "schedule");
  return VVLIC_OK;
}

// Tape buffers for a recording render: per ray `stride` samples (the longest march / spacing,
// capped by the two loop bounds) and a checkpoint every kSegment samples.  A ray marches in
// texture space through [0, tex_max] by step_size * |normalize(d) * scaleVol| per sample, and
// that step is at least step_size * min(scaleVol): the bound holds whatever scaleVol the
// shader receives (with VVLIC_QUIRK_UNIFORM_SCALE_BUG it is scaleInv, and rays run past the
// object box until they leave [0, tex_max]).
vvlic_status prepare_tape(vvlic_ctx* c, int w, int h, RenderArgs& a, cudaStream_t s) {
  const double diag = std::sqrt((double)a.tex_max[0] * a.tex_max[0] + (double)a.tex_max[1] * a.tex_max[1] +
                                (double)a.tex_max[2] * a.tex_max[2]);
  const double min_sv = std::max(1e-6, (double)std::min(std::min(a.scale_vol[0], a.scale_vol[1]), a.scale_vol[2]));
  double bound = std::min(diag / (a.step_size * min_sv) + 3.0, (double)a.num_iter * (double)a.num_iter);
  if (c->params.tape_max_samples > 0) bound = std::min(bound, (double)c->params.tape_max_samples);
  const int stride = std::max(1, (int)std::ceil(bound));
  const int nck = (stride + kSegment - 1) / kSegment;
  const size_t rays = (size_t)w * h;
  // per-sample arrays in 8x4-ray tiles (tape_entry / tape_ck_entry), edge tiles padded
  const size_t slots = (size_t)((w + 7) / 8) * (size_t)((h + 3) / 4) * 32;
  const bool lit = a.illum == VVLIC_ILLUM_GRADIENT;
  const size_t b_is = slots * stride * sizeof(float2), b_ck = slots * nck * 2 * sizeof(float4),
               b_g = lit ? slots * stride * sizeof(uint2) : 0, b_n = rays * sizeof(uint32_t);
  const size_t bytes = b_ck + b_is + b_g + b_n;
  if (c->tape_cap < bytes) {
    if (c->d_tape) cudaFree(c->d_tape);
    c->d_tape = nullptr;
    c->tape_cap = 0;
    cudaError_t e = cudaMalloc(&c->d_tape, bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint tape allocation");
    c->tape_cap = bytes;
  }
  if (!c->d_tape_flag) {
    cudaError_t e = cudaMalloc(&c->d_tape_flag, sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint tape flag");
  }
  char* base = (char*)c->d_tape;
  a.tape_ck = (float4*)base;
  a.tape_is = (float2*)(base + b_ck);
  a.tape_g = lit ? (uint2*)(base + b_ck + b_is) : nullptr;
  a.tape_n = (uint32_t*)(base + b_ck + b_is + b_g);
  a.tape_overflow = c->d_tape_flag;
  a.tape_stride = stride;
  a.tape_nck = nck;
  cudaError_t e = cudaMemsetAsync(c->d_tape_flag, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return cuda_fail(c, e, "adjoint tape flag");
  return VVLIC_OK;
}

}  // namespace

extern "C" vvlic_status vvlic_render_device(vvlic_ctx* c, int32_t vol_id, float* d_out, int32_t w, int32_t h,
                                           uint32_t* d_samples, void* stream) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  auto it = c->vols.find(vol_id);
  if (it == c->vols.end()) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "render: unknown volume %d", vol_id);
  if (!d_out || w < 1 || h < 1 || w > 32768 || h > 32768)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "render: bad image arguments");
  DeviceGuard g(c->device);
  cudaStream_t s = (cudaStream_t)stream;
  RenderArgs a;
  vvlic_status st = build_render_args(c, it->second, w, h, s, a);
  if (st) return st;
  a.out = d_out;
  a.samples = d_samples;
  if (c->params.sampler == VVLIC_SAMPLER_BRICK &&
      (c->params.technique != VVLIC_TECHNIQUE_RAYCAST || c->params.record_tape))
    return fail(c, VVLIC_ERR_UNSUPPORTED, "render: the BRICK sampler renders the RAYCAST technique without a tape");
  if (c->params.technique != VVLIC_TECHNIQUE_RAYCAST) {
    if (c->params.record_tape)
      return fail(c, VVLIC_ERR_UNSUPPORTED, "render: the adjoint tape is recorded by the RAYCAST technique only");
    TechArgs t;
    std::memset(&t, 0, sizeof t);
    t.technique = c->params.technique;
    const Volume& v = it->second;
    if (t.technique == VVLIC_TECHNIQUE_SLICING) {
      derive_slicing(c->view, v.geom, a.step_size, t.v, &t.depth, &t.nslices);
      for (int i = 0; i < 3; ++i) t.c[i] = v.geom.center[i];
    } else if (t.technique == VVLIC_TECHNIQUE_LICVOLUME) {
      if (!v.d_licvol || !v.licvol_valid)
        return fail(c, VVLIC_ERR_NOT_READY, "render: LICVOLUME needs vvlic_compute_lic_volume for volume %d", vol_id);
      t.licvol = v.d_licvol;
      for (int i = 0; i < 3; ++i) t.ln[i] = v.ln[i];
      a.illum = VVLIC_ILLUM_NONE;  // raycast_lic3d_fragment.glsl shades with illumLIC
    }
    cudaError_t e = cudaMemsetAsync(c->d_counters, 0, 4 * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev0, s);
    if (e == cudaSuccess)
      e = launch_technique(v.storage, a, t, c->params.sampler, c->params.integrator,
                           c->params.illum == VVLIC_ILLUM_GRADIENT && t.technique == VVLIC_TECHNIQUE_SLICING, s);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev1, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "render launch");
    c->stats_pending = true;
    c->last_was_batch = false;
    c->tape_flag_pending = false;
    c->stats_steps_per_sample = t.technique == VVLIC_TECHNIQUE_SLICING ? (uint64_t)(a.lb + a.lf) : 0;
    return VVLIC_OK;
  }
  const bool record = c->params.record_tape != 0;
  if (record) {
    c->tape_valid = false;
    if ((st = prepare_tape(c, w, h, a, s))) return st;
  }
  Schedule sch;
  sch.num_sms = c->num_sms;
  const bool grad = c->params.illum == VVLIC_ILLUM_GRADIENT;
  const bool brick = c->params.sampler == VVLIC_SAMPLER_BRICK;
  BrickArgs bargs;
  if (brick && (st = prepare_brick(c, it->second, a, grad, bargs))) return st;
  cudaError_t e = cudaMemsetAsync(c->d_counters, 0, 4 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return cuda_fail(c, e, "render");
  if (!brick && c->params.schedule == VVLIC_SCHEDULE_QUEUE && (st = make_schedule(c, a, it->second.geom, w, h, s, sch)))
    return st;
  e = cudaEventRecord(c->ev0, s);
  if (e == cudaSuccess)
    e = brick ? launch_brick(it->second.storage, a, bargs, c->params.integrator, grad, s)
              : launch_raycast(a, it->second.storage, c->params.sampler, c->params.integrator, grad, sch, s);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev1, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "render launch");
  c->stats_pending = true;
  c->last_was_batch = false;
  c->stats.sample_steps = 0;
  c->stats_steps_per_sample = (uint64_t)(a.lb + a.lf);
  c->tape_flag_pending = record;
  if (record) {
    c->tape_valid = true;
    c->tape_vol = vol_id;
    c->tape_w = w;
    c->tape_h = h;
    c->tape_storage = it->second.storage;
    c->tape_sampler = c->params.sampler;
    c->tape_integ = c->params.integrator;
    c->tape_illum = c->params.illum;
    c->tape_args = a;
  }
  return VVLIC_OK;
}

namespace vvlic_adjoint_out {

__global__ void fixed_to_float_kernel(const long long* acc, int n_tf, int n_op, int n_taps, float* tf, float* op,
                                      float* taps, const unsigned long long* overflow) {
  const float nan = __int_as_float(0x7fc00000);
  const bool bad = *overflow != 0;
  const double k = 1.0 / 1073741824.0;  // 2^-30
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_tf + n_op + n_taps; i += gridDim.x * blockDim.x) {
    const float v = bad ? nan : (float)((double)acc[i] * k);
    if (i < n_tf) {
      if (tf) tf[i] = v;
    } else if (i < n_tf + n_op) {
      if (op) op[i - n_tf] = v;
    } else if (taps) {
      taps[i - n_tf - n_op] = v;
    }
  }
}

}  // namespace vvlic_adjoint_out

extern "C" vvlic_status vvlic_render_adjoint(vvlic_ctx* c, int32_t vol_id, const float* d_dl_drgba, int32_t w,
                                            int32_t h, float* d_dl_dtf, float* d_dl_dopacity, float* d_dl_dtaps,
                                            void* stream) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!d_dl_drgba) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "render_adjoint: null cotangent");
  if (!c->tape_valid || c->tape_vol != vol_id || c->tape_w != w || c->tape_h != h)
    return fail(c, VVLIC_ERR_NOT_READY,
                "render_adjoint: the last render of this context did not record a tape for volume %d at %dx%d "
                "(set params.record_tape)", vol_id, w, h);
  if (c->vols.find(vol_id) == c->vols.end())
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "render_adjoint: unknown volume %d", vol_id);
  DeviceGuard g(c->device);
  cudaStream_t s = (cudaStream_t)stream;
  const int acc_size = 5 * VVLIC_TF_ENTRIES + kMaxTaps;
  cudaError_t e = cudaSuccess;
  if (!c->d_acc) {
    e = cudaMalloc(&c->d_acc, acc_size * sizeof(long long));
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint accumulators");
  }
  e = cudaMemsetAsync(c->d_acc, 0, acc_size * sizeof(long long), s);
  if (e != cudaSuccess) return cuda_fail(c, e, "adjoint");
  const RenderArgs& a = c->tape_args;
  Schedule sch;
  sch.num_sms = c->num_sms;
  auto vt = c->vols.find(vol_id);
  if (vt == c->vols.end()) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "render_adjoint: unknown volume %d", vol_id);
  vvlic_status st = make_schedule(c, a, vt->second.geom, w, h, s, sch);
  if (st) return st;
  e = cudaEventRecord(c->ev0, s);
  const float4* gi = (const float4*)d_dl_drgba;
  if (e == cudaSuccess) {
    const bool lit = c->tape_illum == VVLIC_ILLUM_GRADIENT;
    switch (kernel_storage(c->tape_storage, c->tape_sampler)) {
      case VVLIC_STORAGE_F32: e = launch_adjoint_f32(a, c->tape_sampler, c->tape_integ, lit, gi, c->d_acc, sch, s); break;
      case VVLIC_STORAGE_F16: e = launch_adjoint_f16(a, c->tape_sampler, c->tape_integ, lit, gi, c->d_acc, sch, s); break;
      case VVLIC_STORAGE_UNORM8:
        e = launch_adjoint_u8(a, c->tape_sampler, c->tape_integ, lit, gi, c->d_acc, sch, s);
        break;
      default: e = launch_adjoint_bf16(a, c->tape_sampler, c->tape_integ, lit, gi, c->d_acc, sch, s); break;
    }
  }
  if (e == cudaSuccess) e = cudaEventRecord(c->ev1, s);
  if (e == cudaSuccess) {
    const int n_taps = a.lb + a.lf + 1;
    vvlic_adjoint_out::fixed_to_float_kernel<<<8, 256, 0, s>>>(c->d_acc, 4 * VVLIC_TF_ENTRIES, VVLIC_TF_ENTRIES, n_taps, d_dl_dtf,
                                            d_dl_dopacity, d_dl_dtaps, c->d_tape_flag);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "render_adjoint launch");
  c->stats_pending = true;
  c->tape_flag_pending = true;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_render(vvlic_ctx* c, int32_t vol_id, float* out, int32_t w, int32_t h) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!out || w < 1 || h < 1 || w > 32768 || h > 32768)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "render: bad image arguments");
  DeviceGuard g(c->device);
  const size_t bytes = (size_t)w * h * 4 * sizeof(float);
  if (c->image_cap < bytes) {
    if (c->d_image) cudaFree(c->d_image);
    c->d_image = nullptr;
    c->image_cap = 0;
    cudaError_t e = cudaMalloc(&c->d_image, bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "image allocation");
    c->image_cap = bytes;
  }
  vvlic_status st = vvlic_render_device(c, vol_id, (float*)c->d_image, w, h, nullptr, c->stream);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(out, c->d_image, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "render");
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_render_to_host_async(vvlic_ctx* c, int32_t vol_id, float* out, int32_t w, int32_t h,
                                                  void* stream) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!out || w < 1 || h < 1 || w > 32768 || h > 32768)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "render_to_host_async: bad image arguments");
  DeviceGuard g(c->device);
  const size_t bytes = (size_t)w * h * 4 * sizeof(float);
  if (c->image_cap < bytes) {
    cudaError_t e = cudaDeviceSynchronize();  // a download in flight may still read the image
    if (e != cudaSuccess) return cuda_fail(c, e, "render_to_host_async");
    if (c->d_image) cudaFree(c->d_image);
    c->d_image = nullptr;
    c->image_cap = 0;
    e = cudaMalloc(&c->d_image, bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "image allocation");
    c->image_cap = bytes;
  }
  vvlic_status st = vvlic_render_device(c, vol_id, (float*)c->d_image, w, h, nullptr, stream);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(out, c->d_image, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "render_to_host_async");
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_get_stats(vvlic_ctx* c, vvlic_stats* out) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!out) return VVLIC_ERR_INVALID_ARGUMENT;
  if (c->stats_pending) {
    DeviceGuard g(c->device);
    cudaError_t e = cudaEventSynchronize(c->ev1);
    unsigned long long h[4];
    if (e == cudaSuccess) e = cudaMemcpy(h, c->d_counters, sizeof h, cudaMemcpyDeviceToHost);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    if (e != cudaSuccess) return cuda_fail(c, e, "get_stats");
    c->stats.samples = h[0];
    c->stats.rays = h[1];
    // a batch mixes LIC lengths and counts its sample-steps on the device
    c->stats.sample_steps = c->last_was_batch ? h[2] : h[0] * c->stats_steps_per_sample;
    c->stats.kernel_ms = ms;
    c->stats.check_flags = (uint32_t)h[3];
    if (c->tape_flag_pending && c->d_tape_flag) {
      // rays of the recording render that outgrew their tape (store_pixel counts them)
      unsigned long long over = 0;
      e = cudaMemcpy(&over, c->d_tape_flag, sizeof over, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_fail(c, e, "get_stats");
      if (over) c->stats.check_flags |= VVLIC_CHECK_TAPE_OVERFLOW;
    }
    c->stats_pending = false;
  }
  *out = c->stats;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_compute_lic_volume(vvlic_ctx* c, int32_t vol_id, int32_t nx, int32_t ny, int32_t nz) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  auto it = c->vols.find(vol_id);
  if (it == c->vols.end()) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "compute_lic_volume: unknown volume %d", vol_id);
  if (nx < 1 || ny < 1 || nz < 1 || nx > 2048 || ny > 2048 || nz > 2048)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "compute_lic_volume: dims");
  if (c->params.sampler == VVLIC_SAMPLER_BRICK)
    return fail(c, VVLIC_ERR_UNSUPPORTED, "compute_lic_volume: the BRICK sampler renders the RAYCAST technique only");
  DeviceGuard g(c->device);
  Volume& v = it->second;
  cudaStream_t s = c->stream;
  RenderArgs a;
  vvlic_status st = build_render_args(c, v, 1, 1, s, a);
  if (st) return st;
  const size_t count = (size_t)nx * ny * nz;
  if (v.d_licvol && (size_t)v.ln[0] * v.ln[1] * v.ln[2] != count) {
    cudaStreamSynchronize(s);
    cudaFree(v.d_licvol);
    v.d_licvol = nullptr;
  }
  if (!v.d_licvol) {
    cudaError_t e = cudaMalloc(&v.d_licvol, count * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(c, e, "LIC volume allocation");
  }
  v.ln[0] = nx;
  v.ln[1] = ny;
  v.ln[2] = nz;
  TechArgs t;
  std::memset(&t, 0, sizeof t);
  t.technique = VVLIC_TECHNIQUE_LICVOLUME;
  t.licvol_out = v.d_licvol;
  t.ln[0] = nx;
  t.ln[1] = ny;
  t.ln[2] = nz;
  // lic3d_volume_fragment.glsl composes inc_lic without inc_illum: the uniform scaleVol is the
  // volume's scale whatever the shading variant
  for (int i = 0; i < 3; ++i) a.scale_vol[i] = v.geom.scale[i];
  cudaError_t e = cudaMemsetAsync(c->d_counters, 0, 4 * sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev0, s);
  if (e == cudaSuccess) e = launch_technique(v.storage, a, t, c->params.sampler, c->params.integrator, false, s);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev1, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(c, e, "compute_lic_volume");
  v.licvol_valid = true;
  // the precompute's statistics: one LIC sample per voxel, L_b + L_f streamline steps each
  unsigned long long h[4];
  float ms = 0.f;
  e = cudaMemcpy(h, c->d_counters, sizeof h, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  if (e != cudaSuccess) return cuda_fail(c, e, "compute_lic_volume statistics");
  c->stats.samples = count;
  c->stats.sample_steps = count * (uint64_t)(a.lb + a.lf);
  c->stats.rays = 0;
  c->stats.kernel_ms = ms;
  c->stats.check_flags = (uint32_t)h[3];
  c->stats_pending = false;
  c->last_was_batch = false;
  c->tape_flag_pending = false;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_download_lic_volume(vvlic_ctx* c, int32_t vol_id, float* out, uint64_t capacity) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  auto it = c->vols.find(vol_id);
  if (it == c->vols.end() || !it->second.d_licvol || !it->second.licvol_valid)
    return fail(c, VVLIC_ERR_NOT_READY, "download_lic_volume: no LIC volume for volume %d", vol_id);
  const size_t bytes = (size_t)it->second.ln[0] * it->second.ln[1] * it->second.ln[2] * sizeof(float);
  if (!out || capacity < bytes) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "download_lic_volume: need %zu bytes", bytes);
  DeviceGuard g(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(out, it->second.d_licvol, bytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(c, e, "download_lic_volume");
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_synchronize(vvlic_ctx* c, void* stream, int32_t timeout_ms) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (timeout_ms < 0) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "synchronize: negative timeout");
  DeviceGuard g(c->device);
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::microseconds((int64_t)timeout_ms * 1000);
  cudaStream_t streams[2] = {(cudaStream_t)stream, c->stream};
  for (cudaStream_t st : streams) {
    for (;;) {
      const cudaError_t e = cudaStreamQuery(st);
      if (e == cudaSuccess) break;
      if (e != cudaErrorNotReady) return cuda_fail(c, e, "synchronize");
      if (std::chrono::steady_clock::now() >= deadline)
        return fail(c, VVLIC_ERR_TIMEOUT, "synchronize: work still running after %d ms", timeout_ms);
      std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
  }
  return VVLIC_OK;
}
