// Render entry points: uniform derivation (Renderer::setRenderVolParams, renderer.cpp:925-996),
// lazy construction of the field/noise layouts the chosen sampler reads, and the launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "../../include/vvlic.h"
#include "vvlic_device.cuh"
#include "vvlic_host.hpp"
#include "vvlic_launch.hpp"

using namespace vvlic;

namespace {

vvlic_status ensure_cells(vvlic_ctx* c, Volume& v, cudaStream_t s) {
  if (v.d_cells) return VVLIC_OK;
  const size_t cells = (size_t)(v.n[0] + 1) * (v.n[1] + 1) * (v.n[2] + 1);
  const size_t bytes = cells * 8 * (v.storage == VVLIC_STORAGE_F32 ? 16 : 8);
  cudaError_t e = cudaMalloc(&v.d_cells, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "cell layout allocation");
  v.cell_bytes = bytes;
  e = launch_build_field_cells(v.d_texels, v.n, v.storage, v.d_cells, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "cell layout build");
  return VVLIC_OK;
}

vvlic_status ensure_noise_cells(vvlic_ctx* c, NoiseTex& n, cudaStream_t s) {
  if (n.d_cells) return VVLIC_OK;
  const size_t bytes = (size_t)n.m[0] * n.m[1] * n.m[2] * 8 * n.ch;
  cudaError_t e = cudaMalloc(&n.d_cells, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise cell allocation");
  e = launch_build_noise_cells(n.d_texels, n.m, n.ch, n.d_cells, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise cell build");
  return VVLIC_OK;
}

vvlic_status ensure_texture(vvlic_ctx* c, Volume& v, cudaStream_t s) {
  if (v.tex) return VVLIC_OK;
  if (v.storage == VVLIC_STORAGE_BF16) return fail(c, VVLIC_ERR_UNSUPPORTED, "TEXTURE sampler has no BF16 format");
  cudaChannelFormatDesc desc =
      v.storage == VVLIC_STORAGE_F32 ? cudaCreateChannelDesc<float4>() : cudaCreateChannelDescHalf4();
  cudaExtent ext = make_cudaExtent(v.n[0], v.n[1], v.n[2]);
  cudaError_t e = cudaMalloc3DArray(&v.array, &desc, ext);
  if (e != cudaSuccess) return cuda_fail(c, e, "texture array allocation");
  const size_t tb = v.storage == VVLIC_STORAGE_F32 ? 16 : 8;
  v.array_bytes = (size_t)v.n[0] * v.n[1] * v.n[2] * tb;
  cudaMemcpy3DParms cp;
  std::memset(&cp, 0, sizeof cp);
  cp.srcPtr = make_cudaPitchedPtr(v.d_texels, v.n[0] * tb, v.n[0], v.n[1]);
  cp.dstArray = v.array;
  cp.extent = ext;
  cp.kind = cudaMemcpyDeviceToDevice;
  e = cudaMemcpy3DAsync(&cp, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "texture array copy");
  cudaResourceDesc rd;
  std::memset(&rd, 0, sizeof rd);
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = v.array;
  cudaTextureDesc td;
  std::memset(&td, 0, sizeof td);
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;  // CLAMP_TO_EDGE
  td.filterMode = cudaFilterModeLinear;
  td.readMode = cudaReadModeElementType;
  td.normalizedCoords = 1;  // GL texture coordinates
  e = cudaCreateTextureObject(&v.tex, &rd, &td, nullptr);
  if (e != cudaSuccess) return cuda_fail(c, e, "texture object");
  return VVLIC_OK;
}

// Noise as an R8 / RGBA8 texture read as normalised float with WRAP addressing (GL REPEAT).
vvlic_status ensure_noise_texture(vvlic_ctx* c, NoiseTex& n, cudaStream_t s) {
  if (n.tex) return VVLIC_OK;
  cudaChannelFormatDesc desc =
      n.ch == 4 ? cudaCreateChannelDesc<uchar4>() : cudaCreateChannelDesc<unsigned char>();
  cudaExtent ext = make_cudaExtent(n.m[0], n.m[1], n.m[2]);
  cudaError_t e = cudaMalloc3DArray(&n.array, &desc, ext);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise texture allocation");
  cudaMemcpy3DParms cp;
  std::memset(&cp, 0, sizeof cp);
  cp.srcPtr = make_cudaPitchedPtr(n.d_texels, (size_t)n.m[0] * n.ch, n.m[0], n.m[1]);
  cp.dstArray = n.array;
  cp.extent = ext;
  cp.kind = cudaMemcpyDeviceToDevice;
  e = cudaMemcpy3DAsync(&cp, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise texture copy");
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

// Fill the kernel argument block for one volume and image size.
vvlic_status build_render_args(vvlic_ctx* c, Volume& v, int W, int H, cudaStream_t s, RenderArgs& a) {
  const vvlic_params& p = c->params;
  std::memset(&a, 0, sizeof a);
  if (!c->noise.d_texels) return fail(c, VVLIC_ERR_NOT_READY, "render: no noise uploaded");
  if (p.illum == VVLIC_ILLUM_GRADIENT && c->noise.ch != 4)
    return fail(c, VVLIC_ERR_NOT_READY, "render: gradient lighting needs noise uploaded with gradients");
  if (p.scalar_gate && !c->d_scalar) return fail(c, VVLIC_ERR_NOT_READY, "render: scalar gate on, no scalar volume");
  int lb = p.low_res ? 15 : p.steps_backward, lf = p.low_res ? 15 : p.steps_forward;
  float inv_area = 0.5f;
  if (derive_taps(c, lb, lf, a.taps, &inv_area))
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "render: explicit taps were set for L_b=%d L_f=%d, params have %d/%d",
                c->taps_lb, c->taps_lf, lb, lf);
  vvlic_status st;
  a.n[0] = v.n[0];
  a.n[1] = v.n[1];
  a.n[2] = v.n[2];
  if (p.sampler == VVLIC_SAMPLER_GATHER) {
    a.field = v.d_texels;
    a.noise = c->noise.d_texels;
    a.noise_cells = 0;
  } else {
    if (p.sampler == VVLIC_SAMPLER_CELL) {
      if ((st = ensure_cells(c, v, s))) return st;
      a.field = v.d_cells;
      if ((st = ensure_noise_cells(c, c->noise, s))) return st;
      a.noise = c->noise.d_cells;
      a.noise_cells = 1;
    } else {
      if ((st = ensure_texture(c, v, s))) return st;
      if ((st = ensure_noise_texture(c, c->noise, s))) return st;
      a.tex = v.tex;
      a.noise_tex = c->noise.tex;
    }
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
  derive_rays(c->view, v.geom, W, H, rc);
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
  a.counters = c->d_counters;
  return VVLIC_OK;
}

cudaError_t launch_raycast(const RenderArgs& a, int storage, int sampler, int integ, bool grad, cudaStream_t s) {
  switch (storage) {
    case VVLIC_STORAGE_F32: return launch_raycast_f32(a, sampler, integ, grad, s);
    case VVLIC_STORAGE_F16: return launch_raycast_f16(a, sampler, integ, grad, s);
    default: return launch_raycast_bf16(a, sampler, integ, grad, s);
  }
}

}  // namespace vvlic

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
  cudaError_t e = cudaMemsetAsync(c->d_counters, 0, 4 * sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev0, s);
  if (e == cudaSuccess)
    e = launch_raycast(a, it->second.storage, c->params.sampler, c->params.integrator,
                       c->params.illum == VVLIC_ILLUM_GRADIENT, s);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev1, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "render launch");
  c->stats_pending = true;
  c->stats.sample_steps = 0;
  c->stats_steps_per_sample = (uint64_t)(a.lb + a.lf);
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
    c->stats.sample_steps = h[0] * c->stats_steps_per_sample;
    c->stats.kernel_ms = ms;
    c->stats_pending = false;
  }
  *out = c->stats;
  return VVLIC_OK;
}
