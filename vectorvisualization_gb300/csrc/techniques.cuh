// The reference's other render techniques over the same field, noise and LIC machinery:
//   * SLICING (Renderer::sliceVolume renderer.cpp:1123-1267, ViewSlicing slicing.cpp:42-263,
//     lic3d_slicing_fragment.glsl): samples where each pixel's ray crosses the view-aligned
//     planes d_i = -D/2 + (i+1/2) D/N through the volume centre, front to back; TF on the
//     magnitude, LIC only where tf.a > 0.05, no more blending once dest.a >= 0.95.
//   * VOLUME (Renderer::renderVolume renderer.cpp:1066-1090, vectorfield_fragment.glsl:39-101):
//     direct volume rendering of the encoded directions, src = (field.rgb, TF(field.a).a).
//   * LICVOLUME (Renderer::renderLICVolume renderer.cpp:1311-1374 + lic3d_volume_fragment.glsl,
//     then raycast_lic3d_fragment.glsl): a precomputed volume of LIC intensities (one per voxel
//     centre), ray-cast with illumLIC; REPEAT-wrapped like the reference's VolumeBuffer.
// VOLUME and LICVOLUME stop on the accumulated dest.a > 0.95 as their shaders do.
#pragma once

#include "render_fwd.cuh"

namespace vvlic {

// texture3D(licVolumeSampler, s).r: LINEAR + REPEAT (VolumeBuffer.cpp:43-57), in FP32.
__device__ __forceinline__ float sample_licvol(const TechArgs& t, float3 s) {
  int x0, x1, y0, y1, z0, z1;
  float ax, ay, az;
  repeat_axis_fast(s.x, t.ln[0], x0, x1, ax);
  repeat_axis_fast(s.y, t.ln[1], y0, y1, ay);
  repeat_axis_fast(s.z, t.ln[2], z0, z1, az);
  // up to 2048^3 entries: row offsets in 64 bits
  const size_t nx = (size_t)t.ln[0], nxy = nx * (size_t)t.ln[1];
  const float* v = t.licvol;
  const float* r00 = v + z0 * nxy + y0 * nx;
  const float* r10 = v + z0 * nxy + y1 * nx;
  const float* r01 = v + z1 * nxy + y0 * nx;
  const float* r11 = v + z1 * nxy + y1 * nx;
  const float c00 = lerpf(__ldg(r00 + x0), __ldg(r00 + x1), ax);
  const float c10 = lerpf(__ldg(r10 + x0), __ldg(r10 + x1), ax);
  const float c01 = lerpf(__ldg(r01 + x0), __ldg(r01 + x1), ax);
  const float c11 = lerpf(__ldg(r11 + x0), __ldg(r11 + x1), ax);
  return lerpf(lerpf(c00, c10, ay), lerpf(c01, c11, ay), az);
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
__device__ __forceinline__ float4 slice_pixel(const RenderArgs& a, const TechArgs& t, const float* s_tf, int px,
                                              int py, uint32_t& samples, uint32_t& hit) {
  float4 dest = make_float4(0.f, 0.f, 0.f, 0.f);
  samples = 0;
  hit = 0;
  float o[3], d[3], tn, tf;
  if (!ray_interval(a, px, py, o, d, tn, tf)) return dest;
  hit = 1;
  const float3 O = f3(o[0], o[1], o[2]), D = f3(d[0], d[1], d[2]);
  const float3 V = f3(t.v[0], t.v[1], t.v[2]), C = f3(t.c[0], t.c[1], t.c[2]);
  const float vd = dot3(V, D);
  if (vd == 0.0f) return dest;  // ray parallel to the planes
  const float voc = dot3(V, sub3(O, C));
  const float3 sv = f3(a.scale_vol[0], a.scale_vol[1], a.scale_vol[2]);
  const float3 dir = mul3(norm3(D), sv);
  const float step = t.depth / (float)t.nslices;
  for (int i = 0; i < t.nslices; ++i) {
    if (dest.w >= 0.95f) break;  // lic3d_slicing_fragment.glsl:14 (no later slice changes dest)
    const float di = -0.5f * t.depth + ((float)i + 0.5f) * step;
    const float ti = (di - voc) / vd;
    if (!(ti >= tn && ti <= tf)) continue;  // outside the slice polygon (plane inside the box)
    const float3 x = add3(O, scl3(D, ti));
    const float3 pos = mul3(x, sv);
    const float4 f = Field<ST, FL>::sample(a, pos);
    const float4 tfv = tf_rgba(s_tf, f.w);
    if (!(tfv.w > 0.05f)) continue;
    float4 il = compute_lic<ST, FL, NL, INTEG, GRAD>(a, pos, f);
    ++samples;
    il.w *= a.intensity_scale;
    const float4 src = shade<GRAD>(a, s_tf, il, tfv, pos, dir, f);
    dest = blend(dest, src);
  }
  return dest;
}

template <int ST, int FL>
__device__ __forceinline__ float4 volume_pixel(const RenderArgs& a, const TechArgs& t, const float* s_tf, int px,
                                               int py, uint32_t& samples, uint32_t& hit) {
  float4 dest = make_float4(0.f, 0.f, 0.f, 0.f);
  samples = 0;
  hit = 0;
  float3 pos, dir;
  if (!ray_setup(a, px, py, pos, dir)) return dest;
  hit = 1;
  bool outside = false;
  for (int j = 0; !outside && j < a.num_iter; ++j) {
    for (int i = 0; i < a.num_iter; ++i) {
      const float4 f = Field<ST, FL>::sample(a, pos);
      float4 src;
      if (t.technique == VVLIC_TECHNIQUE_LICVOLUME) {
        const float I = sample_licvol(t, pos);
        const float4 tfv = tf_rgba(s_tf, a.tf_index == VVLIC_TF_INDEX_MAGNITUDE ? f.w : f.z);
        src = shade<false>(a, s_tf, make_float4(0.f, 0.f, 0.f, I), tfv, pos, dir, f);  // illumLIC
      } else {
        src = make_float4(f.x, f.y, f.z, tf_rgba(s_tf, f.w).w);
      }
      ++samples;
      dest = blend(dest, src);
      pos = add3(pos, scl3(dir, a.step_size));
      outside = outside_box(a, pos) || dest.w > a.alpha_thr;
      if (outside) break;
    }
  }
  return dest;
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
__global__ void __launch_bounds__(kThreads, VVLIC_MIN_BLOCKS) technique_kernel(const __grid_constant__ RenderArgs a,
                                                                               const __grid_constant__ TechArgs t) {
  __shared__ __align__(16) float s_tf[5 * VVLIC_TF_ENTRIES];
  load_tf(a, s_tf);
  const int px = blockIdx.x * kTileW + (threadIdx.x % kTileW);
  const int py = blockIdx.y * kTileH + (threadIdx.x / kTileW);
  uint32_t samples = 0, hit = 0;
  if (px < a.W && py < a.H) {
    float4 dest = t.technique == VVLIC_TECHNIQUE_SLICING
                      ? slice_pixel<ST, FL, NL, INTEG, GRAD>(a, t, s_tf, px, py, samples, hit)
                      : volume_pixel<ST, FL>(a, t, s_tf, px, py, samples, hit);
    store_pixel(a, px, py, dest, samples);
  }
  flush_counters(a, samples, hit);
}

// LIC intensity at every voxel centre of the LIC volume: lic3d_volume_fragment.glsl:2-21 with
// pos = ((x+.5)/nx, (y+.5)/ny, (z+.5)/nz) * scaleVol (VolumeBuffer::drawSlice).  A warp takes a
// tile of kLicvolTileW x kLicvolTileH voxels in x, y and kLicvolPairZ consecutive slices; with
// two slices each thread computes both voxels' LIC together (compute_lic2: four independent
// streamline chains, results bit-identical to compute_lic).  On the 512^3 turbulence field (RK4,
// L = 60 each way) the 8x4 tiles took 202.7 ms against 217.9 ms for 32-voxel rows; two slices per
// thread took 211.1 ms in rows and 203.3 ms in tiles, so one slice and 8x4 tiles are the default.
#ifndef VVLIC_LICVOL_TILE
#define VVLIC_LICVOL_TILE 1
#endif
#ifndef VVLIC_LICVOL_PAIR
#define VVLIC_LICVOL_PAIR 0
#endif
#ifndef VVLIC_LICVOL_MIN_BLOCKS
#define VVLIC_LICVOL_MIN_BLOCKS 1
#endif
constexpr int kLicvolTileW = VVLIC_LICVOL_TILE ? 8 : 32, kLicvolTileH = VVLIC_LICVOL_TILE ? 4 : 1;
constexpr int kLicvolPairZ = VVLIC_LICVOL_PAIR ? 2 : 1;

// warp work items of an nx*ny*nz LIC volume
__host__ __device__ inline size_t licvol_items(const int ln[3]) {
  return (size_t)((ln[0] + kLicvolTileW - 1) / kLicvolTileW) * (size_t)((ln[1] + kLicvolTileH - 1) / kLicvolTileH) *
         (size_t)((ln[2] + kLicvolPairZ - 1) / kLicvolPairZ);
}

__device__ __forceinline__ float3 licvol_pos(const RenderArgs& a, const TechArgs& t, int x, int y, int z) {
  return mul3(f3(((float)x + 0.5f) / t.ln[0], ((float)y + 0.5f) / t.ln[1], ((float)z + 0.5f) / t.ln[2]),
              f3(a.scale_vol[0], a.scale_vol[1], a.scale_vol[2]));
}

template <int ST, int FL, int NL, int INTEG>
__global__ void __launch_bounds__(kThreads, VVLIC_LICVOL_MIN_BLOCKS) licvolume_kernel(const __grid_constant__ RenderArgs a,
                                                                                      const __grid_constant__ TechArgs t) {
  const int nx = t.ln[0], ny = t.ln[1], nz = t.ln[2];
  const int tx = (nx + kLicvolTileW - 1) / kLicvolTileW, ty = (ny + kLicvolTileH - 1) / kLicvolTileH;
  const size_t items = licvol_items(t.ln);
  const int lane = threadIdx.x & 31;
  const size_t stride = (size_t)gridDim.x * (blockDim.x >> 5);
  for (size_t wi = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); wi < items; wi += stride) {
    const int x = (int)(wi % tx) * kLicvolTileW + lane % kLicvolTileW;
    const int y = (int)((wi / tx) % ty) * kLicvolTileH + lane / kLicvolTileW;
    const int z = (int)(wi / ((size_t)tx * ty)) * kLicvolPairZ;
    if (x >= nx || y >= ny) continue;
    const size_t v = ((size_t)z * ny + y) * nx + x;
    const float3 p0 = licvol_pos(a, t, x, y, z);
    const float4 f0 = Field<ST, FL>::sample(a, p0);
    if (kLicvolPairZ == 2 && z + 1 < nz) {
      const float3 p1 = licvol_pos(a, t, x, y, z + 1);
      const float4 f1 = Field<ST, FL>::sample(a, p1);
      float4 i0, i1;
      compute_lic2<ST, FL, NL, INTEG, false>(a, p0, f0, p1, f1, i0, i1);
      t.licvol_out[v] = i0.w * a.intensity_scale;
      t.licvol_out[v + (size_t)nx * ny] = i1.w * a.intensity_scale;
    } else {
      t.licvol_out[v] = compute_lic<ST, FL, NL, INTEG, false>(a, p0, f0).w * a.intensity_scale;
    }
  }
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
static cudaError_t launch_tech_one(const RenderArgs& a, const TechArgs& t, cudaStream_t s) {
  if (t.technique == VVLIC_TECHNIQUE_LICVOLUME && t.licvol_out) {
    const size_t threads = licvol_items(t.ln) * 32;
    const int blocks = (int)std::min<size_t>((threads + kThreads - 1) / kThreads, (size_t)152 * 64);
    licvolume_kernel<ST, FL, NL, INTEG><<<std::max(1, blocks), kThreads, 0, s>>>(a, t);
    return cudaGetLastError();
  }
  dim3 grid((a.W + kTileW - 1) / kTileW, (a.H + kTileH - 1) / kTileH);
  technique_kernel<ST, FL, NL, INTEG, GRAD><<<grid, kThreads, 0, s>>>(a, t);
  return cudaGetLastError();
}

template <int ST, int FL, int NL>
static cudaError_t launch_tech_layout(const RenderArgs& a, const TechArgs& t, int integ, bool grad, cudaStream_t s) {
  if (grad) {
    if (integ == VVLIC_EULER) return launch_tech_one<ST, FL, NL, VVLIC_EULER, true>(a, t, s);
    if (integ == VVLIC_HEUN) return launch_tech_one<ST, FL, NL, VVLIC_HEUN, true>(a, t, s);
    return launch_tech_one<ST, FL, NL, VVLIC_RK4, true>(a, t, s);
  }
  if (integ == VVLIC_EULER) return launch_tech_one<ST, FL, NL, VVLIC_EULER, false>(a, t, s);
  if (integ == VVLIC_HEUN) return launch_tech_one<ST, FL, NL, VVLIC_HEUN, false>(a, t, s);
  return launch_tech_one<ST, FL, NL, VVLIC_RK4, false>(a, t, s);
}

template <int ST>
static cudaError_t launch_tech_storage(const RenderArgs& a, const TechArgs& t, int sampler, int integ, bool grad,
                                       cudaStream_t s) {
  switch (sampler) {
    case VVLIC_SAMPLER_GATHER: return launch_tech_layout<ST, kGather, kGather>(a, t, integ, grad, s);
    case VVLIC_SAMPLER_CELL: return launch_tech_layout<ST, kCell, kCell>(a, t, integ, grad, s);
    case VVLIC_SAMPLER_TEXTURE:
      if constexpr (ST == VVLIC_STORAGE_BF16) return cudaErrorNotSupported;  // runs as F16 (kernel_storage)
      else return launch_tech_layout<ST, kTexture, kTexture>(a, t, integ, grad, s);
    case VVLIC_SAMPLER_HYBRID:
      if constexpr (ST == VVLIC_STORAGE_BF16) return cudaErrorNotSupported;
      else return launch_tech_layout<ST, kTexture, kCellFast>(a, t, integ, grad, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vvlic
