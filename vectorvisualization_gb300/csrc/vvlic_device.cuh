// Device-side building blocks of the LIC ray-caster: GL-semantics samplers over the field,
// noise and transfer-function tables, the streamline integrators, computeLIC, the shading models
// and the front-to-back blend.  Each function names the reference GLSL it computes
// (paths within VectorVisualization/shader/).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vvlic.h"

namespace vvlic {

constexpr int kMaxTaps = 2 * VVLIC_MAX_STEPS + 1;

// Memory layouts a sampler reads (field and noise separately).  kCellFast is the kCell noise
// layout filtered with biased bytes (see NoiseCells), the HYBRID sampler's noise.
enum Layout : int { kGather = 0, kCell = 1, kTexture = 2, kCellFast = 3 };

// Kernel arguments of one render job, passed by value as a __grid_constant__ parameter (in
// the constant bank; the taps are read warp-uniformly so they broadcast).
struct RenderArgs {
  const void* field;          // GATHER: n0*n1*n2 RGBA texels; CELL: (n+1)^3 cells of 8 texels
  cudaTextureObject_t tex;    // TEXTURE layout
  int n[3];
  const uint8_t* noise;       // GATHER: m0*m1*m2 texels of noise_ch bytes; CELL: m^3 cells
  cudaTextureObject_t noise_tex;  // TEXTURE layout
  int m[3];
  int noise_ch;               // 1 (value) or 4 (gradient xyz, value)
  const float* scalar;        // optional gate volume
  int sn[3];
  const float* tf;            // 256 RGBA entries followed by 256 opacity entries
  float* out;                 // W*H RGBA
  uint32_t* samples;          // optional per-pixel sample counts
  unsigned long long* counters;  // [0] samples, [1] rays
  int W, H;
  float o0[3], o1[3], o2[3], d0[3], d1[3], d2[3];
  int clamp0;
  float ext[3], tex_max[3], scale_vol[3], scale_vol_inv[3];
  float step_size, h_eff, intensity_scale, alpha_corr, illum_scale, freq_scale, alpha_thr;
  // noise texel-space scale of a streamline position per axis, m * frequency, for value taps
  // (freq_scale) and gradient taps (1 under VVLIC_QUIRK_GRAD_NOISE_NO_FREQ): the cell samplers
  // form u = p * scale - 1/2 with one FMA
  float nscale[3], nscale_grad[3];
  float gate_lo, gate_hi;
  int num_iter, lb, lf, illum, tf_index, sof, gate, quirks;
  float light_pos[3], spec_exp, light_diff[3], light_spec[3], light_amb[3];
  // line-illumination tables (ZOECKLER / MALLO): Zoeckler, Mallo diffuse, Mallo specular,
  // lut_w x lut_h RGBA8 each, x fastest
  const uchar4* luts;
  int lut_w, lut_h;
  // adjoint tape (recording forward / adjoint only): per ray `tape_stride` samples of
  // (intensity, TF coordinate), `tape_nck` checkpoints of (position, dest before the sample)
  // every kSegment samples, and the sample count
  float2* tape_is;
  uint2* tape_g;  // gradient lighting only: per sample the LIC gradient sum G as 4 halves (x, y, z, 0)
  float4* tape_ck;
  uint32_t* tape_n;
  unsigned long long* tape_overflow;  // rays with more samples than tape_stride
  int tape_stride, tape_nck;
  float taps[kMaxTaps];
};

constexpr int kSegment = 32;  // adjoint checkpoint interval (samples)

// Extra arguments of the non-raycast techniques (techniques.cuh).
struct TechArgs {
  int technique;
  // slicing: unit plane normal (view direction, object space), volume centre, depth, count
  float v[3], c[3], depth;
  int nslices;
  // LIC volume: ln[0]*ln[1]*ln[2] intensities, x fastest
  const float* licvol;  // read by LICVOLUME renders
  float* licvol_out;    // written by the precompute
  int ln[3];
};

// ------------------------------------------------------------------------------------------
// small vector helpers
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 scl3(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 mul3(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 norm3(float3 a) {
  float d = dot3(a, a);
  if (!(d > 0.0f)) return f3(0.f, 0.f, 0.f);  // normalize(0) := 0
  return scl3(a, 1.0f / sqrtf(d));
}
__device__ __forceinline__ float lerpf(float a, float b, float t) { return fmaf(t, b - a, a); }
__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {
  return make_float4(lerpf(a.x, b.x, t), lerpf(a.y, b.y, t), lerpf(a.z, b.z, t), lerpf(a.w, b.w, t));
}
__device__ __forceinline__ float4 trilerp(float4 t000, float4 t100, float4 t010, float4 t110, float4 t001,
                                          float4 t101, float4 t011, float4 t111, float ax, float ay, float az) {
  float4 c0 = lerp4(lerp4(t000, t100, ax), lerp4(t010, t110, ax), ay);
  float4 c1 = lerp4(lerp4(t001, t101, ax), lerp4(t011, t111, ax), ay);
  return lerp4(c0, c1, az);
}

// ------------------------------------------------------------------------------------------
// texel decoding per storage precision
// ------------------------------------------------------------------------------------------
// One 32-byte read-only load: the 256-bit vector load of sm_100 and later, one L1 request for
// a whole 32-byte cell instead of two 16-byte ones.  p must be 32-byte aligned.
__device__ __forceinline__ void ldg256(const void* p, uint32_t (&r)[8]) {
  asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "l"(p));
}

// Byte k of w as an exact float without a conversion instruction: assemble the bit pattern
// 0x4B0000bb (= 2^23 + b) with one byte permute and subtract 2^23.
__device__ __forceinline__ float byte_as_float(uint32_t w, int k) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u + (unsigned)k)) - 8388608.0f;
}

// Byte k of w as the float 32768 + b: one byte permute assembles 0x4700bb00 (exponent 2^15,
// the byte in mantissa bits 8..15, so b is exact and 8 mantissa bits lie below it).
__device__ __forceinline__ float byte_biased(uint32_t w, int k) {
  return __uint_as_float(__byte_perm(w, 0x47000000u, 0x7404u + ((unsigned)k << 4)));
}

__device__ __forceinline__ float4 unorm8x4(uint32_t r) {
  const float k = 1.0f / 255.0f;
  return make_float4(byte_as_float(r, 0) * k, byte_as_float(r, 1) * k, byte_as_float(r, 2) * k,
                     byte_as_float(r, 3) * k);
}

template <int ST> struct Texel;
template <> struct Texel<VVLIC_STORAGE_F32> {
  static __device__ __forceinline__ float4 load(const void* base, int idx) {
    return __ldg(reinterpret_cast<const float4*>(base) + idx);
  }
};
template <> struct Texel<VVLIC_STORAGE_F16> {
  static __device__ __forceinline__ float4 decode(uint2 r) {
    __half2 a = *reinterpret_cast<__half2*>(&r.x), b = *reinterpret_cast<__half2*>(&r.y);
    float2 fa = __half22float2(a), fb = __half22float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
  }
  static __device__ __forceinline__ float4 load(const void* base, int idx) {
    return decode(__ldg(reinterpret_cast<const uint2*>(base) + idx));
  }
};
template <> struct Texel<VVLIC_STORAGE_BF16> {
  static __device__ __forceinline__ float4 decode(uint2 r) {
    // bf16 -> f32 is a 16-bit shift
    return make_float4(__uint_as_float(r.x << 16), __uint_as_float(r.x & 0xffff0000u), __uint_as_float(r.y << 16),
                       __uint_as_float(r.y & 0xffff0000u));
  }
  static __device__ __forceinline__ float4 load(const void* base, int idx) {
    return decode(__ldg(reinterpret_cast<const uint2*>(base) + idx));
  }
};
template <> struct Texel<VVLIC_STORAGE_UNORM8> {
  static __device__ __forceinline__ float4 load(const void* base, int idx) {
    return unorm8x4(__ldg(reinterpret_cast<const uint32_t*>(base) + idx));
  }
};

// Texel-space coordinate of a CLAMP_TO_EDGE axis: returns the lower texel index (clamped) and
// the weight of the upper one.  GL: u = s*N - 1/2, i0 = floor(u), alpha = frac(u).
__device__ __forceinline__ void clamp_axis(float s, int n, int& i0, int& i1, float& a) {
  float u = fmaf(s, (float)n, -0.5f);
  u = fminf(fmaxf(u, -1.0f), (float)n);  // also maps NaN to -1; clamped texels are equal there
  float fl = floorf(u);
  a = u - fl;
  int b = (int)fl;
  i0 = min(max(b, 0), n - 1);
  i1 = min(max(b + 1, 0), n - 1);
}

// Bounds-checked builds (-DVVLIC_BOUNDS_CHECK=1): gather indices, tape slots and image pixels
// are tested against their buffers; an out-of-range one sets its VVLIC_CHECK_* bit in
// counters[3] and is replaced by entry 0 (loads) or skipped (stores).  Otherwise the tests
// compile away.
#ifndef VVLIC_BOUNDS_CHECK
#define VVLIC_BOUNDS_CHECK 0
#endif
__device__ __forceinline__ bool in_range(const RenderArgs& a, long long i, long long n, unsigned flag) {
  if (VVLIC_BOUNDS_CHECK && (i < 0 || i >= n)) {
    atomicOr(a.counters + 3, (unsigned long long)flag);
    return false;
  }
  return true;
}

// ------------------------------------------------------------------------------------------
// field sampling: texture3D(volumeSampler, s), LINEAR + CLAMP_TO_EDGE (dataset.cpp:351-357)
// ------------------------------------------------------------------------------------------
template <int ST, int LAYOUT> struct Field;

template <int ST> struct Field<ST, kGather> {
  static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 s) {
    int x0, x1, y0, y1, z0, z1;
    float ax, ay, az;
    clamp_axis(s.x, a.n[0], x0, x1, ax);
    clamp_axis(s.y, a.n[1], y0, y1, ay);
    clamp_axis(s.z, a.n[2], z0, z1, az);
    const int nx = a.n[0], nxy = a.n[0] * a.n[1];
    int r00 = z0 * nxy + y0 * nx, r10 = z0 * nxy + y1 * nx, r01 = z1 * nxy + y0 * nx, r11 = z1 * nxy + y1 * nx;
    if (VVLIC_BOUNDS_CHECK) {
      const long long n = (long long)nxy * a.n[2];
      if (!in_range(a, (long long)r00 + x0, n, VVLIC_CHECK_FIELD) || !in_range(a, (long long)r11 + x1, n, VVLIC_CHECK_FIELD))
        r00 = r10 = r01 = r11 = x0 = x1 = 0;
    }
    const void* f = a.field;
    return trilerp(Texel<ST>::load(f, r00 + x0), Texel<ST>::load(f, r00 + x1), Texel<ST>::load(f, r10 + x0),
                   Texel<ST>::load(f, r10 + x1), Texel<ST>::load(f, r01 + x0), Texel<ST>::load(f, r01 + x1),
                   Texel<ST>::load(f, r11 + x0), Texel<ST>::load(f, r11 + x1), ax, ay, az);
  }
};

// Corner-packed cells: cell c (per axis 0..n) holds texels clamp(c-1) and clamp(c), so the
// cell of coordinate u = s*n + 1/2 is floor(u) clamped to [0, n] for every s.
__device__ __forceinline__ void cell_axis(float s, int n, int& c, float& a) {
  float u = fmaf(s, (float)n, 0.5f);
  u = fminf(fmaxf(u, 0.0f), (float)n + 0.5f);
  float fl = floorf(u);
  a = u - fl;
  c = min((int)fl, n);
}
__device__ __forceinline__ int cell_index(const RenderArgs& a, float3 s, float& ax, float& ay, float& az) {
  int cx, cy, cz;
  cell_axis(s.x, a.n[0], cx, ax);
  cell_axis(s.y, a.n[1], cy, ay);
  cell_axis(s.z, a.n[2], cz, az);
  const int c = (cz * (a.n[1] + 1) + cy) * (a.n[0] + 1) + cx;
  if (VVLIC_BOUNDS_CHECK &&
      !in_range(a, c, (long long)(a.n[0] + 1) * (a.n[1] + 1) * (a.n[2] + 1), VVLIC_CHECK_FIELD))
    return 0;
  return c;
}

__device__ __forceinline__ float4 f4(const uint32_t* r) {
  return make_float4(__uint_as_float(r[0]), __uint_as_float(r[1]), __uint_as_float(r[2]), __uint_as_float(r[3]));
}
template <> struct Field<VVLIC_STORAGE_F32, kCell> {  // 128-byte cells, four 32-byte loads
  static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 s) {
    float ax, ay, az;
    const float4* c = reinterpret_cast<const float4*>(a.field) + 8 * (size_t)cell_index(a, s, ax, ay, az);
    uint32_t q0[8], q1[8], q2[8], q3[8];
    ldg256(c + 0, q0);
    ldg256(c + 2, q1);
    ldg256(c + 4, q2);
    ldg256(c + 6, q3);
    return trilerp(f4(q0), f4(q0 + 4), f4(q1), f4(q1 + 4), f4(q2), f4(q2 + 4), f4(q3), f4(q3 + 4), ax, ay, az);
  }
};
template <int ST> struct Field<ST, kCell> {  // F16 / BF16: 64-byte cells, two 32-byte loads
  static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 s) {
    float ax, ay, az;
    const uint4* c = reinterpret_cast<const uint4*>(a.field) + 4 * (size_t)cell_index(a, s, ax, ay, az);
    uint32_t q0[8], q1[8];
    ldg256(c + 0, q0);
    ldg256(c + 2, q1);
    return trilerp(Texel<ST>::decode(make_uint2(q0[0], q0[1])), Texel<ST>::decode(make_uint2(q0[2], q0[3])),
                   Texel<ST>::decode(make_uint2(q0[4], q0[5])), Texel<ST>::decode(make_uint2(q0[6], q0[7])),
                   Texel<ST>::decode(make_uint2(q1[0], q1[1])), Texel<ST>::decode(make_uint2(q1[2], q1[3])),
                   Texel<ST>::decode(make_uint2(q1[4], q1[5])), Texel<ST>::decode(make_uint2(q1[6], q1[7])), ax, ay, az);
  }
};
template <> struct Field<VVLIC_STORAGE_UNORM8, kCell> {  // 32-byte cells, one 32-byte load
  static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 s) {
    float ax, ay, az;
    uint32_t q[8];
    ldg256(reinterpret_cast<const uint4*>(a.field) + 2 * (size_t)cell_index(a, s, ax, ay, az), q);
    return trilerp(unorm8x4(q[0]), unorm8x4(q[1]), unorm8x4(q[2]), unorm8x4(q[3]), unorm8x4(q[4]), unorm8x4(q[5]),
                   unorm8x4(q[6]), unorm8x4(q[7]), ax, ay, az);
  }
};

template <int ST> struct Field<ST, kTexture> {  // hardware trilinear, normalised coordinates, CLAMP
  static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 s) {
    return tex3D<float4>(a.tex, s.x, s.y, s.z);
  }
};

// ------------------------------------------------------------------------------------------
// noise sampling: texture3D(noiseSampler, s), LINEAR + REPEAT (dataset.cpp:1333-1335), uint8/255.
// Returns (gradient rgb, value); for a one-channel noise the gradient part is 0.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void repeat_axis(float s, int m, int& i0, int& i1, float& a) {
  float u = fmaf(s, (float)m, -0.5f);
  u = fminf(fmaxf(u, -16777216.0f), 16777216.0f);
  float fl = floorf(u);
  a = u - fl;
  int b = (int)fl % m;
  if (b < 0) b += m;
  i0 = b;
  i1 = (b + 1 == m) ? 0 : b + 1;
}

__device__ __forceinline__ float bytef(uint32_t w, int k) { return (float)((w >> (8 * k)) & 0xffu); }

template <int NL> struct Noise;

// Texture coordinate of a noise tap at position p: p * frequency (value taps, and gradient taps
// without VVLIC_QUIRK_GRAD_NOISE_NO_FREQ), else p.
template <bool GRADC> __device__ __forceinline__ float3 noise_coord(const RenderArgs& a, float3 p) {
  if (GRADC && (a.quirks & VVLIC_QUIRK_GRAD_NOISE_NO_FREQ)) return p;
  return scl3(p, a.freq_scale);
}

template <> struct Noise<kGather> {
  template <bool RGBA, bool GRADC> static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 p) {
    const float3 s = noise_coord<GRADC>(a, p);
    int x0, x1, y0, y1, z0, z1;
    float ax, ay, az;
    repeat_axis(s.x, a.m[0], x0, x1, ax);
    repeat_axis(s.y, a.m[1], y0, y1, ay);
    repeat_axis(s.z, a.m[2], z0, z1, az);
    const float k = 1.0f / 255.0f;
    const int mx = a.m[0], mxy = a.m[0] * a.m[1];
    int r00 = z0 * mxy + y0 * mx, r10 = z0 * mxy + y1 * mx, r01 = z1 * mxy + y0 * mx, r11 = z1 * mxy + y1 * mx;
    if (VVLIC_BOUNDS_CHECK) {
      const long long n = (long long)mxy * a.m[2];
      if (!in_range(a, (long long)r00 + x0, n, VVLIC_CHECK_NOISE) || !in_range(a, (long long)r11 + x1, n, VVLIC_CHECK_NOISE))
        r00 = r10 = r01 = r11 = x0 = x1 = 0;
    }
    if (RGBA) {
      const uint32_t* t = reinterpret_cast<const uint32_t*>(a.noise);
      uint32_t t000 = __ldg(t + r00 + x0), t100 = __ldg(t + r00 + x1), t010 = __ldg(t + r10 + x0),
               t110 = __ldg(t + r10 + x1), t001 = __ldg(t + r01 + x0), t101 = __ldg(t + r01 + x1),
               t011 = __ldg(t + r11 + x0), t111 = __ldg(t + r11 + x1);
      float4 r;
      float* rp = &r.x;
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        float c00 = lerpf(bytef(t000, ch), bytef(t100, ch), ax), c10 = lerpf(bytef(t010, ch), bytef(t110, ch), ax);
        float c01 = lerpf(bytef(t001, ch), bytef(t101, ch), ax), c11 = lerpf(bytef(t011, ch), bytef(t111, ch), ax);
        rp[ch] = lerpf(lerpf(c00, c10, ay), lerpf(c01, c11, ay), az) * k;
      }
      return r;
    }
    const uint8_t* t = a.noise;
    float c00 = lerpf((float)__ldg(t + r00 + x0), (float)__ldg(t + r00 + x1), ax);
    float c10 = lerpf((float)__ldg(t + r10 + x0), (float)__ldg(t + r10 + x1), ax);
    float c01 = lerpf((float)__ldg(t + r01 + x0), (float)__ldg(t + r01 + x1), ax);
    float c11 = lerpf((float)__ldg(t + r11 + x0), (float)__ldg(t + r11 + x1), ax);
    return make_float4(0.f, 0.f, 0.f, lerpf(lerpf(c00, c10, ay), lerpf(c01, c11, ay), az) * k);
  }
};

// REPEAT wrap of the position p along an axis of m texels, pm = m * (texture coordinate per
// unit of p): power-of-two extents use a mask, others the integer remainder.
__device__ __forceinline__ void repeat_axis_fast(float p, float pm, int m, int& i0, int& i1, float& a) {
  float u = fmaf(p, pm, -0.5f);
  u = fminf(fmaxf(u, -16777216.0f), 16777216.0f);
  float fl = floorf(u);
  a = u - fl;
  int b = (int)fl;
  if ((m & (m - 1)) == 0) {
    i0 = b & (m - 1);
    i1 = (b + 1) & (m - 1);
  } else {
    b %= m;
    if (b < 0) b += m;
    i0 = b;
    i1 = (b + 1 == m) ? 0 : b + 1;
  }
}
__device__ __forceinline__ void repeat_axis_fast(float s, int m, int& i0, int& i1, float& a) {
  repeat_axis_fast(s, (float)m, m, i0, i1, a);
}

// Noise cells (REPEAT): cell (x0,y0,z0) holds the 8 corners; RGBA: 32 bytes, value-only: 8 bytes.
// The eight trilinear weights are formed once and applied to every channel.
//   EXACT (kCell): each byte becomes an exact float (byte_as_float) before the weighted sum,
//     the trilinear to float rounding.
//   !EXACT (kCellFast): each byte enters the weighted sum as 32768 + b (byte_biased) and the
//     bias comes off once per channel, because the weights sum to 1.  That saves one add per
//     corner and channel.  The accumulator then carries 8 bits below a noise step: the filtered
//     value is within 0.011 of a step (RMS 0.002, no bias) of the exact trilinear.  The texture
//     unit's 8-bit filter weights allow up to about 1.5 steps.
// Noise cells in memory: cell (x, y, z) at (z*my + y)*mx + x, in 32-bit arithmetic (noises up
// to 2^32 cells, 1625^3).  (A 2x2x2-blocked order measured within 1 % on the 512^3 orbit.)
__host__ __device__ __forceinline__ size_t noise_cell_index(int x, int y, int z, const int m[3]) {
  return (size_t)(((unsigned)z * (unsigned)m[1] + (unsigned)y) * (unsigned)m[0] + (unsigned)x);
}
__host__ __device__ __forceinline__ size_t noise_cell_count(const int m[3]) { return (size_t)m[0] * m[1] * m[2]; }

template <bool EXACT> struct NoiseCells {
  static __device__ __forceinline__ float corner(uint32_t w, int k) {
    return EXACT ? byte_as_float(w, k) : byte_biased(w, k);
  }
  template <bool RGBA, bool GRADC> static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 p) {
    int x0, x1, y0, y1, z0, z1;
    float ax, ay, az;
    repeat_axis_fast(p.x, GRADC ? a.nscale_grad[0] : a.nscale[0], a.m[0], x0, x1, ax);
    repeat_axis_fast(p.y, GRADC ? a.nscale_grad[1] : a.nscale[1], a.m[1], y0, y1, ay);
    repeat_axis_fast(p.z, GRADC ? a.nscale_grad[2] : a.nscale[2], a.m[2], z0, z1, az);
    const float k = 1.0f / 255.0f;
    const float bias = EXACT ? 0.0f : 32768.0f;
    const float bx = 1.0f - ax, by = 1.0f - ay, bz = 1.0f - az;
    const float w00 = by * bz, w10 = ay * bz, w01 = by * az, w11 = ay * az;
    const float w[8] = {bx * w00, ax * w00, bx * w10, ax * w10, bx * w01, ax * w01, bx * w11, ax * w11};
    size_t cidx = noise_cell_index(x0, y0, z0, a.m);
    if (VVLIC_BOUNDS_CHECK && !in_range(a, (long long)cidx, (long long)noise_cell_count(a.m), VVLIC_CHECK_NOISE))
      cidx = 0;
    if (RGBA) {
      uint32_t t[8];
      ldg256(reinterpret_cast<const uint4*>(a.noise) + 2 * cidx, t);
      float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        r.x = fmaf(w[i], corner(t[i], 0), r.x);
        r.y = fmaf(w[i], corner(t[i], 1), r.y);
        r.z = fmaf(w[i], corner(t[i], 2), r.z);
        r.w = fmaf(w[i], corner(t[i], 3), r.w);
      }
      return make_float4((r.x - bias) * k, (r.y - bias) * k, (r.z - bias) * k, (r.w - bias) * k);
    }
    const uint2 q = __ldg(reinterpret_cast<const uint2*>(a.noise) + cidx);
    float v = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      v = fmaf(w[i], corner(q.x, i), v);
      v = fmaf(w[4 + i], corner(q.y, i), v);
    }
    return make_float4(0.f, 0.f, 0.f, (v - bias) * k);
  }
};
template <> struct Noise<kCell> : NoiseCells<true> {};
template <> struct Noise<kCellFast> : NoiseCells<false> {};

// Noise through the texture unit: RGBA8 / R8 read as normalised float (x/255), LINEAR filter,
// WRAP addressing on normalised coordinates — GL's REPEAT.
template <> struct Noise<kTexture> {
  template <bool RGBA, bool GRADC> static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 p) {
    const float3 s = noise_coord<GRADC>(a, p);
    if (RGBA) return tex3D<float4>(a.noise_tex, s.x, s.y, s.z);
    return make_float4(0.f, 0.f, 0.f, tex3D<float>(a.noise_tex, s.x, s.y, s.z));
  }
};

// Value of the noise (.a): from an RGBA (-g) noise or a one-channel one.
template <int NL> __device__ __forceinline__ float noise_value(const RenderArgs& a, float3 p) {
  return a.noise_ch == 4 ? Noise<NL>::template sample<true, false>(a, p).w
                         : Noise<NL>::template sample<false, false>(a, p).w;
}

// Scalar-gate volume (freqSampling's scalarSampler), trilinear + CLAMP_TO_EDGE.  Not inlined:
// the gate is off unless a scalar volume is set, and keeping its gathers out of the tap loop's
// register allocation measured 2.4 % faster on the 64-volume unlit batch (1253 vs 1283 ms).
static __device__ __noinline__ float sample_scalar(const RenderArgs& a, float3 s) {
  int x0, x1, y0, y1, z0, z1;
  float ax, ay, az;
  clamp_axis(s.x, a.sn[0], x0, x1, ax);
  clamp_axis(s.y, a.sn[1], y0, y1, ay);
  clamp_axis(s.z, a.sn[2], z0, z1, az);
  const int nx = a.sn[0], nxy = a.sn[0] * a.sn[1];
  const float* t = a.scalar;
  if (VVLIC_BOUNDS_CHECK) {
    const long long n = (long long)nxy * a.sn[2];
    if (!in_range(a, (long long)z0 * nxy + y0 * nx + x0, n, VVLIC_CHECK_SCALAR) ||
        !in_range(a, (long long)z1 * nxy + y1 * nx + x1, n, VVLIC_CHECK_SCALAR))
      x0 = x1 = y0 = y1 = z0 = z1 = 0;
  }
  float c00 = lerpf(__ldg(t + z0 * nxy + y0 * nx + x0), __ldg(t + z0 * nxy + y0 * nx + x1), ax);
  float c10 = lerpf(__ldg(t + z0 * nxy + y1 * nx + x0), __ldg(t + z0 * nxy + y1 * nx + x1), ax);
  float c01 = lerpf(__ldg(t + z1 * nxy + y0 * nx + x0), __ldg(t + z1 * nxy + y0 * nx + x1), ax);
  float c11 = lerpf(__ldg(t + z1 * nxy + y1 * nx + x0), __ldg(t + z1 * nxy + y1 * nx + x1), ax);
  return lerpf(lerpf(c00, c10, ay), lerpf(c01, c11, ay), az);
}

// 1D LINEAR + CLAMP_TO_EDGE lookup in a 256-entry table (transferEdit.cpp:519-540), `tab`
// laid out with `stride` floats per entry.
__device__ __forceinline__ float tf1d(const float* tab, int stride, int ch, float s) {
  float u = fmaf(s, (float)VVLIC_TF_ENTRIES, -0.5f);
  u = fminf(fmaxf(u, -1.0f), (float)VVLIC_TF_ENTRIES);
  float fl = floorf(u);
  float t = u - fl;
  int b = (int)fl;
  int i0 = min(max(b, 0), VVLIC_TF_ENTRIES - 1), i1 = min(max(b + 1, 0), VVLIC_TF_ENTRIES - 1);
  return lerpf(tab[i0 * stride + ch], tab[i1 * stride + ch], t);
}
__device__ __forceinline__ float4 tf_rgba(const float* tab, float s) {
  float u = fmaf(s, (float)VVLIC_TF_ENTRIES, -0.5f);
  u = fminf(fmaxf(u, -1.0f), (float)VVLIC_TF_ENTRIES);
  float fl = floorf(u);
  float t = u - fl;
  int b = (int)fl;
  int i0 = min(max(b, 0), VVLIC_TF_ENTRIES - 1), i1 = min(max(b + 1, 0), VVLIC_TF_ENTRIES - 1);
  float4 a0 = reinterpret_cast<const float4*>(tab)[i0], a1 = reinterpret_cast<const float4*>(tab)[i1];
  return lerp4(a0, a1, t);
}

// ------------------------------------------------------------------------------------------
// LIC: computeLIC / singleLICstep (inc_lic.glsl:152-202, 93-145)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float3 slope(float4 f) { return f3(2.0f * f.x - 1.0f, 2.0f * f.y - 1.0f, 2.0f * f.z - 1.0f); }
// h * slope(f) rounded once: (2f - 1) * h = f * 2h - h, one FMA per component.  It keeps 2h
// and h live; RK4, which holds four slopes, keeps the two-step form to stay within the
// register cap.
__device__ __forceinline__ float3 slope_h(float4 f, float h) {
  const float h2 = 2.0f * h;
  return f3(fmaf(f.x, h2, -h), fmaf(f.y, h2, -h), fmaf(f.z, h2, -h));
}

// One streamline step; replaces `step` with the field value at the new position (the
// first-same-as-last reuse of the reference's `step` in/out argument).
template <int ST, int FL, int INTEG>
__device__ __forceinline__ float3 lic_step(const RenderArgs& a, float3 p, float4& step, float dirs) {
  using F = Field<ST, FL>;
  const float hs = a.sof ? a.h_eff * dirs * step.w : a.h_eff * dirs;
  float3 k1 = INTEG == VVLIC_RK4 ? scl3(slope(step), hs) : slope_h(step, hs);
  if (INTEG == VVLIC_EULER) {
    p = add3(p, k1);
  } else if (INTEG == VVLIC_HEUN) {
    float3 k2 = slope_h(F::sample(a, add3(p, k1)), hs);
    p = add3(p, scl3(add3(k1, k2), 0.5f));
  } else {
    float3 k2 = scl3(slope(F::sample(a, add3(p, scl3(k1, 0.5f)))), hs);
    float3 k3 = scl3(slope(F::sample(a, add3(p, scl3(k2, 0.5f)))), hs);
    float3 k4 = scl3(slope(F::sample(a, add3(p, k3))), hs);
    p = add3(p, scl3(add3(add3(k1, scl3(k2, 2.0f)), add3(scl3(k3, 2.0f), k4)), 1.0f / 6.0f));
  }
  step = F::sample(a, p);
  return p;
}

// freqSampling / freqSamplingGrad (inc_lic.glsl:71-90, 61-68)
template <int NL, bool GRAD> __device__ __forceinline__ float4 noise_tap(const RenderArgs& a, float3 p) {
  if (GRAD) return Noise<NL>::template sample<true, true>(a, p);
  if (a.gate) {
    float s = sample_scalar(a, p);
    if (!(s > a.gate_lo && s < a.gate_hi)) return make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (a.quirks & VVLIC_QUIRK_LUMINANCE_NOISE) return make_float4(0.f, 0.f, 0.f, 1.0f);
  return make_float4(0.f, 0.f, 0.f, noise_value<NL>(a, p));
}

template <bool GRAD> __device__ __forceinline__ void accumulate(float4& acc, float4 n, float w) {
  if (GRAD) {
    acc.x = fmaf(n.x, w, acc.x);
    acc.y = fmaf(n.y, w, acc.y);
    acc.z = fmaf(n.z, w, acc.z);
  }
  acc.w = fmaf(n.w, w, acc.w);
}

// computeLIC: (sum w*gradient_enc.xyz, sum w*noise); only .w without gradients.
// The backward and forward streamlines are independent, so they advance in the same loop
// iteration: two dependent gather chains per thread instead of one (the sum is reassociated
// relative to the reference's backward-then-forward order).
template <int ST, int FL, int NL, int INTEG, bool GRAD>
__device__ __forceinline__ float4 compute_lic(const RenderArgs& a, float3 pos, float4 f0) {
  const int lb = a.lb, lf = a.lf;
  const int both = min(lb, lf);
  float4 n0 = noise_tap<NL, GRAD>(a, pos);
  float w0 = a.taps[lb];
  float4 accb = make_float4(n0.x * w0, n0.y * w0, n0.z * w0, n0.w * w0);
  float4 accf = make_float4(0.f, 0.f, 0.f, 0.f);
  float3 pb = pos, pf = pos;
  float4 sb = f0, sf = f0;
  int i = 1;
  for (; i <= both; ++i) {
    pb = lic_step<ST, FL, INTEG>(a, pb, sb, -1.0f);
    pf = lic_step<ST, FL, INTEG>(a, pf, sf, 1.0f);
    float4 nb = noise_tap<NL, GRAD>(a, pb);
    float4 nf = noise_tap<NL, GRAD>(a, pf);
    accumulate<GRAD>(accb, nb, a.taps[lb - i]);
    accumulate<GRAD>(accf, nf, a.taps[lb + i]);
  }
  for (int j = i; j <= lb; ++j) {
    pb = lic_step<ST, FL, INTEG>(a, pb, sb, -1.0f);
    accumulate<GRAD>(accb, noise_tap<NL, GRAD>(a, pb), a.taps[lb - j]);
  }
  for (int j = i; j <= lf; ++j) {
    pf = lic_step<ST, FL, INTEG>(a, pf, sf, 1.0f);
    accumulate<GRAD>(accf, noise_tap<NL, GRAD>(a, pf), a.taps[lb + j]);
  }
  return make_float4(accb.x + accf.x, accb.y + accf.y, accb.z + accf.z, accb.w + accf.w);
}

// computeLIC of two samples at once (four independent gather chains per thread).  Each sample's
// sums are formed in exactly the order compute_lic uses, so the results are bit-identical.
template <int ST, int FL, int NL, int INTEG, bool GRAD>
__device__ __forceinline__ void compute_lic2(const RenderArgs& a, float3 pa, float4 fa, float3 pbp, float4 fb,
                                             float4& out_a, float4& out_b) {
  const int lb = a.lb, lf = a.lf;
  const int both = min(lb, lf);
  const float w0 = a.taps[lb];
  float4 accab, accaf = make_float4(0.f, 0.f, 0.f, 0.f), accbb, accbf = make_float4(0.f, 0.f, 0.f, 0.f);
  {
    const float4 na = noise_tap<NL, GRAD>(a, pa), nb = noise_tap<NL, GRAD>(a, pbp);
    accab = make_float4(na.x * w0, na.y * w0, na.z * w0, na.w * w0);
    accbb = make_float4(nb.x * w0, nb.y * w0, nb.z * w0, nb.w * w0);
  }
  float3 p0 = pa, p1 = pa, p2 = pbp, p3 = pbp;
  float4 s0 = fa, s1 = fa, s2 = fb, s3 = fb;
  int i = 1;
  for (; i <= both; ++i) {
    p0 = lic_step<ST, FL, INTEG>(a, p0, s0, -1.0f);
    p1 = lic_step<ST, FL, INTEG>(a, p1, s1, 1.0f);
    p2 = lic_step<ST, FL, INTEG>(a, p2, s2, -1.0f);
    p3 = lic_step<ST, FL, INTEG>(a, p3, s3, 1.0f);
    const float4 n0 = noise_tap<NL, GRAD>(a, p0), n1 = noise_tap<NL, GRAD>(a, p1);
    const float4 n2 = noise_tap<NL, GRAD>(a, p2), n3 = noise_tap<NL, GRAD>(a, p3);
    const float wb = a.taps[lb - i], wf = a.taps[lb + i];
    accumulate<GRAD>(accab, n0, wb);
    accumulate<GRAD>(accaf, n1, wf);
    accumulate<GRAD>(accbb, n2, wb);
    accumulate<GRAD>(accbf, n3, wf);
  }
  for (int j = i; j <= lb; ++j) {
    p0 = lic_step<ST, FL, INTEG>(a, p0, s0, -1.0f);
    p2 = lic_step<ST, FL, INTEG>(a, p2, s2, -1.0f);
    accumulate<GRAD>(accab, noise_tap<NL, GRAD>(a, p0), a.taps[lb - j]);
    accumulate<GRAD>(accbb, noise_tap<NL, GRAD>(a, p2), a.taps[lb - j]);
  }
  for (int j = i; j <= lf; ++j) {
    p1 = lic_step<ST, FL, INTEG>(a, p1, s1, 1.0f);
    p3 = lic_step<ST, FL, INTEG>(a, p3, s3, 1.0f);
    accumulate<GRAD>(accaf, noise_tap<NL, GRAD>(a, p1), a.taps[lb + j]);
    accumulate<GRAD>(accbf, noise_tap<NL, GRAD>(a, p3), a.taps[lb + j]);
  }
  out_a = make_float4(accab.x + accaf.x, accab.y + accaf.y, accab.z + accaf.z, accab.w + accaf.w);
  out_b = make_float4(accbb.x + accbf.x, accbb.y + accbf.y, accbb.z + accbf.z, accbb.w + accbf.w);
}

// ------------------------------------------------------------------------------------------
// shading: illumLIC (inc_illum.glsl:158-172) and illumGradient (inc_illum.glsl:1-41)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float alpha_correct(float al, float corr) {
  float base = fmaxf(1.0f - al, 0.0f);
  return 1.0f - powf(base, corr);
}

__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// texture2D on an RGBA8 table with LINEAR + CLAMP_TO_EDGE (illumination.cpp:335-346): texel
// centres at (i + 0.5) / w.  Clamping the coordinate to [0, 1] first is the same for finite
// coordinates and sends a NaN one (a degenerate tangent) to the edge texel.
__device__ __forceinline__ float4 lut2d(const uchar4* t, int w, int h, float s, float r) {
  s = fminf(fmaxf(s, 0.0f), 1.0f);
  r = fminf(fmaxf(r, 0.0f), 1.0f);
  const float u = s * (float)w - 0.5f, v = r * (float)h - 0.5f;
  const float fu = floorf(u), fv = floorf(v);
  const float au = u - fu, av = v - fv;
  const int x0 = max((int)fu, 0), x1 = min((int)fu + 1, w - 1);
  const int y0 = max((int)fv, 0), y1 = min((int)fv + 1, h - 1);
  const uchar4 c00 = __ldg(t + y0 * w + x0), c10 = __ldg(t + y0 * w + x1);
  const uchar4 c01 = __ldg(t + y1 * w + x0), c11 = __ldg(t + y1 * w + x1);
  const float k = 1.0f / 255.0f;
  const float w00 = (1.0f - au) * (1.0f - av) * k, w10 = au * (1.0f - av) * k;
  const float w01 = (1.0f - au) * av * k, w11 = au * av * k;
  return make_float4(w00 * c00.x + w10 * c10.x + w01 * c01.x + w11 * c11.x,
                     w00 * c00.y + w10 * c10.y + w01 * c01.y + w11 * c11.y,
                     w00 * c00.z + w10 * c10.z + w01 * c01.z + w11 * c11.z,
                     w00 * c00.w + w10 * c10.w + w01 * c01.w + w11 * c11.w);
}

// Light direction of every illumination model: normalize(light - pos * scaleVolInv).
__device__ __forceinline__ float3 light_dir(const RenderArgs& a, float3 pos) {
  return norm3(sub3(f3(a.light_pos[0], a.light_pos[1], a.light_pos[2]),
                    mul3(pos, f3(a.scale_vol_inv[0], a.scale_vol_inv[1], a.scale_vol_inv[2]))));
}

// Illuminated-streamline factors of one sample: colour = tf.rgb * I * d + s with d and s from
// the line tables.  `f` is the field sample at `pos` (vectorData), whose encoded direction is
// the streamline tangent.
//   illumZoeckler (inc_illum.glsl:117-154): (L.T, V.T)/2 + 1/2 into the table, V = n(dir);
//     d = L_d * illumScale, s = 0.9 * g (g = L_d with the luminance quirk, else the stored specular);
//   illumMallo (inc_illum.glsl:46-112): B = n(T x V), N = B x T, H = n(V + L), V = n(-dir);
//     d = diffuse(LN/sqrt(1-LT^2), LT) * illumScale,
//     s = sat(specular(LN/sqrt(1-LT^2), HN/sqrt(1-HT^2)) * (1-HT^2)^(e/2)).
__device__ __forceinline__ void line_factors(const RenderArgs& a, float3 pos, float3 dir, float4 f, float3& d,
                                             float3& s) {
  const float3 L = light_dir(a, pos);
  const float3 T = norm3(f3(2.0f * f.x - 1.0f, 2.0f * f.y - 1.0f, 2.0f * f.z - 1.0f));
  if (a.illum == VVLIC_ILLUM_ZOECKLER) {
    const float3 V = norm3(dir);
    const float4 sh = lut2d(a.luts, a.lut_w, a.lut_h, 0.5f * dot3(L, T) + 0.5f, 0.5f * dot3(V, T) + 0.5f);
    const float dd = sh.x * a.illum_scale;
    const float sp = 0.9f * ((a.quirks & VVLIC_QUIRK_ZOECKLER_LUMINANCE) ? sh.y : sh.w);
    d = f3(dd, dd, dd);
    s = f3(sp, sp, sp);
  } else {
    const float3 V = norm3(scl3(dir, -1.0f));
    const float3 B = norm3(cross3(T, V));
    const float3 N = cross3(B, T);
    const float3 Hv = norm3(add3(V, L));
    const float ln = dot3(L, N), lt = dot3(L, T), hn = dot3(Hv, N), ht = dot3(Hv, T);
    const float rl = 1.0f / sqrtf(1.0f - lt * lt), rh = 1.0f / sqrtf(1.0f - ht * ht);
    const float cz = 0.5f * (ln * rl) + 0.5f, cy = 0.5f * lt + 0.5f, cw = 0.5f * (hn * rh) + 0.5f;
    const size_t one = (size_t)a.lut_w * a.lut_h;
    const float4 df = lut2d(a.luts + one, a.lut_w, a.lut_h, cz, cy);
    const float4 sc = lut2d(a.luts + 2 * one, a.lut_w, a.lut_h, cz, cw);
    const float att = powf(rh, -a.spec_exp);  // (1 - (H.T)^2)^(n/2)
    d = scl3(f3(df.x, df.y, df.z), a.illum_scale);
    s = f3(__saturatef(sc.x * att), __saturatef(sc.y * att), __saturatef(sc.z * att));
  }
}

// GRAD kernels (noise gradients fetched) only ever shade with illumGradient; the others with
// illumLIC, illumZoeckler or illumMallo.
template <bool GRAD>
__device__ __forceinline__ float4 shade(const RenderArgs& a, const float* s_tf, float4 il, float4 tf, float3 pos,
                                        float3 dir, float4 f) {
  const float I = il.w;
  float4 col;
  if (!GRAD && (a.illum == VVLIC_ILLUM_ZOECKLER || a.illum == VVLIC_ILLUM_MALLO)) {
    float3 d, s;
    line_factors(a, pos, dir, f, d, s);
    col.x = tf.x * I * d.x + s.x;
    col.y = tf.y * I * d.y + s.y;
    col.z = tf.z * I * d.z + s.z;
  } else if (GRAD) {
    float3 L = light_dir(a, pos);
    float3 V = norm3(scl3(dir, -1.0f));
    float3 N = norm3(f3(-il.x, -il.y, -il.z));
    float3 R = norm3(sub3(scl3(N, 2.0f * dot3(L, N)), L));
    float sp = powf(__saturatef(dot3(R, V)), a.spec_exp) * I;
    float df = __saturatef(dot3(L, N)) * a.illum_scale;
    col.x = (tf.x * I * (a.light_diff[0] * df + 0.3f + a.light_amb[0]) + a.light_spec[0] * sp) * a.illum_scale;
    col.y = (tf.y * I * (a.light_diff[1] * df + 0.3f + a.light_amb[1]) + a.light_spec[1] * sp) * a.illum_scale;
    col.z = (tf.z * I * (a.light_diff[2] * df + 0.3f + a.light_amb[2]) + a.light_spec[2] * sp) * a.illum_scale;
  } else {
    col.x = I * tf.x * a.illum_scale;
    col.y = I * tf.y * a.illum_scale;
    col.z = I * tf.z * a.illum_scale;
  }
  float al = tf1d(s_tf + 4 * VVLIC_TF_ENTRIES, 1, 0, I * 1.3f) * tf.w;
  col.w = alpha_correct(al, a.alpha_corr);
  return col;
}

// Front-to-back blend with per-step clamp (lic3d_fragment.glsl:83-84).
__device__ __forceinline__ float4 blend(float4 dest, float4 src) {
  src.x *= src.w;
  src.y *= src.w;
  src.z *= src.w;
  const float om = 1.0f - dest.w;
  return make_float4(__saturatef(fmaf(om, src.x, dest.x)), __saturatef(fmaf(om, src.y, dest.y)),
                     __saturatef(fmaf(om, src.z, dest.z)), __saturatef(fmaf(om, src.w, dest.w)));
}

// Parametric interval of a pixel's ray inside [0, extent] (the cube faces the reference
// rasterises, renderer.cpp:682-736); false for a miss.
__device__ __forceinline__ bool ray_interval(const RenderArgs& a, int px, int py, float o[3], float d[3], float& tn,
                                             float& tf) {
  const float u = (float)px + 0.5f, v = (float)py + 0.5f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    o[i] = a.o0[i] + u * a.o1[i] + v * a.o2[i];
    d[i] = a.d0[i] + u * a.d1[i] + v * a.d2[i];
  }
  tn = -INFINITY;
  tf = INFINITY;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (d[i] == 0.0f) {
      if (o[i] < 0.0f || o[i] > a.ext[i]) return false;
      continue;
    }
    float inv = 1.0f / d[i];
    float t0 = (0.0f - o[i]) * inv, t1 = (a.ext[i] - o[i]) * inv;
    tn = fmaxf(tn, fminf(t0, t1));
    tf = fminf(tf, fmaxf(t0, t1));
  }
  if (!(tn < tf)) return false;
  if (a.clamp0) {
    if (!(tf > 0.0f)) return false;
    tn = fmaxf(tn, 0.0f);
  }
  return true;
}

// Per-pixel ray start: pos = objPos * scaleVol, dir = normalize(objPos - eye) * scaleVol
// (lic3d_fragment.glsl:12-21).
__device__ __forceinline__ bool ray_setup(const RenderArgs& a, int px, int py, float3& pos, float3& dir) {
  float o[3], d[3], tn, tf;
  if (!ray_interval(a, px, py, o, d, tn, tf)) return false;
  const float3 sv = f3(a.scale_vol[0], a.scale_vol[1], a.scale_vol[2]);
  pos = mul3(f3(o[0] + tn * d[0], o[1] + tn * d[1], o[2] + tn * d[2]), sv);
  dir = mul3(norm3(f3(d[0], d[1], d[2])), sv);
  return true;
}

__device__ __forceinline__ bool outside_box(const RenderArgs& a, float3 p) {
  return p.x < 0.0f || p.y < 0.0f || p.z < 0.0f || p.x > a.tex_max[0] || p.y > a.tex_max[1] || p.z > a.tex_max[2];
}

// Adjoint tape layout: rays grouped in 8x4-pixel tiles (the queue schedule's warp tiles) and,
// within a tile, sample-major with the tile's 32 rays adjacent, so that a warp recording or
// replaying sample k of its tile touches 32 consecutive entries.
constexpr int kTapeTileW = 8, kTapeTileH = 4;
__device__ __forceinline__ size_t tape_tile(const RenderArgs& a, int px, int py) {
  return (size_t)(py / kTapeTileH) * (size_t)((a.W + kTapeTileW - 1) / kTapeTileW) + (size_t)(px / kTapeTileW);
}
__device__ __forceinline__ size_t tape_lane(int px, int py) {
  return (size_t)((py % kTapeTileH) * kTapeTileW + px % kTapeTileW);
}
// tape_is / tape_g entry of sample k of the ray at (px, py)
__device__ __forceinline__ size_t tape_entry(const RenderArgs& a, int px, int py, uint32_t k) {
  return (tape_tile(a, px, py) * (size_t)a.tape_stride + k) * 32 + tape_lane(px, py);
}
// checkpoint of segment s: position at the returned index, dest 32 entries later
__device__ __forceinline__ size_t tape_ck_entry(const RenderArgs& a, int px, int py, uint32_t s) {
  return (tape_tile(a, px, py) * (size_t)a.tape_nck + s) * 64 + tape_lane(px, py);
}
// entries of the per-sample arrays and of the checkpoint array (VVLIC_BOUNDS_CHECK builds)
__device__ __forceinline__ long long tape_entries(const RenderArgs& a) {
  return (long long)((a.W + kTapeTileW - 1) / kTapeTileW) * ((a.H + kTapeTileH - 1) / kTapeTileH) * 32 *
         a.tape_stride;
}
__device__ __forceinline__ long long tape_ck_entries(const RenderArgs& a) {
  return (long long)((a.W + kTapeTileW - 1) / kTapeTileW) * ((a.H + kTapeTileH - 1) / kTapeTileH) * 64 *
         a.tape_nck;
}
__device__ __forceinline__ size_t tape_entry_checked(const RenderArgs& a, int px, int py, uint32_t k) {
  const size_t e = tape_entry(a, px, py, k);
  return in_range(a, (long long)e, tape_entries(a), VVLIC_CHECK_TAPE) ? e : 0;
}

// The whole lic3d_fragment.glsl main() for one pixel: returns dest, counts samples.
template <int ST, int FL, int NL, int INTEG, bool GRAD>
__device__ __forceinline__ float4 trace_pixel(const RenderArgs& a, const float* s_tf, int px, int py,
                                              uint32_t& samples, uint32_t& hit) {
  float4 dest = make_float4(0.f, 0.f, 0.f, 0.f);
  float3 pos, dir;
  samples = 0;
  hit = 0;
  if (!ray_setup(a, px, py, pos, dir)) return dest;
  hit = 1;
  float4 src = make_float4(0.f, 0.f, 0.f, 0.f);
  bool outside = false;
  for (int j = 0; !outside && j < a.num_iter; ++j) {
    for (int i = 0; i < a.num_iter; ++i) {
      const float4 f = Field<ST, FL>::sample(a, pos);
      const float tfc = a.tf_index == VVLIC_TF_INDEX_MAGNITUDE ? f.w : f.z;
      const float4 tf = tf_rgba(s_tf, tfc);
      float4 il = compute_lic<ST, FL, NL, INTEG, GRAD>(a, pos, f);
      il.w *= a.intensity_scale;
      if (a.tape_is) {  // record for the adjoint
        if (samples % kSegment == 0 && samples / kSegment < (uint32_t)a.tape_nck) {
          const size_t ce = tape_ck_entry(a, px, py, samples / kSegment);
          if (in_range(a, (long long)ce + 32, tape_ck_entries(a), VVLIC_CHECK_TAPE)) {
            float4* ck = a.tape_ck + ce;
            ck[0] = make_float4(pos.x, pos.y, pos.z, 0.f);
            ck[32] = dest;
          }
        }
        if (samples < (uint32_t)a.tape_stride &&
            in_range(a, (long long)tape_entry(a, px, py, samples), tape_entries(a), VVLIC_CHECK_TAPE)) {
          const size_t e = tape_entry(a, px, py, samples);
          a.tape_is[e] = make_float2(il.w, tfc);
          if (GRAD) {
            const __half2 xy = __floats2half2_rn(il.x, il.y), z0 = __floats2half2_rn(il.z, 0.0f);
            a.tape_g[e] = make_uint2(*reinterpret_cast<const unsigned*>(&xy), *reinterpret_cast<const unsigned*>(&z0));
          }
        }
      }
      ++samples;
      src = shade<GRAD>(a, s_tf, il, tf, pos, dir, f);
      dest = blend(dest, src);
      pos = add3(pos, scl3(dir, a.step_size));
      outside = outside_box(a, pos) || src.w > a.alpha_thr;
      if (outside) break;
    }
  }
  return dest;
}

// trace_pixel computing the LIC of two consecutive samples together (compute_lic2).  The second
// sample's LIC is speculative: it is discarded when the first sample ends the ray.  Samples,
// images and tapes are identical to trace_pixel's; the nested numIterations loops become one
// bound of numIterations^2 samples (the outer loop only re-enters the inner one).
template <int ST, int FL, int NL, int INTEG, bool GRAD>
__device__ __forceinline__ float4 trace_pixel2(const RenderArgs& a, const float* s_tf, int px, int py,
                                               uint32_t& samples, uint32_t& hit) {
  float4 dest = make_float4(0.f, 0.f, 0.f, 0.f);
  float3 pos, dir;
  samples = 0;
  hit = 0;
  if (!ray_setup(a, px, py, pos, dir)) return dest;
  hit = 1;
  const uint32_t max_samples = (uint32_t)a.num_iter * (uint32_t)a.num_iter;
  const float3 dstep = scl3(dir, a.step_size);
  while (samples < max_samples) {
    const float3 pos1 = add3(pos, dstep);
    const float4 f0 = Field<ST, FL>::sample(a, pos), f1 = Field<ST, FL>::sample(a, pos1);
    float4 il[2];
    compute_lic2<ST, FL, NL, INTEG, GRAD>(a, pos, f0, pos1, f1, il[0], il[1]);
    bool outside = false;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const float4 f = k == 0 ? f0 : f1;
      const float3 p = k == 0 ? pos : pos1;
      const float tfc = a.tf_index == VVLIC_TF_INDEX_MAGNITUDE ? f.w : f.z;
      const float4 tf = tf_rgba(s_tf, tfc);
      float4 l = il[k];
      l.w *= a.intensity_scale;
      if (a.tape_is) {  // record for the adjoint
        if (samples % kSegment == 0 && samples / kSegment < (uint32_t)a.tape_nck) {
          const size_t ce = tape_ck_entry(a, px, py, samples / kSegment);
          if (in_range(a, (long long)ce + 32, tape_ck_entries(a), VVLIC_CHECK_TAPE)) {
            float4* ck = a.tape_ck + ce;
            ck[0] = make_float4(p.x, p.y, p.z, 0.f);
            ck[32] = dest;
          }
        }
        if (samples < (uint32_t)a.tape_stride &&
            in_range(a, (long long)tape_entry(a, px, py, samples), tape_entries(a), VVLIC_CHECK_TAPE)) {
          const size_t e = tape_entry(a, px, py, samples);
          a.tape_is[e] = make_float2(l.w, tfc);
          if (GRAD) {
            const __half2 xy = __floats2half2_rn(l.x, l.y), z0 = __floats2half2_rn(l.z, 0.0f);
            a.tape_g[e] = make_uint2(*reinterpret_cast<const unsigned*>(&xy), *reinterpret_cast<const unsigned*>(&z0));
          }
        }
      }
      ++samples;
      const float4 src = shade<GRAD>(a, s_tf, l, tf, p, dir, f);
      dest = blend(dest, src);
      // the reference's position update pos += dir * stepSize, then its exit test
      pos = add3(p, dstep);
      outside = outside_box(a, pos) || src.w > a.alpha_thr || samples >= max_samples;
      if (outside) break;
    }
    if (outside) break;
  }
  return dest;
}

// Samples whose LIC one thread computes together: 1 (trace_pixel) or 2 (trace_pixel2, twice the
// independent gather chains per thread at more registers per thread).  RK4 kernels, whose four
// serial fetches per step leave a thread mostly waiting, take two: on the 512^3 / 2048^2 RK4
// orbit frames 106.0 against 103.3 Gsample-steps/s at 128 registers (4 CTAs/SM; 102 registers
// measured 105.7).  Euler and Heun kernels take one (two measured +1 % on the lit 1024^2 Heun
// frame with the texture field, -9 % with the cell field).
#ifndef VVLIC_SAMPLES_PER_PASS
#define VVLIC_SAMPLES_PER_PASS 1
#endif
#ifndef VVLIC_RK4_SAMPLES_PER_PASS
#define VVLIC_RK4_SAMPLES_PER_PASS 2
#endif
template <int ST, int FL, int NL, int INTEG, bool GRAD>
__device__ __forceinline__ float4 trace_ray(const RenderArgs& a, const float* s_tf, int px, int py,
                                            uint32_t& samples, uint32_t& hit) {
  constexpr int spp = INTEG == VVLIC_RK4 ? VVLIC_RK4_SAMPLES_PER_PASS : VVLIC_SAMPLES_PER_PASS;
  if constexpr (spp == 2) return trace_pixel2<ST, FL, NL, INTEG, GRAD>(a, s_tf, px, py, samples, hit);
  else return trace_pixel<ST, FL, NL, INTEG, GRAD>(a, s_tf, px, py, samples, hit);
}

}  // namespace vvlic
