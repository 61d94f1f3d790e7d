/*
 * ORACLE — test infrastructure, not product code.
 *
 * A CPU restatement of the voLIC LIC ray-casting hot path (liaoyg/VectorVisualization), written
 * to be checked against and timed beside the CUDA kernels.  Only tests/, the smoke check and
 * bench.py's CPU-baseline / reference arm may call it.  Nothing in the product links it.
 *
 * One template over the arithmetic type Real gives
 *   - the FP64 correctness oracle (Real = double), and
 *   - the FP32 OpenMP CPU baseline (Real = float).
 *
 * What it follows (file:line within VectorVisualization/):
 *   GLSL hot path      shader/lic3d_fragment.glsl:5-99, shader/inc_lic.glsl:61-202,
 *                      shader/inc_illum.glsl:1-172, shader/inc_header.glsl:22-63
 *   other techniques   shader/lic3d_slicing_fragment.glsl, vectorfield_fragment.glsl:39-101,
 *                      lic3d_volume_fragment.glsl, raycast_lic3d_fragment.glsl, slicing.cpp:42-103
 *   uniforms           renderer.cpp:925-996 (setRenderVolParams)
 *   volume geometry    dataset.cpp:139-176 (VectorDataSet::loadData)
 *   view               camera.cpp:56-67 (Camera::setCamera), renderer.cpp:146, 682-736
 *   field encoding     dataset.cpp:533-635 (fillTexDataFloatInterp, with its time lerp)
 *   noise gradients    gradient.cpp:190-531, gradient.h:37-39, dataset.cpp:1270-1286
 *   filter kernel      dataset.cpp:1405-1413, 1470-1512
 *   transfer function  transferEdit.cpp:76-82, 480-543
 *   line illumination  illumination.cpp:96-391 (Zoeckler and Mallo tables)
 *   adjoint            reverse mode of the above (no reference counterpart), FD-checked
 * GL sampler behaviour (texel centres, LINEAR, CLAMP_TO_EDGE / REPEAT / GL_CLAMP with a zero
 * border, uint8 read as x/255) is restated from the OpenGL 2.1 specification, section 3.8.
 *
 * Parity of the GLSL part is unpinned by reference tests (the reference has none and its
 * inputs are not shipped); the noise gradients are pinned against the reference's own
 * gradient.cpp and the .dat reader against its reader.cpp, both compiled here
 * (oracle/build_ref.sh).
 */
#ifndef VVLIC_ORACLE_HPP_
#define VVLIC_ORACLE_HPP_

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/vvlic.h"

#if defined(_OPENMP)
#include <omp.h>
#endif

namespace vvo {

/* ------------------------------------------------------------------------------------- */
/* small vector types                                                                     */
/* ------------------------------------------------------------------------------------- */
template <class R> struct V3 { R x, y, z; };
template <class R> struct V4 { R x, y, z, w; };

template <class R> static inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> static inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> static inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> static inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> static inline V3<R> mul(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> static inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* normalize(0) is defined as 0 (GLSL leaves it undefined). */
template <class R> static inline V3<R> normalize(V3<R> a) {
  R d = dot(a, a);
  if (!(d > R(0))) return {R(0), R(0), R(0)};
  R s = R(1) / std::sqrt(d);
  return a * s;
}
template <class R> static inline R clamp01(R v) { return v < R(0) ? R(0) : (v > R(1) ? R(1) : v); }

/* ------------------------------------------------------------------------------------- */
/* volume geometry: VectorDataSet::loadData (dataset.cpp:139-176)                          */
/* ------------------------------------------------------------------------------------- */
struct Geometry {
  double scale[3], scale_inv[3], extent[3], center[3], tex_max[3];
};

static inline Geometry geometry(const int n[3], const float sd_in[3]) {
  Geometry g;
  float sd[3] = {1.f, 1.f, 1.f};
  if (sd_in) for (int i = 0; i < 3; ++i) sd[i] = sd_in[i];
  /* the reference computes these in float */
  float vol_size[3], max_vol = 0.f;
  int max_tex = 0;
  for (int i = 0; i < 3; ++i) {
    vol_size[i] = (float)n[i] * sd[i];
    if (vol_size[i] > max_vol) max_vol = vol_size[i];
    if (n[i] > max_tex) max_tex = n[i];
  }
  for (int i = 0; i < 3; ++i) {
    float scale = (float)max_tex / ((float)n[i] * sd[i]);
    float scale_inv = (float)n[i] * sd[i] / (float)max_tex;
    float extent = (float)n[i] * sd[i] / max_vol;
    g.scale[i] = scale;
    g.scale_inv[i] = scale_inv;
    g.extent[i] = extent;
    g.center[i] = extent / 2.0f;
    g.tex_max[i] = (double)(extent * scale); /* renderer.cpp:934-937 (float product) */
  }
  return g;
}

/* ------------------------------------------------------------------------------------- */
/* field encoding: fillTexDataFloatInterp (dataset.cpp:533-635).  `next` == NULL is          */
/* interpIndex = 0 (the static upload); otherwise each component is the lerp                */
/* data + t * (next - data), t = (float)interpIndex / InterpSize, evaluated in float as     */
/* dataset.cpp:570 / :593 do, the UCHAR3 lerp truncated back to unsigned char.              */
/* float arithmetic exactly as the reference performs it; compile with -ffp-contract=off.  */
/* An all-zero field (maxLen = 0) gets magnitude 0 where the reference would divide 0/0.   */
/* ------------------------------------------------------------------------------------- */
static inline void encode_field_interp(const void* xyz, const void* next, float t, int dtype, const int n[3],
                                       float* out_rgba) {
  const size_t count = (size_t)n[0] * n[1] * n[2];
  float max_len = -1.0f;
  for (size_t a = 0; a < count; ++a) {
    float len;
    float* o = out_rgba + 4 * a;
    if (dtype == VVLIC_DTYPE_UINT8) {
      /* dataU -= 128 on unsigned char wraps modulo 256 (dataset.cpp:565-569) */
      const uint8_t* u = (const uint8_t*)xyz + 3 * a;
      const uint8_t* w = next ? (const uint8_t*)next + 3 * a : nullptr;
      unsigned char v[3];
      for (int c = 0; c < 3; ++c) {
        const unsigned char d = (unsigned char)(u[c] - 128);
        if (!w) {
          v[c] = d;
        } else {
          const unsigned char e = (unsigned char)(w[c] - 128);
          v[c] = (unsigned char)((float)d + t * (float)((int)e - (int)d));
        }
      }
      len = std::sqrt((float)((int)v[0] * v[0]) + (float)((int)v[1] * v[1]) + (float)((int)v[2] * v[2]));
      if (len < 1e-5f) {
        len = 0.0f;
        o[0] = o[1] = o[2] = 0.5f;
      } else {
        for (int c = 0; c < 3; ++c) o[c] = 0.5f * (float)v[c] / len + 0.5f;
      }
    } else {
      const float* f0 = (const float*)xyz + 3 * a;
      float f[3];
      for (int c = 0; c < 3; ++c) f[c] = next ? f0[c] + t * (((const float*)next)[3 * a + c] - f0[c]) : f0[c];
      len = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
      if (len < 1e-5f) {
        len = 0.0f;
        o[0] = o[1] = o[2] = 0.5f;
      } else {
        for (int c = 0; c < 3; ++c) o[c] = 0.5f * f[c] / len + 0.5f;
      }
    }
    if (len > max_len) max_len = len;
    o[3] = len;
  }
  for (size_t a = 0; a < count; ++a) {
    float* o = out_rgba + 4 * a;
    float len = max_len > 0.0f ? o[3] / max_len : 0.0f;
    o[3] = (len > 1.0f) ? 1.0f : ((len < 0.0f) ? 0.0f : len);
  }
}
static inline void encode_field(const void* xyz, int dtype, const int n[3], float* out_rgba) {
  encode_field_interp(xyz, nullptr, 0.0f, dtype, n, out_rgba);
}

/* Round-to-nearest-even to FP16 / BF16 and back, the storage emulation used to compare with
 * reduced-precision field storage (the reference itself stores RGBA16F). */
static inline float round_to_f16(float f) {
  if (std::isnan(f)) return f;
  float a = std::fabs(f);
  if (a >= 65520.0f) return std::copysign(INFINITY, f);
  if (a < 6.103515625e-05f) { /* subnormal half: quantum 2^-24 */
    float q = std::nearbyint(a * 16777216.0f) / 16777216.0f;
    return std::copysign(q, f);
  }
  int e;
  std::frexp(a, &e); /* a = m * 2^e, m in [0.5,1) */
  float quantum = std::ldexp(1.0f, e - 11);
  float q = std::nearbyint(a / quantum) * quantum;
  return std::copysign(q, f);
}
static inline float round_to_bf16(float f) {
  if (std::isnan(f)) return f;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;
  u &= 0xffff0000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}
/* nearest multiple of 1/255: x*255 rounded in float, then to the nearest integer (ties even) */
static inline float round_to_unorm8(float f) {
  float q = std::nearbyint(f * 255.0f);
  q = q < 0.0f ? 0.0f : (q > 255.0f ? 255.0f : q);
  return q / 255.0f;
}
static inline void round_storage(float* v, size_t count, int storage) {
  if (storage == VVLIC_STORAGE_F16)
    for (size_t i = 0; i < count; ++i) v[i] = round_to_f16(v[i]);
  else if (storage == VVLIC_STORAGE_BF16)
    for (size_t i = 0; i < count; ++i) v[i] = round_to_bf16(v[i]);
  else if (storage == VVLIC_STORAGE_UNORM8)
    for (size_t i = 0; i < count; ++i) v[i] = round_to_unorm8(v[i]);
}

/* ------------------------------------------------------------------------------------- */
/* noise gradients: computeGradients / filterGradients / quantizeGradients                */
/* (gradient.cpp:190-531; GRAD_FILTER_SIZE 5, SIGMA2 5.0f, gradient.h:38-39), RGBA pack    */
/* (dataset.cpp:1270-1286).  Float arithmetic in the reference's order.                    */
/* ------------------------------------------------------------------------------------- */
static inline void noise_gradient_filter_weights(float w[27]) {
  /* filter[((fw+k)*5 + fw+j)*5 + fw+i] for i,j,k in [-2, 0] (gradient.cpp:393-409) */
  float sum = 0.0f;
  int idx = 0;
  for (int k = -2; k < 1; ++k)
    for (int j = -2; j < 1; ++j)
      for (int i = -2; i < 1; ++i) {
        float v = std::exp(-(float)(i * i + j * j + k * k) / 5.0f);
        w[idx++] = v;
        sum += v;
      }
  for (int q = 0; q < 27; ++q) w[q] /= sum;
}

static inline void noise_gradients(const uint8_t* noise, const int m[3], int mode,
                                   const float* sd_in, uint8_t* out_rgba) {
  const int nx = m[0], ny = m[1], nz = m[2];
  float sd[3] = {1.f, 1.f, 1.f};
  if (sd_in) for (int i = 0; i < 3; ++i) sd[i] = sd_in[i];
  const size_t count = (size_t)nx * ny * nz;
  std::vector<float> g(3 * count), fg(3 * count);
  auto V = [&](int x, int y, int z) -> float { return (float)noise[((size_t)z * ny + y) * nx + x]; };
  /* Sobel weights, weights[dir][i+1][j+1][k+1] (gradient.cpp:199-224) */
  static const int W[3][3][3][3] = {
      {{{-1, -3, -1}, {-3, -6, -3}, {-1, -3, -1}}, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, {{1, 3, 1}, {3, 6, 3}, {1, 3, 1}}},
      {{{-1, -3, -1}, {0, 0, 0}, {1, 3, 1}}, {{-3, -6, -3}, {0, 0, 0}, {3, 6, 3}}, {{-1, -3, -1}, {0, 0, 0}, {1, 3, 1}}},
      {{{-1, 0, 1}, {-3, 0, 3}, {-1, 0, 1}}, {{-3, 0, 3}, {-6, 0, 6}, {-3, 0, 3}}, {{-1, 0, 1}, {-3, 0, 3}, {-1, 0, 1}}}};
  /* slices in parallel: every voxel's sums keep their order, so the result is thread-count free */
#if defined(_OPENMP)
#pragma omp parallel for schedule(static)
#endif
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        float* gp = &g[3 * (((size_t)z * ny + y) * nx + x)];
        if (mode == VVLIC_NOISE_GRAD_SOBEL) {
          if (x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1) {
            for (int d = 0; d < 3; ++d) {
              gp[d] = 0.0f;
              for (int i = -1; i < 2; i++)
                for (int j = -1; j < 2; j++)
                  for (int k = -1; k < 2; k++) gp[d] += (float)W[d][i + 1][j + 1][k + 1] * V(x + i, y + j, z + k);
              gp[d] /= 2.0f * sd[d];
            }
          } else {
            gp[0] = (x < 1) ? (V(x + 1, y, z) - V(x, y, z)) / sd[0] : (V(x, y, z) - V(x - 1, y, z)) / sd[0];
            gp[1] = (y < 1) ? (V(x, y + 1, z) - V(x, y, z)) / sd[1] : (V(x, y, z) - V(x, y - 1, z)) / sd[1];
            gp[2] = (z < 1) ? (V(x, y, z + 1) - V(x, y, z)) / sd[2] : (V(x, y, z) - V(x, y, z - 1)) / sd[2];
          }
        } else {
          /* SOBEL 0 branch (gradient.cpp:294-368).  Its high-border test `idx > size-1` never
           * holds, so at the last slice it reads one voxel past the row; those gradients are
           * never read by the asymmetric smoothing window below, so a one-sided difference is
           * used there instead of the out-of-row read. */
          auto cd = [&](int c, int lim, float lo, float mid, float hi, float s) -> float {
            if (c < 1) return (hi - mid) / s;
            if (c >= lim - 1) return (mid - lo) / s;
            return (hi - lo) / s * 0.5f;
          };
          float c0 = V(x, y, z);
          gp[0] = cd(x, nx, x > 0 ? V(x - 1, y, z) : c0, c0, x < nx - 1 ? V(x + 1, y, z) : c0, sd[0]);
          gp[1] = cd(y, ny, y > 0 ? V(x, y - 1, z) : c0, c0, y < ny - 1 ? V(x, y + 1, z) : c0, sd[1]);
          gp[2] = cd(z, nz, z > 0 ? V(x, y, z - 1) : c0, c0, z < nz - 1 ? V(x, y, z + 1) : c0, sd[2]);
        }
      }
  float w[27];
  noise_gradient_filter_weights(w);
#if defined(_OPENMP)
#pragma omp parallel for schedule(static)
#endif
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        int bd = std::min(std::min(std::min(x, nx - x - 1), std::min(y, ny - y - 1)), std::min(z, nz - z - 1));
        int fw = std::min(2, bd);
        size_t gi = 3 * (((size_t)z * ny + y) * nx + x);
        for (int c = 0; c < 3; ++c) {
          float acc = 0.0f;
          for (int k = -fw; k < fw - 1; ++k)
            for (int j = -fw; j < fw - 1; ++j)
              for (int i = -fw; i < fw - 1; ++i) {
                /* the reference indexes the 5x5x5 table with the shrunken fw */
                int widx = ((fw + k) * 5 + fw + j) * 5 + fw + i;
                int wk = widx / 25, wj = (widx / 5) % 5, wi = widx % 5;
                float wv = w[(wk * 3 + wj) * 3 + wi];
                acc += wv * g[3 * (((size_t)(z + k) * ny + (y + j)) * nx + (x + i)) + c];
              }
          fg[gi + c] = acc;
        }
      }
  for (size_t a = 0; a < count; ++a) {
    float gr[3] = {fg[3 * a], fg[3 * a + 1], fg[3 * a + 2]};
    float len = std::sqrt(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
    if (len < 1e-5f) {
      gr[0] = gr[1] = gr[2] = 0.0f;
    } else {
      gr[0] /= len;
      gr[1] /= len;
      gr[2] /= len;
    }
    for (int c = 0; c < 3; ++c) out_rgba[4 * a + c] = (unsigned char)(((double)gr[c] + 1.0) / 2.0 * UCHAR_MAX);
    out_rgba[4 * a + 3] = noise[a];
  }
}

/* ------------------------------------------------------------------------------------- */
/* filter table and taps                                                                   */
/* ------------------------------------------------------------------------------------- */
static inline int next_pow2(int w) {
  int p = 1;
  while (p < w) p <<= 1;
  return p;
}

/* calcFilterKernelInvArea (dataset.cpp:1503-1512); the box filter uses 0.5 (dataset.cpp:1412). */
static inline float filter_inv_area(const uint8_t* t, int W, bool is_box) {
  if (is_box) return 0.5f;
  float area = 0.0f;
  for (int i = 0; i < W; ++i) area += t[i];
  return 0.5f * W * 255.0f / area;
}

/* texture1D(licKernelSampler, s).r: LUMINANCE8 table, LINEAR, GL_CLAMP (border 0) or
 * CLAMP_TO_EDGE (dataset.cpp:1494-1499). */
template <class R> static inline R kernel_lookup(const uint8_t* t, int W, R s, int clamp_mode) {
  if (s < R(0)) s = R(0);
  if (s > R(1)) s = R(1);
  R u = s * R(W) - R(0.5);
  R fl = std::floor(u);
  int i0 = (int)fl;
  R a = u - fl;
  auto tex = [&](int i) -> R {
    if (clamp_mode == VVLIC_KERNEL_CLAMP_EDGE) i = std::min(std::max(i, 0), W - 1);
    else if (i < 0 || i >= W) return R(0);
    return R(t[i]) / R(255);
  };
  return (R(1) - a) * tex(i0) + a * tex(i0 + 1);
}

/* taps[j + L_b] = kernel weight of tap j (j = -L_b..L_f), offsets as accumulated by
 * computeLIC (inc_lic.glsl:156, 172, 182, 191, 196): 0.5, then -= 0.5/L_b per backward step, += 0.5/L_f per
 * forward step. */
template <class R> static inline void filter_taps(const uint8_t* t, int W, int clamp_mode, int lb, int lf, R* taps) {
  taps[lb] = kernel_lookup<R>(t, W, R(0.5), clamp_mode);
  R off = R(0.5);
  R kb = lb > 0 ? R(0.5) / R(lb) : R(0);
  for (int i = 1; i <= lb; ++i) {
    off -= kb;
    taps[lb - i] = kernel_lookup<R>(t, W, off, clamp_mode);
  }
  off = R(0.5);
  R kf = lf > 0 ? R(0.5) / R(lf) : R(0);
  for (int i = 1; i <= lf; ++i) {
    off += kf;
    taps[lb + i] = kernel_lookup<R>(t, W, off, clamp_mode);
  }
}

/* ------------------------------------------------------------------------------------- */
/* GL samplers                                                                             */
/* ------------------------------------------------------------------------------------- */
struct Inputs {
  const float* field;      /* encoded RGBA, n[0]*n[1]*n[2]*4 (already at storage precision) */
  int n[3];
  float slice_dist[3];
  const uint8_t* noise;    /* noise_channels per voxel: 1 (value) or 4 (gradient xyz, value) */
  int m[3];
  int noise_channels;
  const float* scalar;     /* optional, sn[0]*sn[1]*sn[2] */
  int sn[3];
  const float* tf_rgba;    /* 256*4 */
  const float* tf_opac;    /* 256 */
  const double* taps;      /* L_b + L_f + 1 kernel weights */
  double inv_filter_area;
  const float* licvol = nullptr; /* LIC volume (LICVOLUME technique), ln[0]*ln[1]*ln[2] */
  int ln[3] = {0, 0, 0};
  /* line-illumination tables (ZOECKLER / MALLO): Zoeckler, Mallo diffuse, Mallo specular,
   * lut_w*lut_h RGBA8 each, from illum_luts() */
  const uint8_t* luts = nullptr;
  int lut_w = 0, lut_h = 0;
};

/* ------------------------------------------------------------------------------------- */
/* line-illumination tables: Illumination::createIllumTexZoeckler (illumination.cpp:96-200)  */
/* and createIllumTexMallo (:205-330, Simpson rule :355-391), in double in the reference's  */
/* order, stored as the 8-bit textures the reference uploads (createIllumTextures passes   */
/* floatTex to neither builder): round(clamp(v) * 255).                                     */
/* ------------------------------------------------------------------------------------- */
static inline uint8_t gl_unorm8(float v) {
  double c = v;
  if (!(c > 0.0)) c = 0.0;
  if (c > 1.0) c = 1.0;
  return (uint8_t)std::floor(c * 255.0 + 0.5);
}

static inline double mallo_f(double beta, double n, double theta) {
  double y = std::cos(theta - beta);
  if (y < 0.0) y = 0.0;
  return std::pow(y, n) * (std::cos(theta) / 2.0);
}

static inline double mallo_simpson(double alpha, double beta, double n) {
  const double pi = 3.14159265358979323846;
  double a = alpha - pi / 2.0, b = pi / 2.0;
  int m = 10;
  double h = (b - a) / (2.0 * m), sum = 0.0;
  for (int i = 0; i < 2 * m; i += 2) {
    sum += 2.0 * mallo_f(beta, n, a + i * h);
    sum += 4.0 * mallo_f(beta, n, a + (i + 1) * h);
  }
  sum += mallo_f(beta, n, b);
  sum -= mallo_f(beta, n, a); /* f(a) entered twice above */
  return sum * (h / 3.0);
}

/* out: 3 tables of w*h RGBA8 (Zoeckler as LUMINANCE_ALPHA samples it: L, L, L, A). */
static inline void illum_luts(const vvlic_line_material& m, int w, int h, uint8_t* out) {
  const double pi = 3.14159265358979323846;
  double ix = 1.0 / (double)(w - 1), iy = 1.0 / (double)(h - 1);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      double lt = 2.0 * ((double)x * ix) - 1.0, vt = 2.0 * ((double)y * iy) - 1.0;
      double diffuse = std::pow(std::sqrt(1.0 - lt * lt), (double)m.diff_exp);
      double dp = lt * vt - std::sqrt(1.0 - lt * lt) * std::sqrt(1.0 - vt * vt);
      if (dp < -1.0) dp = -1.0;
      if (dp > 1.0) dp = 1.0;
      double td = m.ambient[0] * m.light_color[0] + diffuse * m.diffuse[0] * m.light_color[0];
      double ts = std::pow(std::fabs(dp), (double)m.spec_exp) * m.specular[0] * m.light_color[0];
      td *= 0.5;
      td = td < 0.0 ? 0.0 : (td > 1.0 ? 1.0 : td);
      ts *= 0.5;
      ts = ts < 0.0 ? 0.0 : (ts > 1.0 ? 1.0 : ts);
      uint8_t* o = out + 4 * ((size_t)y * w + x);
      o[0] = o[1] = o[2] = gl_unorm8((float)td);
      o[3] = gl_unorm8((float)ts * 0.9f);
    }
  uint8_t* dt = out + (size_t)4 * w * h;
  uint8_t* st = out + (size_t)8 * w * h;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      double s = ((double)x + 0.5) / w, t = ((double)y + 0.5) / h;
      double alpha = std::acos(2.0 * s - 1.0), beta = std::acos(2.0 * t - 1.0), lt = 2.0 * t - 1.0;
      double diffuse = std::sqrt(1.0 - lt * lt) * (std::sin(alpha) + (pi - alpha) * std::cos(alpha)) * 0.25;
      double specular = 3.5 * mallo_simpson(alpha, beta, m.spec_exp);
      for (int i = 0; i < 4; ++i) {
        size_t o = 4 * ((size_t)y * w + x) + i;
        double c = diffuse * m.diffuse[i] * m.light_color[i];
        dt[o] = gl_unorm8((float)(c < 0.0 ? 0.0 : (c > 1.0 ? 1.0 : c)));
        c = specular * m.specular[i] * m.light_color[i];
        st[o] = gl_unorm8((float)(c < 0.0 ? 0.0 : (c > 1.0 ? 1.0 : c)));
      }
    }
}

/* texture2D(table, (s, r)) with LINEAR + CLAMP_TO_EDGE on an RGBA8 table; a NaN coordinate
 * (degenerate tangent) is taken as 0. */
template <class R> static inline V4<R> tex2d_lut(const uint8_t* t, int w, int h, R s, R r) {
  s = std::fmin(std::fmax(s, R(0)), R(1));
  r = std::fmin(std::fmax(r, R(0)), R(1));
  R u = s * R(w) - R(0.5), v = r * R(h) - R(0.5);
  R fu = std::floor(u), fv = std::floor(v);
  R au = u - fu, av = v - fv;
  int x0 = std::max((int)fu, 0), x1 = std::min((int)fu + 1, w - 1);
  int y0 = std::max((int)fv, 0), y1 = std::min((int)fv + 1, h - 1);
  R c[4];
  for (int k = 0; k < 4; ++k) {
    R t00 = R(t[4 * ((size_t)y0 * w + x0) + k]), t10 = R(t[4 * ((size_t)y0 * w + x1) + k]);
    R t01 = R(t[4 * ((size_t)y1 * w + x0) + k]), t11 = R(t[4 * ((size_t)y1 * w + x1) + k]);
    c[k] = ((R(1) - au) * (R(1) - av) * t00 + au * (R(1) - av) * t10 + (R(1) - au) * av * t01 + au * av * t11) /
           R(255);
  }
  return V4<R>{c[0], c[1], c[2], c[3]};
}

/* LINEAR + CLAMP_TO_EDGE trilinear at texture coordinate s (GL 2.1 eq. 3.23/3.27). */
template <class R> static inline V4<R> tex3d_field(const Inputs& in, V3<R> s) {
  const int* n = in.n;
  R u[3] = {s.x * R(n[0]) - R(0.5), s.y * R(n[1]) - R(0.5), s.z * R(n[2]) - R(0.5)};
  int i0[3], i1[3];
  R a[3];
  for (int d = 0; d < 3; ++d) {
    R uc = u[d];
    if (!(uc > R(-1))) uc = R(-1); /* below -1 (or NaN) both texels clamp to 0 */
    if (uc > R(n[d])) uc = R(n[d]);
    R fl = std::floor(uc);
    a[d] = uc - fl;
    int b = (int)fl;
    i0[d] = std::min(std::max(b, 0), n[d] - 1);
    i1[d] = std::min(std::max(b + 1, 0), n[d] - 1);
  }
  V4<R> r{R(0), R(0), R(0), R(0)};
  for (int c = 0; c < 8; ++c) {
    int xi = (c & 1) ? i1[0] : i0[0], yi = (c & 2) ? i1[1] : i0[1], zi = (c & 4) ? i1[2] : i0[2];
    R w = ((c & 1) ? a[0] : R(1) - a[0]) * ((c & 2) ? a[1] : R(1) - a[1]) * ((c & 4) ? a[2] : R(1) - a[2]);
    const float* t = in.field + 4 * (((size_t)zi * n[1] + yi) * n[0] + xi);
    r.x += w * R(t[0]);
    r.y += w * R(t[1]);
    r.z += w * R(t[2]);
    r.w += w * R(t[3]);
  }
  return r;
}

template <class R> static inline R tex3d_scalar(const Inputs& in, V3<R> s) {
  const int* n = in.sn;
  R u[3] = {s.x * R(n[0]) - R(0.5), s.y * R(n[1]) - R(0.5), s.z * R(n[2]) - R(0.5)};
  int i0[3], i1[3];
  R a[3];
  for (int d = 0; d < 3; ++d) {
    R uc = u[d];
    if (!(uc > R(-1))) uc = R(-1);
    if (uc > R(n[d])) uc = R(n[d]);
    R fl = std::floor(uc);
    a[d] = uc - fl;
    int b = (int)fl;
    i0[d] = std::min(std::max(b, 0), n[d] - 1);
    i1[d] = std::min(std::max(b + 1, 0), n[d] - 1);
  }
  R r = R(0);
  for (int c = 0; c < 8; ++c) {
    int xi = (c & 1) ? i1[0] : i0[0], yi = (c & 2) ? i1[1] : i0[1], zi = (c & 4) ? i1[2] : i0[2];
    R w = ((c & 1) ? a[0] : R(1) - a[0]) * ((c & 2) ? a[1] : R(1) - a[1]) * ((c & 4) ? a[2] : R(1) - a[2]);
    r += w * R(in.scalar[((size_t)zi * n[1] + yi) * n[0] + xi]);
  }
  return r;
}

/* LINEAR + REPEAT trilinear of the uint8 noise; returns RGBA/255 (value in .w; for a
 * one-channel noise the gradient part is 0). */
template <class R> static inline V4<R> tex3d_noise(const Inputs& in, V3<R> s) {
  const int* m = in.m;
  R u[3] = {s.x * R(m[0]) - R(0.5), s.y * R(m[1]) - R(0.5), s.z * R(m[2]) - R(0.5)};
  int i0[3], i1[3];
  R a[3];
  for (int d = 0; d < 3; ++d) {
    R uc = u[d];
    if (!(uc > R(-16777216))) uc = R(-16777216);
    if (uc > R(16777216)) uc = R(16777216);
    R fl = std::floor(uc);
    a[d] = uc - fl;
    long long b = (long long)fl;
    long long md = m[d];
    i0[d] = (int)(((b % md) + md) % md);
    i1[d] = (int)((((b + 1) % md) + md) % md);
  }
  V4<R> r{R(0), R(0), R(0), R(0)};
  const int ch = in.noise_channels;
  for (int c = 0; c < 8; ++c) {
    int xi = (c & 1) ? i1[0] : i0[0], yi = (c & 2) ? i1[1] : i0[1], zi = (c & 4) ? i1[2] : i0[2];
    R w = ((c & 1) ? a[0] : R(1) - a[0]) * ((c & 2) ? a[1] : R(1) - a[1]) * ((c & 4) ? a[2] : R(1) - a[2]);
    const uint8_t* t = in.noise + (size_t)ch * (((size_t)zi * m[1] + yi) * m[0] + xi);
    if (ch == 4) {
      r.x += w * R(t[0]);
      r.y += w * R(t[1]);
      r.z += w * R(t[2]);
      r.w += w * R(t[3]);
    } else {
      r.w += w * R(t[0]);
    }
  }
  R k = R(1) / R(255);
  return V4<R>{r.x * k, r.y * k, r.z * k, r.w * k};
}

/* 1D LINEAR + CLAMP_TO_EDGE lookup in a 256-entry float table with `stride` channels. */
template <class R> static inline R tex1d(const float* t, int stride, int ch, R s) {
  const int N = VVLIC_TF_ENTRIES;
  R u = s * R(N) - R(0.5);
  if (!(u > R(-1))) u = R(-1);
  if (u > R(N)) u = R(N);
  R fl = std::floor(u);
  R a = u - fl;
  int b = (int)fl;
  int i0 = std::min(std::max(b, 0), N - 1), i1 = std::min(std::max(b + 1, 0), N - 1);
  return (R(1) - a) * R(t[i0 * stride + ch]) + a * R(t[i1 * stride + ch]);
}

/* ------------------------------------------------------------------------------------- */
/* uniforms: setRenderVolParams (renderer.cpp:925-996)                                     */
/* ------------------------------------------------------------------------------------- */
template <class R> struct Uniforms {
  R tex_max[3], scale_vol[3], scale_vol_inv[3], extent[3];
  R step_size, gradient_scale, illum_scale, freq_scale;
  int num_iterations, lf, lb;
  R h, h_eff, alpha_correction, intensity_scale;
};

template <class R> static inline Uniforms<R> uniforms(const Inputs& in, const vvlic_params& p) {
  Geometry g = geometry(in.n, in.slice_dist);
  Uniforms<R> u;
  bool bug = (p.quirks & VVLIC_QUIRK_UNIFORM_SCALE_BUG) && p.illum != VVLIC_ILLUM_NONE;
  for (int i = 0; i < 3; ++i) {
    u.tex_max[i] = R(g.tex_max[i]);
    u.extent[i] = R(g.extent[i]);
    u.scale_vol[i] = R(bug ? g.scale_inv[i] : g.scale[i]);
    u.scale_vol_inv[i] = R(bug ? 0.0 : g.scale_inv[i]);
  }
  if (p.low_res) {
    u.step_size = R(2.0f * p.step_size_vol);
    u.freq_scale = R(0.7f * p.freq_scale);
    u.lf = 15;
    u.lb = 15;
    u.h = R(1.0f / 64.0f);
    u.alpha_correction = R(2.0f * p.step_size_vol * 128.0f);
  } else {
    u.step_size = R(p.step_size_vol);
    u.freq_scale = R(p.freq_scale);
    u.lf = p.steps_forward;
    u.lb = p.steps_backward;
    u.h = R(p.step_size_lic);
    u.alpha_correction = R(p.step_size_vol * 128.0f);
  }
  u.gradient_scale = R(p.gradient_scale);
  u.illum_scale = R(p.illum_scale);
  u.num_iterations = p.num_iterations;
  u.h_eff = u.h * R(p.eye_dist_factor);
  u.intensity_scale = R(in.inv_filter_area) / R(u.lf + u.lb) * u.gradient_scale;
  return u;
}

/* ------------------------------------------------------------------------------------- */
/* view: per-pixel ray coefficients (camera.cpp:56-67, renderer.cpp:146)                    */
/* c[0..2] o0, c[3..5] o1, c[6..8] o2, c[9..11] d0, c[12..14] d1, c[15..17] d2, c[18] clamp */
/* ------------------------------------------------------------------------------------- */
static inline void view_rays(const vvlic_view& v, const int n[3], const float sd[3], int W, int H, double* c) {
  Geometry g = geometry(n, sd);
  for (int i = 0; i < 21; ++i) c[i] = 0.0;
  if (v.projection == VVLIC_ORTHOGRAPHIC) {
    for (int i = 0; i < 3; ++i) {
      c[0 + i] = (double)v.ortho_center[i] - v.ortho_right[i] - v.ortho_up[i];
      c[3 + i] = 2.0 * v.ortho_right[i] / W;
      c[6 + i] = 2.0 * v.ortho_up[i] / H;
      c[9 + i] = v.ortho_dir[i];
    }
    c[18] = 0.0;
    return;
  }
  double qx = v.quat[0], qy = v.quat[1], qz = v.quat[2], qw = v.quat[3];
  double qn = std::sqrt(qx * qx + qy * qy + qz * qz + qw * qw);
  if (qn > 0) { qx /= qn; qy /= qn; qz /= qn; qw /= qn; } else { qw = 1; }
  /* rotation matrix of q (glRotatef(2 acos(w), axis), mmath.cpp:213-232) */
  double Rm[3][3] = {{1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)},
                     {2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)},
                     {2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)}};
  auto rt = [&](const double e[3], double* out) { /* R^T e */
    for (int i = 0; i < 3; ++i) out[i] = Rm[0][i] * e[0] + Rm[1][i] * e[1] + Rm[2][i] * e[2];
  };
  /* eye = MV^-1 (0,0,0,1) with MV = T(pan) T(0,0,-dist) R T(-center) */
  double e_eye[3] = {-(double)v.pan[0], -(double)v.pan[1], (double)v.distance - v.pan[2]};
  double eo[3];
  rt(e_eye, eo);
  for (int i = 0; i < 3; ++i) c[i] = eo[i] + g.center[i];
  double aspect = v.aspect > 0 ? (double)v.aspect : (double)W / (double)H;
  double t = std::tan((double)v.fovy_deg * M_PI / 360.0);
  double d0[3] = {-aspect * t, -t, -1.0}, d1[3] = {2.0 * aspect * t / W, 0.0, 0.0}, d2[3] = {0.0, 2.0 * t / H, 0.0};
  rt(d0, c + 9);
  rt(d1, c + 12);
  rt(d2, c + 15);
  c[18] = 1.0;
}

/* Slab test against [0, extent]: returns false for a miss; t_entry on hit. */
template <class R> static inline bool ray_entry(const R o[3], const R d[3], const R ext[3], bool clamp0, R* t_entry,
                                               R* t_exit = nullptr) {
  R tn = -INFINITY, tf = INFINITY;
  for (int i = 0; i < 3; ++i) {
    if (d[i] == R(0)) {
      if (o[i] < R(0) || o[i] > ext[i]) return false;
      continue;
    }
    R inv = R(1) / d[i];
    R t0 = (R(0) - o[i]) * inv, t1 = (ext[i] - o[i]) * inv;
    if (t0 > t1) std::swap(t0, t1);
    tn = std::max(tn, t0);
    tf = std::min(tf, t1);
  }
  if (!(tn < tf)) return false;
  if (clamp0) {
    if (!(tf > R(0))) return false;
    tn = std::max(tn, R(0));
  }
  *t_entry = tn;
  if (t_exit) *t_exit = tf;
  return true;
}

/* ------------------------------------------------------------------------------------- */
/* LIC: computeLIC / singleLICstep (inc_lic.glsl:93-202)                                    */
/* ------------------------------------------------------------------------------------- */
template <class R> struct LicCtx {
  const Inputs* in;
  const vvlic_params* p;
  const Uniforms<R>* u;
  bool grad;      /* USE_NOISE_GRADIENTS (ILLUM_GRADIENT) */
};

/* freqSampling (inc_lic.glsl:71-90) / freqSamplingGrad (:61-68) */
template <class R> static inline V4<R> noise_tap(const LicCtx<R>& c, V3<R> p) {
  const Inputs& in = *c.in;
  if (c.grad) {
    bool nofreq = (c.p->quirks & VVLIC_QUIRK_GRAD_NOISE_NO_FREQ) != 0;
    return tex3d_noise<R>(in, nofreq ? p : p * c.u->freq_scale);
  }
  if (c.p->scalar_gate && in.scalar) {
    R s = tex3d_scalar<R>(in, p);
    if (!(s > R(c.p->gate_lo) && s < R(c.p->gate_hi))) return V4<R>{R(0), R(0), R(0), R(0)};
  }
  if (c.p->quirks & VVLIC_QUIRK_LUMINANCE_NOISE) return V4<R>{R(0), R(0), R(0), R(1)};
  V4<R> n = tex3d_noise<R>(in, p * c.u->freq_scale);
  return V4<R>{R(0), R(0), R(0), n.w};
}

template <class R> static inline V3<R> slope(V4<R> f) {
  return V3<R>{R(2) * f.x - R(1), R(2) * f.y - R(1), R(2) * f.z - R(1)};
}

/* One streamline step from p with current field value `step` in direction dirs (+-1).
 * Returns the new position and replaces `step` with the field there. */
template <class R> static inline V3<R> lic_step(const LicCtx<R>& c, V3<R> p, V4<R>& step, R dirs) {
  const Inputs& in = *c.in;
  R h = c.u->h_eff;
  R sof = c.p->speed_of_flow ? step.w : R(1);
  V3<R> k1 = slope(step) * dirs * sof * h; /* licdir (inc_lic.glsl:180/194, 109, 114) */
  int integ = c.p->integrator;
  if (integ == VVLIC_EULER) {
    p = p + k1;
  } else if (integ == VVLIC_HEUN) {
    V3<R> p2 = p + k1;
    V3<R> k2 = slope(tex3d_field<R>(in, p2)) * dirs * sof * h;
    p = p + (k1 + k2) * R(0.5);
  } else {
    V3<R> k2 = slope(tex3d_field<R>(in, p + k1 * R(0.5))) * dirs * sof * h;
    V3<R> k3 = slope(tex3d_field<R>(in, p + k2 * R(0.5))) * dirs * sof * h;
    V3<R> k4 = slope(tex3d_field<R>(in, p + k3)) * dirs * sof * h;
    p = p + (k1 + k2 * R(2) + k3 * R(2) + k4) * (R(1) / R(6));
  }
  step = tex3d_field<R>(in, p);
  return p;
}

/* computeLIC: returns (sum w*grad_enc.xyz, sum w*noise) */
template <class R> static inline V4<R> compute_lic(const LicCtx<R>& c, V3<R> pos, V4<R> f0) {
  const double* w = c.in->taps;
  const int lb = c.u->lb, lf = c.u->lf;
  V4<R> n0 = noise_tap<R>(c, pos);
  R w0 = R(w[lb]);
  V4<R> acc{n0.x * w0, n0.y * w0, n0.z * w0, n0.w * w0};
  for (int half = 0; half < 2; ++half) {
    R dirs = half == 0 ? R(-1) : R(1);
    int L = half == 0 ? lb : lf;
    V3<R> p = pos;
    V4<R> step = f0;
    for (int i = 1; i <= L; ++i) {
      p = lic_step<R>(c, p, step, dirs);
      V4<R> n = noise_tap<R>(c, p);
      R wi = R(w[half == 0 ? lb - i : lb + i]);
      acc.x += n.x * wi;
      acc.y += n.y * wi;
      acc.z += n.z * wi;
      acc.w += n.w * wi;
    }
  }
  return acc;
}

/* ------------------------------------------------------------------------------------- */
/* shading: illumLIC (inc_illum.glsl:158-172), illumGradient (:1-41)                        */
/* ------------------------------------------------------------------------------------- */
template <class R> static inline R alpha_correct(R a, R corr) {
  R base = R(1) - a;
  if (base < R(0)) base = R(0);
  return R(1) - std::pow(base, corr);
}

template <class R> static inline V3<R> cross(V3<R> a, V3<R> b) {
  return V3<R>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
/* clamp to [0, 1] with NaN -> 0 */
template <class R> static inline R sat_nan0(R v) { return std::fmin(std::fmax(v, R(0)), R(1)); }

/* illumZoeckler (inc_illum.glsl:117-154) / illumMallo (:46-112) as colour = tf.rgb I d + s, with
 * d and s from the line tables; f = vectorData at pos, its encoded rgb the streamline tangent. */
template <class R>
static inline void line_factors(const LicCtx<R>& c, V3<R> pos, V3<R> dir, V4<R> f, R d[3], R sp[3]) {
  const Uniforms<R>& u = *c.u;
  const vvlic_params& p = *c.p;
  const Inputs& in = *c.in;
  V3<R> lp{R(p.light_pos[0]), R(p.light_pos[1]), R(p.light_pos[2])};
  V3<R> sv{u.scale_vol_inv[0], u.scale_vol_inv[1], u.scale_vol_inv[2]};
  V3<R> L = normalize(lp - mul(pos, sv));
  V3<R> T = normalize(V3<R>{R(2) * f.x - R(1), R(2) * f.y - R(1), R(2) * f.z - R(1)});
  if (p.illum == VVLIC_ILLUM_ZOECKLER) {
    V3<R> V = normalize(dir);
    V4<R> sh = tex2d_lut<R>(in.luts, in.lut_w, in.lut_h, R(0.5) * dot(L, T) + R(0.5), R(0.5) * dot(V, T) + R(0.5));
    R g = (p.quirks & VVLIC_QUIRK_ZOECKLER_LUMINANCE) ? sh.y : sh.w;
    for (int ch = 0; ch < 3; ++ch) {
      d[ch] = sh.x * u.illum_scale;
      sp[ch] = R(0.9) * g;
    }
  } else {
    V3<R> V = normalize(dir * R(-1));
    V3<R> B = normalize(cross(T, V));
    V3<R> N = cross(B, T);
    V3<R> H = normalize(V + L);
    R lx = dot(L, N), ly = dot(L, T), lz = dot(H, N), lw = dot(H, T);
    R tx = R(1) / std::sqrt(R(1) - ly * ly), ty = R(1) / std::sqrt(R(1) - lw * lw);
    R cz = R(0.5) * (lx * tx) + R(0.5), cy = R(0.5) * ly + R(0.5), cw = R(0.5) * (lz * ty) + R(0.5);
    size_t one = (size_t)4 * in.lut_w * in.lut_h;
    V4<R> df = tex2d_lut<R>(in.luts + one, in.lut_w, in.lut_h, cz, cy);
    V4<R> sc = tex2d_lut<R>(in.luts + 2 * one, in.lut_w, in.lut_h, cz, cw);
    R att = std::pow(ty, -R(p.spec_exp));
    for (int ch = 0; ch < 3; ++ch) {
      d[ch] = (&df.x)[ch] * u.illum_scale;
      sp[ch] = sat_nan0((&sc.x)[ch] * att);
    }
  }
}

/* f = vectorData at pos; its encoded rgb is the tangent of illumZoeckler / illumMallo. */
template <class R>
static inline V4<R> shade(const LicCtx<R>& c, V4<R> illum, V4<R> tf, V3<R> pos, V3<R> dir, V4<R> f) {
  const Uniforms<R>& u = *c.u;
  const vvlic_params& p = *c.p;
  V4<R> col;
  R I = illum.w;
  if (p.illum == VVLIC_ILLUM_ZOECKLER || p.illum == VVLIC_ILLUM_MALLO) {
    R d[3], sp[3];
    line_factors<R>(c, pos, dir, f, d, sp);
    col.x = tf.x * I * d[0] + sp[0];
    col.y = tf.y * I * d[1] + sp[1];
    col.z = tf.z * I * d[2] + sp[2];
  } else if (p.illum == VVLIC_ILLUM_GRADIENT) {
    V3<R> lp{R(p.light_pos[0]), R(p.light_pos[1]), R(p.light_pos[2])};
    V3<R> sv{u.scale_vol_inv[0], u.scale_vol_inv[1], u.scale_vol_inv[2]};
    V3<R> L = normalize(lp - mul(pos, sv));
    V3<R> V = normalize(dir * R(-1));
    V3<R> N = normalize(V3<R>{-illum.x, -illum.y, -illum.z});
    V3<R> Rf = normalize(N * (R(2) * dot(L, N)) - L);
    R s = clamp01(dot(Rf, V));
    s = std::pow(s, R(p.spec_exp));
    V3<R> spec = V3<R>{R(p.light_specular[0]), R(p.light_specular[1]), R(p.light_specular[2])} * (s * I);
    R dfac = clamp01(dot(L, N));
    V3<R> diff = V3<R>{R(p.light_diffuse[0]), R(p.light_diffuse[1]), R(p.light_diffuse[2])} * (dfac * u.illum_scale);
    V3<R> amb{R(p.light_ambient[0]), R(p.light_ambient[1]), R(p.light_ambient[2])};
    V3<R> base{tf.x * I, tf.y * I, tf.z * I};
    V3<R> lit = mul(base, diff + V3<R>{R(0.3), R(0.3), R(0.3)} + amb) + spec;
    lit = lit * u.illum_scale;
    col.x = lit.x;
    col.y = lit.y;
    col.z = lit.z;
  } else {
    col.x = I * tf.x * u.illum_scale;
    col.y = I * tf.y * u.illum_scale;
    col.z = I * tf.z * u.illum_scale;
  }
  R a = tex1d<R>(c.in->tf_opac, 1, 0, I * R(1.3)) * tf.w;
  col.w = alpha_correct<R>(a, u.alpha_correction);
  return col;
}

/* ------------------------------------------------------------------------------------- */
/* other techniques                                                                        */
/* ------------------------------------------------------------------------------------- */
/* Slab planes of ViewSlicing::setupSlicing (slicing.cpp:42-103): unit view direction v in
 * object space (modelview row 2 / its z translation), depth D = 2 sum |v_i| ext_i/2, N slices. */
static inline void slicing_setup(const vvlic_view& v, const int n[3], const float sd[3], float spacing, double vout[3],
                                 double* depth, int* ns) {
  Geometry g = geometry(n, sd);
  double dv[3];
  if (v.projection == VVLIC_ORTHOGRAPHIC) {
    for (int i = 0; i < 3; ++i) dv[i] = v.ortho_dir[i];
  } else {
    double qx = v.quat[0], qy = v.quat[1], qz = v.quat[2], qw = v.quat[3];
    double qn = std::sqrt(qx * qx + qy * qy + qz * qz + qw * qw);
    if (qn > 0) { qx /= qn; qy /= qn; qz /= qn; qw /= qn; } else { qw = 1; }
    double row2[3] = {2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)};
    double m14 = (double)v.pan[2] - v.distance - (row2[0] * g.center[0] + row2[1] * g.center[1] + row2[2] * g.center[2]);
    for (int i = 0; i < 3; ++i) dv[i] = row2[i] / m14;
  }
  double nn = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
  double d6 = 0.0;
  for (int i = 0; i < 3; ++i) {
    vout[i] = dv[i] / nn;
    d6 += std::fabs(vout[i]) * 0.5 * g.extent[i];
  }
  *depth = 2.0 * d6;
  *ns = (int)(*depth / spacing) + 1;
}

/* texture3D(licVolumeSampler, s).r with LINEAR + REPEAT (VolumeBuffer.cpp:43-57) */
template <class R> static inline R tex3d_licvol(const Inputs& in, V3<R> s) {
  const int* m = in.ln;
  R u[3] = {s.x * R(m[0]) - R(0.5), s.y * R(m[1]) - R(0.5), s.z * R(m[2]) - R(0.5)};
  int i0[3], i1[3];
  R a[3];
  for (int d = 0; d < 3; ++d) {
    R fl = std::floor(u[d]);
    a[d] = u[d] - fl;
    long long b = (long long)fl, md = m[d];
    i0[d] = (int)(((b % md) + md) % md);
    i1[d] = (int)((((b + 1) % md) + md) % md);
  }
  R r = R(0);
  for (int c = 0; c < 8; ++c) {
    int xi = (c & 1) ? i1[0] : i0[0], yi = (c & 2) ? i1[1] : i0[1], zi = (c & 4) ? i1[2] : i0[2];
    R w = ((c & 1) ? a[0] : R(1) - a[0]) * ((c & 2) ? a[1] : R(1) - a[1]) * ((c & 4) ? a[2] : R(1) - a[2]);
    r += w * R(in.licvol[((size_t)zi * m[1] + yi) * m[0] + xi]);
  }
  return r;
}

/* LIC volume precompute (lic3d_volume_fragment.glsl:2-21) at voxel centres of an ln grid. */
template <class R> static inline void lic_volume(const Inputs& in, const vvlic_params& p, const int ln[3], float* out) {
  Uniforms<R> u = uniforms<R>(in, p);
  Geometry g = geometry(in.n, in.slice_dist);
  vvlic_params q = p;
  q.illum = VVLIC_ILLUM_NONE;
  LicCtx<R> c{&in, &q, &u, false};
#if defined(_OPENMP)
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int z = 0; z < ln[2]; ++z)
    for (int y = 0; y < ln[1]; ++y)
      for (int x = 0; x < ln[0]; ++x) {
        V3<R> pos{(R(x) + R(0.5)) / R(ln[0]) * R(g.scale[0]), (R(y) + R(0.5)) / R(ln[1]) * R(g.scale[1]),
                  (R(z) + R(0.5)) / R(ln[2]) * R(g.scale[2])};
        V4<R> f = tex3d_field<R>(in, pos);
        out[((size_t)z * ln[1] + y) * ln[0] + x] = float(compute_lic<R>(c, pos, f).w * u.intensity_scale);
      }
}

/* slicing (lic3d_slicing_fragment.glsl:5-74 over the planes of slicing.cpp:106-114) */
template <class R> static inline uint32_t slice_pixel(const Inputs& in, const vvlic_params& p, const Uniforms<R>& u,
                                                      const R o[3], const R d[3], R tn, R tfar, const double* vv,
                                                      double depth, int ns, float out[4]) {
  Geometry g = geometry(in.n, in.slice_dist);
  LicCtx<R> c{&in, &p, &u, p.illum == VVLIC_ILLUM_GRADIENT};
  V3<R> sv{u.scale_vol[0], u.scale_vol[1], u.scale_vol[2]};
  V3<R> D{d[0], d[1], d[2]};
  V3<R> dir = mul(normalize(D), sv);
  V3<R> V{R(vv[0]), R(vv[1]), R(vv[2])};
  R vd = dot(V, D);
  V4<R> dest{R(0), R(0), R(0), R(0)};
  uint32_t samples = 0;
  if (vd == R(0)) return 0;
  V3<R> oc{o[0] - R(g.center[0]), o[1] - R(g.center[1]), o[2] - R(g.center[2])};
  R voc = dot(V, oc);
  R step = R(depth) / R(ns);
  for (int i = 0; i < ns; ++i) {
    if (dest.w >= R(0.95)) break;
    R di = R(-0.5) * R(depth) + (R(i) + R(0.5)) * step;
    R ti = (di - voc) / vd;
    if (!(ti >= tn && ti <= tfar)) continue;
    V3<R> x{o[0] + ti * d[0], o[1] + ti * d[1], o[2] + ti * d[2]};
    V3<R> pos = mul(x, sv);
    V4<R> f = tex3d_field<R>(in, pos);
    V4<R> tf{tex1d<R>(in.tf_rgba, 4, 0, f.w), tex1d<R>(in.tf_rgba, 4, 1, f.w), tex1d<R>(in.tf_rgba, 4, 2, f.w),
             tex1d<R>(in.tf_rgba, 4, 3, f.w)};
    if (!(tf.w > R(0.05))) continue;
    V4<R> il = compute_lic<R>(c, pos, f);
    ++samples;
    il.w *= u.intensity_scale;
    V4<R> src = shade<R>(c, il, tf, pos, dir, f);
    src.x *= src.w;
    src.y *= src.w;
    src.z *= src.w;
    R om = R(1) - dest.w;
    dest = V4<R>{clamp01(om * src.x + dest.x), clamp01(om * src.y + dest.y), clamp01(om * src.z + dest.z),
                 clamp01(om * src.w + dest.w)};
  }
  out[0] = (float)dest.x;
  out[1] = (float)dest.y;
  out[2] = (float)dest.z;
  out[3] = (float)dest.w;
  return samples;
}

/* ------------------------------------------------------------------------------------- */
/* the ray: lic3d_fragment.glsl:5-99                                                       */
/* ------------------------------------------------------------------------------------- */
template <class R> static inline uint32_t render_pixel(const Inputs& in, const vvlic_params& p, const Uniforms<R>& u,
                                                       const double* rc, int px, int py, float out[4],
                                                       const double* slicing = nullptr) {
  out[0] = out[1] = out[2] = out[3] = 0.0f;
  R o[3], d[3], ext[3];
  R uu = R(px) + R(0.5), vv = R(py) + R(0.5);
  for (int i = 0; i < 3; ++i) {
    o[i] = R(rc[0 + i]) + uu * R(rc[3 + i]) + vv * R(rc[6 + i]);
    d[i] = R(rc[9 + i]) + uu * R(rc[12 + i]) + vv * R(rc[15 + i]);
    ext[i] = u.extent[i];
  }
  R te, tx;
  if (!ray_entry<R>(o, d, ext, rc[18] != 0.0, &te, &tx)) return 0;
  if (p.technique == VVLIC_TECHNIQUE_SLICING)
    return slice_pixel<R>(in, p, u, o, d, te, tx, slicing, slicing[3], (int)slicing[4], out);
  V3<R> sv{u.scale_vol[0], u.scale_vol[1], u.scale_vol[2]};
  V3<R> obj{o[0] + te * d[0], o[1] + te * d[1], o[2] + te * d[2]};
  V3<R> pos = mul(obj, sv);
  V3<R> dir = mul(normalize(V3<R>{d[0], d[1], d[2]}), sv);
  LicCtx<R> c{&in, &p, &u, p.illum == VVLIC_ILLUM_GRADIENT};
  V4<R> dest{R(0), R(0), R(0), R(0)}, src{R(0), R(0), R(0), R(0)};
  uint32_t samples = 0;
  bool outside = false;
  const R thr = R(p.alpha_threshold);
  if (p.technique == VVLIC_TECHNIQUE_VOLUME || p.technique == VVLIC_TECHNIQUE_LICVOLUME) {
    /* vectorfield_fragment.glsl:67-97 / raycast_lic3d_fragment.glsl:35-69: stop on dest.a */
    vvlic_params q = p;
    q.illum = VVLIC_ILLUM_NONE;
    LicCtx<R> cq{&in, &q, &u, false};
    for (int j = 0; !outside && j < u.num_iterations; ++j) {
      for (int i = 0; i < u.num_iterations; ++i) {
        V4<R> f = tex3d_field<R>(in, pos);
        if (p.technique == VVLIC_TECHNIQUE_LICVOLUME) {
          R idx = p.tf_index == VVLIC_TF_INDEX_MAGNITUDE ? f.w : f.z;
          V4<R> tf{tex1d<R>(in.tf_rgba, 4, 0, idx), tex1d<R>(in.tf_rgba, 4, 1, idx), tex1d<R>(in.tf_rgba, 4, 2, idx),
                   tex1d<R>(in.tf_rgba, 4, 3, idx)};
          V4<R> il{R(0), R(0), R(0), tex3d_licvol<R>(in, pos)};
          src = shade<R>(cq, il, tf, pos, dir, f);
        } else {
          src = V4<R>{f.x, f.y, f.z, tex1d<R>(in.tf_rgba, 4, 3, f.w)};
        }
        ++samples;
        src.x *= src.w;
        src.y *= src.w;
        src.z *= src.w;
        R om = R(1) - dest.w;
        dest = V4<R>{clamp01(om * src.x + dest.x), clamp01(om * src.y + dest.y), clamp01(om * src.z + dest.z),
                     clamp01(om * src.w + dest.w)};
        pos = pos + dir * u.step_size;
        outside = pos.x < R(0) || pos.y < R(0) || pos.z < R(0) || pos.x > u.tex_max[0] || pos.y > u.tex_max[1] ||
                  pos.z > u.tex_max[2] || dest.w > thr;
        if (outside) break;
      }
    }
    out[0] = (float)dest.x;
    out[1] = (float)dest.y;
    out[2] = (float)dest.z;
    out[3] = (float)dest.w;
    return samples;
  }
  for (int j = 0; !outside && j < u.num_iterations; ++j) {
    for (int i = 0; i < u.num_iterations; ++i) {
      V4<R> f = tex3d_field<R>(in, pos);
      R idx = p.tf_index == VVLIC_TF_INDEX_MAGNITUDE ? f.w : f.z;
      V4<R> tf{tex1d<R>(in.tf_rgba, 4, 0, idx), tex1d<R>(in.tf_rgba, 4, 1, idx), tex1d<R>(in.tf_rgba, 4, 2, idx),
               tex1d<R>(in.tf_rgba, 4, 3, idx)};
      V4<R> il = compute_lic<R>(c, pos, f);
      ++samples;
      il.w *= u.intensity_scale;
      src = shade<R>(c, il, tf, pos, dir, f);
      src.x *= src.w;
      src.y *= src.w;
      src.z *= src.w;
      R om = R(1) - dest.w;
      dest.x = clamp01(om * src.x + dest.x);
      dest.y = clamp01(om * src.y + dest.y);
      dest.z = clamp01(om * src.z + dest.z);
      dest.w = clamp01(om * src.w + dest.w);
      pos = pos + dir * u.step_size;
      outside = pos.x < R(0) || pos.y < R(0) || pos.z < R(0) || pos.x > u.tex_max[0] || pos.y > u.tex_max[1] ||
                pos.z > u.tex_max[2] || src.w > thr;
      if (outside) break;
    }
  }
  out[0] = (float)dest.x;
  out[1] = (float)dest.y;
  out[2] = (float)dest.z;
  out[3] = (float)dest.w;
  return samples;
}

/* ------------------------------------------------------------------------------------- */
/* adjoint: reverse mode through the ray (illumLIC or illumGradient + blend) w.r.t. the TF  */
/* RGBA table, the opacity table and the filter taps.  Conventions shared with the kernel: */
/* d clamp(u)/du = 1 on [0, 1] and 0 outside; the alpha-correction derivative is 0 where   */
/* its base 1 - a is <= 0; a 1D lookup's derivative in its coordinate is 0 where the       */
/* coordinate is clamped; the termination test is not differentiated.                     */
/* ------------------------------------------------------------------------------------- */
template <class R> struct Lookup {  /* LINEAR + CLAMP_TO_EDGE 1D lookup decomposition */
  int i0, i1;
  R t;           /* weight of i1 */
  R dvds_scale;  /* d(coordinate u)/ds where u is inside the interpolation range, else 0 */
};
template <class R> static inline Lookup<R> lookup1d(R s) {
  const int N = VVLIC_TF_ENTRIES;
  Lookup<R> L;
  R u = s * R(N) - R(0.5);
  bool inside = u > R(0) && u < R(N - 1);
  if (!(u > R(-1))) u = R(-1);
  if (u > R(N)) u = R(N);
  R fl = std::floor(u);
  L.t = u - fl;
  int b = (int)fl;
  L.i0 = std::min(std::max(b, 0), N - 1);
  L.i1 = std::min(std::max(b + 1, 0), N - 1);
  L.dvds_scale = inside ? R(N) : R(0);
  return L;
}

struct AdjointOut {
  double* tf;    /* 256*4 */
  double* opac;  /* 256 */
  double* taps;  /* L_b + L_f + 1 */
};

/* noise taps (gradient xyz, value) of every tap of the LIC at `pos` (order: index j + L_b) */
template <class R> static inline void lic_noise_taps(const LicCtx<R>& c, V3<R> pos, V4<R> f0, std::vector<V4<R>>& n) {
  const int lb = c.u->lb, lf = c.u->lf;
  n.assign(lb + lf + 1, V4<R>{R(0), R(0), R(0), R(0)});
  n[lb] = noise_tap<R>(c, pos);
  for (int half = 0; half < 2; ++half) {
    R dirs = half == 0 ? R(-1) : R(1);
    int L = half == 0 ? lb : lf;
    V3<R> p = pos;
    V4<R> step = f0;
    for (int i = 1; i <= L; ++i) {
      p = lic_step<R>(c, p, step, dirs);
      n[half == 0 ? lb - i : lb + i] = noise_tap<R>(c, p);
    }
  }
}

/* illumGradient's colour (inc_illum.glsl:1-41) and its reverse mode.  Forward: N = n(-G),
 * R = n(2 (L.N) N - L), col_c = (tf_c I (ld_c df + 0.3 + la_c) + ls_c I sat(R.V)^e) is with
 * df = sat(L.N) is.  lit_vjp returns dL/dtf_c, dL/dI (colour part) and dL/dG for a colour
 * cotangent dcol.  sat() has derivative 1 strictly inside (0, 1). */
template <class R> struct Lit {
  V3<R> L, V, m, N, r, Rv;
  R mlen, rlen, ln, rv, df, spf, I;
  bool ln_in, rv_in;
};
template <class R>
static inline Lit<R> lit_setup(const LicCtx<R>& c, V3<R> G, R I, V3<R> pos, V3<R> dir) {
  const Uniforms<R>& u = *c.u;
  const vvlic_params& p = *c.p;
  Lit<R> t;
  V3<R> lp{R(p.light_pos[0]), R(p.light_pos[1]), R(p.light_pos[2])};
  V3<R> sv{u.scale_vol_inv[0], u.scale_vol_inv[1], u.scale_vol_inv[2]};
  t.L = normalize(lp - mul(pos, sv));
  t.V = normalize(dir * R(-1));
  t.m = V3<R>{-G.x, -G.y, -G.z};
  t.mlen = std::sqrt(dot(t.m, t.m));
  t.N = normalize(t.m);
  t.ln = dot(t.L, t.N);
  t.r = t.N * (R(2) * t.ln) - t.L;
  t.rlen = std::sqrt(dot(t.r, t.r));
  t.Rv = normalize(t.r);
  t.rv = dot(t.Rv, t.V);
  t.rv_in = t.rv > R(0) && t.rv < R(1);
  t.ln_in = t.ln > R(0) && t.ln < R(1);
  t.spf = std::pow(clamp01(t.rv), R(p.spec_exp));
  t.df = clamp01(t.ln) * u.illum_scale;
  t.I = I;
  return t;
}
template <class R>
static inline void lit_vjp(const LicCtx<R>& c, const Lit<R>& t, V4<R> tf, const R dcol[3], R dtf[3], R* dI, V3<R>* dG) {
  const Uniforms<R>& u = *c.u;
  const vvlic_params& p = *c.p;
  const R is = u.illum_scale;
  R cdf = R(0), cspf = R(0);
  *dI = R(0);
  for (int ch = 0; ch < 3; ++ch) {
    R ld = R(p.light_diffuse[ch]), la = R(p.light_ambient[ch]), ls = R(p.light_specular[ch]);
    R tfc = (&tf.x)[ch];
    dtf[ch] = dcol[ch] * t.I * (ld * t.df + R(0.3) + la) * is;
    *dI += dcol[ch] * (tfc * (ld * t.df + R(0.3) + la) + ls * t.spf) * is;
    cdf += dcol[ch] * tfc * t.I * ld * is;
    cspf += dcol[ch] * ls * t.I * is;
  }
  V3<R> gN{R(0), R(0), R(0)};
  if (t.ln_in) gN = gN + t.L * (cdf * is);
  if (t.rv_in && t.rlen > R(0) && cspf != R(0)) {
    R e = R(p.spec_exp);
    R dspf = cspf * e * std::pow(t.rv, e - R(1));
    V3<R> gR = t.V * dspf;
    /* R = r / |r| */
    V3<R> gr = (gR - t.Rv * dot(t.Rv, gR)) * (R(1) / t.rlen);
    /* r = 2 (L.N) N - L */
    gN = gN + t.L * (R(2) * dot(t.N, gr)) + gr * (R(2) * t.ln);
  }
  V3<R> gm{R(0), R(0), R(0)};
  if (t.mlen > R(0)) gm = (gN - t.N * dot(t.N, gN)) * (R(1) / t.mlen);
  *dG = gm * R(-1);
}

/* One pixel: forward (storing every sample), then the reverse pass with cotangent g_out. */
template <class R> static inline void adjoint_pixel(const Inputs& in, const vvlic_params& p, const Uniforms<R>& u,
                                                    const double* rc, int px, int py, const float g_out[4],
                                                    AdjointOut& out) {
  R o[3], d[3];
  R uu = R(px) + R(0.5), vv = R(py) + R(0.5);
  for (int i = 0; i < 3; ++i) {
    o[i] = R(rc[0 + i]) + uu * R(rc[3 + i]) + vv * R(rc[6 + i]);
    d[i] = R(rc[9 + i]) + uu * R(rc[12 + i]) + vv * R(rc[15 + i]);
  }
  R te;
  if (!ray_entry<R>(o, d, u.extent, rc[18] != 0.0, &te)) return;
  V3<R> sv{u.scale_vol[0], u.scale_vol[1], u.scale_vol[2]};
  V3<R> pos = mul(V3<R>{o[0] + te * d[0], o[1] + te * d[1], o[2] + te * d[2]}, sv);
  V3<R> dir = mul(normalize(V3<R>{d[0], d[1], d[2]}), sv);
  const bool lit = p.illum == VVLIC_ILLUM_GRADIENT;
  LicCtx<R> c{&in, &p, &u, lit};
  struct Sample {
    V3<R> pos;
    V4<R> f;
    R I, idx;
    V3<R> G;
  };
  std::vector<Sample> smp;
  V4<R> src{R(0), R(0), R(0), R(0)};
  bool outside = false;
  const R thr = R(p.alpha_threshold);
  for (int j = 0; !outside && j < u.num_iterations; ++j) {
    for (int i = 0; i < u.num_iterations; ++i) {
      V4<R> f = tex3d_field<R>(in, pos);
      R idx = p.tf_index == VVLIC_TF_INDEX_MAGNITUDE ? f.w : f.z;
      V4<R> il = compute_lic<R>(c, pos, f);
      R I = il.w * u.intensity_scale;
      smp.push_back(Sample{pos, f, I, idx, V3<R>{il.x, il.y, il.z}});
      /* shade to evaluate the termination test */
      Lookup<R> lt = lookup1d<R>(idx), lo = lookup1d<R>(I * R(1.3));
      R tfa = (R(1) - lt.t) * R(in.tf_rgba[4 * lt.i0 + 3]) + lt.t * R(in.tf_rgba[4 * lt.i1 + 3]);
      R op = (R(1) - lo.t) * R(in.tf_opac[lo.i0]) + lo.t * R(in.tf_opac[lo.i1]);
      src.w = alpha_correct<R>(op * tfa, u.alpha_correction);
      pos = pos + dir * u.step_size;
      outside = pos.x < R(0) || pos.y < R(0) || pos.z < R(0) || pos.x > u.tex_max[0] || pos.y > u.tex_max[1] ||
                pos.z > u.tex_max[2] || src.w > thr;
      if (outside) break;
    }
  }
  const size_t S = smp.size();
  /* forward compositing states D[k] = dest before sample k */
  std::vector<V4<R>> D(S + 1);
  D[0] = V4<R>{R(0), R(0), R(0), R(0)};
  struct Sh {
    Lookup<R> lt, lo;
    V4<R> tf;
    R op, a0, base, alpha;
    V3<R> col;
    Lit<R> lt3;
    R ld[3];
  };
  std::vector<Sh> sh(S);
  for (size_t k = 0; k < S; ++k) {
    Sh& h = sh[k];
    h.lt = lookup1d<R>(smp[k].idx);
    for (int ch = 0; ch < 4; ++ch)
      (&h.tf.x)[ch] = (R(1) - h.lt.t) * R(in.tf_rgba[4 * h.lt.i0 + ch]) + h.lt.t * R(in.tf_rgba[4 * h.lt.i1 + ch]);
    h.lo = lookup1d<R>(smp[k].I * R(1.3));
    h.op = (R(1) - h.lo.t) * R(in.tf_opac[h.lo.i0]) + h.lo.t * R(in.tf_opac[h.lo.i1]);
    h.a0 = h.op * h.tf.w;
    h.base = R(1) - h.a0;
    h.alpha = R(1) - std::pow(h.base > R(0) ? h.base : R(0), u.alpha_correction);
    if (lit) {
      h.lt3 = lit_setup<R>(c, smp[k].G, smp[k].I, smp[k].pos, dir);
      R cc[3];
      for (int ch = 0; ch < 3; ++ch)
        cc[ch] = ((&h.tf.x)[ch] * smp[k].I * (R(p.light_diffuse[ch]) * h.lt3.df + R(0.3) + R(p.light_ambient[ch])) +
                  R(p.light_specular[ch]) * h.lt3.spf * smp[k].I) * u.illum_scale;
      h.col = V3<R>{cc[0], cc[1], cc[2]};
    } else if (p.illum == VVLIC_ILLUM_ZOECKLER || p.illum == VVLIC_ILLUM_MALLO) {
      R sp[3];
      line_factors<R>(c, smp[k].pos, dir, smp[k].f, h.ld, sp);
      h.col = V3<R>{h.tf.x * smp[k].I * h.ld[0] + sp[0], h.tf.y * smp[k].I * h.ld[1] + sp[1],
                    h.tf.z * smp[k].I * h.ld[2] + sp[2]};
    } else {
      h.col = V3<R>{smp[k].I * h.tf.x * u.illum_scale, smp[k].I * h.tf.y * u.illum_scale,
                    smp[k].I * h.tf.z * u.illum_scale};
    }
    V4<R> s{h.col.x * h.alpha, h.col.y * h.alpha, h.col.z * h.alpha, h.alpha};
    R om = R(1) - D[k].w;
    D[k + 1] = V4<R>{clamp01(om * s.x + D[k].x), clamp01(om * s.y + D[k].y), clamp01(om * s.z + D[k].z),
                     clamp01(om * s.w + D[k].w)};
  }
  /* reverse */
  V4<R> g{R(g_out[0]), R(g_out[1]), R(g_out[2]), R(g_out[3])};
  std::vector<V4<R>> n;
  for (size_t kk = S; kk-- > 0;) {
    const Sh& h = sh[kk];
    const V4<R>& Dp = D[kk];
    V4<R> s{h.col.x * h.alpha, h.col.y * h.alpha, h.col.z * h.alpha, h.alpha};
    R om = R(1) - Dp.w;
    R uarr[4] = {om * s.x + Dp.x, om * s.y + Dp.y, om * s.z + Dp.z, om * s.w + Dp.w};
    R gu[4];
    for (int ch = 0; ch < 4; ++ch) gu[ch] = (uarr[ch] >= R(0) && uarr[ch] <= R(1)) ? (&g.x)[ch] : R(0);
    R ds[4];
    for (int ch = 0; ch < 4; ++ch) ds[ch] = om * gu[ch];
    V4<R> gp{gu[0], gu[1], gu[2], gu[3]};
    gp.w -= gu[0] * s.x + gu[1] * s.y + gu[2] * s.z + gu[3] * s.w;
    /* s = (col*alpha, alpha) */
    R dcol[3] = {ds[0] * h.alpha, ds[1] * h.alpha, ds[2] * h.alpha};
    R dalpha = ds[0] * h.col.x + ds[1] * h.col.y + ds[2] * h.col.z + ds[3];
    R dbase_da0 = h.base > R(0) ? u.alpha_correction * std::pow(h.base, u.alpha_correction - R(1)) : R(0);
    R da0 = dalpha * dbase_da0;
    /* a0 = op(1.3 I) * tf.a */
    R dop = da0 * h.tf.w;
    R dtfa = da0 * h.op;
    out.opac[h.lo.i0] += double(dop * (R(1) - h.lo.t));
    out.opac[h.lo.i1] += double(dop * h.lo.t);
    R dI = dop * (R(in.tf_opac[h.lo.i1]) - R(in.tf_opac[h.lo.i0])) * h.lo.dvds_scale * R(1.3);
    R dtf[4] = {R(0), R(0), R(0), dtfa};
    V3<R> dG{R(0), R(0), R(0)};
    if (lit) {
      R dI_col;
      lit_vjp<R>(c, h.lt3, h.tf, dcol, dtf, &dI_col, &dG);
      dI += dI_col;
    } else if (p.illum == VVLIC_ILLUM_ZOECKLER || p.illum == VVLIC_ILLUM_MALLO) {
      for (int ch = 0; ch < 3; ++ch) dtf[ch] = dcol[ch] * smp[kk].I * h.ld[ch];
      dI += dcol[0] * h.tf.x * h.ld[0] + dcol[1] * h.tf.y * h.ld[1] + dcol[2] * h.tf.z * h.ld[2];
    } else {
      /* col = I * tf.rgb * illumScale */
      for (int ch = 0; ch < 3; ++ch) dtf[ch] = dcol[ch] * smp[kk].I * u.illum_scale;
      dI += (dcol[0] * h.tf.x + dcol[1] * h.tf.y + dcol[2] * h.tf.z) * u.illum_scale;
    }
    for (int ch = 0; ch < 4; ++ch) {
      out.tf[4 * h.lt.i0 + ch] += double(dtf[ch] * (R(1) - h.lt.t));
      out.tf[4 * h.lt.i1 + ch] += double(dtf[ch] * h.lt.t);
    }
    /* I = intensity_scale * sum_j w_j n_j, G = sum_j w_j g_j */
    R dIraw = dI * u.intensity_scale;
    if (dIraw != R(0) || dG.x != R(0) || dG.y != R(0) || dG.z != R(0)) {
      lic_noise_taps<R>(c, smp[kk].pos, smp[kk].f, n);
      for (size_t j = 0; j < n.size(); ++j)
        out.taps[j] += double(dIraw * n[j].w + dG.x * n[j].x + dG.y * n[j].y + dG.z * n[j].z);
    }
    g = gp;
  }
}

template <class R> static inline void adjoint(const Inputs& in, const vvlic_params& p, const double* rc, int W,
                                              int H, const float* g_img, AdjointOut& out, int threads) {
  Uniforms<R> u = uniforms<R>(in, p);
  const int ntaps = u.lb + u.lf + 1;
  int nt = 1;
#if defined(_OPENMP)
  if (threads > 0) omp_set_num_threads(threads);
  nt = omp_get_max_threads();
#endif
  std::vector<double> acc((size_t)nt * (1024 + 256 + ntaps), 0.0);
#if defined(_OPENMP)
#pragma omp parallel
#endif
  {
    int tid = 0;
#if defined(_OPENMP)
    tid = omp_get_thread_num();
#endif
    double* base = acc.data() + (size_t)tid * (1024 + 256 + ntaps);
    AdjointOut mine{base, base + 1024, base + 1280};
    const int kChunk = 16;  /* runs of pixels: a few nonzero rows still occupy every core */
    const int per_row = (W + kChunk - 1) / kChunk;
#if defined(_OPENMP)
#pragma omp for schedule(dynamic, 1)
#endif
    for (long long t = 0; t < (long long)H * per_row; ++t)
      for (int py = (int)(t / per_row), px = (int)(t % per_row) * kChunk, pe = std::min(W, px + kChunk); px < pe;
           ++px) {
        const float* g = g_img + 4 * ((size_t)py * W + px);
        /* a zero cotangent contributes exactly zero: rows outside a checked subset cost nothing */
        if (g[0] == 0.0f && g[1] == 0.0f && g[2] == 0.0f && g[3] == 0.0f) continue;
        adjoint_pixel<R>(in, p, u, rc, px, py, g, mine);
      }
  }
  for (int t = 0; t < nt; ++t) {
    const double* b = acc.data() + (size_t)t * (1024 + 256 + ntaps);
    for (int i = 0; i < 1024; ++i) out.tf[i] += b[i];
    for (int i = 0; i < 256; ++i) out.opac[i] += b[1024 + i];
    for (int i = 0; i < ntaps; ++i) out.taps[i] += b[1280 + i];
  }
}

/* Render the rows listed in `rows` (all rows when rows == NULL) into out (nrows x W x 4). */
template <class R> static inline void render(const Inputs& in, const vvlic_params& p, const double* rc, int W, int H,
                                             const int32_t* rows, int nrows, float* out, uint32_t* samples,
                                             int threads, const double* slicing = nullptr) {
  Uniforms<R> u = uniforms<R>(in, p);
  int nr = rows ? nrows : H;
  /* threads take runs of kChunk pixels, so that a few rows still occupy every core */
  const int kChunk = 16;
  const int per_row = (W + kChunk - 1) / kChunk;
  const long long items = (long long)nr * per_row;
#if defined(_OPENMP)
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (long long t = 0; t < items; ++t) {
    const int r = (int)(t / per_row), x0 = (int)(t % per_row) * kChunk;
    const int py = rows ? rows[r] : r;
    for (int px = x0; px < std::min(W, x0 + kChunk); ++px) {
      uint32_t s = render_pixel<R>(in, p, u, rc, px, py, out + 4 * ((size_t)r * W + px), slicing);
      if (samples) samples[(size_t)r * W + px] = s;
    }
  }
  (void)threads;
}

/* ------------------------------------------------------------------------------------- */
/* defaults and filter tables, restated independently of the library                      */
/* ------------------------------------------------------------------------------------- */

/* LICParams() (types.h:91-99) plus the fixed state the reference's shaders run with: the
 * never-written logEyeDist (factor 0.3, inc_lic.glsl:114), the termination threshold 0.95
 * (lic3d_fragment.glsl:91), the scalar-gate bounds (inc_lic.glsl:80), GL LIGHT0 as the
 * application sets it (spot exponent 40, 3DLIC.cpp:736; white diffuse and specular, no
 * ambient) and every reproduced quirk.  Kernel-selection fields stay 0. */
static inline void params_default(vvlic_params& p) {
  std::memset(&p, 0, sizeof p);
  p.step_size_vol = 1.0f / 128.0f;
  p.gradient_scale = 30.0f;
  p.illum_scale = 1.0f;
  p.freq_scale = 1.0f;
  p.num_iterations = 255;
  p.steps_forward = p.steps_backward = 32;
  p.step_size_lic = 0.01f;
  p.integrator = VVLIC_HEUN;
  p.illum = VVLIC_ILLUM_NONE;
  p.tf_index = VVLIC_TF_INDEX_DIR_Z;
  p.gate_lo = 0.1f;
  p.gate_hi = 0.3f;
  p.eye_dist_factor = 0.3f;
  p.alpha_threshold = 0.95f;
  p.quirks = VVLIC_QUIRK_UNIFORM_SCALE_BUG | VVLIC_QUIRK_GRAD_NOISE_NO_FREQ | VVLIC_QUIRK_ZOECKLER_LUMINANCE;
  const float light[3] = {0.5f, 0.5f, 1.5f};
  for (int i = 0; i < 3; ++i) {
    p.light_pos[i] = light[i];
    p.light_diffuse[i] = p.light_specular[i] = 1.0f;
    p.light_ambient[i] = 0.0f;
  }
  p.spec_exp = 40.0f;
  p.technique = VVLIC_TECHNIQUE_RAYCAST;
}

/* Camera() (camera.cpp:42-46): identity rotation, distance 4, fovy 35 degrees; the
 * orthographic fields default to the +z view of the unit cube. */
static inline void view_default(vvlic_view& v) {
  std::memset(&v, 0, sizeof v);
  v.projection = VVLIC_PERSPECTIVE;
  v.quat[3] = 1.0f;
  v.distance = 4.0f;
  v.fovy_deg = 35.0f;
  v.ortho_center[0] = v.ortho_center[1] = 0.5f;
  v.ortho_right[0] = 0.5f;
  v.ortho_up[1] = 0.5f;
  v.ortho_dir[2] = 1.0f;
}

/* LineMat() (illumination.h:42-54) and Illumination() (illumination.cpp:43): white light, ambient 0.1, diffuse
 * 0.5, specular 0.8, exponents 40 / 2, 256 x 256 tables. */
static inline void line_material_default(vvlic_line_material& m) {
  for (int i = 0; i < 4; ++i) {
    m.light_color[i] = 1.0f;
    m.ambient[i] = 0.1f;
    m.diffuse[i] = 0.5f;
    m.specular[i] = 0.8f;
  }
  m.spec_exp = 40.0f;
  m.diff_exp = 2.0f;
  m.width = m.height = 256;
}

/* Filter-kernel table of `width` texels rounded up to a power of two (nextPowerTwo,
 * dataset.cpp:1407).  Box: LICFilter::createBoxFilter, every texel 255 (dataset.cpp:1405-1413).
 * The reference loads the other kernels from PNGs it does not ship; their profiles over the
 * texel centres x_i = (2i + 1) / W - 1 in [-1, 1] (x = tap offset / L) are
 *   triangle 1 - |x|,  cos^2 cos(pi x / 2)^2,  Gaussian exp(-(x L)^2 / (2 sigma^2)), sigma = L/3,
 * stored as round(255 v).  Returns the table width, or 0 for a bad kind or width. */
static inline int filter_table(int kind, int width, uint8_t* out) {
  if (width < 2 || width > 1024) return 0;
  int W = 1;
  while (W < width) W <<= 1;
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < W; ++i) {
    const double x = (double)(2 * i + 1) / (double)W - 1.0;
    double v;
    if (kind == VVLIC_FILTER_BOX) v = 1.0;
    else if (kind == VVLIC_FILTER_TRIANGLE) v = 1.0 - std::fabs(x);
    else if (kind == VVLIC_FILTER_COS2) { const double c = std::cos(0.5 * pi * x); v = c * c; }
    else if (kind == VVLIC_FILTER_GAUSSIAN) v = std::exp(-(x * x) * 4.5);  /* (x L)^2 / (2 (L/3)^2) */
    else return 0;
    v = std::min(std::max(v, 0.0), 1.0);
    out[i] = (uint8_t)std::floor(255.0 * v + 0.5);
  }
  return W;
}

}  // namespace vvo

#endif  // VVLIC_ORACLE_HPP_
