// Illuminated-streamline tables of Illumination::createIllumTextures (illumination.cpp:58-391)
// and their C ABI.  The tables are built once per material on the host in double precision,
// in the reference's order of operations (this file is compiled without contraction so the
// bytes do not depend on the host compiler), stored as the 8-bit textures the reference
// uploads, and sampled bilinearly by the render kernels (shade() in vvlic_device.cuh).
#include <cmath>
#include <cstring>
#include <vector>

#include "vvlic_host.hpp"

namespace vvlic {
namespace {

constexpr double kPi = 3.14159265358979323846;

// glTexImage2D of GL_FLOAT data into an 8-bit normalised format: round(clamp(v, 0, 1) * 255).
// A NaN (never produced by the default material) stores 0.
uint8_t unorm8(float v) {
  double c = v;
  if (!(c > 0.0)) c = 0.0;
  if (c > 1.0) c = 1.0;
  return (uint8_t)std::floor(c * 255.0 + 0.5);
}

double clamp_unit(double v, double lo) { return v < lo ? lo : (v > 1.0 ? 1.0 : v); }

// Integrand of the Mallo specular term, max(0, cos(theta - beta))^n * cos(theta) / 2
// (illumination.cpp:383-391).
double mallo_integrand(double beta, double n, double theta) {
  double c = std::cos(theta - beta);
  if (c < 0.0) c = 0.0;
  return std::pow(c, n) * (std::cos(theta) / 2.0);
}

// Composite Simpson rule with 2m = 20 intervals over [alpha - pi/2, pi/2], accumulated in the
// reference's order: pairs (2 f(x_2k), 4 f(x_2k+1)), then + f(b) - f(a) (illumination.cpp:355-380).
double mallo_specular(double alpha, double beta, double n) {
  const int m = 10;
  const double a = alpha - kPi / 2.0, b = kPi / 2.0, h = (b - a) / (2.0 * m);
  double acc = 0.0;
  for (int i = 0; i < 2 * m; i += 2) {
    acc += 2.0 * mallo_integrand(beta, n, a + i * h);
    acc += 4.0 * mallo_integrand(beta, n, a + (i + 1) * h);
  }
  acc += mallo_integrand(beta, n, b);
  acc -= mallo_integrand(beta, n, a);
  return acc * (h / 3.0);
}

}  // namespace

int lut_size(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

void build_illum_luts(const vvlic_line_material& mat, int w, int h, uint8_t* out) {
  uint8_t* zt = out;
  uint8_t* md = out + (size_t)4 * w * h;
  uint8_t* ms = out + (size_t)8 * w * h;
  // Zoeckler et al. 1996 (illumination.cpp:96-172): x, y sample L.T and V.T on [-1, 1] at
  // x / (w - 1); diffuse = ambient + sqrt(1 - lt^2)^diffExp * diffuse, specular =
  // |lt vt - sqrt(1 - lt^2) sqrt(1 - vt^2)|^specExp * specular, both halved and clamped.
  const double irx = 1.0 / (double)(w - 1), iry = 1.0 / (double)(h - 1);
  const float amb = mat.ambient[0] * mat.light_color[0];  // float product, as in the reference
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const double lt = 2.0 * ((double)x * irx) - 1.0, vt = 2.0 * ((double)y * iry) - 1.0;
      const double diffuse = std::pow(std::sqrt(1.0 - lt * lt), (double)mat.diff_exp);
      double d = lt * vt - std::sqrt(1.0 - lt * lt) * std::sqrt(1.0 - vt * vt);
      d = d < -1.0 ? -1.0 : (d > 1.0 ? 1.0 : d);
      double td = (double)amb + diffuse * mat.diffuse[0] * mat.light_color[0];
      double ts = std::pow(std::fabs(d), (double)mat.spec_exp) * mat.specular[0] * mat.light_color[0];
      td = clamp_unit(td * 0.5, 0.0);
      ts = clamp_unit(ts * 0.5, 0.0);
      const uint8_t L = unorm8((float)td), A = unorm8((float)ts * 0.9f);
      uint8_t* o = zt + 4 * ((size_t)y * w + x);
      o[0] = o[1] = o[2] = L;  // LUMINANCE_ALPHA samples as (L, L, L, A)
      o[3] = A;
    }
  // Mallo et al. 2005 (illumination.cpp:205-290): texel centres s, t; alpha = acos(2s - 1),
  // beta = acos(2t - 1); F_d = sqrt(1 - lt^2) (sin a + (pi - a) cos a) / 4; F_s = 3.5 * the
  // Simpson integral; per channel times material * light colour, clamped.
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const double s = ((double)x + 0.5) / w, t = ((double)y + 0.5) / h;
      const double alpha = std::acos(2.0 * s - 1.0), beta = std::acos(2.0 * t - 1.0), lt = 2.0 * t - 1.0;
      const double fd = std::sqrt(1.0 - lt * lt) * (std::sin(alpha) + (kPi - alpha) * std::cos(alpha)) * 0.25;
      const double fs = 3.5 * mallo_specular(alpha, beta, (double)mat.spec_exp);
      const size_t o = 4 * ((size_t)y * w + x);
      for (int i = 0; i < 4; ++i) {
        md[o + i] = unorm8((float)clamp_unit(fd * mat.diffuse[i] * mat.light_color[i], 0.0));
        ms[o + i] = unorm8((float)clamp_unit(fs * mat.specular[i] * mat.light_color[i], 0.0));
      }
    }
}

vvlic_status ensure_illum_luts(vvlic_ctx* c) {
  if (c->luts_valid) return VVLIC_OK;
  const int w = lut_size(c->line_mat.width), h = lut_size(c->line_mat.height);
  const size_t bytes = (size_t)12 * w * h;
  std::vector<uint8_t> host(bytes);
  build_illum_luts(c->line_mat, w, h, host.data());
  if (c->lut_bytes < bytes) {
    if (c->d_luts) cudaFree(c->d_luts);  // cudaFree waits for the kernels that read the old tables
    c->d_luts = nullptr;
    c->lut_bytes = 0;
    cudaError_t e = cudaMalloc(&c->d_luts, bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "illumination tables");
    c->lut_bytes = bytes;
  }
  cudaError_t e = after_launches(c);  // renders in flight may read the old tables
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_luts, host.data(), bytes, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);  // `host` is pageable and local
  if (e != cudaSuccess) return cuda_fail(c, e, "illumination tables upload");
  c->lut_w = w;
  c->lut_h = h;
  c->luts_valid = true;
  return VVLIC_OK;
}

}  // namespace vvlic

using namespace vvlic;

extern "C" void vvlic_line_material_default(vvlic_line_material* m) {
  if (!m) return;
  for (int i = 0; i < 4; ++i) {
    m->light_color[i] = 1.0f;
    m->ambient[i] = 0.1f;
    m->diffuse[i] = 0.5f;
    m->specular[i] = 0.8f;
  }
  m->spec_exp = 40.0f;
  m->diff_exp = 2.0f;
  m->width = 256;
  m->height = 256;
}

extern "C" vvlic_status vvlic_set_line_material(vvlic_ctx* c, const vvlic_line_material* m) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!m) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_line_material: null material");
  if (m->width < 2 || m->height < 2 || m->width > 4096 || m->height > 4096)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_line_material: table size must be in [2, 4096]");
  const float* all = &m->light_color[0];
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(all[i])) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_line_material: non-finite colour");
  if (!std::isfinite(m->spec_exp) || !std::isfinite(m->diff_exp) || m->spec_exp < 0.0f || m->diff_exp < 0.0f)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_line_material: exponents must be finite and >= 0");
  c->line_mat = *m;
  c->luts_valid = false;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_get_illum_luts(vvlic_ctx* c, uint8_t* zoeckler, uint8_t* mallo_diffuse,
                                            uint8_t* mallo_specular, int32_t* width, int32_t* height) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  DeviceGuard g(c->device);
  vvlic_status st = ensure_illum_luts(c);
  if (st) return st;
  if (width) *width = c->lut_w;
  if (height) *height = c->lut_h;
  const size_t one = (size_t)4 * c->lut_w * c->lut_h;
  uint8_t* dst[3] = {zoeckler, mallo_diffuse, mallo_specular};
  for (int i = 0; i < 3; ++i) {
    if (!dst[i]) continue;
    cudaError_t e = cudaMemcpy(dst[i], (const uint8_t*)c->d_luts + i * one, one, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "get_illum_luts");
  }
  return VVLIC_OK;
}
