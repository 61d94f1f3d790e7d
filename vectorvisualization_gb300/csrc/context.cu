// C ABI of libvvlic: context, uploads, tables, parameters, view and the render entry points.
//
// The host side derives everything the reference computes on the CPU per frame
// (Renderer::setRenderVolParams renderer.cpp:925-996, the view of Camera::setCamera
// camera.cpp:56-67, the filter-kernel lookups of computeLIC inc_lic.glsl:156, 172, 182, 196) and hands it
// to the kernels as one by-value argument block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/vvlic.h"
#include "vvlic_device.cuh"
#include "vvlic_host.hpp"
#include "vvlic_launch.hpp"

using namespace vvlic;

// ------------------------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------------------------
namespace vvlic {

vvlic_status fail(vvlic_ctx* c, vvlic_status s, const char* fmt, ...) {
  if (c) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return s;
}

vvlic_status cuda_fail(vvlic_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation)
    return fail(c, VVLIC_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  return fail(c, VVLIC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// VectorDataSet::loadData geometry (dataset.cpp:139-176), in float like the reference.
Geometry make_geometry(const int n[3], const float* sd_in) {
  Geometry g;
  float sd[3] = {1.f, 1.f, 1.f};
  if (sd_in)
    for (int i = 0; i < 3; ++i) sd[i] = sd_in[i];
  float max_vol = 0.f;
  int max_tex = 0;
  for (int i = 0; i < 3; ++i) {
    max_vol = std::max(max_vol, (float)n[i] * sd[i]);
    max_tex = std::max(max_tex, n[i]);
  }
  for (int i = 0; i < 3; ++i) {
    g.slice_dist[i] = sd[i];
    g.scale[i] = (float)max_tex / ((float)n[i] * sd[i]);
    g.scale_inv[i] = (float)n[i] * sd[i] / (float)max_tex;
    g.extent[i] = (float)n[i] * sd[i] / max_vol;
    g.center[i] = g.extent[i] / 2.0f;
    g.tex_max[i] = g.extent[i] * g.scale[i];
  }
  return g;
}

static int next_pow2(int w) {
  int p = 1;
  while (p < w) p <<= 1;
  return p;
}

// texture1D(licKernelSampler, s).r with LINEAR filtering and GL_CLAMP (zero border) or
// CLAMP_TO_EDGE over a LUMINANCE8 table (dataset.cpp:1470-1500).
static double kernel_lookup(const uint8_t* t, int W, double s, int clamp_mode) {
  s = std::min(std::max(s, 0.0), 1.0);
  double u = s * W - 0.5, fl = std::floor(u), a = u - fl;
  int i0 = (int)fl;
  auto tex = [&](int i) -> double {
    if (clamp_mode == VVLIC_KERNEL_CLAMP_EDGE) i = std::min(std::max(i, 0), W - 1);
    else if (i < 0 || i >= W) return 0.0;
    return t[i] / 255.0;
  };
  return (1.0 - a) * tex(i0) + a * tex(i0 + 1);
}

// Effective LIC lengths: the low-resolution preview substitutes 15/15 (renderer.cpp:956-962).
static void effective_steps(const vvlic_params& p, int* lb, int* lf) {
  *lb = p.low_res ? 15 : p.steps_backward;
  *lf = p.low_res ? 15 : p.steps_forward;
}

// Tap weights w[j], j = -L_b..L_f, at the offsets computeLIC walks (inc_lic.glsl:156, 182, 191, 196).
void derive_taps_from_table(const uint8_t* t, int W, int clamp, bool is_box, int lb, int lf, float* taps,
                            float* inv_area) {
  taps[lb] = (float)kernel_lookup(t, W, 0.5, clamp);
  double off = 0.5, kb = lb > 0 ? 0.5 / lb : 0.0, kf = lf > 0 ? 0.5 / lf : 0.0;
  for (int i = 1; i <= lb; ++i) {
    off -= kb;
    taps[lb - i] = (float)kernel_lookup(t, W, off, clamp);
  }
  off = 0.5;
  for (int i = 1; i <= lf; ++i) {
    off += kf;
    taps[lb + i] = (float)kernel_lookup(t, W, off, clamp);
  }
  if (is_box) {
    *inv_area = 0.5f;  // LICFilter::createBoxFilter (dataset.cpp:1412)
  } else {
    float area = 0.0f;  // calcFilterKernelInvArea (dataset.cpp:1503-1512)
    for (int i = 0; i < W; ++i) area += t[i];
    *inv_area = 0.5f * W * 255.0f / area;
  }
}

vvlic_status derive_taps(const vvlic_ctx* c, int lb, int lf, float* taps, float* inv_area) {
  if (c->taps_override) {
    if (c->taps_lb != lb || c->taps_lf != lf) return VVLIC_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < lb + lf + 1; ++i) taps[i] = c->taps[i];
    *inv_area = c->taps_inv_area;
    return VVLIC_OK;
  }
  derive_taps_from_table(c->filter, c->filter_width, c->filter_clamp, c->filter_is_box, lb, lf, taps, inv_area);
  return VVLIC_OK;
}

// A filter table as vvlic_set_filter_table stores it: centred in the next power of two.
int centre_filter_table(const uint8_t* table, int width, uint8_t* out1024, bool* is_box) {
  const int W = next_pow2(width), shift = (W - width) / 2;
  std::memset(out1024, 0, 1024);
  std::memcpy(out1024 + shift, table, width);
  bool box = true;
  for (int i = 0; i < W; ++i) box = box && out1024[i] == 255;
  *is_box = box;
  return W;
}

// Rays of the view for a volume (camera.cpp:56-67 followed by glTranslatef(-center),
// renderer.cpp:146): origin/direction as affine functions of the pixel centre.
void derive_rays(const vvlic_view& v, const Geometry& g, int W, int H, double* c) {
  for (int i = 0; i < 21; ++i) c[i] = 0.0;
  if (v.projection == VVLIC_ORTHOGRAPHIC) {
    for (int i = 0; i < 3; ++i) {
      c[i] = (double)v.ortho_center[i] - v.ortho_right[i] - v.ortho_up[i];
      c[3 + i] = 2.0 * v.ortho_right[i] / W;
      c[6 + i] = 2.0 * v.ortho_up[i] / H;
      c[9 + i] = v.ortho_dir[i];
    }
    return;
  }
  double x = v.quat[0], y = v.quat[1], z = v.quat[2], w = v.quat[3];
  double qn = std::sqrt(x * x + y * y + z * z + w * w);
  if (qn > 0) {
    x /= qn;
    y /= qn;
    z /= qn;
    w /= qn;
  } else {
    w = 1.0;
  }
  // R(q); object-space vectors are R^T times eye-space vectors
  const double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)},
                          {2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)},
                          {2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)}};
  auto to_obj = [&](double ex, double ey, double ez, double* out) {
    for (int i = 0; i < 3; ++i) out[i] = R[0][i] * ex + R[1][i] * ey + R[2][i] * ez;
  };
  double eye[3];
  to_obj(-(double)v.pan[0], -(double)v.pan[1], (double)v.distance - v.pan[2], eye);
  for (int i = 0; i < 3; ++i) c[i] = eye[i] + g.center[i];
  const double aspect = v.aspect > 0 ? (double)v.aspect : (double)W / H;
  const double t = std::tan((double)v.fovy_deg * M_PI / 360.0);  // gluPerspective(fovy, ...)
  to_obj(-aspect * t, -t, -1.0, c + 9);
  to_obj(2.0 * aspect * t / W, 0.0, 0.0, c + 12);
  to_obj(0.0, 2.0 * t / H, 0.0, c + 15);
  c[18] = 1.0;
}

// Slicing set-up of ViewSlicing::setupSlicing (slicing.cpp:42-103): the unit view direction in
// object space (the third row of the modelview matrix divided by its z translation, pointing
// into the scene), the slab depth D = 2 * sum |v_i| * extent_i / 2 and N = (int)(D / spacing) + 1.
void derive_slicing(const vvlic_view& v, const Geometry& g, float spacing, float vdir[3], float* depth, int* n) {
  double dv[3];
  if (v.projection == VVLIC_ORTHOGRAPHIC) {
    for (int i = 0; i < 3; ++i) dv[i] = v.ortho_dir[i];
  } else {
    double x = v.quat[0], y = v.quat[1], z = v.quat[2], w = v.quat[3];
    double qn = std::sqrt(x * x + y * y + z * z + w * w);
    if (qn > 0) {
      x /= qn;
      y /= qn;
      z /= qn;
      w /= qn;
    } else {
      w = 1.0;
    }
    const double R2[3] = {2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)};  // row 2 of R(q)
    const double Rc_z = R2[0] * g.center[0] + R2[1] * g.center[1] + R2[2] * g.center[2];
    const double m14 = (double)v.pan[2] - v.distance - Rc_z;
    for (int i = 0; i < 3; ++i) dv[i] = R2[i] / m14;
  }
  float f[3] = {(float)dv[0], (float)dv[1], (float)dv[2]};
  const float inv = 1.0f / std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  float d6 = 0.0f;
  for (int i = 0; i < 3; ++i) {
    vdir[i] = f[i] * inv;
    d6 += std::fabs(vdir[i]) * (0.5f * g.extent[i]);
  }
  *depth = 2.0f * d6;
  *n = (int)(*depth / spacing) + 1;
}

}  // namespace vvlic

// ------------------------------------------------------------------------------------------
// defaults
// ------------------------------------------------------------------------------------------
extern "C" void vvlic_params_default(vvlic_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->step_size_vol = 1.0f / 128.0f;  // LICParams() (types.h:91-99)
  p->gradient_scale = 30.0f;
  p->illum_scale = 1.0f;
  p->freq_scale = 1.0f;
  p->num_iterations = 255;
  p->steps_forward = 32;
  p->steps_backward = 32;
  p->step_size_lic = 0.01f;
  p->integrator = VVLIC_HEUN;
  p->illum = VVLIC_ILLUM_NONE;
  p->tf_index = VVLIC_TF_INDEX_DIR_Z;
  p->gate_lo = 0.1f;
  p->gate_hi = 0.3f;
  p->eye_dist_factor = 0.3f;
  p->alpha_threshold = 0.95f;
  p->quirks = VVLIC_QUIRKS_REFERENCE;
  p->light_pos[0] = 0.5f;
  p->light_pos[1] = 0.5f;
  p->light_pos[2] = 1.5f;
  p->spec_exp = 40.0f;
  for (int i = 0; i < 3; ++i) {
    p->light_diffuse[i] = 1.0f;
    p->light_specular[i] = 1.0f;
    p->light_ambient[i] = 0.0f;
  }
  p->sampler = VVLIC_SAMPLER_HYBRID;
  p->schedule = VVLIC_SCHEDULE_QUEUE;
  p->technique = VVLIC_TECHNIQUE_RAYCAST;
}

extern "C" void vvlic_view_default(vvlic_view* v) {
  if (!v) return;
  std::memset(v, 0, sizeof *v);
  v->projection = VVLIC_PERSPECTIVE;
  v->quat[3] = 1.0f;
  v->distance = 4.0f;
  v->fovy_deg = 35.0f;
  v->ortho_center[0] = v->ortho_center[1] = 0.5f;
  v->ortho_right[0] = 0.5f;
  v->ortho_up[1] = 0.5f;
  v->ortho_dir[2] = 1.0f;
}

extern "C" const char* vvlic_status_string(vvlic_status s) {
  switch (s) {
    case VVLIC_OK: return "ok";
    case VVLIC_ERR_INVALID_ARGUMENT: return "invalid argument";
    case VVLIC_ERR_OUT_OF_MEMORY: return "out of memory";
    case VVLIC_ERR_CUDA: return "CUDA error";
    case VVLIC_ERR_NO_DEVICE: return "no CUDA device";
    case VVLIC_ERR_NOT_READY: return "input not set";
    case VVLIC_ERR_TIMEOUT: return "device wait timed out";
    case VVLIC_ERR_UNSUPPORTED: return "unsupported";
    case VVLIC_ERR_BAD_HANDLE: return "bad handle";
    case VVLIC_ERR_IO: return "I/O error";
    case VVLIC_ERR_FORMAT: return "format error";
    default: return "unknown status";
  }
}

extern "C" int32_t vvlic_abi_version(void) { return VVLIC_ABI_VERSION; }

extern "C" vvlic_status vvlic_make_filter_table(int32_t filter, int32_t width, uint8_t* out, int32_t* out_width) {
  if (!out || !out_width || width < 2 || width > 1024) return VVLIC_ERR_INVALID_ARGUMENT;
  const int W = next_pow2(width);
  if (W > 1024) return VVLIC_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < W; ++i) {
    const double t = (i + 0.5) / W;  // texel centre in [0,1]; 0.5 is the streamline centre
    const double d = 2.0 * t - 1.0;  // in [-1, 1]
    double v;
    switch (filter) {
      case VVLIC_FILTER_BOX: v = 1.0; break;
      case VVLIC_FILTER_TRIANGLE: v = 1.0 - std::fabs(d); break;
      case VVLIC_FILTER_COS2: v = std::cos(M_PI * d / 2.0) * std::cos(M_PI * d / 2.0); break;
      case VVLIC_FILTER_GAUSSIAN: v = std::exp(-4.5 * d * d); break;  // sigma = L/3 in tap units
      default: return VVLIC_ERR_INVALID_ARGUMENT;
    }
    out[i] = (uint8_t)std::lround(std::min(std::max(v, 0.0), 1.0) * 255.0);
  }
  *out_width = W;
  return VVLIC_OK;
}

// ------------------------------------------------------------------------------------------
// context
// ------------------------------------------------------------------------------------------
static void default_tables(vvlic_ctx* c) {
  // TransferEdit(): rgb identity, alpha and opacity max(0, i-20) (transferEdit.cpp:76-82)
  for (int i = 0; i < VVLIC_TF_ENTRIES; ++i) {
    for (int ch = 0; ch < 3; ++ch) c->tf[4 * i + ch] = (float)i / 255.0f;
    c->tf[4 * i + 3] = (float)(i < 20 ? 0 : i - 20) / 255.0f;
    c->tf[4 * VVLIC_TF_ENTRIES + i] = (float)(i < 20 ? 0 : i - 20) / 255.0f;
  }
  // LICFilter::createBoxFilter(256) (dataset.cpp:1405-1413), GL_CLAMP
  int w = 0;
  vvlic_make_filter_table(VVLIC_FILTER_BOX, 256, c->filter, &w);
  c->filter_width = w;
  c->filter_clamp = VVLIC_KERNEL_CLAMP_BORDER;
  c->filter_is_box = true;
}

extern "C" vvlic_status vvlic_create(vvlic_ctx** out, int32_t device) {
  if (!out) return VVLIC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) return VVLIC_ERR_NO_DEVICE;
  if (device < 0 || device >= count) return VVLIC_ERR_INVALID_ARGUMENT;
  vvlic_ctx* c = new vvlic_ctx();
  c->device = device;
  vvlic_params_default(&c->params);
  vvlic_view_default(&c->view);
  vvlic_line_material_default(&c->line_mat);
  default_tables(c);
  DeviceGuard g(device);
  if ((e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_tf, sizeof(float) * 5 * VVLIC_TF_ENTRIES)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_counters, sizeof(unsigned long long) * 4)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_scratch_word, sizeof(unsigned) * 4)) != cudaSuccess ||
      (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess ||
      (e = cudaMemcpy(c->d_tf, c->tf, sizeof(float) * 5 * VVLIC_TF_ENTRIES, cudaMemcpyHostToDevice)) != cudaSuccess) {
    vvlic_destroy(c);
    return e == cudaErrorMemoryAllocation ? VVLIC_ERR_OUT_OF_MEMORY : VVLIC_ERR_CUDA;
  }
  *out = c;
  return VVLIC_OK;
}

static void free_volume(Volume& v) {
  if (v.d_licvol) cudaFree(v.d_licvol);
  if (v.tex) cudaDestroyTextureObject(v.tex);
  if (v.array) cudaFreeArray(v.array);
  if (v.d_texels) cudaFree(v.d_texels);
  if (v.d_cells) cudaFree(v.d_cells);
  v = Volume();
}

static void free_noise(NoiseTex& n) {
  if (n.tex) cudaDestroyTextureObject(n.tex);
  if (n.array) cudaFreeArray(n.array);
  if (n.d_texels) cudaFree(n.d_texels);
  if (n.d_cells) cudaFree(n.d_cells);
  n = NoiseTex();
}

extern "C" vvlic_status vvlic_destroy(vvlic_ctx* c) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  DeviceGuard g(c->device);
  cudaDeviceSynchronize();  // renders and stream-ordered updates on any stream
  for (auto& kv : c->vols) free_volume(kv.second);
  free_noise(c->noise);
  if (c->d_scalar) cudaFree(c->d_scalar);
  if (c->d_tf) cudaFree(c->d_tf);
  if (c->d_luts) cudaFree(c->d_luts);
  if (c->d_counters) cudaFree(c->d_counters);
  if (c->d_scratch_word) cudaFree(c->d_scratch_word);
  if (c->d_image) cudaFree(c->d_image);
  if (c->d_upload) cudaFree(c->d_upload);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  if (c->d_field_stage) cudaFree(c->d_field_stage);
  if (c->d_noise_stage) cudaFree(c->d_noise_stage);
  for (cudaEvent_t ev : {c->ev_field_copied, c->ev_field_used, c->ev_noise_copied, c->ev_noise_used})
    if (ev) cudaEventDestroy(ev);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->d_sched) cudaFree(c->d_sched);
  if (c->d_tape) cudaFree(c->d_tape);
  if (c->d_tape_flag) cudaFree(c->d_tape_flag);
  if (c->d_acc) cudaFree(c->d_acc);
  if (c->batch_graph) cudaGraphExecDestroy(c->batch_graph);
  if (c->h_jobs) cudaFreeHost(c->h_jobs);
  if (c->d_jobs) cudaFree(c->d_jobs);
  if (c->d_batch) cudaFree(c->d_batch);
  if (c->ev_jobs) cudaEventDestroy(c->ev_jobs);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return VVLIC_OK;
}

extern "C" const char* vvlic_last_error(const vvlic_ctx* c) { return c ? c->err.c_str() : "null context"; }

// ------------------------------------------------------------------------------------------
// uploads
// ------------------------------------------------------------------------------------------
static bool valid_dims(const int32_t* n) {
  for (int i = 0; i < 3; ++i)
    if (n[i] < 1 || n[i] > 2048) return false;
  return (size_t)(n[0] + 1) * (n[1] + 1) * (n[2] + 1) < (size_t)1 << 31;
}

static vvlic_status grow(vvlic_ctx* c, void** buf, size_t* cap, size_t bytes) {
  if (*cap >= bytes) return VVLIC_OK;
  if (*buf) cudaFree(*buf);
  *buf = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc(buf, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
  *cap = bytes;
  return VVLIC_OK;
}

static vvlic_status encode_into_volume(vvlic_ctx* c, const void* d_xyz, int dtype, const int n[3],
                                       const float* slice_dist, int storage, cudaStream_t s, int32_t* vol_id) {
  Volume v;
  v.n[0] = n[0];
  v.n[1] = n[1];
  v.n[2] = n[2];
  v.storage = storage;
  v.geom = make_geometry(n, slice_dist);
  const size_t count = (size_t)n[0] * n[1] * n[2];
  v.texel_bytes = count * texel_bytes(storage);
  cudaError_t e = cudaMalloc(&v.d_texels, v.texel_bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "field allocation");
  e = launch_encode_field(d_xyz, dtype, n, storage, v.d_texels, c->d_scratch_word, s);
  if (e != cudaSuccess) {
    free_volume(v);
    return cuda_fail(c, e, "field encoding");
  }
  const int id = c->next_vol_id++;
  c->vols[id] = v;
  *vol_id = id;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_upload_field(vvlic_ctx* c, const void* xyz, int32_t dtype, int32_t nx, int32_t ny,
                                          int32_t nz, const float* slice_dist, int32_t storage, int32_t* vol_id) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  const int n[3] = {nx, ny, nz};
  if (!xyz || !vol_id || !valid_dims(n)) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field: bad arguments");
  if (dtype != VVLIC_DTYPE_FLOAT32 && dtype != VVLIC_DTYPE_UINT8)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field: dtype %d", dtype);
  if (storage < VVLIC_STORAGE_F32 || storage > VVLIC_STORAGE_UNORM8)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field: storage %d", storage);
  if (slice_dist)
    for (int i = 0; i < 3; ++i)
      if (!(slice_dist[i] > 0.0f)) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field: slice distance");
  DeviceGuard g(c->device);
  const size_t bytes = (size_t)nx * ny * nz * 3 * (dtype == VVLIC_DTYPE_FLOAT32 ? 4 : 1);
  vvlic_status st = grow(c, &c->d_upload, &c->upload_cap, bytes);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(c->d_upload, xyz, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "upload_field copy");
  st = encode_into_volume(c, c->d_upload, dtype, n, slice_dist, storage, c->stream, vol_id);
  if (st) return st;
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "upload_field");
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_upload_field_interp(vvlic_ctx* c, const void* xyz0, const void* xyz1, int32_t dtype,
                                                 int32_t nx, int32_t ny, int32_t nz, const float* slice_dist,
                                                 int32_t storage, int32_t interp_index, int32_t interp_size,
                                                 int32_t* vol_id) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  const int n[3] = {nx, ny, nz};
  if (!xyz0 || !xyz1 || !vol_id || !valid_dims(n) || interp_size < 1 || interp_index < 0 ||
      interp_index >= interp_size)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field_interp: bad arguments");
  if (slice_dist)
    for (int i = 0; i < 3; ++i)
      if (!(slice_dist[i] > 0.0f)) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field_interp: slice distance");
  if (dtype != VVLIC_DTYPE_FLOAT32 && dtype != VVLIC_DTYPE_UINT8)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field_interp: dtype %d", dtype);
  if (storage < VVLIC_STORAGE_F32 || storage > VVLIC_STORAGE_UNORM8)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field_interp: storage %d", storage);
  DeviceGuard g(c->device);
  const size_t bytes = (size_t)nx * ny * nz * 3 * (dtype == VVLIC_DTYPE_FLOAT32 ? 4 : 1);
  const size_t slot = (bytes + 255) & ~(size_t)255;
  vvlic_status st = grow(c, &c->d_upload, &c->upload_cap, 3 * slot);
  if (st) return st;
  char* base = (char*)c->d_upload;
  cudaError_t e = cudaMemcpyAsync(base, xyz0, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(base + slot, xyz1, bytes, cudaMemcpyHostToDevice, c->stream);
  // (float)interpIndex / InterpSize, as the reference computes it
  const float t = (float)interp_index / (float)interp_size;
  if (e == cudaSuccess) e = launch_interp_field(base, base + slot, dtype, n, t, base + 2 * slot, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "upload_field_interp");
  st = encode_into_volume(c, base + 2 * slot, dtype, n, slice_dist, storage, c->stream, vol_id);
  if (st) return st;
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "upload_field_interp");
  return VVLIC_OK;
}

// Re-encodes the raw vectors at d_xyz into the existing volume and rewrites its cell and texture
// copies, on the context stream; the caller has waited for renders that read the old texels.
static vvlic_status reencode_volume(vvlic_ctx* c, int32_t vol_id, Volume& v, const void* d_xyz, int dtype) {
  cudaError_t e = launch_encode_field(d_xyz, dtype, v.n, v.storage, v.d_texels, c->d_scratch_word, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "field encoding");
  vvlic_status st = refresh_volume_layouts(c, v, c->stream);
  if (st) return st;
  v.licvol_valid = false;  // the precomputed LIC volume belongs to the previous field
  if (c->tape_vol == vol_id) c->tape_valid = false;
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "field update");
  return VVLIC_OK;
}

static vvlic_status update_target(vvlic_ctx* c, int32_t vol_id, int32_t dtype, int32_t nx, int32_t ny, int32_t nz,
                                  const char* what, Volume** v) {
  auto it = c->vols.find(vol_id);
  if (it == c->vols.end()) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "%s: unknown volume %d", what, vol_id);
  if (it->second.n[0] != nx || it->second.n[1] != ny || it->second.n[2] != nz)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "%s: %dx%dx%d does not match the volume's %dx%dx%d", what, nx, ny, nz,
                it->second.n[0], it->second.n[1], it->second.n[2]);
  if (dtype != VVLIC_DTYPE_FLOAT32 && dtype != VVLIC_DTYPE_UINT8)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "%s: dtype %d", what, dtype);
  *v = &it->second;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_update_field(vvlic_ctx* c, int32_t vol_id, const void* xyz, int32_t dtype, int32_t nx,
                                          int32_t ny, int32_t nz) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!xyz) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "update_field: null data");
  Volume* v = nullptr;
  vvlic_status st = update_target(c, vol_id, dtype, nx, ny, nz, "update_field", &v);
  if (st) return st;
  DeviceGuard g(c->device);
  const size_t bytes = (size_t)nx * ny * nz * 3 * (dtype == VVLIC_DTYPE_FLOAT32 ? 4 : 1);
  if ((st = grow(c, &c->d_upload, &c->upload_cap, bytes))) return st;
  // renders launched on any stream may still read the volume's texels
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_upload, xyz, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "update_field copy");
  return reencode_volume(c, vol_id, *v, c->d_upload, dtype);
}

extern "C" vvlic_status vvlic_update_field_interp(vvlic_ctx* c, int32_t vol_id, const void* xyz0, const void* xyz1,
                                                 int32_t dtype, int32_t nx, int32_t ny, int32_t nz,
                                                 int32_t interp_index, int32_t interp_size) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!xyz0 || !xyz1 || interp_size < 1 || interp_index < 0 || interp_index >= interp_size)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "update_field_interp: bad arguments");
  Volume* v = nullptr;
  vvlic_status st = update_target(c, vol_id, dtype, nx, ny, nz, "update_field_interp", &v);
  if (st) return st;
  DeviceGuard g(c->device);
  const int n[3] = {nx, ny, nz};
  const size_t bytes = (size_t)nx * ny * nz * 3 * (dtype == VVLIC_DTYPE_FLOAT32 ? 4 : 1);
  const size_t slot = (bytes + 255) & ~(size_t)255;
  if ((st = grow(c, &c->d_upload, &c->upload_cap, 3 * slot))) return st;
  char* base = (char*)c->d_upload;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpyAsync(base, xyz0, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(base + slot, xyz1, bytes, cudaMemcpyHostToDevice, c->stream);
  // (float)interpIndex / InterpSize, as the reference computes it
  const float t = (float)interp_index / (float)interp_size;
  if (e == cudaSuccess) e = launch_interp_field(base, base + slot, dtype, n, t, base + 2 * slot, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "update_field_interp");
  return reencode_volume(c, vol_id, *v, base + 2 * slot, dtype);
}

// Copy stream and events of the stream-ordered updates, created on first use.
static vvlic_status ensure_async(vvlic_ctx* c) {
  if (c->copy_stream) return VVLIC_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
  for (cudaEvent_t* ev : {&c->ev_field_copied, &c->ev_field_used, &c->ev_noise_copied, &c->ev_noise_used})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return cuda_fail(c, e, "asynchronous update set-up");
  return VVLIC_OK;
}

// A staging buffer of at least `bytes`; growing it first waits for the device (a copy or its
// consumer may still use the old one).
static vvlic_status grow_stage(vvlic_ctx* c, void** buf, size_t* cap, size_t bytes) {
  if (*cap >= bytes) return VVLIC_OK;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(c, e, "staging");
  return grow(c, buf, cap, bytes);
}

extern "C" vvlic_status vvlic_update_field_async(vvlic_ctx* c, int32_t vol_id, const void* xyz, int32_t dtype,
                                                int32_t nx, int32_t ny, int32_t nz, void* stream) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!xyz) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "update_field_async: null data");
  Volume* v = nullptr;
  vvlic_status st = update_target(c, vol_id, dtype, nx, ny, nz, "update_field_async", &v);
  if (st) return st;
  DeviceGuard g(c->device);
  if ((st = ensure_async(c))) return st;
  const size_t bytes = (size_t)nx * ny * nz * 3 * (dtype == VVLIC_DTYPE_FLOAT32 ? 4 : 1);
  if ((st = grow_stage(c, &c->d_field_stage, &c->field_stage_cap, bytes))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  // the copy overwrites the stage once the previous update's encoding has read it; the
  // encoding on `stream` follows the copy and every render enqueued on `stream` before it
  cudaError_t e = cudaStreamWaitEvent(c->copy_stream, c->ev_field_used, 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_field_stage, xyz, bytes, cudaMemcpyHostToDevice, c->copy_stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_field_copied, c->copy_stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_field_copied, 0);
  if (e == cudaSuccess) e = launch_encode_field(c->d_field_stage, dtype, v->n, v->storage, v->d_texels, c->d_scratch_word, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "update_field_async");
  if ((st = refresh_volume_layouts(c, *v, s))) return st;
  e = cudaEventRecord(c->ev_field_used, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "update_field_async");
  v->licvol_valid = false;
  if (c->tape_vol == vol_id) c->tape_valid = false;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_update_field_device(vvlic_ctx* c, int32_t vol_id, const float* d_xyz, int32_t nx,
                                                 int32_t ny, int32_t nz, void* stream) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!d_xyz) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "update_field_device: null data");
  Volume* v = nullptr;
  vvlic_status st = update_target(c, vol_id, VVLIC_DTYPE_FLOAT32, nx, ny, nz, "update_field_device", &v);
  if (st) return st;
  DeviceGuard g(c->device);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = launch_encode_field(d_xyz, VVLIC_DTYPE_FLOAT32, v->n, v->storage, v->d_texels, c->d_scratch_word, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "update_field_device");
  if ((st = refresh_volume_layouts(c, *v, s))) return st;
  v->licvol_valid = false;
  if (c->tape_vol == vol_id) c->tape_valid = false;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_upload_field_device(vvlic_ctx* c, const float* d_xyz, int32_t nx, int32_t ny, int32_t nz,
                                                 const float* slice_dist, int32_t storage, void* stream,
                                                 int32_t* vol_id) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  const int n[3] = {nx, ny, nz};
  if (!d_xyz || !vol_id || !valid_dims(n)) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field_device: bad arguments");
  if (storage < VVLIC_STORAGE_F32 || storage > VVLIC_STORAGE_UNORM8)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field_device: storage %d", storage);
  if (slice_dist)
    for (int i = 0; i < 3; ++i)
      if (!(slice_dist[i] > 0.0f)) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_field_device: slice distance");
  DeviceGuard g(c->device);
  return encode_into_volume(c, d_xyz, VVLIC_DTYPE_FLOAT32, n, slice_dist, storage, (cudaStream_t)stream, vol_id);
}

extern "C" vvlic_status vvlic_free_volume(vvlic_ctx* c, int32_t vol_id) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  auto it = c->vols.find(vol_id);
  if (it == c->vols.end()) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "free_volume: unknown volume %d", vol_id);
  DeviceGuard g(c->device);
  cudaDeviceSynchronize();  // renders in flight on any stream may read the volume
  free_volume(it->second);
  c->vols.erase(it);
  if (c->tape_vol == vol_id) c->tape_valid = false;  // the tape points at the freed buffers
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_volume_bytes(const vvlic_ctx* c, int32_t vol_id, uint64_t* bytes) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  auto it = c->vols.find(vol_id);
  if (it == c->vols.end() || !bytes) return VVLIC_ERR_INVALID_ARGUMENT;
  *bytes = it->second.texel_bytes + it->second.cell_bytes + it->second.array_bytes;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_noise_gradients_device(const uint8_t* d_noise, int32_t mx, int32_t my, int32_t mz,
                                                    int32_t mode, const float* slice_dist, uint8_t* d_rgba,
                                                    void* stream) {
  const int m[3] = {mx, my, mz};
  if (!d_noise || !d_rgba || !valid_dims(m)) return VVLIC_ERR_INVALID_ARGUMENT;
  if (mode != VVLIC_NOISE_GRAD_SOBEL && mode != VVLIC_NOISE_GRAD_CENTRAL) return VVLIC_ERR_INVALID_ARGUMENT;
  // the one-sided border differences read the neighbour at +1: every axis needs two voxels
  if (mx < 2 || my < 2 || mz < 2) return VVLIC_ERR_INVALID_ARGUMENT;
  float sd[3] = {1.f, 1.f, 1.f};
  if (slice_dist)
    for (int i = 0; i < 3; ++i) sd[i] = slice_dist[i];
  float w27[27];
  noise_filter_weights(w27);
  cudaStream_t s = (cudaStream_t)stream;
  float* d_grad = nullptr;
  const size_t bytes = (size_t)mx * my * mz * kNoiseGradBytes;
  cudaError_t e = cudaMallocAsync((void**)&d_grad, bytes, s);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? VVLIC_ERR_OUT_OF_MEMORY : VVLIC_ERR_CUDA;
  e = launch_noise_gradients(d_noise, m, mode, sd, d_grad, d_rgba, w27, s);
  cudaError_t e2 = cudaFreeAsync(d_grad, s);
  if (e != cudaSuccess || e2 != cudaSuccess) return VVLIC_ERR_CUDA;
  return VVLIC_OK;
}

// Upload-buffer layout for noise gradients: the noise bytes, then (256-byte aligned) the raw
// float gradients (kNoiseGradBytes per voxel).
static size_t noise_grad_offset(size_t count) { return (count + 255) & ~(size_t)255; }
static size_t noise_staging_bytes(size_t count) { return noise_grad_offset(count) + count * kNoiseGradBytes; }

// Noise gradients (computeGradients + filterGradients + quantizeGradients + pack) of the noise
// bytes staged at the start of the context's upload buffer (noise_staging_bytes of capacity),
// into d_rgba.
static vvlic_status noise_gradients_staged(vvlic_ctx* c, const int m[3], int mode, uint8_t* d_rgba) {
  const size_t count = (size_t)m[0] * m[1] * m[2];
  const size_t off = noise_grad_offset(count);
  const float sd[3] = {1.f, 1.f, 1.f};
  float w27[27];
  noise_filter_weights(w27);
  cudaError_t e = launch_noise_gradients((const uint8_t*)c->d_upload, m, mode, sd,
                                         (float*)((char*)c->d_upload + off), d_rgba, w27, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise gradients");
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_upload_noise(vvlic_ctx* c, const uint8_t* noise, int32_t mx, int32_t my, int32_t mz,
                                          int32_t mode) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  const int m[3] = {mx, my, mz};
  if (!noise || !valid_dims(m)) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_noise: bad arguments");
  if (mode < VVLIC_NOISE_SCALAR || mode > VVLIC_NOISE_GRAD_CENTRAL)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_noise: mode %d", mode);
  if (mode != VVLIC_NOISE_SCALAR && (mx < 2 || my < 2 || mz < 2))
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_noise: gradients need at least 2 voxels per axis");
  DeviceGuard g(c->device);
  NoiseTex& n = c->noise;
  const size_t count = (size_t)mx * my * mz;
  const int ch = mode == VVLIC_NOISE_SCALAR ? 1 : 4;
  c->tape_valid = false;  // a recorded tape read the previous noise
  if (mode != VVLIC_NOISE_SCALAR) {
    vvlic_status st = grow(c, &c->d_upload, &c->upload_cap, noise_staging_bytes(count));
    if (st) return st;
  }
  // Same extent and layout: rewrite the texels and the cell / texture copies in place once the
  // renders already launched on any stream (which read the previous noise) have finished.
  const bool in_place = n.d_texels && n.m[0] == mx && n.m[1] == my && n.m[2] == mz && n.ch == ch;
  cudaError_t e = cudaSuccess;
  if (in_place) {
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(c, e, "upload_noise");
  } else {
    // the texture object and texels are destroyed below: wait for renders in flight on any
    // stream, as the in-place path does
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(c, e, "upload_noise");
    free_noise(n);
    e = cudaMalloc(&n.d_texels, count * ch);
    if (e != cudaSuccess) return cuda_fail(c, e, "noise allocation");
    n.m[0] = mx;
    n.m[1] = my;
    n.m[2] = mz;
    n.ch = ch;
  }
  n.mode = mode;
  if (mode == VVLIC_NOISE_SCALAR) {
    e = cudaMemcpyAsync(n.d_texels, noise, count, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "noise copy");
  } else {
    e = cudaMemcpyAsync(c->d_upload, noise, count, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "noise copy");
    vvlic_status st = noise_gradients_staged(c, m, mode, n.d_texels);
    if (st) return st;
  }
  if (in_place) {
    vvlic_status st = refresh_noise_layouts(c, n, c->stream);
    if (st) return st;
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "upload_noise");
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_upload_noise_rgba(vvlic_ctx* c, const uint8_t* rgba, int32_t mx, int32_t my, int32_t mz,
                                               int32_t mode) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  const int m[3] = {mx, my, mz};
  if (!rgba || !valid_dims(m)) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_noise_rgba: bad arguments");
  if (mode != VVLIC_NOISE_GRAD_SOBEL && mode != VVLIC_NOISE_GRAD_CENTRAL)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_noise_rgba: mode %d is not a gradient mode", mode);
  DeviceGuard g(c->device);
  cudaError_t e = cudaDeviceSynchronize();  // renders in flight on any stream read the old noise
  if (e != cudaSuccess) return cuda_fail(c, e, "upload_noise_rgba");
  free_noise(c->noise);
  c->tape_valid = false;
  NoiseTex& n = c->noise;
  const size_t bytes = (size_t)mx * my * mz * 4;
  n.m[0] = mx;
  n.m[1] = my;
  n.m[2] = mz;
  n.ch = 4;
  n.mode = mode;
  e = cudaMalloc(&n.d_texels, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "noise allocation");
  e = cudaMemcpyAsync(n.d_texels, rgba, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "upload_noise_rgba");
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_upload_noise_async(vvlic_ctx* c, const uint8_t* noise, int32_t mx, int32_t my,
                                                int32_t mz, int32_t mode, void* stream) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  const int m[3] = {mx, my, mz};
  if (!noise || !valid_dims(m)) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_noise_async: bad arguments");
  if (mode < VVLIC_NOISE_SCALAR || mode > VVLIC_NOISE_GRAD_CENTRAL)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_noise_async: mode %d", mode);
  NoiseTex& n = c->noise;
  const int ch = mode == VVLIC_NOISE_SCALAR ? 1 : 4;
  if (!n.d_texels || n.m[0] != mx || n.m[1] != my || n.m[2] != mz || n.ch != ch)
    return fail(c, VVLIC_ERR_NOT_READY,
                "upload_noise_async: rewrites a noise of the same extent and channels in place; upload the first "
                "one with vvlic_upload_noise");
  DeviceGuard g(c->device);
  vvlic_status st = ensure_async(c);
  if (st) return st;
  const size_t count = (size_t)mx * my * mz;
  if ((st = grow_stage(c, &c->d_noise_stage, &c->noise_stage_cap,
                       mode == VVLIC_NOISE_SCALAR ? count : noise_staging_bytes(count))))
    return st;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaStreamWaitEvent(c->copy_stream, c->ev_noise_used, 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_noise_stage, noise, count, cudaMemcpyHostToDevice, c->copy_stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_noise_copied, c->copy_stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_noise_copied, 0);
  if (e == cudaSuccess) {
    if (mode == VVLIC_NOISE_SCALAR) {
      e = cudaMemcpyAsync(n.d_texels, c->d_noise_stage, count, cudaMemcpyDeviceToDevice, s);
    } else {
      const float sd[3] = {1.f, 1.f, 1.f};
      float w27[27];
      noise_filter_weights(w27);
      e = launch_noise_gradients((const uint8_t*)c->d_noise_stage, m, mode, sd,
                                 (float*)((char*)c->d_noise_stage + noise_grad_offset(count)), n.d_texels, w27, s);
    }
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "upload_noise_async");
  if ((st = refresh_noise_layouts(c, n, s))) return st;
  e = cudaEventRecord(c->ev_noise_used, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "upload_noise_async");
  n.mode = mode;
  c->tape_valid = false;  // a recorded tape read the previous noise
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_upload_scalar(vvlic_ctx* c, const float* scalar, int32_t nx, int32_t ny, int32_t nz) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  const int n[3] = {nx, ny, nz};
  if (!scalar || !valid_dims(n)) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "upload_scalar: bad arguments");
  DeviceGuard g(c->device);
  if (c->d_scalar) cudaFree(c->d_scalar);
  c->d_scalar = nullptr;
  c->tape_valid = false;
  const size_t bytes = (size_t)nx * ny * nz * sizeof(float);
  cudaError_t e = cudaMalloc(&c->d_scalar, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "scalar allocation");
  e = cudaMemcpy(c->d_scalar, scalar, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(c, e, "scalar copy");
  for (int i = 0; i < 3; ++i) c->sn[i] = n[i];
  return VVLIC_OK;
}

namespace vvlic {
// The device tables (TF, line-illumination tables) are read by kernels still in flight on the
// caller's streams.  An update is ordered after the context's last launch (every launch records
// ev1 on its stream), so it applies to later renders only, as a GL state change does.
cudaError_t after_launches(vvlic_ctx* c) { return cudaStreamWaitEvent(c->stream, c->ev1, 0); }
}  // namespace vvlic

extern "C" vvlic_status vvlic_set_tf(vvlic_ctx* c, const float* rgba, const float* opacity) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (rgba) std::memcpy(c->tf, rgba, sizeof(float) * 4 * VVLIC_TF_ENTRIES);
  if (opacity) std::memcpy(c->tf + 4 * VVLIC_TF_ENTRIES, opacity, sizeof(float) * VVLIC_TF_ENTRIES);
  for (int i = 0; i < 5 * VVLIC_TF_ENTRIES; ++i)
    if (!std::isfinite(c->tf[i])) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_tf: non-finite entry %d", i);
  DeviceGuard g(c->device);
  cudaError_t e = after_launches(c);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->d_tf, c->tf, sizeof(float) * 5 * VVLIC_TF_ENTRIES, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "set_tf");
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_get_tf(const vvlic_ctx* c, float* rgba, float* opacity) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (rgba) std::memcpy(rgba, c->tf, sizeof(float) * 4 * VVLIC_TF_ENTRIES);
  if (opacity) std::memcpy(opacity, c->tf + 4 * VVLIC_TF_ENTRIES, sizeof(float) * VVLIC_TF_ENTRIES);
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_set_filter_table(vvlic_ctx* c, const uint8_t* table, int32_t width, int32_t clamp_mode) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!table || width < 1 || width > 1024 || (clamp_mode != VVLIC_KERNEL_CLAMP_BORDER && clamp_mode != VVLIC_KERNEL_CLAMP_EDGE))
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_filter_table: bad arguments");
  // LICFilter::loadData centres the table in the next power of two (dataset.cpp:1446-1458)
  const int W = next_pow2(width), shift = (W - width) / 2;
  std::memset(c->filter, 0, sizeof c->filter);
  std::memcpy(c->filter + shift, table, width);
  bool box = true;
  for (int i = 0; i < W; ++i) box = box && c->filter[i] == 255;
  unsigned sum = 0;
  for (int i = 0; i < W; ++i) sum += c->filter[i];
  if (sum == 0) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_filter_table: all-zero filter");
  c->filter_width = W;
  c->filter_clamp = clamp_mode;
  c->filter_is_box = box;
  c->taps_override = false;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_set_filter_taps(vvlic_ctx* c, const float* taps, int32_t lb, int32_t lf,
                                             float inv_filter_area) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!taps) {
    c->taps_override = false;
    return VVLIC_OK;
  }
  if (lb < 0 || lf < 0 || lb > VVLIC_MAX_STEPS || lf > VVLIC_MAX_STEPS || lb + lf == 0 || !std::isfinite(inv_filter_area))
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_filter_taps: bad arguments");
  for (int i = 0; i < lb + lf + 1; ++i) {
    if (!std::isfinite(taps[i])) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_filter_taps: non-finite tap");
    c->taps[i] = taps[i];
  }
  c->taps_lb = lb;
  c->taps_lf = lf;
  c->taps_inv_area = inv_filter_area;
  c->taps_override = true;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_get_filter_taps(const vvlic_ctx* c, float* taps, int32_t capacity, float* inv_area) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  int lb, lf;
  effective_steps(c->params, &lb, &lf);
  if (!taps || !inv_area || capacity < lb + lf + 1) return VVLIC_ERR_INVALID_ARGUMENT;
  return derive_taps(c, lb, lf, taps, inv_area);
}

static vvlic_status check_params(vvlic_ctx* c, const vvlic_params& p) {
  if (!(p.step_size_vol >= 1e-5f) || !std::isfinite(p.step_size_vol))
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: step_size_vol must be >= 1e-5");
  if (!std::isfinite(p.step_size_lic) || !std::isfinite(p.gradient_scale) || !std::isfinite(p.illum_scale) ||
      !std::isfinite(p.freq_scale) || !std::isfinite(p.eye_dist_factor) || !std::isfinite(p.alpha_threshold))
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: non-finite value");
  if (p.steps_forward < 0 || p.steps_backward < 0 || p.steps_forward > VVLIC_MAX_STEPS ||
      p.steps_backward > VVLIC_MAX_STEPS || p.steps_forward + p.steps_backward == 0)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: steps must be in [0, %d] and not both 0", VVLIC_MAX_STEPS);
  // two nested loops of num_iterations bound every ray (lic3d_fragment.glsl:38-40)
  if (p.num_iterations < 0 || p.num_iterations > 1024)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: num_iterations must be in [0, 1024]");
  if (p.integrator < VVLIC_EULER || p.integrator > VVLIC_RK4)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: integrator %d", p.integrator);
  if (p.illum < VVLIC_ILLUM_NONE || p.illum > VVLIC_ILLUM_MALLO)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: illum %d", p.illum);
  if (p.tf_index != VVLIC_TF_INDEX_DIR_Z && p.tf_index != VVLIC_TF_INDEX_MAGNITUDE)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: tf_index %d", p.tf_index);
  if (p.sampler < VVLIC_SAMPLER_GATHER || p.sampler > VVLIC_SAMPLER_BRICK)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: sampler %d", p.sampler);
  if (p.schedule != VVLIC_SCHEDULE_QUEUE && p.schedule != VVLIC_SCHEDULE_STATIC)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: schedule %d", p.schedule);
  if (p.technique < VVLIC_TECHNIQUE_VOLUME || p.technique > VVLIC_TECHNIQUE_LICVOLUME)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "params: technique %d", p.technique);
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_set_params(vvlic_ctx* c, const vvlic_params* p) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!p) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_params: null");
  vvlic_status st = check_params(c, *p);
  if (st) return st;
  c->params = *p;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_get_params(const vvlic_ctx* c, vvlic_params* p) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!p) return VVLIC_ERR_INVALID_ARGUMENT;
  *p = c->params;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_set_view(vvlic_ctx* c, const vvlic_view* v) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!v) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_view: null");
  if (v->projection != VVLIC_PERSPECTIVE && v->projection != VVLIC_ORTHOGRAPHIC)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_view: projection %d", v->projection);
  if (v->projection == VVLIC_PERSPECTIVE && !(v->fovy_deg > 0.0f && v->fovy_deg < 180.0f))
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_view: fovy");
  if (v->projection == VVLIC_ORTHOGRAPHIC &&
      !(std::fabs(v->ortho_dir[0]) + std::fabs(v->ortho_dir[1]) + std::fabs(v->ortho_dir[2]) > 0.0f))
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "set_view: zero ortho direction");
  c->view = *v;
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_view_rays(const vvlic_ctx* c, int32_t vol_id, int32_t w, int32_t h, double* coeffs) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  auto it = c->vols.find(vol_id);
  if (it == c->vols.end() || !coeffs || w < 1 || h < 1) return VVLIC_ERR_INVALID_ARGUMENT;
  derive_rays(c->view, it->second.geom, w, h, coeffs);
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_composite_background(float* rgba, int32_t w, int32_t h, const float* bg) {
  if (!rgba || w < 1 || h < 1) return VVLIC_ERR_INVALID_ARGUMENT;
  const float white[4] = {1.f, 1.f, 1.f, 1.f};
  const float* b = bg ? bg : white;
  for (size_t i = 0; i < (size_t)w * h; ++i) {
    float* d = rgba + 4 * i;
    const float om = 1.0f - d[3];
    for (int ch = 0; ch < 4; ++ch) d[ch] = std::min(std::max(om * b[ch] + d[ch], 0.0f), 1.0f);
  }
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_download_field(vvlic_ctx* c, int32_t vol_id, void* out, uint64_t capacity) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  auto it = c->vols.find(vol_id);
  if (it == c->vols.end()) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "download_field: unknown volume %d", vol_id);
  if (!out || capacity < it->second.texel_bytes)
    return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "download_field: need %zu bytes", it->second.texel_bytes);
  DeviceGuard g(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(out, it->second.d_texels, it->second.texel_bytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(c, e, "download_field");
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_download_noise(vvlic_ctx* c, void* out, uint64_t capacity) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!c->noise.d_texels) return fail(c, VVLIC_ERR_NOT_READY, "download_noise: no noise uploaded");
  const size_t bytes = (size_t)c->noise.m[0] * c->noise.m[1] * c->noise.m[2] * c->noise.ch;
  if (!out || capacity < bytes) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "download_noise: need %zu bytes", bytes);
  DeviceGuard g(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(out, c->noise.d_texels, bytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(c, e, "download_noise");
  return VVLIC_OK;
}
