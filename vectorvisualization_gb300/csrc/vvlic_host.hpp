// Host-side state of a vvlic context (opaque to callers of the C ABI).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <map>
#include <string>

#include "../../include/vvlic.h"
#include "vvlic_device.cuh"

namespace vvlic {

// VolumeData geometry (dataset.h:21-51 fields scale / scaleInv / extent / center).
struct Geometry {
  float slice_dist[3];
  float scale[3], scale_inv[3], extent[3], center[3], tex_max[3];
};

struct Volume {
  int n[3] = {0, 0, 0};
  int storage = VVLIC_STORAGE_F32;
  Geometry geom{};
  void* d_texels = nullptr;       // x-fastest RGBA texels at `storage` precision
  size_t texel_bytes = 0;
  void* d_cells = nullptr;        // corner-packed cells, built on first CELL render
  size_t cell_bytes = 0;
  cudaArray_t array = nullptr;    // texture copy, built on first TEXTURE render
  cudaTextureObject_t tex = 0;
  size_t array_bytes = 0;
  float* d_licvol = nullptr;      // precomputed LIC volume (vvlic_compute_lic_volume)
  int ln[3] = {0, 0, 0};
  bool licvol_valid = false;      // false after a field update until the next precompute
  CUtensorMap brick_map;          // BRICK sampler: TMA map of the texels for bricks of brick_box
  int brick_box[3] = {0, 0, 0};   // (0: no map encoded)
};

struct NoiseTex {
  int m[3] = {0, 0, 0};
  int ch = 0;                     // 1: value, 4: quantised gradient + value
  int mode = VVLIC_NOISE_SCALAR;
  uint8_t* d_texels = nullptr;
  uint8_t* d_cells = nullptr;     // m^3 cells of 8 corners, built on first CELL render
  cudaArray_t array = nullptr;    // texture copy, built on first TEXTURE render
  cudaTextureObject_t tex = 0;
  CUtensorMap brick_map;          // BRICK sampler: TMA map of the texels for bricks of brick_box
  int brick_box[3] = {0, 0, 0};
};

class DeviceGuard {
 public:
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev_);
    if (prev_ != dev) cudaSetDevice(dev);
    dev_ = dev;
  }
  ~DeviceGuard() {
    if (prev_ != dev_) cudaSetDevice(prev_);
  }

 private:
  int prev_ = 0, dev_ = 0;
};

// The 27 smoothing weights of filterGradients (gradient.cpp:393-409: exp(-(i^2+j^2+k^2)/SIGMA2)
// for i, j, k in [-2, 0], normalised by their float sum), computed in float like the reference.
inline void noise_filter_weights(float w[27]) {
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

}  // namespace vvlic

struct vvlic_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::map<int, vvlic::Volume> vols;
  int next_vol_id = 1;
  vvlic::NoiseTex noise;
  float* d_scalar = nullptr;
  int sn[3] = {0, 0, 0};
  float tf[5 * VVLIC_TF_ENTRIES];  // RGBA entries then opacity entries
  float* d_tf = nullptr;
  uint8_t filter[1024];
  int filter_width = 0;
  int filter_clamp = VVLIC_KERNEL_CLAMP_BORDER;
  bool filter_is_box = true;
  bool taps_override = false;
  float taps[vvlic::kMaxTaps];
  int taps_lb = 0, taps_lf = 0;
  float taps_inv_area = 0.5f;
  vvlic_params params;
  vvlic_view view;
  // line-illumination tables: Zoeckler, Mallo diffuse, Mallo specular, lut_w x lut_h RGBA8 each
  vvlic_line_material line_mat;
  void* d_luts = nullptr;
  size_t lut_bytes = 0;
  int lut_w = 0, lut_h = 0;
  bool luts_valid = false;
  unsigned long long* d_counters = nullptr;
  unsigned* d_scratch_word = nullptr;
  void* d_image = nullptr;
  size_t image_cap = 0;
  void* d_upload = nullptr;
  size_t upload_cap = 0;
  // stream-ordered updates (vvlic_update_field_async / vvlic_upload_noise_async): host copies
  // run on copy_stream into their own staging buffers; the caller's stream waits for a copy
  // (ev_*_copied) before consuming it, and the next copy waits until the consumer is done
  // (ev_*_used)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_field_copied = nullptr, ev_field_used = nullptr, ev_noise_copied = nullptr, ev_noise_used = nullptr;
  void* d_field_stage = nullptr;
  size_t field_stage_cap = 0;
  void* d_noise_stage = nullptr;
  size_t noise_stage_cap = 0;
  unsigned* d_sched = nullptr;    // tile order scratch of the queue schedule
  size_t sched_cap = 0;           // in 4-byte words
  int num_sms = 1;
  // adjoint tape of the last recording render
  void* d_tape = nullptr;
  size_t tape_cap = 0;
  unsigned long long* d_tape_flag = nullptr;  // overflow count of the recording render
  bool tape_flag_pending = false;  // the next get_stats reads d_tape_flag into check_flags
  long long* d_acc = nullptr;                 // fixed-point gradient accumulators
  bool tape_valid = false;
  int tape_vol = 0, tape_w = 0, tape_h = 0, tape_storage = 0, tape_sampler = 0, tape_integ = 0, tape_illum = 0;
  vvlic::RenderArgs tape_args;
  // batches
  vvlic::RenderArgs* h_jobs = nullptr;  // pinned staging of the job table
  size_t h_jobs_cap = 0;
  vvlic::RenderArgs* d_jobs = nullptr;
  size_t d_jobs_cap = 0;
  unsigned* d_batch = nullptr;          // job tile starts + order scratch
  size_t batch_cap = 0;                 // words
  cudaEvent_t ev_jobs = nullptr;        // the staging buffer may be rewritten after this
  cudaGraphExec_t batch_graph = nullptr;
  uint64_t batch_key[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int batch_tile_w = 8;                 // warp tile width (autotuned)
  int batch_sampler_override = -1;      // sampler chosen by the autotuner (-1: the jobs')
  bool last_was_batch = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool stats_pending = false;
  uint64_t stats_steps_per_sample = 0;
  vvlic_stats stats{};
  std::string err;
};

namespace vvlic {
vvlic_status fail(vvlic_ctx* c, vvlic_status s, const char* fmt, ...);
// Builds (first use, or after a material change) and uploads the line-illumination tables.
vvlic_status ensure_illum_luts(vvlic_ctx* c);
// Orders the context stream after the context's last launch (device-table updates).
cudaError_t after_launches(vvlic_ctx* c);
vvlic_status cuda_fail(vvlic_ctx* c, cudaError_t e, const char* what);
// Rewrite the cell and texture copies that exist from the texels, in place (render.cu).
vvlic_status refresh_volume_layouts(vvlic_ctx* c, Volume& v, cudaStream_t s);
vvlic_status refresh_noise_layouts(vvlic_ctx* c, NoiseTex& n, cudaStream_t s);
Geometry make_geometry(const int n[3], const float* slice_dist);
vvlic_status derive_taps(const vvlic_ctx* c, int lb, int lf, float* taps, float* inv_area);
void derive_taps_from_table(const uint8_t* t, int W, int clamp, bool is_box, int lb, int lf, float* taps,
                            float* inv_area);
int centre_filter_table(const uint8_t* table, int width, uint8_t* out1024, bool* is_box);
// Argument block of one render job.  `params`/`view` default to the context's; `filter` (a
// centred 1024-entry table of width `fw`), when given, replaces the context's filter.
struct JobFilter {
  const uint8_t* table = nullptr;
  int width = 0, clamp = 0;
  bool is_box = false;
};
vvlic_status build_render_args_ex(vvlic_ctx* c, Volume& v, int W, int H, cudaStream_t s, const vvlic_params& p,
                                  const vvlic_view& view, const JobFilter* filter, RenderArgs& a);
void derive_rays(const vvlic_view& v, const Geometry& g, int W, int H, double* coeffs);
void derive_slicing(const vvlic_view& v, const Geometry& g, float spacing, float vdir[3], float* depth, int* n);
}  // namespace vvlic
