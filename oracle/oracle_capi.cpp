/*
 * ORACLE — test infrastructure, not product code.
 *
 * C entry points over vvlic_oracle.hpp for ctypes (tests/, the smoke check, bench.py's CPU
 * baseline).  Built into oracle/_build/libvvoracle.so by oracle/Makefile.
 */
#include "vvlic_oracle.hpp"

extern "C" {

/* Oracle inputs as plain pointers; mirrors vvo::Inputs plus the filter table from which the
 * taps are derived (taps == NULL) or explicit taps. */
typedef struct vvo_inputs {
  const float* field;
  int32_t n[3];
  float slice_dist[3];
  const uint8_t* noise;
  int32_t m[3];
  int32_t noise_channels;
  const float* scalar;
  int32_t sn[3];
  const float* tf_rgba;
  const float* tf_opac;
  const uint8_t* filter_table; /* used when taps == NULL */
  int32_t filter_width;
  int32_t filter_clamp;
  int32_t filter_is_box;
  const double* taps;          /* explicit taps (L_b+L_f+1) or NULL */
  double inv_filter_area;      /* used with explicit taps */
  const float* licvol;         /* LIC volume for the LICVOLUME technique, or NULL */
  int32_t ln[3];
  const uint8_t* luts;         /* line-illumination tables (vvo_illum_luts) or NULL */
  int32_t lut_w, lut_h;
} vvo_inputs;

int32_t vvo_abi(void) { return 1; }

void vvo_params_default(vvlic_params* p) { vvo::params_default(*p); }
void vvo_view_default(vvlic_view* v) { vvo::view_default(*v); }
void vvo_line_material_default(vvlic_line_material* m) { vvo::line_material_default(*m); }
int32_t vvo_filter_table(int32_t kind, int32_t width, uint8_t* out) { return vvo::filter_table(kind, width, out); }

void vvo_encode_field(const void* xyz, int32_t dtype, const int32_t n[3], float* out_rgba) {
  int nn[3] = {n[0], n[1], n[2]};
  vvo::encode_field(xyz, dtype, nn, out_rgba);
}

void vvo_encode_field_interp(const void* xyz0, const void* xyz1, int32_t dtype, const int32_t n[3], int32_t index,
                             int32_t size, float* out_rgba) {
  int nn[3] = {n[0], n[1], n[2]};
  vvo::encode_field_interp(xyz0, xyz1, (float)index / (float)size, dtype, nn, out_rgba);
}

/* The Zoeckler and Mallo tables for `mat` at w x h: 3 * w * h * 4 bytes. */
void vvo_illum_luts(const vvlic_line_material* mat, int32_t w, int32_t h, uint8_t* out) {
  vvo::illum_luts(*mat, w, h, out);
}

void vvo_round_storage(float* v, uint64_t count, int32_t storage) { vvo::round_storage(v, (size_t)count, storage); }

void vvo_noise_gradients(const uint8_t* noise, const int32_t m[3], int32_t mode, const float* slice_dist,
                         uint8_t* out_rgba) {
  int mm[3] = {m[0], m[1], m[2]};
  vvo::noise_gradients(noise, mm, mode, slice_dist, out_rgba);
}

void vvo_noise_filter_weights(float* w27) { vvo::noise_gradient_filter_weights(w27); }

float vvo_filter_inv_area(const uint8_t* table, int32_t width, int32_t is_box) {
  return vvo::filter_inv_area(table, width, is_box != 0);
}

void vvo_filter_taps(const uint8_t* table, int32_t width, int32_t clamp_mode, int32_t lb, int32_t lf, double* taps) {
  vvo::filter_taps<double>(table, width, clamp_mode, lb, lf, taps);
}

void vvo_view_rays(const vvlic_view* view, const int32_t n[3], const float* slice_dist, int32_t w, int32_t h,
                   double* coeffs) {
  int nn[3] = {n[0], n[1], n[2]};
  vvo::view_rays(*view, nn, slice_dist, w, h, coeffs);
}

void vvo_geometry(const int32_t n[3], const float* slice_dist, double* out15) {
  int nn[3] = {n[0], n[1], n[2]};
  vvo::Geometry g = vvo::geometry(nn, slice_dist);
  for (int i = 0; i < 3; ++i) {
    out15[i] = g.scale[i];
    out15[3 + i] = g.scale_inv[i];
    out15[6 + i] = g.extent[i];
    out15[9 + i] = g.center[i];
    out15[12 + i] = g.tex_max[i];
  }
}

static int effective_steps(const vvlic_params* p, int* lb, int* lf) {
  if (p->low_res) {
    *lb = 15;
    *lf = 15;
  } else {
    *lb = p->steps_backward;
    *lf = p->steps_forward;
  }
  return *lb + *lf + 1;
}

/* Render rows `rows[0..nrows)` (or all rows if rows == NULL) of a w x h image.
 * precision: 64 = double oracle, 32 = float CPU baseline.  threads <= 0: OpenMP default. */
int32_t vvo_render(const vvo_inputs* vi, const vvlic_params* p, const double* ray_coeffs, int32_t w, int32_t h,
                   const int32_t* rows, int32_t nrows, float* out, uint32_t* samples, int32_t precision,
                   int32_t threads, const vvlic_view* view) {
  int lb, lf;
  int ntaps = effective_steps(p, &lb, &lf);
  std::vector<double> taps(ntaps);
  double inv_area;
  if (vi->taps) {
    for (int i = 0; i < ntaps; ++i) taps[i] = vi->taps[i];
    inv_area = vi->inv_filter_area;
  } else {
    if (!vi->filter_table) return -1;
    vvo::filter_taps<double>(vi->filter_table, vi->filter_width, vi->filter_clamp, lb, lf, taps.data());
    inv_area = vvo::filter_inv_area(vi->filter_table, vi->filter_width, vi->filter_is_box != 0);
  }
  vvo::Inputs in;
  in.field = vi->field;
  for (int i = 0; i < 3; ++i) {
    in.n[i] = vi->n[i];
    in.slice_dist[i] = vi->slice_dist[i];
    in.m[i] = vi->m[i];
    in.sn[i] = vi->sn[i];
  }
  in.noise = vi->noise;
  in.noise_channels = vi->noise_channels;
  in.scalar = vi->scalar;
  in.tf_rgba = vi->tf_rgba;
  in.tf_opac = vi->tf_opac;
  in.taps = taps.data();
  in.inv_filter_area = inv_area;
  in.licvol = vi->licvol;
  for (int i = 0; i < 3; ++i) in.ln[i] = vi->ln[i];
  in.luts = vi->luts;
  in.lut_w = vi->lut_w;
  in.lut_h = vi->lut_h;
  if (p->technique == VVLIC_TECHNIQUE_LICVOLUME && !in.licvol) return -3;
  if ((p->illum == VVLIC_ILLUM_ZOECKLER || p->illum == VVLIC_ILLUM_MALLO) && !in.luts) return -5;
  double slicing[5] = {0, 0, 0, 0, 0};
  if (p->technique == VVLIC_TECHNIQUE_SLICING) {
    if (!view) return -4;
    int ns = 0;
    float spacing = p->low_res ? 2.0f * p->step_size_vol : p->step_size_vol;
    vvo::slicing_setup(*view, in.n, in.slice_dist, spacing, slicing, &slicing[3], &ns);
    slicing[4] = ns;
  }
  if (precision == 32)
    vvo::render<float>(in, *p, ray_coeffs, w, h, rows, nrows, out, samples, threads, slicing);
  else
    vvo::render<double>(in, *p, ray_coeffs, w, h, rows, nrows, out, samples, threads, slicing);
  return 0;
}

/* LIC volume (lic3d_volume_fragment.glsl) of ln[0]*ln[1]*ln[2] voxels into out. */
int32_t vvo_lic_volume(const vvo_inputs* vi, const vvlic_params* p, const int32_t ln[3], float* out) {
  int lb, lf;
  int ntaps = effective_steps(p, &lb, &lf);
  std::vector<double> taps(ntaps);
  double inv_area;
  if (vi->taps) {
    for (int i = 0; i < ntaps; ++i) taps[i] = vi->taps[i];
    inv_area = vi->inv_filter_area;
  } else {
    if (!vi->filter_table) return -1;
    vvo::filter_taps<double>(vi->filter_table, vi->filter_width, vi->filter_clamp, lb, lf, taps.data());
    inv_area = vvo::filter_inv_area(vi->filter_table, vi->filter_width, vi->filter_is_box != 0);
  }
  vvo::Inputs in;
  in.field = vi->field;
  for (int i = 0; i < 3; ++i) {
    in.n[i] = vi->n[i];
    in.slice_dist[i] = vi->slice_dist[i];
    in.m[i] = vi->m[i];
    in.sn[i] = vi->sn[i];
  }
  in.noise = vi->noise;
  in.noise_channels = vi->noise_channels;
  in.scalar = vi->scalar;
  in.tf_rgba = vi->tf_rgba;
  in.tf_opac = vi->tf_opac;
  in.taps = taps.data();
  in.inv_filter_area = inv_area;
  in.licvol = nullptr;
  int l[3] = {ln[0], ln[1], ln[2]};
  vvo::lic_volume<double>(in, *p, l, out);
  return 0;
}

/* FP64 adjoint of the unlit render: accumulates dL/dTF (256*4), dL/dopacity (256) and
 * dL/dtaps (L_b+L_f+1) for the image cotangent g_img (h*w*4). */
int32_t vvo_adjoint(const vvo_inputs* vi, const vvlic_params* p, const double* ray_coeffs, int32_t w, int32_t h,
                    const float* g_img, double* d_tf, double* d_opac, double* d_taps, int32_t threads) {
  int lb, lf;
  int ntaps = effective_steps(p, &lb, &lf);
  std::vector<double> taps(ntaps);
  double inv_area;
  if (vi->taps) {
    for (int i = 0; i < ntaps; ++i) taps[i] = vi->taps[i];
    inv_area = vi->inv_filter_area;
  } else {
    if (!vi->filter_table) return -1;
    vvo::filter_taps<double>(vi->filter_table, vi->filter_width, vi->filter_clamp, lb, lf, taps.data());
    inv_area = vvo::filter_inv_area(vi->filter_table, vi->filter_width, vi->filter_is_box != 0);
  }
  vvo::Inputs in;
  in.field = vi->field;
  for (int i = 0; i < 3; ++i) {
    in.n[i] = vi->n[i];
    in.slice_dist[i] = vi->slice_dist[i];
    in.m[i] = vi->m[i];
    in.sn[i] = vi->sn[i];
  }
  in.noise = vi->noise;
  in.noise_channels = vi->noise_channels;
  in.scalar = vi->scalar;
  in.tf_rgba = vi->tf_rgba;
  in.tf_opac = vi->tf_opac;
  in.taps = taps.data();
  in.inv_filter_area = inv_area;
  in.luts = vi->luts;
  in.lut_w = vi->lut_w;
  in.lut_h = vi->lut_h;
  if ((p->illum == VVLIC_ILLUM_ZOECKLER || p->illum == VVLIC_ILLUM_MALLO) && !in.luts) return -5;
  vvo::AdjointOut out{d_tf, d_opac, d_taps};
  vvo::adjoint<double>(in, *p, ray_coeffs, w, h, g_img, out, threads);
  return 0;
}

int32_t vvo_max_threads(void) {
#if defined(_OPENMP)
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
