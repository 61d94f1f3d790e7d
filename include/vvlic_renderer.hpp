/*
 * vvlic_renderer.hpp — header-only C++ host interface over the C ABI of vvlic.h, with the names
 * and argument meaning of the reference's Renderer (renderer.h:28-125), LICParams
 * (types.h:91-109) and GLSLShader define injection (GLSLShader.cpp:120-136), so code written
 * against the reference's renderer ports by changing types, not logic.
 *
 * Differences: textures are uploaded from host arrays (the reference passes GL texture
 * handles created by VectorDataSet / NoiseDataSet / TransferEdit / LICFilter), render() writes
 * an RGBA float image instead of the GL framebuffer, and failures throw vvlic::Error (the
 * reference prints and continues).
 */
#ifndef VVLIC_RENDERER_HPP_
#define VVLIC_RENDERER_HPP_

#include <cstring>
#include <stdexcept>
#include <string>

#include "vvlic.h"

namespace vvlic {

/* types.h:91-109 */
struct LICParams {
  float stepSizeVol = 1.0f / 128.0f;
  float gradientScale = 30.0f;
  float illumScale = 1.0f;
  float freqScale = 1.0f;
  int numIterations = 255;
  int stepsForward = 32;
  int stepsBackward = 32;
  float stepSizeLIC = 0.01f;
};

/* types.h:63-72: the render techniques (VOLIC_VOLUMEANI is never rendered by the reference) */
enum RenderTechnique { VOLIC_VOLUME = 0, VOLIC_RAYCAST = 1, VOLIC_SLICING = 2, VOLIC_LICVOLUME = 3 };

class Error : public std::runtime_error {
 public:
  Error(vvlic_status s, const std::string& what) : std::runtime_error(what), status(s) {}
  vvlic_status status;
};

class Renderer {
 public:
  explicit Renderer(int device = 0) {
    check(vvlic_create(&ctx_, device), "vvlic_create");
    vvlic_params_default(&params_);
    vvlic_view_default(&view_);
  }
  ~Renderer() {
    if (ctx_) vvlic_destroy(ctx_);
  }
  Renderer(const Renderer&) = delete;
  Renderer& operator=(const Renderer&) = delete;

  /* VectorDataSet::loadData + createTextureIterp + Renderer::setDataTex: xyz is FLOAT3 raw data,
   * x fastest.  Returns the volume id used by render(); the last uploaded volume is current. */
  int setDataTex(const float* xyz, int nx, int ny, int nz, const float* sliceDist = nullptr,
                 int storage = VVLIC_STORAGE_F16) {
    int32_t id = 0;
    check(vvlic_upload_field(ctx_, xyz, VVLIC_DTYPE_FLOAT32, nx, ny, nz, sliceDist, storage, &id), "setDataTex");
    vol_ = id;
    return id;
  }
  /* the UCHAR3 variant (DATRAW_UCHAR) */
  int setDataTex(const unsigned char* xyz, int nx, int ny, int nz, const float* sliceDist = nullptr,
                 int storage = VVLIC_STORAGE_F16) {
    int32_t id = 0;
    check(vvlic_upload_field(ctx_, xyz, VVLIC_DTYPE_UINT8, nx, ny, nz, sliceDist, storage, &id), "setDataTex");
    vol_ = id;
    return id;
  }
  void useVolume(int id) { vol_ = id; }
  /* The animation step of idle() (3DLIC.cpp:129-145): createTextureIterp of the next
   * interpolation stage, here rewriting the current volume in place (same dimensions). */
  void updateDataTex(const float* xyz0, const float* xyz1, int nx, int ny, int nz, int interpIndex,
                     int interpSize) {
    check(vvlic_update_field_interp(ctx_, vol_, xyz0, xyz1, VVLIC_DTYPE_FLOAT32, nx, ny, nz, interpIndex, interpSize),
          "updateDataTex");
  }
  void updateDataTex(const float* xyz, int nx, int ny, int nz) {
    check(vvlic_update_field(ctx_, vol_, xyz, VVLIC_DTYPE_FLOAT32, nx, ny, nz), "updateDataTex");
  }
  /* the same step ordered on a CUDA stream: the host copy overlaps the renders already enqueued
   * there; `xyz` must stay unchanged until the stream has passed the update */
  void updateDataTexAsync(const float* xyz, int nx, int ny, int nz, void* stream) {
    check(vvlic_update_field_async(ctx_, vol_, xyz, VVLIC_DTYPE_FLOAT32, nx, ny, nz, stream), "updateDataTexAsync");
  }
  /* the same step from float32 xyz already in device memory (no host copy) */
  void updateDataTexDevice(const float* d_xyz, int nx, int ny, int nz, void* stream) {
    check(vvlic_update_field_device(ctx_, vol_, d_xyz, nx, ny, nz, stream), "updateDataTexDevice");
  }
  /* VectorDataSet::loadData(file) + createTextureIterp: a .dat/.raw vector data set (the
   * timestep, or the first one for -1) becomes the current volume */
  int loadData(const char* datFile, int timestep = -1, int storage = VVLIC_STORAGE_F16) {
    int32_t id = 0;
    vvlic_status s = vvlic_upload_dat(ctx_, datFile, timestep, storage, &id);
    if (s != VVLIC_OK) throw Error(s, std::string("loadData: ") + vvlic_io_error());
    vol_ = id;
    return id;
  }
  /* Renderer::setTechnique (renderer.h:44); LICVOLUME renders need computeLICVolume first */
  void setTechnique(RenderTechnique rt) {
    params_.technique = (int32_t)rt;
    check(vvlic_set_params(ctx_, &params_), "setTechnique");
  }
  /* Renderer::renderLICVolume (renderer.cpp:1311-1374): the LIC volume of the current volume */
  void computeLICVolume(int nx = 512, int ny = 512, int nz = 512) {
    check(vvlic_compute_lic_volume(ctx_, vol_, nx, ny, nz), "computeLICVolume");
  }

  /* NoiseDataSet::createTexture + Renderer::setNoiseTex; gradients = the -g switch
   * (parseArg.cpp), gradMode = VVLIC_NOISE_GRAD_SOBEL (gradient.h SOBEL 1) or _CENTRAL. */
  void setNoiseTex(const unsigned char* noise, int mx, int my, int mz, bool gradients,
                   int gradMode = VVLIC_NOISE_GRAD_SOBEL) {
    check(vvlic_upload_noise(ctx_, noise, mx, my, mz, gradients ? gradMode : VVLIC_NOISE_SCALAR), "setNoiseTex");
  }
  /* a noise of the current noise's extent and kind, ordered on a CUDA stream like
   * updateDataTexAsync */
  void setNoiseTexAsync(const unsigned char* noise, int mx, int my, int mz, bool gradients, void* stream,
                        int gradMode = VVLIC_NOISE_GRAD_SOBEL) {
    check(vvlic_upload_noise_async(ctx_, noise, mx, my, mz, gradients ? gradMode : VVLIC_NOISE_SCALAR, stream),
          "setNoiseTexAsync");
  }
  /* VolumeDataSet + Renderer::setScalarTex (the freqSampling gate volume) */
  void setScalarTex(const float* scalar, int nx, int ny, int nz) {
    check(vvlic_upload_scalar(ctx_, scalar, nx, ny, nz), "setScalarTex");
  }
  /* TransferEdit::updateTextures + setTFrgbTex / setTFalphaOpacTex; 256 entries in [0,1] */
  void setTFrgbTex(const float* rgba1024) { check(vvlic_set_tf(ctx_, rgba1024, nullptr), "setTFrgbTex"); }
  void setTFalphaOpacTex(const float* opacity256) { check(vvlic_set_tf(ctx_, nullptr, opacity256), "setTFalphaOpacTex"); }
  /* LICFilter::createTexture + Renderer::setLICFilter: the uint8 kernel table */
  void setLICFilter(const unsigned char* table, int width, int clamp = VVLIC_KERNEL_CLAMP_BORDER) {
    check(vvlic_set_filter_table(ctx_, table, width, clamp), "setLICFilter");
  }
  /* LICFilter::loadData(png) + setLICFilter */
  void loadFilter(const char* png) {
    vvlic_status s = vvlic_load_filter_png(ctx_, png);
    if (s != VVLIC_OK) throw Error(s, std::string("loadFilter: ") + vvlic_io_error());
  }
  /* TransferEdit::loadTF(name) + setTFrgbTex / setTFalphaOpacTex */
  void loadTF(const char* name) {
    vvlic_status s = vvlic_load_tf_png(ctx_, name);
    if (s != VVLIC_OK) throw Error(s, std::string("loadTF: ") + vvlic_io_error());
  }
  /* LICFilter::createBoxFilter */
  void setBoxFilter(int width = 256) {
    unsigned char t[1024];
    int32_t w = 0;
    check(vvlic_make_filter_table(VVLIC_FILTER_BOX, width, t, &w), "setBoxFilter");
    setLICFilter(t, w);
  }
  /* Renderer::setLICParams */
  void setLICParams(const LICParams& p) {
    params_.step_size_vol = p.stepSizeVol;
    params_.gradient_scale = p.gradientScale;
    params_.illum_scale = p.illumScale;
    params_.freq_scale = p.freqScale;
    params_.num_iterations = p.numIterations;
    params_.steps_forward = p.stepsForward;
    params_.steps_backward = p.stepsBackward;
    params_.step_size_lic = p.stepSizeLIC;
    check(vvlic_set_params(ctx_, &params_), "setLICParams");
  }
  /* Renderer::loadGLSLShader(defines): the shader variant from the same define text the
   * reference injects ("#define ILLUM_GRADIENT", "#define SPEED_OF_FLOW", ...). */
  void loadGLSLShader(const char* defines) {
    std::string d = defines ? defines : "";
    params_.illum = VVLIC_ILLUM_NONE;
    params_.speed_of_flow = 0;
    if (d.find("ILLUM_GRADIENT") != std::string::npos) params_.illum = VVLIC_ILLUM_GRADIENT;
    if (d.find("ILLUM_ZOECKLER") != std::string::npos) params_.illum = VVLIC_ILLUM_ZOECKLER;
    if (d.find("ILLUM_MALLO") != std::string::npos) params_.illum = VVLIC_ILLUM_MALLO;
    if (d.find("SPEED_OF_FLOW") != std::string::npos) params_.speed_of_flow = 1;
    check(vvlic_set_params(ctx_, &params_), "loadGLSLShader");
  }
  /* Renderer::setCamera + Camera::setCamera */
  void setCamera(const vvlic_view& v) {
    view_ = v;
    check(vvlic_set_view(ctx_, &view_), "setCamera");
  }
  /* Renderer::setLight + updateLightPos: the light in object space */
  void setLight(const float pos[3]) {
    std::memcpy(params_.light_pos, pos, sizeof(float) * 3);
    check(vvlic_set_params(ctx_, &params_), "setLight");
  }
  /* Illumination::setMaterial + createIllumTextures, and the spot exponent the reference copies
   * into GL_LIGHT0 (3DLIC.cpp:735-736); the renderer's setIllum*Tex bindings are implicit. */
  void setLineMaterial(const vvlic_line_material& m) {
    check(vvlic_set_line_material(ctx_, &m), "setLineMaterial");
    params_.spec_exp = m.spec_exp;
    check(vvlic_set_params(ctx_, &params_), "setLineMaterial");
  }
  void setLowRes(bool lowRes) {
    params_.low_res = lowRes ? 1 : 0;
    check(vvlic_set_params(ctx_, &params_), "setLowRes");
  }
  /* Renderer::render -> raycastVolume: writes w*h RGBA floats (row 0 = bottom) to host memory */
  void render(float* rgba, int w, int h) { check(vvlic_render(ctx_, vol_, rgba, w, h), "render"); }
  /* the screenshot of renderBackground (renderer.cpp:1480-1500): PNG of the render buffer, or
   * of the window image composited over white */
  static void saveImage(const char* file, const float* rgba, int w, int h, bool overWhite = false) {
    vvlic_status s = vvlic_image_write(file, rgba, w, h, VVLIC_IMAGE_PNG, overWhite ? 1 : 0);
    if (s != VVLIC_OK) throw Error(s, std::string("saveImage: ") + vvlic_io_error());
  }
  /* asynchronous render into device memory on a CUDA stream */
  void renderDevice(float* d_rgba, int w, int h, void* stream = nullptr) {
    check(vvlic_render_device(ctx_, vol_, d_rgba, w, h, nullptr, stream), "renderDevice");
  }
  /* asynchronous render into host memory (pinned for an overlapping copy) on a CUDA stream;
   * `rgba` holds the image once synchronize(stream) has returned true */
  void renderToHostAsync(float* rgba, int w, int h, void* stream) {
    check(vvlic_render_to_host_async(ctx_, vol_, rgba, w, h, stream), "renderToHostAsync");
  }
  /* waits for the work enqueued on `stream` (NULL: the context's stream); false on timeout */
  bool synchronize(void* stream = nullptr, int timeoutMs = 60000) {
    vvlic_status s = vvlic_synchronize(ctx_, stream, timeoutMs);
    if (s == VVLIC_ERR_TIMEOUT) return false;
    check(s, "synchronize");
    return true;
  }
  vvlic_stats stats() {
    vvlic_stats s;
    check(vvlic_get_stats(ctx_, &s), "stats");
    return s;
  }
  /* full parameter block (variants, quirks, sampler, schedule) */
  vvlic_params& params() { return params_; }
  void applyParams() { check(vvlic_set_params(ctx_, &params_), "applyParams"); }
  vvlic_ctx* handle() { return ctx_; }

 private:
  void check(vvlic_status s, const char* what) {
    if (s != VVLIC_OK) {
      std::string msg = std::string(what) + ": " + vvlic_status_string(s);
      if (ctx_) {
        const char* e = vvlic_last_error(ctx_);
        if (e && *e) msg += std::string(" (") + e + ")";
      }
      throw Error(s, msg);
    }
  }
  vvlic_ctx* ctx_ = nullptr;
  vvlic_params params_;
  vvlic_view view_;
  int vol_ = 0;
};

}  // namespace vvlic

#endif  // VVLIC_RENDERER_HPP_
