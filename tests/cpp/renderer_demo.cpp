// A C++ host program written against vvlic::Renderer the way the reference's 3DLIC.cpp drives
// its Renderer: load a .dat data set and a noise file, set the filter, TF and LICParams, pick
// the shader variant by its define text, render, save the screenshot.  Used by
// tests/test_cpp_host.py; writes the raw float images next to the PNGs for comparison.
//   renderer_demo <dat> <noise> <out_prefix> <w> <h>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "vvlic_renderer.hpp"

static void save_raw(const char* prefix, const char* tag, const std::vector<float>& img) {
  char path[1024];
  std::snprintf(path, sizeof path, "%s_%s.f32", prefix, tag);
  FILE* f = std::fopen(path, "wb");
  if (!f || std::fwrite(img.data(), sizeof(float), img.size(), f) != img.size()) std::exit(3);
  std::fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 6) return 2;
  const int w = std::atoi(argv[4]), h = std::atoi(argv[5]);
  try {
    vvlic::Renderer r(0);
    r.loadData(argv[1], -1, VVLIC_STORAGE_F32);
    int32_t dims[3];
    if (vvlic_noise_read(argv[2], nullptr, 0, dims) != VVLIC_OK) return 4;
    std::vector<unsigned char> noise((size_t)dims[0] * dims[1] * dims[2]);
    if (vvlic_noise_read(argv[2], noise.data(), noise.size(), dims) != VVLIC_OK) return 4;
    r.setNoiseTex(noise.data(), dims[0], dims[1], dims[2], false);
    r.setBoxFilter(256);
    vvlic::LICParams lp;
    lp.stepSizeVol = 1.0f / 64.0f;
    lp.stepsForward = lp.stepsBackward = 8;
    lp.gradientScale = 12.0f;
    r.setLICParams(lp);
    r.params().sampler = VVLIC_SAMPLER_CELL;
    r.params().tf_index = VVLIC_TF_INDEX_MAGNITUDE;
    r.applyParams();
    vvlic_view v;
    vvlic_view_default(&v);
    v.distance = 2.4f;
    r.setCamera(v);
    std::vector<float> img((size_t)w * h * 4);
    r.loadGLSLShader("");
    r.render(img.data(), w, h);
    save_raw(argv[3], "raycast", img);
    char png[1024];
    std::snprintf(png, sizeof png, "%s_raycast.png", argv[3]);
    vvlic::Renderer::saveImage(png, img.data(), w, h, true);
    r.setTechnique(vvlic::VOLIC_SLICING);
    r.render(img.data(), w, h);
    save_raw(argv[3], "slicing", img);
    r.setTechnique(vvlic::VOLIC_RAYCAST);
    r.loadGLSLShader("#define ILLUM_ZOECKLER");
    r.render(img.data(), w, h);
    save_raw(argv[3], "zoeckler", img);
    std::printf("samples %llu\n", (unsigned long long)r.stats().samples);
    // the stream-ordered animation step: the same field re-uploaded in place, then a render
    // into host memory, one wait at the end (the image must equal the first ray-cast)
    vvlic_dat_info info;
    if (vvlic_dat_parse(argv[1], &info) != VVLIC_OK || info.format != VVLIC_DAT_FLOAT || info.components != 3) return 5;
    std::vector<float> xyz((size_t)vvlic_dat_bytes(&info) / sizeof(float));
    if (vvlic_dat_read(&info, info.timestep_begin, xyz.data(), xyz.size() * sizeof(float)) != VVLIC_OK) return 5;
    r.loadGLSLShader("");
    r.updateDataTexAsync(xyz.data(), info.resolution[0], info.resolution[1], info.resolution[2], nullptr);
    std::vector<float> async_img((size_t)w * h * 4);
    r.renderToHostAsync(async_img.data(), w, h, nullptr);
    if (!r.synchronize(nullptr, 120000)) return 6;
    save_raw(argv[3], "async", async_img);
  } catch (const vvlic::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
