/*
 * ORACLE — test infrastructure, not product code.
 *
 * Compiles the reference's own noise-gradient code (VectorVisualization/gradient.cpp:190-531)
 * and its .dat/.raw reader (reader.cpp) unmodified and exposes them through C functions, so the
 * restatement in vvlic_oracle.hpp, the device kernel and the library's reader can be pinned
 * against what the reference itself computes.  Built by
 * oracle/build_ref.sh into oracle/_ref/ (never committed).  VVREF_CENTRAL selects the
 * central-difference branch (SOBEL 0); gradient.h hard-codes SOBEL 1.
 */
#include "gradient.h"
#ifdef VVREF_CENTRAL
#undef SOBEL
#define SOBEL 0
#endif
#include "gradient.cpp"
#include "reader.h"

#include <cstdio>
#include <cstring>
#include <string>

/* VolumeData's destructor lives in dataset.cpp, which is not compiled here; the buffers below
 * are owned by the caller. */
VolumeData::~VolumeData(void) {}

extern "C" int vvref_noise_gradients(const unsigned char* noise, const int m[3], const float sd[3],
                                     unsigned char* out_rgba) {
  VolumeData vd;
  vd.data = (void*)noise;
  vd.newData = NULL;
  vd.dataType = DATRAW_UCHAR;
  vd.dataDim = 1;
  for (int i = 0; i < 3; ++i) {
    vd.size[i] = m[i];
    vd.texSize[i] = m[i];
    vd.sliceDist[i] = sd ? sd[i] : 1.0f;
  }
  float* g = computeGradients(&vd);
  if (!g) return -1;
  filterGradients(&vd, g);
  unsigned char* q = (unsigned char*)quantizeGradients(&vd, g, DATRAW_UCHAR);
  if (!q) return -2;
  /* RGBA pack of NoiseDataSet::createTexture (dataset.cpp:1270-1286) */
  const long count = (long)m[0] * m[1] * m[2];
  for (long a = 0; a < count; ++a) {
    out_rgba[4 * a + 0] = q[3 * a + 0];
    out_rgba[4 * a + 1] = q[3 * a + 1];
    out_rgba[4 * a + 2] = q[3 * a + 2];
    out_rgba[4 * a + 3] = noise[a];
  }
  delete[] g;
  delete[] q;
  return 0;
}

/* DatFile::parseDatFile + getters (reader.cpp:80-262).  Returns 0 on success, -1 when the
 * reference rejects the description. */
extern "C" int vvref_dat_parse(const char* path, char* raw_out, int raw_cap, int sizes[3], float dists[3],
                               int* type, int* dim, int* tbeg, int* tend) {
  DatFile df;
  std::string p(path);
  if (!df.parseDatFile(&p[0])) return -1;
  const char* raw = df.getRawFileName();
  std::snprintf(raw_out, raw_cap, "%s", raw ? raw : "");
  for (int i = 0; i < 3; ++i) {
    sizes[i] = df.getDataSizes()[i];
    dists[i] = df.getDataDists()[i];
  }
  *type = (int)df.getDataType();
  *dim = df.getDataDimension();
  *tbeg = df.getTimeStepBegin();
  *tend = df.getTimeStepEnd();
  return 0;
}

/* DatFile::readRawData (reader.cpp:265-303) of one timestep into out (bytes). */
extern "C" int vvref_dat_read(const char* path, int timestep, void* out, long bytes) {
  DatFile df;
  std::string p(path);
  if (!df.parseDatFile(&p[0])) return -1;
  void* d = df.readRawData(timestep);
  if (!d) return -2;
  std::memcpy(out, d, (size_t)bytes);
  delete[] (char*)d;
  return 0;
}

/* saveGradients (gradient.cpp:149-187) of the reference's own gradients: writes "<path>.grd". */
extern "C" int vvref_save_gradients(const unsigned char* noise, const int m[3], const char* path) {
  VolumeData vd;
  vd.data = (void*)noise;
  vd.newData = NULL;
  vd.dataType = DATRAW_UCHAR;
  vd.dataDim = 1;
  for (int i = 0; i < 3; ++i) {
    vd.size[i] = m[i];
    vd.texSize[i] = m[i];
    vd.sliceDist[i] = 1.0f;
  }
  float* g = computeGradients(&vd);
  if (!g) return -1;
  filterGradients(&vd, g);
  unsigned char* q = (unsigned char*)quantizeGradients(&vd, g, DATRAW_UCHAR);
  std::string p(path);
  const bool ok = q && saveGradients(&vd, &p[0], q, DATRAW_UCHAR, false);
  delete[] g;
  delete[] q;
  return ok ? 0 : -2;
}
