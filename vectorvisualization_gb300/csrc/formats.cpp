// On-disk formats of the reference and the headless image dump: the .dat/.raw volume
// description and raw reader (reader.cpp), the noise volume file (dataset.cpp:1347-1389) and
// the RGBA dump of the render buffer (renderer.cpp:340-420) as PNG or PPM.  Host code only;
// the .dat parser keeps the reference's C stdio line handling (255-byte lines, strstr keys,
// sscanf conversions) so that descriptions parse identically.
#include <ctype.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "vvlic.h"

namespace {

thread_local std::string g_io_error;

vvlic_status io_fail(vvlic_status s, const char* fmt, ...) {
  char buf[1400];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_io_error = buf;
  return s;
}

int type_size(int format) {
  return format == VVLIC_DAT_UCHAR ? 1 : format == VVLIC_DAT_USHORT ? 2 : format == VVLIC_DAT_FLOAT ? 4 : 0;
}

// The raw file name of `timestep`: the pattern formatted with the timestep, 254 characters at
// most, as snprintf(rawFileName, 255, pattern, timestep) produces it.
std::string raw_name(const char* pattern, int timestep) {
  char buf[255];
  // the pattern is the file's own text; it takes at most one integer conversion
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wformat-nonliteral"
  snprintf(buf, sizeof buf, pattern, timestep);
#pragma GCC diagnostic pop
  return buf;
}

bool file_exists(const std::string& p) {
  FILE* f = fopen(p.c_str(), "rb");
  if (!f) return false;
  fclose(f);
  return true;
}

// A raw-file pattern may hold one integer conversion (%d, %i, %03d, ...) for the timestep and
// literal %%; anything else would read arguments that are not there.
bool safe_pattern(const char* p) {
  int conversions = 0;
  for (; *p; ++p) {
    if (*p != '%') continue;
    ++p;
    if (*p == '%') continue;
    while (*p && strchr("-+ #0", *p)) ++p;
    while (*p && isdigit((unsigned char)*p)) ++p;
    if (*p == '.') {
      ++p;
      while (*p && isdigit((unsigned char)*p)) ++p;
    }
    if (*p != 'd' && *p != 'i' && *p != 'u' && *p != 'x' && *p != 'X' && *p != 'o') return false;
    if (++conversions > 1) return false;
  }
  return true;
}

// ---- PNG with stored (uncompressed) deflate blocks ------------------------------------------
uint32_t crc32_update(uint32_t crc, const uint8_t* d, size_t n) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    init = true;
  }
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ d[i]) & 0xFF] ^ (crc >> 8);
  return crc;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

void put_chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  put_be32(out, (uint32_t)data.size());
  const size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  put_be32(out, ~crc32_update(0xFFFFFFFFu, out.data() + start, out.size() - start));
}

std::vector<uint8_t> png_bytes(const uint8_t* rgba_top_first, int w, int h) {
  std::vector<uint8_t> raw;
  raw.reserve((size_t)h * (4 * (size_t)w + 1));
  for (int y = 0; y < h; ++y) {
    raw.push_back(0);  // filter: none
    const uint8_t* row = rgba_top_first + (size_t)y * 4 * w;
    raw.insert(raw.end(), row, row + 4 * (size_t)w);
  }
  std::vector<uint8_t> z = {0x78, 0x01};
  uint32_t a = 1, b = 0;
  for (uint8_t c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  size_t pos = 0;
  do {
    const size_t n = std::min<size_t>(65535, raw.size() - pos);
    const bool last = pos + n == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((uint8_t)(n & 0xFF));
    z.push_back((uint8_t)(n >> 8));
    z.push_back((uint8_t)(~n & 0xFF));
    z.push_back((uint8_t)((~n >> 8) & 0xFF));
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
    pos += n;
  } while (pos < raw.size());
  put_be32(z, (b << 16) | a);
  std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
  std::vector<uint8_t> ihdr;
  put_be32(ihdr, (uint32_t)w);
  put_be32(ihdr, (uint32_t)h);
  ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA, deflate, no filter set, no interlace
  put_chunk(out, "IHDR", ihdr);
  put_chunk(out, "IDAT", z);
  put_chunk(out, "IEND", {});
  return out;
}

}  // namespace

extern "C" const char* vvlic_io_error(void) { return g_io_error.c_str(); }

extern "C" vvlic_status vvlic_dat_parse(const char* dat_path, vvlic_dat_info* info) {
  if (!dat_path || !info) return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "dat_parse: null argument");
  memset(info, 0, sizeof *info);
  info->slice_thickness[0] = info->slice_thickness[1] = info->slice_thickness[2] = 1.0f;
  info->components = 1;
  FILE* fp = fopen(dat_path, "rb");
  if (!fp) return io_fail(VVLIC_ERR_IO, "cannot open .dat file \"%s\"", dat_path);
  char line[255], name[255];
  bool have_name = false;
  vvlic_status st = VVLIC_OK;
  while (st == VVLIC_OK && fgets(line, sizeof line, fp)) {
    if (line[0] == '#') continue;
    const char* colon = strchr(line, ':');
    if (strstr(line, "ObjectFileName")) {
      if (!colon || sscanf(colon + 1, "%254s", name) != 1) {
        st = io_fail(VVLIC_ERR_FORMAT, "parse error: %s", line);
        break;
      }
      have_name = true;
    } else if (strstr(line, "Resolution")) {
      if (!colon || sscanf(colon + 1, "%i %i %i", &info->resolution[0], &info->resolution[1], &info->resolution[2]) != 3)
        st = io_fail(VVLIC_ERR_FORMAT, "parse error: %s", line);
    } else if (strstr(line, "SliceThickness")) {
      if (!colon || sscanf(colon + 1, "%f %f %f", &info->slice_thickness[0], &info->slice_thickness[1],
                           &info->slice_thickness[2]) != 3)
        st = io_fail(VVLIC_ERR_FORMAT, "parse error: %s", line);
    } else if (strstr(line, "Format")) {
      const char* cp;
      if ((cp = strstr(line, "UCHAR")))
        info->format = VVLIC_DAT_UCHAR;
      else if ((cp = strstr(line, "USHORT")))
        info->format = VVLIC_DAT_USHORT;
      else if ((cp = strstr(line, "FLOAT")))
        info->format = VVLIC_DAT_FLOAT;
      else {
        st = io_fail(VVLIC_ERR_FORMAT, "only UCHAR*, USHORT* and FLOAT* data: %s", line);
        break;
      }
      // the component count: the first number after the type name (parseDataDim)
      while (*cp && !isdigit((unsigned char)*cp)) ++cp;
      if (!*cp || sscanf(cp, "%i", &info->components) != 1) info->components = 1;
    } else if (strstr(line, "TimeDependent")) {
      if (!colon || sscanf(colon + 1, "%i %i", &info->timestep_begin, &info->timestep_end) != 2) {
        st = io_fail(VVLIC_ERR_FORMAT, "parse error: %s", line);
      } else if (info->timestep_begin < 0 || info->timestep_end < info->timestep_begin) {
        st = io_fail(VVLIC_ERR_FORMAT, "illegal timestep bounds %d-%d", info->timestep_begin, info->timestep_end);
      }
    }
  }
  fclose(fp);
  if (st != VVLIC_OK) return st;
  if (!have_name) return io_fail(VVLIC_ERR_FORMAT, "no ObjectFileName in \"%s\"", dat_path);
  if (!safe_pattern(name)) return io_fail(VVLIC_ERR_FORMAT, "raw file pattern \"%s\" is not an integer format", name);
  std::string pattern = name;
  if (!file_exists(raw_name(pattern.c_str(), info->timestep_begin))) {
    // relative to the .dat file's directory (DIR_SEP '/' or DIR_SEP_WIN '\\')
    std::string dir = dat_path;
    size_t cut = dir.find_last_of('/');
    if (cut == std::string::npos) cut = dir.find_last_of('\\');
    if (cut == std::string::npos) return io_fail(VVLIC_ERR_IO, "no search path for raw file \"%s\"", name);
    pattern = dir.substr(0, cut + 1) + name;
    if (!file_exists(raw_name(pattern.c_str(), info->timestep_begin)))
      return io_fail(VVLIC_ERR_IO, "cannot open raw file \"%s\"", raw_name(pattern.c_str(), info->timestep_begin).c_str());
  }
  for (int t = info->timestep_begin + 1; t <= info->timestep_end; ++t)
    if (!file_exists(raw_name(pattern.c_str(), t)))
      return io_fail(VVLIC_ERR_IO, "cannot open raw file \"%s\" of timestep %d", raw_name(pattern.c_str(), t).c_str(), t);
  if (pattern.size() >= sizeof info->raw_file) return io_fail(VVLIC_ERR_FORMAT, "raw file path too long");
  memcpy(info->raw_file, pattern.c_str(), pattern.size() + 1);
  return VVLIC_OK;
}

extern "C" uint64_t vvlic_dat_bytes(const vvlic_dat_info* info) {
  if (!info || info->components < 1) return 0;
  for (int i = 0; i < 3; ++i)
    if (info->resolution[i] < 1) return 0;
  return (uint64_t)type_size(info->format) * (uint64_t)info->components * (uint64_t)info->resolution[0] *
         (uint64_t)info->resolution[1] * (uint64_t)info->resolution[2];
}

extern "C" vvlic_status vvlic_dat_read(const vvlic_dat_info* info, int32_t timestep, void* out, uint64_t capacity) {
  if (!info || !out) return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "dat_read: null argument");
  if (timestep < info->timestep_begin || timestep > info->timestep_end)
    return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "timestep %d outside [%d, %d]", timestep, info->timestep_begin,
                   info->timestep_end);
  const uint64_t bytes = vvlic_dat_bytes(info);
  if (bytes == 0) return io_fail(VVLIC_ERR_FORMAT, "dat_read: no data type or resolution");
  if (capacity < bytes) return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "dat_read: need %llu bytes", (unsigned long long)bytes);
  if (!safe_pattern(info->raw_file)) return io_fail(VVLIC_ERR_FORMAT, "raw file pattern is not an integer format");
  const std::string path = raw_name(info->raw_file, timestep);
  FILE* fp = fopen(path.c_str(), "rb");
  if (!fp) return io_fail(VVLIC_ERR_IO, "cannot open raw file \"%s\"", path.c_str());
  const size_t got = fread(out, 1, (size_t)bytes, fp);
  fclose(fp);
  if (got != bytes)
    return io_fail(VVLIC_ERR_IO, "raw file \"%s\" holds %zu of %llu bytes", path.c_str(), got, (unsigned long long)bytes);
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_upload_dat(vvlic_ctx* ctx, const char* dat_path, int32_t timestep, int32_t storage,
                                        int32_t* vol_id) {
  if (!ctx) return VVLIC_ERR_BAD_HANDLE;
  vvlic_dat_info info;
  vvlic_status st = vvlic_dat_parse(dat_path, &info);
  if (st) return st;
  // VectorDataSet::loadData accepts 3-component UCHAR or FLOAT data only (dataset.cpp:122-140)
  if (info.components != 3) return io_fail(VVLIC_ERR_FORMAT, "\"%s\" is not a vector data set", dat_path);
  if (info.format != VVLIC_DAT_UCHAR && info.format != VVLIC_DAT_FLOAT)
    return io_fail(VVLIC_ERR_FORMAT, "only 8-bit integer and 32-bit float vectors are supported");
  std::vector<uint8_t> buf(vvlic_dat_bytes(&info));
  if ((st = vvlic_dat_read(&info, timestep < 0 ? info.timestep_begin : timestep, buf.data(), buf.size()))) return st;
  return vvlic_upload_field(ctx, buf.data(), info.format == VVLIC_DAT_UCHAR ? VVLIC_DTYPE_UINT8 : VVLIC_DTYPE_FLOAT32,
                            info.resolution[0], info.resolution[1], info.resolution[2], info.slice_thickness, storage,
                            vol_id);
}

extern "C" vvlic_status vvlic_noise_read(const char* path, uint8_t* out, uint64_t capacity, int32_t dims[3]) {
  if (!path || !dims) return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "noise_read: null argument");
  FILE* fp = fopen(path, "rb");
  if (!fp) return io_fail(VVLIC_ERR_IO, "cannot open noise file \"%s\"", path);
  int32_t d[3];
  if (fread(d, 4, 3, fp) != 3) {
    fclose(fp);
    return io_fail(VVLIC_ERR_FORMAT, "cannot read the noise header of \"%s\"", path);
  }
  if (d[0] < 1 || d[1] < 1 || d[2] < 1 || (uint64_t)d[0] * d[1] * d[2] > ((uint64_t)1 << 36)) {
    fclose(fp);
    return io_fail(VVLIC_ERR_FORMAT, "noise header of \"%s\" has sizes %d %d %d", path, d[0], d[1], d[2]);
  }
  dims[0] = d[0];
  dims[1] = d[1];
  dims[2] = d[2];
  vvlic_status st = VVLIC_OK;
  if (out) {
    const uint64_t slice = (uint64_t)d[0] * d[1];
    if (capacity < slice * d[2])
      st = io_fail(VVLIC_ERR_INVALID_ARGUMENT, "noise_read: need %llu bytes", (unsigned long long)(slice * d[2]));
    else if (fread(out, (size_t)slice, (size_t)d[2], fp) != (size_t)d[2])
      st = io_fail(VVLIC_ERR_IO, "error reading noise data from \"%s\"", path);
  }
  fclose(fp);
  return st;
}

extern "C" vvlic_status vvlic_noise_write(const char* path, const uint8_t* noise, const int32_t dims[3]) {
  if (!path || !noise || !dims || dims[0] < 1 || dims[1] < 1 || dims[2] < 1)
    return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "noise_write: bad arguments");
  FILE* fp = fopen(path, "wb");
  if (!fp) return io_fail(VVLIC_ERR_IO, "cannot create \"%s\"", path);
  const size_t n = (size_t)dims[0] * dims[1] * dims[2];
  const bool ok = fwrite(dims, 4, 3, fp) == 3 && fwrite(noise, 1, n, fp) == n;
  if (fclose(fp) != 0 || !ok) return io_fail(VVLIC_ERR_IO, "writing \"%s\" failed", path);
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_image_write(const char* path, const float* rgba, int32_t w, int32_t h, int32_t kind,
                                         int32_t composite) {
  if (!path || !rgba || w < 1 || h < 1 || (kind != VVLIC_IMAGE_PPM && kind != VVLIC_IMAGE_PNG))
    return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "image_write: bad arguments");
  // RGBA8 rows top first; the float image's row 0 is the bottom (glGetTexImage order)
  std::vector<uint8_t> px((size_t)w * h * 4);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const float* s = rgba + 4 * ((size_t)y * w + x);
      uint8_t* d = px.data() + 4 * ((size_t)(h - 1 - y) * w + x);
      const float om = 1.0f - s[3];
      for (int c = 0; c < 4; ++c) {
        float v = s[c];
        if (composite) v = std::min(std::max(om * 1.0f + v, 0.0f), 1.0f);  // over white
        int q = (v == v) ? (int)(255.0f * v) : 0;  // (int)(scale * value), NaN -> 0
        d[c] = (uint8_t)(q > 255 ? 255 : (q < 0 ? 0 : q));
      }
    }
  FILE* fp = fopen(path, "wb");
  if (!fp) return io_fail(VVLIC_ERR_IO, "cannot create \"%s\"", path);
  bool ok;
  if (kind == VVLIC_IMAGE_PNG) {
    const std::vector<uint8_t> png = png_bytes(px.data(), w, h);
    ok = fwrite(png.data(), 1, png.size(), fp) == png.size();
  } else {
    // binary P6 with maxval 255 (ppmWrite, imageUtils.cpp:210-244, writes the largest byte as
    // maxval, which rescales the image in viewers; the dump keeps the bytes' meaning)
    std::vector<uint8_t> rgb((size_t)w * h * 3);
    for (size_t i = 0; i < (size_t)w * h; ++i)
      for (int c = 0; c < 3; ++c) rgb[3 * i + c] = px[4 * i + c];
    ok = fprintf(fp, "P6\n%i %i\n255\n", w, h) > 0 && fwrite(rgb.data(), 1, rgb.size(), fp) == rgb.size();
  }
  if (fclose(fp) != 0 || !ok) return io_fail(VVLIC_ERR_IO, "writing \"%s\" failed", path);
  return VVLIC_OK;
}
