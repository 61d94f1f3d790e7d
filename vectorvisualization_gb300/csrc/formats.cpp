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
#include <cstdlib>
#include <cstring>
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

// 8-bit PNG of `ch` channels (2: gray + alpha, 4: RGBA), rows top first.
std::vector<uint8_t> png_bytes(const uint8_t* px_top_first, int w, int h, int ch = 4) {
  std::vector<uint8_t> raw;
  raw.reserve((size_t)h * (ch * (size_t)w + 1));
  for (int y = 0; y < h; ++y) {
    raw.push_back(0);  // filter: none
    const uint8_t* row = px_top_first + (size_t)y * ch * w;
    raw.insert(raw.end(), row, row + ch * (size_t)w);
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
  // 8-bit, colour type 4 (gray + alpha) or 6 (RGBA), deflate, no filter set, no interlace
  ihdr.insert(ihdr.end(), {8, (uint8_t)(ch == 2 ? 4 : 6), 0, 0, 0});
  put_chunk(out, "IHDR", ihdr);
  put_chunk(out, "IDAT", z);
  put_chunk(out, "IEND", {});
  return out;
}

// ---- PNG reading: inflate (RFC 1951) + scanline filters, 8-bit gray / gray+alpha / RGB / RGBA,
// non-interlaced: the images pngRead accepts (imageUtils.cpp:20-100) ---------------------------
struct Bits {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t buf = 0;
  int cnt = 0;
  bool bad = false;
  int get(int k) {  // k bits, least significant first
    while (cnt < k) {
      if (pos >= n) {
        bad = true;
        return 0;
      }
      buf |= (uint32_t)p[pos++] << cnt;
      cnt += 8;
    }
    const int v = (int)(buf & ((1u << k) - 1));
    buf >>= k;
    cnt -= k;
    return v;
  }
};

// Canonical Huffman code: count[l] codes of length l, symbols in code order.
struct Huff {
  uint16_t count[16];
  uint16_t symbol[320];
};

bool huff_build(Huff& h, const uint8_t* len, int n) {
  std::memset(h.count, 0, sizeof h.count);
  for (int s = 0; s < n; ++s) h.count[len[s]]++;
  h.count[0] = 0;
  int left = 1;  // over-subscribed lengths are invalid
  for (int l = 1; l < 16; ++l) {
    left = left * 2 - h.count[l];
    if (left < 0) return false;
  }
  uint16_t offs[16];
  offs[1] = 0;
  for (int l = 1; l < 15; ++l) offs[l + 1] = (uint16_t)(offs[l] + h.count[l]);
  for (int s = 0; s < n; ++s)
    if (len[s]) h.symbol[offs[len[s]]++] = (uint16_t)s;
  return true;
}

int huff_decode(Bits& b, const Huff& h) {
  int code = 0, first = 0, index = 0;
  for (int l = 1; l < 16; ++l) {
    code |= b.get(1);
    if (b.bad) return -1;
    const int c = h.count[l];
    if (code - first < c) return h.symbol[index + (code - first)];
    index += c;
    first = (first + c) << 1;
    code <<= 1;
  }
  return -1;
}

// Length and distance bases of RFC 1951 section 3.2.5.
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(Bits& b, std::vector<uint8_t>& out, const Huff& lit, const Huff& dist, size_t limit) {
  for (;;) {
    int s = huff_decode(b, lit);
    if (s < 0) return false;
    if (s < 256) {
      if (out.size() >= limit) return false;
      out.push_back((uint8_t)s);
    } else if (s == 256) {
      return true;
    } else {
      s -= 257;
      if (s >= 29) return false;
      const size_t len = kLenBase[s] + b.get(kLenExtra[s]);
      const int ds = huff_decode(b, dist);
      if (ds < 0 || ds >= 30) return false;
      const size_t d = kDistBase[ds] + b.get(kDistExtra[ds]);
      if (b.bad || d > out.size() || out.size() + len > limit) return false;
      for (size_t k = 0; k < len; ++k) out.push_back(out[out.size() - d]);
    }
  }
}

// zlib stream (RFC 1950) -> at most `limit` bytes; false on any inconsistency.
bool zlib_inflate(const uint8_t* p, size_t n, size_t limit, std::vector<uint8_t>& out) {
  if (n < 6 || (p[0] & 0x0F) != 8 || ((p[0] << 8) | p[1]) % 31 != 0 || (p[1] & 0x20)) return false;
  Bits b{p + 2, n - 6};
  int last;
  do {
    last = b.get(1);
    const int type = b.get(2);
    if (b.bad) return false;
    if (type == 0) {  // stored
      b.buf = 0;
      b.cnt = 0;
      if (b.pos + 4 > b.n) return false;
      const size_t len = b.p[b.pos] | (b.p[b.pos + 1] << 8), nlen = b.p[b.pos + 2] | (b.p[b.pos + 3] << 8);
      b.pos += 4;
      if (len != (~nlen & 0xFFFF) || b.pos + len > b.n || out.size() + len > limit) return false;
      out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
      b.pos += len;
    } else if (type == 1) {  // fixed codes
      uint8_t l[320];
      for (int i = 0; i < 144; ++i) l[i] = 8;
      for (int i = 144; i < 256; ++i) l[i] = 9;
      for (int i = 256; i < 280; ++i) l[i] = 7;
      for (int i = 280; i < 288; ++i) l[i] = 8;
      Huff lit, dist;
      huff_build(lit, l, 288);
      for (int i = 0; i < 30; ++i) l[i] = 5;
      huff_build(dist, l, 30);
      if (!inflate_codes(b, out, lit, dist, limit)) return false;
    } else if (type == 2) {  // dynamic codes
      const int nlen = b.get(5) + 257, ndist = b.get(5) + 1, ncode = b.get(4) + 4;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t l[320] = {0};
      for (int i = 0; i < ncode; ++i) l[order[i]] = (uint8_t)b.get(3);
      Huff lc;
      if (b.bad || nlen > 286 || ndist > 30 || !huff_build(lc, l, 19)) return false;
      uint8_t lens[320] = {0};
      int i = 0;
      while (i < nlen + ndist) {
        const int s = huff_decode(b, lc);
        if (s < 0) return false;
        if (s < 16) {
          lens[i++] = (uint8_t)s;
          continue;
        }
        int rep, val = 0;
        if (s == 16) {
          if (i == 0) return false;
          val = lens[i - 1];
          rep = 3 + b.get(2);
        } else if (s == 17) {
          rep = 3 + b.get(3);
        } else {
          rep = 11 + b.get(7);
        }
        if (b.bad || i + rep > nlen + ndist) return false;
        while (rep--) lens[i++] = (uint8_t)val;
      }
      Huff lit, dist;
      if (!huff_build(lit, lens, nlen) || !huff_build(dist, lens + nlen, ndist)) return false;
      if (!inflate_codes(b, out, lit, dist, limit)) return false;
    } else {
      return false;
    }
  } while (!last);
  // Adler-32 of the output, big-endian, right after the deflate stream (byte aligned)
  uint32_t a = 1, s2 = 0;
  for (uint8_t c : out) {
    a = (a + c) % 65521u;
    s2 = (s2 + a) % 65521u;
  }
  const size_t q = b.pos;  // the unread bits of the last byte are padding
  if (q + 4 > n - 2) return false;
  const uint8_t* t = p + 2 + q;
  return (((uint32_t)t[0] << 24) | ((uint32_t)t[1] << 16) | ((uint32_t)t[2] << 8) | t[3]) == ((s2 << 16) | a);
}

uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

vvlic_status png_decode(const std::vector<uint8_t>& f, std::vector<uint8_t>& px, int& w, int& h, int& ch) {
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
  if (f.size() < 8 || std::memcmp(f.data(), sig, 8) != 0) return io_fail(VVLIC_ERR_FORMAT, "not a PNG file");
  size_t pos = 8;
  std::vector<uint8_t> idat;
  bool ihdr = false;
  int depth = 0, ctype = 0, interlace = 0;
  while (pos + 12 <= f.size()) {
    const uint32_t len = be32(&f[pos]);
    if (len > f.size() - pos - 12) return io_fail(VVLIC_ERR_FORMAT, "truncated PNG chunk");
    const uint8_t* type = &f[pos + 4];
    const uint8_t* data = &f[pos + 8];
    if (~crc32_update(0xFFFFFFFFu, type, len + 4) != be32(data + len)) return io_fail(VVLIC_ERR_FORMAT, "PNG CRC error");
    if (!std::memcmp(type, "IHDR", 4) && len == 13) {
      w = (int)be32(data);
      h = (int)be32(data + 4);
      depth = data[8];
      ctype = data[9];
      interlace = data[12];
      ihdr = true;
    } else if (!std::memcmp(type, "IDAT", 4)) {
      idat.insert(idat.end(), data, data + len);
    } else if (!std::memcmp(type, "IEND", 4)) {
      break;
    }
    pos += 12 + len;
  }
  if (!ihdr || w < 1 || h < 1 || w > 65536 || h > 65536) return io_fail(VVLIC_ERR_FORMAT, "bad PNG header");
  // pngRead: 8 bits per channel, gray / gray+alpha / RGB / RGBA (imageUtils.cpp:73-95)
  if (depth != 8) return io_fail(VVLIC_ERR_FORMAT, "only 8 bits per channel are supported");
  ch = ctype == 0 ? 1 : ctype == 4 ? 2 : ctype == 2 ? 3 : ctype == 6 ? 4 : 0;
  if (!ch) return io_fail(VVLIC_ERR_FORMAT, "PNG colour type %d (not gray, gray+alpha, RGB or RGBA)", ctype);
  if (interlace) return io_fail(VVLIC_ERR_UNSUPPORTED, "interlaced PNG");
  const size_t stride = (size_t)w * ch;
  std::vector<uint8_t> raw;
  if (!zlib_inflate(idat.data(), idat.size(), (stride + 1) * h, raw) || raw.size() != (stride + 1) * h)
    return io_fail(VVLIC_ERR_FORMAT, "corrupt PNG image data");
  px.assign(stride * h, 0);
  for (int y = 0; y < h; ++y) {
    const uint8_t ft = raw[(stride + 1) * y];
    const uint8_t* src = &raw[(stride + 1) * y + 1];
    uint8_t* row = &px[stride * y];
    const uint8_t* up = y ? &px[stride * (y - 1)] : nullptr;
    for (size_t x = 0; x < stride; ++x) {
      const int a = x >= (size_t)ch ? row[x - ch] : 0, b = up ? up[x] : 0, c = (up && x >= (size_t)ch) ? up[x - ch] : 0;
      int pred;
      switch (ft) {
        case 0: pred = 0; break;
        case 1: pred = a; break;
        case 2: pred = b; break;
        case 3: pred = (a + b) / 2; break;
        case 4: {  // Paeth
          const int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
          pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
          break;
        }
        default: return io_fail(VVLIC_ERR_FORMAT, "PNG filter type %d", ft);
      }
      row[x] = (uint8_t)(src[x] + pred);
    }
  }
  return VVLIC_OK;
}

vvlic_status read_file(const char* path, std::vector<uint8_t>& data) {
  FILE* fp = fopen(path, "rb");
  if (!fp) return io_fail(VVLIC_ERR_IO, "cannot open \"%s\"", path);
  uint8_t buf[65536];
  size_t got;
  while ((got = fread(buf, 1, sizeof buf, fp)) > 0) data.insert(data.end(), buf, buf + got);
  fclose(fp);
  return VVLIC_OK;
}

vvlic_status png_load(const char* path, std::vector<uint8_t>& px, int& w, int& h, int& ch) {
  std::vector<uint8_t> f;
  vvlic_status st = read_file(path, f);
  if (st) return st;
  st = png_decode(f, px, w, h, ch);
  if (st) io_fail(st, "\"%s\": %s", path, std::string(g_io_error).c_str());
  return st;
}

// TransferEdit::setTFFileNames (transferEdit.cpp:113-158): "<base>_rgba<ext>" and
// "<base>_alpha<ext>", or "_rgba.png" / "_alpha.png" appended without an extension.
void tf_file_names(const char* name, std::string& rgba, std::string& alpha) {
  const char* dot = strrchr(name, '.');
  if (!dot) {
    rgba = std::string(name) + "_rgba.png";
    alpha = std::string(name) + "_alpha.png";
  } else {
    const std::string base(name, dot - name);
    rgba = base + "_rgba" + dot;
    alpha = base + "_alpha" + dot;
  }
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

extern "C" vvlic_status vvlic_png_read(const char* path, uint8_t* out, uint64_t capacity, int32_t* w, int32_t* h,
                                      int32_t* channels) {
  if (!path || !w || !h || !channels) return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "png_read: null argument");
  std::vector<uint8_t> px;
  int ww = 0, hh = 0, ch = 0;
  vvlic_status st = png_load(path, px, ww, hh, ch);
  if (st) return st;
  *w = ww;
  *h = hh;
  *channels = ch;
  if (out) {
    if (capacity < px.size())
      return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "png_read: need %zu bytes", px.size());
    std::memcpy(out, px.data(), px.size());
  }
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_load_filter_png(vvlic_ctx* ctx, const char* path) {
  if (!ctx) return VVLIC_ERR_BAD_HANDLE;
  if (!path) return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "load_filter_png: null path");
  std::vector<uint8_t> px;
  int w = 0, h = 0, ch = 0;
  vvlic_status st = png_load(path, px, w, h, ch);
  if (st) return st;
  if (w > 1024) return io_fail(VVLIC_ERR_UNSUPPORTED, "filter kernel \"%s\" is %d texels wide (at most 1024)", path, w);
  // LICFilter::loadData: the first channel of the first row; vvlic_set_filter_table centres it
  // in the next power of two
  std::vector<uint8_t> table((size_t)w);
  for (int i = 0; i < w; ++i) table[(size_t)i] = px[(size_t)i * ch];
  return vvlic_set_filter_table(ctx, table.data(), w, VVLIC_KERNEL_CLAMP_BORDER);
}

extern "C" vvlic_status vvlic_load_tf_png(vvlic_ctx* ctx, const char* name) {
  if (!ctx) return VVLIC_ERR_BAD_HANDLE;
  if (!name) return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "load_tf_png: null name");
  std::string frgba, falpha;
  tf_file_names(name, frgba, falpha);
  float rgba[4 * VVLIC_TF_ENTRIES], opac[VVLIC_TF_ENTRIES];
  vvlic_status st = vvlic_get_tf(ctx, rgba, opac);
  if (st) return st;
  const int n = VVLIC_TF_ENTRIES;
  std::vector<uint8_t> px;
  int w = 0, h = 0, ch = 0;
  // loadRGBATF (transferEdit.cpp:242-285): the first 256 pixels in row order; gray is copied to
  // r, g and b; a second (gray) or fourth (RGB) channel is alpha
  st = png_load(frgba.c_str(), px, w, h, ch);
  if (st == VVLIC_OK && (size_t)w * h < (size_t)n)
    st = io_fail(VVLIC_ERR_FORMAT, "transfer function \"%s\" holds fewer than %d pixels", frgba.c_str(), n);
  if (st == VVLIC_OK) {
    for (int i = 0; i < n; ++i) {
      const uint8_t* q = &px[(size_t)i * ch];
      if (ch < 3) {
        rgba[4 * i] = rgba[4 * i + 1] = rgba[4 * i + 2] = q[0] / 255.0f;
        if (ch == 2) rgba[4 * i + 3] = q[1] / 255.0f;
      } else {
        for (int c = 0; c < 3; ++c) rgba[4 * i + c] = q[c] / 255.0f;
        if (ch == 4) rgba[4 * i + 3] = q[3] / 255.0f;
      }
    }
    return vvlic_set_tf(ctx, rgba, nullptr);
  }
  // loadTF (transferEdit.cpp:224-239) evaluates `!loadRGBATF() && !loadAlphaOpacTF()`: the
  // alpha/opacity file is read only when the RGBA file could not be
  const std::string first_error = g_io_error;
  px.clear();
  st = png_load(falpha.c_str(), px, w, h, ch);
  if (st == VVLIC_OK && (size_t)w * h < (size_t)n)
    st = io_fail(VVLIC_ERR_FORMAT, "transfer function \"%s\" holds fewer than %d pixels", falpha.c_str(), n);
  if (st) return io_fail(st, "%s; %s", first_error.c_str(), std::string(g_io_error).c_str());
  // loadAlphaOpacTF (transferEdit.cpp:288-313): first channel alpha, second opacity
  for (int i = 0; i < n; ++i) {
    const uint8_t* q = &px[(size_t)i * ch];
    rgba[4 * i + 3] = q[0] / 255.0f;
    if (ch == 2) opac[i] = q[1] / 255.0f;
  }
  return vvlic_set_tf(ctx, rgba, opac);
}

extern "C" vvlic_status vvlic_save_tf_png(vvlic_ctx* ctx, const char* name) {
  if (!ctx) return VVLIC_ERR_BAD_HANDLE;
  if (!name) return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "save_tf_png: null name");
  std::string frgba, falpha;
  tf_file_names(name, frgba, falpha);
  float rgba[4 * VVLIC_TF_ENTRIES], opac[VVLIC_TF_ENTRIES];
  vvlic_status st = vvlic_get_tf(ctx, rgba, opac);
  if (st) return st;
  const int n = VVLIC_TF_ENTRIES, rows = 10;
  auto byte = [](float v) -> uint8_t {
    const float c = v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f;  // NaN -> 0
    return (uint8_t)(c * 255.0f + 0.5f);
  };
  // saveTF (transferEdit.cpp:163-221): 10 identical rows, RGBA then (alpha, opacity)
  std::vector<uint8_t> a((size_t)rows * n * 4), b((size_t)rows * n * 2);
  for (int r = 0; r < rows; ++r)
    for (int i = 0; i < n; ++i) {
      for (int c = 0; c < 4; ++c) a[((size_t)r * n + i) * 4 + c] = byte(rgba[4 * i + c]);
      b[((size_t)r * n + i) * 2] = byte(rgba[4 * i + 3]);
      b[((size_t)r * n + i) * 2 + 1] = byte(opac[i]);
    }
  const std::string* names[2] = {&frgba, &falpha};
  const std::vector<uint8_t> files[2] = {png_bytes(a.data(), n, rows, 4), png_bytes(b.data(), n, rows, 2)};
  for (int k = 0; k < 2; ++k) {
    FILE* fp = fopen(names[k]->c_str(), "wb");
    if (!fp) return io_fail(VVLIC_ERR_IO, "cannot create \"%s\"", names[k]->c_str());
    const bool ok = fwrite(files[k].data(), 1, files[k].size(), fp) == files[k].size();
    if (fclose(fp) != 0 || !ok) return io_fail(VVLIC_ERR_IO, "writing \"%s\" failed", names[k]->c_str());
  }
  return VVLIC_OK;
}

extern "C" vvlic_status vvlic_upload_noise_file(vvlic_ctx* ctx, const char* path, int32_t mode) {
  if (!ctx) return VVLIC_ERR_BAD_HANDLE;
  if (!path) return io_fail(VVLIC_ERR_INVALID_ARGUMENT, "upload_noise_file: null path");
  int32_t d[3];
  vvlic_status st = vvlic_noise_read(path, nullptr, 0, d);
  if (st) return st;
  const size_t n = (size_t)d[0] * d[1] * d[2];
  std::vector<uint8_t> noise(n);
  if ((st = vvlic_noise_read(path, noise.data(), n, d))) return st;
  if (mode == VVLIC_NOISE_SCALAR) return vvlic_upload_noise(ctx, noise.data(), d[0], d[1], d[2], mode);
  // loadGradients (gradient.cpp:112-146): "<path>.grd" with at least 3 bytes per voxel
  const std::string grd = std::string(path) + ".grd";
  std::vector<uint8_t> cached;
  if (read_file(grd.c_str(), cached) == VVLIC_OK && cached.size() >= 3 * n) {
    std::vector<uint8_t> rgba(4 * n);
    for (size_t i = 0; i < n; ++i) {  // the RGBA pack of dataset.cpp:1270-1286
      rgba[4 * i] = cached[3 * i];
      rgba[4 * i + 1] = cached[3 * i + 1];
      rgba[4 * i + 2] = cached[3 * i + 2];
      rgba[4 * i + 3] = noise[i];
    }
    return vvlic_upload_noise_rgba(ctx, rgba.data(), d[0], d[1], d[2], mode);
  }
  if ((st = vvlic_upload_noise(ctx, noise.data(), d[0], d[1], d[2], mode))) return st;
  // saveGradients (gradient.cpp:149-187): the quantised x, y, z per voxel for the next time
  std::vector<uint8_t> rgba(4 * n), xyz(3 * n);
  if ((st = vvlic_download_noise(ctx, rgba.data(), rgba.size()))) return st;
  for (size_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) xyz[3 * i + c] = rgba[4 * i + c];
  FILE* fp = fopen(grd.c_str(), "wb");
  if (fp) {
    const bool ok = fwrite(xyz.data(), 1, xyz.size(), fp) == xyz.size();
    if (fclose(fp) != 0 || !ok) remove(grd.c_str());  // no partial cache
  }
  return VVLIC_OK;
}
