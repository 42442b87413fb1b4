// image.cpp -- host image files for the debug env maps (vlb_image_write_*).
//
// The reference writes each probe's env map with stb_image_write's PNG
// writer (src/baker/env_map_generator.cpp:73-112, called from
// light_baker.cpp:306-307 as "<probe>.png").  Here: a PNG of 8-bit RGBA with
// filter type 0 on every row and the zlib stream in stored (uncompressed)
// deflate blocks -- a valid PNG that any reader opens; the compressed bytes
// of stb's encoder are not reproduced.  CRC-32 (ISO 3309 polynomial
// 0xEDB88320, reflected) and Adler-32 follow their published definitions
// (PNG specification section 5.5, RFC 1950).  And a binary PPM (P6, alpha
// dropped).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "vlb_internal.h"

namespace {

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
  for (uint32_t n = 0; n < 256; ++n) {
    uint32_t c = n;
    for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    crc_table[n] = c;
  }
  crc_ready = true;
}

uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xFFFFFFFFu) {
  for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
  return c;
}

void be32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back(uint8_t(x >> 24));
  v.push_back(uint8_t(x >> 16));
  v.push_back(uint8_t(x >> 8));
  v.push_back(uint8_t(x));
}

void chunk(std::vector<uint8_t>& png, const char* type, const std::vector<uint8_t>& data) {
  be32(png, uint32_t(data.size()));
  const size_t start = png.size();
  png.insert(png.end(), type, type + 4);
  png.insert(png.end(), data.begin(), data.end());
  be32(png, crc32(png.data() + start, png.size() - start) ^ 0xFFFFFFFFu);
}

thread_local std::string t_img_err;
vlb_status ifail(vlb_status st, const std::string& m) {
  t_img_err = m;
  return st;
}

}  // namespace

extern "C" {

const char* vlb_image_last_error(void) { return t_img_err.c_str(); }

vlb_status vlb_image_write_png(const char* path, const uint8_t* rgba, uint32_t w, uint32_t h) {
  if (!path || (!rgba && w && h)) return ifail(VLB_ERR_INVALID, "null argument");
  if (w == 0 || h == 0) return ifail(VLB_ERR_INVALID, "empty image");
  if (!crc_ready) crc_init();
  const size_t row = size_t(w) * 4;
  // raw scanlines: filter byte 0 + row bytes
  std::vector<uint8_t> raw;
  raw.reserve((row + 1) * h);
  for (uint32_t y = 0; y < h; ++y) {
    raw.push_back(0);
    raw.insert(raw.end(), rgba + y * row, rgba + (y + 1) * row);
  }
  // zlib stream: header, stored blocks of at most 65535 bytes, Adler-32
  std::vector<uint8_t> z = {0x78, 0x01};
  for (size_t off = 0; off < raw.size() || off == 0;) {
    const size_t len = std::min<size_t>(65535, raw.size() - off);
    const bool last = off + len == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back(uint8_t(len));
    z.push_back(uint8_t(len >> 8));
    z.push_back(uint8_t(~len));
    z.push_back(uint8_t(~len >> 8));
    z.insert(z.end(), raw.begin() + long(off), raw.begin() + long(off + len));
    off += len;
    if (last) break;
  }
  uint32_t a = 1, b = 0;
  for (const uint8_t c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  be32(z, (b << 16) | a);
  std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  std::vector<uint8_t> ihdr;
  be32(ihdr, w);
  be32(ihdr, h);
  ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit, RGBA, deflate, adaptive filtering, no interlace
  chunk(png, "IHDR", ihdr);
  chunk(png, "IDAT", z);
  chunk(png, "IEND", {});
  FILE* f = std::fopen(path, "wb");
  if (!f) return ifail(VLB_ERR_INVALID, std::string("cannot open ") + path);
  const bool ok = std::fwrite(png.data(), 1, png.size(), f) == png.size();
  if (std::fclose(f) != 0 || !ok) return ifail(VLB_ERR_INVALID, std::string("write failed: ") + path);
  return VLB_OK;
}

vlb_status vlb_image_write_ppm(const char* path, const uint8_t* rgba, uint32_t w, uint32_t h) {
  if (!path || (!rgba && w && h)) return ifail(VLB_ERR_INVALID, "null argument");
  if (w == 0 || h == 0) return ifail(VLB_ERR_INVALID, "empty image");
  FILE* f = std::fopen(path, "wb");
  if (!f) return ifail(VLB_ERR_INVALID, std::string("cannot open ") + path);
  std::fprintf(f, "P6\n%u %u\n255\n", w, h);
  std::vector<uint8_t> rgb(size_t(w) * h * 3);
  for (size_t i = 0; i < size_t(w) * h; ++i) std::memcpy(&rgb[3 * i], rgba + 4 * i, 3);
  const bool ok = std::fwrite(rgb.data(), 1, rgb.size(), f) == rgb.size();
  if (std::fclose(f) != 0 || !ok) return ifail(VLB_ERR_INVALID, std::string("write failed: ") + path);
  return VLB_OK;
}

}  // extern "C"
