// Photo::save (src/image.cpp:481-532) without libpng: an 8-bit RGB PNG whose
// bytes are static_cast<png_byte>(value * 255) per channel, as the reference
// writes them. The image data go into zlib "stored" deflate blocks (no
// compression), which every PNG reader accepts; CRC-32 (chunks) and Adler-32
// (zlib stream) are computed here.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "rmn_host.h"

namespace {

struct CrcTable {
  uint32_t t[256];
  CrcTable() {
    for (uint32_t n = 0; n < 256; ++n) {
      uint32_t c = n;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      t[n] = c;
    }
  }
};

void put32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  put32(out, (uint32_t)data.size());
  const size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  put32(out, rmn::png_crc32(0, out.data() + start, out.size() - start));
}

// The reference's byte: static_cast<png_byte>(v * 255). Defined here for
// every float: NaN and values below 0 give 0, values above 1 give 255 (the
// reference's conversion is undefined outside [0, 256)).
uint8_t to_byte(float v) {
  float s = v * 255.0f;
  if (!(s >= 0.0f)) return 0;
  if (s >= 255.0f) return 255;
  return (uint8_t)s;
}

}  // namespace

namespace rmn {

uint32_t png_crc32(uint32_t crc, const uint8_t* p, size_t n) {
  static const CrcTable table;  // initialised once, thread-safe
  crc = ~crc;
  for (size_t i = 0; i < n; ++i) crc = table.t[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
  return ~crc;
}

rmn_status write_png(const float* rgb, int w, int h, const char* path) {
  // scanlines: filter byte 0, then RGB bytes
  const size_t row = 1 + 3 * (size_t)w;
  std::vector<uint8_t> raw(row * h);
  for (int y = 0; y < h; ++y) {
    uint8_t* r = &raw[row * y];
    r[0] = 0;
    for (size_t k = 0; k < 3 * (size_t)w; ++k) r[1 + k] = to_byte(rgb[3 * (size_t)w * y + k]);
  }
  // zlib stream of stored blocks
  std::vector<uint8_t> z;
  z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
  z.push_back(0x78);
  z.push_back(0x01);
  size_t pos = 0;
  do {
    const size_t n = std::min<size_t>(65535, raw.size() - pos);
    const bool last = pos + n == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((uint8_t)(n & 0xff));
    z.push_back((uint8_t)(n >> 8));
    z.push_back((uint8_t)(~n & 0xff));
    z.push_back((uint8_t)((~n >> 8) & 0xff));
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
    pos += n;
  } while (pos < raw.size());
  uint32_t a = 1, b = 0;  // Adler-32
  for (uint8_t c : raw) {
    a = (a + c) % 65521;
    b = (b + a) % 65521;
  }
  put32(z, (b << 16) | a);

  std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  std::vector<uint8_t> ihdr;
  put32(ihdr, (uint32_t)w);
  put32(ihdr, (uint32_t)h);
  ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8 bits, RGB, deflate, filter 0, no interlace
  chunk(out, "IHDR", ihdr);
  chunk(out, "IDAT", z);
  chunk(out, "IEND", {});
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(RMN_ERR_INVALID_ARGUMENT, "could not open %s for writing", path);
  const size_t wrote = std::fwrite(out.data(), 1, out.size(), f);
  const int closed = std::fclose(f);
  if (wrote != out.size() || closed != 0) return fail(RMN_ERR_INTERNAL, "could not write %s", path);
  return RMN_OK;
}

}  // namespace rmn
