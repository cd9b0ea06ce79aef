// Photo::save (src/image.cpp:481-532) without libpng: an 8-bit RGB PNG whose
// bytes are static_cast<png_byte>(value * 255) per channel, as the reference
// writes them. Rows are filtered adaptively and the stream deflated
// (zlib_compress, image_io.cpp) as libpng does by default; the decoded
// pixels, not the file bytes, are what matches the reference's file.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <vector>

#include "rmn_host.h"

namespace {

// CRC-32 of ISO 3309 / PNG section 5.5 (reflected polynomial 0xEDB88320),
// eight bytes per step by "slicing-by-8" (Kounavis and Berry, 2008): t[k][b]
// is the CRC of byte b followed by k zero bytes, so the eight bytes' table
// entries are independent loads XORed together.
struct CrcTable {
  uint32_t t[8][256];
  CrcTable() {
    for (uint32_t n = 0; n < 256; ++n) {
      uint32_t c = n;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      t[0][n] = c;
    }
    for (int k = 1; k < 8; ++k)
      for (int n = 0; n < 256; ++n) t[k][n] = t[0][t[k - 1][n] & 0xff] ^ (t[k - 1][n] >> 8);
  }
};

inline uint32_t load_le32(const uint8_t* p) {
  return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}

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
  const auto& t = table.t;
  crc = ~crc;
  size_t i = 0;
  for (; i + 8 <= n; i += 8) {
    const uint32_t lo = crc ^ load_le32(p + i), hi = load_le32(p + i + 4);
    crc = t[7][lo & 0xff] ^ t[6][lo >> 8 & 0xff] ^ t[5][lo >> 16 & 0xff] ^ t[4][lo >> 24] ^ t[3][hi & 0xff] ^
          t[2][hi >> 8 & 0xff] ^ t[1][hi >> 16 & 0xff] ^ t[0][hi >> 24];
  }
  for (; i < n; ++i) crc = t[0][(crc ^ p[i]) & 0xff] ^ (crc >> 8);
  return ~crc;
}

rmn_status write_png(const float* rgb, int w, int h, const char* path) {
  // scanlines, each with the filter whose bytes have the smallest sum of
  // magnitudes (bytes read as signed), as libpng's adaptive filtering picks
  const size_t stride = 3 * (size_t)w;
  std::vector<uint8_t> raw((stride + 1) * h);
  auto magnitude = [](uint8_t v) -> uint32_t { return v < 128 ? v : 256u - v; };
  // rows in ranges on separate threads: a row's filter depends only on its
  // own bytes and the row above, both taken from the image
  auto filter_rows = [&](int y0, int y1) {
    std::vector<uint8_t> cur(stride), prev(stride, 0), best(stride), trial(stride);
    if (y0 > 0)
      for (size_t k = 0; k < stride; ++k) prev[k] = to_byte(rgb[stride * (y0 - 1) + k]);
    for (int y = y0; y < y1; ++y) {
      for (size_t k = 0; k < stride; ++k) cur[k] = to_byte(rgb[stride * y + k]);
      uint64_t best_sum = UINT64_MAX;
      int best_ft = 0;
      for (int ft = 0; ft < 5; ++ft) {  // one loop per filter type (bpp = 3)
        uint8_t* t = trial.data();
        const uint8_t* x = cur.data();
        const uint8_t* up = prev.data();
        const size_t k = std::min<size_t>(3, stride);
        switch (ft) {
          case 0:
            std::memcpy(t, x, stride);
            break;
          case 1:
            std::memcpy(t, x, k);
            for (size_t i = k; i < stride; ++i) t[i] = (uint8_t)(x[i] - x[i - 3]);
            break;
          case 2:
            for (size_t i = 0; i < stride; ++i) t[i] = (uint8_t)(x[i] - up[i]);
            break;
          case 3:
            for (size_t i = 0; i < k; ++i) t[i] = (uint8_t)(x[i] - (up[i] >> 1));
            for (size_t i = k; i < stride; ++i) t[i] = (uint8_t)(x[i] - ((x[i - 3] + up[i]) >> 1));
            break;
          default:
            for (size_t i = 0; i < k; ++i) t[i] = (uint8_t)(x[i] - up[i]);  // a = c = 0: Paeth picks b
            for (size_t i = k; i < stride; ++i) {
              const int a = x[i - 3], b = up[i], c = up[i - 3];
              const int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
              const int bc = pc < pb ? c : b;
              t[i] = (uint8_t)(x[i] - ((pc < pb ? pc : pb) < pa ? bc : a));
            }
            break;
        }
        uint64_t sum = 0;
        for (size_t i = 0; i < stride; ++i) sum += magnitude(t[i]);
        if (sum < best_sum) {
          best_sum = sum;
          best_ft = ft;
          best.swap(trial);
        }
      }
      uint8_t* r = &raw[(stride + 1) * y];
      r[0] = (uint8_t)best_ft;
      std::memcpy(r + 1, best.data(), stride);
      prev.swap(cur);
    }
  };
  const size_t parts = std::max<size_t>(1, std::min(host_threads(), (size_t)h * stride / (256u << 10)));
  run_threads(parts, [&](size_t k) { filter_rows((int)(h * k / parts), (int)(h * (k + 1) / parts)); });
  const std::vector<uint8_t> z = zlib_compress(raw.data(), raw.size());

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
