// The reference's image decoders, host side (rmn_image_load):
//
//  * PNG -- Material::loadImageFromPNG (src/material.cpp:217-285), libpng
//           with png_set_strip_16, png_set_expand_gray_1_2_4_to_8,
//           png_set_palette_to_rgb, png_set_gray_to_rgb and
//           png_set_strip_alpha: 8-bit RGB out.
//  * DDS -- scripts/dds_to_array.py (imageio's DDS reader) as
//           Material::loadImageFromDDS (src/material.cpp:190-215) consumes
//           it: BC1/BC2/BC3 (DXT1/3/5) blocks to RGBA, uncompressed 32-bit
//           to RGBA and 24-bit to RGB.
//  * HDR -- scripts/hdr_to_array.py (imageio's "HDR-FI" reader) as
//           SkyBox::load (src/component.cpp:69-114) consumes it: Radiance
//           RGBE to float32 RGB, flat or run-length-encoded scanlines.
//
// The library uses none of libpng, imageio and FreeImage. The formats are
// decoded from their published specifications: PNG (ISO/IEC 15948) with zlib
// and deflate (RFC 1950, RFC 1951); Radiance RGBE (G. Ward, "Real Pixels",
// Graphics Gems II, and the Radiance file format notes); the DirectDraw
// Surface header and the S3TC block formats (BC1-BC3) of the DirectX
// documentation. Every decoder reads the whole file into memory, checks each
// length against the bytes present and returns RMN_ERR_INVALID_ARGUMENT for
// a malformed file and RMN_ERR_UNSUPPORTED for a valid variant it does not
// decode.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "rmn_host.h"

namespace {

using rmn::fail;

// ---------------------------------------------------------------- inflate

// A little-endian 8-byte word as loaded, on either byte order.
inline uint64_t le64(uint64_t w) {
  const uint8_t* b = reinterpret_cast<const uint8_t*>(&w);
  uint64_t v = 0;
  for (int i = 7; i >= 0; --i) v = v << 8 | b[i];
  return v;
}

struct BitReader {
  const uint8_t* p;
  size_t n, pos = 0;
  uint64_t buf = 0;
  int cnt = 0;
  BitReader(const uint8_t* p_, size_t n_) : p(p_), n(n_) {}
  void fill() {
    if (pos + 8 <= n) {  // whole bytes that fit, from one unaligned 8-byte load
      uint64_t w;
      std::memcpy(&w, p + pos, 8);
      w = le64(w);
      const int take = (63 - cnt) >> 3;
      buf |= (w & ((1ull << (8 * take)) - 1)) << cnt;  // take <= 7
      pos += take;
      cnt += 8 * take;
      return;
    }
    while (cnt <= 56 && pos < n) {
      buf |= (uint64_t)p[pos++] << cnt;
      cnt += 8;
    }
  }
  uint32_t peek(int k) {  // zeros past the end
    if (cnt < k) fill();
    return (uint32_t)(buf & ((1ull << k) - 1));
  }
  bool skip(int k) {
    if (cnt < k) fill();
    if (cnt < k) return false;
    buf >>= k;
    cnt -= k;
    return true;
  }
  bool get(int k, uint32_t* v) {
    if (cnt < k) fill();
    if (cnt < k) return false;
    *v = (uint32_t)(buf & ((1ull << k) - 1));
    buf >>= k;
    cnt -= k;
    return true;
  }
  void byte_align() {
    const int r = cnt & 7;
    buf >>= r;
    cnt -= r;
  }
};

constexpr int kFastBits = 12;

// Canonical Huffman code (RFC 1951 section 3.2.2): per length the number of
// codes, the symbols ordered by (length, value), and a table that decodes
// codes of up to kFastBits bits in one look-up, indexed by the next
// kFastBits stream bits (codes are packed starting with their first bit in
// the least significant position, hence bit-reversed).
struct Huffman {
  int16_t count[16];
  int16_t symbol[320];
  uint16_t fast[1 << kFastBits];  // symbol << 4 | length; 0 = longer code
};

bool build_huffman(Huffman& h, const uint8_t* len, int n) {
  std::memset(h.count, 0, sizeof h.count);
  for (int i = 0; i < n; ++i) h.count[len[i]]++;
  h.count[0] = 0;
  int left = 1;
  for (int l = 1; l < 16; ++l) {
    left = (left << 1) - h.count[l];
    if (left < 0) return false;  // over-subscribed
  }
  int offs[16];
  offs[1] = 0;
  for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
  for (int i = 0; i < n; ++i)
    if (len[i]) h.symbol[offs[len[i]]++] = (int16_t)i;
  std::memset(h.fast, 0, sizeof h.fast);
  int code = 0, idx = 0;
  for (int l = 1; l <= kFastBits; ++l) {
    for (int k = 0; k < h.count[l]; ++k, ++code, ++idx) {
      uint32_t rev = 0;
      for (int b = 0; b < l; ++b) rev |= (uint32_t)((code >> b) & 1) << (l - 1 - b);
      for (uint32_t f = rev; f < (1u << kFastBits); f += 1u << l) h.fast[f] = (uint16_t)(h.symbol[idx] << 4 | l);
    }
    code <<= 1;
  }
  return true;
}

__attribute__((always_inline)) inline int decode_symbol(BitReader& br, const Huffman& h) {
  const uint16_t e = h.fast[br.peek(kFastBits)];
  if (e) return br.skip(e & 15) ? (e >> 4) : -1;
  int code = 0, first = 0, index = 0;  // a code longer than kFastBits: walk it bit by bit
  for (int l = 1; l < 16; ++l) {
    uint32_t bit;
    if (!br.get(1, &bit)) return -1;
    code |= (int)bit;
    const int c = h.count[l];
    if (code - c < first) return h.symbol[index + code - first];
    index += c;
    first = (first + c) << 1;
    code <<= 1;
  }
  return -1;
}

// RFC 1951 section 3.2.5.
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
const uint8_t kCodeLengthOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// A back-reference: dst[0, len) = the bytes d before each, dst[k] =
// dst[k - d] in order, with len <= room (the bytes left in the output).
// Writes may run up to 7 bytes past len while they stay within room: those
// bytes lie ahead of the output position and are written again before any
// back-reference can read them.
inline void copy_match(uint8_t* dst, size_t d, size_t len, size_t room) {
  const uint8_t* src = dst - d;
  if (d >= 8 && len + 7 <= room) {  // 8 bytes at a time: each read lies wholly before its write
    for (size_t k = 0; k < len; k += 8) {
      uint64_t v;
      std::memcpy(&v, src + k, 8);
      std::memcpy(dst + k, &v, 8);
    }
    return;
  }
  if (d < 8 && len > 16) {  // a short period: copy the pattern at doubling distances
    size_t done = 0, span = d;  // dst[-d, done) holds the pattern; span = done + d
    while (done < len) {
      const size_t n = span < len - done ? span : len - done;
      std::memcpy(dst + done, src, n);  // from dst - d, span (a multiple of d) before, no overlap
      done += n;
      span += n;
    }
    return;
  }
  for (size_t k = 0; k < len; ++k) dst[k] = src[k];
}

// How far an inflate has come, for a thread that consumes its output while
// it runs: out[0, ready) is final (a match copied 8 bytes at a time may
// write a few bytes past its end, never before it).
class InflateProgress {
 public:
  void publish(size_t ready) {
    {
      std::lock_guard<std::mutex> lk(m_);
      ready_ = ready;
    }
    cv_.notify_all();
  }
  void finish() {  // the producer stopped, finished or not
    {
      std::lock_guard<std::mutex> lk(m_);
      done_ = true;
    }
    cv_.notify_all();
  }
  // Waits until out[0, need) is final (true) or the producer stopped short of it (false).
  bool wait_for(size_t need) {
    std::unique_lock<std::mutex> lk(m_);
    cv_.wait(lk, [&] { return ready_ >= need || done_; });
    return ready_ >= need;
  }

 private:
  std::mutex m_;
  std::condition_variable cv_;
  size_t ready_ = 0;
  bool done_ = false;
};
constexpr size_t kPublishStep = 64 << 10;

// A deflate stream into out[0, cap); *produced = bytes written. Returns
// nullptr or a description of what is wrong with the stream. With `prog`,
// the output so far is published at least every 64 KiB of matches and at
// every block's end.
const char* inflate_stream(BitReader& br, uint8_t* out, size_t cap, size_t* produced,
                           InflateProgress* prog = nullptr) {
  size_t o = 0, next_pub = kPublishStep;
  Huffman lit, dist, lens;
  uint32_t final_block = 0;
  do {
    uint32_t hdr;
    if (!br.get(3, &hdr)) return "truncated deflate stream";
    final_block = hdr & 1;
    const uint32_t type = hdr >> 1;
    if (type == 0) {  // stored
      br.byte_align();
      uint32_t len, nlen;
      if (!br.get(16, &len) || !br.get(16, &nlen)) return "truncated deflate stream";
      if ((len ^ 0xffffu) != nlen) return "stored block length check failed";
      if (o + len > cap) return "more image data than the image holds";
      for (; len && br.cnt; --len) {  // bytes already in the bit buffer
        uint32_t b = 0;
        br.get(8, &b);
        out[o++] = (uint8_t)b;
      }
      if (br.pos + len > br.n) return "truncated deflate stream";
      std::memcpy(out + o, br.p + br.pos, len);
      o += len;
      br.pos += len;
      if (prog) prog->publish(o);
      continue;
    }
    if (type == 3) return "invalid deflate block type";
    if (type == 1) {  // fixed codes
      uint8_t l[320];
      for (int i = 0; i < 144; ++i) l[i] = 8;
      for (int i = 144; i < 256; ++i) l[i] = 9;
      for (int i = 256; i < 280; ++i) l[i] = 7;
      for (int i = 280; i < 288; ++i) l[i] = 8;
      build_huffman(lit, l, 288);
      for (int i = 0; i < 30; ++i) l[i] = 5;
      build_huffman(dist, l, 30);
    } else {  // dynamic codes
      uint32_t hlit, hdist, hclen;
      if (!br.get(5, &hlit) || !br.get(5, &hdist) || !br.get(4, &hclen)) return "truncated deflate stream";
      hlit += 257;
      hdist += 1;
      hclen += 4;
      if (hlit > 286 || hdist > 30) return "bad dynamic code counts";
      uint8_t cl[19] = {0};
      for (uint32_t i = 0; i < hclen; ++i) {
        uint32_t v;
        if (!br.get(3, &v)) return "truncated deflate stream";
        cl[kCodeLengthOrder[i]] = (uint8_t)v;
      }
      if (!build_huffman(lens, cl, 19)) return "bad code-length code";
      uint8_t l[320];
      uint32_t i = 0;
      while (i < hlit + hdist) {
        const int sym = decode_symbol(br, lens);
        if (sym < 0) return "bad code lengths";
        if (sym < 16) {
          l[i++] = (uint8_t)sym;
          continue;
        }
        uint32_t rep, extra;
        uint8_t val = 0;
        if (sym == 16) {
          if (i == 0) return "repeat of no code length";
          val = l[i - 1];
          if (!br.get(2, &extra)) return "truncated deflate stream";
          rep = 3 + extra;
        } else if (sym == 17) {
          if (!br.get(3, &extra)) return "truncated deflate stream";
          rep = 3 + extra;
        } else {
          if (!br.get(7, &extra)) return "truncated deflate stream";
          rep = 11 + extra;
        }
        if (i + rep > hlit + hdist) return "code lengths overrun";
        while (rep--) l[i++] = val;
      }
      if (l[256] == 0) return "no end-of-block code";
      if (!build_huffman(lit, l, (int)hlit) || !build_huffman(dist, l + hlit, (int)hdist))
        return "over-subscribed code";
    }
    for (;;) {
      int sym = decode_symbol(br, lit);
      if (sym < 0) return "bad literal/length code";
      if (sym < 256) {
        if (o >= cap) return "more image data than the image holds";
        out[o++] = (uint8_t)sym;
        continue;
      }
      if (sym == 256) break;
      sym -= 257;
      if (sym >= 29) return "bad length symbol";
      uint32_t e;
      if (!br.get(kLenExtra[sym], &e)) return "truncated deflate stream";
      const size_t len = kLenBase[sym] + e;
      const int ds = decode_symbol(br, dist);
      if (ds < 0 || ds >= 30) return "bad distance code";
      if (!br.get(kDistExtra[ds], &e)) return "truncated deflate stream";
      const size_t d = kDistBase[ds] + e;
      if (d > o) return "distance before the start of the data";
      if (o + len > cap) return "more image data than the image holds";
      copy_match(out + o, d, len, cap - o);
      o += len;
      if (prog && o >= next_pub) {
        prog->publish(o);
        next_pub = o + kPublishStep;
      }
    }
    if (prog) prog->publish(o);
  } while (!final_block);
  *produced = o;
  return nullptr;
}

// Adler-32 (RFC 1950 section 8.2). Over 16 bytes p[0..15] the sums advance
// as a += sum p[k], b += 16 a + sum (16 - k) p[k]: the same values the byte
// loop reaches, from sums that do not depend on one another.
uint32_t adler32(const uint8_t* p, size_t n, uint32_t start = 1) {
  uint32_t a = start & 0xffff, b = start >> 16;
  while (n) {
    const size_t m = n < 5552 ? n : 5552;  // largest run without overflow of b
    size_t i = 0;
    for (; i + 16 <= m; i += 16) {
      uint32_t s1 = 0, s2 = 0;
      for (int k = 0; k < 16; ++k) {
        s1 += p[i + k];
        s2 += (uint32_t)(16 - k) * p[i + k];
      }
      b += 16 * a + s2;
      a += s1;
    }
    for (; i < m; ++i) {
      a += p[i];
      b += a;
    }
    a %= 65521;
    b %= 65521;
    p += m;
    n -= m;
  }
  return b << 16 | a;
}

// The zlib stream's header and deflate data into out[0, want) (sized by the
// caller), and its Adler-32 field into *check: everything but the checksum
// comparison.
const char* zlib_inflate_only(const uint8_t* p, size_t n, uint8_t* out, size_t want, uint32_t* check,
                              InflateProgress* prog) {
  if (n < 2) return "truncated zlib stream";
  if ((p[0] & 15) != 8 || (p[0] >> 4) > 7 || ((unsigned)p[0] << 8 | p[1]) % 31 != 0) return "bad zlib header";
  if (p[1] & 0x20) return "zlib preset dictionary";
  BitReader br(p + 2, n - 2);
  size_t got = 0;
  if (const char* err = inflate_stream(br, out, want, &got, prog)) return err;
  if (got != want) return "less image data than the image holds";
  br.byte_align();
  *check = 0;
  for (int i = 0; i < 4; ++i) {
    uint32_t b;
    if (!br.get(8, &b)) return "truncated zlib checksum";
    *check = *check << 8 | b;
  }
  return nullptr;
}

// A zlib stream (RFC 1950) that must inflate to exactly `want` bytes.
const char* zlib_decompress(const uint8_t* p, size_t n, std::vector<uint8_t>& out, size_t want) {
  out.assign(want, 0);
  uint32_t check = 0;
  if (const char* err = zlib_inflate_only(p, n, out.data(), want, &check, nullptr)) return err;
  if (check != adler32(out.data(), out.size())) return "zlib checksum mismatch";
  return nullptr;
}

// ---------------------------------------------------------------- deflate

struct BitWriter {
  std::vector<uint8_t>& out;
  uint64_t buf = 0;
  int cnt = 0;
  explicit BitWriter(std::vector<uint8_t>& o) : out(o) {}
  void put(uint32_t bits, int n) {  // n <= 32, first bit in the least significant position
    buf |= (uint64_t)bits << cnt;
    cnt += n;
    while (cnt >= 8) {
      out.push_back((uint8_t)buf);
      buf >>= 8;
      cnt -= 8;
    }
  }
  void flush() {
    if (cnt > 0) out.push_back((uint8_t)buf);
    buf = 0;
    cnt = 0;
  }
};

// Huffman code lengths for the frequencies, at most max_len bits: the
// optimal tree (two lightest nodes merged first, ties to the lower index);
// while it is too deep, the frequencies are halved (kept >= 1) and the tree
// rebuilt. A single used symbol gets length 1.
void huffman_lengths(const uint32_t* freq, int n, int max_len, uint8_t* len) {
  std::vector<uint32_t> f(freq, freq + n);
  for (;;) {
    std::fill(len, len + n, 0);
    std::vector<std::pair<uint64_t, int>> heap;  // (weight, node), a min-heap
    std::vector<int> parent;
    for (int i = 0; i < n; ++i)
      if (f[i]) {
        heap.push_back({((uint64_t)f[i] << 20) | (uint64_t)parent.size(), (int)parent.size()});
        parent.push_back(-1);
      }
    if (parent.empty()) return;
    if (parent.size() == 1) {
      for (int i = 0; i < n; ++i)
        if (f[i]) len[i] = 1;
      return;
    }
    auto cmp = [](const std::pair<uint64_t, int>& a, const std::pair<uint64_t, int>& b) { return a.first > b.first; };
    std::make_heap(heap.begin(), heap.end(), cmp);
    while (heap.size() > 1) {
      std::pop_heap(heap.begin(), heap.end(), cmp);
      const auto a = heap.back();
      heap.pop_back();
      std::pop_heap(heap.begin(), heap.end(), cmp);
      const auto b = heap.back();
      heap.pop_back();
      const int node = (int)parent.size();
      parent.push_back(-1);
      parent[a.second] = parent[b.second] = node;
      const uint64_t w = ((a.first >> 20) + (b.first >> 20)) << 20 | (uint64_t)node;
      heap.push_back({w, node});
      std::push_heap(heap.begin(), heap.end(), cmp);
    }
    int leaf = 0, deepest = 0;
    for (int i = 0; i < n; ++i) {
      if (!f[i]) continue;
      int d = 0;
      for (int v = leaf; parent[v] >= 0; v = parent[v]) ++d;
      len[i] = (uint8_t)std::min(d, 255);
      deepest = std::max(deepest, d);
      ++leaf;
    }
    if (deepest <= max_len) return;
    for (int i = 0; i < n; ++i)
      if (f[i]) f[i] = (f[i] + 1) >> 1;
  }
}

// Canonical codes of the lengths (RFC 1951 section 3.2.2), bit-reversed for
// writing first bit first.
void canonical_codes(const uint8_t* len, int n, uint32_t* code) {
  int count[16] = {0};
  for (int i = 0; i < n; ++i) count[len[i]]++;
  count[0] = 0;
  uint32_t next[16] = {0};
  uint32_t c = 0;
  for (int l = 1; l < 16; ++l) {
    c = (c + count[l - 1]) << 1;
    next[l] = c;
  }
  for (int i = 0; i < n; ++i) {
    if (!len[i]) continue;
    uint32_t v = next[len[i]]++, r = 0;
    for (int b = 0; b < len[i]; ++b) r |= ((v >> b) & 1u) << (len[i] - 1 - b);
    code[i] = r;
  }
}

struct Symbol {
  uint16_t litlen;  // literal byte, or match length 3..258
  uint16_t dist;    // 0: literal
};

// Length 3..258 -> symbol 257..285 and distance 1..32768 -> code 0..29,
// from tables built once (distances above 256 by (d - 1) >> 7).
struct CodeTables {
  uint16_t len_sym[259];
  uint8_t dist_lo[257], dist_hi[256];
  CodeTables() {
    for (int l = 3; l <= 258; ++l) {
      int s = 28;
      while (kLenBase[s] > l) --s;
      len_sym[l] = (uint16_t)(257 + s);
    }
    auto slow = [](int d) {
      int s = 29;
      while (kDistBase[s] > d) --s;
      return s;
    };
    for (int d = 1; d <= 256; ++d) dist_lo[d] = (uint8_t)slow(d);
    for (int q = 2; q < 256; ++q) dist_hi[q] = (uint8_t)slow((q << 7) + 1);
  }
};
const CodeTables& code_tables() {
  static const CodeTables t;  // initialised once, thread-safe
  return t;
}
int length_symbol(int len) { return code_tables().len_sym[len]; }
int distance_symbol(int d) { return d <= 256 ? code_tables().dist_lo[d] : code_tables().dist_hi[(d - 1) >> 7]; }

// One dynamic-Huffman block of symbols.
void write_block(BitWriter& bw, const std::vector<Symbol>& sy, bool last) {
  uint32_t lf[286] = {0}, df[30] = {0};
  for (const Symbol& s : sy) {
    if (!s.dist) {
      lf[s.litlen]++;
    } else {
      lf[length_symbol(s.litlen)]++;
      df[distance_symbol(s.dist)]++;
    }
  }
  lf[256] = 1;
  bool any_dist = false;
  for (uint32_t x : df) any_dist = any_dist || x;
  if (!any_dist) df[0] = 1;  // one distance code of one bit
  uint8_t ll[286], dl[30];
  huffman_lengths(lf, 286, 15, ll);
  huffman_lengths(df, 30, 15, dl);
  int hlit = 286, hdist = 30;
  while (hlit > 257 && !ll[hlit - 1]) --hlit;
  while (hdist > 1 && !dl[hdist - 1]) --hdist;
  // the code lengths, run-length coded with 16 / 17 / 18
  std::vector<uint8_t> lens(ll, ll + hlit);
  lens.insert(lens.end(), dl, dl + hdist);
  std::vector<std::pair<uint8_t, uint8_t>> rle;  // (symbol, extra value)
  for (size_t i = 0; i < lens.size();) {
    size_t j = i;
    while (j < lens.size() && lens[j] == lens[i]) ++j;
    size_t run = j - i;
    if (lens[i] == 0) {
      while (run >= 11) {
        const size_t k = std::min<size_t>(run, 138);
        rle.push_back({18, (uint8_t)(k - 11)});
        run -= k;
      }
      if (run >= 3) {
        rle.push_back({17, (uint8_t)(run - 3)});
        run = 0;
      }
    } else {
      rle.push_back({lens[i], 0});
      --run;
      while (run >= 3) {
        const size_t k = std::min<size_t>(run, 6);
        rle.push_back({16, (uint8_t)(k - 3)});
        run -= k;
      }
    }
    while (run--) rle.push_back({lens[i], 0});
    i = j;
  }
  uint32_t cf[19] = {0};
  for (const auto& r : rle) cf[r.first]++;
  uint8_t cl[19];
  huffman_lengths(cf, 19, 7, cl);
  int hclen = 19;
  while (hclen > 4 && !cl[kCodeLengthOrder[hclen - 1]]) --hclen;
  uint32_t ccode[19] = {0}, lcode[286] = {0}, dcode[30] = {0};
  canonical_codes(cl, 19, ccode);
  canonical_codes(ll, 286, lcode);
  canonical_codes(dl, 30, dcode);

  bw.put(last ? 1 : 0, 1);
  bw.put(2, 2);
  bw.put((uint32_t)(hlit - 257), 5);
  bw.put((uint32_t)(hdist - 1), 5);
  bw.put((uint32_t)(hclen - 4), 4);
  for (int i = 0; i < hclen; ++i) bw.put(cl[kCodeLengthOrder[i]], 3);
  for (const auto& r : rle) {
    bw.put(ccode[r.first], cl[r.first]);
    if (r.first == 16) bw.put(r.second, 2);
    if (r.first == 17) bw.put(r.second, 3);
    if (r.first == 18) bw.put(r.second, 7);
  }
  for (const Symbol& s : sy) {
    if (!s.dist) {
      bw.put(lcode[s.litlen], ll[s.litlen]);
      continue;
    }
    const int ls = length_symbol(s.litlen) - 257;
    bw.put(lcode[257 + ls], ll[257 + ls]);
    bw.put((uint32_t)(s.litlen - kLenBase[ls]), kLenExtra[ls]);
    const int ds = distance_symbol(s.dist);
    bw.put(dcode[ds], dl[ds]);
    bw.put((uint32_t)(s.dist - kDistBase[ds]), kDistExtra[ds]);
  }
  bw.put(lcode[256], ll[256]);
}

// ---------------------------------------------------------------- PNG

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }
uint32_t le32(const uint8_t* p) { return (uint32_t)p[3] << 24 | (uint32_t)p[2] << 16 | (uint32_t)p[1] << 8 | p[0]; }

// The Paeth predictor: of a, b, c the one closest to p = a + b - c, ties
// resolved in the order a, b, c; written with selects instead of branches.
inline int paeth(int a, int b, int c) {
  const int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
  const int bc = pc < pb ? c : b;
  const int mbc = pc < pb ? pc : pb;
  return mbc < pa ? bc : a;
}

// unfilter_row for B bytes per pixel and a row of whole pixels (n a multiple
// of B): the left (a) and upper-left (c) bytes of the B channels stay in
// registers from one pixel to the next instead of being read back from the
// row just written.
template <int B>
void unfilter_pixels(int ft, const uint8_t* src, const uint8_t* up, uint8_t* out, size_t n) {
  int a[B], c[B];
  for (int j = 0; j < B; ++j) {  // the first pixel: a = c = 0
    const int v = ft == 2 || ft == 4 ? up[j] : ft == 3 ? up[j] >> 1 : 0;
    a[j] = out[j] = (uint8_t)(src[j] + v);
    c[j] = up[j];
  }
  switch (ft) {
    case 1:
      for (size_t i = B; i < n; i += B)
#pragma GCC unroll 4
        for (int j = 0; j < B; ++j) a[j] = out[i + j] = (uint8_t)(src[i + j] + a[j]);
      break;
    case 3:
      for (size_t i = B; i < n; i += B)
#pragma GCC unroll 4
        for (int j = 0; j < B; ++j) a[j] = out[i + j] = (uint8_t)(src[i + j] + ((a[j] + up[i + j]) >> 1));
      break;
    case 4:
      for (size_t i = B; i < n; i += B)
#pragma GCC unroll 4
        for (int j = 0; j < B; ++j) {
          const int b = up[i + j];
          a[j] = out[i + j] = (uint8_t)(src[i + j] + paeth(a[j], b, c[j]));
          c[j] = b;
        }
      break;
  }
}

// One scanline's filter undone (ISO/IEC 15948 section 9): each byte plus the
// predictor from the left (a), upper (b) and upper-left (c) reconstructed
// bytes; bpp = bytes per complete pixel, at least 1.
void unfilter_row(int ft, const uint8_t* src, const uint8_t* up, uint8_t* out, size_t n, int bpp) {
  if ((ft == 1 || ft == 3 || ft == 4) && n >= (size_t)bpp && n % bpp == 0) {
    if (bpp == 3) return unfilter_pixels<3>(ft, src, up, out, n);
    if (bpp == 4) return unfilter_pixels<4>(ft, src, up, out, n);
  }
  const size_t k = (size_t)bpp < n ? (size_t)bpp : n;
  switch (ft) {
    case 0:
      std::memcpy(out, src, n);
      break;
    case 1:
      std::memcpy(out, src, k);
      for (size_t i = k; i < n; ++i) out[i] = (uint8_t)(src[i] + out[i - bpp]);
      break;
    case 2:
      for (size_t i = 0; i < n; ++i) out[i] = (uint8_t)(src[i] + up[i]);
      break;
    case 3:
      for (size_t i = 0; i < k; ++i) out[i] = (uint8_t)(src[i] + (up[i] >> 1));
      for (size_t i = k; i < n; ++i) out[i] = (uint8_t)(src[i] + ((out[i - bpp] + up[i]) >> 1));
      break;
    default:
      for (size_t i = 0; i < k; ++i) out[i] = (uint8_t)(src[i] + up[i]);  // Paeth with a = c = 0 picks b
      for (size_t i = k; i < n; ++i) out[i] = (uint8_t)(src[i] + paeth(out[i - bpp], up[i], up[i - bpp]));
      break;
  }
}

using Decoded = rmn::DecodedImage;

rmn_status decode_png(const std::vector<uint8_t>& f, bool header_only, Decoded& img) {
  static const uint8_t kSig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  if (f.size() < 8 || std::memcmp(f.data(), kSig, 8) != 0) return fail(RMN_ERR_INVALID_ARGUMENT, "not a PNG file");
  size_t at = 8;
  bool have_ihdr = false;
  uint32_t w = 0, h = 0;
  int depth = 0, ctype = 0, interlace = 0;
  std::vector<uint8_t> palette, idat;
  for (;;) {
    if (at + 12 > f.size()) return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: truncated chunk");
    const uint32_t len = be32(&f[at]);
    if (len > f.size() - at - 12) return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: truncated chunk");
    const uint8_t* type = &f[at + 4];
    const uint8_t* data = &f[at + 8];
    const bool critical = !(type[0] & 0x20);
    if (critical && be32(data + len) != rmn::png_crc32(0, type, len + 4))
      return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: CRC error in a %.4s chunk", (const char*)type);
    at += 12 + len;
    if (!have_ihdr && std::memcmp(type, "IHDR", 4) != 0) return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: IHDR not first");
    if (std::memcmp(type, "IHDR", 4) == 0) {
      if (len != 13 || have_ihdr) return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: bad IHDR");
      have_ihdr = true;
      w = be32(data);
      h = be32(data + 4);
      depth = data[8];
      ctype = data[9];
      interlace = data[12];
      const bool ok_depth = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                            (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                            ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
      if (!ok_depth || data[10] != 0 || data[11] != 0 || interlace > 1)
        return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: bad IHDR (color type %d, bit depth %d)", ctype, depth);
      if (w == 0 || h == 0 || w > (1u << 30) || h > (1u << 30) || (uint64_t)w * h > (1ull << 30))
        return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: image size %ux%u out of range", w, h);
      if (header_only) break;
    } else if (std::memcmp(type, "PLTE", 4) == 0) {
      if (len % 3 || len > 768) return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: bad PLTE");
      palette.assign(data, data + len);
    } else if (std::memcmp(type, "IDAT", 4) == 0) {
      idat.insert(idat.end(), data, data + len);
    } else if (std::memcmp(type, "IEND", 4) == 0) {
      break;
    } else if (critical) {
      return fail(RMN_ERR_UNSUPPORTED, "PNG: unknown critical chunk %.4s", (const char*)type);
    }
  }
  img.w = (int)w;
  img.h = (int)h;
  img.channels = 3;
  img.bytes_per_channel = 1;
  if (header_only) return RMN_OK;
  if (ctype == 3 && palette.empty()) return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: palette image without PLTE");

  static const int kChannels[7] = {1, 0, 3, 1, 2, 0, 4};
  const int nch = kChannels[ctype];
  const int bits = nch * depth;       // per pixel
  const int bpp = bits < 8 ? 1 : bits / 8;  // filter unit
  struct Pass { int x0, y0, dx, dy; };
  static const Pass kAdam7[7] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                 {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
  static const Pass kPlain[1] = {{0, 0, 1, 1}};
  const Pass* passes = interlace ? kAdam7 : kPlain;
  const int npass = interlace ? 7 : 1;
  size_t want = 0;
  for (int k = 0; k < npass; ++k) {
    if (passes[k].x0 >= (int)w || passes[k].y0 >= (int)h) continue;  // an empty pass has no rows
    const size_t cols = (w - passes[k].x0 + passes[k].dx - 1) / passes[k].dx;
    const size_t rows = (h - passes[k].y0 + passes[k].dy - 1) / passes[k].dy;
    want += rows * (1 + (cols * bits + 7) / 8);
  }
  img.bytes.assign((size_t)w * h * 3, 0);
  const int maxv = (1 << depth) - 1;
  const int gray_scale = depth < 8 ? 255 / maxv : 1;  // png_set_expand_gray_1_2_4_to_8
  std::vector<uint8_t> raw(want);
  // The scanlines, in stream order: each waits (with `prog`) until the
  // inflate has produced it, and the Adler-32 of the bytes taken so far is
  // kept in *adler / *taken. Returns -1, or the first row's filter type
  // byte that is not one.
  auto unfilter_all = [&](InflateProgress* prog, uint32_t* adler, size_t* taken) -> int {
    size_t at_raw = 0;
    std::vector<uint8_t> prev, cur;
    for (int k = 0; k < npass; ++k) {
      const Pass& ps = passes[k];
      if (ps.x0 >= (int)w || ps.y0 >= (int)h) continue;
      const size_t cols = (w - ps.x0 + ps.dx - 1) / ps.dx;
      const size_t rows = (h - ps.y0 + ps.dy - 1) / ps.dy;
      const size_t stride = (cols * bits + 7) / 8;
      prev.assign(stride, 0);
      cur.assign(stride, 0);
      for (size_t r = 0; r < rows; ++r) {
        if (prog && !prog->wait_for(at_raw + 1 + stride)) return -1;  // the inflate stopped short
        const uint8_t ft = raw[at_raw];
        const uint8_t* src = &raw[at_raw + 1];
        *adler = adler32(&raw[at_raw], 1 + stride, *adler);
        at_raw += 1 + stride;
        *taken = at_raw;
        if (ft > 4) return ft;
        const size_t y = ps.y0 + r * ps.dy;
        uint8_t* px = &img.bytes[(y * w + ps.x0) * 3];
        if (depth == 8 && ctype == 2 && !interlace) {  // the image's own rows are the scanlines
          unfilter_row(ft, src, r ? px - stride : prev.data(), px, stride, bpp);
          continue;
        }
        unfilter_row(ft, src, prev.data(), cur.data(), stride, bpp);
        // samples of this row to 8-bit RGB
        const size_t step = 3 * (size_t)ps.dx;
        const uint8_t* q = cur.data();
        if (depth == 8 && ctype == 2 && ps.dx == 1) {
          std::memcpy(px, q, cols * 3);
        } else if (depth == 8 && (ctype == 2 || ctype == 6)) {
          for (size_t i = 0; i < cols; ++i, px += step, q += nch) px[0] = q[0], px[1] = q[1], px[2] = q[2];
        } else if (depth == 16 && (ctype == 2 || ctype == 6)) {  // png_set_strip_16: the high byte
          for (size_t i = 0; i < cols; ++i, px += step, q += 2 * nch) px[0] = q[0], px[1] = q[2], px[2] = q[4];
        } else if (depth >= 8 && (ctype == 0 || ctype == 4)) {
          const size_t adv = (size_t)nch * (depth / 8);
          for (size_t i = 0; i < cols; ++i, px += step, q += adv) px[0] = px[1] = px[2] = q[0];
        } else {  // 1/2/4/8-bit gray or palette indices
          for (size_t i = 0; i < cols; ++i, px += step) {
            const size_t bit = i * depth;
            const int v = depth == 8 ? q[i] : (q[bit >> 3] >> (8 - depth - (bit & 7))) & maxv;
            if (ctype == 0) {
              px[0] = px[1] = px[2] = (uint8_t)(v * gray_scale);
            } else if ((size_t)v * 3 + 2 < palette.size()) {
              px[0] = palette[v * 3];
              px[1] = palette[v * 3 + 1];
              px[2] = palette[v * 3 + 2];
            }  // an index past the palette stays black
          }
        }
        std::swap(prev, cur);
      }
    }
    return -1;
  };
  // From 1 MiB of scanline data on, the rows are unfiltered on a second
  // thread while the stream inflates. A defect is reported as a reader that
  // inflated everything first would: the stream's (its checksum included)
  // before a row's.
  uint32_t check = 0, adler = 1;
  size_t taken = 0;
  const char* zerr = nullptr;
  int bad_ft = -1;
  bool piped = false;
  if (want >= (1u << 20)) {
    InflateProgress prog;
    std::exception_ptr rexc;
    std::thread rows;
    try {
      rows = std::thread([&] {
        try {
          bad_ft = unfilter_all(&prog, &adler, &taken);
        } catch (...) {
          rexc = std::current_exception();
        }
      });
      piped = true;
    } catch (const std::system_error&) {  // no thread: one after the other below
    }
    if (piped) {
      try {
        zerr = zlib_inflate_only(idat.data(), idat.size(), raw.data(), want, &check, &prog);
      } catch (...) {
        prog.finish();
        rows.join();
        throw;
      }
      prog.finish();
      rows.join();
      if (rexc) std::rethrow_exception(rexc);
    }
  }
  if (!piped) {
    zerr = zlib_inflate_only(idat.data(), idat.size(), raw.data(), want, &check, nullptr);
    if (!zerr) bad_ft = unfilter_all(nullptr, &adler, &taken);
  }
  if (zerr) return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: %s", zerr);
  if (taken < want) adler = adler32(raw.data() + taken, want - taken, adler);  // rows stopped at a defect
  if (adler != check) return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: zlib checksum mismatch");
  if (bad_ft >= 0) return fail(RMN_ERR_INVALID_ARGUMENT, "PNG: bad filter type %d", bad_ft);
  return RMN_OK;
}

// ---------------------------------------------------------------- Radiance HDR

rmn_status decode_hdr(const std::vector<uint8_t>& f, bool header_only, Decoded& img) {
  size_t at = 0;
  auto line = [&](std::string& s) {  // one header line, without its "\n" (or "\r\n")
    s.clear();
    while (at < f.size() && f[at] != '\n') s.push_back((char)f[at++]);
    if (at >= f.size()) return false;
    ++at;
    if (!s.empty() && s.back() == '\r') s.pop_back();
    return true;
  };
  std::string s;
  if (!line(s) || s.size() < 2 || s[0] != '#' || s[1] != '?') return fail(RMN_ERR_INVALID_ARGUMENT, "not a Radiance HDR file");
  for (;;) {  // header lines up to the empty line
    if (!line(s)) return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: truncated header");
    if (s.empty()) break;
    if (s.compare(0, 7, "FORMAT=") == 0 && s != "FORMAT=32-bit_rle_rgbe")
      return fail(RMN_ERR_UNSUPPORTED, "HDR: %s (only 32-bit_rle_rgbe)", s.c_str());
  }
  if (!line(s)) return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: no resolution line");
  int h = 0, w = 0;
  char tail = 0;
  if (std::sscanf(s.c_str(), "-Y %d +X %d%c", &h, &w, &tail) != 2)
    return fail(RMN_ERR_UNSUPPORTED, "HDR: resolution line \"%s\" (only -Y H +X W)", s.c_str());
  if (w <= 0 || h <= 0 || (int64_t)w * h > (1LL << 30)) return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: bad image size");
  img.w = w;
  img.h = h;
  img.channels = 3;
  img.bytes_per_channel = 4;
  if (header_only) return RMN_OK;

  const size_t npx = (size_t)w * h;
  std::vector<uint8_t> rgbe(npx * 4);
  auto take = [&](uint8_t* dst, size_t n) {
    if (f.size() - at < n) return false;
    std::memcpy(dst, &f[at], n);
    at += n;
    return true;
  };
  if (w < 8 || w > 0x7fff) {  // too narrow or too wide for run-length encoding: flat pixels
    if (!take(rgbe.data(), npx * 4)) return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: truncated pixel data");
  } else {
    for (int y = 0; y < h; ++y) {
      uint8_t* row = &rgbe[(size_t)y * w * 4];
      if (f.size() - at < 4) return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: truncated pixel data");
      const uint8_t* q = &f[at];
      if (q[0] != 2 || q[1] != 2 || (q[2] & 0x80)) {  // not run-length encoded: flat from here on
        if (!take(row, npx * 4 - (size_t)y * w * 4)) return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: truncated pixel data");
        break;
      }
      if (((int)q[2] << 8 | q[3]) != w) return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: wrong scanline width");
      at += 4;
      for (int ch = 0; ch < 4; ++ch) {  // each component of the scanline in turn
        int x = 0;
        while (x < w) {
          if (at >= f.size()) return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: truncated pixel data");
          int count = f[at++];
          if (count > 128) {  // a run of one byte
            count -= 128;
            if (count > w - x || at >= f.size()) return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: bad scanline data");
            const uint8_t v = f[at++];
            for (int k = 0; k < count; ++k) row[(x++) * 4 + ch] = v;
          } else {  // literal bytes
            if (count == 0 || count > w - x || f.size() - at < (size_t)count)
              return fail(RMN_ERR_INVALID_ARGUMENT, "HDR: bad scanline data");
            for (int k = 0; k < count; ++k) row[(x++) * 4 + ch] = f[at++];
          }
        }
      }
    }
  }
  img.bytes.resize(npx * 3 * sizeof(float));
  float* out = reinterpret_cast<float*>(img.bytes.data());
  float scales[256];  // RGBE: mantissas m scaled by 2^(e - 128 - 8); exponent 0 is black
  scales[0] = 0.0f;
  for (int e = 1; e < 256; ++e) scales[e] = (float)std::ldexp(1.0, e - 136);
  for (size_t i = 0; i < npx; ++i) {
    const uint8_t* p = &rgbe[i * 4];
    const float scale = scales[p[3]];
    out[i * 3 + 0] = p[0] * scale;
    out[i * 3 + 1] = p[1] * scale;
    out[i * 3 + 2] = p[2] * scale;
  }
  return RMN_OK;
}

// ---------------------------------------------------------------- DDS

void expand565(uint32_t c, uint8_t* rgb) {
  const uint32_t r = c >> 11 & 31, g = c >> 5 & 63, b = c & 31;
  rgb[0] = (uint8_t)(r << 3 | r >> 2);  // bit replication to 8 bits
  rgb[1] = (uint8_t)(g << 2 | g >> 4);
  rgb[2] = (uint8_t)(b << 3 | b >> 2);
}

// One 4x4 colour block (BC1 layout) into 16 RGBA texels. BC1 blocks with
// color0 <= color1 have three colours and transparent black; BC2/BC3 colour
// blocks always have four. Interpolated channels: (2 a + b) / 3 and
// (a + b) / 2, truncated.
void color_block(const uint8_t* blk, bool bc1, uint8_t texel[16][4]) {
  const uint32_t c0 = blk[0] | (uint32_t)blk[1] << 8, c1 = blk[2] | (uint32_t)blk[3] << 8;
  uint8_t pal[4][4];
  expand565(c0, pal[0]);
  expand565(c1, pal[1]);
  pal[0][3] = pal[1][3] = pal[2][3] = pal[3][3] = 255;
  if (!bc1 || c0 > c1) {
    for (int ch = 0; ch < 3; ++ch) {
      pal[2][ch] = (uint8_t)((2 * pal[0][ch] + pal[1][ch]) / 3);
      pal[3][ch] = (uint8_t)((pal[0][ch] + 2 * pal[1][ch]) / 3);
    }
  } else {
    for (int ch = 0; ch < 3; ++ch) {
      pal[2][ch] = (uint8_t)((pal[0][ch] + pal[1][ch]) / 2);
      pal[3][ch] = 0;
    }
    pal[3][3] = 0;
  }
  const uint32_t idx = le32(blk + 4);
  for (int t = 0; t < 16; ++t) std::memcpy(texel[t], pal[idx >> (2 * t) & 3], 4);
}

rmn_status decode_dds(const std::vector<uint8_t>& f, bool header_only, Decoded& img) {
  if (f.size() < 128 || std::memcmp(f.data(), "DDS ", 4) != 0 || le32(&f[4]) != 124)
    return fail(RMN_ERR_INVALID_ARGUMENT, "not a DDS file");
  const uint32_t h = le32(&f[12]), w = le32(&f[16]);
  const uint32_t pf_flags = le32(&f[80]);
  const uint8_t* fourcc = &f[84];
  const uint32_t bitcount = le32(&f[88]);
  const uint32_t mask[4] = {le32(&f[92]), le32(&f[96]), le32(&f[100]), le32(&f[104])};
  if (w == 0 || h == 0 || (uint64_t)w * h > (1ull << 30)) return fail(RMN_ERR_INVALID_ARGUMENT, "DDS: bad image size");
  int block = 0;  // bytes per 4x4 block; 0 = uncompressed
  int kind = 0;   // 1, 2, 3 = BC1, BC2, BC3
  if (pf_flags & 0x4) {  // DDPF_FOURCC
    if (std::memcmp(fourcc, "DXT1", 4) == 0) block = 8, kind = 1;
    else if (std::memcmp(fourcc, "DXT3", 4) == 0) block = 16, kind = 2;
    else if (std::memcmp(fourcc, "DXT5", 4) == 0) block = 16, kind = 3;
    else return fail(RMN_ERR_UNSUPPORTED, "DDS: pixel format %.4s (BC1-BC3 and 24/32-bit RGB only)", (const char*)fourcc);
  } else if (!(pf_flags & 0x40) || (bitcount != 24 && bitcount != 32)) {  // DDPF_RGB
    return fail(RMN_ERR_UNSUPPORTED, "DDS: %u-bit pixel format (BC1-BC3 and 24/32-bit RGB only)", bitcount);
  }
  const bool alpha = block || (pf_flags & 0x1);  // DDPF_ALPHAPIXELS
  img.w = (int)w;
  img.h = (int)h;
  img.channels = (block || bitcount == 32) ? 4 : 3;
  img.bytes_per_channel = 1;
  if (header_only) return RMN_OK;

  const uint8_t* data = f.data() + 128;
  const size_t avail = f.size() - 128;
  img.bytes.assign((size_t)w * h * img.channels, 0);
  if (block) {
    const size_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    if (bw * bh * block > avail) return fail(RMN_ERR_INVALID_ARGUMENT, "DDS: truncated block data");
    // rows of blocks in ranges on separate threads: each writes its own pixel rows
    const size_t parts = std::max<size_t>(1, std::min(rmn::host_threads(), bw * bh / 16384));
    rmn::run_threads(parts, [&](size_t part) {
      uint8_t tex[16][4];
      for (size_t by = bh * part / parts; by < bh * (part + 1) / parts; ++by)
        for (size_t bx = 0; bx < bw; ++bx) {
          const uint8_t* blk = data + (by * bw + bx) * block;
          color_block(kind == 1 ? blk : blk + 8, kind == 1, tex);
          if (kind == 2) {  // explicit 4-bit alpha, expanded by 17
            for (int t = 0; t < 16; ++t) tex[t][3] = (uint8_t)(((blk[t >> 1] >> (4 * (t & 1))) & 15) * 17);
          } else if (kind == 3) {  // interpolated alpha
            const int a0 = blk[0], a1 = blk[1];
            int pal[8] = {a0, a1};
            if (a0 > a1) {
              for (int k = 2; k < 8; ++k) pal[k] = ((8 - k) * a0 + (k - 1) * a1) / 7;
            } else {
              for (int k = 2; k < 6; ++k) pal[k] = ((6 - k) * a0 + (k - 1) * a1) / 5;
              pal[6] = 0;
              pal[7] = 255;
            }
            uint64_t bits = 0;
            for (int k = 0; k < 6; ++k) bits |= (uint64_t)blk[2 + k] << (8 * k);
            for (int t = 0; t < 16; ++t) tex[t][3] = (uint8_t)pal[bits >> (3 * t) & 7];
          }
          for (int t = 0; t < 16; ++t) {
            const size_t x = bx * 4 + (t & 3), y = by * 4 + (t >> 2);
            if (x < w && y < h) std::memcpy(&img.bytes[(y * w + x) * 4], tex[t], 4);
          }
        }
    });
    return RMN_OK;
  }
  const size_t px_bytes = bitcount / 8, pitch = (size_t)w * px_bytes;
  if (pitch * h > avail) return fail(RMN_ERR_INVALID_ARGUMENT, "DDS: truncated pixel data");
  int shift[4], width_bits[4];
  for (int c = 0; c < 4; ++c) {
    uint32_t m = mask[c];
    shift[c] = 0;
    width_bits[c] = 0;
    if (!m) continue;
    while (!(m & 1)) m >>= 1, shift[c]++;
    while (m & 1) m >>= 1, width_bits[c]++;
    if (m || width_bits[c] != 8) return fail(RMN_ERR_UNSUPPORTED, "DDS: channel masks other than 8 contiguous bits");
  }
  if (!mask[0] || !mask[1] || !mask[2]) return fail(RMN_ERR_UNSUPPORTED, "DDS: RGB pixel format without RGB masks");
  for (size_t i = 0; i < (size_t)w * h; ++i) {
    const uint8_t* p = data + i * px_bytes;
    const uint32_t v = px_bytes == 4 ? le32(p) : (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16;
    uint8_t* o = &img.bytes[i * img.channels];
    for (int c = 0; c < 3; ++c) o[c] = (uint8_t)(v >> shift[c]);
    if (img.channels == 4) o[3] = (alpha && mask[3]) ? (uint8_t)(v >> shift[3]) : 255;
  }
  return RMN_OK;
}

// The size first (one allocation, one read), then whatever follows it: a
// file whose size cannot be taken, or that grew meanwhile, is read to its end.
template <class Buf>
bool read_into(const char* path, Buf& out) {
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return false;
  out.clear();
  long size = -1;
  if (std::fseek(fp, 0, SEEK_END) == 0) {
    const long at_end = std::ftell(fp);
    if (std::fseek(fp, 0, SEEK_SET) != 0) {
      std::fclose(fp);
      return false;
    }
    size = at_end;
  }
  if (size > 0) {
    out.resize((size_t)size);
    out.resize(std::fread(&out[0], 1, (size_t)size, fp));
  }
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, fp)) > 0) out.insert(out.end(), buf, buf + n);
  const bool ok = !std::ferror(fp);
  std::fclose(fp);
  return ok;
}

bool read_file(const char* path, std::vector<uint8_t>& out) { return read_into(path, out); }

}  // namespace

namespace rmn {

bool read_whole_file(const char* path, std::vector<uint8_t>& out) { return read_into(path, out); }
bool read_whole_file(const char* path, std::string& out) { return read_into(path, out); }

const char* zlib_inflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out, size_t want) {
  return zlib_decompress(p, n, out, want);
}

// zlib stream (RFC 1950) of `data`: greedy LZ77 over a 32 KiB window (hash
// chains on 3-byte prefixes, at most kChain candidates per position, a match
// of kNice bytes taken at once) and
// dynamic-Huffman blocks of up to 2^16 symbols; stored blocks when that
// would not be smaller.
// Greedy LZ77 over data[s0, s1) with dynamic-Huffman blocks into bw; the
// last block is final when `last`. Matches stay inside [s0, s1) but may
// start up to 32 KiB before s0 (those positions only enter the hash chains).
void deflate_range(const uint8_t* data, size_t n, size_t s0, size_t s1, bool last, BitWriter& bw) {
  constexpr int kHashBits = 15, kWindow = 32768, kChain = 8, kNice = 64, kMaxMatch = 258;
  std::vector<int32_t> head(1 << kHashBits, -1), prev(kWindow, -1);
  auto hash = [&](size_t i) {
    const uint32_t v = (uint32_t)data[i] | (uint32_t)data[i + 1] << 8 | (uint32_t)data[i + 2] << 16;
    return (v * 2654435761u) >> (32 - kHashBits);
  };
  auto insert = [&](size_t i) {
    if (i + 2 >= n) return;
    const uint32_t h = hash(i);
    prev[i & (kWindow - 1)] = head[h];
    head[h] = (int32_t)i;
  };
  for (size_t i = s0 > (size_t)kWindow ? s0 - kWindow : 0; i < s0; ++i) insert(i);
  std::vector<Symbol> sy;
  sy.reserve(1 << 16);
  bool wrote_last = false;
  size_t i = s0;
  while (i < s1) {
    int best = 0, best_d = 0;
    if (i + 2 < s1) {
      const size_t limit = std::min<size_t>(kMaxMatch, s1 - i);
      int32_t cand = head[hash(i)];
      for (int c = 0; c < kChain && cand >= 0 && i - (size_t)cand <= (size_t)kWindow; ++c) {
        const uint8_t* a = data + cand;
        const uint8_t* b = data + i;
        if (a[best] == b[best]) {
          size_t l = 0;
          while (l < limit && a[l] == b[l]) ++l;
          if ((int)l > best) {
            best = (int)l;
            best_d = (int)(i - (size_t)cand);
            if (l == limit || best >= kNice) break;  // long enough
          }
        }
        const int32_t nx = prev[cand & (kWindow - 1)];
        if (nx >= cand) break;  // the slot was reused by a newer position
        cand = nx;
      }
    }
    if (best >= 3) {
      sy.push_back({(uint16_t)best, (uint16_t)best_d});
      for (int k = 0; k < best; ++k) insert(i + k);
      i += best;
    } else {
      sy.push_back({data[i], 0});
      insert(i);
      ++i;
    }
    if (sy.size() == (1u << 16) || i == s1) {
      write_block(bw, sy, last && i == s1);
      wrote_last = last && i == s1;
      sy.clear();
    }
  }
  if (last && !wrote_last) write_block(bw, sy, true);  // an empty input
}

// A zlib stream (RFC 1950) of data[0, n). From 1 MiB on, the data is cut
// into segments of at least 256 KiB compressed on separate threads, each
// ended (but the last) by an empty stored block so that the next starts on
// a byte boundary -- one valid stream, as one thread would write it but for
// the block boundaries.
std::vector<uint8_t> zlib_compress(const uint8_t* data, size_t n) {
  std::vector<uint8_t> out = {0x78, 0x9C};
  const size_t parts = n >= (1u << 20) ? std::max<size_t>(1, std::min(rmn::host_threads(), n / (256u << 10))) : 1;
  if (parts == 1) {
    BitWriter bw(out);
    deflate_range(data, n, 0, n, true, bw);
    bw.flush();
  } else {
    std::vector<std::vector<uint8_t>> seg(parts);
    rmn::run_threads(parts, [&](size_t k) {
      BitWriter bw(seg[k]);
      const bool last = k + 1 == parts;
      deflate_range(data, n, n * k / parts, n * (k + 1) / parts, last, bw);
      if (!last) bw.put(0, 3);  // BFINAL 0, BTYPE 00: a stored block ...
      bw.flush();               // ... from the next byte boundary
      if (!last) seg[k].insert(seg[k].end(), {0x00, 0x00, 0xff, 0xff});  // LEN 0, NLEN
    });
    for (const std::vector<uint8_t>& sg : seg) out.insert(out.end(), sg.begin(), sg.end());
  }
  if (out.size() > n + n / 65535 * 5 + 16) {  // incompressible: stored blocks
    out.assign({0x78, 0x01});
    size_t pos = 0;
    do {
      const size_t k = std::min<size_t>(65535, n - pos);
      out.push_back(pos + k == n ? 1 : 0);
      out.push_back((uint8_t)(k & 0xff));
      out.push_back((uint8_t)(k >> 8));
      out.push_back((uint8_t)(~k & 0xff));
      out.push_back((uint8_t)((~k >> 8) & 0xff));
      out.insert(out.end(), data + pos, data + pos + k);
      pos += k;
    } while (pos < n);
  }
  const uint32_t a = adler32(data, n);
  for (int k = 3; k >= 0; --k) out.push_back((uint8_t)(a >> (8 * k)));
  return out;
}

rmn_status decode_image_file(const char* path, int kind, bool header_only, DecodedImage& img) {
  if (kind != RMN_IMAGE_PNG && kind != RMN_IMAGE_DDS && kind != RMN_IMAGE_HDR)
    return fail(RMN_ERR_INVALID_ARGUMENT, "unknown image kind %d", kind);
  std::vector<uint8_t> file;
  if (!read_file(path, file)) return fail(RMN_ERR_INVALID_ARGUMENT, "could not read %s", path);
  return kind == RMN_IMAGE_PNG   ? decode_png(file, header_only, img)
         : kind == RMN_IMAGE_DDS ? decode_dds(file, header_only, img)
                                 : decode_hdr(file, header_only, img);
}

}  // namespace rmn

extern "C" rmn_status rmn_image_load(const char* path, int32_t kind, rmn_image_desc* info, void* data,
                                     size_t capacity) {
  rmn::clear_error();
  if (!path || !info) return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_image_load needs a path and an info record");
  Decoded img;
  const bool header_only = data == nullptr;
  rmn_status st;
  try {  // no C++ exception crosses the ABI
    st = rmn::decode_image_file(path, kind, header_only, img);
  } catch (const std::bad_alloc&) {
    return fail(RMN_ERR_OUT_OF_MEMORY, "out of host memory decoding %s", path);
  } catch (const std::exception& e) {
    return fail(RMN_ERR_INTERNAL, "decoding %s: %s", path, e.what());
  }
  if (st != RMN_OK) return st;
  info->width = img.w;
  info->height = img.h;
  info->channels = img.channels;
  info->bytes_per_channel = img.bytes_per_channel;
  if (header_only) return RMN_OK;
  const size_t need = (size_t)img.w * img.h * img.channels * img.bytes_per_channel;
  if (capacity < need) return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_image_load: %zu bytes needed, %zu given", need, capacity);
  std::memcpy(data, img.bytes.data(), need);
  return RMN_OK;
}
