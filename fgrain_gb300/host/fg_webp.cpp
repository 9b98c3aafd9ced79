// WebP files of the command-line tool (the image crate's `webp` feature behind image::open and
// ImageBuffer::save, src/image_pipeline.rs:1087-1152; the crate writes lossless WebP): the
// lossless format (VP8L) in both directions.  The decoder follows the format's published
// specification: the four transforms (predictor, colour, subtract-green, colour indexing with
// pixel bundling), the colour cache, meta prefix codes and LZ77 backward references with the
// 120-entry distance map.  The encoder can use each of those (options), so that every decoder
// path can be exercised; by default it writes subtract-green, per-block predictors, backward
// references and a colour cache.  Lossy WebP (VP8) is not supported.  Host code only.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <queue>
#include <stdexcept>
#include <vector>

#include "fgrain_cuda.h"

namespace {

struct WebpError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

constexpr int kCodeLengthOrder[19] = {17, 18, 0, 1, 2, 3, 4, 5, 16, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15};
// Short distance codes 1..120: (dx, dy) offsets, the distance being dx + dy * width.
constexpr int8_t kDistMap[120][2] = {
    {0, 1},  {1, 0},  {1, 1},  {-1, 1}, {0, 2},  {2, 0},  {1, 2},  {-1, 2}, {2, 1},  {-2, 1}, {2, 2},  {-2, 2},
    {0, 3},  {3, 0},  {1, 3},  {-1, 3}, {3, 1},  {-3, 1}, {2, 3},  {-2, 3}, {3, 2},  {-3, 2}, {0, 4},  {4, 0},
    {1, 4},  {-1, 4}, {4, 1},  {-4, 1}, {3, 3},  {-3, 3}, {2, 4},  {-2, 4}, {4, 2},  {-4, 2}, {0, 5},  {3, 4},
    {-3, 4}, {4, 3},  {-4, 3}, {5, 0},  {1, 5},  {-1, 5}, {5, 1},  {-5, 1}, {2, 5},  {-2, 5}, {5, 2},  {-5, 2},
    {4, 4},  {-4, 4}, {3, 5},  {-3, 5}, {5, 3},  {-5, 3}, {0, 6},  {6, 0},  {1, 6},  {-1, 6}, {6, 1},  {-6, 1},
    {2, 6},  {-2, 6}, {6, 2},  {-6, 2}, {4, 5},  {-4, 5}, {5, 4},  {-5, 4}, {3, 6},  {-3, 6}, {6, 3},  {-6, 3},
    {0, 7},  {7, 0},  {1, 7},  {-1, 7}, {5, 5},  {-5, 5}, {7, 1},  {-7, 1}, {4, 6},  {-4, 6}, {6, 4},  {-6, 4},
    {2, 7},  {-2, 7}, {7, 2},  {-7, 2}, {3, 7},  {-3, 7}, {7, 3},  {-7, 3}, {5, 6},  {-5, 6}, {6, 5},  {-6, 5},
    {8, 0},  {4, 7},  {-4, 7}, {7, 4},  {-7, 4}, {8, 1},  {8, 2},  {6, 6},  {-6, 6}, {8, 3},  {5, 7},  {-5, 7},
    {7, 5},  {-7, 5}, {8, 4},  {6, 7},  {-6, 7}, {7, 6},  {-7, 6}, {8, 5},  {7, 7},  {-7, 7}, {8, 6},  {8, 7}};

inline uint32_t A(uint32_t p) { return p >> 24; }
inline uint32_t R(uint32_t p) { return (p >> 16) & 255; }
inline uint32_t G(uint32_t p) { return (p >> 8) & 255; }
inline uint32_t B(uint32_t p) { return p & 255; }
inline uint32_t argb(uint32_t a, uint32_t r, uint32_t g, uint32_t b) {
  return ((a & 255) << 24) | ((r & 255) << 16) | ((g & 255) << 8) | (b & 255);
}
inline uint32_t add_px(uint32_t a, uint32_t b) {
  return argb(A(a) + A(b), R(a) + R(b), G(a) + G(b), B(a) + B(b));
}
inline uint32_t sub_px(uint32_t a, uint32_t b) {
  return argb(A(a) - A(b), R(a) - R(b), G(a) - G(b), B(a) - B(b));
}
inline uint32_t avg2(uint32_t a, uint32_t b) {
  return argb((A(a) + A(b)) / 2, (R(a) + R(b)) / 2, (G(a) + G(b)) / 2, (B(a) + B(b)) / 2);
}
inline int clamp255(int v) { return v < 0 ? 0 : (v > 255 ? 255 : v); }
inline uint32_t select_px(uint32_t L, uint32_t T, uint32_t TL) {
  const int pa = static_cast<int>(A(L)) + static_cast<int>(A(T)) - static_cast<int>(A(TL));
  const int pr = static_cast<int>(R(L)) + static_cast<int>(R(T)) - static_cast<int>(R(TL));
  const int pg = static_cast<int>(G(L)) + static_cast<int>(G(T)) - static_cast<int>(G(TL));
  const int pb = static_cast<int>(B(L)) + static_cast<int>(B(T)) - static_cast<int>(B(TL));
  const int dl = std::abs(pa - static_cast<int>(A(L))) + std::abs(pr - static_cast<int>(R(L))) +
                 std::abs(pg - static_cast<int>(G(L))) + std::abs(pb - static_cast<int>(B(L)));
  const int dt = std::abs(pa - static_cast<int>(A(T))) + std::abs(pr - static_cast<int>(R(T))) +
                 std::abs(pg - static_cast<int>(G(T))) + std::abs(pb - static_cast<int>(B(T)));
  return dl < dt ? L : T;
}
inline uint32_t clamp_full(uint32_t a, uint32_t b, uint32_t c) {
  auto f = [](uint32_t x, uint32_t y, uint32_t z) {
    return static_cast<uint32_t>(clamp255(static_cast<int>(x) + static_cast<int>(y) - static_cast<int>(z)));
  };
  return argb(f(A(a), A(b), A(c)), f(R(a), R(b), R(c)), f(G(a), G(b), G(c)), f(B(a), B(b), B(c)));
}
inline uint32_t clamp_half(uint32_t a, uint32_t b) {
  auto f = [](uint32_t x, uint32_t y) {
    return static_cast<uint32_t>(clamp255(static_cast<int>(x) + (static_cast<int>(x) - static_cast<int>(y)) / 2));
  };
  return argb(f(A(a), A(b)), f(R(a), R(b)), f(G(a), G(b)), f(B(a), B(b)));
}
// Predictor `mode` for pixel (x, y > 0, x > 0) of an image of width w (rightmost TR wraps to the
// current row's first pixel, as the format defines).
inline uint32_t predict(int mode, const uint32_t* p, int x, int y, int w) {
  const size_t i = static_cast<size_t>(y) * w + x;
  const uint32_t L = p[i - 1], T = p[i - w], TL = p[i - w - 1], TR = p[i - w + 1];
  switch (mode) {
    case 0: return 0xff000000u;
    case 1: return L;
    case 2: return T;
    case 3: return TR;
    case 4: return TL;
    case 5: return avg2(avg2(L, TR), T);
    case 6: return avg2(L, TL);
    case 7: return avg2(L, T);
    case 8: return avg2(TL, T);
    case 9: return avg2(T, TR);
    case 10: return avg2(avg2(L, TL), avg2(T, TR));
    case 11: return select_px(L, T, TL);
    case 12: return clamp_full(L, T, TL);
    case 13: return clamp_half(avg2(L, T), TL);
    default: return 0xff000000u;  // 14 and 15 are not defined modes: black, as mode 0
  }
}
inline int ct_delta(uint8_t t, uint8_t c) {
  return (static_cast<int>(static_cast<int8_t>(t)) * static_cast<int>(static_cast<int8_t>(c))) >> 5;
}

// ---------------------------------------------------------------------------------------------
// Decoding

struct BitReader {
  const uint8_t* p;
  size_t n, pos = 0;
  uint64_t acc = 0;
  int bits = 0;
  void fill() {
    while (bits <= 56 && pos < n) {
      acc |= static_cast<uint64_t>(p[pos++]) << bits;
      bits += 8;
    }
  }
  // The next k bits (k <= 32) without consuming them; bits past the end read as zero.
  uint32_t peek(int k) {
    if (bits < k) fill();
    return static_cast<uint32_t>(acc & ((1ull << k) - 1));
  }
  void skip(int k) {
    if (bits < k) fill();
    if (bits < k) throw WebpError("truncated WebP image data");
    acc >>= k;
    bits -= k;
  }
  uint32_t read(int k) {
    if (k == 0) return 0;
    const uint32_t v = peek(k);
    skip(k);
    return v;
  }
};

// A canonical prefix code.  Codes are assigned in order of length, then symbol, and read most
// significant bit first; a table indexed by the next kFast bits (least significant bit first, as
// the stream delivers them) holds every code of at most kFast bits, longer codes are read bit by
// bit.
struct Prefix {
  static constexpr int kFast = 9;
  int single = -1;  // the one symbol of a zero-bit code
  int maxlen = 0;
  std::vector<int> first, count, offset, syms;
  std::vector<int32_t> fast;  // symbol << 4 | length, or -1 for a longer code
  void build(const std::vector<int>& len) {
    int nz = 0, last = -1;
    for (size_t s = 0; s < len.size(); ++s)
      if (len[s]) {
        ++nz;
        last = static_cast<int>(s);
      }
    if (nz == 0) throw WebpError("WebP prefix code without symbols");
    if (nz == 1) {
      single = last;
      return;
    }
    maxlen = 0;
    for (int l : len) maxlen = std::max(maxlen, l);
    count.assign(static_cast<size_t>(maxlen) + 1, 0);
    for (int l : len)
      if (l) ++count[static_cast<size_t>(l)];
    first.assign(static_cast<size_t>(maxlen) + 1, 0);
    offset.assign(static_cast<size_t>(maxlen) + 1, 0);
    int code = 0, off = 0;
    long kraft = 0;
    for (int l = 1; l <= maxlen; ++l) {
      first[static_cast<size_t>(l)] = code;
      offset[static_cast<size_t>(l)] = off;
      code = (code + count[static_cast<size_t>(l)]) << 1;
      off += count[static_cast<size_t>(l)];
      kraft += static_cast<long>(count[static_cast<size_t>(l)]) << (maxlen - l);
    }
    if (kraft != (1L << maxlen)) throw WebpError("WebP prefix code is not complete");
    syms.clear();
    for (int l = 1; l <= maxlen; ++l)
      for (size_t s = 0; s < len.size(); ++s)
        if (len[s] == l) syms.push_back(static_cast<int>(s));
    fast.assign(1u << kFast, -1);
    for (int l = 1; l <= std::min(maxlen, kFast); ++l)
      for (int k = 0; k < count[static_cast<size_t>(l)]; ++k) {
        const uint32_t c = static_cast<uint32_t>(first[static_cast<size_t>(l)] + k);
        uint32_t rev = 0;
        for (int b = 0; b < l; ++b) rev |= ((c >> (l - 1 - b)) & 1u) << b;
        const int32_t e = syms[static_cast<size_t>(offset[static_cast<size_t>(l)] + k)] << 4 | l;
        for (uint32_t hi = 0; hi < (1u << (kFast - l)); ++hi) fast[rev | hi << l] = e;
      }
  }
  int decode(BitReader& r) const {
    if (single >= 0) return single;
    const int32_t e = fast[r.peek(kFast)];
    if (e >= 0) {
      r.skip(e & 15);
      return e >> 4;
    }
    int code = 0;
    for (int l = 1; l <= maxlen; ++l) {
      code = (code << 1) | static_cast<int>(r.read(1));
      const int c = count[static_cast<size_t>(l)];
      if (code - first[static_cast<size_t>(l)] < c)
        return syms[static_cast<size_t>(offset[static_cast<size_t>(l)] + code - first[static_cast<size_t>(l)])];
    }
    throw WebpError("corrupt WebP prefix code");
  }
};

Prefix read_code(BitReader& r, int alphabet) {
  std::vector<int> len(static_cast<size_t>(alphabet), 0);
  if (r.read(1)) {  // simple code: one or two symbols
    const int ns = static_cast<int>(r.read(1)) + 1;
    const int first8 = static_cast<int>(r.read(1));
    const int s0 = static_cast<int>(r.read(first8 ? 8 : 1));
    if (s0 >= alphabet) throw WebpError("WebP simple code symbol out of range");
    len[static_cast<size_t>(s0)] = 1;
    if (ns == 2) {
      const int s1 = static_cast<int>(r.read(8));
      if (s1 >= alphabet) throw WebpError("WebP simple code symbol out of range");
      len[static_cast<size_t>(s1)] = 1;
    }
    Prefix p;
    p.build(len);  // one distinct symbol: a zero-bit code
    return p;
  }
  std::vector<int> cl(19, 0);
  const int ncl = 4 + static_cast<int>(r.read(4));
  for (int i = 0; i < ncl; ++i) cl[static_cast<size_t>(kCodeLengthOrder[i])] = static_cast<int>(r.read(3));
  Prefix clc;
  clc.build(cl);
  int max_symbol = alphabet;
  if (r.read(1)) {
    const int nb = 2 + 2 * static_cast<int>(r.read(3));
    max_symbol = 2 + static_cast<int>(r.read(nb));
    if (max_symbol > alphabet) throw WebpError("WebP code length count out of range");
  }
  int prev = 8, s = 0;
  while (s < alphabet) {
    if (max_symbol-- == 0) break;
    const int c = clc.decode(r);
    if (c < 16) {
      len[static_cast<size_t>(s++)] = c;
      if (c) prev = c;
    } else {
      const int rep = c == 16 ? 3 + static_cast<int>(r.read(2)) : (c == 17 ? 3 + static_cast<int>(r.read(3)) : 11 + static_cast<int>(r.read(7)));
      const int v = c == 16 ? prev : 0;
      if (s + rep > alphabet) throw WebpError("WebP code lengths overrun the alphabet");
      for (int k = 0; k < rep; ++k) len[static_cast<size_t>(s++)] = v;
    }
  }
  Prefix p;
  p.build(len);
  return p;
}

inline int prefix_value(BitReader& r, int sym) {
  if (sym < 4) return sym + 1;
  const int extra = (sym - 2) >> 1;
  const int off = (2 + (sym & 1)) << extra;
  return off + static_cast<int>(r.read(extra)) + 1;
}

std::vector<uint32_t> read_image(BitReader& r, int w, int h, bool main_image) {
  int cache_bits = 0;
  if (r.read(1)) {
    cache_bits = static_cast<int>(r.read(4));
    if (cache_bits < 1 || cache_bits > 11) throw WebpError("bad WebP colour cache size");
  }
  int prefix_bits = 0, meta_w = 1;
  std::vector<uint32_t> meta;
  int ngroups = 1;
  if (main_image && r.read(1)) {
    prefix_bits = static_cast<int>(r.read(3)) + 2;
    meta_w = (w + (1 << prefix_bits) - 1) >> prefix_bits;
    const int meta_h = (h + (1 << prefix_bits) - 1) >> prefix_bits;
    meta = read_image(r, meta_w, meta_h, false);
    for (auto& m : meta) {
      m = (m >> 8) & 0xffff;
      ngroups = std::max(ngroups, static_cast<int>(m) + 1);
    }
  }
  const int cache_size = cache_bits ? 1 << cache_bits : 0;
  std::vector<Prefix> codes(static_cast<size_t>(ngroups) * 5);
  const int sizes[5] = {256 + 24 + cache_size, 256, 256, 256, 40};
  for (int g = 0; g < ngroups; ++g)
    for (int k = 0; k < 5; ++k) codes[static_cast<size_t>(g) * 5 + k] = read_code(r, sizes[k]);
  std::vector<uint32_t> cache(static_cast<size_t>(cache_size), 0);
  const size_t total = static_cast<size_t>(w) * h;
  std::vector<uint32_t> px(total);
  auto insert = [&](uint32_t v) {
    if (cache_bits) cache[(0x1e35a7bdu * v) >> (32 - cache_bits)] = v;
  };
  size_t i = 0;
  while (i < total) {
    const int x = static_cast<int>(i % static_cast<size_t>(w)), y = static_cast<int>(i / static_cast<size_t>(w));
    const int g = meta.empty() ? 0 : static_cast<int>(meta[static_cast<size_t>((y >> prefix_bits) * meta_w + (x >> prefix_bits))]);
    const Prefix* c = &codes[static_cast<size_t>(g) * 5];
    const int s = c[0].decode(r);
    if (s < 256) {
      const uint32_t rr = static_cast<uint32_t>(c[1].decode(r)), bb = static_cast<uint32_t>(c[2].decode(r)),
                     aa = static_cast<uint32_t>(c[3].decode(r));
      px[i] = argb(aa, rr, static_cast<uint32_t>(s), bb);
      insert(px[i++]);
    } else if (s < 256 + 24) {
      const int length = prefix_value(r, s - 256);
      const int dsym = c[4].decode(r);
      const int dcode = prefix_value(r, dsym);
      long dist;
      if (dcode > 120) {
        dist = dcode - 120;
      } else {
        dist = kDistMap[dcode - 1][0] + static_cast<long>(kDistMap[dcode - 1][1]) * w;
        if (dist < 1) dist = 1;
      }
      if (static_cast<size_t>(dist) > i || i + static_cast<size_t>(length) > total) throw WebpError("WebP backward reference out of range");
      for (int k = 0; k < length; ++k, ++i) {
        px[i] = px[i - static_cast<size_t>(dist)];
        insert(px[i]);
      }
    } else {
      const int idx = s - 280;
      if (idx >= cache_size) throw WebpError("WebP colour cache index out of range");
      px[i] = cache[static_cast<size_t>(idx)];
      insert(px[i++]);
    }
  }
  return px;
}

struct Transform {
  int type, bits, w;  // w: the image width when the transform was read
  std::vector<uint32_t> data;
};

struct Image {
  int w, h;
  bool alpha;
  std::vector<uint32_t> px;
};

void locate_vp8l(const uint8_t* d, size_t n, size_t& at, size_t& len) {
  if (n < 20 || std::memcmp(d, "RIFF", 4) != 0 || std::memcmp(d + 8, "WEBP", 4) != 0) throw WebpError("not a WebP file");
  size_t p = 12;
  while (p + 8 <= n) {
    const uint32_t sz = d[p + 4] | d[p + 5] << 8 | d[p + 6] << 16 | static_cast<uint32_t>(d[p + 7]) << 24;
    if (p + 8 + sz > n) throw WebpError("truncated WebP chunk");
    if (std::memcmp(d + p, "VP8L", 4) == 0) {
      at = p + 8;
      len = sz;
      return;
    }
    if (std::memcmp(d + p, "VP8 ", 4) == 0) throw WebpError("lossy WebP (VP8) is not supported, only lossless WebP");
    if (std::memcmp(d + p, "ANIM", 4) == 0) throw WebpError("animated WebP is not supported");
    p += 8 + sz + (sz & 1);
  }
  throw WebpError("WebP file without image data");
}

Image decode(const uint8_t* d, size_t n, bool header_only) {
  size_t at = 0, len = 0;
  locate_vp8l(d, n, at, len);
  BitReader r{d + at, len};
  if (r.read(8) != 0x2f) throw WebpError("bad WebP lossless signature");
  Image im;
  im.w = static_cast<int>(r.read(14)) + 1;
  im.h = static_cast<int>(r.read(14)) + 1;
  im.alpha = r.read(1) != 0;
  if (r.read(3) != 0) throw WebpError("unknown WebP lossless version");
  if (header_only) return im;
  std::vector<Transform> tr;
  int w = im.w;
  bool seen[4] = {false, false, false, false};
  while (r.read(1)) {
    Transform t;
    t.type = static_cast<int>(r.read(2));
    if (seen[t.type]) throw WebpError("WebP transform used twice");
    seen[t.type] = true;
    t.w = w;
    t.bits = 0;
    if (t.type == 0 || t.type == 1) {
      t.bits = static_cast<int>(r.read(3)) + 2;
      const int bw = (w + (1 << t.bits) - 1) >> t.bits, bh = (im.h + (1 << t.bits) - 1) >> t.bits;
      t.data = read_image(r, bw, bh, false);
    } else if (t.type == 3) {
      const int ncol = static_cast<int>(r.read(8)) + 1;
      t.data = read_image(r, ncol, 1, false);
      for (size_t k = 1; k < t.data.size(); ++k) t.data[k] = add_px(t.data[k], t.data[k - 1]);
      t.bits = ncol <= 2 ? 3 : (ncol <= 4 ? 2 : (ncol <= 16 ? 1 : 0));
      w = (w + (1 << t.bits) - 1) >> t.bits;
    }
    tr.push_back(std::move(t));
  }
  std::vector<uint32_t> px = read_image(r, w, im.h, true);
  for (auto it = tr.rbegin(); it != tr.rend(); ++it) {
    const Transform& t = *it;
    const int tw = t.w;
    if (t.type == 2) {
      for (auto& p : px) p = argb(A(p), R(p) + G(p), G(p), B(p) + G(p));
    } else if (t.type == 1) {
      const int bw = (tw + (1 << t.bits) - 1) >> t.bits;
      for (int y = 0; y < im.h; ++y)
        for (int x = 0; x < tw; ++x) {
          const uint32_t e = t.data[static_cast<size_t>((y >> t.bits) * bw + (x >> t.bits))];
          uint32_t& p = px[static_cast<size_t>(y) * tw + x];
          const uint8_t g2r = static_cast<uint8_t>(B(e)), g2b = static_cast<uint8_t>(G(e)), r2b = static_cast<uint8_t>(R(e));
          const int red = static_cast<int>(R(p)) + ct_delta(g2r, static_cast<uint8_t>(G(p)));
          int blue = static_cast<int>(B(p)) + ct_delta(g2b, static_cast<uint8_t>(G(p)));
          blue += ct_delta(r2b, static_cast<uint8_t>(red & 255));
          p = argb(A(p), static_cast<uint32_t>(red), G(p), static_cast<uint32_t>(blue));
        }
    } else if (t.type == 0) {
      const int bw = (tw + (1 << t.bits) - 1) >> t.bits;
      for (int y = 0; y < im.h; ++y)
        for (int x = 0; x < tw; ++x) {
          const size_t i = static_cast<size_t>(y) * tw + x;
          uint32_t pred;
          if (x == 0 && y == 0) pred = 0xff000000u;
          else if (y == 0) pred = px[i - 1];
          else if (x == 0) pred = px[i - static_cast<size_t>(tw)];
          else pred = predict(static_cast<int>(G(t.data[static_cast<size_t>((y >> t.bits) * bw + (x >> t.bits))]) & 15),
                              px.data(), x, y, tw);
          px[i] = add_px(px[i], pred);
        }
    } else {  // colour indexing: unbundle to the width before the transform
      const int ow = tw;
      const int inw = (ow + (1 << t.bits) - 1) >> t.bits;
      const int bpp = 8 >> t.bits;
      std::vector<uint32_t> out(static_cast<size_t>(ow) * im.h);
      for (int y = 0; y < im.h; ++y)
        for (int x = 0; x < ow; ++x) {
          const uint32_t packed = G(px[static_cast<size_t>(y) * inw + (x >> t.bits)]);
          const uint32_t idx = (packed >> ((x & ((1 << t.bits) - 1)) * bpp)) & ((1u << bpp) - 1);
          out[static_cast<size_t>(y) * ow + x] = idx < t.data.size() ? t.data[idx] : 0u;
        }
      px.swap(out);
    }
  }
  if (static_cast<int>(px.size()) != im.w * im.h) throw WebpError("WebP transforms leave a wrong image size");
  im.px = std::move(px);
  return im;
}

// ---------------------------------------------------------------------------------------------
// Encoding

struct BitWriter {
  std::vector<uint8_t> out;
  uint64_t acc = 0;
  int bits = 0;
  void put(uint32_t v, int n) {  // n low bits of v, least significant first
    acc |= static_cast<uint64_t>(v & ((n == 32) ? 0xffffffffu : ((1u << n) - 1u))) << bits;
    bits += n;
    while (bits >= 8) {
      out.push_back(static_cast<uint8_t>(acc));
      acc >>= 8;
      bits -= 8;
    }
  }
  void put_code(uint32_t code, int len) {  // a prefix code, most significant bit first
    for (int i = len - 1; i >= 0; --i) put((code >> i) & 1u, 1);
  }
  void flush() {
    if (bits) put(0, 8 - bits);
  }
};

// Code lengths of at most `limit` bits for the given counts (Huffman, flattening the counts until
// the lengths fit), and the canonical codes.
struct EncCode {
  std::vector<int> len;
  std::vector<uint32_t> code;
  int used = 0, only = -1;
  void build(const std::vector<uint32_t>& freq, int limit) {
    const int n = static_cast<int>(freq.size());
    len.assign(static_cast<size_t>(n), 0);
    code.assign(static_cast<size_t>(n), 0);
    used = 0;
    for (int s = 0; s < n; ++s)
      if (freq[static_cast<size_t>(s)]) {
        ++used;
        only = s;
      }
    if (used <= 1) return;
    std::vector<uint64_t> f(freq.begin(), freq.end());
    for (;;) {
      struct Nd { uint64_t w; int left, right, sym; };
      std::vector<Nd> nodes;
      using QE = std::pair<uint64_t, int>;
      std::priority_queue<QE, std::vector<QE>, std::greater<QE>> q;
      for (int s = 0; s < n; ++s)
        if (f[static_cast<size_t>(s)]) {
          nodes.push_back({f[static_cast<size_t>(s)], -1, -1, s});
          q.push({f[static_cast<size_t>(s)], static_cast<int>(nodes.size()) - 1});
        }
      while (q.size() > 1) {
        const auto a = q.top(); q.pop();
        const auto b = q.top(); q.pop();
        nodes.push_back({a.first + b.first, a.second, b.second, -1});
        q.push({a.first + b.first, static_cast<int>(nodes.size()) - 1});
      }
      int maxl = 0;
      std::vector<std::pair<int, int>> st{{q.top().second, 0}};
      std::fill(len.begin(), len.end(), 0);
      while (!st.empty()) {
        const auto [k, d] = st.back();
        st.pop_back();
        if (nodes[static_cast<size_t>(k)].sym >= 0) {
          len[static_cast<size_t>(nodes[static_cast<size_t>(k)].sym)] = d;
          maxl = std::max(maxl, d);
        } else {
          st.push_back({nodes[static_cast<size_t>(k)].left, d + 1});
          st.push_back({nodes[static_cast<size_t>(k)].right, d + 1});
        }
      }
      if (maxl <= limit) break;
      for (auto& v : f)
        if (v) v = (v >> 1) + 1;
    }
    std::vector<int> cnt(static_cast<size_t>(limit) + 2, 0), next(static_cast<size_t>(limit) + 2, 0);
    for (int l : len)
      if (l) ++cnt[static_cast<size_t>(l)];
    int c = 0;
    for (int l = 1; l <= limit; ++l) {
      c = (c + cnt[static_cast<size_t>(l) - 1]) << 1;
      next[static_cast<size_t>(l)] = c;
    }
    // The decoder assigns codes in order of length, then symbol.
    c = 0;
    for (int l = 1; l <= limit; ++l) {
      next[static_cast<size_t>(l)] = c;
      c = (c + cnt[static_cast<size_t>(l)]) << 1;
    }
    for (int s = 0; s < n; ++s)
      if (len[static_cast<size_t>(s)]) code[static_cast<size_t>(s)] = static_cast<uint32_t>(next[static_cast<size_t>(len[static_cast<size_t>(s)])]++);
  }
  void put(BitWriter& w, int s) const {
    if (used <= 1) return;  // zero-bit code
    w.put_code(code[static_cast<size_t>(s)], len[static_cast<size_t>(s)]);
  }
};

void write_code(BitWriter& w, const EncCode& c, int alphabet) {
  if (c.used <= 1) {
    const int s = c.used ? c.only : 0;
    if (s < 256) {  // simple code, one symbol
      w.put(1, 1);
      w.put(0, 1);
      if (s < 2) {
        w.put(0, 1);
        w.put(static_cast<uint32_t>(s), 1);
      } else {
        w.put(1, 1);
        w.put(static_cast<uint32_t>(s), 8);
      }
      return;
    }
  }
  // Normal code: the code lengths, run-length coded with symbols 0-15, 16 (repeat previous), 17
  // and 18 (runs of zeros), themselves coded with a code of at most 7 bits.
  std::vector<int> len = c.len;
  if (c.used <= 1) {  // one symbol above 255: a single nonzero length, which decodes as zero bits
    len.assign(static_cast<size_t>(alphabet), 0);
    len[static_cast<size_t>(c.only)] = 1;
  }
  struct Tok { int sym, extra, nbits; };
  std::vector<Tok> toks;
  int prev = 8;
  for (int i = 0; i < alphabet;) {
    const int l = len[static_cast<size_t>(i)];
    int run = 1;
    while (i + run < alphabet && len[static_cast<size_t>(i + run)] == l) ++run;
    if (l == 0 && run >= 3) {
      const int take = std::min(run, 138);
      if (take >= 11) toks.push_back({18, take - 11, 7});
      else toks.push_back({17, take - 3, 3});
      i += take;
      continue;
    }
    if (l != 0 && l == prev && run >= 3) {
      const int take = std::min(run, 6);
      toks.push_back({16, take - 3, 2});
      i += take;
      continue;
    }
    toks.push_back({l, 0, 0});
    if (l) prev = l;
    ++i;
  }
  std::vector<uint32_t> f(19, 0);
  for (auto& t : toks) ++f[static_cast<size_t>(t.sym)];
  EncCode clc;
  clc.build(f, 7);
  std::vector<int> cl = clc.len;
  if (clc.used <= 1) cl[static_cast<size_t>(clc.only)] = 1;  // one symbol: a zero-bit code
  int ncl = 19;
  while (ncl > 4 && cl[static_cast<size_t>(kCodeLengthOrder[ncl - 1])] == 0) --ncl;
  w.put(0, 1);
  w.put(static_cast<uint32_t>(ncl - 4), 4);
  for (int i = 0; i < ncl; ++i) w.put(static_cast<uint32_t>(cl[static_cast<size_t>(kCodeLengthOrder[i])]), 3);
  w.put(0, 1);  // all symbols coded
  for (auto& t : toks) {
    clc.put(w, t.sym);
    if (t.nbits) w.put(static_cast<uint32_t>(t.extra), t.nbits);
  }
}

// Prefix coding of a length or distance value v >= 1: the symbol and its extra bits.
inline void value_prefix(int v, int& sym, int& nbits, int& extra) {
  --v;
  if (v < 4) {
    sym = v;
    nbits = 0;
    extra = 0;
    return;
  }
  int hb = 31 - __builtin_clz(static_cast<unsigned>(v));
  const int second = (v >> (hb - 1)) & 1;
  nbits = hb - 1;
  sym = 2 * hb + second;
  extra = v & ((1 << nbits) - 1);
}

// Distance codes (distance + 120) have 40 prefix symbols: at most 2^20.
constexpr size_t kMaxDistance = (1u << 20) - 120;

struct Token { int kind; uint32_t a; int len, dcode; };  // kind 0 literal (a = pixel), 1 cache (a = index), 2 copy

// Entropy-coded image: tokens with optional cache and backward references, one prefix-code group
// per meta block (meta_bits > 0: groups by block parity), written after its header bits.
void write_image(BitWriter& w, const std::vector<uint32_t>& px, int width, int height, bool main_image, int cache_bits,
                 bool backrefs, int meta_bits) {
  const size_t n = px.size();
  std::vector<Token> toks;
  std::vector<uint32_t> cache(cache_bits ? 1u << cache_bits : 0u, 0);
  auto hidx = [&](uint32_t v) { return (0x1e35a7bdu * v) >> (32 - cache_bits); };
  std::vector<int> head(1 << 16, -1), prevp(n, -1);
  auto h3 = [&](size_t i) { return ((px[i] * 0x9E3779B1u) ^ (px[i + 1] * 0x85EBCA77u) ^ (px[i + 2] * 0xC2B2AE3Du)) >> 16; };
  size_t i = 0;
  auto push_hash = [&](size_t k) {
    if (backrefs && k + 2 < n) {
      const uint32_t hh = h3(k);
      prevp[k] = head[hh];
      head[hh] = static_cast<int>(k);
    }
  };
  while (i < n) {
    int best_len = 0;
    size_t best_dist = 0;
    if (backrefs && i + 2 < n) {
      int cand = head[h3(i)];
      for (int tries = 0; cand >= 0 && tries < 16; ++tries, cand = prevp[static_cast<size_t>(cand)]) {
        const size_t d = i - static_cast<size_t>(cand);
        if (d > kMaxDistance) break;  // chains run to older positions
        int l = 0;
        while (i + static_cast<size_t>(l) < n && l < 4096 && px[static_cast<size_t>(cand) + static_cast<size_t>(l)] == px[i + static_cast<size_t>(l)]) ++l;
        if (l > best_len) {
          best_len = l;
          best_dist = d;
        }
      }
    }
    if (best_len >= 3) {
      // The distance code: a short (dx, dy) code when one matches, else distance + 120.
      int dcode = static_cast<int>(best_dist) + 120;
      for (int k = 0; k < 120; ++k) {
        const long dd = kDistMap[k][0] + static_cast<long>(kDistMap[k][1]) * width;
        if (dd == static_cast<long>(best_dist)) {
          dcode = k + 1;
          break;
        }
      }
      toks.push_back({2, 0, best_len, dcode});
      for (int k = 0; k < best_len; ++k) {
        if (cache_bits) cache[hidx(px[i])] = px[i];
        push_hash(i);
        ++i;
      }
      continue;
    }
    if (cache_bits && cache[hidx(px[i])] == px[i]) {
      toks.push_back({1, hidx(px[i]), 0, 0});
    } else {
      toks.push_back({0, px[i], 0, 0});
      if (cache_bits) cache[hidx(px[i])] = px[i];
    }
    push_hash(i);
    ++i;
  }
  // Groups.
  const int cache_size = cache_bits ? 1 << cache_bits : 0;
  int ngroups = 1, meta_w = 1;
  std::vector<uint32_t> meta;
  if (main_image && meta_bits > 0) {
    meta_w = (width + (1 << meta_bits) - 1) >> meta_bits;
    const int meta_h = (height + (1 << meta_bits) - 1) >> meta_bits;
    meta.resize(static_cast<size_t>(meta_w) * meta_h);
    for (int y = 0; y < meta_h; ++y)
      for (int x = 0; x < meta_w; ++x) meta[static_cast<size_t>(y) * meta_w + x] = static_cast<uint32_t>((x + y) & 1);
    ngroups = meta.size() > 1 ? 2 : 1;
  }
  auto group_at = [&](size_t k) {
    if (meta.empty()) return 0;
    const int x = static_cast<int>(k % static_cast<size_t>(width)), y = static_cast<int>(k / static_cast<size_t>(width));
    return static_cast<int>(meta[static_cast<size_t>((y >> meta_bits) * meta_w + (x >> meta_bits))]);
  };
  const int sizes[5] = {256 + 24 + cache_size, 256, 256, 256, 40};
  std::vector<std::vector<uint32_t>> freq(static_cast<size_t>(ngroups) * 5);
  for (int g = 0; g < ngroups; ++g)
    for (int k = 0; k < 5; ++k) freq[static_cast<size_t>(g) * 5 + k].assign(static_cast<size_t>(sizes[k]), 0);
  {
    size_t pos = 0;
    for (auto& t : toks) {
      auto* f = &freq[static_cast<size_t>(group_at(pos)) * 5];
      if (t.kind == 0) {
        ++f[0][G(t.a)];
        ++f[1][R(t.a)];
        ++f[2][B(t.a)];
        ++f[3][A(t.a)];
        ++pos;
      } else if (t.kind == 1) {
        ++f[0][280 + t.a];
        ++pos;
      } else {
        int s, nb, ex;
        value_prefix(t.len, s, nb, ex);
        ++f[0][static_cast<size_t>(256 + s)];
        value_prefix(t.dcode, s, nb, ex);
        ++f[4][static_cast<size_t>(s)];
        pos += static_cast<size_t>(t.len);
      }
    }
  }
  // Header bits.
  if (cache_bits) {
    w.put(1, 1);
    w.put(static_cast<uint32_t>(cache_bits), 4);
  } else {
    w.put(0, 1);
  }
  if (main_image) {
    if (ngroups > 1) {
      w.put(1, 1);
      w.put(static_cast<uint32_t>(meta_bits - 2), 3);
      std::vector<uint32_t> mimg(meta.size());
      for (size_t k = 0; k < meta.size(); ++k) mimg[k] = meta[k] << 8;  // group index in red + green
      write_image(w, mimg, meta_w, static_cast<int>(meta.size() / static_cast<size_t>(meta_w)), false, 0, false, 0);
    } else {
      w.put(0, 1);
    }
  }
  std::vector<EncCode> codes(static_cast<size_t>(ngroups) * 5);
  for (int g = 0; g < ngroups; ++g)
    for (int k = 0; k < 5; ++k) {
      codes[static_cast<size_t>(g) * 5 + k].build(freq[static_cast<size_t>(g) * 5 + k], 15);
      write_code(w, codes[static_cast<size_t>(g) * 5 + k], sizes[k]);
    }
  size_t pos = 0;
  for (auto& t : toks) {
    const EncCode* c = &codes[static_cast<size_t>(group_at(pos)) * 5];
    if (t.kind == 0) {
      c[0].put(w, static_cast<int>(G(t.a)));
      c[1].put(w, static_cast<int>(R(t.a)));
      c[2].put(w, static_cast<int>(B(t.a)));
      c[3].put(w, static_cast<int>(A(t.a)));
      ++pos;
    } else if (t.kind == 1) {
      c[0].put(w, 280 + static_cast<int>(t.a));
      ++pos;
    } else {
      int s, nb, ex;
      value_prefix(t.len, s, nb, ex);
      c[0].put(w, 256 + s);
      w.put(static_cast<uint32_t>(ex), nb);
      value_prefix(t.dcode, s, nb, ex);
      c[4].put(w, s);
      w.put(static_cast<uint32_t>(ex), nb);
      pos += static_cast<size_t>(t.len);
    }
  }
}

}  // namespace

extern "C" fg_status fg_webp_info(const uint8_t* data, size_t n, uint32_t* w, uint32_t* h, uint32_t* has_alpha,
                                  char* msg, size_t msg_cap) {
  if (!data || !w || !h || !has_alpha) return FG_ERR_INVALID_ARG;
  try {
    const Image im = decode(data, n, true);
    *w = static_cast<uint32_t>(im.w);
    *h = static_cast<uint32_t>(im.h);
    *has_alpha = im.alpha ? 1u : 0u;
    return FG_OK;
  } catch (const std::exception& e) {
    if (msg && msg_cap) std::snprintf(msg, msg_cap, "%s", e.what());
    return FG_ERR_INVALID_ARG;
  }
}

extern "C" fg_status fg_webp_decode(const uint8_t* data, size_t n, uint8_t* rgba, size_t cap, char* msg,
                                    size_t msg_cap) {
  if (!data || !rgba) return FG_ERR_INVALID_ARG;
  try {
    const Image im = decode(data, n, false);
    if (static_cast<size_t>(im.w) * im.h * 4 > cap) throw WebpError("output buffer too small");
    for (size_t i = 0; i < im.px.size(); ++i) {
      const uint32_t p = im.px[i];
      rgba[4 * i] = static_cast<uint8_t>(R(p));
      rgba[4 * i + 1] = static_cast<uint8_t>(G(p));
      rgba[4 * i + 2] = static_cast<uint8_t>(B(p));
      rgba[4 * i + 3] = static_cast<uint8_t>(A(p));
    }
    return FG_OK;
  } catch (const std::exception& e) {
    if (msg && msg_cap) std::snprintf(msg, msg_cap, "%s", e.what());
    return FG_ERR_INVALID_ARG;
  }
}

extern "C" fg_status fg_webp_encode(const uint8_t* px, uint32_t w, uint32_t h, uint32_t channels, uint32_t options,
                                    uint8_t* out, size_t cap, size_t* len) {
  if (!px || !out || !len || w == 0 || h == 0 || w > 16384 || h > 16384 ||
      (channels != 1 && channels != 3 && channels != 4))
    return FG_ERR_INVALID_ARG;
  const size_t n = static_cast<size_t>(w) * h;
  std::vector<uint32_t> img(n);
  bool alpha = false;
  for (size_t i = 0; i < n; ++i) {
    const uint8_t* p = px + i * channels;
    const uint32_t r = p[0], g = channels >= 3 ? p[1] : p[0], b = channels >= 3 ? p[2] : p[0];
    const uint32_t a = channels == 4 ? p[3] : 255u;
    alpha |= a != 255;
    img[i] = argb(a, r, g, b);
  }
  BitWriter bw;
  bw.put(0x2f, 8);
  bw.put(w - 1, 14);
  bw.put(h - 1, 14);
  bw.put(alpha ? 1 : 0, 1);
  bw.put(0, 3);
  int width = static_cast<int>(w);
  const int H = static_cast<int>(h);
  // Colour indexing, when asked for and at most 256 colours.
  if (options & FG_WEBP_PALETTE) {
    std::vector<uint32_t> pal(img);
    std::sort(pal.begin(), pal.end());
    pal.erase(std::unique(pal.begin(), pal.end()), pal.end());
    if (pal.size() <= 256) {
      const int nc = static_cast<int>(pal.size());
      const int bits = nc <= 2 ? 3 : (nc <= 4 ? 2 : (nc <= 16 ? 1 : 0));
      bw.put(1, 1);
      bw.put(3, 2);
      bw.put(static_cast<uint32_t>(nc - 1), 8);
      std::vector<uint32_t> delta(pal.size());
      for (size_t k = 0; k < pal.size(); ++k) delta[k] = k ? sub_px(pal[k], pal[k - 1]) : pal[k];
      write_image(bw, delta, nc, 1, false, 0, false, 0);
      const int nw = (width + (1 << bits) - 1) >> bits, bpp = 8 >> bits;
      std::vector<uint32_t> packed(static_cast<size_t>(nw) * H, 0);
      for (int y = 0; y < H; ++y)
        for (int x = 0; x < width; ++x) {
          const uint32_t idx = static_cast<uint32_t>(std::lower_bound(pal.begin(), pal.end(), img[static_cast<size_t>(y) * width + x]) - pal.begin());
          uint32_t& q = packed[static_cast<size_t>(y) * nw + (x >> bits)];
          q = argb(255, 0, G(q) | (idx << ((x & ((1 << bits) - 1)) * bpp)), 0);
        }
      img.swap(packed);
      width = nw;
    }
  }
  if (options & FG_WEBP_SUBTRACT_GREEN) {
    bw.put(1, 1);
    bw.put(2, 2);
    for (auto& p : img) p = argb(A(p), R(p) - G(p), G(p), B(p) - G(p));
  }
  if (options & FG_WEBP_PREDICTOR) {
    const int bits = 4, bwid = (width + 15) >> 4, bh = (H + 15) >> 4;
    std::vector<uint32_t> modes(static_cast<size_t>(bwid) * bh);
    std::vector<uint32_t> res(img.size());
    for (int by = 0; by < bh; ++by)
      for (int bx = 0; bx < bwid; ++bx) {
        int best = (bx + 3 * by) % 14;  // every mode in turn, for testing the decoder
        long best_cost = -1;
        for (int m = 0; m < 14 && !(options & FG_WEBP_ALL_MODES); ++m) {
          long cost = 0;
          for (int y = by * 16; y < std::min(H, by * 16 + 16); ++y)
            for (int x = bx * 16; x < std::min(width, bx * 16 + 16); ++x) {
              if (x == 0 || y == 0) continue;
              const uint32_t d = sub_px(img[static_cast<size_t>(y) * width + x], predict(m, img.data(), x, y, width));
              for (int sh = 0; sh < 32; sh += 8) {
                const int v = static_cast<int>((d >> sh) & 255);
                cost += std::min(v, 256 - v);
              }
            }
          if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = m;
          }
        }
        modes[static_cast<size_t>(by) * bwid + bx] = argb(255, 0, static_cast<uint32_t>(best), 0);
      }
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < width; ++x) {
        const size_t i = static_cast<size_t>(y) * width + x;
        uint32_t pred;
        if (x == 0 && y == 0) pred = 0xff000000u;
        else if (y == 0) pred = img[i - 1];
        else if (x == 0) pred = img[i - static_cast<size_t>(width)];
        else pred = predict(static_cast<int>(G(modes[static_cast<size_t>((y >> bits) * bwid + (x >> bits))])), img.data(), x, y, width);
        res[i] = sub_px(img[i], pred);
      }
    bw.put(1, 1);
    bw.put(0, 2);
    bw.put(static_cast<uint32_t>(bits - 2), 3);
    write_image(bw, modes, bwid, bh, false, 0, false, 0);
    img.swap(res);
  }
  if (options & FG_WEBP_COLOR_TRANSFORM) {
    const int bits = 5, bwid = (width + 31) >> 5, bh = (H + 31) >> 5;
    std::vector<uint32_t> el(static_cast<size_t>(bwid) * bh);
    for (size_t k = 0; k < el.size(); ++k) {  // per-block coefficients (a fixed pseudo-random pattern)
      const uint32_t hsh = static_cast<uint32_t>(k) * 2654435761u;
      el[k] = argb(255, hsh >> 8, hsh >> 16, hsh >> 24);
    }
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < width; ++x) {
        uint32_t& p = img[static_cast<size_t>(y) * width + x];
        const uint32_t e = el[static_cast<size_t>((y >> bits) * bwid + (x >> bits))];
        const uint8_t g2r = static_cast<uint8_t>(B(e)), g2b = static_cast<uint8_t>(G(e)), r2b = static_cast<uint8_t>(R(e));
        const int red = static_cast<int>(R(p)), green = static_cast<int>(G(p));
        const int nr = red - ct_delta(g2r, static_cast<uint8_t>(green));
        const int nb = static_cast<int>(B(p)) - ct_delta(g2b, static_cast<uint8_t>(green)) - ct_delta(r2b, static_cast<uint8_t>(red));
        p = argb(A(p), static_cast<uint32_t>(nr), G(p), static_cast<uint32_t>(nb));
      }
    bw.put(1, 1);
    bw.put(1, 2);
    bw.put(static_cast<uint32_t>(bits - 2), 3);
    write_image(bw, el, bwid, bh, false, 0, false, 0);
  }
  bw.put(0, 1);  // no more transforms
  write_image(bw, img, width, H, true, (options & FG_WEBP_COLOR_CACHE) ? 6 : 0, (options & FG_WEBP_BACKREFS) != 0,
              (options & FG_WEBP_META_CODES) ? 4 : 0);
  bw.flush();
  // RIFF container.
  const size_t body = bw.out.size();
  const size_t chunk = body + (body & 1);
  const size_t total = 12 + 8 + chunk;
  *len = total;
  if (total > cap) return FG_ERR_INVALID_ARG;
  auto le32 = [&](uint8_t* p, uint32_t v) {
    p[0] = static_cast<uint8_t>(v);
    p[1] = static_cast<uint8_t>(v >> 8);
    p[2] = static_cast<uint8_t>(v >> 16);
    p[3] = static_cast<uint8_t>(v >> 24);
  };
  std::memcpy(out, "RIFF", 4);
  le32(out + 4, static_cast<uint32_t>(total - 8));
  std::memcpy(out + 8, "WEBPVP8L", 8);
  le32(out + 16, static_cast<uint32_t>(body));
  std::memcpy(out + 20, bw.out.data(), body);
  if (body & 1) out[20 + body] = 0;
  return FG_OK;
}
