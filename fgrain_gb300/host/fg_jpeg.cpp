// JPEG files of the command-line tool (the image crate's `jpeg` feature behind image::open and
// ImageBuffer::save, src/image_pipeline.rs:1087-1152): sequential Huffman-coded DCT JPEG
// (ITU T.81, SOF0 and SOF1), 8-bit samples, one component (gray) or three (YCbCr, or RGB when an
// Adobe marker says so), any sampling factors, restart intervals, interleaved or per-component
// scans.  The encoder writes baseline JFIF: gray, or YCbCr with 2x2 chroma subsampling, the
// quality scaling of the standard's example tables, and Huffman tables built from the image's own
// symbol counts (T.81 Annex K.2), so no fixed tables are needed.  Host code only.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "fgrain_cuda.h"

namespace {

struct JpegError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// Natural position of the k-th coefficient in zigzag order.
const int kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
                         41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
                         30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

// cos((2x + 1) u pi / 16) * c(u) / 2, the 8-point DCT basis.
struct Basis {
  float m[8][8];
  Basis() {
    for (int x = 0; x < 8; ++x)
      for (int u = 0; u < 8; ++u) {
        const double cu = u == 0 ? std::sqrt(0.5) : 1.0;
        m[x][u] = static_cast<float>(0.5 * cu * std::cos((2 * x + 1) * u * M_PI / 16.0));
      }
  }
};
const Basis kBasis;

// ---------------------------------------------------------------------------------------------
// Decoding

struct Huff {
  bool set = false;
  uint8_t vals[256];
  int maxcode[18], valptr[17], mincode[17];
  void build(const uint8_t bits[16], const uint8_t* v, int n) {
    std::memcpy(vals, v, static_cast<size_t>(n));
    int code = 0, k = 0;
    for (int l = 1; l <= 16; ++l) {
      valptr[l] = k;
      mincode[l] = code;
      code += bits[l - 1];
      k += bits[l - 1];
      maxcode[l] = bits[l - 1] ? code - 1 : -1;
      code <<= 1;
    }
    maxcode[17] = 0x7fffffff;
    set = true;
  }
};

struct Component {
  int id, h, v, tq;
  int td = 0, ta = 0;
  int bw = 0, bh = 0;           // blocks per row / column of the (MCU-padded) plane
  std::vector<uint8_t> plane;   // bw*8 x bh*8 samples
  int pred = 0;
};

struct Reader {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t acc = 0;
  int bits = 0;
  bool marker = false;  // a marker ended the entropy-coded segment
  int fill() {
    while (bits <= 24) {
      uint32_t b = 0;
      if (!marker && pos < n) {
        b = p[pos];
        if (b == 0xFF) {
          const uint8_t nx = pos + 1 < n ? p[pos + 1] : 0;
          if (nx == 0x00) {
            pos += 2;
          } else {
            marker = true;  // leave the marker for the segment parser; feed zeros
            b = 0;
          }
        } else {
          ++pos;
        }
      }
      acc |= b << (24 - bits);
      bits += 8;
    }
    return bits;
  }
  int bit() {
    if (bits == 0) fill();
    const int r = static_cast<int>(acc >> 31);
    acc <<= 1;
    --bits;
    return r;
  }
  int get(int s) {
    int v = 0;
    for (int i = 0; i < s; ++i) v = (v << 1) | bit();
    return v;
  }
  void reset() {  // byte-align after a restart marker
    acc = 0;
    bits = 0;
    marker = false;
  }
};

int decode_sym(Reader& r, const Huff& h) {
  int code = r.bit();
  int l = 1;
  while (l <= 16 && code > h.maxcode[l]) {
    code = (code << 1) | r.bit();
    ++l;
  }
  if (l > 16) throw JpegError("corrupt JPEG data (bad Huffman code)");
  return h.vals[h.valptr[l] + code - h.mincode[l]];
}

inline int extend(int v, int s) { return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v; }

void idct_block(const float in[64], uint8_t* out, int stride) {
  float tmp[64];
  for (int y = 0; y < 8; ++y)
    for (int x = 0; x < 8; ++x) {  // rows: sum over u of F[y][u] basis[x][u]
      float s = 0.0f;
      for (int u = 0; u < 8; ++u) s += in[y * 8 + u] * kBasis.m[x][u];
      tmp[y * 8 + x] = s;
    }
  for (int x = 0; x < 8; ++x)
    for (int y = 0; y < 8; ++y) {
      float s = 0.0f;
      for (int v = 0; v < 8; ++v) s += tmp[v * 8 + x] * kBasis.m[y][v];
      const int q = static_cast<int>(std::lround(s + 128.0f));
      out[y * stride + x] = static_cast<uint8_t>(std::min(std::max(q, 0), 255));
    }
}

struct Decoder {
  Decoder(const uint8_t* data, size_t size) : d(data), n(size) {}
  const uint8_t* d;
  size_t n;
  size_t pos = 0;
  uint16_t q[4][64] = {};
  bool qset[4] = {false, false, false, false};
  Huff dc[4], ac[4];
  std::vector<Component> comp;
  int W = 0, H = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
  int restart = 0;
  bool adobe = false;
  int adobe_transform = -1;
  bool frame = false, done = false;

  uint16_t u16(size_t at) const {
    if (at + 2 > n) throw JpegError("truncated JPEG file");
    return static_cast<uint16_t>(d[at] << 8 | d[at + 1]);
  }

  void parse_frame(size_t at, size_t len, bool header_only) {
    if (len < 6) throw JpegError("bad JPEG frame header");
    if (d[at] != 8) throw JpegError("only 8-bit JPEG samples are supported");
    H = u16(at + 1);
    W = u16(at + 3);
    const int nf = d[at + 5];
    if (W == 0 || H == 0) throw JpegError("JPEG with a zero dimension (or a DNL marker, which is not supported)");
    if (nf != 1 && nf != 3) throw JpegError("only gray and three-component JPEG files are supported");
    if (len < static_cast<size_t>(6 + 3 * nf)) throw JpegError("bad JPEG frame header");
    comp.resize(static_cast<size_t>(nf));
    for (int i = 0; i < nf; ++i) {
      Component& c = comp[static_cast<size_t>(i)];
      c.id = d[at + 6 + 3 * i];
      c.h = d[at + 7 + 3 * i] >> 4;
      c.v = d[at + 7 + 3 * i] & 15;
      c.tq = d[at + 8 + 3 * i];
      if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3) throw JpegError("bad JPEG component parameters");
      hmax = std::max(hmax, c.h);
      vmax = std::max(vmax, c.v);
    }
    mcux = (W + 8 * hmax - 1) / (8 * hmax);
    mcuy = (H + 8 * vmax - 1) / (8 * vmax);
    if (!header_only)
      for (auto& c : comp) {
        c.bw = mcux * c.h;
        c.bh = mcuy * c.v;
        c.plane.assign(static_cast<size_t>(c.bw) * 8 * c.bh * 8, 0);
      }
    frame = true;
  }

  void decode_block(Reader& r, Component& c, int bx, int by) {
    const Huff& hd = dc[c.td];
    const Huff& ha = ac[c.ta];
    if (!hd.set || !ha.set) throw JpegError("JPEG scan uses an undefined Huffman table");
    if (!qset[c.tq]) throw JpegError("JPEG component uses an undefined quantisation table");
    float coef[64] = {};
    const int s = decode_sym(r, hd);
    if (s > 11) throw JpegError("corrupt JPEG data (DC size)");
    if (s) c.pred += extend(r.get(s), s);
    coef[0] = static_cast<float>(c.pred * q[c.tq][0]);
    for (int k = 1; k < 64;) {
      const int rs = decode_sym(r, ha);
      const int run = rs >> 4, sz = rs & 15;
      if (sz == 0) {
        if (run != 15) break;  // end of block
        k += 16;
        continue;
      }
      k += run;
      if (k > 63) throw JpegError("corrupt JPEG data (AC run)");
      coef[kZigzag[k]] = static_cast<float>(extend(r.get(sz), sz) * q[c.tq][k]);
      ++k;
    }
    const int stride = c.bw * 8;
    idct_block(coef, c.plane.data() + static_cast<size_t>(by) * 8 * stride + static_cast<size_t>(bx) * 8, stride);
  }

  // One scan: its header at `at`, its entropy-coded data right after.
  void scan(size_t at, size_t len) {
    if (!frame) throw JpegError("JPEG scan before the frame header");
    const int ns = d[at];
    if (ns < 1 || ns > 4 || len < static_cast<size_t>(1 + 2 * ns + 3)) throw JpegError("bad JPEG scan header");
    std::vector<Component*> sc;
    for (int i = 0; i < ns; ++i) {
      const int cid = d[at + 1 + 2 * i];
      Component* c = nullptr;
      for (auto& k : comp)
        if (k.id == cid) c = &k;
      if (!c) throw JpegError("JPEG scan names an unknown component");
      c->td = d[at + 2 + 2 * i] >> 4;
      c->ta = d[at + 2 + 2 * i] & 15;
      if (c->td > 3 || c->ta > 3) throw JpegError("bad JPEG Huffman table selector");
      sc.push_back(c);
    }
    const int ss = d[at + 1 + 2 * ns], se = d[at + 2 + 2 * ns], ahl = d[at + 3 + 2 * ns];
    if (ss != 0 || se != 63 || ahl != 0) throw JpegError("JPEG scan is not sequential");
    Reader r{d, n};
    r.pos = at + len;
    for (auto* c : sc) c->pred = 0;
    int left = restart;
    auto restart_marker = [&]() {
      // The segment ends at an RSTn marker: skip it and start the next interval.
      size_t p = r.pos;
      while (p + 1 < n && !(d[p] == 0xFF && d[p + 1] >= 0xD0 && d[p + 1] <= 0xD7)) ++p;
      if (p + 1 >= n) throw JpegError("JPEG restart marker missing");
      r.pos = p + 2;
      r.reset();
      for (auto* c : sc) c->pred = 0;
      left = restart;
    };
    if (ns == 1) {
      Component& c = *sc[0];
      const int cw = (W * c.h + hmax - 1) / hmax, ch = (H * c.v + vmax - 1) / vmax;
      const int nbx = (cw + 7) / 8, nby = (ch + 7) / 8;
      for (int by = 0; by < nby; ++by)
        for (int bx = 0; bx < nbx; ++bx) {
          if (restart && left == 0) restart_marker();
          decode_block(r, c, bx, by);
          if (restart) --left;
        }
    } else {
      for (int my = 0; my < mcuy; ++my)
        for (int mx = 0; mx < mcux; ++mx) {
          if (restart && left == 0) restart_marker();
          for (auto* c : sc)
            for (int v = 0; v < c->v; ++v)
              for (int h = 0; h < c->h; ++h) decode_block(r, *c, mx * c->h + h, my * c->v + v);
          if (restart) --left;
        }
    }
    // Continue parsing after the entropy-coded data: find the next marker that is not RSTn.
    size_t p = r.pos;
    while (p + 1 < n) {
      if (d[p] == 0xFF && d[p + 1] != 0x00 && !(d[p + 1] >= 0xD0 && d[p + 1] <= 0xD7) && d[p + 1] != 0xFF) break;
      ++p;
    }
    pos = p;
  }

  void run(bool header_only) {
    if (n < 4 || d[0] != 0xFF || d[1] != 0xD8) throw JpegError("not a JPEG file");
    pos = 2;
    while (pos < n && !done) {
      if (d[pos] != 0xFF) {
        ++pos;  // tolerate stray bytes between segments
        continue;
      }
      const uint8_t m = d[pos + 1 < n ? pos + 1 : pos];
      if (m == 0xFF) {
        ++pos;
        continue;
      }
      pos += 2;
      if (m == 0xD9) {  // EOI
        done = true;
        break;
      }
      if (m == 0x01 || (m >= 0xD0 && m <= 0xD7)) continue;
      const size_t len = u16(pos);
      if (len < 2 || pos + len > n) throw JpegError("truncated JPEG segment");
      const size_t at = pos + 2, body = len - 2;
      if (m == 0xC0 || m == 0xC1) {
        parse_frame(at, body, header_only);
        if (header_only) return;
      } else if (m == 0xC2 || m == 0xC6 || m == 0xCA || m == 0xCE) {
        throw JpegError("progressive JPEG is not supported");
      } else if ((m >= 0xC3 && m <= 0xCF) && m != 0xC4 && m != 0xC8 && m != 0xCC) {
        throw JpegError("arithmetic-coded, lossless and hierarchical JPEG are not supported");
      } else if (m == 0xDB) {
        size_t p = at;
        while (p < at + body) {
          const int pq = d[p] >> 4, tq = d[p] & 15;
          if (tq > 3 || pq > 1) throw JpegError("bad JPEG quantisation table");
          ++p;
          for (int k = 0; k < 64; ++k) {
            q[tq][k] = pq ? u16(p + 2 * static_cast<size_t>(k)) : d[p + static_cast<size_t>(k)];
            if (q[tq][k] == 0) q[tq][k] = 1;
          }
          p += pq ? 128 : 64;
          if (p > at + body) throw JpegError("truncated JPEG quantisation table");
          qset[tq] = true;
        }
      } else if (m == 0xC4) {
        size_t p = at;
        while (p < at + body) {
          const int tc = d[p] >> 4, th = d[p] & 15;
          if (tc > 1 || th > 3 || p + 17 > at + body) throw JpegError("bad JPEG Huffman table");
          uint8_t bits[16];
          int total = 0;
          for (int i = 0; i < 16; ++i) total += bits[i] = d[p + 1 + static_cast<size_t>(i)];
          if (total > 256 || p + 17 + static_cast<size_t>(total) > at + body) throw JpegError("bad JPEG Huffman table");
          (tc ? ac : dc)[th].build(bits, d + p + 17, total);
          p += 17 + static_cast<size_t>(total);
        }
      } else if (m == 0xDD) {
        restart = u16(at);
      } else if (m == 0xEE && body >= 12 && std::memcmp(d + at, "Adobe", 5) == 0) {
        adobe = true;
        adobe_transform = d[at + 11];
      } else if (m == 0xDA) {
        if (header_only) throw JpegError("JPEG scan before the frame header");
        scan(at, body);
        continue;  // scan() set pos past the entropy-coded data
      }
      pos += len;
    }
    if (!frame) throw JpegError("JPEG without a frame header");
  }

  // Upsampled, colour-converted output (gray or RGB).
  // One axis of the sample of component c at output position x (n output positions): the
  // component's two nearest samples and the weight of the second.  A component at half the
  // resolution has its samples centred between output pairs (x maps to x / 2 - 1/4), so it is
  // interpolated linearly, 3/4 and 1/4, clamped at the edges; other ratios take the nearest.
  static void axis(int x, int f, int fmax, int n, int& i0, int& i1, float& w1) {
    w1 = 0.0f;
    if (2 * f == fmax) {
      const int m = (n * f + fmax - 1) / fmax;  // samples that cover the image
      i0 = x / 2;
      i1 = std::min(std::max((x & 1) ? i0 + 1 : i0 - 1, 0), m - 1);
      w1 = 0.25f;
    } else {
      i0 = i1 = x * f / fmax;
    }
  }
  float upsampled(const Component& c, int x, int y) const {
    int x0, x1, y0, y1;
    float wx, wy;
    axis(x, c.h, hmax, W, x0, x1, wx);
    axis(y, c.v, vmax, H, y0, y1, wy);
    const size_t stride = static_cast<size_t>(c.bw) * 8;
    auto at = [&](int yy, int xx) { return static_cast<float>(c.plane[static_cast<size_t>(yy) * stride + static_cast<size_t>(xx)]); };
    const float top = (1.0f - wx) * at(y0, x0) + wx * at(y0, x1);
    const float bottom = (1.0f - wx) * at(y1, x0) + wx * at(y1, x1);
    return (1.0f - wy) * top + wy * bottom;
  }

  void output(uint8_t* out) const {
    const int nc = static_cast<int>(comp.size());
    if (nc == 1) {
      const Component& c = comp[0];
      for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
          out[static_cast<size_t>(y) * W + x] =
              c.plane[static_cast<size_t>(y * c.v / vmax) * c.bw * 8 + static_cast<size_t>(x * c.h / hmax)];
      return;
    }
    const bool rgb = adobe ? adobe_transform == 0 : (comp[0].id == 'R' && comp[1].id == 'G' && comp[2].id == 'B');
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        float s[3];
        for (int k = 0; k < 3; ++k) s[k] = upsampled(comp[static_cast<size_t>(k)], x, y);
        uint8_t* o = out + (static_cast<size_t>(y) * W + x) * 3;
        if (rgb) {
          for (int k = 0; k < 3; ++k) o[k] = static_cast<uint8_t>(std::min(std::max(std::lround(s[k]), 0L), 255L));
          continue;
        }
        // JFIF YCbCr to RGB.
        const float Y = s[0], cb = s[1] - 128.0f, cr = s[2] - 128.0f;
        const float v[3] = {Y + 1.402f * cr, Y - 0.344136f * cb - 0.714136f * cr, Y + 1.772f * cb};
        for (int k = 0; k < 3; ++k) o[k] = static_cast<uint8_t>(std::min(std::max(std::lround(v[k]), 0L), 255L));
      }
  }
};

// ---------------------------------------------------------------------------------------------
// Encoding

// The standard's example quantisation tables (T.81 Annex K.1, K.2), natural order.
const int kLumaQ[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                        14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                        18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                        49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const int kChromaQ[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99, 24, 26, 56, 99, 99, 99,
                          99, 99, 47, 66, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                          99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};

struct Writer {
  std::vector<uint8_t> out;
  uint32_t acc = 0;
  int bits = 0;
  void put(uint32_t v, int n) {
    for (int i = n - 1; i >= 0; --i) {
      acc = (acc << 1) | ((v >> i) & 1u);
      if (++bits == 8) {
        out.push_back(static_cast<uint8_t>(acc));
        if ((acc & 0xFF) == 0xFF) out.push_back(0);  // byte stuffing
        acc = 0;
        bits = 0;
      }
    }
  }
  void flush() {
    if (bits) put((1u << (8 - bits)) - 1u, 8 - bits);  // pad with ones
  }
  void u8(int v) { out.push_back(static_cast<uint8_t>(v)); }
  void u16(int v) {
    u8(v >> 8);
    u8(v & 255);
  }
};

// Code lengths limited to 16 bits from symbol counts (T.81 Annex K.2: Huffman code sizes, then
// the adjustment that moves codes longer than 16 bits), then canonical codes.
struct EncHuff {
  uint8_t bits[16] = {};
  std::vector<uint8_t> vals;
  uint16_t code[256] = {};
  uint8_t size[256] = {};
  void build(const std::vector<long>& freq_in) {
    std::vector<long> freq(257, 0);
    for (int i = 0; i < 256; ++i) freq[static_cast<size_t>(i)] = freq_in[static_cast<size_t>(i)];
    freq[256] = 1;  // a reserved symbol so that no code is all ones
    std::vector<int> codesize(257, 0), others(257, -1);
    for (;;) {
      int v1 = -1, v2 = -1;
      for (int i = 0; i < 257; ++i) {
        if (freq[static_cast<size_t>(i)] == 0) continue;
        if (v1 < 0 || freq[static_cast<size_t>(i)] <= freq[static_cast<size_t>(v1)]) v1 = i;
      }
      for (int i = 0; i < 257; ++i) {
        if (freq[static_cast<size_t>(i)] == 0 || i == v1) continue;
        if (v2 < 0 || freq[static_cast<size_t>(i)] <= freq[static_cast<size_t>(v2)]) v2 = i;
      }
      if (v2 < 0) break;
      freq[static_cast<size_t>(v1)] += freq[static_cast<size_t>(v2)];
      freq[static_cast<size_t>(v2)] = 0;
      for (++codesize[static_cast<size_t>(v1)]; others[static_cast<size_t>(v1)] >= 0;) {
        v1 = others[static_cast<size_t>(v1)];
        ++codesize[static_cast<size_t>(v1)];
      }
      others[static_cast<size_t>(v1)] = v2;
      for (++codesize[static_cast<size_t>(v2)]; others[static_cast<size_t>(v2)] >= 0;) {
        v2 = others[static_cast<size_t>(v2)];
        ++codesize[static_cast<size_t>(v2)];
      }
    }
    int cnt[33] = {};
    for (int i = 0; i < 257; ++i)
      if (codesize[static_cast<size_t>(i)]) ++cnt[std::min(codesize[static_cast<size_t>(i)], 32)];
    for (int i = 32; i > 16; --i) {
      while (cnt[i] > 0) {
        int j = i - 2;
        while (cnt[j] == 0) --j;
        cnt[i] -= 2;
        ++cnt[i - 1];
        cnt[j + 1] += 2;
        --cnt[j];
      }
    }
    int i = 16;
    while (cnt[i] == 0) --i;
    --cnt[i];  // drop the reserved symbol
    for (int l = 1; l <= 16; ++l) bits[l - 1] = static_cast<uint8_t>(cnt[l]);
    // Symbols sorted by code size (then value), as the canonical code assigns them.
    vals.clear();
    for (int l = 1; l <= 32; ++l)
      for (int s = 0; s < 256; ++s)
        if (codesize[static_cast<size_t>(s)] == l) vals.push_back(static_cast<uint8_t>(s));
    int k = 0, c = 0;
    for (int l = 1; l <= 16; ++l) {
      for (int m = 0; m < bits[l - 1]; ++m, ++k) {
        code[vals[static_cast<size_t>(k)]] = static_cast<uint16_t>(c++);
        size[vals[static_cast<size_t>(k)]] = static_cast<uint8_t>(l);
      }
      c <<= 1;
    }
    vals.resize(static_cast<size_t>(k));
  }
};

inline int nbits(int v) {
  v = v < 0 ? -v : v;
  int n = 0;
  while (v) {
    ++n;
    v >>= 1;
  }
  return n;
}

struct Block {
  int16_t c[64];  // quantised, zigzag order
};

void fdct_quant(const float in[64], const int qz[64], Block& b) {
  float tmp[64], coef[64];
  for (int y = 0; y < 8; ++y)  // rows: tmp[y][u] = sum over x of in[y][x] basis[x][u]
    for (int u = 0; u < 8; ++u) {
      float s = 0.0f;
      for (int x = 0; x < 8; ++x) s += in[y * 8 + x] * kBasis.m[x][u];
      tmp[y * 8 + u] = s;
    }
  for (int u = 0; u < 8; ++u)  // columns: coef[v][u] = sum over y of tmp[y][u] basis[y][v]
    for (int v = 0; v < 8; ++v) {
      float s = 0.0f;
      for (int y = 0; y < 8; ++y) s += tmp[y * 8 + u] * kBasis.m[y][v];
      coef[v * 8 + u] = s;
    }
  // Baseline codes DC differences of at most 11 bits and AC values of at most 10: clamp to
  // +-1023 (it only bites at quality 100).
  for (int k = 0; k < 64; ++k) {
    const long v = std::lround(coef[kZigzag[k]] / static_cast<float>(qz[k]));
    b.c[k] = static_cast<int16_t>(std::min(std::max(v, -1023L), 1023L));
  }
}

}  // namespace

extern "C" fg_status fg_jpeg_info(const uint8_t* data, size_t n, uint32_t* w, uint32_t* h, uint32_t* channels,
                                  char* msg, size_t msg_cap) {
  if (!data || !w || !h || !channels) return FG_ERR_INVALID_ARG;
  try {
    Decoder dec(data, n);
    dec.run(true);
    *w = static_cast<uint32_t>(dec.W);
    *h = static_cast<uint32_t>(dec.H);
    *channels = static_cast<uint32_t>(dec.comp.size());
    return FG_OK;
  } catch (const std::exception& e) {
    if (msg && msg_cap) std::snprintf(msg, msg_cap, "%s", e.what());
    return FG_ERR_INVALID_ARG;
  }
}

extern "C" fg_status fg_jpeg_decode(const uint8_t* data, size_t n, uint8_t* out, size_t cap, char* msg,
                                    size_t msg_cap) {
  if (!data || !out) return FG_ERR_INVALID_ARG;
  try {
    Decoder dec(data, n);
    dec.run(false);
    if (static_cast<size_t>(dec.W) * dec.H * dec.comp.size() > cap) throw JpegError("output buffer too small");
    dec.output(out);
    return FG_OK;
  } catch (const std::exception& e) {
    if (msg && msg_cap) std::snprintf(msg, msg_cap, "%s", e.what());
    return FG_ERR_INVALID_ARG;
  }
}

extern "C" fg_status fg_jpeg_encode(const uint8_t* px, uint32_t w, uint32_t h, uint32_t channels, uint32_t quality,
                                    uint32_t options, uint8_t* out, size_t cap, size_t* len) {
  const uint32_t sub = options & 3u;
  if (!px || !out || !len || w == 0 || h == 0 || w > 65535 || h > 65535 || (channels != 1 && channels != 3) ||
      quality < 1 || quality > 100 || sub == 3u || (options & 0xFFF8u) != 0)
    return FG_ERR_INVALID_ARG;
  // IJG quality scaling of the example tables.
  const int scale = quality < 50 ? 5000 / static_cast<int>(quality) : 200 - 2 * static_cast<int>(quality);
  int qz[2][64];
  for (int k = 0; k < 64; ++k) {
    qz[0][k] = std::min(std::max((kLumaQ[kZigzag[k]] * scale + 50) / 100, 1), 255);
    qz[1][k] = std::min(std::max((kChromaQ[kZigzag[k]] * scale + 50) / 100, 1), 255);
  }
  const int nc = static_cast<int>(channels);
  const bool separate = (options & FG_JPEG_SEPARATE_SCANS) != 0 && nc == 3;
  const int restart = static_cast<int>(options >> 16);
  // Luma sampling factors (chroma components are 1x1): 4:2:0, 4:2:2 or 4:4:4.
  const int hs = nc == 3 && sub != FG_JPEG_SUBSAMPLE_444 ? 2 : 1;
  const int vs = nc == 3 && sub == FG_JPEG_SUBSAMPLE_420 ? 2 : 1;
  const int iw = static_cast<int>(w), ih = static_cast<int>(h);
  const int mx = (iw + 8 * hs - 1) / (8 * hs), my = (ih + 8 * vs - 1) / (8 * vs);
  auto sample = [&](int x, int y, int k) -> float {  // edge pixels replicated past the image
    x = std::min(x, iw - 1);
    y = std::min(y, ih - 1);
    const uint8_t* p = px + (static_cast<size_t>(y) * w + static_cast<size_t>(x)) * static_cast<size_t>(nc);
    if (nc == 1) return p[0];
    const float r = p[0], g = p[1], b = p[2];
    if (k == 0) return 0.299f * r + 0.587f * g + 0.114f * b;
    if (k == 1) return -0.168736f * r - 0.331264f * g + 0.5f * b + 128.0f;
    return 0.5f * r - 0.418688f * g - 0.081312f * b + 128.0f;
  };
  // Quantised blocks of each component over the MCU grid (row-major, gw x gh blocks); chroma
  // samples are hs x vs box averages.
  struct Plane {
    int H, V, gw, gh, bw, bh;  // sampling factors, block grid, blocks covering the component
    std::vector<Block> b;
  };
  std::vector<Plane> pl(static_cast<size_t>(nc));
  for (int k = 0; k < nc; ++k) {
    Plane& P = pl[static_cast<size_t>(k)];
    P.H = k ? 1 : hs;
    P.V = k ? 1 : vs;
    P.gw = mx * P.H;
    P.gh = my * P.V;
    P.bw = ((iw * P.H + hs - 1) / hs + 7) / 8;
    P.bh = ((ih * P.V + vs - 1) / vs + 7) / 8;
    P.b.resize(static_cast<size_t>(P.gw) * P.gh);
    const int fx = hs / P.H, fy = vs / P.V;  // pixels per sample
    for (int by = 0; by < P.gh; ++by)
      for (int bx = 0; bx < P.gw; ++bx) {
        float in[64];
        for (int y = 0; y < 8; ++y)
          for (int x = 0; x < 8; ++x) {
            float acc = 0.0f;
            for (int dy = 0; dy < fy; ++dy)
              for (int dx = 0; dx < fx; ++dx) acc += sample((bx * 8 + x) * fx + dx, (by * 8 + y) * fy + dy, k);
            in[y * 8 + x] = acc / static_cast<float>(fx * fy) - 128.0f;
          }
        Block& blk = P.b[static_cast<size_t>(by) * P.gw + bx];
        blk = Block{};
        fdct_quant(in, qz[k ? 1 : 0], blk);
      }
  }
  // The scans: one interleaved scan of MCUs, or one scan per component whose MCU is a single
  // block and which covers only the blocks the component needs.  emit_rst(m) ends the m-th
  // restart interval (not after the scan's last MCU); DC predictions restart with it.
  auto walk = [&](auto&& emit_dc, auto&& emit_ac, auto&& emit_rst, auto&& begin_scan) {
    auto block = [&](int k, const Block& b, int pred[3]) {
      const int t = k ? 1 : 0;
      const int diff = b.c[0] - pred[k];
      pred[k] = b.c[0];
      emit_dc(t, diff);
      int run = 0;
      for (int z = 1; z < 64; ++z) {
        const int v = b.c[z];
        if (v == 0) {
          ++run;
          continue;
        }
        while (run > 15) {
          emit_ac(t, 0xF0, 0, 0);
          run -= 16;
        }
        emit_ac(t, (run << 4) | nbits(v), v, nbits(v));
        run = 0;
      }
      if (run) emit_ac(t, 0x00, 0, 0);
    };
    const int nscans = separate ? nc : 1;
    for (int sc = 0; sc < nscans; ++sc) {
      begin_scan(sc);
      int pred[3] = {0, 0, 0};
      const long total = separate ? static_cast<long>(pl[static_cast<size_t>(sc)].bw) * pl[static_cast<size_t>(sc)].bh
                                  : static_cast<long>(mx) * my;
      for (long m = 0; m < total; ++m) {
        if (separate) {
          const Plane& P = pl[static_cast<size_t>(sc)];
          const int bx = static_cast<int>(m % P.bw), by = static_cast<int>(m / P.bw);
          block(sc, P.b[static_cast<size_t>(by) * P.gw + bx], pred);
        } else {
          const int ux = static_cast<int>(m % mx), uy = static_cast<int>(m / mx);
          for (int k = 0; k < nc; ++k) {
            const Plane& P = pl[static_cast<size_t>(k)];
            for (int v = 0; v < P.V; ++v)
              for (int u = 0; u < P.H; ++u)
                block(k, P.b[static_cast<size_t>(uy * P.V + v) * P.gw + (ux * P.H + u)], pred);
          }
        }
        if (restart && (m + 1) % restart == 0 && m + 1 < total) {
          emit_rst(static_cast<int>(((m + 1) / restart - 1) & 7));
          pred[0] = pred[1] = pred[2] = 0;
        }
      }
    }
  };
  // Symbol counts, then the tables (luma 0, chroma 1).
  std::vector<long> fdc[2] = {std::vector<long>(256, 0), std::vector<long>(256, 0)};
  std::vector<long> fac[2] = {std::vector<long>(256, 0), std::vector<long>(256, 0)};
  walk([&](int t, int diff) { ++fdc[t][static_cast<size_t>(nbits(diff))]; },
       [&](int t, int sym, int, int) { ++fac[t][static_cast<size_t>(sym)]; }, [](int) {}, [](int) {});
  const int ntab = nc == 3 ? 2 : 1;
  EncHuff hdc[2], hac[2];
  for (int t = 0; t < ntab; ++t) {
    hdc[t].build(fdc[t]);
    hac[t].build(fac[t]);
  }
  Writer wr;
  wr.u16(0xFFD8);
  wr.u16(0xFFE0);  // JFIF APP0
  wr.u16(16);
  for (char ch : std::string("JFIF")) wr.u8(ch);
  wr.u8(0);
  wr.u16(0x0101);
  wr.u8(0);
  wr.u16(1);
  wr.u16(1);
  wr.u8(0);
  wr.u8(0);
  for (int t = 0; t < ntab; ++t) {  // DQT
    wr.u16(0xFFDB);
    wr.u16(67);
    wr.u8(t);
    for (int k = 0; k < 64; ++k) wr.u8(qz[t][k]);
  }
  wr.u16(0xFFC0);  // SOF0
  wr.u16(8 + 3 * nc);
  wr.u8(8);
  wr.u16(ih);
  wr.u16(iw);
  wr.u8(nc);
  for (int k = 0; k < nc; ++k) {
    wr.u8(k + 1);
    wr.u8(pl[static_cast<size_t>(k)].H << 4 | pl[static_cast<size_t>(k)].V);
    wr.u8(k ? 1 : 0);
  }
  for (int t = 0; t < ntab; ++t)  // DHT
    for (int cls = 0; cls < 2; ++cls) {
      const EncHuff& e = cls ? hac[t] : hdc[t];
      wr.u16(0xFFC4);
      wr.u16(19 + static_cast<int>(e.vals.size()));
      wr.u8(cls << 4 | t);
      for (int l = 0; l < 16; ++l) wr.u8(e.bits[l]);
      for (uint8_t v : e.vals) wr.u8(v);
    }
  if (restart) {  // DRI
    wr.u16(0xFFDD);
    wr.u16(4);
    wr.u16(restart);
  }
  walk(
      [&](int t, int diff) {
        const int s = nbits(diff);
        wr.put(hdc[t].code[s], hdc[t].size[s]);
        if (s) wr.put(static_cast<uint32_t>(diff < 0 ? diff + (1 << s) - 1 : diff), s);
      },
      [&](int t, int sym, int v, int s) {
        wr.put(hac[t].code[sym], hac[t].size[sym]);
        if (s) wr.put(static_cast<uint32_t>(v < 0 ? v + (1 << s) - 1 : v), s);
      },
      [&](int m) {
        wr.flush();
        wr.u16(0xFFD0 + m);
      },
      [&](int sc) {
        wr.flush();
        const int first = separate ? sc : 0, ns = separate ? 1 : nc;
        wr.u16(0xFFDA);  // SOS
        wr.u16(6 + 2 * ns);
        wr.u8(ns);
        for (int k = first; k < first + ns; ++k) {
          wr.u8(k + 1);
          wr.u8(k ? 0x11 : 0x00);
        }
        wr.u8(0);
        wr.u8(63);
        wr.u8(0);
      });
  wr.flush();
  wr.u16(0xFFD9);
  *len = wr.out.size();
  if (wr.out.size() > cap) return FG_ERR_INVALID_ARG;
  std::memcpy(out, wr.out.data(), wr.out.size());
  return FG_OK;
}
