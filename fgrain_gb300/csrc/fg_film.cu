// Whole photographs on the device: the reference's film renderer around the tile path
// (render_film_black_and_white_tiled and render_film_color_tiled, image_pipeline.rs:299-891 and
// 1017-1085).  Every stage is a memory-bound stencil or pointwise pass in FP32 that keeps the
// reference's operation order (no fused multiply-add), so that the integer and u8 stages (luma,
// resize, gate detection, tile gather) and the PSF and low-pass fields match the CPU bit for bit:
//
//   luma            k_luma                  image_pipeline.rs:259-296
//   resize          k_resample_v/h_u8       image_pipeline.rs:315-342 (image crate's Triangle and
//                                           Lanczos3; weights on the host, passes on the device)
//   camera gate     k_gate_flags/bounds     image_pipeline.rs:137-155
//   gelatin PSF     k_psf_h, k_psf_v        image_pipeline.rs:157-252
//   tile gather     k_gather_tiles          image_pipeline.rs:444-452 (h_effective -> tile)
//   tiles           the batched tile path (fg_batch.cu), one batch for all tiles of all channels
//   blend           k_blend_film            image_pipeline.rs:593-655 (with the weight sums)
//   low-pass        k_gauss_pass x 2        image_pipeline.rs:657-706
//   grain stats     k_high_sum, k_high_fin  image_pipeline.rs:708-716 (FP64 tree sums in a fixed
//                                           order: deterministic; the reference's are sequential
//                                           f32 sums, so its mean and deviation carry rounding
//                                           error of order sqrt(n) ulp that these do not)
//   composite       k_grain                 image_pipeline.rs:725-808
//   scanner OTF     k_otf_pass + k_film_out image_pipeline.rs:825-891 (with the output gates)
//
// The composite calls CUDA's single-precision powf and sinf where the reference calls the C
// library's; the two may differ in the last places, so final pixels may differ by one level where
// a value lies on a rounding boundary.  (FP64 versions would cost the composite ten times more on
// GB300's narrow FP64 pipe.)
#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "fg_image.cuh"

namespace fg {

namespace {

struct FilmGate {
  uint32_t top, bottom, left, right;
};

struct GatherTile {
  const float* img;  // the layer's h_effective, W floats per row
  float* dst;
  uint32_t W, xs, ys, tw, th;
};

struct CopyTile {
  const float* src;
  float* dst;
  unsigned long long n;
};

struct FilmTile {
  const float* d;
  uint32_t tx, ty, xs, ys, tw, th;
};

__device__ __forceinline__ float gate_shadow(float v) {
  const float toe_min = 0.005f, toe_max = 0.14f;
  if (v <= toe_min) return 0.0f;
  if (v >= toe_max) return 1.0f;
  const float t = __fdiv_rn(__fsub_rn(v, toe_min), __fsub_rn(toe_max, toe_min));
  return __fmul_rn(__fmul_rn(t, t), __fsub_rn(3.0f, __fmul_rn(2.0f, t)));
}

__device__ __forceinline__ float gate_highlight(float v) {
  if (v <= 0.65f) return 1.0f;
  if (v >= 0.94f) return 0.0f;
  const float u = __fdiv_rn(__fsub_rn(v, 0.65f), __fsub_rn(0.94f, 0.65f));
  return __fsub_rn(1.0f, __fmul_rn(__fmul_rn(u, u), __fsub_rn(3.0f, __fmul_rn(2.0f, u))));
}

__global__ void k_luma(const uint8_t* __restrict__ rgb, size_t n, float rw, float gw, float bw,
                       uint8_t* __restrict__ out) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
  float v = __fadd_rn(__fadd_rn(__fmul_rn(r, rw), __fmul_rn(g, gw)), __fmul_rn(b, bw));
  v = v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v);
  out[i] = static_cast<uint8_t>(roundf(v));
}

__global__ void k_channel(const uint8_t* __restrict__ rgb, size_t n, int c, uint8_t* __restrict__ out) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = rgb[3 * i + c];
}

__global__ void k_interleave(const uint8_t* __restrict__ r, const uint8_t* __restrict__ g,
                             const uint8_t* __restrict__ b, size_t n, uint8_t* __restrict__ out) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  out[3 * i] = r[i];
  out[3 * i + 1] = g[i];
  out[3 * i + 2] = b[i];
}

// Vertical pass of the resampler: u8 in, f32 out (w x oh), taps summed in order.
__global__ void k_resample_v_u8(const uint8_t* __restrict__ in, uint32_t w, const uint32_t* __restrict__ left,
                                const uint32_t* __restrict__ cnt, const float* __restrict__ wts, uint32_t stride,
                                uint32_t oh, float* __restrict__ out) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(w) * oh) return;
  const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>(i / w);
  const float* wy = wts + static_cast<size_t>(y) * stride;
  float t = 0.0f;
  for (uint32_t k = 0; k < cnt[y]; ++k)
    t = __fadd_rn(t, __fmul_rn(static_cast<float>(in[static_cast<size_t>(left[y] + k) * w + x]), wy[k]));
  out[i] = t;
}

// Horizontal pass: f32 in (w x oh), u8 out (ow x oh), clamped to [0, 255] and rounded half away.
__global__ void k_resample_h_u8(const float* __restrict__ in, uint32_t w, const uint32_t* __restrict__ left,
                                const uint32_t* __restrict__ cnt, const float* __restrict__ wts, uint32_t stride,
                                uint32_t ow, uint32_t oh, uint8_t* __restrict__ out) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(ow) * oh) return;
  const uint32_t x = static_cast<uint32_t>(i % ow), y = static_cast<uint32_t>(i / ow);
  const float* wx = wts + static_cast<size_t>(x) * stride;
  const float* row = in + static_cast<size_t>(y) * w + left[x];
  float t = 0.0f;
  for (uint32_t k = 0; k < cnt[x]; ++k) t = __fadd_rn(t, __fmul_rn(row[k], wx[k]));
  t = t < 0.0f ? 0.0f : (t > 255.0f ? 255.0f : t);
  out[i] = static_cast<uint8_t>(roundf(t));
}

// Rows and columns holding a non-zero pixel (plain stores of 1: order does not matter).
__global__ void k_gate_flags(const uint8_t* __restrict__ src, uint32_t w, uint32_t h, uint32_t* rowany,
                             uint32_t* colany) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(w) * h || !src[i]) return;
  rowany[i / w] = 1u;
  colany[i % w] = 1u;
}

// The camera gate: first and one-past-last non-zero row, and the same for columns.  A column that
// is zero over the gate's rows is zero over all rows (the rows outside the gate are all zero).
__global__ void k_gate_bounds(const uint32_t* __restrict__ rowany, const uint32_t* __restrict__ colany, uint32_t w,
                              uint32_t h, FilmGate* gate) {
  __shared__ unsigned top, last_row, left, last_col;
  if (threadIdx.x == 0) {
    top = h;
    left = w;
    last_row = 0;
    last_col = 0;
  }
  __syncthreads();
  for (uint32_t y = threadIdx.x; y < h; y += blockDim.x)
    if (rowany[y]) {
      atomicMin(&top, y);
      atomicMax(&last_row, y + 1);
    }
  for (uint32_t x = threadIdx.x; x < w; x += blockDim.x)
    if (colany[x]) {
      atomicMin(&left, x);
      atomicMax(&last_col, x + 1);
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    FilmGate g;
    g.top = top;
    g.bottom = top == h ? h : last_row;
    g.left = left;
    g.right = left == w ? w : last_col;
    *gate = g;
  }
}

__constant__ float c_psf_narrow[3] = {0.15f, 0.70f, 0.15f};
__constant__ float c_psf_wide[7] = {0.03f, 0.12f, 0.20f, 0.30f, 0.20f, 0.12f, 0.03f};

// Horizontal PSF passes (narrow 3-tap and wide 7-tap) over the linear exposure inside the gate,
// each normalised by the weight of the taps inside the gate.
__global__ void k_psf_h(const uint8_t* __restrict__ src, uint32_t w, uint32_t h, const FilmGate* __restrict__ gp,
                        float* __restrict__ tn, float* __restrict__ tw) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(w) * h) return;
  const FilmGate g = *gp;
  const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>(i / w);
  if (y < g.top || y >= g.bottom || x < g.left || x >= g.right) {
    tn[i] = 0.0f;
    tw[i] = 0.0f;
    return;
  }
  const uint8_t* row = src + static_cast<size_t>(y) * w;
  float s = 0.0f, ws = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int tap = static_cast<int>(x) + k - 1;
    if (tap >= static_cast<int>(g.left) && tap < static_cast<int>(g.right)) {
      s = __fadd_rn(s, __fmul_rn(__fdiv_rn(static_cast<float>(row[tap]), 255.0f), c_psf_narrow[k]));
      ws = __fadd_rn(ws, c_psf_narrow[k]);
    }
  }
  tn[i] = __fdiv_rn(s, fmaxf(ws, 1e-6f));
  s = 0.0f;
  ws = 0.0f;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    const int tap = static_cast<int>(x) + k - 3;
    if (tap >= static_cast<int>(g.left) && tap < static_cast<int>(g.right)) {
      s = __fadd_rn(s, __fmul_rn(__fdiv_rn(static_cast<float>(row[tap]), 255.0f), c_psf_wide[k]));
      ws = __fadd_rn(ws, c_psf_wide[k]);
    }
  }
  tw[i] = __fdiv_rn(s, fmaxf(ws, 1e-6f));
}

// Vertical PSF passes and the 90 / 10 mix of the two components; zero outside the gate.
__global__ void k_psf_v(const float* __restrict__ tn, const float* __restrict__ tw, uint32_t w, uint32_t h,
                        const FilmGate* __restrict__ gp, float* __restrict__ heff) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(w) * h) return;
  const FilmGate g = *gp;
  const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>(i / w);
  if (y < g.top || y >= g.bottom || x < g.left || x >= g.right) {
    heff[i] = 0.0f;
    return;
  }
  float s = 0.0f, ws = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int tap = static_cast<int>(y) + k - 1;
    if (tap >= static_cast<int>(g.top) && tap < static_cast<int>(g.bottom)) {
      s = __fadd_rn(s, __fmul_rn(tn[static_cast<size_t>(tap) * w + x], c_psf_narrow[k]));
      ws = __fadd_rn(ws, c_psf_narrow[k]);
    }
  }
  const float on = __fdiv_rn(s, fmaxf(ws, 1e-6f));
  s = 0.0f;
  ws = 0.0f;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    const int tap = static_cast<int>(y) + k - 3;
    if (tap >= static_cast<int>(g.top) && tap < static_cast<int>(g.bottom)) {
      s = __fadd_rn(s, __fmul_rn(tw[static_cast<size_t>(tap) * w + x], c_psf_wide[k]));
      ws = __fadd_rn(ws, c_psf_wide[k]);
    }
  }
  const float ow = __fdiv_rn(s, fmaxf(ws, 1e-6f));
  heff[i] = __fadd_rn(__fmul_rn(0.90f, on), __fmul_rn(0.10f, ow));
}

// h_effective -> the batch's exposure tiles; blockIdx.y is the tile.
__global__ void k_gather_tiles(const GatherTile* __restrict__ tiles) {
  const GatherTile t = tiles[blockIdx.y];
  const size_t n = static_cast<size_t>(t.tw) * t.th;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const uint32_t px = static_cast<uint32_t>(i % t.tw), py = static_cast<uint32_t>(i / t.tw);
    t.dst[i] = t.img[static_cast<size_t>(t.ys + py) * t.W + t.xs + px];
  }
}

// Tile densities of a batch -> the image's density array; blockIdx.y is the tile.
__global__ void k_copy_tiles(const CopyTile* __restrict__ tiles) {
  const CopyTile t = tiles[blockIdx.y];
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < t.n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
    t.dst[i] = t.src[i];
}

// Hann weights along one axis, once per image: tab[3 g + 1 + d] is the weight at coordinate g of
// the tile in grid column (or row) g / step + d, d in -1..1 (0 where there is no such tile).
__global__ void k_hann_table(uint32_t n, uint32_t nt, uint32_t step, uint32_t pad, float* __restrict__ tab) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const int c = static_cast<int>(g / step);
  for (int d = -1; d <= 1; ++d) {
    const int t = c + d;
    tab[3 * g + 1 + d] = (t >= 0 && t < static_cast<int>(nt))
                             ? hann_weight(static_cast<uint32_t>(t), g, nt, static_cast<uint32_t>(t) * step, step, pad)
                             : 0.0f;
  }
}

// Hann overlap blend with the weight sums (image_pipeline.rs:593-655): d_norm and the
// equal-power grain scale min(1 / sqrt(max(sum w^2 / max(sum w, 1e-5)^2, 0.05)), 1.45).
__global__ void k_blend_film(const FilmTile* __restrict__ tiles, uint32_t ntiles, uint32_t ntx, uint32_t nty,
                             uint32_t step, const float* __restrict__ hx, const float* __restrict__ hy,
                             uint32_t out_w, uint32_t out_h, float* __restrict__ d_norm, float* __restrict__ gscale) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(out_w) * out_h) return;
  const uint32_t gx = static_cast<uint32_t>(i % out_w), gy = static_cast<uint32_t>(i / out_w);
  const uint32_t cx = gx / step, cy = gy / step;
  float acc = 0.0f, wacc = 0.0f, wsq = 0.0f;
  for (int dy = -1; dy <= 1; ++dy) {
    const int ty = static_cast<int>(cy) + dy;
    if (ty < 0 || ty >= static_cast<int>(nty)) continue;
    for (int dx = -1; dx <= 1; ++dx) {
      const int tx = static_cast<int>(cx) + dx;
      if (tx < 0 || tx >= static_cast<int>(ntx)) continue;
      const uint32_t k = static_cast<uint32_t>(ty) * ntx + static_cast<uint32_t>(tx);
      if (k >= ntiles) continue;
      const FilmTile T = tiles[k];
      if (gx < T.xs || gx >= T.xs + T.tw || gy < T.ys || gy >= T.ys + T.th) continue;
      const float wy = hy[3 * gy + 1 + dy];
      const float wx = hx[3 * gx + 1 + dx];
      const float wv = __fmul_rn(wx, wy);
      const float v = T.d[static_cast<size_t>(gy - T.ys) * T.tw + (gx - T.xs)];
      acc = __fadd_rn(acc, __fmul_rn(v, wv));
      wacc = __fadd_rn(wacc, wv);
      wsq = __fadd_rn(wsq, __fmul_rn(wv, wv));
    }
  }
  const float w_val = fmaxf(wacc, 1e-5f);
  d_norm[i] = __fdiv_rn(acc, w_val);
  const float wsn = fmaxf(__fdiv_rn(wsq, __fmul_rn(w_val, w_val)), 0.05f);
  gscale[i] = fminf(__fdiv_rn(1.0f, __fsqrt_rn(wsn)), 1.45f);
}

// One pass of the low-pass Gaussian, normalised by the weight of the taps inside the image.
__global__ void k_gauss_pass(const float* __restrict__ in, uint32_t w, uint32_t h, const float* __restrict__ kern,
                             int krad, int axis, float* __restrict__ out) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(w) * h) return;
  const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>(i / w);
  const int c = axis == 0 ? static_cast<int>(x) : static_cast<int>(y);
  const int n = axis == 0 ? static_cast<int>(w) : static_cast<int>(h);
  const size_t stride = axis == 0 ? 1 : w;
  const float* base = axis == 0 ? in + static_cast<size_t>(y) * w : in + x;
  float s = 0.0f, ws = 0.0f;
  for (int k = 0; k <= 2 * krad; ++k) {
    const int tap = c + k - krad;
    if (tap >= 0 && tap < n) {
      s = __fadd_rn(s, __fmul_rn(base[static_cast<size_t>(tap) * stride], kern[k]));
      ws = __fadd_rn(ws, kern[k]);
    }
  }
  out[i] = __fdiv_rn(s, fmaxf(ws, 1e-6f));
}

constexpr int STAT_THREADS = 256;
constexpr int STAT_BLOCKS = 1024;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < STAT_THREADS / 32; ++k) t += sh[k];
  return t;
}

// Per-block FP64 partial sums of d_high = d_norm - d_low (phase 0) or of (d_high - mean)^2
// (phase 1), in a fixed order for a fixed launch shape.
__global__ void __launch_bounds__(STAT_THREADS) k_high_sum(const float* __restrict__ dn, const float* __restrict__ dl,
                                                           size_t n, const float* __restrict__ stats, int phase,
                                                           double* __restrict__ part) {
  __shared__ double sh[STAT_THREADS / 32];
  const float mean = phase ? stats[0] : 0.0f;
  double s = 0.0;
  for (size_t i = blockIdx.x * static_cast<size_t>(STAT_THREADS) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * STAT_THREADS) {
    const float d = __fsub_rn(dn[i], dl[i]);
    if (phase) {
      const float e = __fsub_rn(d, mean);
      s += static_cast<double>(__fmul_rn(e, e));
    } else {
      s += static_cast<double>(d);
    }
  }
  const double t = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Sum of the partials: phase 0 writes the mean, phase 1 the deviation max(sqrt(var), 0.035) and
// the grain normalisation min(amp / deviation, 2.2).
__global__ void __launch_bounds__(STAT_THREADS) k_high_fin(const double* __restrict__ part, int nb, size_t n,
                                                           int phase, float amp, float* __restrict__ stats) {
  __shared__ double sh[STAT_THREADS / 32];
  double s = 0.0;
  for (int k = threadIdx.x; k < nb; k += STAT_THREADS) s += part[k];
  const double t = block_sum(s, sh);
  if (threadIdx.x != 0) return;
  const double np = static_cast<double>(n > 0 ? n : 1);
  if (phase == 0) {
    stats[0] = static_cast<float>(t / np);
  } else {
    const float sd = fmaxf(static_cast<float>(sqrt(t / np)), 0.035f);
    stats[1] = sd;
    stats[2] = fminf(__fdiv_rn(amp, sd), 2.2f);
  }
}

// Sensitometric composite (image_pipeline.rs:725-808): grain and tone per pixel.
__global__ void k_grain(const uint8_t* __restrict__ src, const float* __restrict__ heff, const float* __restrict__ dn,
                        const float* __restrict__ dl, const float* __restrict__ gs, const float* __restrict__ stats,
                        size_t n, int pushed, float gamma, float* __restrict__ grain, float* __restrict__ tone) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float pi = 3.14159265358979323846f;
  const float mean = stats[0], norm = stats[2];
  const float raw = __fdiv_rn(static_cast<float>(src[i]), 255.0f);
  const float base = raw <= 0.005f ? 0.0f : __fadd_rn(__fmul_rn(0.35f, raw), __fmul_rn(0.65f, heff[i]));
  const float mid =
      fmaxf(sinf(__fmul_rn(pi, powf(fminf(fmaxf(base, 0.0f), 1.0f), 0.72f))), 0.0f);
  const float vis = __fmul_rn(__fmul_rn(gate_shadow(base), gate_highlight(base)), mid);
  float tv = base;
  if (pushed) {
    tv = base <= 0.5f ? __fmul_rn(0.5f, powf(__fmul_rn(2.0f, base), gamma))
                      : __fsub_rn(1.0f, __fmul_rn(0.5f, powf(__fmul_rn(2.0f, __fsub_rn(1.0f, base)), gamma)));
  }
  const float dd = __fsub_rn(__fsub_rn(dn[i], dl[i]), mean);
  const float sharp = fabsf(dd) > 1e-6f ? copysignf(powf(fabsf(dd), 0.85f), dd) : 0.0f;
  grain[i] = __fmul_rn(__fmul_rn(__fmul_rn(sharp, norm), gs[i]), vis);
  tone[i] = tv;
}

// Vertical OTF pass (when otf is set; else the grain itself), the output gates on the raw pixel
// and the u8 quantisation (image_pipeline.rs:845-891).
__global__ void k_film_out(const float* __restrict__ g, int otf, const uint8_t* __restrict__ src,
                           const float* __restrict__ tone, uint32_t w, uint32_t h, uint8_t* __restrict__ out) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(w) * h) return;
  float sc = g[i];
  if (otf) {
    const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>(i / w);
    const uint32_t ym = y > 0 ? y - 1 : 0, yp = y + 1 < h ? y + 1 : h - 1;
    sc = __fadd_rn(__fadd_rn(__fmul_rn(g[static_cast<size_t>(ym) * w + x], 0.035f), __fmul_rn(g[i], 0.93f)),
                   __fmul_rn(g[static_cast<size_t>(yp) * w + x], 0.035f));
  }
  const float raw = __fdiv_rn(static_cast<float>(src[i]), 255.0f);
  const float gated = __fmul_rn(__fmul_rn(sc, gate_shadow(raw)), gate_highlight(raw));
  float v = __fadd_rn(__fadd_rn(tone[i], 0.0f), gated);
  v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
  out[i] = static_cast<uint8_t>(roundf(__fmul_rn(v, 255.0f)));
}

std::string lower(const char* s) {
  std::string r(s ? s : "");
  for (auto& ch : r) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  return r;
}

// Panchromatic weights (image_pipeline.rs:265-284).
void luma_weights(const char* preset, float w[3]) {
  const std::string s = lower(preset);
  if (s == "tri-x" || s == "trix" || s == "tri-x-400" || s == "tri-x-1600" || s == "trix-1600" || s == "caffenol") {
    w[0] = 0.42f; w[1] = 0.46f; w[2] = 0.12f;
  } else if (s == "hp5" || s == "hp5-plus") {
    w[0] = 0.36f; w[1] = 0.48f; w[2] = 0.16f;
  } else if (s == "t-max" || s == "tmax") {
    w[0] = 0.33f; w[1] = 0.52f; w[2] = 0.15f;
  } else {
    w[0] = 0.38f; w[1] = 0.48f; w[2] = 0.14f;
  }
}

// Grain amplitude of a stock (image_pipeline.rs:718-723).
float base_nominal(const char* preset) {
  const std::string s = lower(preset);
  if (s == "t-max" || s == "tmax") return 0.024f;
  if (s == "hp5" || s == "hp5-plus") return 0.032f;
  if (s == "tri-x-1600" || s == "trix-1600" || s == "caffenol") return 0.042f;
  return 0.038f;
}

void launch_resize_u8(const uint8_t* in, uint32_t w, uint32_t h, uint32_t ow, uint32_t oh, int filter, uint8_t* out,
                      cudaStream_t st) {
  if (ow == w && oh == h) {
    FG_CUDA(cudaMemcpyAsync(out, in, static_cast<size_t>(w) * h, cudaMemcpyDeviceToDevice, st));
    return;
  }
  std::vector<uint32_t> ly, cy, lx, cx;
  std::vector<float> wy, wx;
  uint32_t sy = 0, sx = 0;
  resample_weights(h, oh, filter, ly, cy, wy, sy);
  resample_weights(w, ow, filter, lx, cx, wx, sx);
  DBuf<uint32_t> dl(static_cast<size_t>(oh) * 2 + static_cast<size_t>(ow) * 2, st);
  DBuf<float> dw(wy.size() + wx.size(), st), tmp(static_cast<size_t>(w) * oh, st);
  std::vector<uint32_t> idx;
  idx.insert(idx.end(), ly.begin(), ly.end());
  idx.insert(idx.end(), cy.begin(), cy.end());
  idx.insert(idx.end(), lx.begin(), lx.end());
  idx.insert(idx.end(), cx.begin(), cx.end());
  std::vector<float> wall(wy);
  wall.insert(wall.end(), wx.begin(), wx.end());
  FG_CUDA(cudaMemcpyAsync(dl.p, idx.data(), idx.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  FG_CUDA(cudaMemcpyAsync(dw.p, wall.data(), wall.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  k_resample_v_u8<<<grid_for(tmp.n, 256), 256, 0, st>>>(in, w, dl.p, dl.p + oh, dw.p, sy, oh, tmp.p);
  k_resample_h_u8<<<grid_for(static_cast<size_t>(ow) * oh, 256), 256, 0, st>>>(
      tmp.p, w, dl.p + 2 * oh, dl.p + 2 * oh + ow, dw.p + wy.size(), sx, ow, oh, out);
  FG_CUDA(cudaGetLastError());
}

void launch_psf(const uint8_t* src, uint32_t w, uint32_t h, float* heff, FilmGate* gate_out, cudaStream_t st) {
  const size_t n = static_cast<size_t>(w) * h;
  DBuf<uint32_t> flags(static_cast<size_t>(w) + h, st);
  DBuf<FilmGate> gate(1, st);
  DBuf<float> tn(n, st), tw(n, st);
  FG_CUDA(cudaMemsetAsync(flags.p, 0, flags.n * sizeof(uint32_t), st));
  k_gate_flags<<<grid_for(n, 256), 256, 0, st>>>(src, w, h, flags.p, flags.p + h);
  k_gate_bounds<<<1, 1024, 0, st>>>(flags.p, flags.p + h, w, h, gate.p);
  k_psf_h<<<grid_for(n, 256), 256, 0, st>>>(src, w, h, gate.p, tn.p, tw.p);
  k_psf_v<<<grid_for(n, 256), 256, 0, st>>>(tn.p, tw.p, w, h, gate.p, heff);
  FG_CUDA(cudaGetLastError());
  if (gate_out) FG_CUDA(cudaMemcpyAsync(gate_out, gate.p, sizeof(FilmGate), cudaMemcpyDeviceToHost, st));
}

// Tile grid of an image (image_pipeline.rs:377-424).
struct Grid {
  uint32_t step, pad, ntx, nty;
  std::vector<uint32_t> desc;  // ntiles x (tx, ty, xs, ys, tw, th)
};

Grid make_grid(uint32_t out_w, uint32_t out_h, double grain_px, uint32_t tile_size) {
  Grid g;
  const uint32_t s = static_cast<uint32_t>(std::llround(384.0 * grain_px));
  g.step = std::max(std::min(s, tile_size), 48u);
  g.pad = std::min(std::max(g.step / 10, 12u), 48u);
  g.ntx = (out_w + g.step - 1) / g.step;
  g.nty = (out_h + g.step - 1) / g.step;
  for (uint32_t ty = 0; ty < g.nty; ++ty)
    for (uint32_t tx = 0; tx < g.ntx; ++tx) {
      const uint32_t x0 = tx * g.step, y0 = ty * g.step;
      const uint32_t xs = x0 > g.pad ? x0 - g.pad : 0, ys = y0 > g.pad ? y0 - g.pad : 0;
      const uint32_t xe = std::min(x0 + g.step + g.pad, out_w), ye = std::min(y0 + g.step + g.pad, out_h);
      const uint32_t q[6] = {tx, ty, xs, ys, xe - xs, ye - ys};
      g.desc.insert(g.desc.end(), q, q + 6);
    }
  return g;
}

struct FinishArgs {
  const char* preset;
  double grain_px, strength, push;
  int otf;
};

// Everything after the tiles, on device tile densities: to a u8 image.  fields (device, may be
// null) receives d_norm, d_low, grain, tone, scanned planes; stats (device, 4 floats) the grain
// statistics.
void launch_finish(const FinishArgs& a, uint32_t out_w, uint32_t out_h, const Grid& g,
                   const std::vector<const float*>& tiles, const uint8_t* src, const float* heff, uint8_t* out,
                   float* fields, float* stats, cudaStream_t st) {
  const size_t n = static_cast<size_t>(out_w) * out_h;
  const uint32_t ntiles = static_cast<uint32_t>(tiles.size());
  std::vector<FilmTile> ft(ntiles);
  for (uint32_t t = 0; t < ntiles; ++t) {
    const uint32_t* q = g.desc.data() + 6 * t;
    ft[t] = FilmTile{tiles[t], q[0], q[1], q[2], q[3], q[4], q[5]};
  }
  // Low-pass kernel on the host (image_pipeline.rs:661-671).
  const float sigma = std::fmax(static_cast<float>(a.grain_px) * 1.5f, 1.5f);
  const int krad = static_cast<int>(std::fmin(std::fmax(std::ceil(2.5f * sigma), 2.0f), 48.0f));
  std::vector<float> kern;
  float ksum = 0.0f;
  for (int i = -krad; i <= krad; ++i) {
    const float q = static_cast<float>(i) / sigma;
    const float v = std::exp(-0.5f * (q * q));
    kern.push_back(v);
    ksum += v;
  }
  for (float& v : kern) v /= std::fmax(ksum, 1e-6f);
  const float amp = (base_nominal(a.preset) * (1.0f + 0.15f * static_cast<float>(a.push))) * static_cast<float>(a.strength);
  const float gamma = 1.0f + 0.06f * static_cast<float>(a.push);
  DBuf<FilmTile> dft(ntiles, st);
  DBuf<float> dk(kern.size(), st);
  DBuf<float> planes(fields ? 0 : 5 * n, st), gsc(n, st), tmp(n, st);
  DBuf<float> dstat(stats ? 0 : 4, st);
  DBuf<double> part(STAT_BLOCKS, st);
  float* P = fields ? fields : planes.p;
  float* S = stats ? stats : dstat.p;
  float *dn = P, *dl = P + n, *gr = P + 2 * n, *tn = P + 3 * n, *sc = P + 4 * n;
  // Pageable host sources: each copy has taken its data when it returns.
  FG_CUDA(cudaMemcpyAsync(dft.p, ft.data(), ntiles * sizeof(FilmTile), cudaMemcpyHostToDevice, st));
  FG_CUDA(cudaMemsetAsync(S, 0, 4 * sizeof(float), st));
  FG_CUDA(cudaMemcpyAsync(dk.p, kern.data(), kern.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  const unsigned G = grid_for(n, 256);
  DBuf<float> hx(3 * static_cast<size_t>(out_w), st), hy(3 * static_cast<size_t>(out_h), st);
  k_hann_table<<<grid_for(out_w, 256), 256, 0, st>>>(out_w, g.ntx, g.step, g.pad, hx.p);
  k_hann_table<<<grid_for(out_h, 256), 256, 0, st>>>(out_h, g.nty, g.step, g.pad, hy.p);
  k_blend_film<<<G, 256, 0, st>>>(dft.p, ntiles, g.ntx, g.nty, g.step, hx.p, hy.p, out_w, out_h, dn, gsc.p);
  k_gauss_pass<<<G, 256, 0, st>>>(dn, out_w, out_h, dk.p, krad, 0, tmp.p);
  k_gauss_pass<<<G, 256, 0, st>>>(tmp.p, out_w, out_h, dk.p, krad, 1, dl);
  const int nb = static_cast<int>(std::min<size_t>(STAT_BLOCKS, std::max<size_t>(grid_for(n, STAT_THREADS), 1)));
  k_high_sum<<<nb, STAT_THREADS, 0, st>>>(dn, dl, n, S, 0, part.p);
  k_high_fin<<<1, STAT_THREADS, 0, st>>>(part.p, nb, n, 0, amp, S);
  k_high_sum<<<nb, STAT_THREADS, 0, st>>>(dn, dl, n, S, 1, part.p);
  k_high_fin<<<1, STAT_THREADS, 0, st>>>(part.p, nb, n, 1, amp, S);
  k_grain<<<G, 256, 0, st>>>(src, heff, dn, dl, gsc.p, S, n, a.push > 0.0 ? 1 : 0, gamma, gr, tn);
  if (a.otf) {
    k_otf_pass<<<G, 256, 0, st>>>(gr, tmp.p, out_w, out_h, 0.035f, 0.93f, 0.035f, 0, 1.0f);
    if (fields) k_otf_pass<<<G, 256, 0, st>>>(tmp.p, sc, out_w, out_h, 0.035f, 0.93f, 0.035f, 1, 1.0f);
    k_film_out<<<G, 256, 0, st>>>(tmp.p, 1, src, tn, out_w, out_h, out);  // vertical pass fused
  } else {
    if (fields) FG_CUDA(cudaMemcpyAsync(sc, gr, n * sizeof(float), cudaMemcpyDeviceToDevice, st));
    k_film_out<<<G, 256, 0, st>>>(gr, 0, src, tn, out_w, out_h, out);
  }
  FG_CUDA(cudaGetLastError());
}

void ok(fg_engine* e, fg_status s) {
  if (s != FG_OK) throw Error{s, e->err};
}

// Output size of a render (image_pipeline.rs:306-313).
void output_size(const fg_film_options& o, uint32_t in_w, uint32_t in_h, uint32_t& ow, uint32_t& oh) {
  const double aspect = static_cast<double>(in_w) / static_cast<double>(in_h);
  if (o.out_w == 0 && o.out_h == 0) {
    ow = in_w;
    oh = in_h;
  } else if (o.out_h == 0) {
    ow = o.out_w;
    oh = static_cast<uint32_t>(std::max(std::round(static_cast<double>(o.out_w) / aspect), 1.0));
  } else if (o.out_w == 0) {
    ow = static_cast<uint32_t>(std::max(std::round(static_cast<double>(o.out_h) * aspect), 1.0));
    oh = o.out_h;
  } else {
    ow = o.out_w;
    oh = o.out_h;
  }
}

// One black-and-white layer being rendered: its source, h_effective, grid and scaling.
struct Layer {
  uint64_t seed = 0;
  uint32_t rw = 0, rh = 0;  // render size (the supersampled size when ss > 1)
  uint32_t ow = 0, oh = 0;  // output size
  double grain = 0, strength = 0, push = 0;
  DBuf<uint8_t> src;
  DBuf<float> heff;
  Grid grid;
  uint32_t first_tile = 0;
};

// image_pipeline.rs:299-375 for one layer: resize the gray input to the render size, PSF, scaling
// and tile grid.
void prepare_layer(Layer& L, const uint8_t* gray, uint32_t in_w, uint32_t in_h, const fg_film_options& o,
                   cudaStream_t st) {
  output_size(o, in_w, in_h, L.ow, L.oh);
  const uint32_t ss = std::min(std::max(o.supersample, 1u), 4u);
  L.rw = L.ow * ss;
  L.rh = L.oh * ss;
  const size_t n = static_cast<size_t>(L.rw) * L.rh;
  L.src.alloc(n, st);
  L.heff.alloc(n, st);
  launch_resize_u8(gray, in_w, in_h, L.rw, L.rh, RESAMPLE_LANCZOS3, L.src.p, st);
  launch_psf(L.src.p, L.rw, L.rh, L.heff.p, nullptr, st);
  const double user = o.scale > 0.0 ? o.scale : 1.0;
  double res = 1.0, selwyn = 1.0;
  if (o.auto_scale) {
    const double ref = std::max(static_cast<double>(o.reference_res), 512.0);
    const double edge = std::max(static_cast<double>(std::max(L.rw, L.rh)), 1.0);
    res = std::min(std::max(edge / ref, 0.05), 5.0);
    selwyn = std::sqrt(res);
  }
  L.grain = std::min(std::max(o.grain_size_px * user * res, 0.05), 15.0);
  L.strength = std::max(o.grain_strength * std::sqrt(user) * selwyn, 0.0);
  const std::string p = lower(o.preset);
  L.push = (p.find("1600") != std::string::npos || p == "caffenol") ? std::max(o.push, 2.0) : std::max(o.push, 0.0);
  L.grid = make_grid(L.rw, L.rh, L.grain, o.tile_size);
}

// Renders gray layers (device u8 images of in_w x in_h) into device u8 outputs.  The tiles of all
// layers run as consecutive batches in tile order, each within the byte budget (one batch when
// everything fits); their densities are gathered into one device array before the finish.
// Tiles are independent, so the result does not depend on how they are grouped.
void render_layers(fg_engine* e, std::vector<Layer>& layers, const std::vector<const uint8_t*>& gray, uint32_t in_w,
                   uint32_t in_h, const fg_film_options& o, const std::vector<uint8_t*>& out, fg_film_report* rep) {
  cudaStream_t st = e->stream;
  struct Ev {
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    Ev() {
      for (auto& x : ev) FG_CUDA(cudaEventCreate(&x));
    }
    ~Ev() {
      for (auto& x : ev)
        if (x) cudaEventDestroy(x);
    }
  } ev;
  FG_CUDA(cudaEventRecord(ev.ev[0], st));
  std::vector<fg_tile_params> params;
  std::vector<GatherTile> src;  // where each tile's exposure comes from (dst filled per batch)
  for (size_t l = 0; l < layers.size(); ++l) {
    Layer& L = layers[l];
    prepare_layer(L, gray[l], in_w, in_h, o, st);
    L.first_tile = static_cast<uint32_t>(params.size());
    const size_t nt = L.grid.desc.size() / 6;
    for (size_t t = 0; t < nt; ++t) {
      const uint32_t* q = L.grid.desc.data() + 6 * t;
      const uint64_t seed = L.seed + static_cast<uint64_t>(t) * 73856093ull + static_cast<uint64_t>(q[0]) * 19349663ull +
                            static_cast<uint64_t>(q[1]) * 83492791ull;  // image_pipeline.rs:430-434
      fg_tile_params tp;
      ok(e, fg_tile_params_preset(o.preset, 1.0 / L.grain, q[4], q[5], o.exposure, o.push, seed, &tp));
      params.push_back(tp);
      src.push_back(GatherTile{L.heff.p, nullptr, L.rw, q[2], q[3], q[4], q[5]});
    }
  }
  FG_CUDA(cudaEventRecord(ev.ev[1], st));
  const size_t ntot = params.size();
  std::vector<unsigned long long> doff(ntot);
  unsigned long long dtot = 0;
  for (size_t i = 0; i < ntot; ++i) {
    doff[i] = dtot;
    dtot += static_cast<unsigned long long>(params[i].width_px) * params[i].height_px;
  }
  DBuf<float> dens(std::max<unsigned long long>(dtot, 1), st);
  size_t freeb = 0, totalb = 0;
  FG_CUDA(cudaMemGetInfo(&freeb, &totalb));
  const unsigned long long budget =
      o.batch_bytes ? o.batch_bytes : static_cast<unsigned long long>(0.7 * static_cast<double>(freeb));
  fg_batch_options bo{};
  bo.use_graph = 0;
  bo.autotune = 0;
  for (size_t first = 0; first < ntot;) {
    size_t last = first;
    unsigned long long bytes = 0, slots = 0;
    while (last < ntot) {
      unsigned long long s = 0;
      const unsigned long long b = tile_footprint(params[last], &s);
      if (last > first && (bytes + b > budget || slots + s >= 0x7fffffffull)) break;
      bytes += b;
      slots += s;
      ++last;
    }
    const uint32_t nb = static_cast<uint32_t>(last - first);
    FG_REQUIRE(nb <= 65535, "too many tiles in one batch");
    fg_batch* b = nullptr;
    ok(e, fg_batch_create(e, params.data() + first, nb, &bo, &b));
    struct BatchGuard {
      fg_batch* b;
      ~BatchGuard() { fg_batch_destroy(b); }
    } guard_b{b};
    std::vector<GatherTile> gt(nb);
    std::vector<CopyTile> ct(nb);
    for (uint32_t t = 0; t < nb; ++t) {
      gt[t] = src[first + t];
      ok(e, fg_batch_exposure_device(b, t, &gt[t].dst));
      const float* d = nullptr;
      ok(e, fg_batch_density_device(b, t, &d));
      ct[t] = CopyTile{d, dens.p + doff[first + t],
                       static_cast<unsigned long long>(params[first + t].width_px) * params[first + t].height_px};
    }
    DBuf<GatherTile> dgt(nb, st);
    DBuf<CopyTile> dct(nb, st);
    FG_CUDA(cudaMemcpyAsync(dgt.p, gt.data(), nb * sizeof(GatherTile), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(dct.p, ct.data(), nb * sizeof(CopyTile), cudaMemcpyHostToDevice, st));
    k_gather_tiles<<<dim3(64, nb), 256, 0, st>>>(dgt.p);
    FG_CUDA(cudaGetLastError());
    ok(e, fg_batch_run(b));
    k_copy_tiles<<<dim3(64, nb), 256, 0, st>>>(dct.p);
    FG_CUDA(cudaGetLastError());
    fg_batch_stats bs{};
    ok(e, fg_batch_wait(b, &bs));
    if (rep) {
      rep->total_crystals += bs.crystals;
      rep->developed_crystals += bs.developed;
      rep->total_clumps += bs.clumps;
      rep->photons += bs.photons;
    }
    first = last;
  }
  FG_CUDA(cudaEventRecord(ev.ev[2], st));
  for (size_t l = 0; l < layers.size(); ++l) {
    Layer& L = layers[l];
    const uint32_t nt = static_cast<uint32_t>(L.grid.desc.size() / 6);
    std::vector<const float*> dp(nt);
    for (uint32_t t = 0; t < nt; ++t) dp[t] = dens.p + doff[L.first_tile + t];
    const FinishArgs fa{o.preset, L.grain, L.strength, L.push, o.scanner_otf};
    if (L.rw == L.ow && L.rh == L.oh) {
      launch_finish(fa, L.rw, L.rh, L.grid, dp, L.src.p, L.heff.p, out[l], nullptr, nullptr, st);
    } else {
      DBuf<uint8_t> big(static_cast<size_t>(L.rw) * L.rh, st);
      launch_finish(fa, L.rw, L.rh, L.grid, dp, L.src.p, L.heff.p, big.p, nullptr, nullptr, st);
      launch_resize_u8(big.p, L.rw, L.rh, L.ow, L.oh, RESAMPLE_TRIANGLE, out[l], st);
    }
  }
  FG_CUDA(cudaEventRecord(ev.ev[3], st));
  FG_CUDA(cudaEventSynchronize(ev.ev[3]));
  if (rep) {
    rep->total_tiles += ntot;
    float a = 0, b = 0, c = 0;
    FG_CUDA(cudaEventElapsedTime(&a, ev.ev[0], ev.ev[1]));
    FG_CUDA(cudaEventElapsedTime(&b, ev.ev[1], ev.ev[2]));
    FG_CUDA(cudaEventElapsedTime(&c, ev.ev[2], ev.ev[3]));
    rep->prep_ms += a;
    rep->tiles_ms += b;
    rep->finish_ms += c;
  }
}

}  // namespace

}  // namespace fg

using namespace fg;

extern "C" {

void fg_film_options_default(fg_film_options* o) {
  if (!o) return;
  *o = fg_film_options{};
  o->preset = "tri-x";  // image_pipeline.rs:82-101
  o->grain_size_px = 2.2;
  o->grain_strength = 1.0;
  o->exposure = 1.0;
  o->tile_size = 320;
  o->seed = 42;
  o->scale = 1.0;
  o->reference_res = 6000;
  o->supersample = 1;
  o->eberhard = 1.0;
  o->scanner_otf = 1;
}

fg_status fg_film_output_size(const fg_film_options* o, uint32_t in_w, uint32_t in_h, uint32_t* out_w,
                              uint32_t* out_h) {
  if (!o || !out_w || !out_h || in_w == 0 || in_h == 0) return FG_ERR_INVALID_ARG;
  output_size(*o, in_w, in_h, *out_w, *out_h);
  return FG_OK;
}

fg_status fg_render_film(fg_engine* e, const uint8_t* pixels, uint32_t w, uint32_t h, uint32_t channels,
                         const fg_film_options* o, uint8_t* out, fg_film_report* rep) {
  return guard(e, [&] {
    FG_REQUIRE(pixels && out && o && o->preset, "null argument");
    FG_REQUIRE(w > 0 && h > 0, "empty image");
    FG_REQUIRE(channels == 1 || channels == 3, "channels must be 1 (gray) or 3 (RGB)");
    const bool color = o->color != 0;
    FG_REQUIRE(!color || channels == 3, "colour rendering needs an RGB image");
    FG_REQUIRE(o->tile_size >= 48, "tile_size below the 48-pixel minimum step");
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = e->stream;
    uint32_t ow = 0, oh = 0;
    output_size(*o, w, h, ow, oh);
    FG_REQUIRE(ow > 0 && oh > 0, "empty output size");
    const size_t n = static_cast<size_t>(w) * h, no = static_cast<size_t>(ow) * oh;
    DBuf<uint8_t> in(n * channels, st);
    FG_CUDA(cudaMemcpyAsync(in.p, pixels, n * channels, cudaMemcpyHostToDevice, st));
    const int nl = color ? 3 : 1;
    std::vector<DBuf<uint8_t>> gray(nl), res(nl);
    std::vector<const uint8_t*> gp(nl);
    std::vector<uint8_t*> rp(nl);
    for (int l = 0; l < nl; ++l) {
      res[l].alloc(no, st);
      rp[l] = res[l].p;
    }
    if (color) {
      for (int c = 0; c < 3; ++c) {
        gray[c].alloc(n, st);
        k_channel<<<grid_for(n, 256), 256, 0, st>>>(in.p, n, c, gray[c].p);
        gp[c] = gray[c].p;
      }
    } else if (channels == 3) {
      float wl[3];
      luma_weights(o->preset, wl);
      gray[0].alloc(n, st);
      k_luma<<<grid_for(n, 256), 256, 0, st>>>(in.p, n, wl[0], wl[1], wl[2], gray[0].p);
      gp[0] = gray[0].p;
    } else {
      gp[0] = in.p;
    }
    FG_CUDA(cudaGetLastError());
    std::vector<Layer> layers(nl);
    const uint64_t offs[3] = {0, 10007, 20011};  // image_pipeline.rs:1048-1061
    for (int l = 0; l < nl; ++l) layers[l].seed = o->seed + offs[l];
    fg_film_report r{};
    render_layers(e, layers, gp, w, h, *o, rp, &r);
    if (color) {
      DBuf<uint8_t> rgb(3 * no, st);
      k_interleave<<<grid_for(no, 256), 256, 0, st>>>(rp[0], rp[1], rp[2], no, rgb.p);
      FG_CUDA(cudaGetLastError());
      FG_CUDA(cudaMemcpyAsync(out, rgb.p, 3 * no, cudaMemcpyDeviceToHost, st));
    } else {
      FG_CUDA(cudaMemcpyAsync(out, rp[0], no, cudaMemcpyDeviceToHost, st));
    }
    FG_CUDA(cudaStreamSynchronize(st));
    if (rep) {
      r.in_w = w;
      r.in_h = h;
      r.out_w = ow;
      r.out_h = oh;
      r.elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      *rep = r;
    }
  });
}

fg_status fg_panchromatic_luma(fg_engine* e, const uint8_t* rgb, uint32_t w, uint32_t h, const char* preset,
                               uint8_t* out) {
  return guard(e, [&] {
    FG_REQUIRE(rgb && out && preset && w > 0 && h > 0, "null argument or empty image");
    cudaStream_t st = e->stream;
    const size_t n = static_cast<size_t>(w) * h;
    DBuf<uint8_t> a(3 * n, st), b(n, st);
    float wl[3];
    luma_weights(preset, wl);
    FG_CUDA(cudaMemcpyAsync(a.p, rgb, 3 * n, cudaMemcpyHostToDevice, st));
    k_luma<<<grid_for(n, 256), 256, 0, st>>>(a.p, n, wl[0], wl[1], wl[2], b.p);
    FG_CUDA(cudaGetLastError());
    FG_CUDA(cudaMemcpyAsync(out, b.p, n, cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
  });
}

fg_status fg_resize_u8(fg_engine* e, const uint8_t* in, uint32_t w, uint32_t h, uint32_t ow, uint32_t oh,
                       int32_t filter, uint8_t* out) {
  return guard(e, [&] {
    FG_REQUIRE(in && out && w > 0 && h > 0 && ow > 0 && oh > 0, "null argument or empty image");
    FG_REQUIRE(filter == FG_FILTER_TRIANGLE || filter == FG_FILTER_LANCZOS3, "unknown filter");
    cudaStream_t st = e->stream;
    DBuf<uint8_t> a(static_cast<size_t>(w) * h, st), b(static_cast<size_t>(ow) * oh, st);
    FG_CUDA(cudaMemcpyAsync(a.p, in, a.n, cudaMemcpyHostToDevice, st));
    launch_resize_u8(a.p, w, h, ow, oh, filter == FG_FILTER_TRIANGLE ? RESAMPLE_TRIANGLE : RESAMPLE_LANCZOS3, b.p, st);
    FG_CUDA(cudaMemcpyAsync(out, b.p, b.n, cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
  });
}

fg_status fg_gelatin_psf(fg_engine* e, const uint8_t* src, uint32_t w, uint32_t h, float* h_eff, uint32_t* gate) {
  return guard(e, [&] {
    FG_REQUIRE(src && h_eff && w > 0 && h > 0, "null argument or empty image");
    cudaStream_t st = e->stream;
    const size_t n = static_cast<size_t>(w) * h;
    DBuf<uint8_t> a(n, st);
    DBuf<float> b(n, st);
    FilmGate g{};
    FG_CUDA(cudaMemcpyAsync(a.p, src, n, cudaMemcpyHostToDevice, st));
    launch_psf(a.p, w, h, b.p, &g, st);
    FG_CUDA(cudaMemcpyAsync(h_eff, b.p, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (gate) {
      gate[0] = g.top;
      gate[1] = g.bottom;
      gate[2] = g.left;
      gate[3] = g.right;
    }
  });
}

fg_status fg_film_finish(fg_engine* e, const fg_finish_cfg* cfg, uint32_t out_w, uint32_t out_h, uint32_t tile_step,
                         uint32_t pad, uint32_t ntiles, const uint32_t* desc, const float* const* tiles,
                         const uint8_t* src, const float* h_eff, uint8_t* out, float* fields, float* stats) {
  return guard(e, [&] {
    FG_REQUIRE(cfg && cfg->preset && desc && tiles && src && h_eff && out, "null argument");
    FG_REQUIRE(out_w > 0 && out_h > 0 && tile_step > 0 && ntiles > 0, "empty image or tile list");
    cudaStream_t st = e->stream;
    Grid g;
    g.step = tile_step;
    g.pad = pad;
    g.ntx = (out_w + tile_step - 1) / tile_step;
    g.nty = (out_h + tile_step - 1) / tile_step;
    FG_REQUIRE(ntiles == g.ntx * g.nty, "tile list does not match the grid (one tile per grid cell, index ty * ntx + tx)");
    g.desc.assign(desc, desc + 6 * static_cast<size_t>(ntiles));
    size_t tot = 0;
    for (uint32_t t = 0; t < ntiles; ++t) {
      const uint32_t* q = desc + 6 * t;
      FG_REQUIRE(q[1] * g.ntx + q[0] == t, "tiles must be listed in grid order (index ty * ntx + tx)");
      FG_REQUIRE(q[2] + q[4] <= out_w && q[3] + q[5] <= out_h, "tile outside the image");
      tot += static_cast<size_t>(q[4]) * q[5];
    }
    const size_t n = static_cast<size_t>(out_w) * out_h;
    DBuf<float> d(std::max<size_t>(tot, 1), st), he(n, st), fl(fields ? 5 * n : 0, st), sd(4, st);
    DBuf<uint8_t> s8(n, st), o8(n, st);
    std::vector<const float*> dp(ntiles);
    size_t off = 0;
    for (uint32_t t = 0; t < ntiles; ++t) {
      const size_t k = static_cast<size_t>(desc[6 * t + 4]) * desc[6 * t + 5];
      if (k) FG_CUDA(cudaMemcpyAsync(d.p + off, tiles[t], k * sizeof(float), cudaMemcpyHostToDevice, st));
      dp[t] = d.p + off;
      off += k;
    }
    FG_CUDA(cudaMemcpyAsync(s8.p, src, n, cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(he.p, h_eff, n * sizeof(float), cudaMemcpyHostToDevice, st));
    const FinishArgs fa{cfg->preset, cfg->grain_size_px, cfg->grain_strength, cfg->push, cfg->scanner_otf};
    launch_finish(fa, out_w, out_h, g, dp, s8.p, he.p, o8.p, fields ? fl.p : nullptr, sd.p, st);
    FG_CUDA(cudaMemcpyAsync(out, o8.p, n, cudaMemcpyDeviceToHost, st));
    if (fields) FG_CUDA(cudaMemcpyAsync(fields, fl.p, 5 * n * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (stats) FG_CUDA(cudaMemcpyAsync(stats, sd.p, 4 * sizeof(float), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
  });
}

}  // extern "C"
