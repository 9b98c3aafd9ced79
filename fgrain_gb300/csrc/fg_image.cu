// Image-level stages around the tile path: the Hann overlap blend of tile densities
// (image_pipeline.rs:593-649), the scanner OTF (image_pipeline.rs:825-855) and the Triangle-filter
// downsample of supersampled renders (image_pipeline.rs:315-330, the image crate's separable tent
// filter).  All three are memory-bound stencils in FP32 that repeat the reference's operation
// order exactly (no fused multiply-add), so the device reproduces the CPU bit for bit apart from
// the Hann cosine (correctly rounded here; the reference calls the C library's cosf).
#include <algorithm>
#include <cmath>
#include <vector>

#include "fg_image.cuh"

namespace fg {

namespace {

__device__ __forceinline__ uint32_t clamp_lo(uint32_t v) { return v > 0 ? v - 1 : 0; }
__device__ __forceinline__ uint32_t clamp_hi(uint32_t v, uint32_t n) { return v + 1 < n ? v + 1 : n - 1; }

struct BlendTile {
  uint32_t tx, ty, xs, ys, tw, th;
  unsigned long long off;  // first density value of the tile in the packed buffer
};

// d_norm = sum_t d_t w_t / max(sum_t w_t, 1e-5) per pixel, the tiles accumulated in tile order as
// the reference does.  Tile (tx, ty) has index ty * ntx + tx; a pixel lies in at most 3 x 3 tiles.
__global__ void k_blend(const BlendTile* __restrict__ tiles, uint32_t ntiles, uint32_t ntx, uint32_t nty,
                        uint32_t step, uint32_t pad, uint32_t out_w, uint32_t out_h, const float* __restrict__ d,
                        float* __restrict__ out) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(out_w) * out_h) return;
  const uint32_t gx = static_cast<uint32_t>(i % out_w), gy = static_cast<uint32_t>(i / out_w);
  const uint32_t cx = gx / step, cy = gy / step;
  float acc = 0.0f, wacc = 0.0f;
  for (int dy = -1; dy <= 1; ++dy) {
    const int ty = static_cast<int>(cy) + dy;
    if (ty < 0 || ty >= static_cast<int>(nty)) continue;
    for (int dx = -1; dx <= 1; ++dx) {
      const int tx = static_cast<int>(cx) + dx;
      if (tx < 0 || tx >= static_cast<int>(ntx)) continue;
      const uint32_t k = static_cast<uint32_t>(ty) * ntx + static_cast<uint32_t>(tx);
      if (k >= ntiles) continue;
      const BlendTile T = tiles[k];
      if (gx < T.xs || gx >= T.xs + T.tw || gy < T.ys || gy >= T.ys + T.th) continue;
      const float wy = hann_weight(T.ty, gy, nty, T.ty * step, step, pad);
      const float wx = hann_weight(T.tx, gx, ntx, T.tx * step, step, pad);
      const float wv = __fmul_rn(wx, wy);
      const float v = d[T.off + static_cast<size_t>(gy - T.ys) * T.tw + (gx - T.xs)];
      acc = __fadd_rn(acc, __fmul_rn(v, wv));
      wacc = __fadd_rn(wacc, wv);
    }
  }
  out[i] = __fdiv_rn(acc, fmaxf(wacc, 1e-5f));
}

// One pass of the separable tent filter: out(o) = sum_i w[o][i] in(left[o] + i) along x (axis 0)
// or y, summed in i order.
__global__ void k_tent_pass(const float* __restrict__ in, uint32_t w, uint32_t h, const uint32_t* __restrict__ left,
                            const uint32_t* __restrict__ cnt, const float* __restrict__ wts, uint32_t stride, int axis,
                            uint32_t ow, uint32_t oh, float* __restrict__ out) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(ow) * oh) return;
  const uint32_t x = static_cast<uint32_t>(i % ow), y = static_cast<uint32_t>(i / ow);
  const uint32_t o = axis == 0 ? x : y;
  const float* wo = wts + static_cast<size_t>(o) * stride;
  float s = 0.0f;
  for (uint32_t k = 0; k < cnt[o]; ++k) {
    const float v = axis == 0 ? in[static_cast<size_t>(y) * w + left[o] + k] : in[static_cast<size_t>(left[o] + k) * w + x];
    s = __fadd_rn(s, __fmul_rn(wo[k], v));
  }
  (void)h;
  out[i] = s;
}

}  // namespace

void resample_weights(uint32_t n, uint32_t m, int filter, std::vector<uint32_t>& left, std::vector<uint32_t>& cnt,
                      std::vector<float>& wts, uint32_t& stride) {
  const float ratio = static_cast<float>(n) / static_cast<float>(m);
  const float sratio = ratio < 1.0f ? 1.0f : ratio;
  const float support = (filter == RESAMPLE_TRIANGLE ? 1.0f : 3.0f) * sratio;
  stride = static_cast<uint32_t>(std::ceil(support * 2.0f)) + 2;
  left.assign(m, 0);
  cnt.assign(m, 0);
  wts.assign(static_cast<size_t>(m) * stride, 0.0f);
  auto kernel = [filter](float x) {
    if (filter == RESAMPLE_TRIANGLE) {
      const float a = std::fabs(x);
      return a < 1.0f ? 1.0f - a : 0.0f;
    }
    auto sinc = [](float t) {
      const float a = t * 3.14159265358979323846f;
      return t == 0.0f ? 1.0f : std::sin(a) / a;
    };
    return std::fabs(x) < 3.0f ? sinc(x) * sinc(x / 3.0f) : 0.0f;
  };
  for (uint32_t o = 0; o < m; ++o) {
    float c = (static_cast<float>(o) + 0.5f) * ratio;
    const int64_t l = std::clamp<int64_t>(static_cast<int64_t>(std::floor(c - support)), 0, static_cast<int64_t>(n) - 1);
    const int64_t r = std::clamp<int64_t>(static_cast<int64_t>(std::ceil(c + support)), l + 1, static_cast<int64_t>(n));
    c -= 0.5f;
    const uint32_t k = static_cast<uint32_t>(std::min<int64_t>(r - l, stride));
    float sum = 0.0f;
    for (uint32_t q = 0; q < k; ++q) {
      const float wv = kernel((static_cast<float>(l + q) - c) / sratio);
      wts[static_cast<size_t>(o) * stride + q] = wv;
      sum += wv;
    }
    for (uint32_t q = 0; q < k; ++q) wts[static_cast<size_t>(o) * stride + q] /= sum;
    left[o] = static_cast<uint32_t>(l);
    cnt[o] = k;
  }
}

// Separable 3-tap clamp-to-edge pass in the reference's operation order (a k0 + b k1 + c k2),
// optionally scaled: the scanner OTF (two passes) and the differentiable scan's forward.
__global__ void k_otf_pass(const float* __restrict__ in, float* __restrict__ out, uint32_t w, uint32_t h, float k0,
                           float k1, float k2, int axis, float scale) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(w) * h) return;
  const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>(i / w);
  size_t im, ip;
  if (axis == 0) {
    im = static_cast<size_t>(y) * w + clamp_lo(x);
    ip = static_cast<size_t>(y) * w + clamp_hi(x, w);
  } else {
    im = static_cast<size_t>(clamp_lo(y)) * w + x;
    ip = static_cast<size_t>(clamp_hi(y, h)) * w + x;
  }
  const float v = __fadd_rn(__fadd_rn(__fmul_rn(in[im], k0), __fmul_rn(in[i], k1)), __fmul_rn(in[ip], k2));
  out[i] = scale == 1.0f ? v : __fmul_rn(v, scale);
}

void launch_otf(const float* in, float* tmp, float* out, uint32_t w, uint32_t h, const float k[3], float scale,
                cudaStream_t st) {
  const size_t np = static_cast<size_t>(w) * h;
  if (!np) return;
  k_otf_pass<<<grid_for(np, 256), 256, 0, st>>>(in, tmp, w, h, k[0], k[1], k[2], 0, 1.0f);
  k_otf_pass<<<grid_for(np, 256), 256, 0, st>>>(tmp, out, w, h, k[0], k[1], k[2], 1, scale);
  FG_CUDA(cudaGetLastError());
}

}  // namespace fg

using namespace fg;

extern "C" {

fg_status fg_scanner_otf(fg_engine* e, const float* in, uint32_t w, uint32_t h, const float* taps, float* out) {
  return guard(e, [&] {
    FG_REQUIRE(in && out && w > 0 && h > 0, "null argument or empty image");
    const float ref[3] = {0.035f, 0.93f, 0.035f};  // image_pipeline.rs:830
    const float* k = taps ? taps : ref;
    cudaStream_t st = e->stream;
    const size_t np = static_cast<size_t>(w) * h;
    DBuf<float> a(np, st), b(np, st), c(np, st);
    FG_CUDA(cudaMemcpyAsync(a.p, in, np * sizeof(float), cudaMemcpyHostToDevice, st));
    launch_otf(a.p, b.p, c.p, w, h, k, 1.0f, st);
    FG_CUDA(cudaMemcpyAsync(out, c.p, np * sizeof(float), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
  });
}

fg_status fg_resize_triangle(fg_engine* e, const float* in, uint32_t w, uint32_t h, uint32_t ow, uint32_t oh,
                             float* out) {
  return guard(e, [&] {
    FG_REQUIRE(in && out && w > 0 && h > 0 && ow > 0 && oh > 0, "null argument or empty image");
    cudaStream_t st = e->stream;
    std::vector<uint32_t> ly, cy, lx, cx;
    std::vector<float> wy, wx;
    uint32_t sy = 0, sx = 0;
    resample_weights(h, oh, RESAMPLE_TRIANGLE, ly, cy, wy, sy);
    resample_weights(w, ow, RESAMPLE_TRIANGLE, lx, cx, wx, sx);
    DBuf<float> a(static_cast<size_t>(w) * h, st), t(static_cast<size_t>(w) * oh, st), o(static_cast<size_t>(ow) * oh, st);
    DBuf<uint32_t> dly(oh, st), dcy(oh, st), dlx(ow, st), dcx(ow, st);
    DBuf<float> dwy(wy.size(), st), dwx(wx.size(), st);
    FG_CUDA(cudaMemcpyAsync(a.p, in, a.n * sizeof(float), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(dly.p, ly.data(), oh * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(dcy.p, cy.data(), oh * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(dlx.p, lx.data(), ow * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(dcx.p, cx.data(), ow * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(dwy.p, wy.data(), wy.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(dwx.p, wx.data(), wx.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    // Vertical pass first, then horizontal (the image crate's order).
    k_tent_pass<<<grid_for(t.n, 256), 256, 0, st>>>(a.p, w, h, dly.p, dcy.p, dwy.p, sy, 1, w, oh, t.p);
    k_tent_pass<<<grid_for(o.n, 256), 256, 0, st>>>(t.p, w, oh, dlx.p, dcx.p, dwx.p, sx, 0, ow, oh, o.p);
    FG_CUDA(cudaGetLastError());
    FG_CUDA(cudaMemcpyAsync(out, o.p, o.n * sizeof(float), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
  });
}

fg_status fg_blend_tiles(fg_engine* e, uint32_t out_w, uint32_t out_h, uint32_t tile_step, uint32_t pad,
                         uint32_t ntiles, const uint32_t* desc, const float* const* tiles, float* d_norm) {
  return guard(e, [&] {
    FG_REQUIRE(desc && tiles && d_norm && out_w > 0 && out_h > 0 && tile_step > 0 && ntiles > 0, "null argument");
    cudaStream_t st = e->stream;
    const uint32_t ntx = (out_w + tile_step - 1) / tile_step, nty = (out_h + tile_step - 1) / tile_step;
    FG_REQUIRE(ntiles == ntx * nty, "tile list does not match the grid (one tile per grid cell, index ty * ntx + tx)");
    std::vector<BlendTile> bt(ntiles);
    unsigned long long off = 0;
    for (uint32_t t = 0; t < ntiles; ++t) {
      const uint32_t* q = desc + 6 * t;
      bt[t] = BlendTile{q[0], q[1], q[2], q[3], q[4], q[5], off};
      FG_REQUIRE(q[1] * ntx + q[0] == t, "tiles must be listed in grid order (index ty * ntx + tx)");
      FG_REQUIRE(q[2] + q[4] <= out_w && q[3] + q[5] <= out_h, "tile outside the image");
      off += static_cast<unsigned long long>(q[4]) * q[5];
    }
    DBuf<BlendTile> dbt(ntiles, st);
    DBuf<float> d(std::max<unsigned long long>(off, 1), st), o(static_cast<size_t>(out_w) * out_h, st);
    FG_CUDA(cudaMemcpyAsync(dbt.p, bt.data(), ntiles * sizeof(BlendTile), cudaMemcpyHostToDevice, st));
    for (uint32_t t = 0; t < ntiles; ++t)
      if (bt[t].tw && bt[t].th)
        FG_CUDA(cudaMemcpyAsync(d.p + bt[t].off, tiles[t], static_cast<size_t>(bt[t].tw) * bt[t].th * sizeof(float),
                                cudaMemcpyHostToDevice, st));
    k_blend<<<grid_for(o.n, 256), 256, 0, st>>>(dbt.p, ntiles, ntx, nty, tile_step, pad, out_w, out_h, d.p, o.p);
    FG_CUDA(cudaGetLastError());
    FG_CUDA(cudaMemcpyAsync(d_norm, o.p, o.n * sizeof(float), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
  });
}

}  // extern "C"
