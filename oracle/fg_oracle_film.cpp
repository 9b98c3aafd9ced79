// CPU oracle, image stages either side of the tile path (TEST INFRASTRUCTURE ONLY: the tests
// use it as the checker of the CUDA library's film renderer; the product never links it).
//
// Restates, in single precision and in the reference's operation order (built with
// -ffp-contract=off, so nothing is fused):
//   image_pipeline.rs:259-296    panchromatic luma                       -> or_luma
//   image_pipeline.rs:315-342    the image crate's separable resampler   -> or_resize_u8
//                                (Triangle for the supersample downsample, Lanczos3 for the
//                                input rescale; image 0.25.10 imageops::sample: vertical pass to
//                                f32, horizontal pass, round-half-away and clamp to u8)
//   image_pipeline.rs:133-252    camera gate and gelatin PSF             -> or_gelatin_psf
//   image_pipeline.rs:593-891    Hann blend with weights, DoG low-pass   -> or_film_finish
//                                split, grain statistics, sensitometric
//                                composite, scanner OTF, output gates
// The grain statistics are sequential f32 sums, as Iterator::sum::<f32> computes them.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fg_oracle.h"

namespace {

float smoothstep_gate_lo(float v) {  // shadow gate (image_pipeline.rs:731-740, 866-872)
  const float toe_min = 0.005f, toe_max = 0.14f;
  if (v <= toe_min) return 0.0f;
  if (v >= toe_max) return 1.0f;
  const float t = (v - toe_min) / (toe_max - toe_min);
  return t * t * (3.0f - 2.0f * t);
}

float smoothstep_gate_hi(float v) {  // highlight gate (image_pipeline.rs:746-753, 875-882)
  if (v <= 0.65f) return 1.0f;
  if (v >= 0.94f) return 0.0f;
  const float u = (v - 0.65f) / (0.94f - 0.65f);
  return 1.0f - u * u * (3.0f - 2.0f * u);
}

// Resampling weights of one axis (image 0.25.10 imageops::sample vertical_sample /
// horizontal_sample): filter 0 Triangle (support 1), 1 Lanczos3 (support 3).
float resample_kernel(int filter, float x) {
  if (filter == 0) {
    const float a = std::fabs(x);
    return a < 1.0f ? 1.0f - a : 0.0f;
  }
  auto sinc = [](float t) {
    const float a = t * 3.14159265358979323846f;
    return t == 0.0f ? 1.0f : std::sin(a) / a;
  };
  return std::fabs(x) < 3.0f ? sinc(x) * sinc(x / 3.0f) : 0.0f;
}

void resample_axis(uint32_t n, uint32_t m, int filter, std::vector<uint32_t>& left,
                   std::vector<std::vector<float>>& w) {
  const float ratio = static_cast<float>(n) / static_cast<float>(m);
  const float sratio = ratio < 1.0f ? 1.0f : ratio;
  const float support = (filter == 0 ? 1.0f : 3.0f) * sratio;
  left.assign(m, 0);
  w.assign(m, {});
  for (uint32_t o = 0; o < m; ++o) {
    float c = (static_cast<float>(o) + 0.5f) * ratio;
    int64_t l = static_cast<int64_t>(std::floor(c - support));
    l = std::clamp<int64_t>(l, 0, static_cast<int64_t>(n) - 1);
    int64_t r = static_cast<int64_t>(std::ceil(c + support));
    r = std::clamp<int64_t>(r, l + 1, static_cast<int64_t>(n));
    c -= 0.5f;
    float sum = 0.0f;
    for (int64_t i = l; i < r; ++i) {
      const float v = resample_kernel(filter, (static_cast<float>(i) - c) / sratio);
      w[o].push_back(v);
      sum += v;
    }
    for (float& v : w[o]) v /= sum;
    left[o] = static_cast<uint32_t>(l);
  }
}

}  // namespace

extern "C" {

int or_luma_weights(const char* preset, float out[3]) {
  if (!preset || !out) return 1;
  std::string s(preset);
  for (auto& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  if (s == "tri-x" || s == "trix" || s == "tri-x-400" || s == "tri-x-1600" || s == "trix-1600" || s == "caffenol") {
    out[0] = 0.42f; out[1] = 0.46f; out[2] = 0.12f;
  } else if (s == "hp5" || s == "hp5-plus") {
    out[0] = 0.36f; out[1] = 0.48f; out[2] = 0.16f;
  } else if (s == "t-max" || s == "tmax") {
    out[0] = 0.33f; out[1] = 0.52f; out[2] = 0.15f;
  } else {
    out[0] = 0.38f; out[1] = 0.48f; out[2] = 0.14f;
  }
  return 0;
}

float or_film_base_nominal(const char* preset) {
  std::string s(preset ? preset : "");
  for (auto& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  if (s == "t-max" || s == "tmax") return 0.024f;
  if (s == "hp5" || s == "hp5-plus") return 0.032f;
  if (s == "tri-x-1600" || s == "trix-1600" || s == "caffenol") return 0.042f;
  return 0.038f;
}

int or_luma(const uint8_t* rgb, uint32_t w, uint32_t h, const float wts[3], uint8_t* out) {
  const int64_t n = static_cast<int64_t>(w) * h;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const float r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
    float v = r * wts[0] + g * wts[1] + b * wts[2];
    v = v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v);
    out[i] = static_cast<uint8_t>(std::round(v));
  }
  return 0;
}

int or_resize_u8(const uint8_t* in, uint32_t w, uint32_t h, uint32_t ow, uint32_t oh, int filter,
                 uint8_t* out) {
  if (!w || !h || !ow || !oh) return 1;
  if (ow == w && oh == h) {
    std::memcpy(out, in, static_cast<size_t>(w) * h);
    return 0;
  }
  std::vector<uint32_t> left;
  std::vector<std::vector<float>> wt;
  resample_axis(h, oh, filter, left, wt);
  std::vector<float> tmp(static_cast<size_t>(w) * oh);
  // Rows are independent: OpenMP splits them, each pixel keeps its sequential tap order.
#pragma omp parallel for schedule(static)
  for (uint32_t y = 0; y < oh; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      float t = 0.0f;
      for (size_t i = 0; i < wt[y].size(); ++i)
        t += static_cast<float>(in[static_cast<size_t>(left[y] + i) * w + x]) * wt[y][i];
      tmp[static_cast<size_t>(y) * w + x] = t;
    }
  resample_axis(w, ow, filter, left, wt);
#pragma omp parallel for schedule(static)
  for (uint32_t y = 0; y < oh; ++y)
    for (uint32_t x = 0; x < ow; ++x) {
      float t = 0.0f;
      for (size_t i = 0; i < wt[x].size(); ++i) t += tmp[static_cast<size_t>(y) * w + left[x] + i] * wt[x][i];
      t = t < 0.0f ? 0.0f : (t > 255.0f ? 255.0f : t);
      out[static_cast<size_t>(y) * ow + x] = static_cast<uint8_t>(std::round(t));
    }
  return 0;
}

int or_gelatin_psf(const uint8_t* src, uint32_t w, uint32_t h, float* heff, uint32_t gate[4]) {
  const size_t n = static_cast<size_t>(w) * h;
  auto px = [&](uint32_t x, uint32_t y) { return src[static_cast<size_t>(y) * w + x]; };
  uint32_t top = 0;
  while (top < h) {
    bool all0 = true;
    for (uint32_t x = 0; x < w && all0; ++x) all0 = px(x, top) == 0;
    if (!all0) break;
    ++top;
  }
  uint32_t bottom = h;
  while (bottom > top) {
    bool all0 = true;
    for (uint32_t x = 0; x < w && all0; ++x) all0 = px(x, bottom - 1) == 0;
    if (!all0) break;
    --bottom;
  }
  uint32_t left = 0;
  while (left < w) {
    bool all0 = true;
    for (uint32_t y = top; y < bottom && all0; ++y) all0 = px(left, y) == 0;
    if (!all0) break;
    ++left;
  }
  uint32_t right = w;
  while (right > left) {
    bool all0 = true;
    for (uint32_t y = top; y < bottom && all0; ++y) all0 = px(right - 1, y) == 0;
    if (!all0) break;
    --right;
  }
  if (gate) { gate[0] = top; gate[1] = bottom; gate[2] = left; gate[3] = right; }
  std::vector<float> lin(n, 0.0f);
  for (uint32_t y = top; y < bottom; ++y)
    for (uint32_t x = left; x < right; ++x) lin[static_cast<size_t>(y) * w + x] = static_cast<float>(px(x, y)) / 255.0f;
  const float wn[3] = {0.15f, 0.70f, 0.15f};
  const float ww[7] = {0.03f, 0.12f, 0.20f, 0.30f, 0.20f, 0.12f, 0.03f};
  auto pass = [&](const std::vector<float>& in, std::vector<float>& out, const float* k, int rad, int axis) {
#pragma omp parallel for schedule(static)
    for (uint32_t y = top; y < bottom; ++y)
      for (uint32_t x = left; x < right; ++x) {
        float sum = 0.0f, ws = 0.0f;
        for (int i = 0; i <= 2 * rad; ++i) {
          if (axis == 0) {
            const int64_t tap = static_cast<int64_t>(x) + i - rad;
            if (tap >= left && tap < right) {
              sum += in[static_cast<size_t>(y) * w + static_cast<size_t>(tap)] * k[i];
              ws += k[i];
            }
          } else {
            const int64_t tap = static_cast<int64_t>(y) + i - rad;
            if (tap >= top && tap < bottom) {
              sum += in[static_cast<size_t>(tap) * w + x] * k[i];
              ws += k[i];
            }
          }
        }
        out[static_cast<size_t>(y) * w + x] = sum / std::fmax(ws, 1e-6f);
      }
  };
  std::vector<float> tn(n, 0.0f), on(n, 0.0f), tw(n, 0.0f), ow(n, 0.0f);
  pass(lin, tn, wn, 1, 0);
  pass(tn, on, wn, 1, 1);
  pass(lin, tw, ww, 3, 0);
  pass(tw, ow, ww, 3, 1);
  for (size_t i = 0; i < n; ++i) heff[i] = 0.0f;
#pragma omp parallel for schedule(static)
  for (uint32_t y = top; y < bottom; ++y)
    for (uint32_t x = left; x < right; ++x) {
      const size_t i = static_cast<size_t>(y) * w + x;
      heff[i] = 0.90f * on[i] + 0.10f * ow[i];
    }
  return 0;
}

int or_film_finish(const or_finish_cfg* cfg, uint32_t out_w, uint32_t out_h, uint32_t tile_step, uint32_t pad,
                   uint32_t ntiles, const uint32_t* desc, const float* const* tiles, const uint8_t* src,
                   const float* heff, uint8_t* out, float* fields, float* stats) {
  const size_t n = static_cast<size_t>(out_w) * out_h;
  const uint32_t ntx = (out_w + tile_step - 1) / tile_step, nty = (out_h + tile_step - 1) / tile_step;
  // Hann overlap accumulation (image_pipeline.rs:593-649), tiles in list order.
  std::vector<float> acc(n, 0.0f), wacc(n, 0.0f), wsq(n, 0.0f);
  const float pad2 = static_cast<float>(2 * pad);
  const float pi = 3.14159265358979323846f;
  auto hann = [&](uint32_t t, uint32_t g, uint32_t nt, uint32_t o0) {
    if (t > 0 && g < o0 + pad) {
      const float u = (static_cast<float>(g) - (static_cast<float>(o0) - static_cast<float>(pad))) / pad2;
      return 0.5f - 0.5f * std::cos(pi * std::fmin(std::fmax(u, 0.0f), 1.0f));
    }
    if (t + 1 < nt && g >= o0 + tile_step - pad) {
      const float u = (static_cast<float>(g) - (static_cast<float>(o0 + tile_step) - static_cast<float>(pad))) / pad2;
      return 0.5f + 0.5f * std::cos(pi * std::fmin(std::fmax(u, 0.0f), 1.0f));
    }
    return 1.0f;
  };
  for (uint32_t t = 0; t < ntiles; ++t) {
    const uint32_t tx = desc[6 * t], ty = desc[6 * t + 1], xs = desc[6 * t + 2], ys = desc[6 * t + 3];
    const uint32_t tw = desc[6 * t + 4], th = desc[6 * t + 5];
    for (uint32_t py = 0; py < th; ++py) {
      const uint32_t gy = ys + py;
      const float wy = hann(ty, gy, nty, ty * tile_step);
      for (uint32_t px = 0; px < tw; ++px) {
        const uint32_t gx = xs + px;
        const float wv = hann(tx, gx, ntx, tx * tile_step) * wy;
        const size_t gi = static_cast<size_t>(gy) * out_w + gx;
        acc[gi] += tiles[t][static_cast<size_t>(py) * tw + px] * wv;
        wacc[gi] += wv;
        wsq[gi] += wv * wv;
      }
    }
  }
  std::vector<float> dn(n);
  for (size_t i = 0; i < n; ++i) dn[i] = acc[i] / std::fmax(wacc[i], 1e-5f);
  // Low-frequency split (image_pipeline.rs:651-706).
  const float sigma = std::fmax(static_cast<float>(cfg->grain_size_px) * 1.5f, 1.5f);
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
  std::vector<float> tl(n), dl(n);
  for (uint32_t y = 0; y < out_h; ++y)
    for (uint32_t x = 0; x < out_w; ++x) {
      float s = 0.0f, ws = 0.0f;
      for (int k = 0; k <= 2 * krad; ++k) {
        const int64_t tap = static_cast<int64_t>(x) + k - krad;
        if (tap >= 0 && tap < out_w) {
          s += dn[static_cast<size_t>(y) * out_w + static_cast<size_t>(tap)] * kern[k];
          ws += kern[k];
        }
      }
      tl[static_cast<size_t>(y) * out_w + x] = s / std::fmax(ws, 1e-6f);
    }
  for (uint32_t y = 0; y < out_h; ++y)
    for (uint32_t x = 0; x < out_w; ++x) {
      float s = 0.0f, ws = 0.0f;
      for (int k = 0; k <= 2 * krad; ++k) {
        const int64_t tap = static_cast<int64_t>(y) + k - krad;
        if (tap >= 0 && tap < out_h) {
          s += tl[static_cast<size_t>(tap) * out_w + x] * kern[k];
          ws += kern[k];
        }
      }
      dl[static_cast<size_t>(y) * out_w + x] = s / std::fmax(ws, 1e-6f);
    }
  // Grain statistics (image_pipeline.rs:708-716): sequential f32 sums.
  const float np1 = static_cast<float>(std::max<size_t>(n, 1));
  float s1 = 0.0f;
  for (size_t i = 0; i < n; ++i) s1 += dn[i] - dl[i];
  const float mean = s1 / np1;
  float s2 = 0.0f;
  for (size_t i = 0; i < n; ++i) {
    const float d = dn[i] - dl[i] - mean;
    s2 += d * d;
  }
  const float sd = std::fmax(std::sqrt(s2 / np1), 0.035f);
  const float push_mult = 1.0f + 0.15f * static_cast<float>(cfg->push);
  const float amp = cfg->base_nominal * push_mult;
  const float norm = std::fmin((amp * static_cast<float>(cfg->strength)) / sd, 2.2f);
  if (stats) { stats[0] = mean; stats[1] = sd; stats[2] = norm; stats[3] = 0.0f; }
  // Sensitometric composite (image_pipeline.rs:728-808).
  const bool pushed = cfg->push > 0.0;
  const float gamma = 1.0f + 0.06f * static_cast<float>(cfg->push);
  std::vector<float> grain(n), tone(n);
  for (size_t i = 0; i < n; ++i) {
    const float w_val = std::fmax(wacc[i], 1e-5f);
    const float wsn = std::fmax(wsq[i] / (w_val * w_val), 0.05f);
    const float gs = std::fmin(1.0f / std::sqrt(wsn), 1.45f);
    const float d_high = dn[i] - dl[i];
    const float raw = static_cast<float>(src[i]) / 255.0f;
    const float base = raw <= 0.005f ? 0.0f : 0.35f * raw + 0.65f * heff[i];
    const float sg = smoothstep_gate_lo(base), hg = smoothstep_gate_hi(base);
    const float mid = std::fmax(std::sin(pi * std::pow(std::fmin(std::fmax(base, 0.0f), 1.0f), 0.72f)), 0.0f);
    const float vis = sg * hg * mid;
    float tv = base;
    if (pushed) {
      tv = base <= 0.5f ? 0.5f * std::pow(2.0f * base, gamma) : 1.0f - 0.5f * std::pow(2.0f * (1.0f - base), gamma);
    }
    const float dd = d_high - mean;
    const float sharp = std::fabs(dd) > 1e-6f ? std::copysign(1.0f, dd) * std::pow(std::fabs(dd), 0.85f) : 0.0f;
    grain[i] = sharp * norm * gs * vis;
    tone[i] = tv;
  }
  // Scanner OTF (image_pipeline.rs:825-855) and the output gates (image_pipeline.rs:857-891).
  std::vector<float> scanned(grain);
  if (cfg->scanner_otf) {
    const float k[3] = {0.035f, 0.93f, 0.035f};
    std::vector<float> tmp(n);
    for (uint32_t y = 0; y < out_h; ++y)
      for (uint32_t x = 0; x < out_w; ++x) {
        const uint32_t xm = x > 0 ? x - 1 : 0, xp = std::min(x + 1, out_w - 1);
        const size_t r = static_cast<size_t>(y) * out_w;
        tmp[r + x] = grain[r + xm] * k[0] + grain[r + x] * k[1] + grain[r + xp] * k[2];
      }
    for (uint32_t y = 0; y < out_h; ++y) {
      const uint32_t ym = y > 0 ? y - 1 : 0, yp = std::min(y + 1, out_h - 1);
      for (uint32_t x = 0; x < out_w; ++x)
        scanned[static_cast<size_t>(y) * out_w + x] = tmp[static_cast<size_t>(ym) * out_w + x] * k[0] +
                                                      tmp[static_cast<size_t>(y) * out_w + x] * k[1] +
                                                      tmp[static_cast<size_t>(yp) * out_w + x] * k[2];
    }
  }
  for (size_t i = 0; i < n; ++i) {
    const float raw = static_cast<float>(src[i]) / 255.0f;
    const float gated = scanned[i] * smoothstep_gate_lo(raw) * smoothstep_gate_hi(raw);
    float v = tone[i] + 0.0f + gated;
    v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
    out[i] = static_cast<uint8_t>(std::round(v * 255.0f));
  }
  if (fields) {
    std::memcpy(fields, dn.data(), n * sizeof(float));
    std::memcpy(fields + n, dl.data(), n * sizeof(float));
    std::memcpy(fields + 2 * n, grain.data(), n * sizeof(float));
    std::memcpy(fields + 3 * n, tone.data(), n * sizeof(float));
    std::memcpy(fields + 4 * n, scanned.data(), n * sizeof(float));
  }
  return 0;
}

}  // extern "C"
