// The differentiable scan and its hand-written adjoint.
//
// Scanned signal S = OTF_s(e T) per pixel: T is the stratified mean transmittance of the scan
// (k_scan, per-crystal opacities sigma_c), e an exposure multiplier and OTF_s the scanner's
// separable 3-tap clamp-to-edge filter (image_pipeline.rs:825-855) with taps (g, 1, g) / (1 + 2 g),
// g = exp(-1 / (2 s^2)); s = 0.3904441347190481 gives the reference's taps (0.035, 0.93, 0.035).
//
// For an upstream gradient G = dL/dS the adjoint returns
//   dL/de       = sum_p G_p OTF_s(T)_p
//   dL/ds       = e sum_p G_p (d OTF_s / ds)(T)_p
//   dL/dsigma_c = sum_p W_p dT_p/dsigma_c,   W = e OTF_s^T(G),
//                 dT_p/dsigma_c = -(1/spp) sum over the pixel's rays of T_ray chord_c(ray).
// The per-crystal part recomputes the forward from the developed mask (k_scan_adjoint) rather than
// storing per-ray intermediates.  Reductions are FP64 and deterministic; the per-crystal sums use
// FP64 atomics.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fg_internal.h"

namespace fg {

namespace {

struct Taps {
  double k[3], dk[3];
};

Taps otf_taps(double s) {
  FG_REQUIRE(s > 0.0 && std::isfinite(s), "OTF width must be positive");
  Taps t;
  const double g = std::exp(-1.0 / (2.0 * s * s));
  const double n = 1.0 + 2.0 * g;
  t.k[0] = t.k[2] = g / n;
  t.k[1] = 1.0 / n;
  const double dg = g / (s * s * s);
  t.dk[0] = t.dk[2] = dg / (n * n);
  t.dk[1] = -2.0 * dg / (n * n);
  return t;
}

__device__ __forceinline__ uint32_t clampm(uint32_t v) { return v > 0 ? v - 1 : 0; }
__device__ __forceinline__ uint32_t clampp(uint32_t v, uint32_t n) { return v + 1 < n ? v + 1 : n - 1; }

// Per-block partial sums of G OTF(T) and G dOTF(T)/ds (FP64), from each pixel's 3x3 neighbourhood.
constexpr int RED_THREADS = 256;
__global__ void __launch_bounds__(RED_THREADS) k_otf_grads(const float* __restrict__ T, const float* __restrict__ G,
                                                           uint32_t w, uint32_t h, Taps tp, double* partial) {
  double s0 = 0.0, s1 = 0.0;
  const size_t np = static_cast<size_t>(w) * h;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < np;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>(i / w);
    const uint32_t xs[3] = {clampm(x), x, clampp(x, w)};
    const uint32_t ys[3] = {clampm(y), y, clampp(y, h)};
    double o = 0.0, d = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float* row = T + static_cast<size_t>(ys[j]) * w;
      double hv = 0.0, dh = 0.0;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const double v = row[xs[q]];
        hv += tp.k[q] * v;
        dh += tp.dk[q] * v;
      }
      o += tp.k[j] * hv;
      d += tp.dk[j] * hv + tp.k[j] * dh;
    }
    const double g = G[i];
    s0 += g * o;
    s1 += g * d;
  }
  __shared__ double r0[RED_THREADS], r1[RED_THREADS];
  r0[threadIdx.x] = s0;
  r1[threadIdx.x] = s1;
  __syncthreads();
  for (int o = RED_THREADS / 2; o > 0; o >>= 1) {
    if (static_cast<int>(threadIdx.x) < o) {
      r0[threadIdx.x] += r0[threadIdx.x + o];
      r1[threadIdx.x] += r1[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = r0[0];
    partial[2 * blockIdx.x + 1] = r1[0];
  }
}

__global__ void k_sum_partials(const double* partial, int n, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a = 0.0, b = 0.0;
  for (int i = 0; i < n; ++i) {
    a += partial[2 * i];
    b += partial[2 * i + 1];
  }
  out[0] = a;
  out[1] = b;
}

// Weight of output position o on input position i for one clamp-to-edge 3-tap pass.
__device__ __forceinline__ double tap_weight(uint32_t o, uint32_t i, uint32_t n, const double k[3]) {
  double wv = 0.0;
  if (clampm(o) == i) wv += k[0];
  if (o == i) wv += k[1];
  if (clampp(o, n) == i) wv += k[2];
  return wv;
}

// wpx = -e OTF^T(G) = -e H^T(V^T(G)): the weight of each pixel's transmittance in the loss,
// negated for the per-crystal adjoint (dT/dsigma carries a minus sign).
__global__ void k_otf_adjoint(const float* __restrict__ G, uint32_t w, uint32_t h, Taps tp, double e,
                              float* __restrict__ wpx) {
  const size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<size_t>(w) * h) return;
  const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>(i / w);
  double acc = 0.0;
  for (int dy = -1; dy <= 1; ++dy) {
    const int oy = static_cast<int>(y) + dy;
    if (oy < 0 || oy >= static_cast<int>(h)) continue;
    const double wy = tap_weight(static_cast<uint32_t>(oy), y, h, tp.k);
    if (wy == 0.0) continue;
    for (int dx = -1; dx <= 1; ++dx) {
      const int ox = static_cast<int>(x) + dx;
      if (ox < 0 || ox >= static_cast<int>(w)) continue;
      const double wx = tap_weight(static_cast<uint32_t>(ox), x, w, tp.k);
      acc += wx * wy * G[static_cast<size_t>(oy) * w + ox];
    }
  }
  wpx[i] = static_cast<float>(-e * acc);
}

// T per pixel (device) for the differentiable scan: the forward scan in Negative mode with the
// given per-crystal opacities (Morton order on the device, or null for the config's opacity).
void scan_T(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg& cfg, uint64_t seed, const float* sigma_sorted,
            float* T) {
  fg_scan_cfg c = cfg;
  c.mode = 0;
  ScanOut so;
  so.out = T;
  scan(e, em, c, seed, sigma_sorted, so);
}

}  // namespace
}  // namespace fg

using namespace fg;

extern "C" {

fg_status fg_scan_signal(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg* cfg, uint64_t seed,
                         const float* sigma_per_crystal, double exposure, double otf_sigma, float* signal,
                         float* transmittance) {
  return guard(e, [&] {
    FG_REQUIRE(em && cfg && (signal || transmittance), "null argument");
    FG_REQUIRE(std::isfinite(exposure), "exposure multiplier must be finite");
    cudaStream_t st = e->stream;
    begin_call(e);
    const Taps tp = otf_taps(otf_sigma);
    const size_t np = static_cast<size_t>(cfg->width_px) * cfg->height_px;
    DBuf<float> sig, T(std::max<size_t>(np, 1), st), H(std::max<size_t>(np, 1), st), S(std::max<size_t>(np, 1), st);
    if (sigma_per_crystal) {
      const std::vector<float> sv = to_sorted(em, sigma_per_crystal);
      sig.alloc(std::max<size_t>(sv.size(), 1), st);
      if (!sv.empty()) FG_CUDA(cudaMemcpyAsync(sig.p, sv.data(), sv.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    }
    FG_CUDA(cudaEventRecord(e->timer.ev[0], st));
    scan_T(e, em, *cfg, seed, sigma_per_crystal ? sig.p : nullptr, T.p);
    const float kf[3] = {static_cast<float>(tp.k[0]), static_cast<float>(tp.k[1]), static_cast<float>(tp.k[2])};
    launch_otf(T.p, H.p, S.p, cfg->width_px, cfg->height_px, kf, static_cast<float>(exposure), st);
    FG_CUDA(cudaEventRecord(e->timer.ev[1], st));
    if (signal) FG_CUDA(cudaMemcpyAsync(signal, S.p, np * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (transmittance) FG_CUDA(cudaMemcpyAsync(transmittance, T.p, np * sizeof(float), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    e->timings.scan_ms = elapsed(e->timer.ev[0], e->timer.ev[1]);
    e->timings.total_ms = e->timings.scan_ms;
    end_call(e);
  });
}

fg_status fg_scan_backward(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg* cfg, uint64_t seed,
                           const float* sigma_per_crystal, double exposure, double otf_sigma, const float* dL_dsignal,
                           float* dL_dsigma, double* dL_dexposure, double* dL_dotf_sigma) {
  return guard(e, [&] {
    FG_REQUIRE(em && cfg && dL_dsignal, "null argument");
    FG_REQUIRE(std::isfinite(exposure), "exposure multiplier must be finite");
    cudaStream_t st = e->stream;
    begin_call(e);
    const Taps tp = otf_taps(otf_sigma);
    const uint32_t w = cfg->width_px, h = cfg->height_px;
    const size_t np = static_cast<size_t>(w) * h;
    DBuf<float> sig, T(std::max<size_t>(np, 1), st), Gd(std::max<size_t>(np, 1), st), W(std::max<size_t>(np, 1), st);
    if (sigma_per_crystal) {
      const std::vector<float> sv = to_sorted(em, sigma_per_crystal);
      sig.alloc(std::max<size_t>(sv.size(), 1), st);
      if (!sv.empty()) FG_CUDA(cudaMemcpyAsync(sig.p, sv.data(), sv.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    }
    if (np) FG_CUDA(cudaMemcpyAsync(Gd.p, dL_dsignal, np * sizeof(float), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaEventRecord(e->timer.ev[0], st));
    // Forward transmittance, recomputed from the developed mask.
    scan_T(e, em, *cfg, seed, sigma_per_crystal ? sig.p : nullptr, T.p);
    // Exposure multiplier and OTF width.
    const int nblk = static_cast<int>(std::min<size_t>((np + RED_THREADS - 1) / RED_THREADS, 1024));
    DBuf<double> part(2 * static_cast<size_t>(std::max(nblk, 1)), st), sums(2, st);
    FG_CUDA(cudaMemsetAsync(sums.p, 0, 2 * sizeof(double), st));
    if (np) {
      k_otf_grads<<<nblk, RED_THREADS, 0, st>>>(T.p, Gd.p, w, h, tp, part.p);
      k_sum_partials<<<1, 32, 0, st>>>(part.p, nblk, sums.p);
      FG_CUDA(cudaGetLastError());
    }
    double hs[2] = {0.0, 0.0};
    FG_CUDA(cudaMemcpyAsync(hs, sums.p, sizeof(hs), cudaMemcpyDeviceToHost, st));
    // Per-crystal opacities.
    DBuf<double> g;
    if (dL_dsigma && em->n) {
      k_otf_adjoint<<<grid_for(np, 256), 256, 0, st>>>(Gd.p, w, h, tp, exposure, W.p);
      FG_CUDA(cudaGetLastError());
      g.alloc(em->n, st);
      FG_CUDA(cudaMemsetAsync(g.p, 0, em->n * sizeof(double), st));
      scan_adjoint(e, em, *cfg, seed, sigma_per_crystal ? sig.p : nullptr, W.p, g.p);
    }
    FG_CUDA(cudaEventRecord(e->timer.ev[1], st));
    std::vector<double> gs(dL_dsigma ? em->n : 0);
    if (dL_dsigma && em->n) FG_CUDA(cudaMemcpyAsync(gs.data(), g.p, em->n * sizeof(double), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (dL_dexposure) *dL_dexposure = hs[0];
    if (dL_dotf_sigma) *dL_dotf_sigma = exposure * hs[1];
    if (dL_dsigma) {
      std::vector<float> gf(gs.begin(), gs.end());
      from_sorted(em, gf, dL_dsigma);
    }
    e->timings.scan_ms = elapsed(e->timer.ev[0], e->timer.ev[1]);
    e->timings.total_ms = e->timings.scan_ms;
    end_call(e);
  });
}

}  // extern "C"
