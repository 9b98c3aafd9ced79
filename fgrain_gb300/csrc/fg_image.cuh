// Shared pieces of the image stages (fg_image.cu, fg_film.cu).
#pragma once
#include <vector>

#include "fg_internal.h"

namespace fg {

// Hann weight of global coordinate g in tile t of nt along one axis (image_pipeline.rs:613-638).
__device__ __forceinline__ float hann_weight(uint32_t t, uint32_t g, uint32_t nt, uint32_t o0, uint32_t step,
                                            uint32_t pad) {
  const float pad2 = static_cast<float>(2 * pad);
  const float pi = 3.14159265358979323846f;
  if (t > 0 && g < o0 + pad) {
    const float u = __fdiv_rn(__fsub_rn(static_cast<float>(g), __fsub_rn(static_cast<float>(o0), static_cast<float>(pad))), pad2);
    const float c = static_cast<float>(cos(static_cast<double>(__fmul_rn(pi, fminf(fmaxf(u, 0.0f), 1.0f)))));
    return __fsub_rn(0.5f, __fmul_rn(0.5f, c));
  }
  if (t + 1 < nt && g >= o0 + step - pad) {
    const float u = __fdiv_rn(__fsub_rn(static_cast<float>(g), __fsub_rn(static_cast<float>(o0 + step), static_cast<float>(pad))),
                              pad2);
    const float c = static_cast<float>(cos(static_cast<double>(__fmul_rn(pi, fminf(fmaxf(u, 0.0f), 1.0f)))));
    return __fadd_rn(0.5f, __fmul_rn(0.5f, c));
  }
  return 1.0f;
}

// Resampling weights of the image crate's separable filter for n samples to m (image 0.25.10
// imageops::sample): filter 0 Triangle (support 1), 1 Lanczos3 (support 3); the support scales
// with the ratio when shrinking and each output's weights are normalised to sum 1.  Output o
// reads cnt[o] inputs from left[o] with weights wts[o * stride + k].
enum : int { RESAMPLE_TRIANGLE = 0, RESAMPLE_LANCZOS3 = 1 };
void resample_weights(uint32_t n, uint32_t m, int filter, std::vector<uint32_t>& left, std::vector<uint32_t>& cnt,
                      std::vector<float>& wts, uint32_t& stride);

// Separable 3-tap clamp-to-edge pass (fg_image.cu): out = in[-1] k0 + in[0] k1 + in[+1] k2 along
// x (axis 0) or y, optionally scaled.
__global__ void k_otf_pass(const float* __restrict__ in, float* __restrict__ out, uint32_t w, uint32_t h, float k0,
                           float k1, float k2, int axis, float scale);

}  // namespace fg
