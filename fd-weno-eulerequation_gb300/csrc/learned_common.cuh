// Definitions shared by the learned-indicator translation units: the
// network's parameter layout, its GELU, and the per-cell window
// normalisation of the features.
#pragma once

#include "convert.cuh"
#include "wenofd_internal.h"

namespace wenofd {
namespace lrn {

constexpr int kIn = 50, kHid = 32;
constexpr int oW1 = 0, oB1 = 1600, oW2 = 1632, oB2 = 2656, oW3 = 2688, oB3 = 2720;
constexpr int kParams = 2721;
constexpr float kFlat = 1e-4f;  // relative range below which a window counts as flat

__device__ __forceinline__ float gelu(float z) {
  const float k = 0.7978845608028654f;  // sqrt(2/pi)
  return 0.5f * z * (1.0f + tanhf(k * (z + 0.044715f * z * z * z)));
}

__device__ __forceinline__ float gelu_grad(float z) {
  const float k = 0.7978845608028654f;
  const float t = tanhf(k * (z + 0.044715f * z * z * z));
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * k * (1.0f + 3.0f * 0.044715f * z * z);
}

__device__ __forceinline__ float pressure32(float gamma, float r, float mu, float mv, float E) {
  const float u = mu / r, v = mv / r;
  return (gamma - 1.0f) * (E - 0.5f * r * (u * u + v * v));
}

// (v - centre) * (1 / max|v - centre|) over the 25-point window, or zeros when the
// window is flat (range <= 1e-4 (|centre| + 1e-12)).
__device__ __forceinline__ void normalise(const float w[25], float out[25]) {
  const float c = w[12];
  float R = 0.0f;
#pragma unroll
  for (int k = 0; k < 25; ++k) R = fmaxf(R, fabsf(w[k] - c));
  if (R <= kFlat * (fabsf(c) + 1e-12f)) {
#pragma unroll
    for (int k = 0; k < 25; ++k) out[k] = 0.0f;
    return;
  }
  const float inv = 1.0f / R;
#pragma unroll
  for (int k = 0; k < 25; ++k) out[k] = (w[k] - c) * inv;
}

// GELU for inference: the same tanh form with the hardware tanh
// approximation (the BF16 operands that follow are coarser than its error).
__device__ __forceinline__ float gelu_fast(float z) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.7978845608028654f * (z + 0.044715f * z * z * z)));
  return 0.5f * z * (1.0f + t);
}

inline int grid_for(long long work, int threads, int cap) {
  long long b = (work + threads - 1) / threads;
  if (b > cap) b = cap;
  return int(b < 1 ? 1 : b);
}

}  // namespace lrn
}  // namespace wenofd
