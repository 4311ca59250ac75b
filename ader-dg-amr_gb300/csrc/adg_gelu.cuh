// GELU activation of the learned seed's network (shared by the SIMT training
// kernels and the tensor-core inference kernel).
#pragma once

#include <cuda_runtime.h>

namespace adg {
namespace mlp {

// GELU, tanh form (Hendrycks & Gimpel 2016): 0.5 z (1 + tanh(k (z + a z^3))).
constexpr float kGeluK = 0.7978845608028654f;  // sqrt(2/pi)
constexpr float kGeluA = 0.044715f;

__device__ __forceinline__ float gelu(float z) {
  const float t = tanhf(kGeluK * (z + kGeluA * z * z * z));
  return 0.5f * z * (1.0f + t);
}

__device__ __forceinline__ float gelu_grad(float z) {
  const float t = tanhf(kGeluK * (z + kGeluA * z * z * z));
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * kGeluK * (1.0f + 3.0f * kGeluA * z * z);
}

}  // namespace mlp
}  // namespace adg
