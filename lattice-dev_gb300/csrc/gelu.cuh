// gelu.cuh -- the closure network's activation: GELU in its tanh form,
//   gelu(z)  = z/2 (1 + tanh(u)),  u = sqrt(2/pi) (z + 0.044715 z^3),
//   gelu'(z) = (1 + t)/2 + z/2 (1 - t^2) sqrt(2/pi) (1 + 3 0.044715 z^2),  t = tanh(u),
// with tanh from the hardware approximation (tanh.approx.f32, relative error
// about 2^-11, below the BF16 rounding of the stored activations).
#pragma once

namespace lat {
namespace net {

__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float gelu_t(float z) {
  const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
  return 0.5f * z * (1.0f + tanh_hw(u));
}

__device__ __forceinline__ float gelu_t_d(float z) {
  const float z2 = z * z;
  const float t = tanh_hw(0.7978845608028654f * (z + 0.044715f * z2 * z));
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * 0.7978845608028654f * (1.0f + 0.134145f * z2);
}

}  // namespace net
}  // namespace lat
