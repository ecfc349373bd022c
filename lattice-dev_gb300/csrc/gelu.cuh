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

// two values per instruction (packed FP32 arithmetic), same formula:
// u = (sqrt(2/pi) z) (1 + 0.044715 z^2), gelu = (z/2) tanh(u) + z/2
__device__ __forceinline__ float2 gelu_t2(float2 z) {
  const float2 p = __ffma2_rn(__fmul2_rn(z, z), make_float2(0.044715f, 0.044715f), make_float2(1.0f, 1.0f));
  const float2 u = __fmul2_rn(__fmul2_rn(z, make_float2(0.7978845608028654f, 0.7978845608028654f)), p);
  const float2 hz = __fmul2_rn(z, make_float2(0.5f, 0.5f));
  return __ffma2_rn(hz, make_float2(tanh_hw(u.x), tanh_hw(u.y)), hz);
}

__device__ __forceinline__ float gelu_t_d(float z) {
  const float z2 = z * z;
  const float t = tanh_hw(0.7978845608028654f * (z + 0.044715f * z2 * z));
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * 0.7978845608028654f * (1.0f + 0.134145f * z2);
}

// gelu'(z) on two values per instruction, same formula:
// (1 + t)/2 + (sqrt(2/pi) z/2) (1 + 3 0.044715 z^2) (1 - t^2)
__device__ __forceinline__ float2 gelu_t_d2(float2 z) {
  const float2 z2 = __fmul2_rn(z, z);
  const float2 p = __ffma2_rn(z2, make_float2(0.044715f, 0.044715f), make_float2(1.0f, 1.0f));
  const float2 u = __fmul2_rn(__fmul2_rn(z, make_float2(0.7978845608028654f, 0.7978845608028654f)), p);
  const float2 t = make_float2(tanh_hw(u.x), tanh_hw(u.y));
  const float2 q = __ffma2_rn(z2, make_float2(0.134145f, 0.134145f), make_float2(1.0f, 1.0f));
  const float2 w = __fmul2_rn(__fmul2_rn(z, make_float2(0.3989422804014327f, 0.3989422804014327f)), q);
  const float2 om = __ffma2_rn(__fmul2_rn(t, t), make_float2(-1.0f, -1.0f), make_float2(1.0f, 1.0f));
  return __ffma2_rn(w, om, __ffma2_rn(t, make_float2(0.5f, 0.5f), make_float2(0.5f, 0.5f)));
}

}  // namespace net
}  // namespace lat
