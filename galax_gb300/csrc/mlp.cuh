// The potential-surrogate MLP: 3 -> 256 -> 256 -> 256 -> 256 -> 1, SiLU.
// Parameter vector layout (float32, contiguous) and the activation functions
// shared by the training and inference kernels.
#pragma once

#include <cstdint>

namespace gal {
namespace mlp {

constexpr int H = 256;
// offsets into the parameter vector
constexpr int64_t OFF_W1 = 0;                   // [H][3]
constexpr int64_t OFF_B1 = OFF_W1 + H * 3;      // [H]
constexpr int64_t OFF_W2 = OFF_B1 + H;          // [H][H] (row = output unit)
constexpr int64_t OFF_B2 = OFF_W2 + H * H;
constexpr int64_t OFF_W3 = OFF_B2 + H;
constexpr int64_t OFF_B3 = OFF_W3 + H * H;
constexpr int64_t OFF_W4 = OFF_B3 + H;
constexpr int64_t OFF_B4 = OFF_W4 + H * H;
constexpr int64_t OFF_W5 = OFF_B4 + H;          // [H]
constexpr int64_t OFF_B5 = OFF_W5 + H;          // [1]
constexpr int64_t NPARAM = OFF_B5 + 1;          // 198,657

// On the device the exponential and the reciprocal come from the SFU
// (__expf, __frcp_rn: a few units in the last place, ~1e-6 relative at
// worst), which keeps the elementwise work of the training products short;
// the network's activations are rounded to bfloat16 anyway.
__host__ __device__ __forceinline__ float sigmoidf_(float z) {
#ifdef __CUDA_ARCH__
  return __frcp_rn(1.0f + __expf(-z));
#else
  return 1.0f / (1.0f + expf(-z));
#endif
}
__host__ __device__ __forceinline__ float silu(float z) { return z * sigmoidf_(z); }
__host__ __device__ __forceinline__ float dsilu(float z) {
  const float s = sigmoidf_(z);
  return s * (1.0f + z * (1.0f - s));
}
__host__ __device__ __forceinline__ float d2silu(float z) {
  const float s = sigmoidf_(z);
  return s * (1.0f - s) * (2.0f + z * (1.0f - 2.0f * s));
}

// Round to bfloat16 (nearest even) and back to float.
__host__ __device__ __forceinline__ float bf16r(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return f;  // inf / nan unchanged
  u += 0x7fffu + ((u >> 16) & 1u);
  u &= 0xffff0000u;
  float r;
  memcpy(&r, &u, 4);
  return r;
}

}  // namespace mlp
}  // namespace gal
