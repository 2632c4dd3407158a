// The surrogate network's activation for inference, two values at a time:
// GELU in its tanh form, 0.5 z (1 + tanh(c (z + a z^3))), c = sqrt(2/pi),
// a = 0.044715 (Hendrycks & Gimpel, 2016), evaluated on packed FP16 pairs
// with the hardware tanh.approx.f16x2.  Its result is rounded to BF16 (the
// next layer's operand), whose 8-bit significand is coarser than FP16's 11
// bits, and its error stays below that rounding for |z| < 64; one tanh
// instruction serves two activations, which halves the load on the
// multi-function unit that bounds the network's epilogues.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace wrach {

// GELU of (z0, z1), rounded to a BF16 pair (z0 in the low half).
__device__ __forceinline__ uint32_t gelu2_bf16(float z0, float z1) {
  const __half2 z = __floats2half2_rn(z0, z1);
  const __half2 z2 = __hmul2(z, z);
  const __half2 p = __hfma2(__float2half2_rn(0.7978845608028654f * 0.044715f), z2,
                            __float2half2_rn(0.7978845608028654f));
  const __half2 u = __hmul2(z, p);
  uint32_t t;
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(*reinterpret_cast<const uint32_t*>(&u)));
  const __half2 h = __hmul2(__float2half2_rn(0.5f), z);
  const __half2 g = __hfma2(h, *reinterpret_cast<const __half2*>(&t), h);
  const float2 f = __half22float2(g);
  __nv_bfloat162 b = __floats2bfloat162_rn(f.x, f.y);
  return *reinterpret_cast<uint32_t*>(&b);
}

}  // namespace wrach
