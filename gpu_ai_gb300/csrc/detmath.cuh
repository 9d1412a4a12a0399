// detmath.cuh -- float arithmetic of the search kernels with a fixed sequence
// of correctly rounded operations, so that a CPU restatement (numpy float32
// scalars) reproduces every result bit for bit.
//
// Every product, sum, quotient and square root is an explicit round-to-nearest
// intrinsic, which the compiler never fuses into an FMA.  The elementary
// functions are this file's own, from textbook methods:
//   det_log  ln x = e ln 2 + ln m with m in [sqrt(1/2), sqrt(2)), and
//            ln m = 2 atanh(s), s = (m - 1) / (m + 1), by its odd power series
//            up to s^11 (|s| <= 0.172, so the next term is below 1e-10);
//   det_exp  Cody & Waite's reduction x = k ln 2 + r with ln 2 split into a
//            16-bit head (k * head is exact for |k| <= 128) and a tail, the
//            Taylor polynomial of e^r to degree 7 (|r| <= 0.347: remainder
//            below 6e-9), scaled by 2^k built from its exponent bits;
//   det_tanh (1 - e^(-2|x|)) / (1 + e^(-2|x|)) with the sign of x.
// Constants are given as their float bit patterns (the correctly rounded
// values of 1/k, 1/k!, ln 2 and log2 e).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ga {
namespace dm {

__device__ __forceinline__ float cf(uint32_t bits) { return __uint_as_float(bits); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }

constexpr uint32_t kLn2 = 0x3f317218u, kLog2e = 0x3fb8aa3bu, kLn2Hi = 0x3f317200u, kLn2Lo = 0x35bfbe8eu;
constexpr uint32_t kSqrt2 = 0x3fb504f3u;
constexpr uint32_t kInv3 = 0x3eaaaaabu, kInv5 = 0x3e4ccccdu, kInv7 = 0x3e124925u, kInv9 = 0x3de38e39u,
                   kInv11 = 0x3dba2e8cu;
constexpr uint32_t kInvF3 = 0x3e2aaaabu, kInvF4 = 0x3d2aaaabu, kInvF5 = 0x3c088889u, kInvF6 = 0x3ab60b61u,
                   kInvF7 = 0x39500d01u;

// Natural logarithm of a positive normal float.
__device__ __forceinline__ float det_log(float x) {
  const uint32_t u = __float_as_uint(x);
  int e = (int)(u >> 23) - 127;
  float m = __uint_as_float((u & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > cf(kSqrt2)) {
    m = mul(m, 0.5f);
    e += 1;
  }
  const float s = div(sub(m, 1.0f), add(m, 1.0f));
  const float s2 = mul(s, s);
  float p = cf(kInv11);
  p = add(mul(p, s2), cf(kInv9));
  p = add(mul(p, s2), cf(kInv7));
  p = add(mul(p, s2), cf(kInv5));
  p = add(mul(p, s2), cf(kInv3));
  p = add(mul(p, s2), 1.0f);
  return add(mul((float)e, cf(kLn2)), mul(mul(2.0f, s), p));
}

// e^x for x <= 0 (0 below -87).
__device__ __forceinline__ float det_exp(float x) {
  if (!(x >= -87.0f)) return 0.0f;
  const float k = rintf(mul(x, cf(kLog2e)));
  const float r = sub(sub(x, mul(k, cf(kLn2Hi))), mul(k, cf(kLn2Lo)));
  float p = cf(kInvF7);
  p = add(mul(p, r), cf(kInvF6));
  p = add(mul(p, r), cf(kInvF5));
  p = add(mul(p, r), cf(kInvF4));
  p = add(mul(p, r), cf(kInvF3));
  p = add(mul(p, r), 0.5f);
  p = add(mul(p, r), 1.0f);
  p = add(mul(p, r), 1.0f);
  const int ki = (int)k;  // -126 <= k <= 0
  return mul(p, __uint_as_float((uint32_t)(ki + 127) << 23));
}

__device__ __forceinline__ float det_tanh(float x) {
  const float a = fabsf(x);
  float y;
  if (a > 9.0f) {
    y = 1.0f;
  } else {
    const float t = det_exp(mul(-2.0f, a));
    y = div(sub(1.0f, t), add(1.0f, t));
  }
  return x < 0.0f ? -y : y;
}

}  // namespace dm
}  // namespace ga
