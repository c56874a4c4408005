// Double-float arithmetic on the FP32 pipe (GB300's FP64 pipe runs ~1/73 of
// the FP32 rate): an FP64 operand is split into an FP32 pair hi + lo, a
// product term is formed with its exact FP32 rounding error (fma) plus the
// cross terms, and a sum is kept as an FP32 sum s with its rounding errors
// collected in t (Dekker's exact product, Knuth's two-sum).  A term carries
// ~2^-48 relative error, a sum of m terms ~2^-48 sqrt(m) of sum |a b|.
#pragma once

#include <cuda_runtime.h>

namespace bsg {

// x = hi + lo from the IEEE bits, with integer and FP32 operations only
// (FP64 and integer-to-float conversions run on GB300's narrow FP64-rate
// units): hi keeps the top 24 bits of the significand (truncated), lo the
// next 29 rounded to nearest to 24, so hi + lo carries ~48 bits.  The 29-bit
// remainder becomes a float through its two halves, each exact as
// (2^23 + v) - 2^23, and one fma that rounds once.  A lo below FP32's
// normal range (|x| < 2^-75) is dropped; x outside FP32's exponent range
// becomes 0 (|x| < 2^-126) or +-inf (|x| >= 2^128).  No FP64 instruction, so
// none can be predicated into a caller's hot loop.
__device__ __forceinline__ float2 df_split(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hw = unsigned(b >> 32), lw = unsigned(b);
  const int e = int((hw >> 20) & 0x7ffu);  // biased double exponent
  const int fe = e - 1023 + 127;
  const unsigned sign = hw & 0x80000000u;
  if (fe <= 0) return make_float2(0.f, 0.f);  // zero, double subnormal or below FP32's range
  if (fe >= 255) return make_float2(__uint_as_float(sign | 0x7f800000u), 0.f);
  const float h = __uint_as_float(sign | (unsigned(fe) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
  // the remaining 29 significand bits are r * 2^(e - 1023 - 52)
  const int pe = e - 1075 + 127;
  float l = 0.f;
  if (pe > 0) {
    const unsigned r = lw & 0x1fffffffu;
    const float rh = __uint_as_float(0x4B000000u | (r >> 14)) - 8388608.f;      // r >> 14 < 2^15
    const float rl = __uint_as_float(0x4B000000u | (r & 0x3fffu)) - 8388608.f;  // < 2^14
    l = fmaf(rh, 16384.f, rl) * __uint_as_float(unsigned(pe) << 23);
  }
  return make_float2(h, sign ? -l : l);
}

// (s, t) += a b
__device__ __forceinline__ void df_mac(float& s, float& t, float2 a, float2 b) {
  const float p = a.x * b.x;
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  const float u = s + p;
  const float bb = u - s;
  t += e + ((s - (u - bb)) + (p - bb));
  s = u;
}

// s + t renormalised to hi + lo (Knuth's two-sum)
__device__ __forceinline__ float2 df_norm(float s, float t) {
  const float h = s + t;
  const float bb = h - s;
  return make_float2(h, (s - (h - bb)) + (t - bb));
}

// a + b, renormalised
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  const float s = a.x + b.x;
  const float bb = s - a.x;
  const float e = (a.x - (s - bb)) + (b.x - bb);
  return df_norm(s, e + (a.y + b.y));
}

// a b, renormalised
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  float s = 0.f, t = 0.f;
  df_mac(s, t, a, b);
  return df_norm(s, t);
}

__device__ __forceinline__ double df_val(float2 a) { return double(a.x) + double(a.y); }

// (s, t) summed over the warp (every lane gets the sum)
__device__ __forceinline__ void df_warp_sum(float& s, float& t) {
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
    const float t2 = __shfl_xor_sync(0xffffffffu, t, o);
    const float u = s + s2;
    const float bb = u - s;
    t += t2 + ((s - (u - bb)) + (s2 - bb));
    s = u;
  }
}

}  // namespace bsg
