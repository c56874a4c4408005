// Complex arithmetic policies for the hafnian DP (FP64, split, FP32).
#pragma once
#include <cuda_runtime.h>

namespace bsg {

// ---- plain FP64 ---------------------------------------------------------------
struct PrecF64 {
  using C = double2;   // stored value
  using CA = C;        // class-pair table entry
  using CF = C;        // DP state table entry
  using Acc = double2; // accumulator
  static __device__ __forceinline__ Acc zero() { return make_double2(0.0, 0.0); }
  static __device__ __forceinline__ C one() { return make_double2(1.0, 0.0); }
  static __device__ __forceinline__ void mac(Acc& acc, const C& a, const C& f) {
    acc.x = fma(a.x, f.x, fma(-a.y, f.y, acc.x));
    acc.y = fma(a.x, f.y, fma(a.y, f.x, acc.y));
  }
  // acc = a f (the first term of a sum)
  static __device__ __forceinline__ void mac_init(Acc& acc, const C& a, const C& f) {
    acc = zero();
    mac(acc, a, f);
  }
  // scaled by 1/r (r small positive integer)
  static __device__ __forceinline__ C finish(const Acc& acc, int r, const double* inv_d, const float2*) {
    if (r == 1) return acc;
    double s = inv_d[r];
    return make_double2(acc.x * s, acc.y * s);
  }
  static __device__ __forceinline__ double2 to_c128(const C& v) { return v; }
  static __host__ __device__ __forceinline__ C from_c128(double2 v) { return v; }
};

// ---- plain FP32 (the reference's complex64 working precision) ------------------
struct PrecF32 {
  using C = float2;
  using CA = C;
  using CF = C;
  using Acc = float2;
  static __device__ __forceinline__ Acc zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ C one() { return make_float2(1.f, 0.f); }
  static __device__ __forceinline__ void mac(Acc& acc, const C& a, const C& f) {
    acc.x = fmaf(a.x, f.x, fmaf(-a.y, f.y, acc.x));
    acc.y = fmaf(a.x, f.y, fmaf(a.y, f.x, acc.y));
  }
  static __device__ __forceinline__ void mac_init(Acc& acc, const C& a, const C& f) {
    acc = zero();
    mac(acc, a, f);
  }
  static __device__ __forceinline__ C finish(const Acc& acc, int r, const double*, const float2* inv_f) {
    if (r == 1) return acc;
    float s = inv_f[r].x;
    return make_float2(acc.x * s, acc.y * s);
  }
  static __device__ __forceinline__ double2 to_c128(const C& v) { return make_double2(v.x, v.y); }
  static __host__ __device__ __forceinline__ C from_c128(double2 v) { return make_float2(float(v.x), float(v.y)); }
};

// ---- split: each real part is an unevaluated pair hi + lo of FP32 words ---------
// Products use the exact FMA residual of hi*hi plus the two cross terms;
// sums are Knuth two-sums with a compensation word.  Everything runs on the
// FP32 pipe (64x the FP64 rate on GB300) with a ~2^-44 relative error.
struct SplitAcc {
  float rs, rt, is, it;  // real (sum, compensation), imaginary (sum, compensation)
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// s + t += (xh + xl) * (yh + yl)
__device__ __forceinline__ void split_mac1(float& s, float& t, float xh, float xl, float yh, float yl) {
  float p = xh * yh;
  float e = fmaf(xh, yh, -p);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  float s2, err;
  two_sum(s, p, s2, err);
  s = s2;
  t += err + e;
}

// s + t = (xh + xl) * (yh + yl): the first term of a sum, where the two-sum
// with a zero accumulator would be the identity
__device__ __forceinline__ void split_mul1(float& s, float& t, float xh, float xl, float yh, float yl) {
  const float p = xh * yh;
  float e = fmaf(xh, yh, -p);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  s = p;
  t = e;
}

struct PrecSplit {
  using C = float4;  // (re_hi, re_lo, im_hi, im_lo)
  using CA = C;
  using CF = C;
  using Acc = SplitAcc;
  static __device__ __forceinline__ Acc zero() { return SplitAcc{0.f, 0.f, 0.f, 0.f}; }
  static __device__ __forceinline__ C one() { return make_float4(1.f, 0.f, 0.f, 0.f); }
  static __device__ __forceinline__ void mac(Acc& acc, const C& a, const C& f) {
    split_mac1(acc.rs, acc.rt, a.x, a.y, f.x, f.y);
    split_mac1(acc.rs, acc.rt, -a.z, -a.w, f.z, f.w);
    split_mac1(acc.is, acc.it, a.x, a.y, f.z, f.w);
    split_mac1(acc.is, acc.it, a.z, a.w, f.x, f.y);
  }
  // acc = a f: the first product of each part starts the pair directly
  static __device__ __forceinline__ void mac_init(Acc& acc, const C& a, const C& f) {
    split_mul1(acc.rs, acc.rt, a.x, a.y, f.x, f.y);
    split_mac1(acc.rs, acc.rt, -a.z, -a.w, f.z, f.w);
    split_mul1(acc.is, acc.it, a.x, a.y, f.z, f.w);
    split_mac1(acc.is, acc.it, a.z, a.w, f.x, f.y);
  }
  static __device__ __forceinline__ void renorm(float s, float t, float& h, float& l) {
    h = s + t;
    l = t - (h - s);
  }
  static __device__ __forceinline__ void mul(float xh, float xl, float yh, float yl, float& h, float& l) {
    float p = xh * yh;
    float e = fmaf(xh, yh, -p);
    e = fmaf(xh, yl, e);
    e = fmaf(xl, yh, e);
    renorm(p, e, h, l);
  }
  static __device__ __forceinline__ C finish(const Acc& acc, int r, const double*, const float2* inv_f) {
    float rh, rl, ih, il;
    renorm(acc.rs, acc.rt, rh, rl);
    renorm(acc.is, acc.it, ih, il);
    if (r == 1) return make_float4(rh, rl, ih, il);  // r: warp-uniform
    const float2 iv = inv_f[r];
    C out;
    mul(rh, rl, iv.x, iv.y, out.x, out.y);
    mul(ih, il, iv.x, iv.y, out.z, out.w);
    return out;
  }
  static __device__ __forceinline__ double2 to_c128(const C& v) {
    return make_double2(double(v.x) + double(v.y), double(v.z) + double(v.w));
  }
  static __host__ __device__ __forceinline__ C from_c128(double2 v) {
    float rh = float(v.x);
    float rl = float(v.x - double(rh));
    float ih = float(v.y);
    float il = float(v.y - double(ih));
    return make_float4(rh, rl, ih, il);
  }
};

}  // namespace bsg
