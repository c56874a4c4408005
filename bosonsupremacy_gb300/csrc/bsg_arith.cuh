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
// FP32 pipe (64x the FP64 rate on GB300) with a ~2^-44 relative error; the
// real and imaginary halves run as packed FP32 pairs.

// ---- packed FP32 pairs (sm_100+ f32x2: one instruction for both halves) ----------
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
  float2 d;
  asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 f2_neg(float2 a) { return make_float2(-a.x, -a.y); }

// s + t += (xh + xl) (yh + yl) for both halves of a pair: the exact FMA
// residual of xh yh plus the two cross terms, a Knuth two-sum into s and the
// compensation into t
__device__ __forceinline__ void split_mac2(float2& s, float2& t, float2 xh, float2 xl, float2 yh, float2 yl) {
  const float2 p = f2_mul(xh, yh);
  float2 e = f2_fma(xh, yh, f2_neg(p));
  e = f2_fma(xh, yl, e);
  e = f2_fma(xl, yh, e);
  const float2 s2 = f2_add(s, p);
  const float2 bb = f2_sub(s2, s);
  const float2 err = f2_add(f2_sub(s, f2_sub(s2, bb)), f2_sub(p, bb));
  s = s2;
  t = f2_add(t, f2_add(err, e));
}
// s + t = (xh + xl) (yh + yl): the first term of a sum, where the two-sum
// with a zero accumulator would be the identity
__device__ __forceinline__ void split_mul2(float2& s, float2& t, float2 xh, float2 xl, float2 yh, float2 yl) {
  const float2 p = f2_mul(xh, yh);
  float2 e = f2_fma(xh, yh, f2_neg(p));
  e = f2_fma(xh, yl, e);
  e = f2_fma(xl, yh, e);
  s = p;
  t = e;
}

// Split precision with packed pairs.  A DP value is (re_hi, im_hi, re_lo,
// im_lo), so its hi and lo halves are natural pairs; a Sigma entry keeps the
// 16-byte (re_hi, re_lo, im_hi, im_lo) and is broadcast into pairs at use
// (storing the broadcast pairs doubles Sigma's cache footprint: slower).  A
// complex product a f = (ar fr - ai fi) + i (ar fi + ai fr) is two packed
// products:
//   (ar, ar) o (fr, fi) = (ar fr, ar fi)      -> accumulator (re, im)
//   (ai, ai) o (fr, fi) = (ai fr, ai fi)      -> accumulator (im, -re)
// and the two accumulators are combined once per DP state.
struct SplitAcc2 {
  float2 s, t;    // (re, im): sum, compensation
  float2 s2, t2;  // (im, -re): sum, compensation
};

struct PrecSplit {
  using C = float4;   // Sigma entries: (re_hi, re_lo, im_hi, im_lo)
  using CA = C;
  using CF = float4;  // DP values: (re_hi, im_hi, re_lo, im_lo)
  using Acc = SplitAcc2;
  static __device__ __forceinline__ Acc zero() {
    const float2 z = make_float2(0.f, 0.f);
    return SplitAcc2{z, z, z, z};
  }
  static __device__ __forceinline__ CF one() { return make_float4(1.f, 0.f, 0.f, 0.f); }
  // broadcast pairs (x, x) of the hi and lo words of a Sigma entry
  static __device__ __forceinline__ void pairs(const C& a, float2& rh, float2& rl, float2& ih, float2& il) {
    rh = make_float2(a.x, a.x);
    rl = make_float2(a.y, a.y);
    ih = make_float2(a.z, a.z);
    il = make_float2(a.w, a.w);
  }
  static __device__ __forceinline__ void mac(Acc& acc, const C& a, const CF& f) {
    float2 rh, rl, ih, il;
    pairs(a, rh, rl, ih, il);
    const float2 yh = make_float2(f.x, f.y), yl = make_float2(f.z, f.w);
    split_mac2(acc.s, acc.t, rh, rl, yh, yl);
    split_mac2(acc.s2, acc.t2, ih, il, yh, yl);
  }
  // acc = a f: the first product of each part starts the pair directly
  static __device__ __forceinline__ void mac_init(Acc& acc, const C& a, const CF& f) {
    float2 rh, rl, ih, il;
    pairs(a, rh, rl, ih, il);
    const float2 yh = make_float2(f.x, f.y), yl = make_float2(f.z, f.w);
    split_mul2(acc.s, acc.t, rh, rl, yh, yl);
    split_mul2(acc.s2, acc.t2, ih, il, yh, yl);
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
  // (re, im) = (s, t) + (-s2.y, s2.x): a double-float sum per half, then
  // renormalised and scaled by 1/r (r a small positive integer)
  static __device__ __forceinline__ CF finish(const Acc& acc, int r, const double*, const float2* inv_f) {
    const float2 b = make_float2(-acc.s2.y, acc.s2.x), bt = make_float2(-acc.t2.y, acc.t2.x);
    const float2 u = f2_add(acc.s, b);
    const float2 bb = f2_sub(u, acc.s);
    const float2 err = f2_add(f2_sub(acc.s, f2_sub(u, bb)), f2_sub(b, bb));
    const float2 v = f2_add(f2_add(acc.t, bt), err);
    float2 h = f2_add(u, v);
    float2 l = f2_sub(v, f2_sub(h, u));
    if (r != 1) {  // r: warp-uniform
      const float2 iv = inv_f[r];
      const float2 ih = make_float2(iv.x, iv.x), il = make_float2(iv.y, iv.y);
      const float2 p = f2_mul(h, ih);
      float2 e = f2_fma(h, ih, f2_neg(p));
      e = f2_fma(h, il, e);
      e = f2_fma(l, ih, e);
      h = f2_add(p, e);
      l = f2_sub(e, f2_sub(h, p));
    }
    return make_float4(h.x, h.y, l.x, l.y);
  }
  static __device__ __forceinline__ double2 to_c128(const CF& v) {
    return make_double2(double(v.x) + double(v.z), double(v.y) + double(v.w));
  }
  static __host__ __device__ __forceinline__ C from_c128(double2 v) {
    const float rh = float(v.x), rl = float(v.x - double(rh));
    const float ih = float(v.y), il = float(v.y - double(ih));
    return make_float4(rh, rl, ih, il);
  }
};

}  // namespace bsg
