// Double-float arithmetic: a value is the unevaluated sum h + l of two floats
// (about 48 significant bits), built from the error-free transforms
// two-sum (Knuth) and two-product via FMA (Dekker / Ogita-Rump-Oishi).
//
// The mixed-precision path forms reprojection residuals with it: the point in
// the camera frame carries ~1e-7 relative error in plain FP32, which is 3e-5 px
// at 500 px focal length and makes the LM cost noisy at the 1e-6 relative
// level the stopping rule needs.  FP64 would fix that but runs far slower than
// FP32 on this part; double-float runs on the FP32 pipes.
//
// Requires IEEE float semantics (no fast-math reassociation); FMA contraction is
// harmless here because the products that must be exact use fmaf explicitly.
#pragma once
#include <cuda_runtime.h>

namespace spgo {

struct df {
  float h, l;
};

__device__ __forceinline__ df df_make(float h) { return df{h, 0.f}; }

__device__ __forceinline__ df df_from_double(double x) {
  const float h = (float)x;
  return df{h, (float)(x - (double)h)};
}

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return df{s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return df{s, b - (s - a)};
}

__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = a * b;
  return df{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ df operator+(const df &a, const df &b) {
  df s = two_sum(a.h, b.h);
  s.l += a.l + b.l;
  return fast_two_sum(s.h, s.l);
}

__device__ __forceinline__ df operator-(const df &a) { return df{-a.h, -a.l}; }
__device__ __forceinline__ df operator-(const df &a, const df &b) { return a + (-b); }

__device__ __forceinline__ df operator*(const df &a, const df &b) {
  df p = two_prod(a.h, b.h);
  p.l += a.h * b.l + a.l * b.h;
  return fast_two_sum(p.h, p.l);
}

__device__ __forceinline__ df operator*(const df &a, float b) {
  df p = two_prod(a.h, b);
  p.l += a.l * b;
  return fast_two_sum(p.h, p.l);
}

__device__ __forceinline__ df operator/(const df &a, const df &b) {
  const float q1 = a.h / b.h;
  const df r = a - b * q1;
  const float q2 = r.h / b.h;
  return fast_two_sum(q1, q2);
}

// sum_j (a_j + al_j)(b_j) for three double-float b_j and double-float
// coefficients (ah, al): the three leading products exactly (two-product), their
// sum with two error-free additions, all cross and low terms in one float.
// ~31 FP32 operations instead of ~46 for three products and two additions.
__device__ __forceinline__ df df_dot3(float a0h, float a0l, float a1h, float a1l, float a2h, float a2l,
                                      const df &b0, const df &b1, const df &b2) {
  const df p0 = two_prod(a0h, b0.h), p1 = two_prod(a1h, b1.h), p2 = two_prod(a2h, b2.h);
  const df s01 = two_sum(p0.h, p1.h);
  const df s = two_sum(s01.h, p2.h);
  float lo = ((p0.l + p1.l) + (p2.l + s01.l)) + s.l;
  lo = fmaf(a0h, b0.l, lo);
  lo = fmaf(a1h, b1.l, lo);
  lo = fmaf(a2h, b2.l, lo);
  lo = fmaf(a0l, b0.h, lo);
  lo = fmaf(a1l, b1.h, lo);
  lo = fmaf(a2l, b2.h, lo);
  return fast_two_sum(s.h, lo);
}

// a0 b0 + a1 b1 + a2 b2 + a3 b3 as a double-float: the four products exactly
// (two-product), their high parts by a cascade of error-free sums, every low part
// and error term in one float (~2^-44 relative to the terms' magnitudes)
__device__ __forceinline__ df sum4_prod(float a0, float b0, float a1, float b1, float a2, float b2, float a3,
                                        float b3) {
  const df p0 = two_prod(a0, b0), p1 = two_prod(a1, b1), p2 = two_prod(a2, b2), p3 = two_prod(a3, b3);
  const df s = two_sum(p0.h, p1.h), t = two_sum(p2.h, p3.h);
  const df u = two_sum(s.h, t.h);
  const float lo = ((p0.l + p1.l) + (p2.l + p3.l)) + ((s.l + t.l) + u.l);
  return fast_two_sum(u.h, lo);
}

// Running sum kept unnormalised (h plus an accumulated error term): the next add
// depends on the previous one through a single float addition.  Read with
// df_acc_value.
struct df_acc {
  float h = 0.f, l = 0.f;
  __device__ __forceinline__ void add(float xh, float xl) {
    const float sh = h + xh;
    const float bb = sh - h;
    l += ((h - (sh - bb)) + (xh - bb)) + xl;
    h = sh;
  }
};
__device__ __forceinline__ double df_acc_value(const df_acc &a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ df &operator+=(df &a, const df &b) {
  a = a + b;
  return a;
}

// A double split into a double-float with integer operations only (FP64 runs at a
// small fraction of the FP32 rate on this GPU, conversions included): h = x with its
// mantissa truncated to 24 bits, l = the remaining 29 bits rounded to 24.  Below 2^-126
// it becomes 0; beyond the float range, infinity (NaN stays NaN).
__device__ __forceinline__ df df_split_double(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(u >> 32), lo32 = (unsigned)u;
  const int e = (int)((hi32 >> 20) & 0x7ffu) - 1023;  // unbiased exponent
  const unsigned sign = hi32 & 0x80000000u;
  if (e < -126) return df{0.f, 0.f};
  if (e > 127) {  // beyond the float range: infinity, or NaN for a NaN
    const bool nan = e == 1024 && ((hi32 & 0xfffffu) | lo32) != 0u;
    return df{__uint_as_float(sign | (nan ? 0x7fc00000u : 0x7f800000u)), 0.f};
  }
  const float h = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | ((hi32 & 0xfffffu) << 3) | (lo32 >> 29));
  // the low 29 mantissa bits carry weight 2^(e - 52)
  const int el = e - 52;
  const float scale = el >= -126 ? __uint_as_float((unsigned)(el + 127) << 23) : 0.f;
  const float l = __uint_as_float(__float_as_uint(__uint2float_rn(lo32 & 0x1fffffffu) * scale) | sign);
  return df{h, l};
}

// a - b for plain floats, exactly, as a double-float
__device__ __forceinline__ df df_sub(float a, float b) { return two_sum(a, -b); }

__device__ __forceinline__ float df_to_float(const df &a) { return a.h + a.l; }
__device__ __forceinline__ double df_to_double(const df &a) { return (double)a.h + (double)a.l; }

}  // namespace spgo
