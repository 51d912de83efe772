// Double-float ("df64") arithmetic: a value is an unevaluated sum hi + lo of two
// FP32 numbers, ~48 significant bits.  GB300 issues FP32 at 64x its FP64 rate,
// so the fused kernels can carry FP64 fields as FP32 pairs and do their
// arithmetic on the pairs.
//
// Algorithms (published, restated here): Knuth's TwoSum for error-free
// addition, Dekker's FastTwoSum for renormalisation, and the FMA-based exact
// product (Ogita, Rump, Oishi, "Accurate sum and dot product", 2005, Alg. 3.1
// and the TwoProduct-by-FMA variant).  The operators below defer
// renormalisation: a sum is TwoSum of the high parts with the low parts and the
// error term added in FP32 (8 operations), a product keeps the FMA error terms
// in the low part (4 operations), and df_norm() renormalises once per stencil
// update (3 operations).  Each operation's absolute error stays ~2^-47 of its
// operands while the low parts are a few ulps of the high parts.
#pragma once
#include <cstdint>

namespace girih {

struct __align__(8) Df64 {
  float hi, lo;
  Df64() = default;
  __host__ __device__ constexpr Df64(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr Df64(int v) : hi((float)v), lo(0.f) {}
  __host__ __device__ constexpr Df64(float v) : hi(v), lo(0.f) {}
};

__device__ __forceinline__ void df_fast_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ void df_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ Df64 operator+(Df64 a, Df64 b) {
  float s, e;
  df_two_sum(a.hi, b.hi, s, e);
  return Df64(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ Df64 operator-(Df64 a) { return Df64(-a.hi, -a.lo); }
__device__ __forceinline__ Df64 operator-(Df64 a, Df64 b) { return a + (-b); }

// 2a - b: the sum above of (2 a.hi, 2 a.lo) and -b with each product by 2 (exact)
// folded into an FMA, which then rounds as the separate subtraction does, so
// the result is the same bit for bit (wherever 2 a.hi does not overflow) in 8
// operations instead of 10.
__device__ __forceinline__ Df64 twice_minus(Df64 a, Df64 b) {
  const float s = __fmaf_rn(2.f, a.hi, -b.hi);
  const float bb = __fmaf_rn(-2.f, a.hi, s);  // s - 2 a.hi
  const float e = __fadd_rn(__fmaf_rn(2.f, a.hi, -__fsub_rn(s, bb)), __fsub_rn(-b.hi, bb));
  return Df64(s, __fadd_rn(e, __fmaf_rn(2.f, a.lo, -b.lo)));
}

__device__ __forceinline__ Df64 operator*(Df64 a, Df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // exact error of the product
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return Df64(p, e);
}

// Renormalise: |lo| <= ulp(hi)/2.
__device__ __forceinline__ Df64 df_norm(Df64 a) {
  Df64 r;
  df_fast_two_sum(a.hi, a.lo, r.hi, r.lo);
  return r;
}

// Host-side split of a double constant into (hi, lo) with round-to-nearest hi.
inline Df64 df_from_double_host(double d) {
  const float h = (float)d;
  return Df64(h, (float)(d - (double)h));
}

// Device split of an FP64 value using integer operations only (the FP64 pipe
// is the scarce unit): hi = the top 24 significand bits (truncated), lo = the
// next 29 bits rounded to 24.  Values outside the FP32 exponent range set
// *range_bad and return 0; zeros and FP64 subnormals become 0.
__device__ __forceinline__ Df64 df_split(double d, unsigned &range_bad) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int E = (int)((b >> 52) & 0x7FF);
  const int e = E - 1023;
  if (E == 0 || e < -126) return Df64(0.f, 0.f);
  if (e > 127) {
    range_bad = 1u;
    return Df64(0.f, 0.f);
  }
  const unsigned long long M = b & 0xFFFFFFFFFFFFFull;
  const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)(M >> 29));
  const unsigned rem = (unsigned)(M & 0x1FFFFFFFull);  // value rem * 2^(e-52)
  // scale by 2^(e-52) through the exponent field; below 2^-74 the low part is
  // under the FP32 normal range and is dropped (relative size < 2^-48 of hi)
  float lo = e >= -74 ? __uint2float_rn(rem) * __uint_as_float((unsigned)(e - 52 + 127) << 23) : 0.f;
  if (sign) lo = -lo;
  return Df64(hi, lo);
}

__device__ __forceinline__ double df_to_double(Df64 x) { return (double)x.hi + (double)x.lo; }

// Two double-float values (two neighbouring x columns) with their high and
// low parts packed as FP32 pairs: the operators above, each instruction a
// packed f32x2 one (sm_100-class GPUs execute f32x2 add / multiply / FMA as one
// FMA-pipe instruction for two values, each rounded as its scalar counterpart),
// so every lane computes exactly what the scalar Df64 code computes.  a - b is
// fma(-1, b, a): the same single rounding as a scalar subtraction.
struct Df2 {
  float2 hi, lo;
};

__device__ __forceinline__ float2 f2m1() { return make_float2(-1.f, -1.f); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(f2m1(), b, a); }

__device__ __forceinline__ Df2 df2(Df64 a, Df64 b) { return Df2{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)}; }
__device__ __forceinline__ Df64 df2_x(const Df2 &a) { return Df64(a.hi.x, a.lo.x); }
__device__ __forceinline__ Df64 df2_y(const Df2 &a) { return Df64(a.hi.y, a.lo.y); }

__device__ __forceinline__ Df2 operator+(Df2 a, Df2 b) {
  const float2 s = f2add(a.hi, b.hi);
  const float2 bb = f2sub(s, a.hi);
  const float2 e = f2add(f2sub(a.hi, f2sub(s, bb)), f2sub(b.hi, bb));
  return Df2{s, f2add(e, f2add(a.lo, b.lo))};
}

__device__ __forceinline__ Df2 operator-(Df2 a, Df2 b) {
  const float2 s = f2sub(a.hi, b.hi);  // TwoSum of a.hi and -b.hi
  const float2 bb = f2sub(s, a.hi);
  const float2 e = f2sub(f2sub(a.hi, f2sub(s, bb)), f2add(b.hi, bb));  // (a - (s - bb)) + (-b - bb)
  return Df2{s, f2add(e, f2sub(a.lo, b.lo))};
}

// exact; twice(a) - b rounds as the scalar twice_minus(a, b), bit for bit
__device__ __forceinline__ Df2 twice(Df2 a) { return Df2{f2add(a.hi, a.hi), f2add(a.lo, a.lo)}; }

__device__ __forceinline__ Df2 operator*(Df2 a, Df2 b) {
  const float2 p = __fmul2_rn(a.hi, b.hi);
  float2 e = __ffma2_rn(a.hi, b.hi, __fmul2_rn(f2m1(), p));  // exact error of the product
  e = __ffma2_rn(a.hi, b.lo, e);
  e = __ffma2_rn(a.lo, b.hi, e);
  return Df2{p, e};
}

__device__ __forceinline__ Df2 df_norm(Df2 a) {
  const float2 s = f2add(a.hi, a.lo);
  return Df2{s, f2sub(a.lo, f2sub(s, a.hi))};
}

}  // namespace girih
