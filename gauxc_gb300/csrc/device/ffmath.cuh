// Integer / FP32 helpers that keep the mixed path off GB300's throttled FP64
// pipe: power-of-two scales from IEEE bit patterns, fixed-point digits by
// integer arithmetic, and float-float (hi + lo) values.
#pragma once
#include <cstdint>

namespace gb300 {
namespace ff {

// |v| as an ordered integer key (IEEE magnitude bits are monotonic).
__device__ __forceinline__ unsigned long long abs_key(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFULL;
}

// Exponent es with max|v| < 2^es, from the largest abs_key; 0 keys give -1022.
__device__ __forceinline__ int scale_exponent(unsigned long long key) {
  const int E = (int)(key >> 52);
  return E == 0 ? -1022 : E - 1022;
}

__device__ __forceinline__ double pow2(int e) {
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// q = round(v * 2^(42 - es)) for |v| < 2^es, by shifting the mantissa.
__device__ __forceinline__ long long fixed42(double v, int es) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int E = (int)((b >> 52) & 0x7FF);
  if (E == 0) return 0;
  const long long mant = (long long)((b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52));
  const int sh = 1075 - E - 42 + es;  // right shift (>= 11 when |v| < 2^es)
  long long q = sh > 62 ? 0 : (mant + (1LL << (sh - 1))) >> sh;
  return (b >> 63) ? -q : q;
}

// Balanced base-128 digits of q (|q| <= 2^42): q = sum_i d_i 128^(S-1-i),
// d_0 in [-128, 128], others in [-64, 63].  Writes d_i * 2^(-7 i) (exact in bf16).
template <int S, typename Store>
__device__ __forceinline__ void digits(long long q, Store&& store) {
  float d[S];
#pragma unroll
  for (int i = S - 1; i > 0; --i) {
    const long long di = ((q + 64) & 127) - 64;
    d[i] = (float)di;
    q = (q - di) >> 7;
  }
  d[0] = (float)q;
  float sc = 1.f;
#pragma unroll
  for (int i = 0; i < S; ++i) {
    store(i, d[i] * sc);
    sc *= (1.f / 128.f);
  }
}

// v = hi + lo with hi the leading 24 bits of v (truncated) and lo the rest
// rounded to 24 bits; values below 2^-126 flush to zero.
__device__ __forceinline__ float2 split(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e < -126) return make_float2(0.f, 0.f);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((m >> 29) & 0x7FFFFF));
  const unsigned rem = (unsigned)(m & ((1u << 29) - 1));
  float lo = 0.f;
  if (rem && e - 52 >= -126) lo = __uint2float_rn(rem) * __uint_as_float((unsigned)(e - 52 + 127) << 23);
  return make_float2(hi, sign ? -lo : lo);
}

// s + e = a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (hi, lo) * (xh, xl) to about 2^-47 relative
__device__ __forceinline__ float2 mul(float2 a, float2 x) {
  const float p = a.x * x.x;
  float e = fmaf(a.x, x.x, -p);
  e = fmaf(a.x, x.y, e);
  e = fmaf(a.y, x.x, e);
  return make_float2(p, e);
}

}  // namespace ff
}  // namespace gb300
