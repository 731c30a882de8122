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

// Balanced base-128 digits of q (|q| < 2^(7 S)): q = sum_i d_i 128^(S-1-i),
// d_0 in [-128, 128], the others in [-64, 63]; store(i, x) receives the exact
// float x = d_i 2^(-7 i), whose top 16 bits are its BF16 pattern (at most 8
// significant bits).  Adding 64 128^k (k = 0..S-2) turns digits 1..S-1 into
// the plain 7-bit fields f_i = d_i + 64 of u = q + bias (field i at bit
// 7 (S-1-i)), and digit 0 into the arithmetic rest u >> 7 (S-1): no carry
// chain.  OR-ing a field into the bits of 1.5 2^23 gives the float
// 1.5 2^23 + f exactly, and one FMA by 2^(-7 i) takes the offset
// (1.5 2^23 + 64) 2^(-7 i) off exactly.
template <int S, typename Store>
__device__ __forceinline__ void digits_f32(long long q, Store&& store) {
  static_assert(S >= 2 && S <= 6, "fields below bit 35");
  constexpr long long kBias = 64LL * ((1LL << (7 * (S - 1))) - 1) / 127;
  const long long u = q + kBias;
  const unsigned lo = (unsigned)u, hi = (unsigned)((unsigned long long)u >> 32);
  const int d0 = (int)(u >> (7 * (S - 1)));
  store(0, __int_as_float(0x4B400000 + d0) - 12582912.f);
#pragma unroll
  for (int i = 1; i < S; ++i) {
    const int sh = 7 * (S - 1 - i);
    const unsigned f = (sh + 7 <= 32 ? lo >> sh : __funnelshift_r(lo, hi, sh)) & 127u;
    const float sc = __int_as_float((127 - 7 * i) << 23);
    store(i, fmaf(__int_as_float(0x4B400000 | (int)f), sc, -12582976.f * sc));
  }
}

// Two BF16 patterns in one word: the top halves of floats a (low) and b (high).
__device__ __forceinline__ unsigned pack_bf16x2(float a, float b) {
  return __byte_perm(__float_as_uint(a), __float_as_uint(b), 0x7632);
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

// 2^e as a float for e in the normal range, 0 below it (and above it, which
// the callers never reach).
__device__ __forceinline__ float pow2f(int e) {
  return (e >= -126 && e <= 127) ? __uint_as_float((unsigned)(e + 127) << 23) : 0.f;
}

// (hi + lo) * 2^e2 as a double, built with integer arithmetic (no FP64
// instructions).  Both parts are aligned to the larger exponent with 30 guard
// bits (error below 2^-54 of the larger part), summed exactly in 64 bits and
// rounded once to 53 bits.  Results below the double normal range return 0;
// float subnormal inputs count as 0.
__device__ __forceinline__ double to_double(float hi, float lo, int e2) {
  const unsigned hb = __float_as_uint(hi), lb = __float_as_uint(lo);
  const int eh = (int)((hb >> 23) & 0xFF), el = (int)((lb >> 23) & 0xFF);
  const int E = eh > el ? eh : el;
  if (E == 0) return 0.0;
  long long H = 0, L = 0;
  if (eh != 0 && E - eh < 55) H = ((long long)((hb & 0x7FFFFFu) | 0x800000u) << 30) >> (E - eh);
  if (el != 0 && E - el < 55) L = ((long long)((lb & 0x7FFFFFu) | 0x800000u) << 30) >> (E - el);
  if (hb >> 31) H = -H;
  if (lb >> 31) L = -L;
  const long long T = H + L;  // value = T * 2^(E - 180 + e2), |T| < 2^55
  if (T == 0) return 0.0;
  const unsigned long long sign = T < 0 ? (1ULL << 63) : 0ULL;
  unsigned long long M = T < 0 ? (unsigned long long)(-T) : (unsigned long long)T;
  const int msb = 63 - __clzll((long long)M);
  int ex = E - 180 + e2;
  if (msb > 52) {
    const int sh = msb - 52;
    M = (M + (1ULL << (sh - 1))) >> sh;
    ex += sh;
    if (M >> 53) {
      M >>= 1;
      ex += 1;
    }
  } else {
    M <<= (52 - msb);
    ex -= 52 - msb;
  }
  const int be = ex + 52 + 1023;
  if (be <= 0) return 0.0;
  if (be >= 2047) return __longlong_as_double((long long)(sign | (0x7FFULL << 52)));
  return __longlong_as_double((long long)(sign | ((unsigned long long)be << 52) | (M & 0xFFFFFFFFFFFFFULL)));
}

// Exact conversion as a separate function, the cold path of f2d_scaled.
static __device__ __noinline__ double to_double_cold(float hi, float lo, int e2) {
  return to_double(hi, lo, e2);
}

// f * 2^e2 as a double, exactly: the float's fields are written into a
// double bit pattern with integer operations only (no FP64 instruction).
// Zero gives 0; subnormal or non-finite floats and results outside the
// normal range take the exact routine.
__device__ __forceinline__ double f2d_scaled(float f, int e2) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu;
  const unsigned eo = e + 896u + (unsigned)e2;  // biased exponent of the result
  if (e - 1u < 254u && eo - 1u < 2046u)
    return __hiloint2double((int)((b & 0x80000000u) | (eo << 20) | ((b >> 3) & 0xFFFFFu)),
                            (int)(b << 29));
  if ((b & 0x7FFFFFFFu) == 0u) return 0.0;
  return to_double_cold(f, 0.f, e2);
}

// a + b for float-float values (hi, lo)
__device__ __forceinline__ float2 add(float2 a, float2 b) {
  float s, e;
  two_sum(a.x, b.x, s, e);
  return make_float2(s, a.y + b.y + e);
}

// ---------------------------------------------------------------- float-float type
// Unevaluated sum hi + lo of two floats (about 46 significant bits), with the
// arithmetic the generated collocation templates use.  Device code builds
// values from doubles by bit manipulation (no FP64 instructions).
struct ffl {
  float hi, lo;
  ffl() = default;
  __host__ __device__ constexpr ffl(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ ffl(double v) {
#ifdef __CUDA_ARCH__
    const float2 t = split(v);
    hi = t.x;
    lo = t.y;
#else
    hi = (float)v;
    lo = (float)(v - (double)hi);
#endif
  }
  __host__ __device__ ffl(int v) : ffl((double)v) {}
};

// s + e = a + b for |a| >= |b| (or a == 0)
__host__ __device__ __forceinline__ ffl fast_two_sum(float a, float b) {
  const float s = a + b;
  return ffl(s, b - (s - a));
}
__host__ __device__ __forceinline__ ffl operator+(ffl a, ffl b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb);
  return fast_two_sum(s, e + a.lo + b.lo);
}
__host__ __device__ __forceinline__ ffl operator-(ffl a) { return ffl(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ ffl operator-(ffl a, ffl b) { return a + (-b); }
__host__ __device__ __forceinline__ ffl operator*(ffl a, ffl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__host__ __device__ __forceinline__ ffl& operator+=(ffl& a, ffl b) { return a = a + b; }
__host__ __device__ __forceinline__ ffl& operator*=(ffl& a, ffl b) { return a = a * b; }

// exp(x) for a float-float x <= 0, about 2^-46 relative; 0 below e^-87.
// Method (table-driven, after Tang's exp): m = rint(32 x / ln 2) = 32 k + j,
// r = x - m ln2/32 with ln2/32 split into three floats (the first has 12
// significant bits, so m times it is exact for |m| < 4096), |r| <= ln2/64;
// exp(r) = 1 + r + r^2 h(r), h = 1/2 + r/6 + r^2/24 + r^3/120 + r^4/720
// (truncation r^7/5040 below 2^-55, so no bias from the series; the last
// three terms of h in FP32, their error scaled down by r^2); exp(x) = 2^k
// 2^(j/32) exp(r), with 2^(j/32) from `tab` (32 float-float values,
// exp2_table()).  CPU emulation over x in [-40, 0]: largest relative error
// 1.1e-14, mean -9e-17.
__device__ __forceinline__ ffl exp_neg(ffl x, const float2* __restrict__ tab) {
  if (x.hi < -87.f) return ffl(0.f, 0.f);
  const float m = rintf(x.hi * 46.166241308446828f);  // 32 / ln 2
  const int mi = (int)m;
  const int j = mi & 31, k = mi >> 5;                  // mi = 32 k + j
  const float L1 = 0x1.62ep-6f, L2 = 0x1.0bfbe8p-20f, L3 = 0x1.cf79acp-45f;  // ln2/32
  ffl r = x + ffl(-m * L1, 0.f);                       // m L1 exact
  const float p2 = m * L2;
  r = r + ffl(-p2, -fmaf(m, L2, -p2));                 // m L2 as an exact product pair
  r = r + ffl(-m * L3, 0.f);
  const float t =
      r.hi * r.hi * fmaf(r.hi, fmaf(r.hi, 0.0013888888888888889f, 0.008333333333333333f), 0.041666666666666667f);
  const ffl h = (ffl(0.5f, 0.f) + r * ffl(0.16666667163372040f, -4.9670538793122887e-09f)) +
                ffl(t, 0.f);
  const ffl e = ffl(1.f, 0.f) + (r + (r * r) * h);
  const float2 tj = tab[j];
  const ffl y = e * ffl(tj.x, tj.y);
  const float s = k >= -126 ? __uint_as_float((unsigned)(k + 127) << 23) : 0.f;
  return ffl(y.hi * s, y.lo * s);
}

// q = round(v * 2^(42 - es)) for a float v with |v| < 2^es, by shifting the mantissa.
__device__ __forceinline__ long long fixed42f(float v, int es) {
  const unsigned b = __float_as_uint(v);
  const int E = (int)((b >> 23) & 0xFF);
  if (E == 0) return 0;
  const long long mant = (long long)((b & 0x7FFFFFu) | 0x800000u);
  const int sh = E - 150 + 42 - es;  // v * 2^(42 - es) = mant * 2^sh
  long long q;
  if (sh >= 0)
    q = sh > 38 ? 0 : mant << sh;  // |v| < 2^es keeps q below 2^42
  else
    q = -sh > 62 ? 0 : (mant + (1LL << (-sh - 1))) >> (-sh);
  return (b >> 31) ? -q : q;
}

// q = round(v * 2^(42 - es)) for a float-float v (|v| < 2^es)
__device__ __forceinline__ long long fixed42(ffl v, int es) {
  return fixed42f(v.hi, es) + fixed42f(v.lo, es);
}

// Power-of-two exponent e with |x| < 2^e for the largest |hi| of float-float
// values, given as the float magnitude bits of that hi (0 gives -126).
__device__ __forceinline__ int scale_exponent_f(unsigned key) {
  const int E = (int)(key >> 23);
  return E == 0 ? -126 : E - 126;
}

}  // namespace ff
}  // namespace gb300
