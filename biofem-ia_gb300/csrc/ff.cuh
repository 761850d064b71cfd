/*
 * Float-float numbers: a value held as the unevaluated sum hi + lo of two
 * floats with |lo| <= ulp(hi) / 2, about 48 significant bits, computed on
 * the FP32 pipe.  On GB300 the FP64 pipe issues at 1/64 of the FP32 rate,
 * so a float-float operation of 3 to 20 FP32 instructions still costs a
 * fraction of one FP64 instruction.
 *
 * Built from the error-free transformations of Knuth (TwoSum), Dekker
 * (Fast2Sum, with |a| >= |b|) and the FMA form of TwoProd (a b - fl(a b) is
 * exact when computed by one fused multiply-add), composed as in the
 * double-word literature: the accurate sum adds the low parts through a
 * second TwoSum (cancellation-safe), the product folds the cross terms into
 * the error term, division and square root take one Newton correction of the
 * float quotient / root.  No operation depends on how the compiler contracts
 * expressions: every product that must stay exact is an explicit fmaf.
 */
#ifndef BIOFEM_FF_CUH
#define BIOFEM_FF_CUH

#include <cmath>
#include <cstdint>
#include <cstring>

namespace biofem {

struct FF {
  float hi, lo;
  FF() = default;
  __host__ __device__ constexpr FF(float h, float l) : hi(h), lo(l) {}
  /* from a double: hi the rounded value, lo the rounded remainder */
  __host__ __device__ FF(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ FF(int i) : hi((float)i), lo(0.f) {}
};

__host__ __device__ __forceinline__ double ff_to_double(FF a) { return (double)a.hi + (double)a.lo; }

__host__ __device__ __forceinline__ FF ff_fast_two_sum(float a, float b)
{
  const float s = a + b;
  return FF(s, b - (s - a));
}

__host__ __device__ __forceinline__ FF ff_two_sum(float a, float b)
{
  const float s = a + b;
  const float bb = s - a;
  return FF(s, (a - (s - bb)) + (b - bb));
}

__host__ __device__ __forceinline__ FF ff_two_prod(float a, float b)
{
  const float p = a * b;
  return FF(p, fmaf(a, b, -p));
}

__host__ __device__ __forceinline__ FF operator+(FF a, FF b)
{
  FF s = ff_two_sum(a.hi, b.hi);
  const FF t = ff_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = ff_fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return ff_fast_two_sum(s.hi, s.lo);
}

__host__ __device__ __forceinline__ FF operator-(FF a) { return FF(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ FF operator-(FF a, FF b) { return a + (-b); }

__host__ __device__ __forceinline__ FF operator*(FF a, FF b)
{
  FF p = ff_two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, p.lo);
  p.lo = fmaf(a.lo, b.hi, p.lo);
  return ff_fast_two_sum(p.hi, p.lo);
}

__host__ __device__ __forceinline__ FF operator/(FF a, FF b)
{
  const float q1 = a.hi / b.hi;
  const FF r = a - b * FF(q1, 0.f);
  const float q2 = r.hi / b.hi;
  return ff_fast_two_sum(q1, q2);
}

__host__ __device__ __forceinline__ FF &operator+=(FF &a, FF b) { a = a + b; return a; }

__host__ __device__ __forceinline__ bool operator>(FF a, FF b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__host__ __device__ __forceinline__ bool operator<(FF a, FF b) { return b > a; }
__host__ __device__ __forceinline__ bool operator<=(FF a, FF b) { return !(a > b); }
__host__ __device__ __forceinline__ bool operator>=(FF a, FF b) { return !(b > a); }

__host__ __device__ __forceinline__ FF dabs(FF a) { return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f) ? -a : a; }

/* sqrt(a) = s + (a - s^2) / (2 s), s the float root */
__host__ __device__ __forceinline__ FF dsqrt(FF a)
{
  if (!(a.hi > 0.f)) return FF(sqrtf(a.hi), 0.f);
  const float s = sqrtf(a.hi);
  const FF r = a - ff_two_prod(s, s);
  return ff_fast_two_sum(s, r.hi / (2.f * s));
}

__host__ __device__ __forceinline__ FF val(FF a) { return a; }

/* Bit-level conversions between double and float-float that run on the
   integer and FP32 pipes only (no double-precision instruction): on this GPU
   the FP64 pipe issues at 1/64 of the FP32 rate, and the conversion
   instructions share it.  IEEE-754 binary64 = sign | 11-bit exponent | 52-bit
   fraction; binary32 = sign | 8-bit exponent | 23-bit fraction. */
__host__ __device__ __forceinline__ uint64_t ff_bits64(double d)
{
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t b;
  memcpy(&b, &d, 8);
  return b;
#endif
}
__host__ __device__ __forceinline__ double ff_from_bits64(uint64_t b)
{
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, 8);
  return d;
#endif
}
__host__ __device__ __forceinline__ uint32_t ff_bits32(float f)
{
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t b;
  memcpy(&b, &f, 4);
  return b;
#endif
}
__host__ __device__ __forceinline__ float ff_from_bits32(uint32_t b)
{
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, 4);
  return f;
#endif
}

/* d as hi + lo: hi = d with its fraction cut to 23 bits, lo = the remaining
   29 bits (converted to float, so at most 5 of them are rounded away: hi + lo
   equals d to 2^-47 relative), then renormalised.  |d| below 2^-126 gives 0,
   infinities and NaN give themselves. */
__host__ __device__ __forceinline__ FF ff_split(double d)
{
  const uint64_t b = ff_bits64(d);
  const uint32_t sign = (uint32_t)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7ff);
  const uint64_t m = b & 0xfffffffffffffull;
  if (e == 0x7ff) return FF(ff_from_bits32(sign | 0x7f800000u | (m ? 0x400000u : 0u)), 0.f);
  const int ef = e - 1023 + 127;
  if (ef >= 255) return FF(ff_from_bits32(sign | 0x7f800000u), 0.f);
  if (ef <= 0) return FF(ff_from_bits32(sign), 0.f);
  const float hi = ff_from_bits32(sign | ((uint32_t)ef << 23) | (uint32_t)(m >> 29));
  /* the remainder is rem * 2^(e - 1023 - 52): scale by two exact powers of two
     (each within the float exponent range for every |d| >= 2^-126) */
  const float rem = (float)(uint32_t)(m & 0x1fffffffu);
  const int sh = e - 1023 - 52;                          /* -178 .. 75 */
  const int sh1 = sh < -100 ? -100 : sh, sh2 = sh - sh1;  /* sh1 >= -100, sh2 in -78 .. 0 */
  float lo = rem * ff_from_bits32((uint32_t)(sh1 + 127) << 23) * ff_from_bits32((uint32_t)(sh2 + 127) << 23);
  if (sign) lo = -lo;
  return ff_fast_two_sum(hi, lo);
}

/* (double)f exactly, from the bits: a normal float's 24-bit significand fits
   the double's; subnormal floats (below 2^-126) give 0. */
__host__ __device__ __forceinline__ double ff_widen(float f)
{
  const uint32_t b = ff_bits32(f);
  const uint64_t sign = (uint64_t)(b >> 31) << 63;
  const uint32_t ef = (b >> 23) & 0xff;
  const uint64_t m = b & 0x7fffffu;
  if (ef == 0) return ff_from_bits64(sign);
  if (ef == 255) return ff_from_bits64(sign | 0x7ff0000000000000ull | (m << 29));
  return ff_from_bits64(sign | ((uint64_t)(ef - 127 + 1023) << 52) | (m << 29));
}

/* hi + lo as a double: two exact widenings and one double addition. */
__host__ __device__ __forceinline__ double ff_to_double_bits(FF a) { return ff_widen(a.hi) + ff_widen(a.lo); }

/* s += a x for a float a and a float-float x: the head product a x.hi exact
   (two-product), added to s.hi by two-sum; the tails and a x.lo go to the
   low word (the accumulation of the float-float matvec). */
__host__ __device__ __forceinline__ void ff_axpy(FF &s, float a, FF x)
{
  const FF p = ff_two_prod(a, x.hi);
  FF t = ff_two_sum(s.hi, p.hi);
  t.lo += fmaf(a, x.lo, s.lo + p.lo);
  s = ff_fast_two_sum(t.hi, t.lo);
}

} /* namespace biofem */
#endif
