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

} /* namespace biofem */
#endif
