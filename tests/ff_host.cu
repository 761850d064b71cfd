/* Host check of the float-float arithmetic (biofem-ia_gb300/csrc/ff.cuh) for
   tests/test_ff_host.py: for seeded operand pairs spanning 1e-12 .. 1e12 (and
   nearly cancelling pairs for the sum), prints the largest error of +, -, *,
   /, sqrt against long double, relative to the result (sum: to the larger
   operand, the bound a double-word sum guarantees under cancellation). */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "../biofem-ia_gb300/csrc/ff.cuh"

using namespace biofem;

static uint64_t g_state = 0x9e3779b97f4a7c15ull;
static double urand()
{
  g_state = g_state * 6364136223846793005ull + 1442695040888963407ull;
  return (double)(g_state >> 11) * (1.0 / 9007199254740992.0);
}
static double operand()
{
  const double mag = std::pow(10.0, -12.0 + 24.0 * urand());
  return (urand() < 0.5 ? -1.0 : 1.0) * mag * (1.0 + urand());
}
static long double ld(FF a) { return (long double)a.hi + (long double)a.lo; }
/* the operand as the float-float value it becomes, exactly */
static long double ldv(double d) { return ld(FF(d)); }

int main()
{
  double e_add = 0, e_cancel = 0, e_mul = 0, e_div = 0, e_sqrt = 0;
  for (int k = 0; k < 200000; k++) {
    const double a = operand(), b = operand();
    const FF A(a), B(b);
    const long double la = ldv(a), lb = ldv(b);
    const long double s = la + lb;
    e_add = std::fmax(e_add, (double)(std::fabs(ld(A + B) - s) / std::fmax(std::fabs(la), std::fabs(lb))));
    const double c = -a * (1.0 + 1e-9 * (urand() - 0.5));   /* nearly cancelling */
    const FF C(c);
    const long double lc = ldv(c);
    e_cancel = std::fmax(e_cancel, (double)(std::fabs(ld(A + C) - (la + lc)) / std::fabs(la)));
    e_mul = std::fmax(e_mul, (double)(std::fabs(ld(A * B) - la * lb) / std::fabs(la * lb)));
    e_div = std::fmax(e_div, (double)(std::fabs(ld(A / B) - la / lb) / std::fabs(la / lb)));
    const double p = std::fabs(a);
    const long double lp = ldv(p);
    e_sqrt = std::fmax(e_sqrt, (double)(std::fabs(ld(dsqrt(FF(p))) - std::sqrt(lp)) / std::sqrt(lp)));
  }
  /* the bit-level conversions: ff_split(d) = d to 2^-47 and normalised;
     ff_widen(f) = (double)f bit for bit; ff_to_double_bits(a) = hi + lo in double */
  double e_split = 0.0;
  long bad_norm = 0, bad_widen = 0, bad_todouble = 0;
  for (int k = 0; k < 200000; k++) {
    const double d = operand();
    const FF a = ff_split(d);
    e_split = std::fmax(e_split, (double)(std::fabs(ld(a) - (long double)d) / std::fabs((long double)d)));
    if (std::fabs(a.lo) > std::ldexp(std::fabs(a.hi), -24)) bad_norm++;
    const float f = (float)d;
    const double w = ff_widen(f), wr = (double)f;
    if (std::memcmp(&w, &wr, 8) != 0) bad_widen++;
    const FF b(d);
    const double t = ff_to_double_bits(b), tr = (double)b.hi + (double)b.lo;
    if (std::memcmp(&t, &tr, 8) != 0) bad_todouble++;
  }
  const FF z = ff_split(0.0), nz = ff_split(-0.0);
  const bool zeros = z.hi == 0.f && z.lo == 0.f && nz.hi == 0.f && std::signbit(nz.hi) && ff_widen(0.f) == 0.0;
  /* the float-float matvec's row sums: 324 terms (36 blocks x 9) of float K
     values over four decades times split double x, accumulated by ff_axpy,
     against long double, relative to sum |K x| */
  double e_dot = 0.0;
  for (int r = 0; r < 4000; r++) {
    FF s(0.f, 0.f);
    long double exact = 0.0L, mag = 0.0L;
    for (int k = 0; k < 324; k++) {
      const float a = (float)((urand() < 0.5 ? -1.0 : 1.0) * std::pow(10.0, -2.0 + 4.0 * urand()));
      const double x = (urand() < 0.5 ? -1.0 : 1.0) * std::pow(10.0, -3.0 + 3.0 * urand());
      ff_axpy(s, a, ff_split(x));
      exact += (long double)a * (long double)x;
      mag += std::fabs((long double)a * (long double)x);
    }
    e_dot = std::fmax(e_dot, (double)(std::fabs((long double)ff_to_double_bits(s) - exact) / mag));
  }
  std::printf("%.3e %.3e %.3e %.3e %.3e %.3e %ld %ld %ld %d %.3e\n", e_add, e_cancel, e_mul, e_div, e_sqrt, e_split,
              bad_norm, bad_widen, bad_todouble, zeros ? 1 : 0, e_dot);
  return 0;
}
