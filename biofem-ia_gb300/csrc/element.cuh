/*
 * Element physics of the active-strain Kirchhoff-Love shell, written once for
 * double and for a one-direction dual number (value + derivative), so the same
 * code gives the internal force and, lane by lane, the columns of its
 * derivative.
 *
 * The element is reduced to 15 "generalised coordinates"
 *   y = (a1, a2, Aaa, Abb, Aab) = N x_patch,
 * the centroid tangents and second derivatives of the Loop-subdivision patch
 * (active_strain.c:514-540 regular, :668-694 irregular).  The internal force
 * of the reference (ElemUpdFint, active_strain.c:1762-1995) is exactly
 *   Fb_a = sum_r N[r][a] f_r(y)   (r over the 5 rows of N, 3 components each)
 * with five force vectors f_r built from the membrane and bending resultants
 *   N^ab = pref0 sum_q w_q S_q^ab,  M^ab = pref0 sum_q w_q theta3_q S_q^ab:
 *   f1 = N11 a1 + N12 a2 - (gc1.Q) n,  f2 = N22 a2 + N12 a1 - (gc2.Q) n,
 *   f3 = -M11 n,  f4 = -M22 n,  f5 = -2 M12 n,   Q = M11 Aaa + M22 Abb + 2 M12 Aab.
 * The element stiffness is therefore K_e = N^T (df/dy) N.
 *
 * The stress S_q (ElemCGDefTens .. ModElemC33, active_strain.c:1332-1707,
 * 2048-2138) is evaluated in closed form.  With the reference-configuration
 * covariant fibre components t_i = g0_i . f, s = G^-1 t, phi = f.f, and the
 * active gradient Fa_cart = I - gamma f f^T:
 *   Fa.Cont = G^-1 - gamma s s^T,   Fa_inv.Cov = G + gamma' t t^T,
 *   gamma' = gamma / (1 - gamma phi);
 *   A = Fa.Cont G = I - gamma s t^T,  H = Fa_inv.Cov G^-1 = I + gamma' t s^T,
 *   A^T H = I.
 * Hence, for the "C_inv.Cont" matrix Ci of each C33 sub-iteration:
 *   Ce_inv = A Ci A^T,  Je = sqrt(rho / det Ci),  rho = 1 / (det G (1-gamma phi)^2),
 *   S  = mu (G^-1 + c1 s s^T) + alpha/2 (Ci + A Ci H),   c1 = 2 gamma' + gamma'^2 phi,
 *   CC3333 = 1/4 [2(beta-alpha) Qvv^2 + 4 beta Qvv Qwe - 4 alpha Qvw Qve
 *                 + (2beta-alpha) Qwe^2 - alpha Qww Qee],
 *   Qxy = (A^T x)^T Ci (A^T y),  v = Fa_inv.Cov G^-1 e3,  w = H v,
 *   alpha = K (Je^2 - Je) - mu,  beta = K Je (2 Je - 1) / 2,
 * which is the contraction the reference evaluates with its 3^6 and 3^8 loops
 * (active_strain.c:1381-1434, 1494-1532, 1592-1651).  The per-(element, qp)
 * reference constants (G^-1 entries, s, t, rho, A^T v, A^T w, A^T e3) are
 * computed once per mesh.
 */
#ifndef BIOFEM_ELEMENT_CUH
#define BIOFEM_ELEMENT_CUH

#include "biofem_host.h"
#include "ff.cuh"

namespace biofem {

/* ---------------- scalar types ---------------- */
/* One-direction dual number over the real type R (double or float). */
template <class R> struct D1 { R v, d; };
typedef D1<double> D1d;
typedef D1<float> D1f;

template <class R> __host__ __device__ __forceinline__ R val(R a) { return a; }
template <class R> __host__ __device__ __forceinline__ R val(const D1<R> &a) { return a.v; }

template <class R> __host__ __device__ __forceinline__ D1<R> operator+(D1<R> a, D1<R> b) { return {a.v + b.v, a.d + b.d}; }
template <class R> __host__ __device__ __forceinline__ D1<R> operator-(D1<R> a, D1<R> b) { return {a.v - b.v, a.d - b.d}; }
template <class R> __host__ __device__ __forceinline__ D1<R> operator-(D1<R> a) { return {-a.v, -a.d}; }
template <class R> __host__ __device__ __forceinline__ D1<R> operator*(D1<R> a, D1<R> b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
template <class R> __host__ __device__ __forceinline__ D1<R> operator+(D1<R> a, R b) { return {a.v + b, a.d}; }
template <class R> __host__ __device__ __forceinline__ D1<R> operator+(R a, D1<R> b) { return {a + b.v, b.d}; }
template <class R> __host__ __device__ __forceinline__ D1<R> operator-(D1<R> a, R b) { return {a.v - b, a.d}; }
template <class R> __host__ __device__ __forceinline__ D1<R> operator-(R a, D1<R> b) { return {a - b.v, -b.d}; }
template <class R> __host__ __device__ __forceinline__ D1<R> operator*(D1<R> a, R b) { return {a.v * b, a.d * b}; }
template <class R> __host__ __device__ __forceinline__ D1<R> operator*(R a, D1<R> b) { return {a * b.v, a * b.d}; }
/* Quotients take one reciprocal for value and derivative (the dual types are
   used only by the tangent kernels, whose primal values feed derivatives
   alone; the residual is evaluated separately in the plain type). */
template <class R> __host__ __device__ __forceinline__ D1<R> operator/(D1<R> a, D1<R> b)
{
  const R r = R(1) / b.v, q = a.v * r;
  return {q, (a.d - q * b.d) * r};
}
template <class R> __host__ __device__ __forceinline__ D1<R> operator/(R a, D1<R> b)
{
  const R r = R(1) / b.v, q = a * r;
  return {q, -(q * b.d) * r};
}
template <class R> __host__ __device__ __forceinline__ D1<R> operator/(D1<R> a, R b) { const R r = R(1) / b; return {a.v * r, a.d * r}; }
__host__ __device__ __forceinline__ D1d dsqrt(D1d a) { double r = sqrt(a.v); return {r, a.d * (0.5 / r)}; }
__host__ __device__ __forceinline__ D1f dsqrt(D1f a) { float r = sqrtf(a.v); return {r, a.d * (0.5f / r)}; }
/* K-direction dual number (the constitutive derivatives of the tangent
   kernels carry 2 or 3 metric directions per lane). */
template <class R, int K> struct DK { R v; R d[K]; };
template <class R, int K> __host__ __device__ __forceinline__ R val(const DK<R, K> &a) { return a.v; }
#define BIOFEM_DK_LOOP _Pragma("unroll") for (int i = 0; i < K; i++)
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator+(const DK<R, K> &a, const DK<R, K> &b)
{ DK<R, K> c; c.v = a.v + b.v; BIOFEM_DK_LOOP c.d[i] = a.d[i] + b.d[i]; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator-(const DK<R, K> &a, const DK<R, K> &b)
{ DK<R, K> c; c.v = a.v - b.v; BIOFEM_DK_LOOP c.d[i] = a.d[i] - b.d[i]; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator-(const DK<R, K> &a)
{ DK<R, K> c; c.v = -a.v; BIOFEM_DK_LOOP c.d[i] = -a.d[i]; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator*(const DK<R, K> &a, const DK<R, K> &b)
{ DK<R, K> c; c.v = a.v * b.v; BIOFEM_DK_LOOP c.d[i] = a.d[i] * b.v + a.v * b.d[i]; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator+(const DK<R, K> &a, R b)
{ DK<R, K> c = a; c.v = a.v + b; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator+(R a, const DK<R, K> &b)
{ DK<R, K> c = b; c.v = a + b.v; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator-(const DK<R, K> &a, R b)
{ DK<R, K> c = a; c.v = a.v - b; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator-(R a, const DK<R, K> &b)
{ DK<R, K> c; c.v = a - b.v; BIOFEM_DK_LOOP c.d[i] = -b.d[i]; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator*(const DK<R, K> &a, R b)
{ DK<R, K> c; c.v = a.v * b; BIOFEM_DK_LOOP c.d[i] = a.d[i] * b; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator*(R a, const DK<R, K> &b)
{ DK<R, K> c; c.v = a * b.v; BIOFEM_DK_LOOP c.d[i] = a * b.d[i]; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator/(const DK<R, K> &a, const DK<R, K> &b)
{ DK<R, K> c; const R r = R(1) / b.v; c.v = a.v * r; BIOFEM_DK_LOOP c.d[i] = (a.d[i] - c.v * b.d[i]) * r; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator/(R a, const DK<R, K> &b)
{ DK<R, K> c; const R r = R(1) / b.v; c.v = a * r; BIOFEM_DK_LOOP c.d[i] = -(c.v * b.d[i]) * r; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> operator/(const DK<R, K> &a, R b)
{ DK<R, K> c; const R r = R(1) / b; c.v = a.v * r; BIOFEM_DK_LOOP c.d[i] = a.d[i] * r; return c; }
template <class R, int K> __host__ __device__ __forceinline__ DK<R, K> dsqrt(const DK<R, K> &a)
{ DK<R, K> c; c.v = sqrt(a.v); const R h = R(0.5) / c.v; BIOFEM_DK_LOOP c.d[i] = a.d[i] * h; return c; }
#undef BIOFEM_DK_LOOP
__host__ __device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }
__host__ __device__ __forceinline__ float dsqrt(float a) { return sqrtf(a); }
__host__ __device__ __forceinline__ double dabs(double a) { return fabs(a); }
__host__ __device__ __forceinline__ float dabs(float a) { return fabsf(a); }

/* real type underlying a scalar */
template <class T> struct RealOf { typedef T type; };
template <class R> struct RealOf<D1<R>> { typedef R type; };

template <class T> struct V3 { T x, y, z; };
template <class T> __host__ __device__ __forceinline__ V3<T> operator+(const V3<T> &a, const V3<T> &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> __host__ __device__ __forceinline__ V3<T> operator-(const V3<T> &a, const V3<T> &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T, class S> __host__ __device__ __forceinline__ V3<T> scl(const S &s, const V3<T> &a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> __host__ __device__ __forceinline__ T dot(const V3<T> &a, const V3<T> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> __host__ __device__ __forceinline__ V3<T> cross(const V3<T> &a, const V3<T> &b)
{
  return {a.y * b.z - b.y * a.z, b.x * a.z - a.x * b.z, a.x * b.y - b.x * a.y};
}

/* One-hot directions of the FP64 tangent's chain rule.  Lane 3 r + c of an
   element group differentiates along the Cartesian component c of the r-th
   of (a1, a2, Aaa, Abb, Aab); a product with that unit vector is a selection
   of primal values (integer pipe), not FP64 arithmetic. */
__device__ __forceinline__ double ineg(double x)
{
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)(1ull << 63));
}
__device__ __forceinline__ float ineg(float x) { return __int_as_float(__float_as_int(x) ^ (int)(1u << 31)); }

template <class R> __device__ __forceinline__ R comp(const V3<R> &v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : v.z); }

/* e_c x v */
template <class R> __device__ __forceinline__ V3<R> ecross(int c, const V3<R> &v)
{
  return {c == 1 ? v.z : (c == 2 ? ineg(v.y) : R(0)), c == 0 ? ineg(v.z) : (c == 2 ? v.x : R(0)),
          c == 0 ? v.y : (c == 1 ? ineg(v.x) : R(0))};
}

/* v, -v or 0 */
template <class R> __device__ __forceinline__ V3<R> sel_sign(const V3<R> &v, bool on, bool neg)
{
  return {on ? (neg ? ineg(v.x) : v.x) : R(0), on ? (neg ? ineg(v.y) : v.y) : R(0),
          on ? (neg ? ineg(v.z) : v.z) : R(0)};
}

/* v + s e_c: one add */
template <class R> __device__ __forceinline__ V3<R> add_at(const V3<R> &v, int c, R s)
{
  const R t = comp(v, c) + s;
  return {c == 0 ? t : v.x, c == 1 ? t : v.y, c == 2 ? t : v.z};
}

/* a x b + acc and a.b + acc as FMA chains */
template <class R> __device__ __forceinline__ V3<R> cross_acc(const V3<R> &a, const V3<R> &b, const V3<R> &acc)
{
  return {fma(a.y, b.z, fma(-b.y, a.z, acc.x)), fma(b.x, a.z, fma(-a.x, b.z, acc.y)),
          fma(a.x, b.y, fma(-b.x, a.y, acc.z))};
}
template <class R> __device__ __forceinline__ R dot_acc(const V3<R> &a, const V3<R> &b, R acc)
{
  return fma(a.z, b.z, fma(a.y, b.y, fma(a.x, b.x, acc)));
}

/* Reference constants of one (element, qp), see the header comment. */
template <class R> struct QpRef {
  R gc00, gc11, gc01, gc22;   /* G^-1 entries used by S */
  R s[3], t[3];
  R rho;
  R av[3], aw[3], ae[3];      /* A^T v, A^T w, A^T e3 */
};

/* Material / quadrature constants in the working precision R. */
template <class R> struct EPar {
  R mu, K, hhalf;
  R theta[kMaxQp], w[kMaxQp];
  int nq, iters;
  int tnormal;   /* 1: thickness metric from the tangential part of a3,alpha (extension) */
};

template <class R> __host__ __device__ __forceinline__ EPar<R> epar(const KParams &p);
template <> __host__ __device__ __forceinline__ EPar<double> epar<double>(const KParams &p)
{
  EPar<double> e;
  e.mu = p.mu; e.K = p.K; e.hhalf = p.hhalf; e.nq = p.nq; e.iters = p.iters; e.tnormal = p.tnormal;
  for (int q = 0; q < kMaxQp; q++) { e.theta[q] = p.theta[q]; e.w[q] = p.w[q]; }
  return e;
}
/* Float-float parameters (the FP32-bulk residual) */
/* float-float parameters were split on the host */
template <> __host__ __device__ __forceinline__ EPar<FF> epar<FF>(const KParams &p)
{
  EPar<FF> e;
  e.mu = FF(p.mu2[0], p.mu2[1]); e.K = FF(p.K2[0], p.K2[1]); e.hhalf = FF(p.hhalf2[0], p.hhalf2[1]);
  e.nq = p.nq; e.iters = p.iters; e.tnormal = p.tnormal;
  for (int q = 0; q < kMaxQp; q++) {
    e.theta[q] = FF(p.theta2[q][0], p.theta2[q][1]);
    e.w[q] = FF(p.w2[q][0], p.w2[q][1]);
  }
  return e;
}
/* FP32 parameters were converted on the host: no FP64 work in FP32 kernels */
template <> __host__ __device__ __forceinline__ EPar<float> epar<float>(const KParams &p)
{
  EPar<float> e;
  e.mu = p.muf; e.K = p.Kf; e.hhalf = p.hhalff; e.nq = p.nq; e.iters = p.iters; e.tnormal = p.tnormal;
  for (int q = 0; q < kMaxQp; q++) { e.theta[q] = p.thetaf[q]; e.w[q] = p.wf[q]; }
  return e;
}

/* Quadratic form (A^T x)^T Ci (A^T y) with Ci = [[c00 c01 0][c01 c11 0][0 0 c22]]. */
template <class T, class R>
__host__ __device__ __forceinline__ T qform(const T &c00, const T &c11, const T &c01, const T &c22,
                                            const R *x, const R *y)
{
  return x[0] * (c00 * y[0] + c01 * y[1]) + x[1] * (c01 * y[0] + c11 * y[1]) + (x[2] * y[2]) * c22;
}

/* Primal values of the C33 sub-iterations of one thickness point that the
   FP64 tangent's derivative-only form reads (qp_stress_tl): the residual
   kernel of the same call records them (SoA over elements).  Slots: the
   initial cofactors and inverses, then per sub-iteration it (base
   kTapeInit + kTapeIt * it) the values named in qp_stress. */
constexpr int kTapeInit = 6;    /* cof00 cof11 cof01 cofx 1/det 1/(g00 g11 - g01^2) */
constexpr int kTapeIt = 23;
enum {
  kTpC00, kTpC11, kTpC01, kTpC22, kTpPre, kTpQd, kTpHJ, kTpJe, kTpAlpha, kTpBeta, kTpB33,
  kTpQvv, kTpQww, kTpQee, kTpQvw, kTpQve, kTpQwe, kTpICC, kTpDC, kTpLo, kTpB0, kTpB1, kTpB2
};
__host__ __device__ __forceinline__ int tape_per_qp(int iters) { return kTapeInit + kTapeIt * iters; }

/* Stress of one thickness point after the C33 sub-iterations:
   returns S^11, S^22, S^12 in sv[0..2]; status bit 1 on a vanishing CC3333.
   Every sub-iteration ends with the C33 update (ModElemC33); the stress is
   taken before the last one, so final_update = false skips that update
   (CC3333 and its check included) when only the stress is wanted and another
   kernel of the same call performs the check.  c33_out receives C33 after
   the last update; tape (stride ts) receives the primal values of
   qp_stress_tl (the arithmetic is the same with or without it). */
template <class T, class R>
__host__ __device__ __forceinline__ void qp_stress(const T gm[6] /* 00 11 01 02 12 22 */, const QpRef<R> &r,
                                                   R gam, R gamp, R c1, R mu, R K,
                                                   int iters, T sv[3], int &status, T *c33_out = nullptr,
                                                   bool final_update = true, R *tape = nullptr, size_t ts = 0)
{
  const R one = R(1), two = R(2), half = R(0.5), quarter = R(0.25);
  const T &g00 = gm[0], &g11 = gm[1], &g01 = gm[2], &g02 = gm[3], &g12 = gm[4], &g22 = gm[5];
  /* ElemCGDefTens: C_inv in-plane = in-plane block of gm^-1, C33 = 1 */
  T cof00 = g11 * g22 - g12 * g12;
  T cof11 = g00 * g22 - g02 * g02;
  T cof01 = g02 * g12 - g01 * g22;
  const T cofx = g01 * g12 - g11 * g02;
  T det = g00 * cof00 + g01 * cof01 + g02 * cofx;
  T idet = one / det;
  T c00 = cof00 * idet, c11 = cof11 * idet, c01 = cof01 * idet;
  T c22 = T{one};
  T C33 = T{one};
  if (tape) {
    tape[0] = val(cof00); tape[ts] = val(cof11); tape[2 * ts] = val(cof01); tape[3 * ts] = val(cofx);
    tape[4 * ts] = val(idet);
  }
  for (int it = 0; it < iters; it++) {
    R *tp = tape ? tape + (size_t)(kTapeInit + kTapeIt * it) * ts : nullptr;
    const T u0 = c00 * r.t[0] + c01 * r.t[1];
    const T u1 = c01 * r.t[0] + c11 * r.t[1];
    const T u2 = c22 * r.t[2];
    const T tau = r.t[0] * u0 + r.t[1] * u1 + r.t[2] * u2;
    const T pre = c00 * c11 - c01 * c01;
    const T detci = pre * c22;
    const T qrd = r.rho / detci;
    const T Je = dsqrt(qrd);
    const T alpha = K * (Je * Je - Je) - mu;
    const T beta = (half * K) * Je * (two * Je - one);
    const T half_a = half * alpha;
    const R gg = gam * gamp;
    /* S^33 */
    const T B33 = two * c22 + (gamp - gam) * r.s[2] * u2 - gg * r.s[2] * r.s[2] * tau;
    const T S33 = mu * (r.gc22 + c1 * r.s[2] * r.s[2]) + half_a * B33;
    if (tp) {
      tp[kTpC00 * ts] = val(c00); tp[kTpC11 * ts] = val(c11); tp[kTpC01 * ts] = val(c01); tp[kTpC22 * ts] = val(c22);
      tp[kTpPre * ts] = val(pre); tp[kTpQd * ts] = val(qrd) / val(detci); tp[kTpHJ * ts] = half / val(Je);
      tp[kTpJe * ts] = val(Je); tp[kTpAlpha * ts] = val(alpha); tp[kTpBeta * ts] = val(beta); tp[kTpB33 * ts] = val(B33);
    }
    if (it == iters - 1) {
      const T B0 = two * c00 + (gamp - gam) * r.s[0] * u0 - gg * r.s[0] * r.s[0] * tau;
      const T B1 = two * c11 + (gamp - gam) * r.s[1] * u1 - gg * r.s[1] * r.s[1] * tau;
      const T B2 = two * c01 + gamp * r.s[1] * u0 - gam * r.s[0] * u1 - gg * r.s[0] * r.s[1] * tau;
      sv[0] = mu * (r.gc00 + c1 * r.s[0] * r.s[0]) + half_a * B0;
      sv[1] = mu * (r.gc11 + c1 * r.s[1] * r.s[1]) + half_a * B1;
      sv[2] = mu * (r.gc01 + c1 * r.s[0] * r.s[1]) + half_a * B2;
      if (tp) { tp[kTpB0 * ts] = val(B0); tp[kTpB1 * ts] = val(B1); tp[kTpB2 * ts] = val(B2); }
    }
    if (!final_update && it == iters - 1) break;
    /* CC3333 */
    const T qvv = qform(c00, c11, c01, c22, r.av, r.av);
    const T qww = qform(c00, c11, c01, c22, r.aw, r.aw);
    const T qee = qform(c00, c11, c01, c22, r.ae, r.ae);
    const T qvw = qform(c00, c11, c01, c22, r.av, r.aw);
    const T qve = qform(c00, c11, c01, c22, r.av, r.ae);
    const T qwe = qform(c00, c11, c01, c22, r.aw, r.ae);
    const T twob = two * beta;
    const T CC = quarter * (two * (beta - alpha) * qvv * qvv + two * twob * qvv * qwe - R(4) * alpha * qvw * qve
                            + (twob - alpha) * qwe * qwe - alpha * qww * qee);
    /* ModElemC33 (active_strain.c:1654-1707) */
    if (!(dabs(val(CC)) > R(1e-14))) { status |= 1; return; }
    T dC = -S33 / CC;
    if (tp) {
      tp[kTpQvv * ts] = val(qvv); tp[kTpQww * ts] = val(qww); tp[kTpQee * ts] = val(qee);
      tp[kTpQvw * ts] = val(qvw); tp[kTpQve * ts] = val(qve); tp[kTpQwe * ts] = val(qwe);
      tp[kTpICC * ts] = one / val(CC); tp[kTpDC * ts] = val(dC); tp[kTpLo * ts] = one;
    }
    T Ct = C33 + dC;
    if (val(g00) * (val(g11) * val(Ct)) - val(g01) * (val(g01) * val(Ct)) <= R(0)) {
      R lo = R(0), hi = one;
      for (int bk = 0; bk < 16; bk++) {
        const R mid = half * (lo + hi);
        const R ct = val(C33) + mid * val(dC);
        if (val(g00) * (val(g11) * ct) - val(g01) * (val(g01) * ct) > R(0)) lo = mid; else hi = mid;
      }
      dC = dC * lo;
      Ct = C33 + dC;
      if (tp) tp[kTpLo * ts] = lo;
    }
    C33 = Ct;
    if (it + 1 < iters) {
      /* C_inv = INV([[gm00 gm01 0][gm01 gm11 0][0 0 C33]]): the in-plane block
         is the same in every later sub-iteration */
      if (it == 0) {
        const T id2 = one / (g00 * g11 - g01 * g01);
        c00 = g11 * id2; c11 = g00 * id2; c01 = -g01 * id2;
        if (tape) tape[5 * ts] = val(id2);
      }
      c22 = one / C33;
    }
  }
  if (c33_out) *c33_out = C33;
}

/* Derivative of qp_stress along KD directions dgm of the metric, from the
   primal values qp_stress recorded in tp (stride ts): only derivatives are
   computed, operation by operation.  The C33 update after the last stress is
   not differentiated (the tangent needs the stress only). */
template <class R, int KD>
__device__ __forceinline__ void qp_stress_tl(const R gm[6], const R dgm[6][KD], const QpRef<R> &r, R gam, R gamp,
                                             R c1, R mu, R K, int iters, const R *tp0, size_t ts, R sv[3],
                                             R dsv[3][KD])
{
  const R two = R(2), half = R(0.5), quarter = R(0.25), four = R(4);
  const R g00 = gm[0], g11 = gm[1], g01 = gm[2], g02 = gm[3], g12 = gm[4], g22 = gm[5];
  const R cof00 = tp0[0], cof01 = tp0[2 * ts], cofx = tp0[3 * ts], idet = tp0[4 * ts];
  const R cof11 = tp0[ts];
  R dc00[KD], dc11[KD], dc01[KD], dc22[KD], dC33[KD];
#pragma unroll
  for (int i = 0; i < KD; i++) {
    const R d00 = dgm[0][i], d11 = dgm[1][i], d01 = dgm[2][i], d02 = dgm[3][i], d12 = dgm[4][i], d22 = dgm[5][i];
    const R dcof00 = d11 * g22 + g11 * d22 - two * g12 * d12;
    const R dcof11 = d00 * g22 + g00 * d22 - two * g02 * d02;
    const R dcof01 = d02 * g12 + g02 * d12 - d01 * g22 - g01 * d22;
    const R dcofx = d01 * g12 + g01 * d12 - d11 * g02 - g11 * d02;
    const R ddet = d00 * cof00 + g00 * dcof00 + d01 * cof01 + g01 * dcof01 + d02 * cofx + g02 * dcofx;
    const R didet = -(idet * idet) * ddet;
    dc00[i] = dcof00 * idet + cof00 * didet;
    dc11[i] = dcof11 * idet + cof11 * didet;
    dc01[i] = dcof01 * idet + cof01 * didet;
    dc22[i] = R(0);
    dC33[i] = R(0);
  }
  const R gg = gam * gamp;
  for (int it = 0; it < iters; it++) {
    const R *tp = tp0 + (size_t)(kTapeInit + kTapeIt * it) * ts;
    const R c00 = tp[kTpC00 * ts], c11 = tp[kTpC11 * ts], c01 = tp[kTpC01 * ts], c22 = tp[kTpC22 * ts];
    const R pre = tp[kTpPre * ts], qd = tp[kTpQd * ts], hJ = tp[kTpHJ * ts], Je = tp[kTpJe * ts];
    const R alpha = tp[kTpAlpha * ts], beta = tp[kTpBeta * ts], B33 = tp[kTpB33 * ts];
    const R half_a = half * alpha;
    const bool last = it == iters - 1;
    R B0 = R(0), B1 = R(0), B2 = R(0);
    if (last) {
      B0 = tp[kTpB0 * ts]; B1 = tp[kTpB1 * ts]; B2 = tp[kTpB2 * ts];
      sv[0] = mu * (r.gc00 + c1 * r.s[0] * r.s[0]) + half_a * B0;
      sv[1] = mu * (r.gc11 + c1 * r.s[1] * r.s[1]) + half_a * B1;
      sv[2] = mu * (r.gc01 + c1 * r.s[0] * r.s[1]) + half_a * B2;
    }
    R qvv = R(0), qww = R(0), qee = R(0), qvw = R(0), qve = R(0), qwe = R(0), iCC = R(0), dC = R(0), lo = R(1);
    if (!last) {
      qvv = tp[kTpQvv * ts]; qww = tp[kTpQww * ts]; qee = tp[kTpQee * ts];
      qvw = tp[kTpQvw * ts]; qve = tp[kTpQve * ts]; qwe = tp[kTpQwe * ts];
      iCC = tp[kTpICC * ts]; dC = tp[kTpDC * ts]; lo = tp[kTpLo * ts];
    }
#pragma unroll
    for (int i = 0; i < KD; i++) {
      const R du0 = dc00[i] * r.t[0] + dc01[i] * r.t[1];
      const R du1 = dc01[i] * r.t[0] + dc11[i] * r.t[1];
      const R du2 = dc22[i] * r.t[2];
      const R dtau = r.t[0] * du0 + r.t[1] * du1 + r.t[2] * du2;
      const R dpre = dc00[i] * c11 + c00 * dc11[i] - two * c01 * dc01[i];
      const R ddetci = dpre * c22 + pre * dc22[i];
      const R dJe = hJ * (-(qd * ddetci));
      const R dalpha = K * (two * Je - R(1)) * dJe;
      const R dbeta = (half * K) * (four * Je - R(1)) * dJe;
      const R dhalf_a = half * dalpha;
      const R dB33 = two * dc22[i] + (gamp - gam) * r.s[2] * du2 - gg * r.s[2] * r.s[2] * dtau;
      const R dS33 = dhalf_a * B33 + half_a * dB33;
      if (last) {
        const R dB0 = two * dc00[i] + (gamp - gam) * r.s[0] * du0 - gg * r.s[0] * r.s[0] * dtau;
        const R dB1 = two * dc11[i] + (gamp - gam) * r.s[1] * du1 - gg * r.s[1] * r.s[1] * dtau;
        const R dB2 = two * dc01[i] + gamp * r.s[1] * du0 - gam * r.s[0] * du1 - gg * r.s[0] * r.s[1] * dtau;
        dsv[0][i] = dhalf_a * B0 + half_a * dB0;
        dsv[1][i] = dhalf_a * B1 + half_a * dB1;
        dsv[2][i] = dhalf_a * B2 + half_a * dB2;
        continue;
      }
      const R dqvv = qform(dc00[i], dc11[i], dc01[i], dc22[i], r.av, r.av);
      const R dqww = qform(dc00[i], dc11[i], dc01[i], dc22[i], r.aw, r.aw);
      const R dqee = qform(dc00[i], dc11[i], dc01[i], dc22[i], r.ae, r.ae);
      const R dqvw = qform(dc00[i], dc11[i], dc01[i], dc22[i], r.av, r.aw);
      const R dqve = qform(dc00[i], dc11[i], dc01[i], dc22[i], r.av, r.ae);
      const R dqwe = qform(dc00[i], dc11[i], dc01[i], dc22[i], r.aw, r.ae);
      const R dCC = quarter * (two * (dbeta - dalpha) * qvv * qvv + four * (beta - alpha) * qvv * dqvv
                               + four * dbeta * qvv * qwe + four * beta * (dqvv * qwe + qvv * dqwe)
                               - four * dalpha * qvw * qve - four * alpha * (dqvw * qve + qvw * dqve)
                               + (two * dbeta - dalpha) * qwe * qwe + two * (two * beta - alpha) * qwe * dqwe
                               - dalpha * qww * qee - alpha * (dqww * qee + qww * dqee));
      const R ddC = lo * (-(dS33 + dC * dCC) * iCC);
      dC33[i] = dC33[i] + ddC;
    }
    if (last) break;
    /* the in-plane inverse from iteration 1 on, and c22 = 1/C33 */
    const R *tpn = tp0 + (size_t)(kTapeInit + kTapeIt * (it + 1)) * ts;
    const R c22n = tpn[kTpC22 * ts];
    const R id2 = tp0[5 * ts];
#pragma unroll
    for (int i = 0; i < KD; i++) {
      if (it == 0) {
        const R dden = dgm[0][i] * g11 + g00 * dgm[1][i] - two * g01 * dgm[2][i];
        const R did2 = -(id2 * id2) * dden;
        dc00[i] = dgm[1][i] * id2 + g11 * did2;
        dc11[i] = dgm[0][i] * id2 + g00 * did2;
        dc01[i] = -(dgm[2][i] * id2 + g01 * did2);
      }
      dc22[i] = -(c22n * c22n) * dC33[i];
    }
  }
}

/* Mid-surface geometry of the element from y = (a1, a2, Aaa, Abb, Aab). */
template <class T> struct ElemGeom {
  V3<T> a1, a2, Aaa, Abb, Aab, n, gc1, gc2, a31, a32;
};

template <class T, class R>
__host__ __device__ __forceinline__ ElemGeom<T> elem_geom(const T y[15], const EPar<R> &p)
{
  const R one = R(1);
  ElemGeom<T> g;
  g.a1 = {y[0], y[1], y[2]}; g.a2 = {y[3], y[4], y[5]};
  g.Aaa = {y[6], y[7], y[8]}; g.Abb = {y[9], y[10], y[11]}; g.Aab = {y[12], y[13], y[14]};
  const V3<T> cr = cross(g.a1, g.a2);
  const T cn = dsqrt(dot(cr, cr));
  const T icn = one / cn;
  g.n = scl(icn, cr);
  const V3<T> t1 = cross(g.a2, g.n);
  g.gc1 = scl(one / dot(g.a1, t1), t1);
  const V3<T> t2 = cross(g.n, g.a1);
  g.gc2 = scl(one / dot(g.a2, t2), t2);
  g.a31 = scl(icn, cross(g.Aaa, g.a2) + cross(g.a1, g.Aab));
  g.a32 = scl(icn, cross(g.Aab, g.a2) + cross(g.a1, g.Abb));
  if (p.tnormal) {   /* n_,alpha: drop the J_,alpha / J n part of the unnormalised derivative */
    g.a31 = g.a31 - scl(dot(g.a31, g.n), g.n);
    g.a32 = g.a32 - scl(dot(g.a32, g.n), g.n);
  }
  return g;
}

/* Primal geometry the FP64 tangent's chain rule reads, stored once per element
   by the residual kernel of the same call (SoA over elements): n, 1/|a1 x a2|,
   t1 = a2 x n, t2 = n x a1, 1/(a1.t1), 1/(a2.t2), u31 = Aaa x a2 + a1 x Aab,
   u32 = Aab x a2 + a1 x Abb (elem_geom's intermediates); kGeomShape values,
   followed by elem_res_store's. */

template <class R>
__host__ __device__ __forceinline__ void elem_geom_store(const R y[15], R *gp, size_t stride)
{
  const R one = R(1);
  const V3<R> a1 = {y[0], y[1], y[2]}, a2 = {y[3], y[4], y[5]};
  const V3<R> Aaa = {y[6], y[7], y[8]}, Abb = {y[9], y[10], y[11]}, Aab = {y[12], y[13], y[14]};
  const V3<R> cr = cross(a1, a2);
  const R cn = dsqrt(dot(cr, cr));
  const R icn = one / cn;
  const V3<R> n = scl(icn, cr);
  const V3<R> t1 = cross(a2, n), t2 = cross(n, a1);
  const R s1 = one / dot(a1, t1), s2 = one / dot(a2, t2);
  const V3<R> u31 = cross(Aaa, a2) + cross(a1, Aab), u32 = cross(Aab, a2) + cross(a1, Abb);
  const R v[kGeomPrimal] = {n.x, n.y, n.z, icn, t1.x, t1.y, t1.z, t2.x, t2.y, t2.z, s1, s2,
                            u31.x, u31.y, u31.z, u32.x, u32.y, u32.z};
#pragma unroll
  for (int k = 0; k < kGeomShape; k++) gp[k * stride] = v[k];
}

/* The rest of the tangent's primal values (slots kGeomShape.. of the same
   block): the pref0-scaled resultants N0 N1 N2 M0 M1 M2, Q, gc1.Q, gc2.Q,
   gc1, gc2 (elem_out's intermediates, the same expressions). */
template <class T, class R>
__host__ __device__ __forceinline__ void elem_res_store(const ElemGeom<T> &g, T N0, T N1, T N2, T M0, T M1, T M2,
                                                        R pref0, R *gp, size_t stride)
{
  const R two = R(2);
  N0 = pref0 * N0; N1 = pref0 * N1; N2 = pref0 * N2;
  M0 = pref0 * M0; M1 = pref0 * M1; M2 = pref0 * M2;
  const T twoM2 = two * M2;
  const V3<T> Q = scl(M0, g.Aaa) + scl(M1, g.Abb) + scl(twoM2, g.Aab);
  const R v[kGeomPrimal - kGeomShape] = {
      val(N0), val(N1), val(N2), val(M0), val(M1), val(M2), val(Q.x), val(Q.y), val(Q.z),
      val(dot(g.gc1, Q)), val(dot(g.gc2, Q)),
      val(g.gc1.x), val(g.gc1.y), val(g.gc1.z), val(g.gc2.x), val(g.gc2.y), val(g.gc2.z)};
#pragma unroll
  for (int k = 0; k < kGeomPrimal - kGeomShape; k++) gp[(kGeomShape + k) * stride] = v[k];
}

/* Metric (00 11 01 02 12 22) of the thickness point theta3 (ElemUpdateG). */
template <class T, class R>
__host__ __device__ __forceinline__ void qp_metric(const ElemGeom<T> &g, R th3, T gm[6])
{
  const V3<T> g1 = g.a1 + scl(th3, g.a31), g2 = g.a2 + scl(th3, g.a32);
  gm[0] = dot(g1, g1); gm[1] = dot(g2, g2); gm[2] = dot(g1, g2);
  gm[3] = dot(g1, g.n); gm[4] = dot(g2, g.n); gm[5] = dot(g.n, g.n);
}

template <class R>
__host__ __device__ __forceinline__ QpRef<R> load_qpref(const R *ref, int stride, int q)
{
  QpRef<R> r;
  const R *rq = ref + (size_t)kRefPerQp * q * stride;
  r.gc00 = rq[0]; r.gc11 = rq[(size_t)1 * stride]; r.gc01 = rq[(size_t)2 * stride]; r.gc22 = rq[(size_t)3 * stride];
  for (int k = 0; k < 3; k++) {
    r.s[k] = rq[(size_t)(4 + k) * stride];
    r.t[k] = rq[(size_t)(7 + k) * stride];
    r.av[k] = rq[(size_t)(11 + k) * stride];
    r.aw[k] = rq[(size_t)(14 + k) * stride];
    r.ae[k] = rq[(size_t)(17 + k) * stride];
  }
  r.rho = rq[(size_t)10 * stride];
  return r;
}

/* The 15 force components from the resultants (ElemUpdFint, Nᵀ applied by the caller). */
template <class T, class R>
__host__ __device__ __forceinline__ void elem_out(const ElemGeom<T> &g, T N0, T N1, T N2, T M0, T M1, T M2, R pref0,
                                                  T f[15])
{
  const R two = R(2);
  N0 = pref0 * N0; N1 = pref0 * N1; N2 = pref0 * N2;
  M0 = pref0 * M0; M1 = pref0 * M1; M2 = pref0 * M2;
  const T twoM2 = two * M2;
  const V3<T> Q = scl(M0, g.Aaa) + scl(M1, g.Abb) + scl(twoM2, g.Aab);
  const V3<T> f1 = scl(N0, g.a1) + scl(N2, g.a2) - scl(dot(g.gc1, Q), g.n);
  const V3<T> f2 = scl(N1, g.a2) + scl(N2, g.a1) - scl(dot(g.gc2, Q), g.n);
  f[0] = f1.x; f[1] = f1.y; f[2] = f1.z;
  f[3] = f2.x; f[4] = f2.y; f[5] = f2.z;
  f[6] = -(M0 * g.n.x); f[7] = -(M0 * g.n.y); f[8] = -(M0 * g.n.z);
  f[9] = -(M1 * g.n.x); f[10] = -(M1 * g.n.y); f[11] = -(M1 * g.n.z);
  f[12] = -(twoM2 * g.n.x); f[13] = -(twoM2 * g.n.y); f[14] = -(twoM2 * g.n.z);
}

/* f(y): the 15 force components of the element.
   ref points at the element's first SoA constant (type R); stride = ne. */
template <class T, class R>
__host__ __device__ __forceinline__ void elem_forces(const T y[15], const EPar<R> &p, const R *ref, int stride,
                                                     T f[15], int &status, R *gm_out = nullptr, R *tape_out = nullptr,
                                                     R *gp_out = nullptr)
{
  const ElemGeom<T> g = elem_geom<T, R>(y, p);
  const int nq = p.nq;
  const R gam = ref[(size_t)(kRefPerQp * nq + 0) * stride];
  const R gamp = ref[(size_t)(kRefPerQp * nq + 1) * stride];
  const R c1 = ref[(size_t)(kRefPerQp * nq + 2) * stride];
  const R pref0 = ref[(size_t)(kRefPerQp * nq + 3) * stride];
  const T zero = T{R(0)};
  T N0 = zero, N1 = zero, N2 = zero, M0 = zero, M1 = zero, M2 = zero;
  for (int q = 0; q < nq; q++) {
    const QpRef<R> r = load_qpref(ref, stride, q);
    const R th3 = p.hhalf * p.theta[q];
    T gm[6];
    qp_metric(g, th3, gm);
    if (gm_out)   /* the metric of every thickness point, SoA over elements, for the tangent */
      for (int c = 0; c < 6; c++) gm_out[(size_t)(6 * q + c) * stride] = val(gm[c]);
    T sv[3];
    qp_stress(gm, r, gam, gamp, c1, p.mu, p.K, p.iters, sv, status, (T *)nullptr, true,
              tape_out ? tape_out + (size_t)q * tape_per_qp(p.iters) * stride : nullptr, (size_t)stride);
    const R wq = p.w[q], wt = p.w[q] * th3;
    N0 = N0 + wq * sv[0]; N1 = N1 + wq * sv[1]; N2 = N2 + wq * sv[2];
    M0 = M0 + wt * sv[0]; M1 = M1 + wt * sv[1]; M2 = M2 + wt * sv[2];
  }
  if (gp_out) elem_res_store(g, N0, N1, N2, M0, M1, M2, pref0, gp_out, (size_t)stride);
  elem_out(g, N0, N1, N2, M0, M1, M2, pref0, f);
}

/* UpdateElementThickness (active_strain.c:2198-2224): h0 sqrt(C33) with C33
   the mean over the thickness points of C33 after the sub-iterations (1 when
   that mean is not positive). */
template <class R>
__host__ __device__ __forceinline__ R elem_thickness(const R y[15], const EPar<R> &p, const R *ref, int stride, R h0,
                                                     int &status)
{
  const ElemGeom<R> g = elem_geom<R, R>(y, p);
  const int nq = p.nq;
  const R gam = ref[(size_t)(kRefPerQp * nq + 0) * stride];
  const R gamp = ref[(size_t)(kRefPerQp * nq + 1) * stride];
  const R c1 = ref[(size_t)(kRefPerQp * nq + 2) * stride];
  R sum = R(0);
  for (int q = 0; q < nq; q++) {
    const QpRef<R> r = load_qpref(ref, stride, q);
    R gm[6], sv[3], c33 = R(1);
    qp_metric(g, p.hhalf * p.theta[q], gm);
    qp_stress(gm, r, gam, gamp, c1, p.mu, p.K, p.iters, sv, status, &c33);
    sum += c33;
  }
  const R C33 = nq > 0 ? sum / (R)nq : R(1);
  return h0 * (C33 > R(0) ? sqrt(C33) : R(1));
}

/* Metric components the stress is differentiated along: 00 11 01 02 12.  The
   sixth, g33 = n.n, is 1 for every y (d(n.n) = 2 n.dn = 0), so its column of
   the constitutive derivative is never used; with the tangential thickness
   metric g_alpha.n = (a_alpha + th a3,alpha).n is 0 for every y as well, which
   leaves 00 11 01. */
template <class R>
__host__ __device__ __forceinline__ int metric_dirs(const EPar<R> &p) { return p.tnormal ? 3 : 5; }

/* Jobs (q, k0..k0+KD-1) of the split tangent: stress of thickness point q
   with KD metric directions (the last job of a point may carry unused
   directions); jac layout as in elem_forces_split. */
template <class R, int KD>
__device__ __forceinline__ void constitutive_jobs(const ElemGeom<R> *g0, const R *gmq, const EPar<R> &p, const R *ref,
                                                  int stride, int lane, R gam, R gamp, R c1, R *jac, int &status)
{
  typedef DK<R, KD> T;
  const int ndirs = metric_dirs(p);
  const int per_q = (ndirs + KD - 1) / KD;
  for (int job = lane; job < per_q * p.nq; job += 16) {
    const int q = job / per_q, k0 = (job - per_q * q) * KD;
    R gmv[6];
    if (gmq) {
#pragma unroll
      for (int c = 0; c < 6; c++) gmv[c] = gmq[(size_t)(6 * q + c) * stride];
    } else {
      qp_metric(*g0, p.hhalf * p.theta[q], gmv);
    }
    T gm[6];
#pragma unroll
    for (int c = 0; c < 6; c++) {
      gm[c].v = gmv[c];
#pragma unroll
      for (int i = 0; i < KD; i++) gm[c].d[i] = (c == k0 + i && c < ndirs) ? R(1) : R(0);
    }
    T sv[3];
    /* the stress only: the residual kernel of the same call checks the last CC3333 */
    qp_stress(gm, load_qpref(ref, stride, q), gam, gamp, c1, p.mu, p.K, p.iters, sv, status, (T *)nullptr, false);
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
      for (int t = 0; t < KD; t++)
        if (k0 + t < ndirs) jac[q * 21 + 6 * i + k0 + t] = sv[i].d[t];
    }
    if (k0 == 0) {
#pragma unroll
      for (int i = 0; i < 3; i++) jac[q * 21 + 18 + i] = sv[i].v;
    }
  }
}

/* Element forces and their derivative along y_lane, for a group of 16 lanes
   sharing one element (lane l < 15 carries direction l of y).  The
   constitutive update depends on y only through the 6 metric components of
   each thickness point, so it is differentiated along those: job (q, k) =
   derivative of the stress of point q along metric component k, one job per
   lane per round; each lane then applies the chain rule with its own metric
   derivative.  That is 5 nq (3 nq with the tangential thickness metric)
   constitutive derivative directions per element instead of 16 nq.  The primal values are the plain R-precision evaluation.
   jac: this group's scratch, kMaxQp * 21 values; the 16 lanes of the group
   and the other group of the warp must all call this (it synchronises the
   warp). */
template <class R>
__device__ __forceinline__ void elem_forces_split(const R y[15], const EPar<R> &p, const R *ref, int stride, int lane,
                                                  R *jac, D1<R> f[15], int &status, const R *gmq = nullptr)
{
  typedef D1<R> T;
  const int nq = p.nq;
  const R gam = ref[(size_t)(kRefPerQp * nq + 0) * stride];
  const R gamp = ref[(size_t)(kRefPerQp * nq + 1) * stride];
  const R c1 = ref[(size_t)(kRefPerQp * nq + 2) * stride];
  const R pref0 = ref[(size_t)(kRefPerQp * nq + 3) * stride];
  /* constitutive derivatives: jac[q*21 + 6*i + k] = d sv_i / d gm_k (k < ndirs),
     jac[q*21 + 18 + i] = sv_i; FP64: KD metric directions per job, the fewest
     for which the ceil(ndirs / KD) nq jobs fit one round of 16 lanes */
  {
    /* the primal metric of each thickness point: stored by the residual
       kernel of the same call (gmq), or from the element geometry here */
    ElemGeom<R> g0;
    if (!gmq) g0 = elem_geom<R, R>(y, p);
    if constexpr (sizeof(R) == 4) {
      /* FP32: one direction per job (wider duals spill under the FP32 kernel's register cap) */
      constitutive_jobs<R, 1>(&g0, gmq, p, ref, stride, lane, gam, gamp, c1, jac, status);
    } else {
      const int ndirs = metric_dirs(p);
      if (ndirs * nq <= 16) constitutive_jobs<R, 1>(&g0, gmq, p, ref, stride, lane, gam, gamp, c1, jac, status);
      else if (((ndirs + 1) / 2) * nq <= 16) constitutive_jobs<R, 2>(&g0, gmq, p, ref, stride, lane, gam, gamp, c1, jac, status);
      else constitutive_jobs<R, 3>(&g0, gmq, p, ref, stride, lane, gam, gamp, c1, jac, status);
    }
  }
  __syncwarp();
  const int ndirs = metric_dirs(p);
  T yd[15];
#pragma unroll
  for (int c = 0; c < 15; c++) yd[c] = T{y[c], c == lane ? R(1) : R(0)};
  const ElemGeom<T> g = elem_geom<T, R>(yd, p);
  const T zero = T{R(0), R(0)};
  T N0 = zero, N1 = zero, N2 = zero, M0 = zero, M1 = zero, M2 = zero;
  for (int q = 0; q < nq; q++) {
    const R th3 = p.hhalf * p.theta[q];
    T gm[6];
    qp_metric(g, th3, gm);
    T sv[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      R d = R(0);
#pragma unroll
      for (int c = 0; c < 5; c++)
        if (c < ndirs) d += jac[q * 21 + 6 * i + c] * gm[c].d;
      sv[i] = T{jac[q * 21 + 18 + i], d};
    }
    const R wq = p.w[q], wt = p.w[q] * th3;
    N0 = N0 + wq * sv[0]; N1 = N1 + wq * sv[1]; N2 = N2 + wq * sv[2];
    M0 = M0 + wt * sv[0]; M1 = M1 + wt * sv[1]; M2 = M2 + wt * sv[2];
  }
  elem_out(g, N0, N1, N2, M0, M1, M2, pref0, f);
}

/* constitutive_jobs in derivative-only form: the primal metric (gmq) and the
   primal C33 sub-iteration values (tape) come from the residual kernel. */
template <class R, int KD>
__device__ __forceinline__ void constitutive_jobs_tl(const R *gmq, const R *tape, const EPar<R> &p, const R *ref,
                                                     int stride, int lane, R gam, R gamp, R c1, R *jac)
{
  const int ndirs = metric_dirs(p);
  const int per_q = (ndirs + KD - 1) / KD;
  const int tq = tape_per_qp(p.iters);
  for (int job = lane; job < per_q * p.nq; job += 16) {
    const int q = job / per_q, k0 = (job - per_q * q) * KD;
    R gmv[6], dgm[6][KD];
#pragma unroll
    for (int c = 0; c < 6; c++) {
      gmv[c] = gmq[(size_t)(6 * q + c) * stride];
#pragma unroll
      for (int i = 0; i < KD; i++) dgm[c][i] = (c == k0 + i && c < ndirs) ? R(1) : R(0);
    }
    R sv[3], dsv[3][KD];
    qp_stress_tl<R, KD>(gmv, dgm, load_qpref(ref, stride, q), gam, gamp, c1, p.mu, p.K, p.iters,
                        tape + (size_t)q * tq * stride, (size_t)stride, sv, dsv);
    /* columns g00 and g11 doubled: the chain rule forms d g00 / 2 = dg1.g1 and d g11 / 2 = dg2.g2 */
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
      for (int t = 0; t < KD; t++)
        if (k0 + t < ndirs) jac[q * 21 + 6 * i + k0 + t] = k0 + t < 2 ? R(2) * dsv[i][t] : dsv[i][t];
    }
    if (k0 == 0) {
#pragma unroll
      for (int i = 0; i < 3; i++) jac[q * 21 + 18 + i] = sv[i];
    }
  }
}

/* The chain rule of elem_forces_split along y_lane in tangent-linear form: the
   primal geometry and resultants come from the residual kernel (gp, SoA
   stride: elem_geom_store, elem_res_store), the stress derivatives from the
   constitutive jobs (jac), so only derivatives are computed here.  Lane
   3 r + c carries the unit direction of component c of the r-th of
   (a1, a2, Aaa, Abb, Aab) (lane 15: none), and every product with it is a
   selection (one-hot helpers above).  The derivatives follow elem_geom,
   qp_metric and elem_out operation by operation:
     dcr = da1 x a2 + a1 x da2,  d|cr| = n.dcr (= t1_c or t2_c),
     dn = (dcr - n d|cr|)/|cr|,  d(1/|cr|) = -d|cr|/|cr|^2,
     dt1 = da2 x n + a2 x dn,  d(1/(a1.t1)) = -(da1.t1 + a1.dt1)/(a1.t1)^2, ...
   df holds d f_r / d y_lane. */
template <class R>
__device__ __forceinline__ void elem_forces_split_tl(const R y[15], const EPar<R> &p, const R *ref, int stride,
                                                     const R *gp, int lane, R *jac, R df[15], const R *gmq,
                                                     const R *tape)
{
  const int nq = p.nq;
  const R gam = ref[(size_t)(kRefPerQp * nq + 0) * stride];
  const R gamp = ref[(size_t)(kRefPerQp * nq + 1) * stride];
  const R c1 = ref[(size_t)(kRefPerQp * nq + 2) * stride];
  const R pref0 = ref[(size_t)(kRefPerQp * nq + 3) * stride];
  const int ndirs = metric_dirs(p);
  if (ndirs * nq <= 16) constitutive_jobs_tl<R, 1>(gmq, tape, p, ref, stride, lane, gam, gamp, c1, jac);
  else if (((ndirs + 1) / 2) * nq <= 16) constitutive_jobs_tl<R, 2>(gmq, tape, p, ref, stride, lane, gam, gamp, c1, jac);
  else constitutive_jobs_tl<R, 3>(gmq, tape, p, ref, stride, lane, gam, gamp, c1, jac);
  __syncwarp();
  const R zero = R(0), one = R(1), two = R(2);
  R g[kGeomPrimal];
#pragma unroll
  for (int k = 0; k < kGeomPrimal; k++) g[k] = gp[(size_t)k * stride];
  const V3<R> n = {g[0], g[1], g[2]}, t1 = {g[4], g[5], g[6]}, t2 = {g[7], g[8], g[9]};
  const R icn = g[3], s1 = g[10], s2 = g[11];
  const V3<R> u31 = {g[12], g[13], g[14]}, u32 = {g[15], g[16], g[17]};
  const R N0 = g[18], N1 = g[19], N2 = g[20], M0 = g[21], M1 = g[22], M2 = g[23];   /* pref0-scaled */
  const V3<R> Q = {g[24], g[25], g[26]};
  const R q1 = g[27], q2 = g[28];
  const V3<R> gc1 = {g[29], g[30], g[31]}, gc2 = {g[32], g[33], g[34]};
  const V3<R> a1 = {y[0], y[1], y[2]}, a2 = {y[3], y[4], y[5]};
  const V3<R> Aaa = {y[6], y[7], y[8]}, Abb = {y[9], y[10], y[11]}, Aab = {y[12], y[13], y[14]};
  const int r = lane / 3, c = lane - 3 * r;
  /* geometry */
  const V3<R> dcr = sel_sign(ecross(c, r == 0 ? a2 : a1), r < 2, r == 1);
  const R dcn = r == 0 ? comp(t1, c) : (r == 1 ? comp(t2, c) : zero);
  const V3<R> dn = scl(icn, dcr - scl(dcn, n));
  const R dicn = -(icn * icn) * dcn;
  const V3<R> dt1 = cross_acc(a2, dn, sel_sign(ecross(c, n), r == 1, false));
  const R ds1 = -(s1 * s1) * dot_acc(a1, dt1, r == 0 ? comp(t1, c) : zero);
  const V3<R> dgc1 = scl(ds1, t1) + scl(s1, dt1);
  const V3<R> dt2 = cross_acc(dn, a1, sel_sign(ecross(c, n), r == 0, true));
  const R ds2 = -(s2 * s2) * dot_acc(a2, dt2, r == 1 ? comp(t2, c) : zero);
  const V3<R> dgc2 = scl(ds2, t2) + scl(s2, dt2);
  /* du31 = dAaa x a2 + Aaa x da2 + da1 x Aab + a1 x dAab and
     du32 = dAab x a2 + Aab x da2 + da1 x Abb + a1 x dAbb: one term each */
  const V3<R> v31 = r == 0 ? Aab : (r == 1 ? Aaa : (r == 2 ? a2 : a1));
  const V3<R> du31 = sel_sign(ecross(c, v31), r < 3 || r == 4, r == 1 || r == 4);
  const V3<R> v32 = r == 0 ? Abb : (r == 1 ? Aab : (r == 3 ? a1 : a2));
  const V3<R> du32 = sel_sign(ecross(c, v32), r < 2 || r == 3 || r == 4, r == 1 || r == 3);
  V3<R> a31 = scl(icn, u31), a32 = scl(icn, u32);
  V3<R> da31 = scl(icn, du31) + scl(dicn, u31), da32 = scl(icn, du32) + scl(dicn, u32);
  if (p.tnormal) {   /* a3,alpha - (a3,alpha . n) n */
    const R p31 = dot(a31, n), p32 = dot(a32, n);
    const R dp31 = dot(da31, n) + dot(a31, dn), dp32 = dot(da32, n) + dot(a32, dn);
    da31 = da31 - scl(dp31, n) - scl(p31, dn);
    da32 = da32 - scl(dp32, n) - scl(p32, dn);
    a31 = a31 - scl(p31, n);
    a32 = a32 - scl(p32, n);
  }
  const V3<R> da1 = {r == 0 && c == 0 ? one : zero, r == 0 && c == 1 ? one : zero, r == 0 && c == 2 ? one : zero};
  const V3<R> da2 = {r == 1 && c == 0 ? one : zero, r == 1 && c == 1 ? one : zero, r == 1 && c == 2 ? one : zero};
  /* resultant derivatives by the chain rule through each thickness point's metric */
  R dN0 = zero, dN1 = zero, dN2 = zero, dM0 = zero, dM1 = zero, dM2 = zero;
  for (int q = 0; q < nq; q++) {
    const R th3 = p.hhalf * p.theta[q];
    const V3<R> g1 = a1 + scl(th3, a31), g2 = a2 + scl(th3, a32);
    const V3<R> dg1 = da1 + scl(th3, da31), dg2 = da2 + scl(th3, da32);
    /* halves of d g00 and d g11: their stress columns are stored doubled */
    const R dgm[5] = {dot(dg1, g1), dot(dg2, g2), dot_acc(g1, dg2, dot(dg1, g2)), dot_acc(g1, dn, dot(dg1, n)),
                      dot_acc(g2, dn, dot(dg2, n))};
    R dsv[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      R d = zero;
#pragma unroll
      for (int k = 0; k < 5; k++)
        if (k < ndirs) d += jac[q * 21 + 6 * i + k] * dgm[k];
      dsv[i] = d;
    }
    const R wq = p.w[q], wt = p.w[q] * th3;
    dN0 = dN0 + wq * dsv[0]; dN1 = dN1 + wq * dsv[1]; dN2 = dN2 + wq * dsv[2];
    dM0 = dM0 + wt * dsv[0]; dM1 = dM1 + wt * dsv[1]; dM2 = dM2 + wt * dsv[2];
  }
  /* elem_out */
  dN0 = pref0 * dN0; dN1 = pref0 * dN1; dN2 = pref0 * dN2; dM0 = pref0 * dM0; dM1 = pref0 * dM1; dM2 = pref0 * dM2;
  const R twoM2 = two * M2, dtwoM2 = two * dM2;
  /* dQ = dM0 Aaa + M0 dAaa + dM1 Abb + M1 dAbb + d(2 M2) Aab + 2 M2 dAab */
  const V3<R> dQ = add_at(scl(dM0, Aaa) + scl(dM1, Abb) + scl(dtwoM2, Aab), c,
                          r == 2 ? M0 : (r == 3 ? M1 : (r == 4 ? twoM2 : zero)));
  const R dq1 = dot_acc(gc1, dQ, dot(dgc1, Q)), dq2 = dot_acc(gc2, dQ, dot(dgc2, Q));
  /* df1 = dN0 a1 + N0 da1 + dN2 a2 + N2 da2 - dq1 n - q1 dn,
     df2 = dN1 a2 + N1 da2 + dN2 a1 + N2 da1 - dq2 n - q2 dn */
  const V3<R> df1 = add_at(scl(dN0, a1) + scl(dN2, a2) - scl(dq1, n) - scl(q1, dn), c,
                           r == 0 ? N0 : (r == 1 ? N2 : zero));
  const V3<R> df2 = add_at(scl(dN1, a2) + scl(dN2, a1) - scl(dq2, n) - scl(q2, dn), c,
                           r == 1 ? N1 : (r == 0 ? N2 : zero));
  df[0] = df1.x; df[1] = df1.y; df[2] = df1.z;
  df[3] = df2.x; df[4] = df2.y; df[5] = df2.z;
  const V3<R> dm0 = scl(dM0, n) + scl(M0, dn), dm1 = scl(dM1, n) + scl(M1, dn), dm2 = scl(dtwoM2, n) + scl(twoM2, dn);
  df[6] = -dm0.x; df[7] = -dm0.y; df[8] = -dm0.z;
  df[9] = -dm1.x; df[10] = -dm1.y; df[11] = -dm1.z;
  df[12] = -dm2.x; df[13] = -dm2.y; df[14] = -dm2.z;
}

/* ---------------- tangent contraction (row assembly) ---------------- */
/* The element stiffness is K_e = N^T D N with D = df/dy (15 x 15) and N the
   5 x nen basis table acting on each Cartesian component.  The row assembly
   forms it one block row a at a time:
     w = (N[:,a] (x) I3)^T D          (3 x 15, w[15 i + k] = sum_r N[r][a] D[3r+i][k]),
     K_ab[i][j] = sum_s N[s][b] w[15 i + 3 s + j],
   plus, when a and b are corner slots of the triangle, the follower-pressure
   block: the cross-product matrix of sc v_b, v_b the corner's vector.
   Both sums run over the five basis rows, so the operands are kept with that
   index innermost, padded to 8, for vector loads: the table as
   tabT[8 b + s] = N[s][b] and w as wT[8 (3 i + j) + s] = w[15 i + 3 s + j]. */
constexpr int kRowPad = 8;

/* five consecutive values from a 16-byte aligned address */
template <class R>
__host__ __device__ __forceinline__ void load5(const R *p, R v[5])
{
#ifdef __CUDA_ARCH__
  if constexpr (sizeof(R) == 4) {
    const float4 a = *reinterpret_cast<const float4 *>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = p[4];
  } else {
    const double2 a = *reinterpret_cast<const double2 *>(p), b = *reinterpret_cast<const double2 *>(p + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = p[4];
  }
#else
  for (int k = 0; k < 5; k++) v[k] = p[k];
#endif
}

/* Entry t < 45 of w for the row slot whose table column is tabT_a (= tabT +
   8 a); *pos receives its place in wT. */
template <class R>
__host__ __device__ __forceinline__ R row_wt_entry(const R *D, const R *tabT_a, int t, int *pos)
{
  const int i = t / 15, k = t - 15 * i, s = k / 3, j = k - 3 * s;
  R n[5];
  load5(tabT_a, n);
  R acc = R(0);
#pragma unroll
  for (int r = 0; r < 5; r++) acc = fma(n[r], D[(3 * r + i) * 15 + k], acc);
  *pos = kRowPad * (3 * i + j) + s;
  return acc;
}

/* acc + K_ab[i][j], q = 3 i + j, from wT_q = wT + 8 q and tabT_b = tabT + 8 b,
   as one chain of fused multiply-adds. */
template <class R>
__host__ __device__ __forceinline__ R row_block_accum(const R *wT_q, const R *tabT_b, R acc)
{
  R w[5], n[5];
  load5(wT_q, w);
  load5(tabT_b, n);
#pragma unroll
  for (int s = 0; s < 5; s++) acc = fma(n[s], w[s], acc);
  return acc;
}

/* Entry (i, j) of the follower-pressure block d c / d x_k = [s v]x (the cross
   product matrix of s v), for runtime i, j. */
template <class R>
__host__ __device__ __forceinline__ R skew_entry(int i, int j, const R v[3], R s)
{
  if (i == j) return R(0);
  const int m3 = 3 - i - j;
  const R vm = m3 == 0 ? v[0] : (m3 == 1 ? v[1] : v[2]);
  const R t = s * vm;
  return (j - i + 3) % 3 == 1 ? -t : t;
}

} /* namespace biofem */
#endif
