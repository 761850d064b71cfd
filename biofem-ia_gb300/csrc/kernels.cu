/*
 * sm_103a kernels of the element residual / tangent / assembly path.
 *
 *   k_positions      x (Vec layout) -> padded node positions; ghost nodes
 *                    x_g = x_nv2 + x_nv1 - x_nv3 (GlobalGhost, bending.c:1763-1814)
 *   k_ref_prep       one-time reference geometry per element (geom0 + the
 *                    reference half of ElemUpdateG and ElemActDefGrad)
 *   k_elem_residual  one thread per element: geometry, closed-form stress,
 *                    element forces Fb (ElemUpdFint) and the follower-pressure
 *                    corner force (SurfaceNormalPressure, external.c:589-624)
 *                    (and, for the FP64 tangent, the primal values its
 *                    derivative-only form reads: thickness-point metrics,
 *                    geometry, resultants, C33 sub-iteration values)
 *   k_elem_tangent   16 lanes per element: the stress is differentiated along
 *                    the metric components of each thickness point (one job
 *                    per lane), then lane j carries d/dy_j through the
 *                    geometry and the chain rule, giving column j of
 *                    D = df/dy, stored per element (kDeStride values, with the
 *                    follower-pressure corner vectors) for the row assembly
 *   k_elem_residual_ff  the FP32-bulk residual: k_elem_residual's element math
 *                    in float-float numbers on the FP32 pipe
 *   k_node_gather    one thread per node: Fint / Fext (and FDynamic's Fdyn)
 *                    summed over the node's element contributions in element
 *                    order (the order FInternalAct's VecSetValues loop adds
 *                    them), R = Fint - Fext + Fdyn, clamp rows R = x - X,
 *                    ghost rows 0 (main.c:844-1016)
 *   k_row_assemble   one warp per row node: for every element holding the
 *                    node, K_e's block row N_a^T D N (and the pressure blocks)
 *                    added into the row's blocks in shared memory in a fixed
 *                    order, then the row written once
 *   k_scale          R *= 1 / max(|Fext|_inf, 1) (main.c:1020-1026); the row
 *                    assembly applies the same factor to K as it writes it
 *   k_elem_thickness UpdateElementThickness (output); k_dyn_diag / k_dyn_update
 *                    the dynamic term's tangent diagonal and xAccVel
 *
 * Assembly is deterministic: every sum runs in a fixed order given by the
 * precomputed node-to-element lists, independent of the launch
 * configuration; nothing is accumulated with atomics.
 */
#include <cuda_runtime.h>

#include "element.cuh"

namespace biofem {

/* ---------------- helpers ---------------- */
__device__ __forceinline__ void load_node(const double *pos, int node, double &x, double &y, double &z)
{
  const double2 a = __ldg(reinterpret_cast<const double2 *>(pos) + 2 * (size_t)node);
  const double b = __ldg(pos + 4 * (size_t)node + 2);
  x = a.x; y = a.y; z = b;
}

__device__ __forceinline__ void set_status(int *status, int bits)
{
  if (bits) atomicOr(status, bits);
}

/* y = N x over the element patch (regular table or IN arrays of valence v). */
__device__ __forceinline__ void gather_y(const double *pos, const int *patch, int e, int nen, const double *tab,
                                         double y[15])
{
  for (int k = 0; k < 15; k++) y[k] = 0.0;
  const int4 *p4 = reinterpret_cast<const int4 *>(patch + 16 * (size_t)e);
  int nodes[16];
  const int4 q0 = __ldg(p4), q1 = __ldg(p4 + 1), q2 = __ldg(p4 + 2), q3 = __ldg(p4 + 3);
  nodes[0] = q0.x; nodes[1] = q0.y; nodes[2] = q0.z; nodes[3] = q0.w;
  nodes[4] = q1.x; nodes[5] = q1.y; nodes[6] = q1.z; nodes[7] = q1.w;
  nodes[8] = q2.x; nodes[9] = q2.y; nodes[10] = q2.z; nodes[11] = q2.w;
  nodes[12] = q3.x; nodes[13] = q3.y; nodes[14] = q3.z; nodes[15] = q3.w;
#pragma unroll 4
  for (int i = 0; i < nen; i++) {
    double x, yy, z;
    load_node(pos, nodes[i], x, yy, z);
#pragma unroll
    for (int r = 0; r < 5; r++) {
      const double c = tab[r * 16 + i];
      y[3 * r] += c * x; y[3 * r + 1] += c * yy; y[3 * r + 2] += c * z;
    }
  }
}

/* gather_y for a group of 16 lanes sharing one element: lane l < 15 sums
   component l (row l / 3, coordinate l % 3) in gather_y's order, then the
   group exchanges the 15 sums, so every lane ends with gather_y's y at one
   fifteenth of the FP64 work. */
__device__ __forceinline__ void gather_y_group(const double *pos, const int *patch, int e, int nen, const double *tab,
                                               int lane, double y[15])
{
  double s = 0.0;
  if (lane < 15) {
    const int r = lane / 3, d = lane - 3 * r;
    const int *pe = patch + 16 * (size_t)e;
    for (int i = 0; i < nen; i++) s += tab[r * 16 + i] * __ldg(pos + 4 * (size_t)__ldg(pe + i) + d);
  }
#pragma unroll
  for (int c = 0; c < 15; c++) y[c] = __shfl_sync(0xffffffffu, s, c, 16);
}

/* ---------------- positions / ghosts ---------------- */
__global__ void k_positions(int nv, int ng, const double *__restrict__ x, const int *__restrict__ ghost3,
                            double *__restrict__ pos)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double o[4] = {0.0, 0.0, 0.0, 0.0};
  if (i < nv) {
    o[0] = x[3 * (size_t)i]; o[1] = x[3 * (size_t)i + 1]; o[2] = x[3 * (size_t)i + 2];
  } else if (i < nv + ng) {
    const int g = i - nv;
    const int n1 = ghost3[3 * g], n2 = ghost3[3 * g + 1], n3 = ghost3[3 * g + 2];
    for (int d = 0; d < 3; d++) o[d] = x[3 * (size_t)n2 + d] + x[3 * (size_t)n1 + d] - x[3 * (size_t)n3 + d];
  } else {
    return;
  }
  double2 *dst = reinterpret_cast<double2 *>(pos) + 2 * (size_t)i;
  dst[0] = make_double2(o[0], o[1]);
  dst[1] = make_double2(o[2], o[3]);
}

/* ---------------- reference preparation ---------------- */
/* 3x3 inverse by cofactors (math.c:75-89 form). */
__device__ __forceinline__ void inv3(const double A[3][3], double B[3][3])
{
  const double det = A[0][0] * (A[2][2] * A[1][1] - A[2][1] * A[1][2]) - A[1][0] * (A[2][2] * A[0][1] - A[2][1] * A[0][2])
                   + A[2][0] * (A[1][2] * A[0][1] - A[1][1] * A[0][2]);
  const double c = 1.0 / det;
  B[0][0] = c * (A[2][2] * A[1][1] - A[2][1] * A[1][2]);
  B[0][1] = -c * (A[2][2] * A[0][1] - A[2][1] * A[0][2]);
  B[0][2] = c * (A[1][2] * A[0][1] - A[1][1] * A[0][2]);
  B[1][0] = -c * (A[2][2] * A[1][0] - A[2][0] * A[1][2]);
  B[1][1] = c * (A[2][2] * A[0][0] - A[2][0] * A[0][2]);
  B[1][2] = -c * (A[1][2] * A[0][0] - A[1][0] * A[0][2]);
  B[2][0] = c * (A[2][1] * A[1][0] - A[2][0] * A[1][1]);
  B[2][1] = -c * (A[2][1] * A[0][0] - A[2][0] * A[0][1]);
  B[2][2] = c * (A[1][1] * A[0][0] - A[1][0] * A[0][1]);
}

__device__ __forceinline__ double det3(const double A[3][3])
{
  return A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0])
       + A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
}

__global__ void k_ref_prep(DevMesh m, KParams p, const double *__restrict__ fib, const double *__restrict__ gscale,
                           double *__restrict__ eref)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ne) return;
  const int info = m.einfo[e];
  const int nen = info & 0xff, tabi = info >> 8;
  double y[15];
  gather_y(m.pos, m.patch, e, nen, m.ntab + tabi * 80, y);
  const V3<double> a1 = {y[0], y[1], y[2]}, a2 = {y[3], y[4], y[5]};
  const V3<double> Aaa = {y[6], y[7], y[8]}, Abb = {y[9], y[10], y[11]}, Aab = {y[12], y[13], y[14]};
  const V3<double> cr = cross(a1, a2);
  const double cn = sqrt(dot(cr, cr));
  const V3<double> n = {cr.x / cn, cr.y / cn, cr.z / cn};
  V3<double> a31 = cross(Aaa, a2) + cross(a1, Aab), a32 = cross(Aab, a2) + cross(a1, Abb);
  a31 = {a31.x / cn, a31.y / cn, a31.z / cn};
  a32 = {a32.x / cn, a32.y / cn, a32.z / cn};
  if (p.tnormal) {
    a31 = a31 - scl(dot(a31, n), n);
    a32 = a32 - scl(dot(a32, n), n);
  }
  /* Fa_cart = afac (I - gam f f^T): the fibre activation (-cart_fib_act 1)
     has afac = 1; the isotropic one (-cart_fib_act 0,
     active_strain.c:1238-1255), diag(a, a, 1/a^2) with a = 1 - gamma, is
     a (I - (1 - 1/a^3) e3 e3^T).  The scale afac divides the mu part of the
     stress by afac^2 and rho by afac^6 (det Fa_cart = afac^3 (1 - gam phi));
     Ci + A Ci H, CC3333 and the quadratic forms do not depend on it. */
  double afac = 1.0, gam;
  V3<double> f;
  if (!p.iso_act) {
    f = {fib[3 * (size_t)e], fib[3 * (size_t)e + 1], fib[3 * (size_t)e + 2]};
    gam = p.gamma * gscale[e];
  } else {
    afac = 1.0 - p.gamma * gscale[e];
    f = {0.0, 0.0, 1.0};
    gam = 1.0 - 1.0 / (afac * afac * afac);
  }
  const double ia2 = 1.0 / (afac * afac);
  const double phi = dot(f, f);
  const double gamp = gam / (1.0 - gam * phi);
  const double c1 = (2.0 * gamp + gamp * gamp * phi) * ia2;
  /* flat reference triangle area (AreaNormal, io.c:1646-1669) */
  double X[3][3];
  for (int k = 0; k < 3; k++) load_node(m.pos, m.etri[3 * (size_t)e + k], X[k][0], X[k][1], X[k][2]);
  const V3<double> d21 = {X[1][0] - X[0][0], X[1][1] - X[0][1], X[1][2] - X[0][2]};
  const V3<double> d31 = {X[2][0] - X[0][0], X[2][1] - X[0][1], X[2][2] - X[0][2]};
  const V3<double> ca = cross(d21, d31);
  const double dA0 = 0.5 * sqrt(ca.x * ca.x + ca.y * ca.y + ca.z * ca.z);
  const size_t ne = p.ne;
  for (int q = 0; q < p.nq; q++) {
    const double th3 = p.hhalf * p.theta[q];
    const V3<double> g[3] = {a1 + scl(th3, a31), a2 + scl(th3, a32), n};
    double G[3][3], Gi[3][3];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) G[i][j] = dot(g[i], g[j]);
    inv3(G, Gi);
    double t[3], s[3];
    for (int i = 0; i < 3; i++) t[i] = dot(g[i], f);
    for (int i = 0; i < 3; i++) s[i] = Gi[i][0] * t[0] + Gi[i][1] * t[1] + Gi[i][2] * t[2];
    const double omg = 1.0 - gam * phi;
    const double a3 = afac * afac * afac;
    const double rho = 1.0 / (det3(G) * omg * omg * (a3 * a3));
    /* v = Fa_inv.Cov G^-1 e3, w = Fa_inv.Cov G^-1 v, A^T x = G (Fa.Cont x) */
    double u[3] = {Gi[0][2], Gi[1][2], Gi[2][2]};
    double v[3], gv[3], w[3];
    const double tu = t[0] * u[0] + t[1] * u[1] + t[2] * u[2];
    for (int i = 0; i < 3; i++) v[i] = G[i][0] * u[0] + G[i][1] * u[1] + G[i][2] * u[2] + gamp * t[i] * tu;
    for (int i = 0; i < 3; i++) gv[i] = Gi[i][0] * v[0] + Gi[i][1] * v[1] + Gi[i][2] * v[2];
    const double tgv = t[0] * gv[0] + t[1] * gv[1] + t[2] * gv[2];
    for (int i = 0; i < 3; i++) w[i] = G[i][0] * gv[0] + G[i][1] * gv[1] + G[i][2] * gv[2] + gamp * t[i] * tgv;
    auto aT = [&](const double xin[3], double out[3]) {
      double fa[3];
      const double sx = s[0] * xin[0] + s[1] * xin[1] + s[2] * xin[2];
      for (int i = 0; i < 3; i++) fa[i] = Gi[i][0] * xin[0] + Gi[i][1] * xin[1] + Gi[i][2] * xin[2] - gam * s[i] * sx;
      for (int i = 0; i < 3; i++) out[i] = G[i][0] * fa[0] + G[i][1] * fa[1] + G[i][2] * fa[2];
    };
    double av[3], aw[3], ae[3];
    const double e3[3] = {0.0, 0.0, 1.0};
    aT(v, av); aT(w, aw); aT(e3, ae);
    double *o = eref + (size_t)kRefPerQp * q * ne + e;
    o[0] = Gi[0][0] * ia2; o[1 * ne] = Gi[1][1] * ia2; o[2 * ne] = 0.5 * (Gi[0][1] + Gi[1][0]) * ia2;
    o[3 * ne] = Gi[2][2] * ia2;
    for (int k = 0; k < 3; k++) {
      o[(4 + k) * ne] = s[k]; o[(7 + k) * ne] = t[k];
      o[(11 + k) * ne] = av[k]; o[(14 + k) * ne] = aw[k]; o[(17 + k) * ne] = ae[k];
    }
    o[10 * ne] = rho;
  }
  double *o = eref + (size_t)kRefPerQp * p.nq * ne + e;
  o[0] = gam; o[ne] = gamp; o[2 * ne] = c1; o[3 * ne] = 0.5 * (2.0 * p.hhalf) * dA0;
}

/* ---------------- residual element kernel ---------------- */
/* Pressure corner force of element e: each corner receives n P dA / 3 =
   P (x2-x1)x(x3-x1) / 6 (SurfaceNormalPressure, external.c:589-624); the dead
   load takes the same expression on the reference corners
   (SurfaceConstNormalPressure, Nf and dA0 of Init, external.c:699-730). */
__device__ __forceinline__ void elem_pressure_force(const DevMesh &m, const KParams &p, int e)
{
  const size_t ne = p.ne;
  double X[3][3];
  for (int k = 0; k < 3; k++) {
    const size_t c = (size_t)m.etri[3 * (size_t)e + k];
    if (p.pres_dead) { X[k][0] = m.X[3 * c]; X[k][1] = m.X[3 * c + 1]; X[k][2] = m.X[3 * c + 2]; }
    else load_node(m.pos, (int)c, X[k][0], X[k][1], X[k][2]);
  }
  const V3<double> d21 = {X[1][0] - X[0][0], X[1][1] - X[0][1], X[1][2] - X[0][2]};
  const V3<double> d31 = {X[2][0] - X[0][0], X[2][1] - X[0][1], X[2][2] - X[0][2]};
  const V3<double> ca = cross(d21, d31);
  const double nrm = sqrt(ca.x * ca.x + ca.y * ca.y + ca.z * ca.z);
  const double dA = 0.5 * nrm;
  m.fp[e] = (ca.x / nrm) * p.pressure * dA / 3.;
  m.fp[ne + e] = (ca.y / nrm) * p.pressure * dA / 3.;
  m.fp[2 * ne + e] = (ca.z / nrm) * p.pressure * dA / 3.;
}

__global__ void __launch_bounds__(128) k_elem_residual(DevMesh m, KParams p, double *__restrict__ gm_out,
                                                       double *__restrict__ gp_out, double *__restrict__ tape_out)
{
  __shared__ double tabs[kNumTables * 80];
  for (int i = threadIdx.x; i < kNumTables * 80; i += blockDim.x) tabs[i] = m.ntab[i];
  __syncthreads();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ne) return;
  const int info = m.einfo[e];
  const int nen = info & 0xff, tabi = info >> 8;
  const double *tab = tabs + tabi * 80;
  double y[15];
  gather_y(m.pos, m.patch, e, nen, tab, y);
  double f[15];
  int st = 0;
  const EPar<double> ep = epar<double>(p);
  elem_forces<double, double>(y, ep, m.eref + e, p.ne, f, st, gm_out ? gm_out + e : nullptr,
                              tape_out ? tape_out + e : nullptr, gp_out ? gp_out + e : nullptr);
  if (gp_out) elem_geom_store<double>(y, gp_out + e, (size_t)p.ne);   /* the tangent's primal geometry */
  set_status(m.status, st);
  /* Fb_a = sum_r N[r][a] f_r, stored slot-major: fb[(3a+d)*ne + e] */
  const size_t ne = p.ne;
  for (int a = 0; a < nen; a++) {
    double fx = 0.0, fy = 0.0, fz = 0.0;
#pragma unroll
    for (int r = 0; r < 5; r++) {
      const double c = tab[r * 16 + a];
      fx += c * f[3 * r]; fy += c * f[3 * r + 1]; fz += c * f[3 * r + 2];
    }
    m.fb[(3 * a) * ne + e] = fx;
    m.fb[(3 * a + 1) * ne + e] = fy;
    m.fb[(3 * a + 2) * ne + e] = fz;
  }
  if (p.pressure != 0.0) elem_pressure_force(m, p, e);
}

/* ---------------- FP32-bulk residual (float-float) ---------------- */
/* The residual of the FP32-bulk form, on the FP32 pipe with float-float
   numbers (ff.cuh, about 48 significant bits): one thread per element, the
   element math of k_elem_residual.  Plain FP32 does not keep the residual's
   1e-6 budget on these meshes: rounding y = N x alone to FP32 moves R by
   ~1e-6 relative (C1, C2) and the FP32 stress by ~5e-6, so the residual takes
   float-float, whose error sits near 1e-13.  Node positions are taken
   relative to the element's first corner in FP64 before the split, the shift
   is put back through (sum_i N_r[i]) x_c; the element forces leave as
   doubles (hi + lo is exact in FP64) for the FP64 node sums. */
__global__ void __launch_bounds__(128, 3) k_elem_residual_ff(DevMesh m, KParams p)
{
  __shared__ FF tabs[kNumTables * 85];   /* tables, then their row sums */
  const FF *ntab = static_cast<const FF *>(m.ntabFF);
  for (int i = threadIdx.x; i < kNumTables * 85; i += blockDim.x) tabs[i] = ntab[i];
  __syncthreads();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ne) return;
  const int info = m.einfo[e];
  const int nen = info & 0xff, tabi = info >> 8;
  const FF *tab = tabs + tabi * 80, *tsum = tabs + kNumTables * 80 + tabi * 5;
  double xc[3];
  load_node(m.pos, m.etri[3 * (size_t)e], xc[0], xc[1], xc[2]);
  FF y[15];
  {
    const FF c[3] = {ff_split(xc[0]), ff_split(xc[1]), ff_split(xc[2])};
#pragma unroll
    for (int r = 0; r < 5; r++)
#pragma unroll
      for (int d = 0; d < 3; d++) y[3 * r + d] = tsum[r] * c[d];
  }
  const int *pe = m.patch + 16 * (size_t)e;
  for (int i = 0; i < nen; i++) {
    double X, Y, Z;
    load_node(m.pos, __ldg(pe + i), X, Y, Z);
    const FF d[3] = {ff_split(X - xc[0]), ff_split(Y - xc[1]), ff_split(Z - xc[2])};
#pragma unroll
    for (int r = 0; r < 5; r++) {
      const FF c = tab[r * 16 + i];
#pragma unroll
      for (int k = 0; k < 3; k++) y[3 * r + k] = y[3 * r + k] + c * d[k];
    }
  }
  FF f[15];
  int st = 0;
  const EPar<FF> ep = epar<FF>(p);
  elem_forces<FF, FF>(y, ep, static_cast<const FF *>(m.erefFF) + e, p.ne, f, st);
  set_status(m.status, st);
  const size_t ne = p.ne;
  for (int a = 0; a < nen; a++) {
    FF fx = FF(0.f, 0.f), fy = FF(0.f, 0.f), fz = FF(0.f, 0.f);
#pragma unroll
    for (int r = 0; r < 5; r++) {
      const FF c = tab[r * 16 + a];
      fx = fx + c * f[3 * r]; fy = fy + c * f[3 * r + 1]; fz = fz + c * f[3 * r + 2];
    }
    m.fb[(3 * a) * ne + e] = ff_to_double_bits(fx);
    m.fb[(3 * a + 1) * ne + e] = ff_to_double_bits(fy);
    m.fb[(3 * a + 2) * ne + e] = ff_to_double_bits(fz);
  }
  if (p.pressure != 0.0) elem_pressure_force(m, p, e);
}

__global__ void k_to_ff(const double *__restrict__ a, FF *__restrict__ b, long long n)
{
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) b[t] = FF(a[t]);
}

/* ---------------- tangent element kernel ---------------- */
constexpr int kTanElemsPerCta = 8;   /* 16 lanes per element, 128 threads */

/* The pressure block vectors of one element (follower-pressure load
   stiffness): every corner carries P/6 (x2-x1)x(x3-x1), so d/dx1 = [b-a]x,
   d/dx2 = -[b]x, d/dx3 = [a]x with a = x2-x1, b = x3-x1; stored after D in
   the element's block for the row assembly. */
template <class R>
__device__ __forceinline__ void store_pressure_vectors(const R av[3], const R bv[3], R *dst)
{
#pragma unroll
  for (int d = 0; d < 3; d++) {
    dst[d] = bv[d] - av[d];
    dst[3 + d] = -bv[d];
    dst[6 + d] = av[d];
  }
}

__global__ void __launch_bounds__(128, 3) k_elem_tangent(DevMesh m, KParams p)
{
  __shared__ double tabs[kNumTables * 80];
  __shared__ double Jsh[kTanElemsPerCta][kMaxQp * 21]; /* constitutive derivatives per thickness point */
  for (int i = threadIdx.x; i < kNumTables * 80; i += blockDim.x) tabs[i] = m.ntab[i];
  __syncthreads();
  const int lane = threadIdx.x & 15;
  const int slot = threadIdx.x >> 4;
  const int e = blockIdx.x * kTanElemsPerCta + slot;
  const bool live = e < p.ne;
  const int ee = live ? e : p.ne - 1;
  const int info = m.einfo[ee];
  const int nen = info & 0xff, tabi = info >> 8;
  const double *tab = tabs + tabi * 80;
  double y[15];
  gather_y_group(m.pos, m.patch, ee, nen, tab, lane, y);
  double fd[15];
  const EPar<double> ep = epar<double>(p);
  /* the thickness-point metrics, the primal geometry and resultants and the
     primal C33 sub-iteration values come from k_elem_residual, launched
     before this kernel (which also performs the CC3333 checks) */
  elem_forces_split_tl<double>(y, ep, m.eref + ee, p.ne, m.gpr + ee, lane, Jsh[slot], fd, m.gmq + ee, m.gtape + ee);
  if (!live) return;
  /* column `lane` of D = df/dy, row-major in the element's block */
  double *De = m.De + (size_t)kDeStride * e;
  if (lane < 15) {
#pragma unroll
    for (int r = 0; r < 15; r++) De[r * 15 + lane] = fd[r];
  } else if (p.pressure != 0.0 && !p.pres_dead) {
    double X[3][3];
    for (int k = 0; k < 3; k++) load_node(m.pos, m.etri[3 * (size_t)e + k], X[k][0], X[k][1], X[k][2]);
    const double av[3] = {X[1][0] - X[0][0], X[1][1] - X[0][1], X[1][2] - X[0][2]};
    const double bv[3] = {X[2][0] - X[0][0], X[2][1] - X[0][1], X[2][2] - X[0][2]};
    store_pressure_vectors<double>(av, bv, De + kDePres);
  }
}

/* ---------------- FP32-bulk tangent ---------------- */
/* Same element math as k_elem_tangent in single precision.  Node positions
   are shifted to the element's first corner in FP64 (one node per lane, then
   shared by shuffles) and rounded to FP32, so the FP32 values carry the
   element-size digits; the shift is put back through (sum_i N_r[i]) * x_c,
   which is not zero for the truncated second-derivative rows (their rows sum
   to -1e-4 / -1e-4 / +2e-4).  D = df/dy is written in FP32 for the row assembly. */
__global__ void __launch_bounds__(128, 5) k_elem_tangent_f32(DevMesh m, KParams p)
{
  __shared__ float tabs[kNumTables * 80];
  __shared__ float tsum[kNumTables * 5];
  __shared__ float JshF[kTanElemsPerCta][kMaxQp * 21];
  for (int i = threadIdx.x; i < kNumTables * 85; i += blockDim.x) {
    if (i < kNumTables * 80) tabs[i] = m.ntabF[i]; else tsum[i - kNumTables * 80] = m.ntabF[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 15;
  const int slot = threadIdx.x >> 4;
  const int e = blockIdx.x * kTanElemsPerCta + slot;
  const bool live = e < p.ne;
  const int ee = live ? e : p.ne - 1;
  const int info = m.einfo[ee];
  const int nen = info & 0xff, tabi = info >> 8;
  const float *tab = tabs + tabi * 80;
  /* shifted coordinates: lane i < nen owns patch node i */
  const int c0 = m.etri[3 * (size_t)ee];
  double xc, yc, zc;
  load_node(m.pos, c0, xc, yc, zc);
  float dx = 0.f, dy = 0.f, dz = 0.f;
  if (lane < nen) {
    const int node = m.patch[16 * (size_t)ee + lane];
    double X, Y, Z;
    load_node(m.pos, node, X, Y, Z);
    dx = (float)(X - xc); dy = (float)(Y - yc); dz = (float)(Z - zc);
  }
  float y[15];
#pragma unroll
  for (int r = 0; r < 5; r++) {
    const float sr = tsum[tabi * 5 + r];
    y[3 * r] = sr * (float)xc; y[3 * r + 1] = sr * (float)yc; y[3 * r + 2] = sr * (float)zc;
  }
  const unsigned hmask = 0xffffffffu;
  for (int i = 0; i < 16; i++) {
    const float ax = __shfl_sync(hmask, dx, i, 16), ay = __shfl_sync(hmask, dy, i, 16), az = __shfl_sync(hmask, dz, i, 16);
    if (i < nen) {
#pragma unroll
      for (int r = 0; r < 5; r++) {
        const float c = tab[r * 16 + i];
        y[3 * r] = fmaf(c, ax, y[3 * r]); y[3 * r + 1] = fmaf(c, ay, y[3 * r + 1]); y[3 * r + 2] = fmaf(c, az, y[3 * r + 2]);
      }
    }
  }
  D1f fd[15];
  int st = 0;
  const EPar<float> ep = epar<float>(p);
  elem_forces_split<float>(y, ep, m.erefF + ee, p.ne, lane, JshF[slot], fd, st);
  if (live) set_status(m.status, st);
  /* pressure vectors from the shifted corner coordinates */
  const int cs = m.ecorner[ee];
  const int cslot[3] = {cs & 31, (cs >> 5) & 31, (cs >> 10) & 31};
  float xk[3][3];
  for (int k = 0; k < 3; k++) {
    xk[k][0] = __shfl_sync(hmask, dx, cslot[k], 16);
    xk[k][1] = __shfl_sync(hmask, dy, cslot[k], 16);
    xk[k][2] = __shfl_sync(hmask, dz, cslot[k], 16);
  }
  if (!live) return;
  float *De = m.DeF + (size_t)kDeStride * e;
  if (lane < 15) {
#pragma unroll
    for (int r = 0; r < 15; r++) De[r * 15 + lane] = fd[r].d;
  } else if (p.pres6f != 0.f && !p.pres_dead) {
    const float av[3] = {xk[1][0] - xk[0][0], xk[1][1] - xk[0][1], xk[1][2] - xk[0][2]};
    const float bv[3] = {xk[2][0] - xk[0][0], xk[2][1] - xk[0][1], xk[2][2] - xk[0][2]};
    store_pressure_vectors<float>(av, bv, De + kDePres);
  }
}

/* ---------------- node gather (residual assembly) ---------------- */
__device__ __forceinline__ unsigned long long abs_bits(double v)
{
  return (unsigned long long)__double_as_longlong(fabs(v));
}

__global__ void k_node_gather(DevMesh m, KParams p, const double *__restrict__ x, double *__restrict__ R,
                              double *__restrict__ parts)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long lmax = 0ull;
  if (i < p.nt) {
    const size_t ne = p.ne;
    double fi[3] = {0.0, 0.0, 0.0}, fe[3] = {0.0, 0.0, 0.0};
    for (int c = m.rptr[i]; c < m.rptr[i + 1]; c++) {
      const size_t base = (size_t)m.ridx[c];   /* 3*slot*ne + e */
      fi[0] += m.fb[base]; fi[1] += m.fb[base + ne]; fi[2] += m.fb[base + 2 * ne];
    }
    if (p.pressure != 0.0)
      for (int c = m.pptr[i]; c < m.pptr[i + 1]; c++) {
        const size_t e = (size_t)m.pidx[c];
        fe[0] += m.fp[e]; fe[1] += m.fp[ne + e]; fe[2] += m.fp[2 * ne + e];
      }
    const int kind = m.rowkind[i];
    /* FDynamic (main.c:1178-1270, the path of an active-strain run):
       triangle-order sum of the node's inertial (and damping) force over the
       real triangles with this corner */
    double fd[3] = {0.0, 0.0, 0.0};
    if (p.dyn && (kind == 0 || (parts && i < p.nv))) {
      for (int c = m.dptr[i]; c < m.dptr[i + 1]; c++) {
        const double M = p.dyn_rhoh0 * m.dA0[m.didx[c]] / 3;
        const double C = p.dyn_damp ? p.dyn_dampf * M : 0.0;
        for (int d = 0; d < 3; d++) {
          const size_t o = 3 * (size_t)i + d;
          double f;
          if (!p.dyn_central) {
            const double facc = M * (p.dyn_M1 * m.xn[o] + p.dyn_M2 * m.xd[o] + p.dyn_M3 * m.xdd[o]);
            const double fvel = C * (p.dyn_C1 * m.xn[o] + p.dyn_C2 * m.xd[o] + p.dyn_C3 * m.xdd[o]);
            f = M * p.dyn_M1 * x[o] + C * p.dyn_C1 * x[o] - facc - fvel;
          } else {
            f = M * (x[o] - 2 * m.xn[o] + m.xnm1[o]) / (p.dyn_dt * p.dyn_dt) + C * (x[o] - m.xn[o]) / p.dyn_dt;
          }
          fd[d] += f;
        }
      }
    }
    for (int d = 0; d < 3; d++) {
      double r;
      if (kind == 2) r = 0.0;
      else if (kind == 1) r = x[3 * (size_t)i + d] - m.X[3 * (size_t)i + d];
      else if (p.dyn) r = (-1.0 * fe[d] + fi[d]) + 1. * fd[d];
      else r = -1.0 * fe[d] + fi[d];
      R[3 * (size_t)i + d] = r;
      if (parts) {   /* unscaled Fint, Fext, Fdyn of the real nodes (ghost entries 0) */
        const size_t n3 = 3 * (size_t)p.nt, o = 3 * (size_t)i + d;
        const bool real = i < p.nv;
        parts[o] = real ? fi[d] : 0.0;
        parts[n3 + o] = real ? fe[d] : 0.0;
        parts[2 * n3 + o] = real ? fd[d] : 0.0;
      }
      const unsigned long long b = abs_bits(fe[d]);
      lmax = b > lmax ? b : lmax;
    }
  }
  /* warp max then one atomic per warp */
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_down_sync(0xffffffffu, lmax, o);
    lmax = v > lmax ? v : lmax;
  }
  if ((threadIdx.x & 31) == 0 && lmax) atomicMax(m.fmax, lmax);
}

/* ---------------- row assembly (tangent) ---------------- */
/* One warp per row node i.  For every element e whose patch holds i at slot a
   (the row's contribution list, element order) and every slot b of that
   patch, K_ib += (N[:,a] (x) I3)^T D_e (N[:,b] (x) I3), with D_e = df/dy the
   element kernel stored, plus the follower-pressure block when a and b are
   corner slots; a ghost slot b adds to the blocks of its parents with signs
   +, +, - (x_g = x_nv2 + x_nv1 - x_nv3).  The row's blocks accumulate in
   shared memory in a fixed order (contributions in element order; within an
   element the real slots, then the ghost slots in slot order), so K is
   deterministic; FP32 sums are compensated (Kahan).  Clamped and ghost rows
   are identity rows.  K is scaled by 1/max(|Fext|_inf, 1) as it is written
   (main.c:1020-1026; k_node_gather, launched before, found the max); with
   colmajor each 3x3 block is stored column by column. */
constexpr int kRowWarps = 4;
constexpr int kRowChunk = 4;          /* contributions whose slots and w are formed together */

__device__ __forceinline__ int row_find(const int *cols, int nb, int node)
{
  int lo = 0, hi = nb - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cols[mid] < node) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__host__ __device__ __forceinline__ size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

/* one warp's shared buffers; every part starts on 16 bytes */
template <class R> struct RowAsmBuf {
  R *acc, *comp;      /* the row's 9 nb block values (and their compensations, FP32) */
  R *wT;              /* kRowChunk x 9 x 8: w of each contribution of the chunk */
  R *gv;              /* 9 x 16 values of the ghost slots of one contribution */
  int *cols;          /* the row's block columns */
  int *rec;           /* kRowChunk row-assembly records (kRowRec ints each) */
};

__host__ __device__ __forceinline__ size_t row_buf_bytes(int maxblk, size_t rsize)
{
  const size_t nacc = 9 * (size_t)maxblk * (rsize == 4 ? 2 : 1);
  return align16(nacc * rsize) + kRowChunk * 9 * kRowPad * rsize + 144 * rsize + align16(4 * (size_t)maxblk) +
         kRowChunk * kRowRec * 4;
}

template <class R>
__device__ __forceinline__ RowAsmBuf<R> row_buf(unsigned char *base, int maxblk)
{
  RowAsmBuf<R> b;
  const size_t nacc = 9 * (size_t)maxblk;
  b.acc = reinterpret_cast<R *>(base);
  b.comp = b.acc + nacc;
  unsigned char *q = base + align16(nacc * (sizeof(R) == 4 ? 2 : 1) * sizeof(R));
  b.wT = reinterpret_cast<R *>(q);
  q += kRowChunk * 9 * kRowPad * sizeof(R);
  b.gv = reinterpret_cast<R *>(q);
  q += 144 * sizeof(R);
  b.cols = reinterpret_cast<int *>(q);
  q += align16(4 * (size_t)maxblk);
  b.rec = reinterpret_cast<int *>(q);
  return b;
}

/* The records of the contributions [cb, cb + CH) of a row ending at c1, one
   16-byte piece per lane (lanes < 5 np); zero past the row. */
template <int CH>
__device__ __forceinline__ int4 row_rec_load(const int *rrec, int cb, int c1, int lane)
{
  static_assert(kRowRec % 4 == 0 && (kRowRec / 4) * CH <= 32, "a chunk's records must fit one piece per lane");
  const int np = min(CH, c1 - cb);
  if (np <= 0 || lane >= (kRowRec / 4) * np) return make_int4(0, 0, 0, 0);
  return __ldg(reinterpret_cast<const int4 *>(rrec) + (size_t)(kRowRec / 4) * cb + lane);
}

template <class R>
__device__ __forceinline__ void row_add(R *acc, R *comp, int idx, R v)
{
  if constexpr (sizeof(R) == 4) {
    const R s = acc[idx], yv = v - comp[idx];
    const R t = s + yv;
    comp[idx] = (t - s) - yv;
    acc[idx] = t;
  } else {
    acc[idx] += v;
  }
}

/* The row's contributions are taken kRowChunk at a time: one pass forms the
   slot targets of all their patch slots (a binary search in the row's block
   columns; a ghost slot packs its three parents' targets), one pass forms
   all their w (45 values each, so the chunk's D loads are in flight
   together), then the contributions are added one after another in element
   order: lane t of 9 nen takes block b = t / 9, entry q = t % 9.  FP64
   values are fused into the block accumulator (acc + sum_s N[s][b] wT[q][s]
   as one FMA chain), FP32 values are formed alone and added with Kahan
   compensation; a ghost slot's values go to its parents after the real
   slots, in slot order, and so do a repeated real node's (a patch at an open
   boundary that is no ring holds some node twice: kRowSlotDup, one target),
   so that no two lanes add into one block at once. */
template <class R>
__global__ void __launch_bounds__(32 * kRowWarps) k_row_assemble(DevMesh m, KParams p, const R *__restrict__ De,
                                                                 const R *__restrict__ ntab, R psc, R *__restrict__ K,
                                                                 int maxblk, int colmajor)
{
  extern __shared__ __align__(16) unsigned char row_smem[];
  R *tabsT = reinterpret_cast<R *>(row_smem);       /* m.ntabs x 16 x 8: N[s][b] at 8 b + s */
  for (int t = threadIdx.x; t < m.ntabs * 16 * kRowPad; t += blockDim.x) {
    const int tb = t / (16 * kRowPad), r = t - tb * 16 * kRowPad, b = r / kRowPad, sidx = r - b * kRowPad;
    tabsT[t] = sidx < 5 ? ntab[tb * 80 + sidx * 16 + b] : R(0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int i = blockIdx.x * kRowWarps + wid;
  if (i >= p.nt) return;
  RowAsmBuf<R> B = row_buf<R>(row_smem + align16(m.ntabs * 16 * kRowPad * sizeof(R)) +
                              (size_t)wid * row_buf_bytes(maxblk, sizeof(R)), maxblk);
  const int k0 = m.rowptr[i], nb = m.rowptr[i + 1] - k0;
  const int kind = m.rowkind[i];
  R *Kr = K + 9 * (size_t)k0;
  if (kind != 0) {   /* clamped (R = x - X) and ghost (R = 0) rows: identity */
    for (int t = lane; t < 9 * nb; t += 32) {
      const int q = t % 9;
      Kr[t] = (m.colind[k0 + t / 9] == i && (q == 0 || q == 4 || q == 8)) ? R(1) : R(0);
    }
    return;
  }
  for (int t = lane; t < nb; t += 32) B.cols[t] = m.colind[k0 + t];
  for (int t = lane; t < 9 * nb; t += 32) {
    B.acc[t] = R(0);
    if constexpr (sizeof(R) == 4) B.comp[t] = R(0);
  }
  const bool pres_live = p.pressure != 0.0 && !p.pres_dead;
  const int c1 = m.rptr[i + 1];
  int4 nrec = row_rec_load<kRowChunk>(m.rrec, m.rptr[i], c1, lane);
  for (int cb = m.rptr[i]; cb < c1; cb += kRowChunk) {
    const int np = min(kRowChunk, c1 - cb);
    if (lane < (kRowRec / 4) * np) reinterpret_cast<int4 *>(B.rec)[lane] = nrec;
    nrec = row_rec_load<kRowChunk>(m.rrec, cb + kRowChunk, c1, lane);   /* the next chunk's, in flight meanwhile */
    __syncwarp();   /* also orders the cols / acc set-up and the previous chunk's reads */
    /* w of the chunk: lane u -> contribution u / 45, entry u % 45 */
    for (int u = lane; u < 45 * np; u += 32) {
      const int pc = u / 45, t = u - 45 * pc;
      const int *rc = B.rec + kRowRec * pc;
      const int e = rc[0] & ((1 << 27) - 1), a = rc[0] >> 27, info = rc[1];
      int pos;
      const R v = row_wt_entry(De + (size_t)kDeStride * e, tabsT + (info >> 8) * 16 * kRowPad + kRowPad * a, t, &pos);
      B.wT[9 * kRowPad * pc + pos] = v;
    }
    __syncwarp();
    for (int pc = 0; pc < np; pc++) {
      const int *rc = B.rec + kRowRec * pc;
      const int e = rc[0] & ((1 << 27) - 1), a = rc[0] >> 27, info = rc[1], cs = rc[2];
      const int nen = info & 0xff;
      const R *tabT = tabsT + (info >> 8) * 16 * kRowPad;
      const R *wT = B.wT + 9 * kRowPad * pc;
      const unsigned *slot = reinterpret_cast<const unsigned *>(rc + 4);
      const int cslot0 = cs & 31, cslot1 = (cs >> 5) & 31, cslot2 = (cs >> 10) & 31;
      const bool acorner = pres_live && (a == cslot0 || a == cslot1 || a == cslot2);
      const bool ghost_lane = lane < nen && (slot[lane] & kRowSlotGhost);
      const unsigned gmask = __ballot_sync(0xffffffffu, ghost_lane);
      for (int t = lane; t < 9 * nen; t += 32) {
        const int b = t / 9, q = t - 9 * b;
        const unsigned sl = slot[b];
        const bool ghost = (sl & kRowSlotGhost) != 0;
        const int idx = 9 * (int)(sl & 1023u) + q;
        R v;
        if constexpr (sizeof(R) == 8) v = row_block_accum(wT + kRowPad * q, tabT + kRowPad * b, ghost ? R(0) : B.acc[idx]);
        else v = row_block_accum(wT + kRowPad * q, tabT + kRowPad * b, R(0));
        if (acorner) {
          const int kc = b == cslot0 ? 0 : (b == cslot1 ? 1 : (b == cslot2 ? 2 : -1));
          if (kc >= 0) v += skew_entry(q / 3, q % 3, De + (size_t)kDeStride * e + kDePres + 3 * kc, psc);
        }
        if (ghost) B.gv[t] = v;
        else if constexpr (sizeof(R) == 8) B.acc[idx] = v;
        else row_add(B.acc, B.comp, idx, v);
      }
      if (gmask) {
        __syncwarp();
        /* ghost slots, in slot order: lane 9k + q adds to entry q of parent k */
        for (unsigned gm = gmask; gm; gm &= gm - 1) {
          const int b = __ffs(gm) - 1;
          if (lane < ((slot[b] & kRowSlotDup) ? 9 : 27)) {   /* a repeated real node has one target */
            const int k = lane / 9, q = lane - 9 * k;
            const int pos = (int)((slot[b] >> (10 * k)) & 1023u);
            const R v = B.gv[9 * b + q];
            row_add(B.acc, B.comp, 9 * pos + q, k == 2 ? -v : v);
          }
          __syncwarp();
        }
      }
      __syncwarp();
    }
  }
  __syncwarp();
  /* dynamic term diagonal, scale, write-out */
  const double fmax = __longlong_as_double((long long)*m.fmax);
  const R sc = fmax > 1.0 ? R(1.0 / fmax) : R(1);
  const int pd = row_find(B.cols, nb, i);
  for (int t = lane; t < 9 * nb; t += 32) {
    R v = B.acc[t];
    const int q = t % 9;
    if (p.dyn && t / 9 == pd && (q == 0 || q == 4 || q == 8)) v += R(m.dyn_diag[i]);
    if (fmax > 1.0) {
      if constexpr (sizeof(R) == 4) v = (R)((double)v * (1.0 / fmax)); else v = v * sc;
    }
    Kr[colmajor ? t - q + 3 * (q % 3) + q / 3 : t] = v;
  }
}

/* FP32 row assembly with the row's blocks owned by lanes: lane k owns block k
   of the row in registers (9 values) and, in rows of more than 32 blocks
   (most interior rows: 36 on average in a regular mesh), block 32 + k in
   shared memory.  One pass over the row's contributions, kRowChunk at a
   time: slot targets and an inverse map (owned block -> real patch slot) in
   shared memory, then w of each contribution (lane t and t + 32 of its 45
   entries), then each owned block's values formed by its owner lane (N[.][b]
   from the table, the 9 x 5 values of w read by every lane at once) and fused
   into a per-chunk partial sum; a ghost slot's values go to the lanes owning
   its parents, after the real slots, in slot order, and so do those of a
   slot repeating an earlier slot's real node (kRowSlotDup, one owner).  The partial sums are
   added into the row with Kahan compensation once per chunk, in element
   order; the second 32 blocks' pass is skipped for a chunk that touches none
   of them. */
constexpr int kRowRegMax = 64;

struct RowRegBuf {
  float *wT;          /* kRowChunk x 9 x 8 */
  float *acc1;        /* 32 x 9 values of the owned blocks 32..63 ([lane][q]); the write-out staging */
  float *comp;        /* 9 x 32 Kahan compensations of the owned blocks 0..31 ([q][lane]) */
  float *comp1;       /* 32 x 9 compensations of the owned blocks 32..63 ([lane][q]) */
  int *cols;          /* kRowRegMax */
  int *rec;           /* kRowChunk row-assembly records */
  unsigned char *inv; /* kRowChunk x 64: real slot of each owned block, 255 none */
};

__host__ __device__ __forceinline__ size_t row_reg_bytes()
{
  return kRowChunk * 9 * kRowPad * 4 + 3 * 9 * 32 * 4 + kRowRegMax * 4 + kRowChunk * kRowRec * 4 + kRowChunk * 64;
}

__device__ __forceinline__ RowRegBuf row_reg_buf(unsigned char *q)
{
  RowRegBuf b;
  b.wT = reinterpret_cast<float *>(q);
  q += kRowChunk * 9 * kRowPad * 4;
  b.acc1 = reinterpret_cast<float *>(q);
  q += 9 * 32 * 4;
  b.comp = reinterpret_cast<float *>(q);
  q += 9 * 32 * 4;
  b.comp1 = reinterpret_cast<float *>(q);
  q += 9 * 32 * 4;
  b.cols = reinterpret_cast<int *>(q);
  q += kRowRegMax * 4;
  b.rec = reinterpret_cast<int *>(q);
  q += kRowChunk * kRowRec * 4;
  b.inv = q;
  return b;
}

/* tmp[q] += sum_s N[s] wT[8 q + s] for the nine entries of one block */
__device__ __forceinline__ void row_reg_block(const float *wT, const float n[5], float tmp[9])
{
#pragma unroll
  for (int q = 0; q < 9; q++) tmp[q] = row_block_accum(wT + kRowPad * q, n, tmp[q]);
}

/* The chunk's contributions to owned block k (k = lane or 32 + lane, inverse
   map column kc) added into tmp: the real slot mapped to k (with its
   follower-pressure term), then the ghost slots whose parents include k. */
__device__ __forceinline__ void row_reg_chunk(const RowRegBuf &B, const float *tabsT, const float *De, float psc,
                                              bool pres_live, int np, int lane, int k, int kc, float tmp[9])
{
  for (int pc = 0; pc < np; pc++) {
    const int *rc = B.rec + kRowRec * pc;
    const int a = rc[0] >> 27, info = rc[1], cs = rc[2];
    const int nen = info & 0xff;
    const float *tabT = tabsT + (info >> 8) * 16 * kRowPad;
    const float *wT = B.wT + 9 * kRowPad * pc;
    const unsigned *slot = reinterpret_cast<const unsigned *>(rc + 4);
    const int b = B.inv[64 * pc + kc];
    if (b != 255) {
      float n[5];
      load5(tabT + kRowPad * b, n);
      row_reg_block(wT, n, tmp);
      const int cslot0 = cs & 31, cslot1 = (cs >> 5) & 31, cslot2 = (cs >> 10) & 31;
      if (pres_live && (a == cslot0 || a == cslot1 || a == cslot2)) {
        const int kcr = b == cslot0 ? 0 : (b == cslot1 ? 1 : (b == cslot2 ? 2 : -1));
        if (kcr >= 0) {
          const float *vv = De + (size_t)kDeStride * (rc[0] & ((1 << 27) - 1)) + kDePres + 3 * kcr;
#pragma unroll
          for (int q = 0; q < 9; q++) tmp[q] += skew_entry(q / 3, q % 3, vv, psc);
        }
      }
    }
    /* ghost slots, in slot order: the owners of the three parents add +, +, - */
    const bool ghost_lane = lane < nen && (slot[lane] & kRowSlotGhost);
    for (unsigned gm = __ballot_sync(0xffffffffu, ghost_lane); gm; gm &= gm - 1) {
      const int gb = __ffs(gm) - 1;
      const unsigned sl = slot[gb];
      const int pos0 = (int)(sl & 1023u), pos1 = (int)((sl >> 10) & 1023u), pos2 = (int)((sl >> 20) & 1023u);
      if (k == pos0 || k == pos1 || k == pos2) {   /* a repeated real node: pos0 = pos1, pos2 none */
        float n[5], v[9];
        load5(tabT + kRowPad * gb, n);
#pragma unroll
        for (int q = 0; q < 9; q++) v[q] = 0.f;
        row_reg_block(wT, n, v);
        const float sg = k == pos2 ? -1.f : 1.f;
#pragma unroll
        for (int q = 0; q < 9; q++) tmp[q] = fmaf(sg, v[q], tmp[q]);
      }
    }
  }
}

__global__ void __launch_bounds__(32 * kRowWarps, 8) k_row_assemble_f32(DevMesh m, KParams p, const float *__restrict__ De,
                                                                     const float *__restrict__ ntab, float psc,
                                                                     float *__restrict__ K, int colmajor)
{
  extern __shared__ __align__(16) unsigned char row_smem[];
  float *tabsT = reinterpret_cast<float *>(row_smem);
  for (int t = threadIdx.x; t < m.ntabs * 16 * kRowPad; t += blockDim.x) {
    const int tb = t / (16 * kRowPad), r = t - tb * 16 * kRowPad, b = r / kRowPad, sidx = r - b * kRowPad;
    tabsT[t] = sidx < 5 ? ntab[tb * 80 + sidx * 16 + b] : 0.f;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int i = blockIdx.x * kRowWarps + wid;
  if (i >= p.nt) return;
  RowRegBuf B = row_reg_buf(row_smem + align16(m.ntabs * 16 * kRowPad * 4) + (size_t)wid * row_reg_bytes());
  const int k0 = m.rowptr[i], nb = m.rowptr[i + 1] - k0;
  float *Kr = K + 9 * (size_t)k0;
  if (m.rowkind[i] != 0) {   /* clamped and ghost rows: identity */
    for (int t = lane; t < 9 * nb; t += 32) {
      const int q = t % 9;
      Kr[t] = (m.colind[k0 + t / 9] == i && (q == 0 || q == 4 || q == 8)) ? 1.f : 0.f;
    }
    return;
  }
  for (int t = lane; t < nb; t += 32) B.cols[t] = m.colind[k0 + t];
  /* the two w entries of this lane: t0 = lane, t1 = lane + 32 (< 45) */
  const int wi0 = lane / 15, wk0 = lane - 15 * wi0;
  const int wpos0 = kRowPad * (3 * wi0 + wk0 % 3) + wk0 / 3, wd0 = wi0 * 15 + wk0;
  const int t1 = lane + 32, wi1 = t1 / 15, wk1 = t1 - 15 * wi1;
  const int wpos1 = kRowPad * (3 * wi1 + wk1 % 3) + wk1 / 3, wd1 = wi1 * 15 + wk1;
  const bool has1 = t1 < 45;
  const bool pres_live = p.pressure != 0.0 && !p.pres_dead;
  const bool two = nb > 32;
  const double fmax = __longlong_as_double((long long)*m.fmax);
  float acc[9], tmp[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    acc[q] = 0.f;
    B.comp[32 * q + lane] = 0.f;
    B.acc1[9 * lane + q] = 0.f;
    B.comp1[9 * lane + q] = 0.f;
  }
  __syncwarp();
  const int pd = row_find(B.cols, nb, i);
  const int c1 = m.rptr[i + 1];
  int4 nrec = row_rec_load<kRowChunk>(m.rrec, m.rptr[i], c1, lane);
  for (int cb = m.rptr[i]; cb < c1; cb += kRowChunk) {
    const int np = min(kRowChunk, c1 - cb);
    if (lane < (kRowRec / 4) * np) reinterpret_cast<int4 *>(B.rec)[lane] = nrec;
    nrec = row_rec_load<kRowChunk>(m.rrec, cb + kRowChunk, c1, lane);   /* the next chunk's, in flight meanwhile */
    for (int u = lane; u < kRowChunk * 16; u += 32) reinterpret_cast<unsigned *>(B.inv)[u] = 0xffffffffu;
    __syncwarp();
    /* inverse map: owned block -> real slot (lane u -> contribution u / 16, slot u % 16);
       hi: the chunk reaches a block from 32 on (a real slot or a ghost's parent) */
    bool hi = false;
    for (int u = lane; u < 16 * np; u += 32) {
      const int pc = u >> 4, b = u & 15;
      const int *rc = B.rec + kRowRec * pc;
      const unsigned sl = (unsigned)rc[4 + b];
      if (b < (rc[1] & 0xff)) {
        if (!(sl & kRowSlotGhost)) {
          B.inv[64 * pc + sl] = (unsigned char)b;
          hi |= sl >= 32u;
        } else {
          hi |= (sl & 1023u) >= 32u ||
                (!(sl & kRowSlotDup) && (((sl >> 10) & 1023u) >= 32u || ((sl >> 20) & 1023u) >= 32u));
        }
      }
    }
    hi = __any_sync(0xffffffffu, hi);
    for (int pc = 0; pc < np; pc++) {
      const int *rc = B.rec + kRowRec * pc;
      const int e = rc[0] & ((1 << 27) - 1), a = rc[0] >> 27, info = rc[1];
      const float *D = De + (size_t)kDeStride * e;
      float n[5];
      load5(tabsT + (info >> 8) * 16 * kRowPad + kRowPad * a, n);
      float v0 = 0.f, v1 = 0.f;
#pragma unroll
      for (int r = 0; r < 5; r++) v0 = fmaf(n[r], __ldg(D + 45 * r + wd0), v0);
      B.wT[9 * kRowPad * pc + wpos0] = v0;
      if (has1) {
#pragma unroll
        for (int r = 0; r < 5; r++) v1 = fmaf(n[r], __ldg(D + 45 * r + wd1), v1);
        B.wT[9 * kRowPad * pc + wpos1] = v1;
      }
    }
    __syncwarp();
    /* h = 0: blocks 0..31, compensated into acc (registers); h = 1: blocks
       32..63, into acc1 (each lane's own shared-memory column) */
    for (int h = 0; h < (hi ? 2 : 1); h++) {
#pragma unroll
      for (int q = 0; q < 9; q++) tmp[q] = 0.f;
      row_reg_chunk(B, tabsT, De, psc, pres_live, np, lane, 32 * h + lane, 32 * h + lane, tmp);
      if (h == 0) {
#pragma unroll
        for (int q = 0; q < 9; q++) {
          const float y = tmp[q] - B.comp[32 * q + lane];
          const float t = acc[q] + y;
          B.comp[32 * q + lane] = (t - acc[q]) - y;
          acc[q] = t;
        }
      } else {
#pragma unroll
        for (int q = 0; q < 9; q++) {
          const float s = B.acc1[9 * lane + q];
          const float y = tmp[q] - B.comp1[9 * lane + q];
          const float t = s + y;
          B.comp1[9 * lane + q] = (t - s) - y;
          B.acc1[9 * lane + q] = t;
        }
      }
    }
    __syncwarp();   /* records, inverse map and wT are rewritten by the next chunk */
  }
  /* dynamic term diagonal, scale, block layout; blocks 32.. are written first
     (from acc1, in place), then acc1 stages blocks 0..31 */
  auto finish = [&](float v, int k, int q) {
    if (p.dyn && k == pd && (q == 0 || q == 4 || q == 8)) v += (float)m.dyn_diag[i];
    if (fmax > 1.0) v = (float)((double)v * (1.0 / fmax));
    return v;
  };
  if (two) {
    if (32 + lane < nb) {
      float v[9];
#pragma unroll
      for (int q = 0; q < 9; q++) v[q] = finish(B.acc1[9 * lane + q], 32 + lane, q);
#pragma unroll
      for (int q = 0; q < 9; q++) B.acc1[9 * lane + (colmajor ? 3 * (q % 3) + q / 3 : q)] = v[q];
    }
    __syncwarp();
    for (int t = lane; t < 9 * (nb - 32); t += 32) Kr[9 * 32 + t] = B.acc1[t];
    __syncwarp();
  }
  if (lane < nb) {
#pragma unroll
    for (int q = 0; q < 9; q++) B.acc1[9 * lane + (colmajor ? 3 * (q % 3) + q / 3 : q)] = finish(acc[q], lane, q);
  }
  __syncwarp();
  const int nw = 9 * min(32, nb);
  for (int t = lane; t < nw; t += 32) Kr[t] = B.acc1[t];
}

/* Row-assembly records (see DevMesh::rrec), built on the device once per
   mesh: one warp per row, lanes over (contribution, patch slot); the slot's
   target is its node's position in the row's sorted columns (a lower-bound
   search), a ghost slot packs its parents nv2, nv1, nv3 at 10 bits each with
   kRowSlotGhost, and a slot repeating an earlier slot's real node is marked
   kRowSlotGhost | kRowSlotDup with its one target (it then takes the ghost
   slots' serial path).  Rows with an identity block get zero records. */
__device__ __forceinline__ unsigned col_lower_bound(const int *cols, int nb, int node)
{
  int lo = 0, hi = nb;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cols[mid] < node) lo = mid + 1; else hi = mid;
  }
  return (unsigned)lo;
}

__global__ void k_row_records(DevMesh m, KParams p, int *__restrict__ rrec)
{
  const int lane = threadIdx.x & 31;
  const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (i >= p.nt) return;
  const int c0 = m.rptr[i], c1 = m.rptr[i + 1];
  const bool live = m.rowkind[i] == 0;
  const int k0 = m.rowptr[i], nb = m.rowptr[i + 1] - k0;
  const int *cols = m.colind + k0;
  for (int u = lane; u < 16 * (c1 - c0); u += 32) {
    const int c = c0 + (u >> 4), b = u & 15;
    int *r = rrec + (size_t)kRowRec * c;
    const int code = m.ridx[c];                  /* 3 a ne + e */
    const int e = code % p.ne, a = code / (3 * p.ne);
    const int info = m.einfo[e], nen = info & 0xff;
    if (b == 0) {
      r[0] = live ? (e | (a << 27)) : 0;
      r[1] = live ? info : 0;
      r[2] = live ? m.ecorner[e] : 0;
      r[3] = 0;
    }
    unsigned sl = 0;
    if (live && b < nen) {
      const int *pe = m.patch + 16 * (size_t)e;
      const int node = pe[b];
      if (node < p.nv) {
        sl = col_lower_bound(cols, nb, node);
        for (int b2 = 0; b2 < b; b2++)
          if (pe[b2] == node) { sl |= kRowSlotGhost | kRowSlotDup | (sl << 10) | (1023u << 20); break; }
      } else {
        const int g = node - p.nv;
        sl = kRowSlotGhost | col_lower_bound(cols, nb, m.ghost3[3 * g + 1]) |
             (col_lower_bound(cols, nb, m.ghost3[3 * g]) << 10) | (col_lower_bound(cols, nb, m.ghost3[3 * g + 2]) << 20);
      }
    }
    r[4 + b] = (int)sl;
  }
}

int launch_row_records(const DevMesh &m, const KParams &p, int *rrec, void *stream)
{
  const long long threads = 32LL * p.nt;
  k_row_records<<<(unsigned)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(m, p, rrec);
  return (int)cudaGetLastError();
}

/* ---------------- scaling ---------------- */
__global__ void k_scale(DevMesh m, KParams p, double *__restrict__ R)
{
  const double fmax = __longlong_as_double((long long)*m.fmax);
  if (!(fmax > 1.0)) return;
  const double sc = 1.0 / fmax;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 3LL * p.nt) R[t] = R[t] * sc;
}

/* ---------------- launchers ---------------- */
static inline int blocks_for(long long n, int bs) { return (int)((n + bs - 1) / bs); }

int launch_ref_prep(const DevMesh &m, const KParams &p, const double *fib, const double *gscale, double *eref_out, void *stream)
{
  k_ref_prep<<<blocks_for(p.ne, 128), 128, 0, (cudaStream_t)stream>>>(m, p, fib, gscale, eref_out);
  return (int)cudaGetLastError();
}

int launch_positions(const DevMesh &m, const KParams &p, const double *x, void *stream)
{
  k_positions<<<blocks_for(p.nt, 256), 256, 0, (cudaStream_t)stream>>>(p.nv, p.ng, x, m.ghost3, m.pos);
  return (int)cudaGetLastError();
}

int launch_elem_residual(const DevMesh &m, const KParams &p, void *stream, bool store_metric)
{
  k_elem_residual<<<blocks_for(p.ne, 128), 128, 0, (cudaStream_t)stream>>>(m, p, store_metric ? m.gmq : nullptr,
                                                                          store_metric ? m.gpr : nullptr,
                                                                          store_metric ? m.gtape : nullptr);
  return (int)cudaGetLastError();
}

int launch_elem_residual_ff(const DevMesh &m, const KParams &p, void *stream)
{
  k_elem_residual_ff<<<blocks_for(p.ne, 128), 128, 0, (cudaStream_t)stream>>>(m, p);
  return (int)cudaGetLastError();
}

int launch_to_ff(const double *a, void *b, long long n, void *stream)
{
  k_to_ff<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(a, static_cast<FF *>(b), n);
  return (int)cudaGetLastError();
}

int launch_elem_tangent(const DevMesh &m, const KParams &p, void *stream)
{
  k_elem_tangent<<<blocks_for(p.ne, kTanElemsPerCta), 128, 0, (cudaStream_t)stream>>>(m, p);
  return (int)cudaGetLastError();
}

int launch_elem_tangent_f32(const DevMesh &m, const KParams &p, void *stream)
{
  k_elem_tangent_f32<<<blocks_for(p.ne, kTanElemsPerCta), 128, 0, (cudaStream_t)stream>>>(m, p);
  return (int)cudaGetLastError();
}


__global__ void k_to_float(const double *__restrict__ a, float *__restrict__ b, long long n)
{
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) b[t] = (float)a[t];
}

int launch_to_float(const double *a, float *b, long long n, void *stream)
{
  k_to_float<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(a, b, n);
  return (int)cudaGetLastError();
}

/* UpdateElementThickness (active_strain.c:2198-2224): one thread per element,
   the residual kernel's geometry and stress with C33 of every thickness point
   kept; thickness = h0 sqrt(mean C33). */
__global__ void __launch_bounds__(128) k_elem_thickness(DevMesh m, KParams p, double h0, double *__restrict__ th)
{
  __shared__ double tabs[kNumTables * 80];
  for (int i = threadIdx.x; i < kNumTables * 80; i += blockDim.x) tabs[i] = m.ntab[i];
  __syncthreads();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.ne) return;
  const int info = m.einfo[e];
  const int nen = info & 0xff, tabi = info >> 8;
  double y[15];
  gather_y(m.pos, m.patch, e, nen, tabs + tabi * 80, y);
  int st = 0;
  const EPar<double> ep = epar<double>(p);
  th[e] = elem_thickness<double>(y, ep, m.eref + e, p.ne, h0, st);
  set_status(m.status, st);
}

int launch_elem_thickness(const DevMesh &m, const KParams &p, double h0, double *th, void *stream)
{
  k_elem_thickness<<<blocks_for(p.ne, 128), 128, 0, (cudaStream_t)stream>>>(m, p, h0, th);
  return (int)cudaGetLastError();
}

/* d Fdyn / d x: per free node, the triangle-order sum over its corner
   triangles of M M1 + C C1 (Newmark) or M / dt^2 + C / dt (central) */
__global__ void k_dyn_diag(DevMesh m, KParams p)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.nt) return;
  double s = 0.0;
  if (m.rowkind[i] == 0) {
    for (int c = m.dptr[i]; c < m.dptr[i + 1]; c++) {
      const double M = p.dyn_rhoh0 * m.dA0[m.didx[c]] / 3;
      const double C = p.dyn_damp ? p.dyn_dampf * M : 0.0;
      s += p.dyn_central ? M / (p.dyn_dt * p.dyn_dt) + C / p.dyn_dt : M * p.dyn_M1 + C * p.dyn_C1;
    }
  }
  m.dyn_diag[i] = s;
}

/* xAccVel (main.c:1367-1412; with the DMPlex context the n_v real nodes),
   then xnm1 <- xn, xn <- x over every entry (main.c:571-572) */
__global__ void k_dyn_update(DevMesh m, KParams p, const double *__restrict__ x)
{
  const size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (j >= 3 * (size_t)p.nt) return;
  if (j < 3 * (size_t)p.nv) {
    const double xddn = m.xdd[j];
    const double a = p.dyn_M1 * (x[j] - m.xn[j]) - p.dyn_M2 * m.xd[j] - p.dyn_M3 * m.xdd[j];
    m.xdd[j] = a;
    m.xd[j] = m.xd[j] + p.dyn_U2 * xddn + p.dyn_U3 * a;
  }
  m.xnm1[j] = m.xn[j];
  m.xn[j] = x[j];
}

int launch_dyn_diag(const DevMesh &m, const KParams &p, void *stream)
{
  k_dyn_diag<<<blocks_for(p.nt, 256), 256, 0, (cudaStream_t)stream>>>(m, p);
  return (int)cudaGetLastError();
}

int launch_dyn_update(const DevMesh &m, const KParams &p, const double *x, void *stream)
{
  k_dyn_update<<<blocks_for(3LL * p.nt, 256), 256, 0, (cudaStream_t)stream>>>(m, p, x);
  return (int)cudaGetLastError();
}

int launch_node_gather(const DevMesh &m, const KParams &p, const double *x, double *R, void *stream, double *parts)
{
  cudaMemsetAsync(m.fmax, 0, sizeof(unsigned long long), (cudaStream_t)stream);
  k_node_gather<<<blocks_for(p.nt, 256), 256, 0, (cudaStream_t)stream>>>(m, p, x, R, parts);
  return (int)cudaGetLastError();
}

/* the staged tables (only the cap table when the mesh has cap elements),
   then each warp's row buffer */
size_t row_assemble_smem(int maxblk, bool f32, int ntabs)
{
  if (f32) return align16(ntabs * 16 * kRowPad * 4) + kRowWarps * row_reg_bytes();
  return align16(ntabs * 16 * kRowPad * 8) + kRowWarps * row_buf_bytes(maxblk, 8);
}

int row_assemble_max_blocks(bool f32) { return f32 ? kRowRegMax : kMaxRowBlocks; }

int launch_row_assemble(const DevMesh &m, const KParams &p, void *K, bool f32, bool colmajor, void *stream)
{
  const int grid = blocks_for(p.nt, kRowWarps);
  const size_t smem = row_assemble_smem(m.maxblk, f32, m.ntabs);
  if (f32)
    k_row_assemble_f32<<<grid, 32 * kRowWarps, smem, (cudaStream_t)stream>>>(
        m, p, m.DeF, m.ntabF, -p.pres6f, static_cast<float *>(K), (int)colmajor);
  else
    k_row_assemble<double><<<grid, 32 * kRowWarps, smem, (cudaStream_t)stream>>>(
        m, p, m.De, m.ntab, -p.pressure / 6.0, static_cast<double *>(K), m.maxblk, (int)colmajor);
  return (int)cudaGetLastError();
}

int row_assemble_configure(int maxblk, bool f32, int ntabs)
{
  const size_t smem = row_assemble_smem(maxblk, f32, ntabs);
  cudaError_t e = f32 ? cudaFuncSetAttribute(k_row_assemble_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                      : cudaFuncSetAttribute(k_row_assemble<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return (int)e;
}

int launch_scale(const DevMesh &m, const KParams &p, double *R, void *stream)
{
  k_scale<<<blocks_for(3LL * p.nt, 256), 256, 0, (cudaStream_t)stream>>>(m, p, R);
  return (int)cudaGetLastError();
}

} /* namespace biofem */
