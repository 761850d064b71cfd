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
 *                    geometry and the chain rule, giving column j of df/dy;
 *                    the half-warp then forms K_e = N^T (df/dy) N
 *                    (contract_element: T = (df/dy) N held in registers)
 *   k_node_gather    one thread per node: Fint / Fext (and FDynamic's Fdyn)
 *                    summed over the node's element contributions in element
 *                    order (the order FInternalAct's VecSetValues loop adds
 *                    them), R = Fint - Fext + Fdyn, clamp rows R = x - X,
 *                    ghost rows 0 (main.c:844-1016)
 *   k_block_gather   one thread per tangent value: sum of the element-matrix
 *                    entries mapped to that 3x3 block, in element order
 *   k_scale          R *= 1 / max(|Fext|_inf, 1) (main.c:1020-1026); the block
 *                    gathers apply the same factor to K as they write it
 *   k_elem_thickness UpdateElementThickness (output); k_dyn_diag / k_dyn_update
 *                    the dynamic term's tangent diagonal and xAccVel
 *
 * Assembly is deterministic: every sum runs in a fixed order given by the
 * precomputed element-to-node / element-to-block maps, independent of the
 * launch configuration.
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
  const V3<double> f = {fib[3 * (size_t)e], fib[3 * (size_t)e + 1], fib[3 * (size_t)e + 2]};
  const double gam = p.gamma * gscale[e];
  const double phi = dot(f, f);
  const double gamp = gam / (1.0 - gam * phi);
  const double c1 = 2.0 * gamp + gamp * gamp * phi;
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
    const double rho = 1.0 / (det3(G) * omg * omg);
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
    o[0] = Gi[0][0]; o[1 * ne] = Gi[1][1]; o[2 * ne] = 0.5 * (Gi[0][1] + Gi[1][0]); o[3 * ne] = Gi[2][2];
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
  /* follower pressure: each corner receives n P dA / 3 = P (x2-x1)x(x3-x1) / 6 */
  if (p.pressure != 0.0) {
    double X[3][3];
    for (int k = 0; k < 3; k++) load_node(m.pos, m.etri[3 * (size_t)e + k], X[k][0], X[k][1], X[k][2]);
    const V3<double> d21 = {X[1][0] - X[0][0], X[1][1] - X[0][1], X[1][2] - X[0][2]};
    const V3<double> d31 = {X[2][0] - X[0][0], X[2][1] - X[0][1], X[2][2] - X[0][2]};
    const V3<double> ca = cross(d21, d31);
    const double nrm = sqrt(ca.x * ca.x + ca.y * ca.y + ca.z * ca.z);
    const double dA = 0.5 * nrm;
    m.fp[e] = (ca.x / nrm) * p.pressure * dA / 3.;
    m.fp[ne + e] = (ca.y / nrm) * p.pressure * dA / 3.;
    m.fp[2 * ne + e] = (ca.z / nrm) * p.pressure * dA / 3.;
  }
}

/* ---------------- tangent element kernel ---------------- */
constexpr int kTanElemsPerCta = 8;   /* 16 lanes per element, 128 threads */

__global__ void __launch_bounds__(128) k_elem_tangent(DevMesh m, KParams p)
{
  __shared__ double tabs[kNumTables * 80];
  /* D = df/dy per element, row stride 19 (3 mod 16 eight-byte banks: the 9
     (i, j) rows and columns the lanes read fall in distinct banks) */
  constexpr int kDRow = 19, kDSlot = 15 * kDRow;
  __shared__ double Dsh[kTanElemsPerCta * kDSlot];
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
  /* column `lane` of D = df/dy */
  double *D = Dsh + slot * kDSlot;
  if (lane < 15) {
#pragma unroll
    for (int r = 0; r < 15; r++) D[r * kDRow + lane] = fd[r];
  }
  /* the element forces come from k_elem_residual, launched before this kernel */
  __syncwarp();
  if (!live) return;
  /* Follower-pressure load stiffness: every corner carries P/6 (x2-x1)x(x3-x1),
     so d/dx1 = [b-a]x, d/dx2 = -[b]x, d/dx3 = [a]x with a = x2-x1, b = x3-x1,
     entering K = dR/dx with a minus sign at the corner rows. */
  const int cs = m.ecorner[e];
  const int cslot[3] = {cs & 31, (cs >> 5) & 31, (cs >> 10) & 31};
  double X[3][3];
  for (int k = 0; k < 3; k++) load_node(m.pos, m.etri[3 * (size_t)e + k], X[k][0], X[k][1], X[k][2]);
  const double av[3] = {X[1][0] - X[0][0], X[1][1] - X[0][1], X[1][2] - X[0][2]};
  const double bv[3] = {X[2][0] - X[0][0], X[2][1] - X[0][1], X[2][2] - X[0][2]};
  const double vv[3][3] = {{bv[0] - av[0], bv[1] - av[1], bv[2] - av[2]}, {-bv[0], -bv[1], -bv[2]}, {av[0], av[1], av[2]}};
  contract_element<double>(D, kDRow, tab, nen, lane, cslot, p.pressure != 0.0, vv, -p.pressure / 6.0,
                           m.ke + (size_t)m.kofs[e] * 9);
}

/* ---------------- FP32-bulk tangent ---------------- */
/* Same element math as k_elem_tangent in single precision.  Node positions
   are shifted to the element's first corner in FP64 (one node per lane, then
   shared by shuffles) and rounded to FP32, so the FP32 values carry the
   element-size digits; the shift is put back through (sum_i N_r[i]) * x_c,
   which is not zero for the truncated second-derivative rows (their rows sum
   to -1e-4 / -1e-4 / +2e-4).  Element matrices are written in FP32. */
__global__ void __launch_bounds__(128, 4) k_elem_tangent_f32(DevMesh m, KParams p)
{
  __shared__ float tabs[kNumTables * 80];
  __shared__ float tsum[kNumTables * 5];
  /* D = df/dy per element: row stride 20 and element stride 323 (3 mod 32
     banks) keep the 9 (i, j) rows and columns the lanes read in distinct banks */
  constexpr int kDRow = 20, kDSlot = 323;
  __shared__ float Dsh[kTanElemsPerCta * kDSlot];
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
  float *D = Dsh + slot * kDSlot;
  if (lane < 15) {
#pragma unroll
    for (int r = 0; r < 15; r++) D[r * kDRow + lane] = fd[r].d;
  }
  /* pressure stiffness from the shifted corner coordinates */
  const int cs = m.ecorner[ee];
  const int cslot[3] = {cs & 31, (cs >> 5) & 31, (cs >> 10) & 31};
  float xk[3][3];
  for (int k = 0; k < 3; k++) {
    xk[k][0] = __shfl_sync(hmask, dx, cslot[k], 16);
    xk[k][1] = __shfl_sync(hmask, dy, cslot[k], 16);
    xk[k][2] = __shfl_sync(hmask, dz, cslot[k], 16);
  }
  __syncwarp();
  if (!live) return;
  const float av[3] = {xk[1][0] - xk[0][0], xk[1][1] - xk[0][1], xk[1][2] - xk[0][2]};
  const float bv[3] = {xk[2][0] - xk[0][0], xk[2][1] - xk[0][1], xk[2][2] - xk[0][2]};
  const float vv[3][3] = {{bv[0] - av[0], bv[1] - av[1], bv[2] - av[2]}, {-bv[0], -bv[1], -bv[2]}, {av[0], av[1], av[2]}};
  contract_element<float>(D, kDRow, tab, nen, lane, cslot, p.pres6f != 0.f, vv, -p.pres6f,
                          m.keF + (size_t)m.kofs[e] * 9);
}

/* FP32 block gather with compensated (Kahan) summation in element order. */
__global__ void k_block_gather_f32(DevMesh m, KParams p, float *__restrict__ K, const int *__restrict__ perm)
{
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 9 * m.nnzb) return;
  const long long kk = t / 9;
  const int w = (int)(t - 9 * kk);
  const long long k = perm ? perm[kk] : kk;
  const double fmax = __longlong_as_double((long long)*m.fmax);   /* read early: its latency hides under the sum */
  const int row = m.blkrow[k];
  const int kind = m.rowkind[row];
  float s = 0.f;
  if (kind != 0) {
    s = (m.colind[k] == row && (w == 0 || w == 4 || w == 8)) ? 1.f : 0.f;
  } else {
    float comp = 0.f;
    long long c = m.cptr[k];
    const long long cend = m.cptr[k + 1];
    /* four gathered loads in flight per step; the compensated sum keeps the list order */
    for (; c + 4 <= cend; c += 4) {
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int id = m.cidx[c + u];
        const int neg = (int)((unsigned)(id < 0) << 31);
        v[u] = __int_as_float(__float_as_int(m.keF[(size_t)(id < 0 ? -(id + 1) : id) * 9 + w]) ^ neg);
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float yv = v[u] - comp;
        const float tt = s + yv;
        comp = (tt - s) - yv;
        s = tt;
      }
    }
    for (; c < cend; c++) {
      const int id = m.cidx[c];
      const int neg = (int)((unsigned)(id < 0) << 31);   /* sign flip of a chain-rule contribution, integer pipe */
      const float v = __int_as_float(__float_as_int(m.keF[(size_t)(id < 0 ? -(id + 1) : id) * 9 + w]) ^ neg);
      const float yv = v - comp;
      const float tt = s + yv;
      comp = (tt - s) - yv;
      s = tt;
    }
    if (p.dyn && m.colind[k] == row && (w == 0 || w == 4 || w == 8)) s += (float)m.dyn_diag[row];
  }
  /* R and K scale by 1/max(|Fext|_inf, 1) (main.c:1020-1026; k_node_gather
     found the max); ghost rows stay identity */
  if (fmax > 1.0 && kind != 2) {
    const double sc = 1.0 / fmax;
    s = (float)(s * sc);
  }
  K[9 * k + w] = s;
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
    /* FDynamic (main.c:1293-1360, the serial path): triangle-order sum of the
       node's inertial (and damping) force over every triangle with this
       corner, ghost and bridging triangles included */
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

/* ---------------- block gather (tangent assembly) ---------------- */
__global__ void k_block_gather(DevMesh m, KParams p, double *__restrict__ K, const int *__restrict__ perm)
{
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 9 * m.nnzb) return;
  const long long kk = t / 9;
  const int w = (int)(t - 9 * kk);
  const long long k = perm ? perm[kk] : kk;   /* blocks of one row by decreasing contribution count */
  const double fmax = __longlong_as_double((long long)*m.fmax);   /* read early: its latency hides under the sum */
  const int row = m.blkrow[k];
  const int kind = m.rowkind[row];
  double s = 0.0;
  if (kind != 0) {
    s = (m.colind[k] == row && (w == 0 || w == 4 || w == 8)) ? 1.0 : 0.0;
  } else {
    long long c = m.cptr[k];
    const long long cend = m.cptr[k + 1];
    /* four gathered loads in flight per step; the sum keeps the list order
       (s - v and s + (-v) round alike) */
    /* the sign of a chain-rule contribution is flipped on the integer pipe
       (the FP64 pipe, which bounds this kernel, then sees one add each) */
    for (; c + 4 <= cend; c += 4) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int id = m.cidx[c + u];
        const long long neg = (long long)(id < 0) << 63;
        const long long bits = __double_as_longlong(m.ke[(size_t)(id < 0 ? -(id + 1) : id) * 9 + w]);
        v[u] = __longlong_as_double(bits ^ neg);
      }
#pragma unroll
      for (int u = 0; u < 4; u++) s += v[u];
    }
    for (; c < cend; c++) {
      const int id = m.cidx[c];
      const long long neg = (long long)(id < 0) << 63;
      const long long bits = __double_as_longlong(m.ke[(size_t)(id < 0 ? -(id + 1) : id) * 9 + w]);
      s += __longlong_as_double(bits ^ neg);
    }
    if (p.dyn && m.colind[k] == row && (w == 0 || w == 4 || w == 8)) s += m.dyn_diag[row];
  }
  /* the scale 1/max(|Fext|_inf, 1) of R and K (main.c:1020-1026; k_node_gather
     found the max), applied as the value is written; ghost rows stay identity */
  if (fmax > 1.0 && kind != 2) {
    const double sc = 1.0 / fmax;
    s = s * sc;
  }
  K[9 * k + w] = s;
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

int launch_block_gather_f32(const DevMesh &m, const KParams &p, float *K, void *stream, bool k_on_host)
{
  if (m.nnzb == 0) return 0;
  k_block_gather_f32<<<blocks_for(9 * m.nnzb, 256), 256, 0, (cudaStream_t)stream>>>(m, p, K, k_on_host ? nullptr : m.gperm);
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

/* xAccVel (main.c:1367-1412, the serial path over n_v + n_ghosts nodes),
   then xnm1 <- xn, xn <- x (main.c:571-572) */
__global__ void k_dyn_update(DevMesh m, KParams p, const double *__restrict__ x)
{
  const size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (j >= 3 * (size_t)p.nt) return;
  const double xddn = m.xdd[j];
  const double a = p.dyn_M1 * (x[j] - m.xn[j]) - p.dyn_M2 * m.xd[j] - p.dyn_M3 * m.xdd[j];
  m.xdd[j] = a;
  m.xd[j] = m.xd[j] + p.dyn_U2 * xddn + p.dyn_U3 * a;
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

int launch_block_gather(const DevMesh &m, const KParams &p, double *K, void *stream, bool k_on_host)
{
  if (m.nnzb == 0) return 0;
  /* K in HBM: each row's blocks by decreasing contribution count; K in mapped
     host memory: plain block order, so the stores stream out in address order */
  k_block_gather<<<blocks_for(9 * m.nnzb, 256), 256, 0, (cudaStream_t)stream>>>(m, p, K, k_on_host ? nullptr : m.gperm);
  return (int)cudaGetLastError();
}

int launch_scale(const DevMesh &m, const KParams &p, double *R, void *stream)
{
  k_scale<<<blocks_for(3LL * p.nt, 256), 256, 0, (cudaStream_t)stream>>>(m, p, R);
  return (int)cudaGetLastError();
}

} /* namespace biofem */
