/*
 * Device Newton solve of R(x) = 0 with the assembled tangent: replaces the
 * reference's matrix-free PETSc SNES (newtonls + MFFD + GMRES, main.c:461-551)
 * for one quasi-static load step.
 *
 *   Newton:   x <- x + alpha dx,  K(x) dx = -R(x),  backtracking on ||R||
 *             (sufficient decrease 1e-4, halving up to 12 times), stop at
 *             ||R|| <= rtol ||R0|| (or atol).
 *   Linear:   restarted GMRES(m) with right block-Jacobi(3x3) preconditioning,
 *             classical Gram-Schmidt applied twice, Givens rotations on the
 *             host; all vectors, the BSR matvec and the dot products on the
 *             device in FP64 (the tangent values may be FP32 for an
 *             FP32-bulk handle).
 * Ghost rows of K are identity and their residual is zero, so ghost entries
 * of x never move.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "biofem_host.h"

namespace biofem {

int noalloc_fail(int code, const std::string &msg);   /* error reporting (bridge.cu) */

/* ---------------- kernels ---------------- */
template <class KT>
__global__ void k_bsr_matvec(int nb, const int *__restrict__ rowptr, const int *__restrict__ colind,
                             const KT *__restrict__ K, const double *__restrict__ x, double *__restrict__ y)
{
  /* 4 lanes per block row, lane q takes blocks q, q+4, ... */
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = t >> 2, q = t & 3;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  if (row < nb) {
    for (int k = rowptr[row] + q; k < rowptr[row + 1]; k += 4) {
      const int c = colind[k];
      const double x0 = x[3 * (size_t)c], x1 = x[3 * (size_t)c + 1], x2 = x[3 * (size_t)c + 2];
      const KT *b = K + 9 * (size_t)k;
      s0 += (double)b[0] * x0 + (double)b[1] * x1 + (double)b[2] * x2;
      s1 += (double)b[3] * x0 + (double)b[4] * x1 + (double)b[5] * x2;
      s2 += (double)b[6] * x0 + (double)b[7] * x1 + (double)b[8] * x2;
    }
  }
  for (int o = 1; o < 4; o <<= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if (row < nb && q == 0) { y[3 * (size_t)row] = s0; y[3 * (size_t)row + 1] = s1; y[3 * (size_t)row + 2] = s2; }
}

/* inverse of every diagonal block (block-Jacobi) */
template <class KT>
__global__ void k_bj_setup(int nb, const int *__restrict__ rowptr, const int *__restrict__ colind,
                           const KT *__restrict__ K, double *__restrict__ Dinv, int *__restrict__ status)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  double a[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
    if (colind[k] == i) { for (int v = 0; v < 9; v++) a[v] = (double)K[9 * (size_t)k + v]; break; }
  const double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8], c02 = a[3] * a[7] - a[4] * a[6];
  const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  double *o = Dinv + 9 * (size_t)i;
  if (!(fabs(det) > 0.0) || !isfinite(det)) {
    atomicOr(status, 2);
    for (int v = 0; v < 9; v++) o[v] = (v % 4 == 0) ? 1.0 : 0.0;
    return;
  }
  const double id = 1.0 / det;
  o[0] = c00 * id; o[1] = (a[2] * a[7] - a[1] * a[8]) * id; o[2] = (a[1] * a[5] - a[2] * a[4]) * id;
  o[3] = c01 * id; o[4] = (a[0] * a[8] - a[2] * a[6]) * id; o[5] = (a[2] * a[3] - a[0] * a[5]) * id;
  o[6] = c02 * id; o[7] = (a[1] * a[6] - a[0] * a[7]) * id; o[8] = (a[0] * a[4] - a[1] * a[3]) * id;
}

__global__ void k_bj_apply(int nb, const double *__restrict__ Dinv, const double *__restrict__ r, double *__restrict__ z)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double *d = Dinv + 9 * (size_t)i;
  const double r0 = r[3 * (size_t)i], r1 = r[3 * (size_t)i + 1], r2 = r[3 * (size_t)i + 2];
  z[3 * (size_t)i] = d[0] * r0 + d[1] * r1 + d[2] * r2;
  z[3 * (size_t)i + 1] = d[3] * r0 + d[4] * r1 + d[5] * r2;
  z[3 * (size_t)i + 2] = d[6] * r0 + d[7] * r1 + d[8] * r2;
}

/* partial dot products of w with the first nv basis vectors (column stride
   ld): block (c, j) reduces column j over the c-th strided chunk */
constexpr int kDotBlocks = 128;
__global__ void k_multidot(int n, int nv, const double *__restrict__ V, size_t ld, const double *__restrict__ w,
                           double *__restrict__ part)
{
  __shared__ double red[8];
  const int j = blockIdx.y;
  const double *v = V + (size_t)j * ld;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += v[i] * w[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += red[k];
    part[(size_t)j * gridDim.x + blockIdx.x] = t;
  }
}

__global__ void k_reduce_parts(int nv, int nparts, const double *__restrict__ part, double *__restrict__ out)
{
  const int j = blockIdx.x;
  double v = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) v += part[(size_t)j * nparts + k];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __shared__ double s[32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += s[k];
    out[j] = t;
  }
}

/* w -= V h (first nv columns) */
__global__ void k_multi_axpy(int n, int nv, const double *__restrict__ V, size_t ld, const double *__restrict__ h,
                             double *__restrict__ w, double sign)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int j = 0; j < nv; j++) s += V[(size_t)j * ld + i] * h[j];
  w[i] += sign * s;
}

__global__ void k_scale_copy(int n, const double *__restrict__ a, double s, double *__restrict__ b)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i] * s;
}

__global__ void k_axpby(int n, double a, const double *__restrict__ x, double b, double *__restrict__ y)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}

__global__ void k_zero_ghost(int nv, int nt, double *__restrict__ v)
{
  const int i = nv * 3 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 3 * nt) v[i] = 0.0;
}

/* ---------------- host side ---------------- */
static inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }

struct SolverWork {
  int n = 0, nb = 0, m = 0;
  double *V = nullptr, *z = nullptr, *w = nullptr, *dinv = nullptr, *part = nullptr, *dots = nullptr;
  double *dx = nullptr, *xt = nullptr, *Rt = nullptr, *xh = nullptr;
  double *hdots = nullptr;   /* pinned */
};

class Gmres {
 public:
  Gmres(const DevMesh &dm, const KParams &kp, bool f32, const void *K, SolverWork &w, cudaStream_t st)
      : dm_(dm), kp_(kp), f32_(f32), K_(K), w_(w), st_(st) {}

  int matvec(const double *x, double *y)
  {
    if (f32_) k_bsr_matvec<float><<<nblk(4LL * w_.nb, 256), 256, 0, st_>>>(w_.nb, dm_.rowptr, dm_.colind, (const float *)K_, x, y);
    else k_bsr_matvec<double><<<nblk(4LL * w_.nb, 256), 256, 0, st_>>>(w_.nb, dm_.rowptr, dm_.colind, (const double *)K_, x, y);
    return (int)cudaGetLastError();
  }
  int precond(const double *r, double *z)
  {
    k_bj_apply<<<nblk(w_.nb, 256), 256, 0, st_>>>(w_.nb, w_.dinv, r, z);
    return (int)cudaGetLastError();
  }
  /* h[0..nv) = V[:, 0..nv)^T v, returned on the host */
  int dots(int nv, const double *v, double *h)
  {
    k_multidot<<<dim3(kDotBlocks, nv), 256, 0, st_>>>(w_.n, nv, w_.V, (size_t)w_.n, v, w_.part);
    k_reduce_parts<<<nv, 128, 0, st_>>>(nv, kDotBlocks, w_.part, w_.dots);
    cudaMemcpyAsync(w_.hdots, w_.dots, nv * sizeof(double), cudaMemcpyDeviceToHost, st_);
    cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return (int)e;
    for (int j = 0; j < nv; j++) h[j] = w_.hdots[j];
    return 0;
  }
  /* dot of two arbitrary vectors (uses the part buffer with V as one column) */
  int dot2(const double *a, const double *b, double &out)
  {
    k_multidot<<<dim3(kDotBlocks, 1), 256, 0, st_>>>(w_.n, 1, a, (size_t)w_.n, b, w_.part);
    k_reduce_parts<<<1, 128, 0, st_>>>(1, kDotBlocks, w_.part, w_.dots);
    cudaMemcpyAsync(w_.hdots, w_.dots, sizeof(double), cudaMemcpyDeviceToHost, st_);
    cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return (int)e;
    out = w_.hdots[0];
    return 0;
  }

  /* solve K dx = b (dx zeroed on entry); returns iterations in *its */
  int solve(const double *b, double *dx, double rtol, int maxit, int *its, double *relres)
  {
    const int n = w_.n, m = w_.m;
    double *V = w_.V;
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), h(m + 1), h2(m + 1), y(m);
    double bnorm2;
    int rc = dot2(b, b, bnorm2);
    if (rc) return rc;
    const double bnorm = std::sqrt(bnorm2);
    *its = 0;
    *relres = 0.0;
    cudaMemsetAsync(dx, 0, n * sizeof(double), st_);
    if (bnorm == 0.0) return 0;
    double beta = bnorm;
    /* r = b - K dx; dx = 0 on the first cycle */
    k_scale_copy<<<nblk(n, 256), 256, 0, st_>>>(n, b, 1.0, w_.w);
    while (*its < maxit) {
      k_scale_copy<<<nblk(n, 256), 256, 0, st_>>>(n, w_.w, 1.0 / beta, V);
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int j = 0;
      double res = beta;
      for (; j < m && *its < maxit; j++) {
        double *vj = V + (size_t)j * n, *vn = V + (size_t)(j + 1) * n;
        if ((rc = precond(vj, w_.z)) || (rc = matvec(w_.z, vn))) return rc;
        /* classical Gram-Schmidt, twice */
        if ((rc = dots(j + 1, vn, h.data()))) return rc;   /* also leaves h in w_.dots */
        k_multi_axpy<<<nblk(n, 256), 256, 0, st_>>>(n, j + 1, V, (size_t)n, w_.dots, vn, -1.0);
        if ((rc = dots(j + 1, vn, h2.data()))) return rc;
        k_multi_axpy<<<nblk(n, 256), 256, 0, st_>>>(n, j + 1, V, (size_t)n, w_.dots, vn, -1.0);
        for (int i = 0; i <= j; i++) h[i] += h2[i];
        double nn;
        if ((rc = dot2(vn, vn, nn))) return rc;
        const double hn = std::sqrt(nn);
        for (int i = 0; i <= j; i++) H[(size_t)i * m + j] = h[i];
        H[(size_t)(j + 1) * m + j] = hn;
        for (int i = 0; i < j; i++) {
          const double a = H[(size_t)i * m + j], bb = H[(size_t)(i + 1) * m + j];
          H[(size_t)i * m + j] = cs[i] * a + sn[i] * bb;
          H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * bb;
        }
        const double a = H[(size_t)j * m + j], bb = H[(size_t)(j + 1) * m + j];
        const double r = std::hypot(a, bb);
        cs[j] = r > 0 ? a / r : 1.0; sn[j] = r > 0 ? bb / r : 0.0;
        H[(size_t)j * m + j] = r; H[(size_t)(j + 1) * m + j] = 0.0;
        g[j + 1] = -sn[j] * g[j]; g[j] = cs[j] * g[j];
        (*its)++;
        res = std::fabs(g[j + 1]);
        if (hn > 0) k_scale_copy<<<nblk(n, 256), 256, 0, st_>>>(n, vn, 1.0 / hn, vn);
        if (res <= rtol * bnorm || hn == 0.0) { j++; break; }
      }
      /* y = H^-1 g, dx += M^-1 V y */
      for (int i = j - 1; i >= 0; i--) {
        double s = g[i];
        for (int k = i + 1; k < j; k++) s -= H[(size_t)i * m + k] * y[k];
        y[i] = s / H[(size_t)i * m + i];
      }
      cudaMemcpyAsync(w_.dots, y.data(), j * sizeof(double), cudaMemcpyHostToDevice, st_);
      cudaMemsetAsync(w_.w, 0, n * sizeof(double), st_);
      k_multi_axpy<<<nblk(n, 256), 256, 0, st_>>>(n, j, V, (size_t)n, w_.dots, w_.w, 1.0);
      if ((rc = precond(w_.w, w_.z))) return rc;
      k_axpby<<<nblk(n, 256), 256, 0, st_>>>(n, 1.0, w_.z, 1.0, dx);
      *relres = res / bnorm;
      if (res <= rtol * bnorm) break;
      /* restart: w = b - K dx */
      if ((rc = matvec(dx, w_.w))) return rc;
      k_axpby<<<nblk(n, 256), 256, 0, st_>>>(n, 1.0, b, -1.0, w_.w);
      double rr;
      if ((rc = dot2(w_.w, w_.w, rr))) return rc;
      beta = std::sqrt(rr);
      *relres = beta / bnorm;
      if (beta <= rtol * bnorm) break;
    }
    return (int)cudaGetLastError();
  }

 private:
  const DevMesh &dm_;
  const KParams &kp_;
  bool f32_;
  const void *K_;
  SolverWork &w_;
  cudaStream_t st_;
};

SolverWork *solver_create(int n, int nb, int m, int *rc)
{
  SolverWork *w = new SolverWork();
  w->n = n; w->nb = nb; w->m = m;
  cudaError_t e = cudaSuccess;
  const size_t dn = sizeof(double) * (size_t)n;
  if (e == cudaSuccess) e = cudaMalloc(&w->V, dn * (size_t)(m + 1));
  if (e == cudaSuccess) e = cudaMalloc(&w->z, dn);
  if (e == cudaSuccess) e = cudaMalloc(&w->w, dn);
  if (e == cudaSuccess) e = cudaMalloc(&w->dx, dn);
  if (e == cudaSuccess) e = cudaMalloc(&w->xt, dn);
  if (e == cudaSuccess) e = cudaMalloc(&w->Rt, dn);
  if (e == cudaSuccess) e = cudaMalloc(&w->xh, dn);
  if (e == cudaSuccess) e = cudaMalloc(&w->dinv, sizeof(double) * 9 * (size_t)nb);
  if (e == cudaSuccess) e = cudaMalloc(&w->part, sizeof(double) * (size_t)(m + 1) * kDotBlocks);
  if (e == cudaSuccess) e = cudaMalloc(&w->dots, sizeof(double) * (m + 1));
  if (e == cudaSuccess) e = cudaMallocHost(&w->hdots, sizeof(double) * (m + 1));
  *rc = (int)e;
  if (e != cudaSuccess) { solver_destroy(w); return nullptr; }
  return w;
}

void solver_destroy(SolverWork *w)
{
  if (!w) return;
  cudaFree(w->V); cudaFree(w->z); cudaFree(w->w); cudaFree(w->dx); cudaFree(w->xt); cudaFree(w->Rt);
  cudaFree(w->xh); cudaFree(w->dinv); cudaFree(w->part); cudaFree(w->dots); cudaFreeHost(w->hdots);
  delete w;
}

double *solver_xbuf(SolverWork *w) { return w->xh; }
int solver_m(const SolverWork *w) { return w->m; }

/* Newton on device data; x is a device vector (updated in place). */
int newton_device(const DevMesh &dm, const KParams &kp, bool f32, void *dK, double *dR, double *x,
                  const BiofemNewtonOptions &o, BiofemNewtonStats &s, SolverWork *wp, cudaStream_t st,
                  ResidualFn residual, JacobianFn jacobian, void *ctx,
                  std::string &err)
{
  const int n = 3 * kp.nt, nb = kp.nt;
  SolverWork &w = *wp;
  Gmres gm(dm, kp, f32, dK, w, st);
  int rc;
  auto norm = [&](const double *v, double &out) -> int {
    double d2;
    int r = gm.dot2(v, v, d2);
    out = std::sqrt(d2);
    return r;
  };
  s = BiofemNewtonStats();
  if ((rc = residual(ctx, x, dR, (void *)st))) { err = "residual"; return rc; }
  s.residual_evals++;
  double rn;
  if ((rc = norm(dR, rn))) { err = "norm"; return rc; }
  s.r0 = rn;
  s.rhist[0] = rn;
  for (int it = 0; it < o.max_newton; it++) {
    if (rn <= o.rtol * s.r0 || rn <= o.atol) { s.converged = 1; break; }
    if ((rc = jacobian(ctx, x, dR, dK, (void *)st))) { err = "jacobian"; return rc; }
    s.jacobian_evals++;
    if (f32) k_bj_setup<float><<<nblk(nb, 256), 256, 0, st>>>(nb, dm.rowptr, dm.colind, (const float *)dK, w.dinv, dm.status);
    else k_bj_setup<double><<<nblk(nb, 256), 256, 0, st>>>(nb, dm.rowptr, dm.colind, (const double *)dK, w.dinv, dm.status);
    /* rhs = -R */
    k_scale_copy<<<nblk(n, 256), 256, 0, st>>>(n, dR, -1.0, w.Rt);
    int its = 0;
    double relres = 0.0;
    if ((rc = gm.solve(w.Rt, w.dx, o.gmres_rtol, o.gmres_max_it, &its, &relres))) { err = "gmres"; return rc; }
    s.gmres_its_total += its;
    s.gmres_its_last = its;
    s.gmres_relres_last = relres;
    k_zero_ghost<<<nblk(3LL * (kp.nt - kp.nv), 256), 256, 0, st>>>(kp.nv, kp.nt, w.dx);
    /* backtracking on ||R|| */
    double alpha = 1.0, rnew = 0.0;
    for (int ls = 0; ls < 12; ls++) {
      k_scale_copy<<<nblk(n, 256), 256, 0, st>>>(n, x, 1.0, w.xt);
      k_axpby<<<nblk(n, 256), 256, 0, st>>>(n, alpha, w.dx, 1.0, w.xt);
      if ((rc = residual(ctx, w.xt, dR, (void *)st))) { err = "residual"; return rc; }
      s.residual_evals++;
      if ((rc = norm(dR, rnew))) { err = "norm"; return rc; }
      if (!o.line_search || rnew <= (1.0 - 1e-4 * alpha) * rn || !std::isfinite(rn)) break;
      alpha *= 0.5;
    }
    k_scale_copy<<<nblk(n, 256), 256, 0, st>>>(n, w.xt, 1.0, x);
    rn = rnew;
    s.newton_its++;
    if (s.newton_its < 64) s.rhist[s.newton_its] = rn;
  }
  if (rn <= o.rtol * s.r0 || rn <= o.atol) s.converged = 1;
  s.rfinal = rn;
  return (int)cudaStreamSynchronize(st);
}

} /* namespace biofem */
