/*
 * Device Newton solve of R(x) = 0 with the assembled tangent: replaces the
 * reference's matrix-free PETSc SNES (newtonls + MFFD + GMRES, main.c:461-551)
 * for one quasi-static load step.
 *
 *   Newton:   x <- x + alpha dx,  K(x) dx = -R(x),  backtracking on ||R||
 *             (sufficient decrease 1e-4, halving up to 12 times), stop at
 *             ||R|| <= rtol ||R0|| (or atol); linear solves to a fixed
 *             relative tolerance or to Eisenstat-Walker forcing terms.
 *   Linear:   restarted flexible GMRES(m) (the preconditioned directions are
 *             kept), preconditioned by smoothed-aggregation multigrid (FP32
 *             V-cycle, amg.cu) or by block-Jacobi(3x3); classical
 *             Gram-Schmidt applied twice, Givens rotations and the small
 *             triangular solve on the device; all Krylov vectors and the
 *             dot products in FP64; the BSR matvec in FP64, or, with the FP32
 *             tangent of an FP32-bulk handle, in float-float arithmetic on
 *             the FP32 pipe (about 47 bits, against K's own 24).  One iteration: preconditioner,
 *             matvec, two projection passes (dot products with an in-kernel
 *             deterministic reduction, the second also doing the Givens
 *             step), and two updates.
 * Ghost rows of K are identity and their residual is zero, so ghost entries
 * of x never move.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "amg.h"
#include "biofem_host.h"
#include "ff.cuh"

namespace biofem {

int noalloc_fail(int code, const std::string &msg);   /* error reporting (bridge.cu) */

/* ---------------- kernels ---------------- */
struct GmState;
__device__ __forceinline__ bool gm_done(const GmState *gs);

template <class KT>
__global__ void k_bsr_matvec(int nb, const int *__restrict__ rowptr, const int *__restrict__ colind,
                             const KT *__restrict__ K, const double *__restrict__ x, double *__restrict__ y,
                             const GmState *__restrict__ gs)
{
  if (gs && gm_done(gs)) return;
  /* one half-warp per block row; lane q of the half takes whole 3x3 blocks
     q, q+16, ... so every lane issues its block's nine value loads and its
     column's three x loads independently of the others */
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = t >> 4, q = t & 15;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  if (row < nb) {
    const int k1 = rowptr[row + 1];
    for (int k = rowptr[row] + q; k < k1; k += 16) {
      const int c = colind[k];
      const KT *b = K + 9 * (size_t)k;
      const double a0 = (double)b[0], a1 = (double)b[1], a2 = (double)b[2], a3 = (double)b[3], a4 = (double)b[4];
      const double a5 = (double)b[5], a6 = (double)b[6], a7 = (double)b[7], a8 = (double)b[8];
      const double x0 = x[3 * (size_t)c], x1 = x[3 * (size_t)c + 1], x2 = x[3 * (size_t)c + 2];
      s0 += a0 * x0 + a1 * x1 + a2 * x2;
      s1 += a3 * x0 + a4 * x1 + a5 * x2;
      s2 += a6 * x0 + a7 * x1 + a8 * x2;
    }
  }
  for (int o = 1; o < 16; o <<= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if (row < nb && q == 0) { y[3 * (size_t)row] = s0; y[3 * (size_t)row + 1] = s1; y[3 * (size_t)row + 2] = s2; }
}

/* x as float pairs hi + lo (bit operations), once per matvec: every column
   is read by ~36 block rows */
__global__ void k_split_ff(int n, const double *__restrict__ x, float2 *__restrict__ xs, const GmState *__restrict__ gs)
{
  if (gs && gm_done(gs)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const FF f = ff_split(x[i]);
  xs[i] = make_float2(f.hi, f.lo);
}

/* y = K x for FP32 K and FP64 x on the FP32 pipe: x comes split into float
   pairs (hi + lo, k_split_ff), each product K hi is formed exactly
   (two-product) and summed into a float-float accumulator with two-sum, K lo
   goes to its low part; the half-warp's partial sums are combined as
   float-float and widened to FP64 at the end.  About 47 significant bits
   (K itself carries 24); GB300's FP64 pipe runs at 1/64 of the FP32 rate. */
__global__ void k_bsr_matvec_ff(int nb, const int *__restrict__ rowptr, const int *__restrict__ colind,
                                const float *__restrict__ K, const float2 *__restrict__ xs, double *__restrict__ y,
                                const GmState *__restrict__ gs)
{
  if (gs && gm_done(gs)) return;
  /* one half-warp per block row, lane q taking whole blocks q, q + 16, ... */
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = t >> 4, q = t & 15;
  FF s0(0.f, 0.f), s1(0.f, 0.f), s2(0.f, 0.f);
  if (row < nb) {
    const int k1 = rowptr[row + 1];
    for (int k = rowptr[row] + q; k < k1; k += 16) {
      const int c = colind[k];
      const float *b = K + 9 * (size_t)k;
      const float2 p0 = xs[3 * (size_t)c], p1 = xs[3 * (size_t)c + 1], p2 = xs[3 * (size_t)c + 2];
      const FF x0(p0.x, p0.y), x1(p1.x, p1.y), x2(p2.x, p2.y);
      ff_axpy(s0, b[0], x0); ff_axpy(s0, b[1], x1); ff_axpy(s0, b[2], x2);
      ff_axpy(s1, b[3], x0); ff_axpy(s1, b[4], x1); ff_axpy(s1, b[5], x2);
      ff_axpy(s2, b[6], x0); ff_axpy(s2, b[7], x1); ff_axpy(s2, b[8], x2);
    }
  }
  for (int o = 1; o < 16; o <<= 1) {
    s0 = s0 + FF(__shfl_xor_sync(0xffffffffu, s0.hi, o), __shfl_xor_sync(0xffffffffu, s0.lo, o));
    s1 = s1 + FF(__shfl_xor_sync(0xffffffffu, s1.hi, o), __shfl_xor_sync(0xffffffffu, s1.lo, o));
    s2 = s2 + FF(__shfl_xor_sync(0xffffffffu, s2.hi, o), __shfl_xor_sync(0xffffffffu, s2.lo, o));
  }
  if (row < nb && q == 0) {
    y[3 * (size_t)row] = ff_to_double_bits(s0);
    y[3 * (size_t)row + 1] = ff_to_double_bits(s1);
    y[3 * (size_t)row + 2] = ff_to_double_bits(s2);
  }
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

__global__ void k_bj_apply(int nb, const double *__restrict__ Dinv, const double *__restrict__ r, double *__restrict__ z,
                           const GmState *__restrict__ gs)
{
  if (gs && gm_done(gs)) return;
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

/* ---------------- device-resident GMRES state ---------------- */
struct GmState {
  int done;        /* 1 once the cycle has converged or broken down */
  int jdone;       /* iterations completed in this cycle */
  double bnorm, tol, resid, inv_hn;
};

/* Gram-Schmidt projections.  k_gs_dots forms the partial dot products of w
   with columns 0..nv-1 of V (plus w.w as column nv on the second pass), 8
   columns per grid row and kGsChunks strided row chunks per column; the last
   block to finish (counted on an atomic ticket, the partials made visible by
   a fence) reduces the partials of every column in a fixed order, so the
   result does not depend on block scheduling.  On the second pass the same
   block completes the Arnoldi column: H[:, j] = h1 + h2, the previous Givens
   rotations, a new rotation, the residual estimate and 1/h_{j+1,j}. */
constexpr int kGsChunks = 304;      /* 2 x 152 SMs */
constexpr int kGsCols = 8;
constexpr int kMaxRestart = 200;

__global__ void __launch_bounds__(256) k_gs_dots(int n, int nv, int pass2, const double *__restrict__ V, size_t ld,
                                                 const double *__restrict__ w, double *__restrict__ part,
                                                 unsigned *__restrict__ ticket, double *__restrict__ out,
                                                 const double *__restrict__ h1, int j, int m, double *__restrict__ H,
                                                 double *__restrict__ cs, double *__restrict__ sn,
                                                 double *__restrict__ g, GmState *__restrict__ gs)
{
  if (gs->done) return;
  __shared__ double red[kGsCols][8];
  __shared__ double hs[kMaxRestart + 2];
  __shared__ double col[kMaxRestart + 2], css[kMaxRestart], sns[kMaxRestart];
  __shared__ int last;
  const int ncol = nv + (pass2 ? 1 : 0);
  const int j0 = blockIdx.y * kGsCols;
  const int nj = min(kGsCols, ncol - j0);
  double acc[kGsCols];
#pragma unroll
  for (int k = 0; k < kGsCols; k++) acc[k] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double wi = w[i];
#pragma unroll
    for (int k = 0; k < kGsCols; k++) {
      if (k < nj) {
        const int c = j0 + k;
        const double vi = (c < nv) ? V[(size_t)c * ld + i] : wi;
        acc[k] += vi * wi;
      }
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < kGsCols; k++) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[k][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < nj) {
    double t = 0.0;
    for (int q = 0; q < nw; q++) t += red[threadIdx.x][q];
    part[(size_t)(j0 + threadIdx.x) * gridDim.x + blockIdx.x] = t;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x * gridDim.y - 1;
  __syncthreads();
  if (!last) return;
  /* the last block: fixed-order reduction of every column */
  for (int c = wid; c < ncol; c += nw) {
    double v = 0.0;
    for (int p = lane; p < (int)gridDim.x; p += 32) v += __ldcg(part + (size_t)c * gridDim.x + p);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) hs[c] = v;
  }
  if (threadIdx.x == 0) *ticket = 0u;
  __syncthreads();
  for (int c = threadIdx.x; c < ncol; c += blockDim.x) out[c] = hs[c];
  if (!pass2) return;
  for (int i = threadIdx.x; i <= j; i += blockDim.x) col[i] = h1[i] + hs[i];
  for (int i = threadIdx.x; i < j; i += blockDim.x) { css[i] = cs[i]; sns[i] = sn[i]; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double h2sq = 0.0;
    for (int i = 0; i <= j; i++) h2sq += hs[i] * hs[i];
    const double hn2 = hs[j + 1] - h2sq;       /* w1.w1 - |h2|^2 = |w2|^2 */
    const double hn = hn2 > 0.0 ? sqrt(hn2) : 0.0;
    for (int i = 0; i < j; i++) {
      const double a = col[i], b = col[i + 1];
      col[i] = css[i] * a + sns[i] * b;
      col[i + 1] = -sns[i] * a + css[i] * b;
    }
    const double a = col[j], b = hn;
    const double r = hypot(a, b);
    cs[j] = r > 0 ? a / r : 1.0;
    sn[j] = r > 0 ? b / r : 0.0;
    col[j] = r;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
    gs->resid = fabs(g[j + 1]);
    gs->jdone = j + 1;
    gs->inv_hn = hn > 0.0 ? 1.0 / hn : 0.0;
    if (gs->resid <= gs->tol * gs->bnorm || hn == 0.0 || !(hn == hn)) gs->done = 1;
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= j; i += blockDim.x) H[(size_t)i * m + j] = col[i];
}

__global__ void k_axpy_gm(int n, int nv, const double *__restrict__ V, size_t ld, const double *__restrict__ h,
                          double *__restrict__ w, const GmState *__restrict__ gs)
{
  if (gs->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int j = 0; j < nv; j++) s += V[(size_t)j * ld + i] * h[j];
  w[i] -= s;
}

__device__ __forceinline__ bool gm_done(const GmState *gs) { return gs->done != 0; }

/* Second projection and normalisation in one pass: v = (w - V h) / h_{j+1,j}.
   With nv = 0 it starts a cycle: v0 = r / beta.  Skipped once the cycle has
   converged (the next basis vector is unused).  w and v may be the same
   vector, and v may be a column of V beyond the nv read (no restrict on
   them). */
__global__ void k_gs_update(int n, int nv, const double *V, size_t ld, const double *__restrict__ h,
                            const double *w, double *v, const GmState *__restrict__ gs)
{
  if (gs->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = 0; k < nv; k++) s += V[(size_t)k * ld + i] * h[k];
  v[i] = (w[i] - s) * gs->inv_hn;
}

/* y = H^-1 g over the completed iterations (one thread) */
__global__ void k_backsolve(int m, const double *__restrict__ H, const double *__restrict__ g, double *__restrict__ y,
                            const GmState *__restrict__ gs)
{
  if (threadIdx.x != 0) return;
  const int k = gs->jdone;
  for (int i = k - 1; i >= 0; i--) {
    double s = g[i];
    for (int c = i + 1; c < k; c++) s -= H[(size_t)i * m + c] * y[c];
    y[i] = s / H[(size_t)i * m + i];
  }
}

/* dx += Z y over the completed iterations (flexible GMRES keeps the
   preconditioned directions Z) */
__global__ void k_combine(int n, const double *__restrict__ Z, size_t ld, const double *__restrict__ y,
                          double *__restrict__ dx, const GmState *__restrict__ gs)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = gs->jdone;
  double s = 0.0;
  for (int j = 0; j < k; j++) s += Z[(size_t)j * ld + i] * y[j];
  dx[i] += s;
}

/* cycle start: beta = sqrt(rr), v0 = r / beta, g = (beta, 0, ...), flags reset */
__global__ void k_cycle_start(int m, const double *__restrict__ rr, double *__restrict__ g, GmState *__restrict__ gs)
{
  if (threadIdx.x != 0) return;
  const double beta = sqrt(rr[0]);
  if (gs->bnorm < 0.0) gs->bnorm = beta;       /* first cycle: dx = 0, r = b */
  gs->resid = beta;
  gs->jdone = 0;
  gs->inv_hn = beta > 0.0 ? 1.0 / beta : 0.0;
  gs->done = (beta <= gs->tol * gs->bnorm || beta == 0.0) ? 1 : 0;
  for (int i = 0; i <= m; i++) g[i] = 0.0;
  g[0] = beta;
}

/* solve start: tolerance in, ||b|| unknown until the first cycle */
__global__ void k_solve_begin(double tol, GmState *__restrict__ gs)
{
  if (threadIdx.x != 0) return;
  gs->tol = tol;
  gs->bnorm = -1.0;
  gs->done = 0;
  gs->jdone = 0;
}

/* ---------------- host side ---------------- */
static inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }

/* Host waits of the solver.  A serving worker sets t_blocking_waits so that
   its thread sleeps on a blocking-sync event instead of spinning in
   cudaStreamSynchronize: with one worker per core the spinning threads took
   the cores the other requests' host preparation needed. */
thread_local bool t_blocking_waits = false;

static cudaError_t host_wait(cudaStream_t st, cudaEvent_t evb)
{
  if (t_blocking_waits && evb) {
    cudaError_t e = cudaEventRecord(evb, st);
    return e != cudaSuccess ? e : cudaEventSynchronize(evb);
  }
  return cudaStreamSynchronize(st);
}

/* Page-locked scalars a solver reads back (its GMRES state, one dot product,
   the element status word), from a process-wide free list: freeing
   page-locked memory can synchronise the whole device, which would make
   every request that finishes wait for all the others. */
struct PinnedScalars {
  GmState gs;
  double scal;
  int stat;
};
static std::mutex g_pin_mu;
static std::vector<PinnedScalars *> g_pin_free;

static PinnedScalars *pin_acquire()
{
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    if (!g_pin_free.empty()) {
      PinnedScalars *p = g_pin_free.back();
      g_pin_free.pop_back();
      return p;
    }
  }
  void *p = nullptr;
  return cudaMallocHost(&p, sizeof(PinnedScalars)) == cudaSuccess ? static_cast<PinnedScalars *>(p) : nullptr;
}

static void pin_release(PinnedScalars *p)
{
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_pin_free.push_back(p);
}

struct SolverWork {
  int n = 0, nb = 0, m = 0;
  double *V = nullptr, *Z = nullptr, *w = nullptr, *dinv = nullptr, *part = nullptr;
  double *h1 = nullptr, *h2 = nullptr, *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr, *y = nullptr;
  double *dx = nullptr, *xt = nullptr, *Rt = nullptr, *xh = nullptr;
  GmState *gs = nullptr;
  unsigned *ticket = nullptr;  /* last-block counter of k_gs_dots (returns to 0 after each launch) */
  PinnedScalars *pin = nullptr;   /* the page-locked block of the three below */
  GmState *hgs = nullptr;    /* pinned host copy */
  double *hscal = nullptr;   /* pinned host scalar */
  int *hstat = nullptr;      /* pinned host copy of the element status word */
  cudaEvent_t ev = nullptr;
  cudaEvent_t evb = nullptr; /* blocking-sync event for host_wait */
  /* captured pieces of a restart cycle (start, iteration chunks, end) and
     the arguments they were captured for */
  std::vector<cudaGraphExec_t> gexec;
  const double *g_b = nullptr;
  double *g_dx = nullptr;
  const void *g_K = nullptr;
  const void *g_pc = nullptr;   /* preconditioner the graph was captured with (null: block-Jacobi) */
  cudaStream_t st = nullptr;   /* allocation stream */
  long long bytes = 0;         /* device memory allocated above */
};

/* Restarted flexible GMRES(m), right-preconditioned (multigrid V-cycle or
   block-Jacobi); the Arnoldi process, the Givens rotations and the small
   triangular solve all run on the device.  Kernels skip their work once the
   cycle has converged, so the host enqueues a chunk of iterations ahead and
   reads the convergence flag after each chunk. */
class Gmres {
 public:
  Gmres(const DevMesh &dm, const KParams &kp, bool f32, const void *K, SolverWork &w, AmgHier *amg, cudaStream_t st)
      : dm_(dm), kp_(kp), f32_(f32), K_(K), w_(w), amg_(amg), st_(st) {}

  void matvec(const double *x, double *y, const GmState *gs)
  {
    if (f32_) {
      /* the split x lives in the line search's trial vector, unused while GMRES runs */
      float2 *xs = reinterpret_cast<float2 *>(w_.xt);
      k_split_ff<<<nblk(w_.n, 256), 256, 0, st_>>>(w_.n, x, xs, gs);
      k_bsr_matvec_ff<<<nblk(16LL * w_.nb, 256), 256, 0, st_>>>(w_.nb, dm_.rowptr, dm_.colind, (const float *)K_, xs, y, gs);
    }
    else k_bsr_matvec<double><<<nblk(16LL * w_.nb, 256), 256, 0, st_>>>(w_.nb, dm_.rowptr, dm_.colind, (const double *)K_, x, y, gs);
  }
  /* z = M^-1 r: smoothed-aggregation V-cycle, or block-Jacobi */
  void precond(const double *r, double *z, const GmState *gs)
  {
    if (amg_) amg_apply(amg_, r, z, reinterpret_cast<const int *>(gs), st_);
    else k_bj_apply<<<nblk(w_.nb, 256), 256, 0, st_>>>(w_.nb, w_.dinv, r, z, gs);
  }
  /* a . b into a host double (synchronous) */
  int dot2(const double *a, const double *b, double &out)
  {
    k_multidot<<<dim3(kDotBlocks, 1), 256, 0, st_>>>(w_.n, 1, a, (size_t)w_.n, b, w_.part);
    k_reduce_parts<<<1, 128, 0, st_>>>(1, kDotBlocks, w_.part, w_.h1);
    cudaMemcpyAsync(w_.hscal, w_.h1, sizeof(double), cudaMemcpyDeviceToHost, st_);
    cudaError_t e = host_wait(st_, w_.evb);
    if (e != cudaSuccess) return (int)e;
    out = *w_.hscal;
    return 0;
  }

  /* A restart cycle in three kinds of piece: the start (r = b - K dx,
     ||r||, v_0), the iterations in chunks of kChunk (kernels after
     convergence do nothing), and the end (the triangular solve and
     dx += Z y).  The host reads the convergence state after every chunk, so
     a cycle that converges after a few iterations launches a few chunks, not
     all m iterations.  The tolerance and ||b|| live in the device state, so
     the pieces captured for a set of buffers serve every later cycle. */
  static constexpr int kChunk = 3;

  int nchunks() const { return (w_.m + kChunk - 1) / kChunk; }

  void enqueue_start(const double *b, double *dx)
  {
    const int n = w_.n, m = w_.m;
    GmState *gs = w_.gs;
    matvec(dx, w_.w, nullptr);
    k_axpby<<<nblk(n, 256), 256, 0, st_>>>(n, 1.0, b, -1.0, w_.w);
    k_multidot<<<dim3(kDotBlocks, 1), 256, 0, st_>>>(n, 1, w_.w, (size_t)n, w_.w, w_.part);
    k_reduce_parts<<<1, 128, 0, st_>>>(1, kDotBlocks, w_.part, w_.h1);
    k_cycle_start<<<1, 32, 0, st_>>>(m, w_.h1, w_.g, gs);
    k_gs_update<<<nblk(n, 256), 256, 0, st_>>>(n, 0, w_.V, (size_t)n, w_.h2, w_.w, w_.V, gs);
  }

  /* iterations j0 .. j1-1, then the state to the host */
  void enqueue_iters(int j0, int j1)
  {
    const int n = w_.n, m = w_.m;
    double *V = w_.V;
    GmState *gs = w_.gs;
    const int nch = std::min(kGsChunks, nblk(n, 256));       /* row chunks per column */
    for (int j = j0; j < j1; j++) {
      double *vn = V + (size_t)(j + 1) * n, *zj = w_.Z + (size_t)j * n;
      precond(V + (size_t)j * n, zj, gs);                     /* z_j = M^-1 v_j */
      matvec(zj, vn, gs);                                     /* w = K z_j */
      const dim3 g1(nch, (j + 1 + kGsCols - 1) / kGsCols), g2(nch, (j + 2 + kGsCols - 1) / kGsCols);
      k_gs_dots<<<g1, 256, 0, st_>>>(n, j + 1, 0, V, (size_t)n, vn, w_.part, w_.ticket, w_.h1, nullptr, j, m,
                                     w_.H, w_.cs, w_.sn, w_.g, gs);
      k_axpy_gm<<<nblk(n, 256), 256, 0, st_>>>(n, j + 1, V, (size_t)n, w_.h1, vn, gs);
      k_gs_dots<<<g2, 256, 0, st_>>>(n, j + 1, 1, V, (size_t)n, vn, w_.part, w_.ticket, w_.h2, w_.h1, j, m,
                                     w_.H, w_.cs, w_.sn, w_.g, gs);
      k_gs_update<<<nblk(n, 256), 256, 0, st_>>>(n, j + 1, V, (size_t)n, w_.h2, vn, vn, gs);
    }
    cudaMemcpyAsync(w_.hgs, gs, sizeof(GmState), cudaMemcpyDeviceToHost, st_);
  }

  void enqueue_end(double *dx)
  {
    const int n = w_.n, m = w_.m;
    k_backsolve<<<1, 32, 0, st_>>>(m, w_.H, w_.g, w_.y, w_.gs);
    k_combine<<<nblk(n, 256), 256, 0, st_>>>(n, w_.Z, (size_t)n, w_.y, dx, w_.gs);
    cudaMemcpyAsync(w_.hgs, w_.gs, sizeof(GmState), cudaMemcpyDeviceToHost, st_);
  }

  /* piece p: 0 the start, 1 .. nchunks() the iteration chunks, nchunks() + 1
     the end; launched from its captured graph (enqueued directly on the
     legacy default stream, which cannot be captured) */
  int run_piece(int p, const double *b, double *dx)
  {
    auto enqueue = [&]() {
      if (p == 0) enqueue_start(b, dx);
      else if (p <= nchunks()) enqueue_iters((p - 1) * kChunk, std::min(p * kChunk, w_.m));
      else enqueue_end(dx);
    };
    if (st_ == nullptr) { enqueue(); return (int)cudaGetLastError(); }
    const int npieces = nchunks() + 2;
    if ((int)w_.gexec.size() != npieces || w_.g_b != b || w_.g_dx != dx || w_.g_K != K_ ||
        w_.g_pc != (const void *)amg_) {
      for (cudaGraphExec_t g : w_.gexec) if (g) cudaGraphExecDestroy(g);
      w_.gexec.assign(npieces, nullptr);
      w_.g_b = b; w_.g_dx = dx; w_.g_K = K_; w_.g_pc = amg_;
    }
    if (!w_.gexec[p]) {
      cudaGraph_t graph = nullptr;
      cudaError_t e = cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return (int)e;
      enqueue();
      e = cudaStreamEndCapture(st_, &graph);
      if (e != cudaSuccess) return (int)e;
      e = cudaGraphInstantiate(&w_.gexec[p], graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return (int)e;
    }
    return (int)cudaGraphLaunch(w_.gexec[p], st_);
  }

  /* solve K dx = b (dx zeroed on entry); iterations in *its.  Per cycle: the
     start, iteration chunks until the state says converged (one host
     synchronisation per chunk), the end. */
  int solve(const double *b, double *dx, double rtol, int maxit, int *its, double *relres)
  {
    const int n = w_.n;
    *its = 0;
    *relres = 0.0;
    cudaMemsetAsync(dx, 0, n * sizeof(double), st_);
    k_solve_begin<<<1, 32, 0, st_>>>(rtol, w_.gs);
    int rc = 0;
    while (*its < maxit) {
      if ((rc = run_piece(0, b, dx))) return rc;
      for (int c = 1; c <= nchunks(); c++) {
        if ((rc = run_piece(c, b, dx))) return rc;
        cudaError_t e = host_wait(st_, w_.evb);
        if (e != cudaSuccess) return (int)e;
        if (w_.hgs->done) break;
      }
      if ((rc = run_piece(nchunks() + 1, b, dx))) return rc;
      cudaError_t e = host_wait(st_, w_.evb);
      if (e != cudaSuccess) return (int)e;
      const GmState &h = *w_.hgs;
      *its += h.jdone;
      *relres = h.bnorm > 0.0 ? h.resid / h.bnorm : 0.0;
      if (h.bnorm == 0.0 || h.resid <= rtol * h.bnorm || h.jdone == 0) break;
    }
    return (int)cudaGetLastError();
  }

 private:
  const DevMesh &dm_;
  const KParams &kp_;
  bool f32_;
  const void *K_;
  SolverWork &w_;
  AmgHier *amg_;
  cudaStream_t st_;
};

SolverWork *solver_create(int n, int nb, int m, void *stream, int *rc)
{
  SolverWork *w = new SolverWork();
  w->n = n; w->nb = nb; w->m = m;
  w->st = (cudaStream_t)stream;
  cudaError_t e = cudaSuccess;
  const size_t dn = sizeof(double) * (size_t)n;
  auto A = [&](void **p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMallocAsync(p, bytes, w->st);
    if (e == cudaSuccess) w->bytes += (long long)bytes;
  };
  A((void **)&w->V, dn * (size_t)(m + 1));
  A((void **)&w->Z, dn * (size_t)m); A((void **)&w->w, dn); A((void **)&w->dx, dn); A((void **)&w->xt, dn);
  A((void **)&w->Rt, dn); A((void **)&w->xh, dn);
  A((void **)&w->dinv, sizeof(double) * 9 * (size_t)nb);
  A((void **)&w->part, sizeof(double) * (size_t)(m + 2) * std::max(kDotBlocks, kGsChunks));
  A((void **)&w->h1, sizeof(double) * (m + 2)); A((void **)&w->h2, sizeof(double) * (m + 2));
  A((void **)&w->H, sizeof(double) * (size_t)(m + 1) * m);
  A((void **)&w->cs, sizeof(double) * m); A((void **)&w->sn, sizeof(double) * m);
  A((void **)&w->g, sizeof(double) * (m + 1)); A((void **)&w->y, sizeof(double) * m);
  A((void **)&w->gs, sizeof(GmState));
  A((void **)&w->ticket, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemsetAsync(w->ticket, 0, sizeof(unsigned), w->st);
  if (e == cudaSuccess) {
    w->pin = pin_acquire();
    if (!w->pin) e = cudaErrorMemoryAllocation;
    else { w->hgs = &w->pin->gs; w->hscal = &w->pin->scal; w->hstat = &w->pin->stat; }
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->evb, cudaEventDisableTiming | cudaEventBlockingSync);
  if (e == cudaSuccess) e = cudaStreamSynchronize(w->st);
  *rc = (int)e;
  if (e != cudaSuccess) { solver_destroy(w); return nullptr; }
  return w;
}

void solver_destroy(SolverWork *w)
{
  if (!w) return;
  cudaStream_t st = w->st;
  cudaStreamSynchronize(st);
  void *ptrs[] = {w->V, w->Z, w->w, w->dx, w->xt, w->Rt, w->xh, w->dinv, w->part, w->h1, w->h2, w->H,
                  w->cs, w->sn, w->g, w->y, w->gs, w->ticket};
  for (void *p : ptrs) if (p) cudaFreeAsync(p, st);
  cudaStreamSynchronize(st);
  if (w->ev) cudaEventDestroy(w->ev);
  if (w->evb) cudaEventDestroy(w->evb);
  for (cudaGraphExec_t g : w->gexec) if (g) cudaGraphExecDestroy(g);
  pin_release(w->pin);    /* after the graphs that write into it */
  delete w;
}

double *solver_xbuf(SolverWork *w) { return w->xh; }
int solver_m(const SolverWork *w) { return w->m; }
long long solver_device_bytes(const SolverWork *w) { return w ? w->bytes : 0; }

/* Newton on device data; x is a device vector (updated in place). */
int newton_device(const DevMesh &dm, const KParams &kp, bool f32, void *dK, double *dR, double *x,
                  const BiofemNewtonOptions &o, BiofemNewtonStats &s, SolverWork *wp, AmgHier *amg, cudaStream_t st,
                  ResidualFn residual, JacobianFn jacobian, void *ctx,
                  std::string &err)
{
  const int n = 3 * kp.nt, nb = kp.nt;
  SolverWork &w = *wp;
  Gmres gm(dm, kp, f32, dK, w, amg, st);
  int rc;
  auto norm = [&](const double *v, double &out) -> int {
    double d2 = 0.0;
    int r = gm.dot2(v, v, d2);
    out = std::sqrt(d2);
    return r;
  };
  /* ||R|| of the residual just evaluated, and whether every element's C33
     solve stayed in its domain (status bit 1 clear).  The word is cleared
     after reading; bit 2 (a singular diagonal block, replaced by the
     identity in the preconditioner) needs no action. */
  auto checked_norm = [&](const double *v, double &out, bool &in_domain) -> int {
    cudaMemcpyAsync(w.hstat, dm.status, sizeof(int), cudaMemcpyDeviceToHost, st);
    int r = norm(v, out);                 /* synchronises the stream */
    in_domain = (*w.hstat & 1) == 0;
    if (*w.hstat) cudaMemsetAsync(dm.status, 0, sizeof(int), st);
    return r;
  };
  s = BiofemNewtonStats();
  if ((rc = residual(ctx, x, dR, (void *)st))) { err = "residual"; return rc; }
  s.residual_evals++;
  double rn;
  bool ok = true;
  if ((rc = checked_norm(dR, rn, ok))) { err = "norm"; return rc; }
  if (!ok) { err = "CC3333 too small in the C33 solve at the initial state (ModElemC33, active_strain.c:1676)"; return 72; }
  s.r0 = rn;
  s.rhist[0] = rn;
  const double target = std::max(o.rtol * s.r0, o.atol);
  double eta = 0.3, rn_prev = rn;
  for (int it = 0; it < o.max_newton; it++) {
    if (rn <= o.rtol * s.r0 || rn <= o.atol) { s.converged = 1; break; }
    double ksp_rtol = o.gmres_rtol;
    if (o.forcing == 1) {            /* Eisenstat-Walker, version 2 */
      const double alpha = 1.6180339887498949, gamma = 1.0;
      if (it > 0) {
        double e = gamma * std::pow(rn / rn_prev, alpha);
        const double guard = gamma * std::pow(eta, alpha);
        if (guard > 0.1) e = std::max(e, guard);
        eta = e;
      }
      eta = std::min(eta, 0.9);
      ksp_rtol = std::max(std::max(eta, o.gmres_rtol), std::min(0.9, 0.5 * target / rn));
    }
    rn_prev = rn;
    if ((rc = jacobian(ctx, x, dR, dK, (void *)st))) { err = "jacobian"; return rc; }
    s.jacobian_evals++;
    if (amg) {
      if ((rc = amg_numeric(amg, dK, f32, st))) { err = "multigrid setup"; return rc; }
    } else if (f32) {
      k_bj_setup<float><<<nblk(nb, 256), 256, 0, st>>>(nb, dm.rowptr, dm.colind, (const float *)dK, w.dinv, dm.status);
    } else {
      k_bj_setup<double><<<nblk(nb, 256), 256, 0, st>>>(nb, dm.rowptr, dm.colind, (const double *)dK, w.dinv, dm.status);
    }
    /* rhs = -R */
    k_scale_copy<<<nblk(n, 256), 256, 0, st>>>(n, dR, -1.0, w.Rt);
    int its = 0;
    double relres = 0.0;
    if ((rc = gm.solve(w.Rt, w.dx, ksp_rtol, o.gmres_max_it, &its, &relres))) { err = "gmres"; return rc; }
    s.gmres_its_total += its;
    s.gmres_its_last = its;
    s.gmres_relres_last = relres;
    if (kp.nt > kp.nv) k_zero_ghost<<<nblk(3LL * (kp.nt - kp.nv), 256), 256, 0, st>>>(kp.nv, kp.nt, w.dx);
    /* backtracking on ||R|| */
    double alpha = 1.0, rnew = 0.0;
    for (int ls = 0; ls < 12; ls++) {
      k_scale_copy<<<nblk(n, 256), 256, 0, st>>>(n, x, 1.0, w.xt);
      k_axpby<<<nblk(n, 256), 256, 0, st>>>(n, alpha, w.dx, 1.0, w.xt);
      if ((rc = residual(ctx, w.xt, dR, (void *)st))) { err = "residual"; return rc; }
      s.residual_evals++;
      if ((rc = checked_norm(dR, rnew, ok))) { err = "norm"; return rc; }
      /* a trial state outside the C33 solve's domain is a failed step:
         shorten it, as a line search does on a function-domain error */
      if (!ok) { rnew = INFINITY; alpha *= 0.5; continue; }
      if (!o.line_search || rnew <= (1.0 - 1e-4 * alpha) * rn || !std::isfinite(rn)) break;
      alpha *= 0.5;
    }
    if (!ok) { err = "CC3333 too small in the C33 solve on every trial step (ModElemC33, active_strain.c:1676)"; return 72; }
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
