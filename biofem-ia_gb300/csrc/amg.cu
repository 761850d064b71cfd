/*
 * Device part of the smoothed-aggregation preconditioner (see amg.h): the
 * numeric setup from the current tangent and the FP32 V-cycle.
 *
 * Vectors on a level are node-major (bs entries per node).  Operator-style
 * kernels give each block row to a half-warp whose lanes take whole blocks;
 * the row result is reduced over the half-warp and one lane applies the
 * row-local update.  Every value is produced by exactly one thread in a fixed
 * order, so the preconditioner is deterministic.  The apply kernels take the
 * Krylov cycle's "done" flag and do nothing once it is set, so a cycle can be
 * enqueued (or replayed as a graph) past its convergence.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "amg.h"

namespace biofem {
namespace {

constexpr int kPowerIts = 12;
constexpr int kRedBlocks = 304;      /* 2 x 152 SMs */

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }

struct LevelPar {        /* device, per level */
  float lambda, theta_inv, c1, c2, omega;
};

/* ---------------- small dense helpers ---------------- */
template <int BS>
__device__ __forceinline__ void load_vec(const float *__restrict__ v, int i, float out[BS])
{
#pragma unroll
  for (int r = 0; r < BS; r++) out[r] = v[(size_t)i * BS + r];
}

/* acc[BS] over the half-warp: sum of A_ik x_k for the row's blocks */
template <int BS>
__device__ __forceinline__ void row_apply(const int *__restrict__ rowptr, const int *__restrict__ colind,
                                          const float *__restrict__ A, const float *__restrict__ x, int row, int q,
                                          bool live, float acc[BS])
{
#pragma unroll
  for (int r = 0; r < BS; r++) acc[r] = 0.f;
  if (live) {
    const int k1 = rowptr[row + 1];
    for (int k = rowptr[row] + q; k < k1; k += 16) {
      const int c = colind[k];
      const float *a = A + (size_t)k * BS * BS;
      float xv[BS], av[BS * BS];
      if constexpr (BS == 6) {
        /* a 6x6 block is 144 bytes and a 6-vector 24 bytes, so the block
           comes in nine 16-byte loads and the vector in three 8-byte ones */
#pragma unroll
        for (int j = 0; j < 9; j++) {
          const float4 v4 = __ldg(reinterpret_cast<const float4 *>(a) + j);
          av[4 * j] = v4.x; av[4 * j + 1] = v4.y; av[4 * j + 2] = v4.z; av[4 * j + 3] = v4.w;
        }
#pragma unroll
        for (int j = 0; j < 3; j++) {
          const float2 v2 = *(reinterpret_cast<const float2 *>(x + (size_t)c * BS) + j);
          xv[2 * j] = v2.x; xv[2 * j + 1] = v2.y;
        }
      } else {
#pragma unroll
        for (int j = 0; j < BS * BS; j++) av[j] = a[j];
#pragma unroll
        for (int s = 0; s < BS; s++) xv[s] = x[(size_t)c * BS + s];
      }
#pragma unroll
      for (int r = 0; r < BS; r++)
#pragma unroll
        for (int s = 0; s < BS; s++) acc[r] = fmaf(av[r * BS + s], xv[s], acc[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < BS; r++)
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
}

template <int BS>
__device__ __forceinline__ void dmul(const float *__restrict__ D, int i, const float in[BS], float out[BS])
{
  const float *d = D + (size_t)i * BS * BS;
#pragma unroll
  for (int r = 0; r < BS; r++) {
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < BS; c++) s = fmaf(d[r * BS + c], in[c], s);
    out[r] = s;
  }
}

__device__ __forceinline__ bool is_done(const int *done) { return done && *(volatile const int *)done; }

/* A prolongation block of BS x 6 floats: the 144-byte blocks of BS = 6 start
   on 16 bytes, the 72-byte blocks of BS = 3 on 8 bytes (cudaMalloc bases,
   whole blocks per index). */
template <int BS>
__device__ __forceinline__ void load_pblock(const float *__restrict__ p, float out[BS * kAmgCoarseBs])
{
  static_assert(kAmgCoarseBs == 6, "block loads assume 6 coarse components");
  if constexpr (BS == 6) {
#pragma unroll
    for (int j = 0; j < 9; j++) {
      const float4 v = __ldg(reinterpret_cast<const float4 *>(p) + j);
      out[4 * j] = v.x; out[4 * j + 1] = v.y; out[4 * j + 2] = v.z; out[4 * j + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < BS * 3; j++) {
      const float2 v = __ldg(reinterpret_cast<const float2 *>(p) + j);
      out[2 * j] = v.x; out[2 * j + 1] = v.y;
    }
  }
}

/* a 6-component node vector (24 bytes, 8-byte aligned) */
__device__ __forceinline__ void load6(const float *__restrict__ v, float out[6])
{
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const float2 w = reinterpret_cast<const float2 *>(v)[j];
    out[2 * j] = w.x; out[2 * j + 1] = w.y;
  }
}

/* ---------------- numeric setup kernels ---------------- */
__global__ void k_to_f32(long long n, const double *__restrict__ a, float *__restrict__ b)
{
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

/* inverse of each diagonal block by Gauss-Jordan with partial pivoting; a
   vanishing pivot leaves that unknown as identity */
template <int BS>
__global__ void k_dinv(int n, const int *__restrict__ diag, const float *__restrict__ A, float *__restrict__ Dinv)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float a[BS][BS], v[BS][BS];
  const int k = diag[i];
  float scale = 0.f;
#pragma unroll
  for (int r = 0; r < BS; r++)
#pragma unroll
    for (int c = 0; c < BS; c++) {
      a[r][c] = k >= 0 ? A[(size_t)k * BS * BS + r * BS + c] : (r == c ? 1.f : 0.f);
      v[r][c] = r == c ? 1.f : 0.f;
      scale = fmaxf(scale, fabsf(a[r][c]));
    }
  if (!(scale > 0.f)) scale = 1.f;
#pragma unroll
  for (int p = 0; p < BS; p++) {
    int piv = p;
    float best = fabsf(a[p][p]);
#pragma unroll
    for (int r = p + 1; r < BS; r++)
      if (fabsf(a[r][p]) > best) { best = fabsf(a[r][p]); piv = r; }
    if (piv != p) {
#pragma unroll
      for (int c = 0; c < BS; c++) {
        float t = a[p][c]; a[p][c] = a[piv][c]; a[piv][c] = t;
        t = v[p][c]; v[p][c] = v[piv][c]; v[piv][c] = t;
      }
    }
    if (!(best > 1e-12f * scale)) {             /* singular direction: identity */
#pragma unroll
      for (int c = 0; c < BS; c++) { a[p][c] = c == p ? 1.f : 0.f; }
    }
    const float inv = 1.f / a[p][p];
#pragma unroll
    for (int c = 0; c < BS; c++) { a[p][c] *= inv; v[p][c] *= inv; }
#pragma unroll
    for (int r = 0; r < BS; r++) {
      if (r == p) continue;
      const float f = a[r][p];
#pragma unroll
      for (int c = 0; c < BS; c++) { a[r][c] = fmaf(-f, a[p][c], a[r][c]); v[r][c] = fmaf(-f, v[p][c], v[r][c]); }
    }
  }
  float *o = Dinv + (size_t)i * BS * BS;
#pragma unroll
  for (int r = 0; r < BS; r++)
#pragma unroll
    for (int c = 0; c < BS; c++) o[r * BS + c] = v[r][c];
}

/* one power-iteration step on D^-1 A: y = D^-1 A x / s_prev (x = a fixed
   pseudo-random vector on the first step), and ||y|| into norm_out via a
   fixed-order last-block reduction */
__device__ __forceinline__ float start_vec(unsigned i)
{
  unsigned h = i * 2654435761u;
  h ^= h >> 15; h *= 2246822519u; h ^= h >> 13;
  return (float)(h & 0xffffu) * (1.f / 32768.f) - 1.f;
}

template <int BS>
__global__ void __launch_bounds__(256) k_power(int n, const int *__restrict__ rowptr, const int *__restrict__ colind,
                                               const float *__restrict__ A, const float *__restrict__ Dinv,
                                               const float *__restrict__ x, const float *__restrict__ s_prev,
                                               float *__restrict__ y, float *__restrict__ part,
                                               unsigned *__restrict__ ticket, float *__restrict__ norm_out)
{
  __shared__ float red[8];
  __shared__ int last;
  const int lane = threadIdx.x & 31, q = threadIdx.x & 15;
  const float s = s_prev ? 1.f / fmaxf(*s_prev, 1e-30f) : 1.f;
  float local = 0.f;
  const int rows_per_pass = gridDim.x * (blockDim.x >> 4);
  const int npass = (n + rows_per_pass - 1) / rows_per_pass;
  for (int pass = 0; pass < npass; pass++) {
    const int row = pass * rows_per_pass + blockIdx.x * (blockDim.x >> 4) + (threadIdx.x >> 4);
    const bool live = row < n;
    float acc[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = 0.f;
    if (live) {
      const int k1 = rowptr[row + 1];
      for (int k = rowptr[row] + q; k < k1; k += 16) {
        const int c = colind[k];
        const float *a = A + (size_t)k * BS * BS;
        float xv[BS];
#pragma unroll
        for (int t = 0; t < BS; t++) xv[t] = x ? x[(size_t)c * BS + t] : start_vec((unsigned)(c * BS + t));
#pragma unroll
        for (int r = 0; r < BS; r++)
#pragma unroll
          for (int t = 0; t < BS; t++) acc[r] = fmaf(a[r * BS + t], xv[t], acc[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < BS; r++)
#pragma unroll
      for (int o = 1; o < 16; o <<= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
    if (live && q == 0) {
      float out[BS];
      dmul<BS>(Dinv, row, acc, out);
#pragma unroll
      for (int r = 0; r < BS; r++) {
        out[r] *= s;
        y[(size_t)row * BS + r] = out[r];
        local = fmaf(out[r], out[r], local);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if (lane == 0) red[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    part[blockIdx.x] = t;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  if (threadIdx.x < 32) {
    float t = 0.f;
    for (int p = threadIdx.x; p < (int)gridDim.x; p += 32) t += __ldcg(part + p);
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) { *norm_out = sqrtf(t); *ticket = 0u; }
  }
}

/* Chebyshev interval [lambda/30, 1.1 lambda] for degree 2, and the
   prolongator damping omega = 4 / (3 lambda) */
__global__ void k_level_params(const float *__restrict__ lam_in, LevelPar *__restrict__ par)
{
  if (threadIdx.x != 0) return;
  const float lam = fmaxf(*lam_in, 1e-20f);
  const float hi = 1.1f * lam, lo = lam / 30.f;
  const float theta = 0.5f * (hi + lo), delta = 0.5f * (hi - lo), sigma = theta / delta;
  const float rho0 = 1.f / sigma, rho1 = 1.f / (2.f * sigma - rho0);
  par->lambda = lam;
  par->theta_inv = 1.f / theta;
  par->c1 = rho1 * rho0;
  par->c2 = 2.f * rho1 / delta;
  par->omega = 4.f / (3.f * lam);
}

/* P_iJ = [agg(i) = J] Q_i - omega D_i^-1 sum_{j in row i, agg(j) = J} A_ij Q_j */
template <int BS>
__global__ void k_pvals(long long nnzp, const int *__restrict__ pblkrow, const int *__restrict__ pcol,
                        const int *__restrict__ rowptr, const int *__restrict__ colind, const float *__restrict__ A,
                        const float *__restrict__ Dinv, const int *__restrict__ agg, const float *__restrict__ Q,
                        const LevelPar *__restrict__ par, float *__restrict__ P)
{
  const long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (b >= nnzp) return;
  constexpr int C = kAmgCoarseBs;
  const int i = pblkrow[b], J = pcol[b];
  float acc[BS][C];
#pragma unroll
  for (int r = 0; r < BS; r++)
#pragma unroll
    for (int c = 0; c < C; c++) acc[r][c] = 0.f;
  for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
    const int j = colind[k];
    if (agg[j] != J) continue;
    const float *a = A + (size_t)k * BS * BS;
    const float *qj = Q + (size_t)j * BS * C;
#pragma unroll
    for (int r = 0; r < BS; r++)
#pragma unroll
      for (int s = 0; s < BS; s++) {
        const float ars = a[r * BS + s];
#pragma unroll
        for (int c = 0; c < C; c++) acc[r][c] = fmaf(ars, qj[s * C + c], acc[r][c]);
      }
  }
  const float om = par->omega;
  const float *d = Dinv + (size_t)i * BS * BS;
  const bool own = agg[i] == J;
  const float *qi = Q + (size_t)i * BS * C;
  float *o = P + (size_t)b * BS * C;
#pragma unroll
  for (int r = 0; r < BS; r++)
#pragma unroll
    for (int c = 0; c < C; c++) {
      float s = 0.f;
#pragma unroll
      for (int t = 0; t < BS; t++) s = fmaf(d[r * BS + t], acc[t][c], s);
      o[r * C + c] = (own ? qi[r * C + c] : 0.f) - om * s;
    }
}

__device__ __forceinline__ int find_col(const int *__restrict__ col, int lo, int hi, int key)
{
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    const int v = col[mid];
    if (v == key) return mid;
    if (v < key) lo = mid + 1; else hi = mid;
  }
  return -1;
}

/* T_iJ = sum_k A_ik P_kJ */
template <int BS>
__global__ void k_tvals(long long nnzt, const int *__restrict__ tblkrow, const int *__restrict__ tcol,
                        const int *__restrict__ rowptr, const int *__restrict__ colind, const float *__restrict__ A,
                        const int *__restrict__ prow, const int *__restrict__ pcol, const float *__restrict__ P,
                        float *__restrict__ T)
{
  const long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (b >= nnzt) return;
  constexpr int C = kAmgCoarseBs;
  const int i = tblkrow[b], J = tcol[b];
  float acc[BS][C];
#pragma unroll
  for (int r = 0; r < BS; r++)
#pragma unroll
    for (int c = 0; c < C; c++) acc[r][c] = 0.f;
  for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
    const int j = colind[k];
    const int pb = find_col(pcol, prow[j], prow[j + 1], J);
    if (pb < 0) continue;
    const float *a = A + (size_t)k * BS * BS;
    const float *p = P + (size_t)pb * BS * C;
#pragma unroll
    for (int r = 0; r < BS; r++)
#pragma unroll
      for (int s = 0; s < BS; s++) {
        const float ars = a[r * BS + s];
#pragma unroll
        for (int c = 0; c < C; c++) acc[r][c] = fmaf(ars, p[s * C + c], acc[r][c]);
      }
  }
  float *o = T + (size_t)b * BS * C;
#pragma unroll
  for (int r = 0; r < BS; r++)
#pragma unroll
    for (int c = 0; c < C; c++) o[r * C + c] = acc[r][c];
}

/* Ac_IJ = sum_{i in P^T row I} P_iI^T T_iJ, plus 1 on the diagonal of dead
   coarse unknowns: one warp per coarse block, lanes take the fine rows in
   turn, fixed xor-tree reduction of the 36 partial sums */
template <int BS>
__global__ void __launch_bounds__(256) k_cvals(long long nnzc, const int *__restrict__ cblkrow, const int *__restrict__ ccol,
                                               const int *__restrict__ rrow, const int *__restrict__ rcol,
                                               const int *__restrict__ rmap, const float *__restrict__ P,
                                               const int *__restrict__ trow, const int *__restrict__ tcol,
                                               const float *__restrict__ T, const unsigned char *__restrict__ dead,
                                               float *__restrict__ Ac)
{
  const long long b = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (b >= nnzc) return;                           /* whole warps leave together */
  constexpr int C = kAmgCoarseBs;
  const int I = cblkrow[b], J = ccol[b];
  float acc[C][C];
#pragma unroll
  for (int r = 0; r < C; r++)
#pragma unroll
    for (int c = 0; c < C; c++) acc[r][c] = 0.f;
  for (int t = rrow[I] + lane; t < rrow[I + 1]; t += 32) {
    const int i = rcol[t];
    const int tb = find_col(tcol, trow[i], trow[i + 1], J);
    if (tb < 0) continue;
    const float *p = P + (size_t)rmap[t] * BS * C;      /* BS x C, used transposed */
    const float *tt = T + (size_t)tb * BS * C;
#pragma unroll
    for (int s = 0; s < BS; s++)
#pragma unroll
      for (int r = 0; r < C; r++) {
        const float psr = p[s * C + r];
#pragma unroll
        for (int c = 0; c < C; c++) acc[r][c] = fmaf(psr, tt[s * C + c], acc[r][c]);
      }
  }
#pragma unroll
  for (int r = 0; r < C; r++)
#pragma unroll
    for (int c = 0; c < C; c++)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[r][c] += __shfl_xor_sync(0xffffffffu, acc[r][c], o);
  if (lane != 0) return;
  if (I == J)
#pragma unroll
    for (int r = 0; r < C; r++)
      if (dead[(size_t)I * C + r]) acc[r][r] += 1.f;
  float *o = Ac + (size_t)b * C * C;
#pragma unroll
  for (int r = 0; r < C; r++)
#pragma unroll
    for (int c = 0; c < C; c++) o[r * C + c] = acc[r][c];
}

/* coarsest operator to a dense row-major N x N matrix (one block) */
template <int BS>
__global__ void k_dense_assemble(int n, const int *__restrict__ rowptr, const int *__restrict__ colind,
                                 const float *__restrict__ A, float *__restrict__ D)
{
  const int N = n * BS;
  for (int t = threadIdx.x; t < N * N; t += blockDim.x) D[t] = 0.f;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
      const int j = colind[k];
      for (int r = 0; r < BS; r++)
        for (int c = 0; c < BS; c++) D[(size_t)(i * BS + r) * N + j * BS + c] = A[(size_t)k * BS * BS + r * BS + c];
    }
}

/* In-place Gauss-Jordan inverse with partial pivoting in shared memory (one
   block, N <= kAmgMaxDense); a vanishing pivot is replaced by 1 */
__global__ void __launch_bounds__(1024) k_dense_invert(int N, float *__restrict__ D)
{
  extern __shared__ float sm[];
  float *a = sm;                       /* N*N */
  float *colk = sm + N * N;            /* N */
  __shared__ int perm[kAmgMaxDense];
  __shared__ int piv_s;
  __shared__ float scale_s;
  for (int t = threadIdx.x; t < N * N; t += blockDim.x) a[t] = D[t];
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int t = 0; t < N * N; t++) s = fmaxf(s, fabsf(a[t]));
    scale_s = s > 0.f ? s : 1.f;
  }
  __syncthreads();
  for (int k = 0; k < N; k++) {
    if (threadIdx.x == 0) {
      int p = k;
      float best = fabsf(a[k * N + k]);
      for (int r = k + 1; r < N; r++)
        if (fabsf(a[r * N + k]) > best) { best = fabsf(a[r * N + k]); p = r; }
      perm[k] = p;
      piv_s = p;
    }
    __syncthreads();
    const int p = piv_s;
    if (p != k)
      for (int c = threadIdx.x; c < N; c += blockDim.x) {
        const float t = a[k * N + c]; a[k * N + c] = a[p * N + c]; a[p * N + c] = t;
      }
    __syncthreads();
    float pv = a[k * N + k];
    if (!(fabsf(pv) > 1e-12f * scale_s)) pv = 1.f;
    const float inv = 1.f / pv;
    __syncthreads();
    for (int c = threadIdx.x; c < N; c += blockDim.x) a[k * N + c] = (c == k ? 1.f : a[k * N + c]) * inv;
    for (int r = threadIdx.x; r < N; r += blockDim.x) colk[r] = r == k ? 0.f : a[r * N + k];
    __syncthreads();
    for (int r = threadIdx.x; r < N; r += blockDim.x)
      if (r != k) a[r * N + k] = 0.f;
    __syncthreads();
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
      const int r = t / N, c = t - r * N;
      if (r != k) a[t] = fmaf(-colk[r], a[k * N + c], a[t]);
    }
    __syncthreads();
  }
  for (int k = N - 1; k >= 0; k--) {
    const int p = perm[k];
    if (p != k)
      for (int r = threadIdx.x; r < N; r += blockDim.x) {
        const float t = a[r * N + k]; a[r * N + k] = a[r * N + p]; a[r * N + p] = t;
      }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < N * N; t += blockDim.x) D[t] = a[t];
}

/* ---------------- V-cycle kernels ---------------- */
__global__ void k_in_f32(int n, const double *__restrict__ v, float *__restrict__ b, const int *done)
{
  if (is_done(done)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)v[i];
}

__global__ void k_out_f64(int n, const float *__restrict__ x, double *__restrict__ z, const int *done)
{
  if (is_done(done)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z[i] = (double)x[i];
}

/* smoothing start from x = 0: r = D^-1 b, d = r / theta */
template <int BS>
__global__ void k_sm_start0(int n, const float *__restrict__ Dinv, const float *__restrict__ b, float *__restrict__ r,
                            float *__restrict__ d, const LevelPar *__restrict__ par, const int *done)
{
  if (is_done(done)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float bv[BS], rv[BS];
  load_vec<BS>(b, i, bv);
  dmul<BS>(Dinv, i, bv, rv);
  const float ti = par->theta_inv;
#pragma unroll
  for (int t = 0; t < BS; t++) { r[(size_t)i * BS + t] = rv[t]; d[(size_t)i * BS + t] = rv[t] * ti; }
}

/* smoothing start from x: r = D^-1 (b - A x), d = r / theta */
template <int BS>
__global__ void __launch_bounds__(256) k_sm_start(int n, const int *__restrict__ rowptr, const int *__restrict__ colind,
                                                  const float *__restrict__ A, const float *__restrict__ Dinv,
                                                  const float *__restrict__ b, const float *__restrict__ x,
                                                  float *__restrict__ r, float *__restrict__ d,
                                                  const LevelPar *__restrict__ par, const int *done)
{
  if (is_done(done)) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = t >> 4, q = t & 15;
  const bool live = row < n;
  float acc[BS];
  row_apply<BS>(rowptr, colind, A, x, row, q, live, acc);
  if (!live || q) return;
  float e[BS], rv[BS];
#pragma unroll
  for (int s = 0; s < BS; s++) e[s] = b[(size_t)row * BS + s] - acc[s];
  dmul<BS>(Dinv, row, e, rv);
  const float ti = par->theta_inv;
#pragma unroll
  for (int s = 0; s < BS; s++) { r[(size_t)row * BS + s] = rv[s]; d[(size_t)row * BS + s] = rv[s] * ti; }
}

/* second Chebyshev step: r1 = r - D^-1 A d, d1 = c1 d + c2 r1,
   x = (init ? 0 : x) + d + d1 */
template <int BS>
__global__ void __launch_bounds__(256) k_sm_step(int n, const int *__restrict__ rowptr, const int *__restrict__ colind,
                                                 const float *__restrict__ A, const float *__restrict__ Dinv,
                                                 const float *__restrict__ r, const float *__restrict__ d,
                                                 float *__restrict__ x, int init, const LevelPar *__restrict__ par,
                                                 const int *done)
{
  if (is_done(done)) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = t >> 4, q = t & 15;
  const bool live = row < n;
  float acc[BS];
  row_apply<BS>(rowptr, colind, A, d, row, q, live, acc);
  if (!live || q) return;
  float u[BS];
  dmul<BS>(Dinv, row, acc, u);
  const float c1 = par->c1, c2 = par->c2;
#pragma unroll
  for (int s = 0; s < BS; s++) {
    const size_t o = (size_t)row * BS + s;
    const float d0 = d[o];
    const float d1 = c1 * d0 + c2 * (r[o] - u[s]);
    x[o] = (init ? 0.f : x[o]) + d0 + d1;
  }
}

/* res = b - A x */
template <int BS>
__global__ void __launch_bounds__(256) k_resid(int n, const int *__restrict__ rowptr, const int *__restrict__ colind,
                                               const float *__restrict__ A, const float *__restrict__ b,
                                               const float *__restrict__ x, float *__restrict__ res, const int *done)
{
  if (is_done(done)) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = t >> 4, q = t & 15;
  const bool live = row < n;
  float acc[BS];
  row_apply<BS>(rowptr, colind, A, x, row, q, live, acc);
  if (!live || q) return;
#pragma unroll
  for (int s = 0; s < BS; s++) res[(size_t)row * BS + s] = b[(size_t)row * BS + s] - acc[s];
}

/* bc_I = sum_{i in P^T row I} P_iI^T res_i: one warp per coarse node, lanes
   take the fine rows in turn and a fixed xor-tree adds their partials */
template <int BS>
__global__ void __launch_bounds__(256) k_restrict(int na, const int *__restrict__ rrow, const int *__restrict__ rcol,
                                                  const int *__restrict__ rmap, const float *__restrict__ P,
                                                  const float *__restrict__ res, float *__restrict__ bc, const int *done)
{
  if (is_done(done)) return;
  const int I = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (I >= na) return;                              /* whole warps leave together */
  constexpr int C = kAmgCoarseBs;
  float acc[C];
#pragma unroll
  for (int c = 0; c < C; c++) acc[c] = 0.f;
  for (int t = rrow[I] + lane; t < rrow[I + 1]; t += 32) {
    const int i = rcol[t];
    float pb[BS * C], rv[BS];
    load_pblock<BS>(P + (size_t)rmap[t] * BS * C, pb);
    if constexpr (BS == 6) {
      load6(res + (size_t)i * BS, rv);
    } else {
#pragma unroll
      for (int s = 0; s < BS; s++) rv[s] = res[(size_t)i * BS + s];
    }
#pragma unroll
    for (int s = 0; s < BS; s++) {
#pragma unroll
      for (int c = 0; c < C; c++) acc[c] = fmaf(pb[s * C + c], rv[s], acc[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < C; c++)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  if (lane < C) {
    float v = acc[0];
#pragma unroll
    for (int c = 1; c < C; c++) if (lane == c) v = acc[c];
    bc[(size_t)I * C + lane] = v;
  }
}

/* x_i += sum_J P_iJ xc_J */
template <int BS>
__global__ void k_prolong(int n, const int *__restrict__ prow, const int *__restrict__ pcol, const float *__restrict__ P,
                          const float *__restrict__ xc, float *__restrict__ x, const int *done)
{
  if (is_done(done)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  constexpr int C = kAmgCoarseBs;
  float acc[BS];
#pragma unroll
  for (int s = 0; s < BS; s++) acc[s] = 0.f;
  for (int k = prow[i]; k < prow[i + 1]; k++) {
    float pb[BS * C], xl[C];
    load_pblock<BS>(P + (size_t)k * BS * C, pb);
    load6(xc + (size_t)pcol[k] * C, xl);
#pragma unroll
    for (int s = 0; s < BS; s++)
#pragma unroll
      for (int c = 0; c < C; c++) acc[s] = fmaf(pb[s * C + c], xl[c], acc[s]);
  }
#pragma unroll
  for (int s = 0; s < BS; s++) x[(size_t)i * BS + s] += acc[s];
}

/* x = D b for the dense coarsest inverse (one block) */
__global__ void k_dense_apply(int N, const float *__restrict__ D, const float *__restrict__ b, float *__restrict__ x,
                              const int *done)
{
  if (is_done(done)) return;
  __shared__ float bs[kAmgMaxDense];
  for (int i = threadIdx.x; i < N; i += blockDim.x) bs[i] = b[i];
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    float s = 0.f;
    for (int j = 0; j < N; j++) s = fmaf(D[(size_t)i * N + j], bs[j], s);
    x[i] = s;
  }
}

}  // namespace

/* ---------------- host side ---------------- */
struct AmgLevelDev {
  int n = 0, bs = 0, na = 0;
  long long nnzA = 0, nnzP = 0, nnzT = 0, nnzC = 0;
  const int *rowptr = nullptr, *colind = nullptr;
  int *diag = nullptr, *agg = nullptr;
  const float *A = nullptr;
  float *Aown = nullptr, *Dinv = nullptr, *Q = nullptr, *P = nullptr, *T = nullptr;
  int *prow = nullptr, *pcol = nullptr, *pblkrow = nullptr;
  int *rrow = nullptr, *rcol = nullptr, *rmap = nullptr;
  int *trow = nullptr, *tcol = nullptr, *tblkrow = nullptr;
  int *cblkrow = nullptr;
  unsigned char *dead = nullptr;
  float *b = nullptr, *x = nullptr, *r = nullptr, *d = nullptr, *y = nullptr;
  LevelPar *par = nullptr;
  float *norms = nullptr;     /* kPowerIts power-iteration norms */
};

struct AmgHier {
  int nt = 0, nl = 0;
  AmgLevelDev L[kAmgMaxLevels];
  bool dense = false;
  int N = 0;
  float *Ad = nullptr;
  float *A0f = nullptr;      /* FP32 copy of an FP64 tangent */
  float *part = nullptr;
  unsigned *ticket = nullptr;
  std::vector<void *> allocs;
  long long bytes = 0;
  cudaStream_t st = nullptr;
  cudaGraph_t num_graph = nullptr;      /* numeric setup, captured for one tangent buffer */
  cudaGraphExec_t num_exec = nullptr;
  const void *num_K = nullptr;
};

namespace {

template <class T>
int dalloc_(AmgHier *h, T **p, size_t count)
{
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMallocAsync((void **)p, count * sizeof(T), h->st);
  if (e != cudaSuccess) return (int)e;
  h->allocs.push_back(*p);
  h->bytes += (long long)(count * sizeof(T));
  return 0;
}

template <class T>
int dup_(AmgHier *h, T **p, const std::vector<T> &v)
{
  int rc = dalloc_(h, p, v.size());
  if (rc || v.empty()) return rc;
  return (int)cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, h->st);
}

template <int BS>
void numeric_level(AmgHier *h, int l, cudaStream_t st)
{
  AmgLevelDev &L = h->L[l];
  k_dinv<BS><<<nblk(L.n, 128), 128, 0, st>>>(L.n, L.diag, L.A, L.Dinv);
  const int grid = std::min(kRedBlocks, nblk(16LL * L.n, 256));
  for (int it = 0; it < kPowerIts; it++) {
    const float *xin = it == 0 ? nullptr : (it & 1 ? L.y : L.r);
    float *yout = it & 1 ? L.r : L.y;
    k_power<BS><<<grid, 256, 0, st>>>(L.n, L.rowptr, L.colind, L.A, L.Dinv, xin, it == 0 ? nullptr : L.norms + it - 1,
                                      yout, h->part, h->ticket, L.norms + it);
  }
  k_level_params<<<1, 32, 0, st>>>(L.norms + kPowerIts - 1, L.par);
  if (l == h->nl - 1) return;
  AmgLevelDev &Cn = h->L[l + 1];
  k_pvals<BS><<<nblk(L.nnzP, 128), 128, 0, st>>>(L.nnzP, L.pblkrow, L.pcol, L.rowptr, L.colind, L.A, L.Dinv, L.agg, L.Q,
                                                 L.par, L.P);
  k_tvals<BS><<<nblk(L.nnzT, 128), 128, 0, st>>>(L.nnzT, L.tblkrow, L.tcol, L.rowptr, L.colind, L.A, L.prow, L.pcol,
                                                 L.P, L.T);
  k_cvals<BS><<<nblk(32LL * L.nnzC, 256), 256, 0, st>>>(L.nnzC, L.cblkrow, Cn.colind, L.rrow, L.rcol, L.rmap, L.P, L.trow,
                                                 L.tcol, L.T, L.dead, Cn.Aown);
}

template <int BS>
void smooth_down(AmgHier *h, int l, const int *done, cudaStream_t st)
{
  AmgLevelDev &L = h->L[l];
  k_sm_start0<BS><<<nblk(L.n, 128), 128, 0, st>>>(L.n, L.Dinv, L.b, L.r, L.d, L.par, done);
  k_sm_step<BS><<<nblk(16LL * L.n, 256), 256, 0, st>>>(L.n, L.rowptr, L.colind, L.A, L.Dinv, L.r, L.d, L.x, 1, L.par, done);
}

template <int BS>
void smooth_up(AmgHier *h, int l, const int *done, cudaStream_t st)
{
  AmgLevelDev &L = h->L[l];
  k_sm_start<BS><<<nblk(16LL * L.n, 256), 256, 0, st>>>(L.n, L.rowptr, L.colind, L.A, L.Dinv, L.b, L.x, L.r, L.d, L.par,
                                                        done);
  k_sm_step<BS><<<nblk(16LL * L.n, 256), 256, 0, st>>>(L.n, L.rowptr, L.colind, L.A, L.Dinv, L.r, L.d, L.x, 0, L.par, done);
}

template <int BS>
void down_to_coarse(AmgHier *h, int l, const int *done, cudaStream_t st)
{
  AmgLevelDev &L = h->L[l];
  AmgLevelDev &Cn = h->L[l + 1];
  smooth_down<BS>(h, l, done, st);
  k_resid<BS><<<nblk(16LL * L.n, 256), 256, 0, st>>>(L.n, L.rowptr, L.colind, L.A, L.b, L.x, L.y, done);
  k_restrict<BS><<<nblk(32LL * L.na, 256), 256, 0, st>>>(L.na, L.rrow, L.rcol, L.rmap, L.P, L.y, Cn.b, done);
}

template <int BS>
void up_from_coarse(AmgHier *h, int l, const int *done, cudaStream_t st)
{
  AmgLevelDev &L = h->L[l];
  AmgLevelDev &Cn = h->L[l + 1];
  k_prolong<BS><<<nblk(L.n, 128), 128, 0, st>>>(L.n, L.prow, L.pcol, L.P, Cn.x, L.x, done);
  smooth_up<BS>(h, l, done, st);
}

}  // namespace

AmgHier *amg_create(int nt, const std::vector<int> &rowptr, const std::vector<int> &colind,
                    const std::vector<unsigned char> &rowkind, const std::vector<double> &X, const int *tri, int ntri,
                    const int *d_rowptr, const int *d_colind, bool k_is_f32, cudaStream_t st, int *rc)
{
  std::vector<AmgLevelHost> H;
  const int nl = amg_symbolic(nt, rowptr, colind, rowkind, X, tri, ntri, H);
  AmgHier *h = new AmgHier();
  h->nt = nt;
  h->nl = nl;
  h->st = st;
  int e = 0;
  for (int l = 0; l < nl && !e; l++) {
    const AmgLevelHost &S = H[l];
    AmgLevelDev &L = h->L[l];
    L.n = S.n; L.bs = S.bs; L.na = (l < nl - 1) ? S.na : 0;
    L.nnzA = (long long)S.colind.size();
    if (l == 0) { L.rowptr = d_rowptr; L.colind = d_colind; }
    const size_t nv = (size_t)S.n * S.bs;
    if (!e) e = dup_(h, &L.diag, S.diag);
    if (!e) e = dalloc_(h, &L.Dinv, (size_t)S.n * S.bs * S.bs);
    if (!e) e = dalloc_(h, &L.b, nv);
    if (!e) e = dalloc_(h, &L.x, nv);
    if (!e) e = dalloc_(h, &L.r, nv);
    if (!e) e = dalloc_(h, &L.d, nv);
    if (!e) e = dalloc_(h, &L.y, nv);
    if (!e) e = dalloc_(h, &L.par, 1);
    if (!e) e = dalloc_(h, &L.norms, kPowerIts);
    if (l < nl - 1) {
      L.nnzP = (long long)S.pcol.size();
      L.nnzT = (long long)S.tcol.size();
      L.nnzC = (long long)S.ccol.size();
      if (!e) e = dup_(h, &L.agg, S.agg);
      if (!e) e = dup_(h, &L.Q, S.Q);
      if (!e) e = dup_(h, &L.prow, S.prow);
      if (!e) e = dup_(h, &L.pcol, S.pcol);
      if (!e) e = dup_(h, &L.pblkrow, S.pblkrow);
      if (!e) e = dup_(h, &L.rrow, S.rrow);
      if (!e) e = dup_(h, &L.rcol, S.rcol);
      if (!e) e = dup_(h, &L.rmap, S.rmap);
      if (!e) e = dup_(h, &L.trow, S.trow);
      if (!e) e = dup_(h, &L.tcol, S.tcol);
      if (!e) e = dup_(h, &L.tblkrow, S.tblkrow);
      if (!e) e = dup_(h, &L.cblkrow, S.cblkrow);
      if (!e) e = dup_(h, &L.dead, S.dead);
      if (!e) e = dalloc_(h, &L.P, (size_t)L.nnzP * S.bs * kAmgCoarseBs);
      if (!e) e = dalloc_(h, &L.T, (size_t)L.nnzT * S.bs * kAmgCoarseBs);
    }
    if (l > 0) {
      int *rp = nullptr, *ci = nullptr;
      if (!e) e = dup_(h, &rp, S.rowptr);
      if (!e) e = dup_(h, &ci, S.colind);
      L.rowptr = rp; L.colind = ci;
      if (!e) e = dalloc_(h, &L.Aown, (size_t)L.nnzA * S.bs * S.bs);
      L.A = L.Aown;
    }
  }
  const AmgLevelDev &Lc = h->L[nl - 1];
  h->N = Lc.n * Lc.bs;
  h->dense = h->N <= kAmgMaxDense;
  if (!e && h->dense) e = dalloc_(h, &h->Ad, (size_t)h->N * h->N);
  if (!e && !k_is_f32) e = dalloc_(h, &h->A0f, (size_t)h->L[0].nnzA * 9);
  if (!e) e = dalloc_(h, &h->part, kRedBlocks);
  if (!e) e = dalloc_(h, &h->ticket, 1);
  if (!e) e = (int)cudaMemsetAsync(h->ticket, 0, sizeof(unsigned), st);
  if (!e && h->dense) {
    /* one limit for every hierarchy (handles on other threads launch the
       same kernel): the largest dense size */
    const size_t smem = ((size_t)kAmgMaxDense * kAmgMaxDense + kAmgMaxDense) * sizeof(float);
    e = (int)cudaFuncSetAttribute(k_dense_invert, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  if (!e) e = (int)cudaStreamSynchronize(st);
  *rc = e;
  if (e) { amg_destroy(h); return nullptr; }
  return h;
}

void amg_destroy(AmgHier *h)
{
  if (!h) return;
  cudaStreamSynchronize(h->st);
  if (h->num_exec) cudaGraphExecDestroy(h->num_exec);
  if (h->num_graph) cudaGraphDestroy(h->num_graph);
  for (void *p : h->allocs) cudaFreeAsync(p, h->st);
  cudaStreamSynchronize(h->st);
  delete h;
}

int amg_levels(const AmgHier *h) { return h ? h->nl : 0; }
long long amg_device_bytes(const AmgHier *h) { return h ? h->bytes : 0; }

static void enqueue_numeric(AmgHier *h, const void *K, bool k_is_f32, cudaStream_t st)
{
  AmgLevelDev &L0 = h->L[0];
  if (k_is_f32) {
    L0.A = (const float *)K;
  } else {
    const long long nv = L0.nnzA * 9;
    k_to_f32<<<nblk(nv, 256), 256, 0, st>>>(nv, (const double *)K, h->A0f);
    L0.A = h->A0f;
  }
  for (int l = 0; l < h->nl; l++) {
    if (h->L[l].bs == 3) numeric_level<3>(h, l, st);
    else numeric_level<6>(h, l, st);
  }
  if (h->dense) {
    const AmgLevelDev &Lc = h->L[h->nl - 1];
    if (Lc.bs == 3) k_dense_assemble<3><<<1, 256, 0, st>>>(Lc.n, Lc.rowptr, Lc.colind, Lc.A, h->Ad);
    else k_dense_assemble<6><<<1, 256, 0, st>>>(Lc.n, Lc.rowptr, Lc.colind, Lc.A, h->Ad);
    const size_t smem = ((size_t)h->N * h->N + h->N) * sizeof(float);
    k_dense_invert<<<1, 1024, smem, st>>>(h->N, h->Ad);
  }
}

/* The numeric setup is a fixed launch sequence over fixed buffers, so it is
   captured once per tangent buffer and replayed for every new tangent. */
int amg_numeric(AmgHier *h, const void *K, bool k_is_f32, cudaStream_t st)
{
  if (!k_is_f32 && !h->A0f) return (int)cudaErrorInvalidValue;
  if (st == nullptr) {                         /* the legacy default stream cannot be captured */
    enqueue_numeric(h, K, k_is_f32, st);
    return (int)cudaGetLastError();
  }
  if (!h->num_exec || h->num_K != K) {
    if (h->num_exec) { cudaGraphExecDestroy(h->num_exec); h->num_exec = nullptr; }
    if (h->num_graph) { cudaGraphDestroy(h->num_graph); h->num_graph = nullptr; }
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return (int)e;
    enqueue_numeric(h, K, k_is_f32, st);
    e = cudaStreamEndCapture(st, &h->num_graph);
    if (e != cudaSuccess) return (int)e;
    e = cudaGraphInstantiate(&h->num_exec, h->num_graph, 0);
    if (e != cudaSuccess) return (int)e;
    h->num_K = K;
  }
  return (int)cudaGraphLaunch(h->num_exec, st);
}

void amg_apply(AmgHier *h, const double *v, double *z, const int *done, cudaStream_t st)
{
  const int nl = h->nl;
  AmgLevelDev &L0 = h->L[0];
  const int n0 = L0.n * L0.bs;
  k_in_f32<<<nblk(n0, 256), 256, 0, st>>>(n0, v, L0.b, done);
  for (int l = 0; l < nl - 1; l++) {
    if (h->L[l].bs == 3) down_to_coarse<3>(h, l, done, st);
    else down_to_coarse<6>(h, l, done, st);
  }
  AmgLevelDev &Lc = h->L[nl - 1];
  if (h->dense) {
    k_dense_apply<<<1, 256, 0, st>>>(h->N, h->Ad, Lc.b, Lc.x, done);
  } else if (Lc.bs == 3) {
    smooth_down<3>(h, nl - 1, done, st);
    smooth_up<3>(h, nl - 1, done, st);
  } else {
    smooth_down<6>(h, nl - 1, done, st);
    smooth_up<6>(h, nl - 1, done, st);
  }
  for (int l = nl - 2; l >= 0; l--) {
    if (h->L[l].bs == 3) up_from_coarse<3>(h, l, done, st);
    else up_from_coarse<6>(h, l, done, st);
  }
  k_out_f64<<<nblk(n0, 256), 256, 0, st>>>(n0, L0.x, z, done);
}

}  // namespace biofem
