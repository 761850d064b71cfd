/*
 * Tensor-core probe for the FP32 row contraction of the tangent assembly.
 *
 * The core of k_row_assemble_f32: for one row, chunks of 4 contributions; a
 * contribution carries w (9 x 5: entry q = 3i + j, basis row s) and, for
 * each of the row's 32 blocks k, a basis column N[.][b] picked through an
 * inverse map (b = inv[k], or no column); the row's output is
 *   out[q][k] = sum over contributions of sum_s w[q][s] N[s][inv[k]].
 * Three forms of that sum, each one warp per row, same inputs:
 *   fma   lane k owns block k: 45 FFMA per contribution into a per-chunk
 *         partial sum, Kahan-added into the row once per chunk (the library's
 *         form);
 *   tf32  the chunk as one product A (16 x 24: the 9 w rows over the 4 x 5
 *         (contribution, basis row) pairs) times B (24 x 32: the picked
 *         columns), mma.sync.m16n8k8 TF32 with FP32 accumulators carried
 *         across chunks (12 MMAs per chunk);
 *   3xtf32 the same with each operand split into a TF32 head and tail,
 *         A_h B_h + A_h B_t + A_t B_h (36 MMAs per chunk).
 * Each form's error is measured against an FP64 sum on the host.  Prints one
 * JSON line.
 *
 *   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o row_contract_tc row_contract_tc.cu && ./row_contract_tc
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <cuda_runtime.h>

#define CK(x)                                                                    \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return 1;                                                                  \
    }                                                                            \
  } while (0)

constexpr int kRows = 49152;      /* C2 has 49,601 rows */
constexpr int kChunks = 3;        /* 12 contributions per row */
constexpr int kPc = 4;            /* contributions per chunk */
constexpr int kBlocks = 32;       /* blocks per row */
constexpr int kSlots = 16;        /* basis table columns */
constexpr int kWarps = 4;

/* inputs per (row, chunk): w [kPc][9][8] floats (s < 5 used) and inv [kPc][32] bytes (255 = none) */
struct Inputs {
  const float *w;
  const unsigned char *inv;
  const float *tab;   /* [kSlots][8]: N[s][b] at 8 b + s */
};

__device__ __forceinline__ uint32_t to_tf32(float x)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float c[4], const uint32_t a[4], const uint32_t b[2])
{
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
               "{%0, %1, %2, %3};\n"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(32 * kWarps) k_fma(Inputs in, float *out)
{
  __shared__ __align__(16) float ws[kWarps][kPc * 9 * 8];
  __shared__ __align__(16) float tabs[kSlots * 8];
  for (int t = threadIdx.x; t < kSlots * 8; t += blockDim.x) tabs[t] = in.tab[t];
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int row = blockIdx.x * kWarps + wid;
  if (row >= kRows) return;
  float *wT = ws[wid];
  float acc[9], comp[9];
  for (int q = 0; q < 9; q++) { acc[q] = 0.f; comp[q] = 0.f; }
  for (int ch = 0; ch < kChunks; ch++) {
    const size_t base = (size_t)row * kChunks + ch;
    const float4 *src = reinterpret_cast<const float4 *>(in.w + base * kPc * 72);
    for (int u = lane; u < kPc * 18; u += 32) reinterpret_cast<float4 *>(wT)[u] = src[u];
    __syncwarp();
    float tmp[9];
    for (int q = 0; q < 9; q++) tmp[q] = 0.f;
    for (int pc = 0; pc < kPc; pc++) {
      const int b = in.inv[base * kPc * 32 + pc * 32 + lane];
      if (b != 255) {
        const float4 n4 = *reinterpret_cast<const float4 *>(tabs + 8 * b);
        const float n[5] = {n4.x, n4.y, n4.z, n4.w, tabs[8 * b + 4]};
#pragma unroll
        for (int q = 0; q < 9; q++) {
          const float *wq = wT + 72 * pc + 8 * q;
          const float4 w4 = *reinterpret_cast<const float4 *>(wq);
          float t = tmp[q];
          t = fmaf(n[0], w4.x, t); t = fmaf(n[1], w4.y, t); t = fmaf(n[2], w4.z, t); t = fmaf(n[3], w4.w, t);
          tmp[q] = fmaf(n[4], wq[4], t);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 9; q++) {
      const float y = tmp[q] - comp[q];
      const float t = acc[q] + y;
      comp[q] = (t - acc[q]) - y;
      acc[q] = t;
    }
    __syncwarp();
  }
  for (int q = 0; q < 9; q++) out[((size_t)row * 9 + q) * kBlocks + lane] = acc[q];
}

/* A = w rows (16 x 24, q < 9 used; column kk = 5 pc + s, kk < 20 used),
   B = picked columns (24 x 32, B[5 pc + s][k] = N[s][inv_pc[k]]).
   Fragments of m16n8k8 (g = lane / 4, t = lane % 4):
   a0 (g, t), a1 (g + 8, t), a2 (g, t + 4), a3 (g + 8, t + 4);
   b0 (t, g), b1 (t + 4, g) of the 8 x 8 tile; c0/c1 (g, 2t / 2t + 1), c2/c3 (g + 8, ...). */
template <int SPLIT>
__global__ void __launch_bounds__(32 * kWarps) k_tc(Inputs in, float *out)
{
  __shared__ __align__(16) float ws[kWarps][kPc * 9 * 8];
  __shared__ float bs[kWarps][24][40];   /* row stride 40: fragment loads hit 32 distinct banks */
  __shared__ __align__(16) float tabs[kSlots * 8];
  for (int t = threadIdx.x; t < kSlots * 8; t += blockDim.x) tabs[t] = in.tab[t];
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int row = blockIdx.x * kWarps + wid;
  if (row >= kRows) return;
  const int g = lane >> 2, t = lane & 3;
  float *wT = ws[wid];
  float (*B)[40] = bs[wid];
  for (int r = 20; r < 24; r++) B[r][lane] = 0.f;   /* rows 20..23 (padding of K = 20 to 24): zero once */
  float c[4][4];
  for (int n = 0; n < 4; n++) for (int k = 0; k < 4; k++) c[n][k] = 0.f;
  for (int ch = 0; ch < kChunks; ch++) {
    const size_t base = (size_t)row * kChunks + ch;
    const float4 *src = reinterpret_cast<const float4 *>(in.w + base * kPc * 72);
    for (int u = lane; u < kPc * 18; u += 32) reinterpret_cast<float4 *>(wT)[u] = src[u];
    /* column k = lane of B: the picked basis column of each contribution */
    for (int pc = 0; pc < kPc; pc++) {
      const int b = in.inv[base * kPc * 32 + pc * 32 + lane];
#pragma unroll
      for (int s = 0; s < 5; s++) B[5 * pc + s][lane] = b != 255 ? tabs[8 * b + s] : 0.f;
    }
    __syncwarp();
#pragma unroll
    for (int ks = 0; ks < 3; ks++) {
      float af[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const int q = g + (r & 1) * 8, kk = 8 * ks + t + (r >> 1) * 4;
        const int pc = kk / 5, s = kk - 5 * pc;
        af[r] = (q < 9 && kk < 20) ? wT[72 * pc + 8 * q + s] : 0.f;
      }
      uint32_t ah[4], al[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        ah[r] = to_tf32(af[r]);
        if (SPLIT) al[r] = to_tf32(af[r] - __uint_as_float(ah[r]));
      }
#pragma unroll
      for (int n = 0; n < 4; n++) {
        const float b0 = B[8 * ks + t][8 * n + g], b1 = B[8 * ks + t + 4][8 * n + g];
        uint32_t bh[2] = {to_tf32(b0), to_tf32(b1)};
        mma_tf32(c[n], ah, bh);
        if (SPLIT) {
          uint32_t bl[2] = {to_tf32(b0 - __uint_as_float(bh[0])), to_tf32(b1 - __uint_as_float(bh[1]))};
          mma_tf32(c[n], ah, bl);
          mma_tf32(c[n], al, bh);
        }
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int n = 0; n < 4; n++)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int q = g + (k >> 1) * 8, col = 8 * n + 2 * t + (k & 1);
      if (q < 9) out[((size_t)row * 9 + q) * kBlocks + col] = c[n][k];
    }
}

int main()
{
  const size_t nch = (size_t)kRows * kChunks;
  std::vector<float> w(nch * kPc * 72, 0.f), tab(kSlots * 8, 0.f);
  std::vector<unsigned char> inv(nch * kPc * 32, 255);
  uint64_t st = 88172645463325252ull;
  auto rnd = [&]() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return (double)(st >> 11) / 9007199254740992.0; };
  for (int b = 0; b < kSlots; b++)
    for (int s = 0; s < 5; s++) tab[8 * b + s] = (float)(2 * rnd() - 1);
  for (size_t c = 0; c < nch * kPc; c++) {
    for (int q = 0; q < 9; q++)
      for (int s = 0; s < 5; s++) w[c * 72 + 8 * q + s] = (float)(2 * rnd() - 1);
    /* 12 of the 32 blocks get a column, as a regular patch does */
    int used = 0;
    for (int k = 0; k < 32 && used < 12; k++)
      if (rnd() < 0.45) inv[c * 32 + k] = (unsigned char)(used++);
  }
  float *dw, *dtab, *dout;
  unsigned char *dinv;
  CK(cudaMalloc(&dw, w.size() * 4));
  CK(cudaMalloc(&dtab, tab.size() * 4));
  CK(cudaMalloc(&dinv, inv.size()));
  CK(cudaMalloc(&dout, (size_t)kRows * 9 * kBlocks * 4));
  CK(cudaMemcpy(dw, w.data(), w.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dtab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dinv, inv.data(), inv.size(), cudaMemcpyHostToDevice));
  Inputs in{dw, dinv, dtab};
  /* FP64 reference for the first 2048 rows */
  const int nref = 2048;
  std::vector<double> ref((size_t)nref * 9 * kBlocks, 0.0);
  double scale = 0.0;
  for (int r = 0; r < nref; r++)
    for (int ch = 0; ch < kChunks; ch++)
      for (int pc = 0; pc < kPc; pc++) {
        const size_t c = ((size_t)r * kChunks + ch) * kPc + pc;
        for (int k = 0; k < 32; k++) {
          const int b = inv[c * 32 + k];
          if (b == 255) continue;
          for (int q = 0; q < 9; q++) {
            double v = 0.0;
            for (int s = 0; s < 5; s++) v += (double)w[c * 72 + 8 * q + s] * (double)tab[8 * b + s];
            ref[((size_t)r * 9 + q) * kBlocks + k] += v;
          }
        }
      }
  for (double v : ref) scale = std::fmax(scale, std::fabs(v));
  const int grid = kRows / kWarps;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const char *names[3] = {"fma", "tf32", "3xtf32"};
  printf("{\"rows\": %d, \"contributions_per_row\": %d, \"blocks_per_row\": %d", kRows, kChunks * kPc, kBlocks);
  std::vector<float> h((size_t)kRows * 9 * kBlocks);
  for (int v = 0; v < 3; v++) {
    auto launch = [&]() {
      if (v == 0) k_fma<<<grid, 32 * kWarps>>>(in, dout);
      else if (v == 1) k_tc<0><<<grid, 32 * kWarps>>>(in, dout);
      else k_tc<1><<<grid, 32 * kWarps>>>(in, dout);
    };
    for (int i = 0; i < 3; i++) launch();
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    float best = 1e30f;
    for (int i = 0; i < 20; i++) {
      CK(cudaEventRecord(e0));
      launch();
      CK(cudaEventRecord(e1));
      CK(cudaEventSynchronize(e1));
      float ms;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      best = std::fmin(best, ms);
    }
    CK(cudaMemcpy(h.data(), dout, h.size() * 4, cudaMemcpyDeviceToHost));
    double err = 0.0;
    for (size_t i = 0; i < ref.size(); i++) err = std::fmax(err, std::fabs((double)h[i] - ref[i]));
    printf(", \"%s_ms\": %.4f, \"%s_max_err_rel\": %.3e", names[v], best, names[v], err / scale);
  }
  printf("}\n");
  CK(cudaFree(dw));
  CK(cudaFree(dtab));
  CK(cudaFree(dinv));
  CK(cudaFree(dout));
  return 0;
}
