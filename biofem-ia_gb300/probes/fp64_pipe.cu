/*
 * FP64 pipe probe: the FP64 FMA rate of this GPU by two routes, so that the
 * roofline of the FP64 element kernels is taken against a measured figure.
 *
 *   dfma   every thread runs 8 independent fma() chains (DFMA instructions);
 *   dmma   every warp runs 4 independent mma.sync.m8n8k4 f64 chains (the FP64
 *          tensor-core instruction; 2*8*8*4 = 512 flops per warp instruction);
 *   mixed  half the warps of each block take the dfma loop, half the dmma loop.
 *
 * Each kernel writes one value per thread (so nothing is dead code) and is
 * timed with CUDA events after a warm-up.  The grid is 152 SMs x 8 blocks of
 * 256 threads.  Prints one JSON line.
 *
 *   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fp64_pipe fp64_pipe.cu && ./fp64_pipe
 */
#include <cstdio>
#include <cuda_runtime.h>

#define CK(x)                                                                    \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return 1;                                                                  \
    }                                                                            \
  } while (0)

constexpr int kIters = 4096;

__device__ __forceinline__ void dfma_loop(double seed, double *out)
{
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = seed + k;
  const double b = 0.999999, c = 1e-9;
  for (int i = 0; i < kIters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  *out = s;
}

__device__ __forceinline__ void dmma_loop(double seed, double *out)
{
  /* m8n8k4: A one double per lane, B one double per lane, C/D two per lane */
  double a = seed, b = 1.0 - seed * 1e-6;
  double c[4][2];
#pragma unroll
  for (int k = 0; k < 4; k++) { c[k][0] = k; c[k][1] = -k; }
  for (int i = 0; i < kIters / 4; i++) {
#pragma unroll
    for (int k = 0; k < 4; k++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 4; k++) s += c[k][0] + c[k][1];
  *out = s;
}

__global__ void k_dfma(double *out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  dfma_loop(1e-3 * t, out + t);
}

__global__ void k_dmma(double *out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  dmma_loop(1e-3 * (t & 31), out + t);
}

__global__ void k_mixed(double *out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if ((threadIdx.x >> 5) & 1) dmma_loop(1e-3 * (t & 31), out + t);
  else dfma_loop(1e-3 * t, out + t);
}

int main()
{
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int threads = 256, blocks = sms * 8, n = blocks * threads, warps = n / 32;
  double *out = nullptr;
  CK(cudaMalloc(&out, sizeof(double) * n));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  /* flops per launch: dfma 2 per fma; dmma 512 per warp instruction */
  const double f_dfma = 2.0 * 8 * kIters * n;
  const double f_dmma = 512.0 * 4 * (kIters / 4) * warps;
  const double f_mixed = 0.5 * f_dfma + 0.5 * f_dmma;
  void (*kern[3])(double *) = {k_dfma, k_dmma, k_mixed};
  const double flops[3] = {f_dfma, f_dmma, f_mixed};
  const char *name[3] = {"dfma", "dmma", "mixed"};
  double best[3];
  for (int k = 0; k < 3; k++) {
    for (int w = 0; w < 3; w++) kern[k]<<<blocks, threads>>>(out);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    best[k] = 1e30;
    for (int r = 0; r < 10; r++) {
      CK(cudaEventRecord(e0));
      kern[k]<<<blocks, threads>>>(out);
      CK(cudaEventRecord(e1));
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best[k]) best[k] = ms;
    }
  }
  printf("{\"sms\": %d, \"blocks\": %d, \"threads\": %d", sms, blocks, threads);
  for (int k = 0; k < 3; k++)
    printf(", \"%s_ms\": %.4f, \"%s_tflops\": %.4f", name[k], best[k], name[k], flops[k] / (best[k] * 1e-3) / 1e12);
  printf("}\n");
  CK(cudaFree(out));
  return 0;
}
