// fp64_rates.cu -- arithmetic-rate microbenchmark behind the FP64 design choices.
//
// Three kernels, each a fixed grid of independent dependency chains in registers (no memory
// traffic inside the timed loop), timed with CUDA events after a warm-up launch:
//   dfma  : FP64 FMA on the FP64 pipe, 8 independent chains per thread       (2 flop / FMA)
//   dmma  : FP64 tensor-core MMA, mma.sync.aligned.m8n8k4 f64, 4 independent
//           accumulator tiles per warp                                       (512 flop / warp MMA)
//   ffma  : FP32 FMA, 8 independent chains per thread, for scale            (2 flop / FMA)
// Prints one JSON object: TFLOP/s of each and the grid used.
#include <cstdio>
#include <cuda_runtime.h>

#define CK(x)                                                                        \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) {                                                         \
      fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));                       \
      return 1;                                                                      \
    }                                                                                \
  } while (0)

__global__ void k_dfma(double* out, int iters) {
  const double b = 0.999999, c = 1e-7;
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-6 * (threadIdx.x + k);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_ffma(float* out, int iters) {
  const float b = 0.999999f, c = 1e-7f;
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0f + 1e-6f * (threadIdx.x + k);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], b, c);
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// D = A B + C for an 8x8x4 FP64 tile: per thread one A and one B element, two C/D elements
__global__ void k_dmma(double* out, int iters) {
  const int lane = threadIdx.x & 31;
  const double a = 1.0 + 1e-3 * lane, b = 0.5 - 1e-4 * lane;
  double d[4][2];
#pragma unroll
  for (int t = 0; t < 4; ++t) d[t][0] = d[t][1] = 1e-3 * t;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int t = 0; t < 4; ++t)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(d[t][0]), "+d"(d[t][1])
                   : "d"(a), "d"(b));
  double s = 0.0;
#pragma unroll
  for (int t = 0; t < 4; ++t) s += d[t][0] + d[t][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename K, typename T>
static float time_kernel(K k, T* out, int grid, int block, int iters) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k<<<grid, block>>>(out, iters / 8);  // warm-up
  cudaEventRecord(e0);
  k<<<grid, block>>>(out, iters);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

int main() {
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int block = 256, grid = sms * 8, iters = 1 << 16;
  const double threads = (double)grid * block;
  double* d64 = nullptr;
  float* d32 = nullptr;
  CK(cudaMalloc(&d64, sizeof(double) * grid * block));
  CK(cudaMalloc(&d32, sizeof(float) * grid * block));
  const float ms_dfma = time_kernel(k_dfma, d64, grid, block, iters);
  const float ms_ffma = time_kernel(k_ffma, d32, grid, block, iters);
  const float ms_dmma = time_kernel(k_dmma, d64, grid, block, iters);
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  const double f_dfma = threads * iters * 8 * 2, f_ffma = f_dfma;
  const double f_dmma = threads / 32 * iters * 4 * 512.0;
  printf("{\"sms\": %d, \"grid\": %d, \"block\": %d, \"iters\": %d, "
         "\"dfma_tflops\": %.4f, \"dmma_tflops\": %.4f, \"ffma_tflops\": %.4f, "
         "\"dfma_ms\": %.3f, \"dmma_ms\": %.3f, \"ffma_ms\": %.3f}\n",
         sms, grid, block, iters, f_dfma / (ms_dfma * 1e-3) / 1e12, f_dmma / (ms_dmma * 1e-3) / 1e12,
         f_ffma / (ms_ffma * 1e-3) / 1e12, ms_dfma, ms_dmma, ms_ffma);
  cudaFree(d64);
  cudaFree(d32);
  return 0;
}
