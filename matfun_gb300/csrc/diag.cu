// diag.cu -- the FP64 fused-multiply-add throughput of the current GPU: the denominator of the FP64 roofline that
// bounds the FP64 kernels of this library (reported by the benchmark beside the HBM one).
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/matfun_cuda.h"

namespace {
constexpr int CHAINS = 8, ITER = 2048;

__global__ void dfma_chains(double *out, double a, double b) {
  double x[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; c++) x[c] = threadIdx.x + c;
  for (int i = 0; i < ITER; i++) {
#pragma unroll
    for (int c = 0; c < CHAINS; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CHAINS; c++) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" int matfun_cuda_fp64_peak(double *tflops) {
  if (!tflops) return -1;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return -2;
  const int blocks = sms * 8, threads = 256;
  double *buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return -2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dfma_chains<<<blocks, threads>>>(buf, 0.999, 1e-3);  // warm-up
  cudaEventRecord(e0);
  dfma_chains<<<blocks, threads>>>(buf, 0.999, 1e-3);
  cudaEventRecord(e1);
  float ms = 0.f;
  const cudaError_t e = cudaEventSynchronize(e1);
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (e != cudaSuccess || ms <= 0.f) return -2;
  *tflops = 2.0 * CHAINS * ITER * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return 0;
}
