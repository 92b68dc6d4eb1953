// diag.cu -- the fused-multiply-add throughput of the current GPU in FP64 and FP32: the denominators of the pipe
// rooflines of this library's kernels (the FP64 kernels are bound by the FP64 pipe; the benchmark reports both
// fractions beside the HBM one).
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/matfun_cuda.h"

namespace {
constexpr int CHAINS = 8, ITER = 2048;

// CHAINS independent FMA chains per thread, ITER steps each: 2 * CHAINS * ITER flop per thread
template <typename T>
__global__ void fma_chains(T *out, T a, T b) {
  T x[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; c++) x[c] = (T)(threadIdx.x + c);
  for (int i = 0; i < ITER; i++) {
#pragma unroll
    for (int c = 0; c < CHAINS; c++) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < CHAINS; c++) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
int fma_peak(double *tflops) {
  if (!tflops) return -1;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return -2;
  // FP32: more resident warps to cover the FMA latency at the higher issue rate
  const int blocks = sms * (sizeof(T) == 8 ? 8 : 16), threads = 256;
  T *buf = nullptr;
  if (cudaMalloc(&buf, sizeof(T) * blocks * threads) != cudaSuccess) return -2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<T><<<blocks, threads>>>(buf, (T)0.999, (T)1e-3);  // warm-up
  cudaEventRecord(e0);
  fma_chains<T><<<blocks, threads>>>(buf, (T)0.999, (T)1e-3);
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
}  // namespace

extern "C" int matfun_cuda_fp64_peak(double *tflops) { return fma_peak<double>(tflops); }

extern "C" int matfun_cuda_fp32_peak(double *tflops) { return fma_peak<float>(tflops); }
