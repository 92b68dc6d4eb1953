// diag.cu -- diagnostic entry points: the FP64 fused-multiply-add throughput of the current GPU, the denominator of
// the FP64 roofline that bounds the FP64 kernels of this library (reported by the benchmark beside the HBM one); and
// a probe of the FP32 symmetric eigensystem that returns its intermediate values per matrix, for comparison with a
// host build of the same header.
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/matfun_cuda.h"
#include "smf_mixed_math.cuh"

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
template <bool MAT>
__global__ void smf_f32_probe_kernel(int64_t n, const float *__restrict__ x, float *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) mf::smf_f32_probe_one<MAT>(x + (MAT ? 9 : 6) * i, out + mf::SMF_F32_PROBE * i);
}
}  // namespace

extern "C" int matfun_cuda_smf_f32_probe(int mat, int64_t n, const float *x, float *out, void *stream) {
  if (n < 0 || (n > 0 && (!x || !out))) return -1;
  if (n == 0) return 0;
  if (n > (int64_t)INT_MAX * 128) return -2;
  const unsigned blocks = (unsigned)((n + 127) / 128);
  const cudaStream_t st = (cudaStream_t)stream;
  if (mat) smf_f32_probe_kernel<true><<<blocks, 128, 0, st>>>(n, x, out);
  else smf_f32_probe_kernel<false><<<blocks, 128, 0, st>>>(n, x, out);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

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
