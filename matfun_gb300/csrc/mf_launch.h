// mf_launch.h -- internal launch interface between the C ABI layer (capi.cu) and the kernel translation units
// (one per family and kind).  Arguments are validated and normalised by the caller: n > 0, the grid within limits,
// sqrt of the general family arrives as pow with al = 0.5, al = 0.5 for smf sqrt and 0 for exp / log.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

namespace mf {

// Raises a kernel's dynamic shared memory limit to `bytes` on the current device, once per device.
// cudaFuncSetAttribute acts on the current device's copy of the kernel only, so a process that launches the kernel
// on several GPUs needs the call on each of them; `done` holds one bit per device (devices 0..63) and may be set by
// several host threads at once.
template <typename Kernel>
cudaError_t smem_limit_per_device(Kernel kernel, int bytes, std::atomic<unsigned long long> &done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? 1ull << dev : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}
#define MF_SMF_DECL(k)                                                                                          \
  cudaError_t smf_launch_##k(double al, int64_t n, const double *x, bool mat, double *F, double *J, double *H, \
                             cudaStream_t st, int *asym = nullptr, bool reorder = true);
MF_SMF_DECL(exp)
MF_SMF_DECL(log)
MF_SMF_DECL(sqrt)
MF_SMF_DECL(pow)
#undef MF_SMF_DECL
// (reorder: allow the batch-wide ordering by spectral class, gmf_kernels.cuh; off where the arrays are host memory)
#define MF_GMF_DECL(k)                                                                                      \
  cudaError_t gmf_launch_##k(double al, int64_t n, const double *A, double *F, double *J, double *H, cudaStream_t st, \
                             bool reorder = true);
MF_GMF_DECL(exp)
MF_GMF_DECL(log)
MF_GMF_DECL(pow)
#undef MF_GMF_DECL
// the tangent of |f(A)|^2 / 2 (F, G = J^T F, K = J^T J + F : H; F and G may be null), general family, FP64
#define MF_GMFT_DECL(k)                                                                                         \
  cudaError_t gmf_tangent_launch_##k(double al, int64_t n, const double *A, double *F, double *G, double *K, \
                                     cudaStream_t st);
MF_GMFT_DECL(exp)
MF_GMFT_DECL(log)
MF_GMFT_DECL(pow)
#undef MF_GMFT_DECL
// mixed precision (FP32 storage, FP32 bulk arithmetic, FP64 deviator and Rayleigh quotients), symmetric family
#define MF_SMFX_DECL(k)                                                                                            \
  cudaError_t smf_mixed_launch_##k(double al, int64_t n, const float *x, bool mat, float *F, float *J, float *H, \
                                   cudaStream_t st);
MF_SMFX_DECL(exp)
MF_SMFX_DECL(log)
MF_SMFX_DECL(sqrt)
MF_SMFX_DECL(pow)
#undef MF_SMFX_DECL
// mixed precision, general family: FP32 storage and J / H assembly, FP64 spectral analysis and series
#define MF_GMFX_DECL(k) \
  cudaError_t gmf_mixed_launch_##k(double al, int64_t n, const float *A, float *F, float *J, float *H, cudaStream_t st);
MF_GMFX_DECL(exp)
MF_GMFX_DECL(log)
MF_GMFX_DECL(pow)
#undef MF_GMFX_DECL
// adjoints (matrix layout): any of F, Abar = J^T W, JV = J V, HWV = W . H . V; kind normalised as above
cudaError_t gmf_adjoint_launch(int kind, double al, int64_t n, const double *A, const double *W, const double *V,
                               double *F, double *Abar, double *JV, double *HWV, cudaStream_t st);
cudaError_t smf_adjoint_launch(int kind, double al, int64_t n, const double *A, const double *W, const double *V,
                               double *F, double *Abar, double *JV, double *HWV, cudaStream_t st);
// the same in mixed precision (FP32 arrays)
cudaError_t gmf_adjoint_launch_f32(int kind, double al, int64_t n, const float *A, const float *W, const float *V,
                                   float *F, float *Abar, float *JV, float *HWV, cudaStream_t st);
cudaError_t smf_adjoint_launch_f32(int kind, double al, int64_t n, const float *A, const float *W, const float *V,
                                   float *F, float *Abar, float *JV, float *HWV, cudaStream_t st);
// the three FP64 entry points by family (0 smf Voigt, 1 smf matrix, 2 gmf) with the reference's argument checks and
// return codes (0, -1, -2); *err (optional) receives the CUDA error of a failed launch (capi.cu)
int eval_f64(int family, int kind, double alpha, int64_t n, const double *x, double *F, double *J, double *H,
             cudaStream_t st, cudaError_t *err);
}  // namespace mf
