// gmf_pow.cu -- the pow instantiations of the gmf kernels (gmf_kernels.cuh), one translation unit per kind.
#include "gmf_kernels.cuh"

namespace mf {
cudaError_t gmf_launch_pow(double al, int64_t n, const double *A, double *F, double *J, double *H,
                            cudaStream_t st, bool reorder) {
  return gmf_launch_t<POW>(al, n, A, F, J, H, st, reorder);
}
cudaError_t gmf_tangent_launch_pow(double al, int64_t n, const double *A, double *F, double *G, double *K,
                                  cudaStream_t st) {
  return gmf_tangent_t<POW>(al, n, A, F, G, K, st);
}
}  // namespace mf
