// gmf_mixed_exp.cu -- the exp instantiations of the mixed-precision gmf kernel (gmf_kernels.cuh with float storage).
#include "gmf_kernels.cuh"

namespace mf {
cudaError_t gmf_mixed_launch_exp(double al, int64_t n, const float *A, float *F, float *J, float *H,
                                cudaStream_t st) {
  return gmf_launch_t<EXP, float>(al, n, A, F, J, H, st);
}
}  // namespace mf
