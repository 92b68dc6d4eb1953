// smf_sqrt.cu -- the sqrt instantiations of the smf kernels (smf_kernels.cuh), one translation unit per kind.
#include "smf_kernels.cuh"

namespace mf {
cudaError_t smf_launch_sqrt(double al, int64_t n, const double *x, bool mat, double *F, double *J, double *H,
                            cudaStream_t st, int *asym, bool reorder) {
  return smf_launch_t<SQRT>(al, n, x, mat, F, J, H, st, asym, reorder);
}
}  // namespace mf
