// smf_mixed_pow.cu -- the pow instantiations of the mixed-precision smf kernel (smf_mixed.cuh).
#include "smf_mixed.cuh"

namespace mf {
cudaError_t smf_mixed_launch_pow(double al, int64_t n, const float *x, bool mat, float *F, float *J, float *H,
                                cudaStream_t st) {
  return smf_mixed_launch_t<POW>(al, n, x, mat, F, J, H, st);
}
}  // namespace mf
