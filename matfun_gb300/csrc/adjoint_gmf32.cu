// adjoint_gmf32.cu -- instantiations of the mixed-precision general-family adjoint kernels (adjoint.cuh).
#include "adjoint.cuh"

namespace mf {
cudaError_t gmf_adjoint_launch_f32(int kind, double al, int64_t n, const float *A, const float *W, const float *V,
                                   float *F, float *Abar, float *JV, float *HWV, cudaStream_t st) {
  switch (kind) {
    case EXP: return gmf_adjoint_t<EXP, float>(al, n, A, W, V, F, Abar, JV, HWV, st);
    case LOG: return gmf_adjoint_t<LOG, float>(al, n, A, W, V, F, Abar, JV, HWV, st);
    default: return gmf_adjoint_t<POW, float>(al, n, A, W, V, F, Abar, JV, HWV, st);
  }
}
}  // namespace mf
