// adjoint_smf32.cu -- instantiations of the mixed-precision symmetric-family adjoint kernels (adjoint.cuh).
#include "adjoint.cuh"

namespace mf {
cudaError_t smf_adjoint_launch_f32(int kind, double al, int64_t n, const float *A, const float *W, const float *V,
                                   float *F, float *Abar, float *JV, float *HWV, cudaStream_t st) {
  switch (kind) {
    case EXP: return smf_adjoint_f32_t<EXP>(al, n, A, W, V, F, Abar, JV, HWV, st);
    case LOG: return smf_adjoint_f32_t<LOG>(al, n, A, W, V, F, Abar, JV, HWV, st);
    case SQRT: return smf_adjoint_f32_t<SQRT>(al, n, A, W, V, F, Abar, JV, HWV, st);
    default: return smf_adjoint_f32_t<POW>(al, n, A, W, V, F, Abar, JV, HWV, st);
  }
}
}  // namespace mf
