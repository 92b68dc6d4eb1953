// adjoint_gmf.cu -- instantiations of the general-family adjoint kernels (adjoint.cuh).
#include "adjoint.cuh"

namespace mf {
cudaError_t gmf_adjoint_launch(int kind, double al, int64_t n, const double *A, const double *W, const double *V,
                               double *F, double *Abar, double *JV, double *HWV, cudaStream_t st) {
  switch (kind) {
    case EXP: return gmf_adjoint_t<EXP>(al, n, A, W, V, F, Abar, JV, HWV, st);
    case LOG: return gmf_adjoint_t<LOG>(al, n, A, W, V, F, Abar, JV, HWV, st);
    default: return gmf_adjoint_t<POW>(al, n, A, W, V, F, Abar, JV, HWV, st);
  }
}
}  // namespace mf
