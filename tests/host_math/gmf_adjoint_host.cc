// gmf_adjoint_host.cc -- the tile of the general adjoint kernels (gmf_adjoint_tile.cuh) compiled for the host and run
// as a CTA of one thread per matrix (host_cta.h), so that a CPU test can hold F, Abar = J^T W, JV = J V and
// HWV = W.H.V of both storage types -- the FP64 record and, for FP32 arrays, the record with its scale factors folded
// in and rounded to FP32 once, contracted in FP32 -- against the oracle.  The test builds this file with g++
// (tests/test_gmf_math_host.py).
#include "host_cta.h"
#include "host_intrinsics.h"

#include "../../matfun_gb300/csrc/gmf_adjoint_tile.cuh"

using namespace mf;

namespace {

template <int KIND, int ORDER, typename T>
void run(double al, int64_t n, const T *A, const T *W, const T *V, T *F, T *Abar, T *JV, T *HWV) {
  GmfCoef C;
  gmf_coef(KIND, al, ORDER, C, sizeof(T) == 4);  // (the launch constants the device launch of this storage type takes)
  static GadjSmemT<1> S;
  for (int64_t i = 0; i < n; i++) gmf_adjoint_tile<KIND, ORDER, T, 1>(i, 1, A, W, V, F, Abar, JV, HWV, C, nullptr, S);
}

template <typename T>
int dispatch(int kind, double al, int64_t n, const T *A, const T *W, const T *V, T *F, T *Abar, T *JV, T *HWV) {
  if (kind < 0 || kind > 3) return -1;
  if (kind == 3) kind = 2, al = 0.5;  // sqrt is pow 0.5, as the C ABI maps it
  if (kind != 2) al = 0.0;
  const bool o2 = HWV != nullptr;
  switch (kind) {
    case 0: o2 ? run<EXP, 2>(al, n, A, W, V, F, Abar, JV, HWV) : run<EXP, 1>(al, n, A, W, V, F, Abar, JV, HWV); break;
    case 1: o2 ? run<LOG, 2>(al, n, A, W, V, F, Abar, JV, HWV) : run<LOG, 1>(al, n, A, W, V, F, Abar, JV, HWV); break;
    default: o2 ? run<POW, 2>(al, n, A, W, V, F, Abar, JV, HWV) : run<POW, 1>(al, n, A, W, V, F, Abar, JV, HWV); break;
  }
  return 0;
}

}  // namespace

// order 2 when HWV is requested, else 1, as gmf_cuda_adjoint picks it; outputs may be null
extern "C" int gmf_adjoint_f64(int kind, double al, int64_t n, const double *A, const double *W, const double *V,
                               double *F, double *Abar, double *JV, double *HWV) {
  return dispatch<double>(kind, al, n, A, W, V, F, Abar, JV, HWV);
}

extern "C" int gmf_adjoint_f32(int kind, double al, int64_t n, const float *A, const float *W, const float *V,
                               float *F, float *Abar, float *JV, float *HWV) {
  return dispatch<float>(kind, al, n, A, W, V, F, Abar, JV, HWV);
}
