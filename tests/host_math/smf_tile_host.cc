// smf_tile_host.cc -- the tiles of the symmetric family (smf_tile.cuh, FP64; smf_mixed_tile.cuh, FP32) compiled for the
// host and run as a CTA of one thread per matrix, so that a CPU test can hold the kernels' whole per-matrix path --
// input staging, the symmetric part of the matrix layout, the eigensystem, the divided differences, the product-vector
// forms of J and H and their expansion into the output layouts with the layout weights -- against the oracle.  With
// TPB = 1 every cooperative loop of a tile runs in its one thread and its barriers have nothing to wait for.  The test
// builds this file with g++ (tests/test_smf_tile_host.py).  The adjoint tiles (smf_adjoint_tile.cuh) run the same way.
#include "host_cta.h"
#include "host_intrinsics.h"

#include "../../matfun_gb300/csrc/smf_adjoint_tile.cuh"
#include "../../matfun_gb300/csrc/smf_mixed_tile.cuh"
#include "../../matfun_gb300/csrc/smf_tile.cuh"

using namespace mf;

namespace {

template <int KIND, int ORDER, bool MAT>
void f64_run(double al, int64_t n, const double *x, double *F, double *J, double *H, int *asym) {
  SmfCoef C;
  smf_coef(KIND, al, C);
  SmfTileSmem<ORDER, MAT, 1> TS;
  for (int64_t i = 0; i < n; i++) smf_tile<KIND, ORDER, MAT, 1>(i, 1, x, F, J, H, C, asym, TS);
}

template <int KIND, int ORDER, bool MAT>
void f32_run(double al, int64_t n, const float *x, float *F, float *J, float *H) {
  SmfCoefF C;
  smf_coef_f(KIND, al, C);
  SmfxTileSmem<ORDER, MAT, 1> TS;
  for (int64_t i = 0; i < n; i++) smf_mixed_tile<KIND, ORDER, MAT, 1>(i, 1, x, F, J, H, C, TS);
}

// the instantiations the test uses: every order for log, order 2 for the other kinds; both layouts
template <typename T, typename Run>
int dispatch(int kind, int order, int mat, Run run) {
  if (kind == LOG) {
    if (order == 0) return mat ? run.template go<LOG, 0, true>() : run.template go<LOG, 0, false>();
    if (order == 1) return mat ? run.template go<LOG, 1, true>() : run.template go<LOG, 1, false>();
    return mat ? run.template go<LOG, 2, true>() : run.template go<LOG, 2, false>();
  }
  if (order != 2) return -1;
  switch (kind) {
    case EXP: return mat ? run.template go<EXP, 2, true>() : run.template go<EXP, 2, false>();
    case POW: return mat ? run.template go<POW, 2, true>() : run.template go<POW, 2, false>();
    case SQRT: return mat ? run.template go<SQRT, 2, true>() : run.template go<SQRT, 2, false>();
    default: return -1;
  }
}

struct Run64 {
  double al;
  int64_t n;
  const double *x;
  double *F, *J, *H;
  int *asym;
  template <int K, int O, bool M>
  int go() const {
    f64_run<K, O, M>(al, n, x, F, J, H, asym);
    return 0;
  }
};

struct Run32 {
  double al;
  int64_t n;
  const float *x;
  float *F, *J, *H;
  template <int K, int O, bool M>
  int go() const {
    f32_run<K, O, M>(al, n, x, F, J, H);
    return 0;
  }
};

}  // namespace

// kind: 0 exp, 1 log, 2 pow (al), 3 sqrt, as the C ABI; order 0..2 (0 and 1 for log only); mat: 9-entry rows, else
// Voigt 6-vectors; J / H may be null below their order; asym counts non-symmetric matrices of the matrix layout
extern "C" int smf_tile_f64(int kind, double al, int order, int mat, int64_t n, const double *x, double *F, double *J,
                            double *H, int *asym) {
  if (kind != 2) al = kind == 3 ? 0.5 : 0.0;
  return dispatch<double>(kind, order, mat, Run64{al, n, x, F, J, H, asym});
}

extern "C" int smf_tile_f32(int kind, double al, int order, int mat, int64_t n, const float *x, float *F, float *J,
                            float *H) {
  if (kind != 2) al = kind == 3 ? 0.5 : 0.0;
  return dispatch<float>(kind, order, mat, Run32{al, n, x, F, J, H});
}

namespace {

template <int KIND, int ORDER>
void adj64(double al, int64_t n, const double *A, const double *W, const double *V, double *F, double *Abar,
           double *JV, double *HWV) {
  SmfCoef C;
  smf_coef(KIND, al, C);
  SadjSmem<double, 1> S;
  for (int64_t i = 0; i < n; i++) smf_adjoint_tile<KIND, ORDER, 1>(i, 1, A, W, V, F, Abar, JV, HWV, C, S);
}

template <int KIND, int ORDER>
void adj32(double al, int64_t n, const float *A, const float *W, const float *V, float *F, float *Abar, float *JV,
           float *HWV) {
  SmfCoefF C;
  smf_coef_f(KIND, al, C);
  SadjSmem<float, 1> S;
  for (int64_t i = 0; i < n; i++) smf_adjoint_tile_f32<KIND, ORDER, 1>(i, 1, A, W, V, F, Abar, JV, HWV, C, S);
}

template <typename T, typename Fn>
int adj_dispatch(int kind, int order, Fn fn) {
  switch (kind) {
    case EXP: return order == 2 ? fn.template go<EXP, 2>() : fn.template go<EXP, 1>();
    case LOG: return order == 2 ? fn.template go<LOG, 2>() : fn.template go<LOG, 1>();
    case POW: return order == 2 ? fn.template go<POW, 2>() : fn.template go<POW, 1>();
    case SQRT: return order == 2 ? fn.template go<SQRT, 2>() : fn.template go<SQRT, 1>();
    default: return -1;
  }
}

template <typename T>
struct Adj {
  double al;
  int64_t n;
  const T *A, *W, *V;
  T *F, *Abar, *JV, *HWV;
  template <int K, int O>
  int go() const {
    if constexpr (sizeof(T) == 8) adj64<K, O>(al, n, A, W, V, F, Abar, JV, HWV);
    else adj32<K, O>(al, n, A, W, V, F, Abar, JV, HWV);
    return 0;
  }
};

}  // namespace

// the adjoint tiles: order 2 when HWV is requested, else 1, as smf_cuda_adjoint picks it; outputs may be null
extern "C" int smf_adjoint_f64(int kind, double al, int64_t n, const double *A, const double *W, const double *V,
                               double *F, double *Abar, double *JV, double *HWV) {
  if (kind != 2) al = kind == 3 ? 0.5 : 0.0;
  return adj_dispatch<double>(kind, HWV ? 2 : 1, Adj<double>{al, n, A, W, V, F, Abar, JV, HWV});
}

extern "C" int smf_adjoint_f32(int kind, double al, int64_t n, const float *A, const float *W, const float *V,
                               float *F, float *Abar, float *JV, float *HWV) {
  if (kind != 2) al = kind == 3 ? 0.5 : 0.0;
  return adj_dispatch<float>(kind, HWV ? 2 : 1, Adj<float>{al, n, A, W, V, F, Abar, JV, HWV});
}
