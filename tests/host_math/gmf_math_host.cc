// gmf_math_host.cc -- phase A of the gmf kernels (gmf_device.cuh: scaling, closed-form roots, pair refinement,
// branch-cut pair, groups, the confluent group series and the record F, r1, r2, D2', D3', sc1, sc2) compiled for the
// host from the kernels' own header, so that a CPU test can hold it against the oracle.  The test builds this file
// with g++ (recipe in tests/test_gmf_math_host.py) and contracts the record into J and H in NumPy, as phase B does:
//   J_abcd = sc1 T4[ac, db],  H_abcdef = sc2 (T6[ac, de, fb] + T6[ae, fc, db]),  r_0 = I,
//   T4[x, y] = sum_mn r_m[x] D2'_mn r_n[y],  T6[x, y, z] = sum_mnp r_m[x] r_n[y] r_p[z] D3'_mnp.
// The warp votes of the series take a warp of one lane (host_intrinsics.h).  ff = 1 runs the float-float group series
// of the FP32-storage kernels (gmf_finish<..., true>), ff = 2 the same with those kernels' launch constants (their
// group radii and series stop, gmf_coef fp32), ff = 0 the FP64 / split series of the FP64 kernels.
#include "host_intrinsics.h"
#include "../../matfun_gb300/csrc/gmf_device.cuh"

using namespace mf;

namespace {

template <int KIND, int ORDER, bool FF>
void all(double al, int64_t n, const double *A, double *F, double *R12, double *D2, double *D3, double *sc,
         bool f32coef) {
  GmfCoef C;
  gmf_coef(KIND, al, ORDER, C, f32coef);
  for (int64_t i = 0; i < n; i++) {
    GmfState St;
    gmf_classify<KIND, ORDER>(A + 9 * i, C, St);
    GmfRec R;
    gmf_finish<KIND, ORDER, FF>(St, C, R);
    for (int k = 0; k < 9; k++) {
      F[9 * i + k] = R.F[k];
      R12[18 * i + k] = ORDER >= 1 ? R.r1[k] : 0.0;
      R12[18 * i + 9 + k] = ORDER >= 1 ? R.r2[k] : 0.0;
    }
    for (int k = 0; k < 6; k++) D2[6 * i + k] = ORDER >= 1 ? R.D2[k] : 0.0;
    for (int k = 0; k < 10; k++) D3[10 * i + k] = ORDER >= 2 ? R.D3[k] : 0.0;
    sc[2 * i] = ORDER >= 1 ? R.sc1 : 0.0;
    sc[2 * i + 1] = ORDER >= 2 ? R.sc2 : 0.0;
  }
}

template <int KIND, bool FF>
void by_order(int order, double al, int64_t n, const double *A, double *F, double *R12, double *D2, double *D3,
              double *sc, bool f32coef) {
  if (order == 2) all<KIND, 2, FF>(al, n, A, F, R12, D2, D3, sc, f32coef);
  else if (order == 1) all<KIND, 1, FF>(al, n, A, F, R12, D2, D3, sc, f32coef);
  else all<KIND, 0, FF>(al, n, A, F, R12, D2, D3, sc, f32coef);
}

template <int KIND>
void by_ff(int ff, int order, double al, int64_t n, const double *A, double *F, double *R12, double *D2, double *D3,
           double *sc) {
  if (ff) by_order<KIND, true>(order, al, n, A, F, R12, D2, D3, sc, ff == 2);
  else by_order<KIND, false>(order, al, n, A, F, R12, D2, D3, sc, false);
}

}  // namespace

// kind: 0 exp, 1 log, 2 pow (al), 3 sqrt (pow 0.5, as the C ABI); outputs per matrix: F (9), r1 then r2 (18), D2' (6,
// at 00 11 22 01 02 12), D3' (10, sym3 order), sc1 and sc2 (2)
extern "C" int gmf_math(int kind, double al, int order, int ff, int64_t n, const double *A, double *F, double *R12,
                        double *D2, double *D3, double *sc) {
  if (kind < 0 || kind > 3 || order < 0 || order > 2) return -1;
  if (kind == 3) kind = 2, al = 0.5;
  if (kind != 2) al = 0.0;
  switch (kind) {
    case 0: by_ff<EXP>(ff, order, al, n, A, F, R12, D2, D3, sc); break;
    case 1: by_ff<LOG>(ff, order, al, n, A, F, R12, D2, D3, sc); break;
    default: by_ff<POW>(ff, order, al, n, A, F, R12, D2, D3, sc); break;
  }
  return 0;
}
