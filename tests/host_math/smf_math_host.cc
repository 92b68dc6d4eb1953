// smf_math_host.cc -- the per-matrix math of the symmetric family (eigensystem, f of the eigenvalues, first and second
// divided differences), FP32 mixed form (smf_mixed_math.cuh) and FP64 form (smf_device.cuh), compiled for the host
// from the same headers the kernels use, so that a CPU test can hold that math against the oracle.  The test builds
// this file with g++ (recipe in tests/test_smf_math_host.py) and assembles F, J and H from the outputs in NumPy.
//
// Outputs per matrix: lam[3] eigenvalues, fl[3] = f(lam), V[9] eigenvectors (row-major, columns are the vectors),
// D[9] first divided differences (D[a][b] = f[lam_a, lam_b], D[a][a] = f'(lam_a)), D2[27] second divided differences.
#include "host_intrinsics.h"
#include "../../matfun_gb300/csrc/smf_mixed_math.cuh"

using namespace mf;

namespace {

template <int KIND, bool MAT>
void f32_one(const float *xi, const SmfCoefF &C, float *lam, float *fl, float *V, float *D, float *D2) {
  SmfInF in;
  if (MAT) sym_in_f(xi, in);
  else voigt_in_f(xi, in);
  SmfSpecF Sp;
  smf_spectrum_f<KIND, MAT>(in, C, Sp);
  float Dm[3][3], T[3][3][3];
  smf_dm_f<KIND>(Sp, C, Dm);
  smf_d2_f<KIND>(Sp, Dm, C, T);
  for (int a = 0; a < 3; a++) {
    lam[a] = Sp.lf[a];
    fl[a] = Sp.fl[a];
    for (int b = 0; b < 3; b++) {
      V[3 * a + b] = Sp.V[a][b];
      D[3 * a + b] = Dm[a][b];
      for (int c = 0; c < 3; c++) D2[9 * a + 3 * b + c] = T[a][b][c];
    }
  }
}

template <int KIND, bool MAT>
void f32_all(double al, int64_t n, const float *x, float *lam, float *fl, float *V, float *D, float *D2) {
  SmfCoefF C;
  smf_coef_f(KIND, al, C);
  const int nin = MAT ? 9 : 6;
  for (int64_t i = 0; i < n; i++)
    f32_one<KIND, MAT>(x + nin * i, C, lam + 3 * i, fl + 3 * i, V + 9 * i, D + 9 * i, D2 + 27 * i);
}

template <int KIND>
void f64_all(double al, int64_t n, const double *v6, double *lam, double *fl, double *V, double *D, double *D2) {
  SmfCoef C;
  smf_coef(KIND, al, C);
  for (int64_t i = 0; i < n; i++) {
    double l[3], f[3], W[3][3];
    smf_eigen<KIND>(v6 + 6 * i, al, l, f, W);
    double Dm[3][3];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++)
        Dm[a][b] = a == b ? smf_deriv<KIND>(l[a], f[a], C) : smf_dd1<KIND>(l[a], l[b], f[a], f[b], C);
    // the kernel's order of the arguments: (i, j, l) sorted by index, i <= j <= l
    for (int a = 0; a < 3; a++)
      for (int b = a; b < 3; b++)
        for (int c = b; c < 3; c++) {
          const double d = (a == b && b == c)
                               ? smf_dd2_same<KIND>(l[a], f[a], Dm[a][a], C)
                               : smf_dd2<KIND>(l[a], l[b], l[c], f[a], f[b], f[c], Dm[a][b], Dm[a][c], Dm[b][c], C);
          const int p[6][3] = {{a, b, c}, {a, c, b}, {b, a, c}, {b, c, a}, {c, a, b}, {c, b, a}};
          for (const auto &q : p) D2[27 * i + 9 * q[0] + 3 * q[1] + q[2]] = d;
        }
    for (int a = 0; a < 3; a++) {
      lam[3 * i + a] = l[a];
      fl[3 * i + a] = f[a];
      for (int b = 0; b < 3; b++) {
        V[9 * i + 3 * a + b] = W[a][b];
        D[9 * i + 3 * a + b] = Dm[a][b];
      }
    }
  }
}

}  // namespace

// kind: 0 exp, 1 log, 2 pow (al), 3 sqrt (al = 0.5), as the C ABI; mat: 9-entry matrix rows, else Voigt 6-vectors
extern "C" int smf_math_f32(int kind, double al, int mat, int64_t n, const float *x, float *lam, float *fl, float *V,
                            float *D, float *D2) {
  if (kind != 2) al = kind == 3 ? 0.5 : 0.0;
#define MF_F32(K)                                                   \
  (mat ? f32_all<K, true>(al, n, x, lam, fl, V, D, D2) : f32_all<K, false>(al, n, x, lam, fl, V, D, D2))
  switch (kind) {
    case 0: MF_F32(EXP); return 0;
    case 1: MF_F32(LOG); return 0;
    case 2: MF_F32(POW); return 0;
    case 3: MF_F32(SQRT); return 0;
    default: return -1;
  }
#undef MF_F32
}

// FP64 form on Voigt 6-vectors (the matrix layout's symmetric part is formed by the caller)
extern "C" int smf_math_f64(int kind, double al, int64_t n, const double *v6, double *lam, double *fl, double *V,
                            double *D, double *D2) {
  if (kind != 2) al = kind == 3 ? 0.5 : 0.0;
  switch (kind) {
    case 0: f64_all<EXP>(al, n, v6, lam, fl, V, D, D2); return 0;
    case 1: f64_all<LOG>(al, n, v6, lam, fl, V, D, D2); return 0;
    case 2: f64_all<POW>(al, n, v6, lam, fl, V, D, D2); return 0;
    case 3: f64_all<SQRT>(al, n, v6, lam, fl, V, D, D2); return 0;
    default: return -1;
  }
}

