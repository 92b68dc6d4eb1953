// smf_adjoint_tile.cuh -- one tile of the symmetric adjoint kernels (smf_cuda_adjoint, FP64; smf_cuda_adjoint_f32,
// FP32): the matrices base .. base + cnt - 1 by a CTA of TPB threads, one thread per matrix between a coalesced load
// of A, W, V and a coalesced store of F, Abar, JV, HWV through shared memory.  The contractions in the eigenbasis
// are those of the Daleckii-Krein form and its second-order form (adjoint.cuh).
#pragma once

#include "smf_mixed_math.cuh"
#include "smf_device.cuh"

namespace mf {

// the contractions in the eigenbasis: Wt = U^T sym(W) U, Vt = U^T sym(V) U; Abar = U (D o Wt) U^T,
// JV = U (D o Vt) U^T, HWV = U (Q + Q^T) U^T with Q_xy = sum_z D2_xyz Wt_xz Vt_yz (outputs may be null)
template <typename T, int ORDER>
MF_D void smf_adj_apply(const T (&U)[3][3], const T (&Dm)[3][3], const T (&D2)[3][3][3], const T *w, const T *v,
                        T *oAbar, T *oJV, T *oHWV) {
  T Wt[3][3], Vt[3][3];
  auto rotate = [&](const T *Xg, T Xt[3][3]) {
    T Xs[3][3], Tm[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) Xs[i][j] = T(0.5) * (Xg[3 * i + j] + Xg[3 * j + i]);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int b = 0; b < 3; b++) Tm[i][b] = Xs[i][0] * U[0][b] + Xs[i][1] * U[1][b] + Xs[i][2] * U[2][b];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) Xt[a][b] = U[0][a] * Tm[0][b] + U[1][a] * Tm[1][b] + U[2][a] * Tm[2][b];
  };
  auto back = [&](T Y[3][3], T *out) {  // out = U Y U^T
    T Tm[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int b = 0; b < 3; b++) Tm[i][b] = U[i][0] * Y[0][b] + U[i][1] * Y[1][b] + U[i][2] * Y[2][b];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) out[3 * i + j] = Tm[i][0] * U[j][0] + Tm[i][1] * U[j][1] + Tm[i][2] * U[j][2];
  };
  if (oAbar || oHWV) rotate(w, Wt);
  if (oJV || oHWV) rotate(v, Vt);
  if (oAbar) {
    T Y[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) Y[a][b] = Dm[a][b] * Wt[a][b];
    back(Y, oAbar);
  }
  if (oJV) {
    T Y[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) Y[a][b] = Dm[a][b] * Vt[a][b];
    back(Y, oJV);
  }
  if (ORDER >= 2 && oHWV) {
    T Q[3][3], Y[3][3];
#pragma unroll
    for (int x = 0; x < 3; x++)
#pragma unroll
      for (int y = 0; y < 3; y++)
        Q[x][y] = D2[x][y][0] * Wt[x][0] * Vt[y][0] + D2[x][y][1] * Wt[x][1] * Vt[y][1] +
                  D2[x][y][2] * Wt[x][2] * Vt[y][2];
#pragma unroll
    for (int x = 0; x < 3; x++)
#pragma unroll
      for (int y = 0; y < 3; y++) Y[x][y] = Q[x][y] + Q[y][x];
    back(Y, oHWV);
  }
}

// shared memory of one tile: inputs A, W, V and the four output stagings F, Abar, JV, HWV
template <typename T, int TPB>
struct SadjSmem {
  T sx[TPB * 9], sw[TPB * 9], sv[TPB * 9], so[4][TPB * 9];
};

template <int KIND, int ORDER, int TPB>
MF_D void smf_adjoint_tile(int64_t base, int cnt, const double *__restrict__ A, const double *__restrict__ W,
                           const double *__restrict__ V, double *__restrict__ F, double *__restrict__ Abar,
                           double *__restrict__ JV, double *__restrict__ HWV, const SmfCoef &C,
                           SadjSmem<double, TPB> &S) {
  const int tid = threadIdx.x;
  for (int e = tid; e < cnt * 9; e += TPB) {
    S.sx[e] = A[base * 9 + e];
    if (W) S.sw[e] = W[base * 9 + e];
    if (V) S.sv[e] = V[base * 9 + e];
  }
  __syncthreads();
  if (tid < cnt) {
    const double *xi = S.sx + tid * 9;
    double v6[6];  // symmetric part (NaN if not symmetric, smf_kernel.hpp:408-421)
    {
      double mx = 0.0;
#pragma unroll
      for (int k = 0; k < 9; k++) mx = sel(fabs(xi[k]) > mx, fabs(xi[k]), mx);
      const double tol = 1e-8 * mx;
      bool sym = !(fabs(xi[1] - xi[3]) > tol) & !(fabs(xi[2] - xi[6]) > tol) & !(fabs(xi[5] - xi[7]) > tol);
      v6[0] = xi[0]; v6[1] = xi[4]; v6[2] = xi[8];
      v6[3] = 0.5 * (xi[1] + xi[3]); v6[4] = 0.5 * (xi[2] + xi[6]); v6[5] = 0.5 * (xi[5] + xi[7]);
#pragma unroll
      for (int k = 0; k < 6; k++) v6[k] = sel(sym, v6[k], __longlong_as_double(0x7FF8000000000000ll));
    }
    double lam[3], fl[3], U[3][3];
    smf_eigen<KIND>(v6, C.al, lam, fl, U);
    if (F) {
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++)
          S.so[0][tid * 9 + 3 * a + b] = U[a][0] * fl[0] * U[b][0] + U[a][1] * fl[1] * U[b][1] + U[a][2] * fl[2] * U[b][2];
    }
    if (Abar || JV || HWV) {
      const double D01 = smf_dd1<KIND>(lam[0], lam[1], fl[0], fl[1], C);
      const double D02 = smf_dd1<KIND>(lam[0], lam[2], fl[0], fl[2], C);
      const double D12 = smf_dd1<KIND>(lam[1], lam[2], fl[1], fl[2], C);
      const double Dm[3][3] = {{smf_deriv<KIND>(lam[0], fl[0], C), D01, D02},
                               {D01, smf_deriv<KIND>(lam[1], fl[1], C), D12},
                               {D02, D12, smf_deriv<KIND>(lam[2], fl[2], C)}};
      double D2[3][3][3];
      if (ORDER >= 2 && HWV) {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = i; j < 3; j++)
#pragma unroll
            for (int l = j; l < 3; l++) {
              const double d = (i == j && j == l) ? smf_dd2_same<KIND>(lam[i], fl[i], Dm[i][i], C)
                                                  : smf_dd2<KIND>(lam[i], lam[j], lam[l], fl[i], fl[j], fl[l],
                                                                  Dm[i][j], Dm[i][l], Dm[j][l], C);
              D2[i][j][l] = D2[i][l][j] = D2[j][i][l] = D2[j][l][i] = D2[l][i][j] = D2[l][j][i] = d;
            }
      }
      smf_adj_apply<double, ORDER>(U, Dm, D2, S.sw + tid * 9, S.sv + tid * 9, Abar ? S.so[1] + tid * 9 : nullptr,
                                   JV ? S.so[2] + tid * 9 : nullptr, HWV ? S.so[3] + tid * 9 : nullptr);
    }
  }
  __syncthreads();
  double *dst[4] = {F, Abar, JV, HWV};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (!dst[q]) continue;
    for (int e = tid; e < cnt * 9; e += TPB) dst[q][base * 9 + e] = S.so[q][e];
  }
}

// mixed precision: FP32 arrays, the eigensystem and divided differences of smf_mixed_math.cuh, FP32 contractions
template <int KIND, int ORDER, int TPB>
MF_D void smf_adjoint_tile_f32(int64_t base, int cnt, const float *__restrict__ A, const float *__restrict__ W,
                               const float *__restrict__ V, float *__restrict__ F, float *__restrict__ Abar,
                               float *__restrict__ JV, float *__restrict__ HWV, const SmfCoefF &C,
                               SadjSmem<float, TPB> &S) {
  const int tid = threadIdx.x;
  for (int e = tid; e < cnt * 9; e += TPB) {
    S.sx[e] = A[base * 9 + e];
    if (W) S.sw[e] = W[base * 9 + e];
    if (V) S.sv[e] = V[base * 9 + e];
  }
  __syncthreads();
  if (tid < cnt) {
    SmfInF in;
    sym_in_f(S.sx + tid * 9, in);
    SmfSpecF Sp;
    smf_spectrum_f<KIND, true>(in, C, Sp);
    if (F) {
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++)
          S.so[0][tid * 9 + 3 * a + b] = Sp.V[a][0] * Sp.fl[0] * Sp.V[b][0] + Sp.V[a][1] * Sp.fl[1] * Sp.V[b][1] +
                                       Sp.V[a][2] * Sp.fl[2] * Sp.V[b][2];
    }
    if (Abar || JV || HWV) {
      float Dm[3][3], D2[3][3][3];
      smf_dm_f<KIND>(Sp, C, Dm);
      if (ORDER >= 2 && HWV) smf_d2_f<KIND>(Sp, Dm, C, D2);
      smf_adj_apply<float, ORDER>(Sp.V, Dm, D2, S.sw + tid * 9, S.sv + tid * 9, Abar ? S.so[1] + tid * 9 : nullptr,
                                  JV ? S.so[2] + tid * 9 : nullptr, HWV ? S.so[3] + tid * 9 : nullptr);
    }
  }
  __syncthreads();
  float *dst[4] = {F, Abar, JV, HWV};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (!dst[q]) continue;
    for (int e = tid; e < cnt * 9; e += TPB) dst[q][base * 9 + e] = S.so[q][e];
  }
}

}  // namespace mf
