// smf_kernels.cu -- symmetric family (smf_cuda_eval / smf_cuda_eval_matrix): F, J, H of f(A) for symmetric 3x3
// matrices, FP64, Voigt or matrix layout.  Replaces smf_eval_kernel / smf_hess_kernel of the reference
// (cuda/src/matfun_cuda.cu:28-96).
//
// One CTA = 64 matrices (two warps).  Phase A: one thread per matrix computes the eigensystem, f, the divided
// differences and the distinct entries of J (21 values of the symmetric form K) and H (56 values of the symmetric
// form G'), see smf_device.cuh, into shared memory.  Phase B: the CTA expands them into the output layout with
// fully coalesced stores (64 consecutive doubles per store instruction); the layout weights (powers of two) are
// applied on the exponent bits, not on the FP64 pipe.
#pragma once
#include "smf_device.cuh"
#include "mf_launch.h"

namespace mf {

constexpr int SMF_TPB = 64;

// x * 2^k for k in [-3, 1], exact; integer exponent arithmetic for normal x, a multiplication otherwise
MF_D double mulpow2(double x, int k) {
  if (k == 0) return x;
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e > 3 && e < 0x7FE) return __longlong_as_double(b + ((long long)k << 52));
  return x * __longlong_as_double((long long)(1023 + k) << 52);
}

// Voigt index of matrix entry m = 3a + b, and log2 of its derivative weight (smf_kernel.hpp:384-389)
MF_D constexpr int midx(int m) { return m % 4 == 0 ? m / 4 : (m == 1 || m == 3 ? 3 : (m == 2 || m == 6 ? 4 : 5)); }
MF_D constexpr int mwt_log2(int m) { return m % 4 == 0 ? 0 : -1; }

template <int KIND, int ORDER, bool MAT>
__global__ void __launch_bounds__(SMF_TPB) smf_kernel(int64_t n, const double *__restrict__ x,
                                                      double *__restrict__ F, double *__restrict__ J,
                                                      double *__restrict__ H, const SmfCoef C) {
  constexpr int NIN = MAT ? 9 : 6, NF = MAT ? 9 : 6, NJ = NF * NF, NH = NJ * NF;
  __shared__ double sX[SMF_TPB * NIN];
  __shared__ double sF[SMF_TPB * NF];
  __shared__ double sK[ORDER >= 1 ? SMF_TPB * 21 : 1];
  __shared__ double sG[ORDER >= 2 ? SMF_TPB * 56 : 1];
  const int tid = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * SMF_TPB;
  const int cnt = (int)min((int64_t)SMF_TPB, n - base);

  for (int e = tid; e < cnt * NIN; e += SMF_TPB) sX[e] = x[base * NIN + e];  // coalesced input
  __syncthreads();

  if (tid < cnt) {
    double v[6];
    const double *xi = sX + tid * NIN;
    if (MAT) {  // symmetric part; all NaN if |a_ij - a_ji| > 1e-8 max|a| (smf_kernel.hpp:408-421)
      double mx = 0.0;
#pragma unroll
      for (int k = 0; k < 9; k++) mx = sel(fabs(xi[k]) > mx, fabs(xi[k]), mx);
      double tol = 1e-8 * mx;
      bool sym = !(fabs(xi[1] - xi[3]) > tol) & !(fabs(xi[2] - xi[6]) > tol) & !(fabs(xi[5] - xi[7]) > tol);
      v[0] = xi[0]; v[1] = xi[4]; v[2] = xi[8];
      v[3] = 0.5 * (xi[1] + xi[3]); v[4] = 0.5 * (xi[2] + xi[6]); v[5] = 0.5 * (xi[5] + xi[7]);
#pragma unroll
      for (int k = 0; k < 6; k++) v[k] = sel(sym, v[k], __longlong_as_double(0x7FF8000000000000ll));
    } else {
#pragma unroll
      for (int k = 0; k < 6; k++) v[k] = xi[k];
    }
    double lam[3], fl[3], V[3][3];
    smf_eigen<KIND>(v, C.al, lam, fl, V);
    // F = V diag(f) V^T
    double Fv[6];
#pragma unroll
    for (int s = 0; s < 6; s++) {
      const int a = vk_(s), b = vl_(s);
      Fv[s] = V[a][0] * fl[0] * V[b][0] + V[a][1] * fl[1] * V[b][1] + V[a][2] * fl[2] * V[b][2];
    }
    if (MAT) {
#pragma unroll
      for (int m = 0; m < 9; m++) sF[tid * 9 + m] = Fv[midx(m)];
    } else {
#pragma unroll
      for (int s = 0; s < 6; s++) sF[tid * 6 + s] = Fv[s];
    }
    if (ORDER >= 1) {
      // divided differences D (smf_kernel.hpp:299-302)
      double D01 = smf_dd1<KIND>(lam[0], lam[1], fl[0], fl[1], C);
      double D02 = smf_dd1<KIND>(lam[0], lam[2], fl[0], fl[2], C);
      double D12 = smf_dd1<KIND>(lam[1], lam[2], fl[1], fl[2], C);
      double D00 = smf_deriv<KIND>(lam[0], fl[0], C), D11 = smf_deriv<KIND>(lam[1], fl[1], C);
      double D22 = smf_deriv<KIND>(lam[2], fl[2], C);
      double Et[6][6];
      smf_et(V, Et);
      // K(I, p) = sum_ab D_ab Et_I,ab Et_p,ab  (off-diagonal pairs counted twice)
      double Dw[6] = {D00, D11, D22, 2.0 * D01, 2.0 * D02, 2.0 * D12};
      double *k_out = sK + tid * 21;
#pragma unroll
      for (int I = 0; I < 6; I++) {
        double de[6];
#pragma unroll
        for (int s = 0; s < 6; s++) de[s] = Dw[s] * Et[I][s];
#pragma unroll
        for (int p = I; p < 6; p++) {
          double acc = de[0] * Et[p][0];
#pragma unroll
          for (int s = 1; s < 6; s++) acc = fma(de[s], Et[p][s], acc);
          k_out[sym2(I, p)] = acc;
        }
      }
      if (ORDER >= 2) {
        // second divided differences over the 10 distinct triples (smf_kernel.hpp:328-338)
        double D2[3][3][3];
        double Dm[3][3] = {{D00, D01, D02}, {D01, D11, D12}, {D02, D12, D22}};
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = i; j < 3; j++)
#pragma unroll
            for (int l = j; l < 3; l++) {
              double d = smf_dd2<KIND>(lam[i], lam[j], lam[l], fl[i], fl[j], fl[l], Dm[i][j], Dm[i][l],
                                             Dm[j][l], C);
              D2[i][j][l] = D2[i][l][j] = D2[j][i][l] = D2[j][l][i] = D2[l][i][j] = D2[l][j][i] = d;
            }
        // G'(I, y, z) = sum_ab Et_I,ab S^yz_ab,  S^yz = W + W^T,  W_ab = sum_m D2_amb Et_y,am Et_z,mb
        double *g_out = sG + tid * 56;
#pragma unroll
        for (int y = 0; y < 6; y++) {
          double Ay[3][3][3];  // D2_amb Et_y,am
#pragma unroll
          for (int a = 0; a < 3; a++)
#pragma unroll
            for (int m = 0; m < 3; m++) {
              const int am = a == m ? a : a + m + 2;
#pragma unroll
              for (int b = 0; b < 3; b++) Ay[a][m][b] = D2[a][m][b] * Et[y][am];
            }
#pragma unroll
          for (int z = y; z < 6; z++) {
            double S[6];
#pragma unroll
            for (int s = 0; s < 6; s++) {
              const int a = vk_(s), b = vl_(s);
              double w = 0.0;
#pragma unroll
              for (int m = 0; m < 3; m++) {
                const int mb = m == b ? m : m + b + 2, ma = m == a ? m : m + a + 2;
                w = fma(Ay[a][m][b], Et[z][mb], w);
                w = fma(Ay[b][m][a], Et[z][ma], w);
              }
              S[s] = w;
            }
#pragma unroll
            for (int I = 0; I <= y; I++) {
              double acc = Et[I][0] * S[0];
              acc = fma(Et[I][1], S[1], acc);
              acc = fma(Et[I][2], S[2], acc);
              double off = Et[I][3] * S[3];
              off = fma(Et[I][4], S[4], off);
              off = fma(Et[I][5], S[5], off);
              g_out[sym3(I, y, z)] = acc + (off + off);
            }
          }
        }
      }
    }
  }
  __syncthreads();

  // ---- phase B: coalesced expansion into the output layout
  for (int e = tid; e < cnt * NF; e += SMF_TPB) F[base * NF + e] = sF[e];
  if (ORDER >= 1) {
    constexpr int KJ = (NJ + SMF_TPB - 1) / SMF_TPB;
    int jidx[KJ], jexp[KJ];
#pragma unroll
    for (int k = 0; k < KJ; k++) {
      const int w = min(tid + SMF_TPB * k, NJ - 1);
      int I, p, ex;
      if (MAT) {
        I = midx(w / 9); p = midx(w % 9);
        ex = (I >= 3 ? -1 : 0) + mwt_log2(w % 9);
      } else {
        I = w / 6; p = w % 6;
        ex = I >= 3 ? -1 : 0;
      }
      jidx[k] = sym2(min(I, p), max(I, p));
      jexp[k] = ex;
    }
    for (int mi = 0; mi < cnt; mi++) {
      double *o = J + (base + mi) * NJ;
      const double *s = sK + mi * 21;
#pragma unroll
      for (int k = 0; k < KJ; k++)
        if (tid + SMF_TPB * k < NJ) o[tid + SMF_TPB * k] = mulpow2(s[jidx[k]], jexp[k]);
    }
  }
  if (ORDER >= 2) {
    constexpr int KH = (NH + SMF_TPB - 1) / SMF_TPB;
    int hidx[KH], hexp[KH];
#pragma unroll
    for (int k = 0; k < KH; k++) {
      const int w = min(tid + SMF_TPB * k, NH - 1);
      int I, p, q, ex;
      if (MAT) {
        const int m = w / 81, c = (w / 9) % 9, e = w % 9;
        I = midx(m); p = midx(c); q = midx(e);
        ex = (I >= 3 ? -1 : 0) + mwt_log2(c) + mwt_log2(e);
      } else {
        I = w / 36; p = (w / 6) % 6; q = w % 6;
        ex = I >= 3 ? -1 : 0;
      }
      sort3(I, p, q);
      hidx[k] = sym3(I, p, q);
      hexp[k] = ex;
    }
    for (int mi = 0; mi < cnt; mi++) {
      double *o = H + (base + mi) * NH;
      const double *s = sG + mi * 56;
#pragma unroll
      for (int k = 0; k < KH; k++)
        if (tid + SMF_TPB * k < NH) o[tid + SMF_TPB * k] = mulpow2(s[hidx[k]], hexp[k]);
    }
  }
}

template <int KIND, bool MAT>
cudaError_t smf_launch_kind(int order, cudaStream_t st, unsigned blocks, int64_t n, const double *x,
                                   double *F, double *J, double *H, const SmfCoef &C) {
  if (order == 2) smf_kernel<KIND, 2, MAT><<<blocks, SMF_TPB, 0, st>>>(n, x, F, J, H, C);
  else if (order == 1) smf_kernel<KIND, 1, MAT><<<blocks, SMF_TPB, 0, st>>>(n, x, F, J, H, C);
  else smf_kernel<KIND, 0, MAT><<<blocks, SMF_TPB, 0, st>>>(n, x, F, J, H, C);
  return cudaGetLastError();
}

// host: the launch constants of a call (kind already normalised: sqrt has al = 0.5)
inline void smf_coef(int kind, double al, SmfCoef &C) {
  C.al = al;
  double bh = al - 1.0, bb = bh - al;
  C.bh1 = bh;
  C.bl1 = (al - (bh - bb)) + (-1.0 - bb);
  auto zpow = [](double e) { return e < 0 ? HUGE_VAL : (e == 0 ? 1.0 : 0.0); };
  C.zp1 = zpow(al - 1.0);
  C.z2 = al == 1.0 ? 0.0 : al * (al - 1.0) / 2.0 * zpow(al - 2.0);
  C.tau = (kind == POW && 3.0 / al < DD2_TAU) ? 3.0 / al : DD2_TAU;
  if (kind == EXP) {
    double f = 0.5;
    for (int k = 0; k < DD2_TERMS; k++) { C.c2[k] = f; f /= (k + 3.0); }
  } else if (kind == LOG) {
    for (int k = 0; k < DD2_TERMS; k++) C.c2[k] = (k % 2 ? 1.0 : -1.0) / (k + 2.0);
  } else {
    double b = al * (al - 1.0) / 2.0;
    for (int k = 0; k < DD2_TERMS; k++) { C.c2[k] = b; b *= (al - k - 2.0) / (k + 3.0); }
  }
}

// one kind (instantiated in smf_<kind>.cu so that the kinds compile in parallel)
template <int KIND>
cudaError_t smf_launch_t(double al, int64_t n, const double *x, bool mat, double *F, double *J, double *H,
                         cudaStream_t st) {
  SmfCoef C;
  smf_coef(KIND, al, C);
  const int order = H ? 2 : (J ? 1 : 0);
  const unsigned blocks = (unsigned)((n + SMF_TPB - 1) / SMF_TPB);
  return mat ? smf_launch_kind<KIND, true>(order, st, blocks, n, x, F, J, H, C)
             : smf_launch_kind<KIND, false>(order, st, blocks, n, x, F, J, H, C);
}

}  // namespace mf
