// smf_mixed.cuh -- mixed-precision symmetric family: FP32 input and output, FP32 for the bulk of the arithmetic.
//
// FP64 is kept only where FP32 would lose the result:
//   * the eigensystem (deviator, the cubic's trigonometric root, cross-product eigenvector, Jacobi rotation, Rayleigh
//     quotients): with condition numbers up to 1e6 and eigenvalue gaps down to 1e-12 an FP32 eigensolve loses the
//     small eigenvalues and the near-degenerate pairs entirely;
//   * the differences of eigenvalues that feed the near-coalescent branches of the divided differences (z, u, w and
//     the denominators of the difference formulas), taken from the FP64 eigenvalues before rounding to FP32.
// f(lambda), the first and second divided differences (stable forms, cluster series), the product vectors and the
// J / H forms of smf_kernels.cuh run in FP32.  The FP64 share per matrix drops from ~2.5k to ~0.4k operations, so
// on GB300 (FP64 at 1/74 of FP32) the kernel moves towards the HBM roofline, and FP32 storage halves the bytes.
// Accuracy against the FP64 oracle is stated per kind and order in the tests (<= 1e-6 relative, max-norm).
#pragma once
#include "smf_kernels.cuh"

namespace mf {

struct SmfCoefF {
  float al, alm1;   // exponent and exponent - 1
  float zp1, z2;    // 0^(al - 1), f''(0)/2 for powers
  float tau;        // cluster radius of the second divided difference
  float c2[DD2_TERMS];
};

MF_D float self(bool m, float a, float b) { return m ? a : b; }

// x * 2^k for k in [-3, 1], exact for normal floats (exponent arithmetic), a multiplication otherwise
MF_D float mulpow2f(float x, int k) {
  if (k == 0) return x;
  const int b = __float_as_int(x);
  const int e = (b >> 23) & 0xFF;
  if (e > 3 && e < 0xFE) return __int_as_float(b + (k << 23));
  return x * __int_as_float((127 + k) << 23);
}

template <int KIND>
MF_D float fun_f(float x, float al) {
  if (KIND == EXP) return expf(x);
  if (KIND == LOG) return logf(x);
  if (!(x > 0.f)) return 0.f;
  return KIND == SQRT ? sqrtf(x) : powf(x, al);
}

// f[a, b] in FP32 from FP64 eigenvalues (their difference and sum taken in FP64) -- smf_kernel.hpp:84-115
template <int KIND>
MF_D float dd1_f(double a, double b, float fa, float fb, const SmfCoefF &C) {
  if (KIND == EXP) {
    const float d = (float)fabs(a - b);
    return self(a > b, fa, fb) * self(d > 0.f, -expm1f(-d) / d, 1.f);
  }
  if (KIND == LOG) {
    const float s = (float)(0.5 * (a + b)), z = (float)(a - b) / (float)(a + b), az = fabsf(z), z2 = z * z;
    if (az < 1e-3f) return (1.f + z2 / 3.f + z2 * z2 / 5.f + z2 * z2 * z2 / 7.f) / s;
    if (az >= 0.5f) return (logf((float)a) - logf((float)b)) / (float)(a - b);
    return atanhf(z) / z / s;
  }
  a = sel(a > 0, a, 0.0);
  b = sel(b > 0, b, 0.0);
  if (KIND == SQRT) return 1.f / (sqrtf((float)a) + sqrtf((float)b));
  const double sd = 0.5 * (a + b);
  const float s = (float)sd, ss = self(s > 0.f, s, 1.f);
  const float z = (float)(a - b) / (2.f * ss), az = fabsf(z);
  const bool zero = az == 0.f, near = !zero & (az < 0.5f);
  if (!zero & !near) return (fa - fb) / (float)(a - b);
  const float g = zero ? C.al : (expm1f(C.al * log1pf(z)) - expm1f(C.al * log1pf(-z))) / (2.f * z);
  return (s > 0.f ? powf(ss, C.alm1) : C.zp1) * g;
}

template <int KIND>
MF_D float deriv_f(double x, float fx, const SmfCoefF &C) {
  if (KIND == EXP) return fx;
  if (KIND == LOG) return 1.f / (float)x;
  const float xf = self(x > 0, (float)x, 0.f);
  if (KIND == SQRT) return 1.f / (2.f * sqrtf(xf));
  return xf > 0.f ? C.al * powf(xf, C.alm1) : C.al * C.zp1;
}

// f[li, lj, lk] in FP32; the ordering and the differences of the FP64 eigenvalues in FP64 -- smf_kernel.hpp:148-192
template <int KIND>
MF_D float dd2_f(double li, double lj, double lk, float fi, float fj, float fk, float Dij, float Dik, float Djk,
                 const SmfCoefF &C) {
  if (KIND == POW || KIND == SQRT) {
    li = sel(li > 0, li, 0.0); lj = sel(lj > 0, lj, 0.0); lk = sel(lk > 0, lk, 0.0);
  }
  const double dA = lk - li, dB = lj - li, dC = lk - lj;
  const float aA = fabsf((float)dA), aB = fabsf((float)dB), aC = fabsf((float)dC);
  const bool useA = (aA >= aB) & (aA >= aC), useB = !useA & (aB >= aC);
  const float num = self(useA, Djk - Dij, self(useB, Djk - Dik, Dik - Dij));
  const float den = (float)sel(useA, dA, sel(useB, dB, dC));
  const double mn = sel(li < lj, li, lj), mx = sel(li < lj, lj, li);
  const double lo = sel(mn < lk, mn, lk), hi = sel(mx > lk, mx, lk), t = sel(mx < lk, mx, lk), mid = sel(mn > t, mn, t);
  const float u0 = (float)(lo - mid), w0 = (float)(hi - mid), midf = (float)mid;
  bool cluster;
  if (KIND == EXP) cluster = (w0 - u0) <= 1.f;
  else cluster = (midf > 0.f) & (-u0 <= C.tau * midf) & (w0 <= C.tau * midf);
  float out;
  if (cluster) {
    const float fm = self(mid == li, fi, self(mid == lj, fj, fk));
    float u, w, scale;
    if (KIND == EXP) {
      u = u0; w = w0; scale = fm;
    } else {
      u = u0 / midf; w = w0 / midf;
      scale = (KIND == LOG ? 1.f : fm) / (midf * midf);
    }
    float h = 1.f, wk = 1.f, s = C.c2[0];
#pragma unroll
    for (int k = 1; k < DD2_TERMS; k++) {
      wk = wk * w;
      h = fmaf(u, h, wk);
      s = fmaf(C.c2[k], h, s);
    }
    out = scale * s;
  } else {
    out = num / self(den != 0.f, den, 1.f);
  }
  if (KIND == POW || KIND == SQRT) out = self(hi > 0, out, C.z2);
  return out;
}

template <int KIND>
MF_D float dd2_same_f(double l, float fl, float Dll, const SmfCoefF &C) {
  if (KIND == POW || KIND == SQRT) l = sel(l > 0, l, 0.0);
  const float lf = (float)l;
  bool cluster = KIND == EXP ? true : (lf > 0.f);
  float out = KIND == EXP ? self(cluster, fl * C.c2[0], Dll - Dll)
                          : self(cluster, ((KIND == LOG ? 1.f : fl) / (lf * lf)) * C.c2[0], Dll - Dll);
  if (KIND == POW || KIND == SQRT) out = self(lf > 0.f, out, C.z2);
  return out;
}

constexpr int SMFX_TPB = 64;  // matrices per CTA of the standalone kernel

template <int ORDER, bool MAT, int TPB>
struct SmfxTileSmem {
  static constexpr int NIN = MAT ? 9 : 6, NF = MAT ? 9 : 6;
  float sX[TPB * NIN];
  float sF[TPB * NF];
  float sK[ORDER >= 1 ? TPB * 21 : 1];
  float sG[ORDER >= 2 ? TPB * 56 : 1];
};

template <int KIND, int ORDER, bool MAT, int SMFX_TPB>
MF_D void smf_mixed_tile(int64_t base, int cnt, const float *__restrict__ x, float *__restrict__ F,
                         float *__restrict__ J, float *__restrict__ H, const SmfCoefF &C,
                         SmfxTileSmem<ORDER, MAT, SMFX_TPB> &TS) {
  constexpr int NIN = MAT ? 9 : 6, NF = MAT ? 9 : 6, NJ = NF * NF, NH = NJ * NF;
  float *sX = TS.sX, *sF = TS.sF, *sK = TS.sK, *sG = TS.sG;
  const int tid = threadIdx.x;
  for (int e = tid; e < cnt * NIN; e += SMFX_TPB) sX[e] = x[base * NIN + e];
  __syncthreads();
  if (tid < cnt) {
    double v[6];
    const float *xi = sX + tid * NIN;
    if (MAT) {  // symmetric part; NaN if |a_ij - a_ji| > 1e-8 max|a| (checked in FP64 on the FP32 values)
      double a9[9], mx = 0.0;
#pragma unroll
      for (int k = 0; k < 9; k++) { a9[k] = xi[k]; mx = sel(fabs(a9[k]) > mx, fabs(a9[k]), mx); }
      const double tol = 1e-8 * mx;
      bool sym = !(fabs(a9[1] - a9[3]) > tol) & !(fabs(a9[2] - a9[6]) > tol) & !(fabs(a9[5] - a9[7]) > tol);
      v[0] = a9[0]; v[1] = a9[4]; v[2] = a9[8];
      v[3] = 0.5 * (a9[1] + a9[3]); v[4] = 0.5 * (a9[2] + a9[6]); v[5] = 0.5 * (a9[5] + a9[7]);
#pragma unroll
      for (int k = 0; k < 6; k++) v[k] = sel(sym, v[k], __longlong_as_double(0x7FF8000000000000ll));
    } else {
#pragma unroll
      for (int k = 0; k < 6; k++) v[k] = xi[k];
    }
    SmfEig E;
    smf_eigsys<KIND>(v, E);
    float fl[3], V[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      fl[i] = fun_f<KIND>((float)E.lam[i], C.al);
#pragma unroll
      for (int j = 0; j < 3; j++) V[i][j] = (float)E.V[i][j];
    }
    if (KIND == LOG) {
      const float mf = (float)E.m, lms = logf((float)(E.m * E.sig));
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const float xd = (float)E.xd[i];
        fl[i] = self(fabsf(xd) <= 0.5f * mf, lms + log1pf(xd / mf), fl[i]);
      }
    }
    float Fv[6];
#pragma unroll
    for (int s = 0; s < 6; s++) {
      const int a = vk_(s), b = vl_(s);
      Fv[s] = V[a][0] * fl[0] * V[b][0] + V[a][1] * fl[1] * V[b][1] + V[a][2] * fl[2] * V[b][2];
    }
    if (MAT) {
#pragma unroll
      for (int m = 0; m < 9; m++) sF[tid * 9 + m] = Fv[m % 4 == 0 ? m / 4 : (m == 1 || m == 3 ? 3 : (m == 2 || m == 6 ? 4 : 5))];
    } else {
#pragma unroll
      for (int s = 0; s < 6; s++) sF[tid * 6 + s] = Fv[s];
    }
    if (ORDER >= 1) {
      const double *lam = E.lam;
      const float D01 = dd1_f<KIND>(lam[0], lam[1], fl[0], fl[1], C), D02 = dd1_f<KIND>(lam[0], lam[2], fl[0], fl[2], C);
      const float D12 = dd1_f<KIND>(lam[1], lam[2], fl[1], fl[2], C);
      const float D00 = deriv_f<KIND>(lam[0], fl[0], C), D11 = deriv_f<KIND>(lam[1], fl[1], C);
      const float D22 = deriv_f<KIND>(lam[2], fl[2], C);
      float P[6][3];
#pragma unroll
      for (int s6 = 0; s6 < 6; s6++)
#pragma unroll
        for (int a = 0; a < 3; a++) P[s6][a] = V[vk_(s6)][a] * V[vl_(s6)][a];
      const float Dm[3][3] = {{D00, D01, D02}, {D01, D11, D12}, {D02, D12, D22}};
      {
        float Bv[21];
#pragma unroll
        for (int g = 0; g < 6; g++) {
          float dy[3];
#pragma unroll
          for (int a = 0; a < 3; a++) dy[a] = Dm[a][0] * P[g][0] + Dm[a][1] * P[g][1] + Dm[a][2] * P[g][2];
#pragma unroll
          for (int b2 = 0; b2 <= g; b2++) Bv[sym2(b2, g)] = P[b2][0] * dy[0] + P[b2][1] * dy[1] + P[b2][2] * dy[2];
        }
        float *k_out = sK + tid * 21;
#pragma unroll
        for (int I = 0; I < 6; I++)
#pragma unroll
          for (int p = I; p < 6; p++) {
            float acc = 0.f;
            bool first = true;
#pragma unroll
            for (int u1 = 0; u1 < 2; u1++)
#pragma unroll
              for (int u2 = 0; u2 < 2; u2++) {
                if ((u1 && vk_(I) == vl_(I)) || (u2 && vk_(p) == vl_(p))) continue;
                const int s1 = u1 ? vl_(I) : vk_(I), t1 = u1 ? vk_(I) : vl_(I);
                const int s2 = u2 ? vl_(p) : vk_(p), t2 = u2 ? vk_(p) : vl_(p);
                const int pa = pidx(s1, s2), pb = pidx(t1, t2);
                const float v2 = Bv[sym2(min(pa, pb), max(pa, pb))];
                acc = first ? v2 : acc + v2;
                first = false;
              }
            k_out[sym2(I, p)] = acc;
          }
      }
      if (ORDER >= 2) {
        float D2[3][3][3];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = i; j < 3; j++)
#pragma unroll
            for (int l = j; l < 3; l++) {
              const float d = (i == j && j == l) ? dd2_same_f<KIND>(lam[i], fl[i], Dm[i][i], C)
                                                 : dd2_f<KIND>(lam[i], lam[j], lam[l], fl[i], fl[j], fl[l], Dm[i][j],
                                                               Dm[i][l], Dm[j][l], C);
              D2[i][j][l] = D2[i][l][j] = D2[j][i][l] = D2[j][l][i] = D2[l][i][j] = D2[l][j][i] = d;
            }
        float Tv[56];
#pragma unroll
        for (int g = 0; g < 6; g++) {
          float M[3][3];
#pragma unroll
          for (int a = 0; a < 3; a++)
#pragma unroll
            for (int mm = a; mm < 3; mm++)
              M[a][mm] = M[mm][a] = D2[a][mm][0] * P[g][0] + D2[a][mm][1] * P[g][1] + D2[a][mm][2] * P[g][2];
#pragma unroll
          for (int h = 0; h <= g; h++) {
            float W[3];
#pragma unroll
            for (int a = 0; a < 3; a++) W[a] = M[a][0] * P[h][0] + M[a][1] * P[h][1] + M[a][2] * P[h][2];
#pragma unroll
            for (int f = 0; f <= h; f++) Tv[sym3(f, h, g)] = P[f][0] * W[0] + P[f][1] * W[1] + P[f][2] * W[2];
          }
        }
        float *g_out = sG + tid * 56;
#pragma unroll
        for (int z = 0; z < 6; z++)
#pragma unroll
          for (int y = 0; y <= z; y++)
#pragma unroll
            for (int I = 0; I <= y; I++) {
              float acc = 0.f;
              bool first = true;
#pragma unroll
              for (int u1 = 0; u1 < 2; u1++)
#pragma unroll
                for (int u2 = 0; u2 < 2; u2++)
#pragma unroll
                  for (int u3 = 0; u3 < 2; u3++) {
                    if ((u1 && vk_(I) == vl_(I)) || (u2 && vk_(y) == vl_(y)) || (u3 && vk_(z) == vl_(z))) continue;
                    const int s1 = u1 ? vl_(I) : vk_(I), t1 = u1 ? vk_(I) : vl_(I);
                    const int s2 = u2 ? vl_(y) : vk_(y), t2 = u2 ? vk_(y) : vl_(y);
                    const int s3 = u3 ? vl_(z) : vk_(z), t3 = u3 ? vk_(z) : vl_(z);
                    int a1 = pidx(s1, s2), a2 = pidx(t2, s3), a3 = pidx(t1, t3);
                    sort3(a1, a2, a3);
                    const float v3 = Tv[sym3(a1, a2, a3)];
                    acc = first ? v3 : acc + v3;
                    first = false;
                  }
              g_out[sym3(I, y, z)] = acc;
            }
      }
    }
  }
  __syncthreads();
  for (int e = tid; e < cnt * NF; e += SMFX_TPB) F[base * NF + e] = sF[e];
  if (ORDER >= 1) {
    constexpr int KJ = (NJ + SMFX_TPB - 1) / SMFX_TPB;
    int jidx[KJ], jexp[KJ];
#pragma unroll
    for (int k = 0; k < KJ; k++) {
      const int w = min(tid + SMFX_TPB * k, NJ - 1);
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
      float *o = J + (base + mi) * NJ;
      const float *s = sK + mi * 21;
#pragma unroll
      for (int k = 0; k < KJ; k++)
        if (tid + SMFX_TPB * k < NJ) o[tid + SMFX_TPB * k] = mulpow2f(s[jidx[k]], jexp[k]);
    }
  }
  if (ORDER >= 2) {
    constexpr int KH = (NH + SMFX_TPB - 1) / SMFX_TPB;
    int hidx[KH], hexp[KH];
#pragma unroll
    for (int k = 0; k < KH; k++) {
      const int w = min(tid + SMFX_TPB * k, NH - 1);
      int I, p, q, ex;
      if (MAT) {
        const int m = w / 81, c = (w / 9) % 9, e = w % 9;
        I = midx(m); p = midx(c); q = midx(e);
        ex = 1 + (I >= 3 ? -1 : 0) + mwt_log2(c) + mwt_log2(e);
      } else {
        I = w / 36; p = (w / 6) % 6; q = w % 6;
        ex = 1 + (I >= 3 ? -1 : 0);
      }
      sort3(I, p, q);
      hidx[k] = sym3(I, p, q);
      hexp[k] = ex;
    }
    for (int mi = 0; mi < cnt; mi++) {
      float *o = H + (base + mi) * NH;
      const float *s = sG + mi * 56;
#pragma unroll
      for (int k = 0; k < KH; k++)
        if (tid + SMFX_TPB * k < NH) o[tid + SMFX_TPB * k] = mulpow2f(s[hidx[k]], hexp[k]);
    }
  }
}

template <int KIND, int ORDER, bool MAT>
__global__ void __launch_bounds__(SMFX_TPB) smf_mixed_kernel(int64_t n, const float *__restrict__ x,
                                                             float *__restrict__ F, float *__restrict__ J,
                                                             float *__restrict__ H, const SmfCoefF C) {
  __shared__ SmfxTileSmem<ORDER, MAT, SMFX_TPB> TS;
  const int64_t base = (int64_t)blockIdx.x * SMFX_TPB;
  smf_mixed_tile<KIND, ORDER, MAT, SMFX_TPB>(base, (int)min((int64_t)SMFX_TPB, n - base), x, F, J, H, C, TS);
}

inline void smf_coef_f(int kind, double al, SmfCoefF &C) {
  SmfCoef D;
  smf_coef(kind, al, D);
  C.al = (float)al;
  C.alm1 = (float)(al - 1.0);
  C.zp1 = (float)D.zp1;
  C.z2 = (float)D.z2;
  C.tau = (float)D.tau;
  for (int k = 0; k < DD2_TERMS; k++) C.c2[k] = (float)D.c2[k];
}

template <int KIND>
cudaError_t smf_mixed_launch_t(double al, int64_t n, const float *x, bool mat, float *F, float *J, float *H,
                               cudaStream_t st) {
  SmfCoefF C;
  smf_coef_f(KIND, al, C);
  const int order = H ? 2 : (J ? 1 : 0);
  const unsigned blocks = (unsigned)((n + SMFX_TPB - 1) / SMFX_TPB);
  if (mat) {
    if (order == 2) smf_mixed_kernel<KIND, 2, true><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else if (order == 1) smf_mixed_kernel<KIND, 1, true><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else smf_mixed_kernel<KIND, 0, true><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
  } else {
    if (order == 2) smf_mixed_kernel<KIND, 2, false><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else if (order == 1) smf_mixed_kernel<KIND, 1, false><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else smf_mixed_kernel<KIND, 0, false><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
  }
  return cudaGetLastError();
}

}  // namespace mf
