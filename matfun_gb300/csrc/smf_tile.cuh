// smf_tile.cuh -- one tile of the symmetric family (smf_cuda_eval / smf_cuda_eval_matrix), FP64, Voigt or matrix
// layout: the code a CTA of the standalone kernel, of the ordered launch and of the batched persistent kernel runs.
//
// One CTA = 64 matrices (two warps).  Phase A: one thread per matrix computes the eigensystem, f, the divided
// differences and the distinct entries of J (21 values of the symmetric form K) and H (56 values of the symmetric
// form G'), see smf_device.cuh, into shared memory.  Both forms are evaluated through the product vectors
// P_kl = (V_ka V_la)_a of rows of V: J from the 21 values of B(x, y) = sum D_ab x_a y_b, H from the 56 values of
// T(x, y, z) = sum D2_amb x_a y_m z_b, about half the FP64 instructions of assembling V S V^T per index pair.
// Phase B: the CTA expands them into the output layout with coalesced stores (64 consecutive doubles of a row per
// store instruction); the layout weights (powers of two) are applied on the exponent bits, not on the FP64 pipe.
#pragma once

#include "smf_device.cuh"

namespace mf {

constexpr int SMF_TPB = 64;  // matrices per CTA of the standalone kernel

// index of the product vector of the Cartesian pair (k, l) (Voigt order 00 11 22 01 02 12)
MF_D constexpr int pidx(int k, int l) { return k == l ? k : k + l + 2; }

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

// shared memory of one tile of TPB matrices
template <int ORDER, bool MAT, int TPB>
struct SmfTileSmem {
  static constexpr int NIN = MAT ? 9 : 6, NF = MAT ? 9 : 6;
  double sX[TPB * NIN];
  double sF[TPB * NF];
  double sK[ORDER >= 1 ? TPB * 21 : 1];
  double sG[ORDER >= 2 ? TPB * 56 : 1];
  long long gidx[TPB];  // tile position -> matrix index in the arrays
};

// order 2: whether a matrix's eigenvalues hold a pair inside the cluster radius of the second divided differences
// (exp: |a - b| <= tau; log, powers: |a - b| <= tau max(a, b), max > 0): without one, every f[x, y, z] of the matrix
// takes the difference formula (smf_dd2)
template <int KIND>
MF_D bool smf_any_cluster(const double lam[3], const SmfCoef &C) {
  auto close = [&](double a, double b) -> bool {
    const double d = fabs(a - b);
    if (KIND == EXP) return d <= C.tau;
    const double m = fmax(a, b);
    return (m > 0) & (d <= C.tau * m);
  };
  return close(lam[0], lam[1]) | close(lam[0], lam[2]) | close(lam[1], lam[2]);
}

// one tile: matrices base .. base + cnt - 1 (cnt <= SMF_TPB) by a CTA of NT >= SMF_TPB threads (the standalone kernel
// and the batched persistent kernel run the same code): phase A by the first cnt threads, the cooperative loads and
// stores by all NT; idx (optional): tile position p holds matrix idx[base + p] of the arrays instead of base + p (the
// ordered launch).  At order 2 the matrices are dealt out to the threads anew after the eigensystem: those with a
// cluster (smf_any_cluster) go to the last threads, so that the warps before them run the difference formula on
// every lane instead of both branches of the second divided differences; results do not depend on the assignment.
template <int KIND, int ORDER, bool MAT, int SMF_TPB, int NT = SMF_TPB>
MF_D void smf_tile(int64_t base, int cnt, const double *__restrict__ x, double *__restrict__ F,
                   double *__restrict__ J, double *__restrict__ H, const SmfCoef &C, int *__restrict__ asym,
                   SmfTileSmem<ORDER, MAT, SMF_TPB> &TS, const int *__restrict__ idx = nullptr) {
  constexpr int NIN = MAT ? 9 : 6, NF = MAT ? 9 : 6, NJ = NF * NF, NH = NJ * NF;
  double *sX = TS.sX, *sF = TS.sF, *sK = TS.sK, *sG = TS.sG;
  const int tid = threadIdx.x;

  for (int e = tid; e < cnt * NIN; e += NT) {  // coalesced input (row-wise under idx)
    const int p = e / NIN;
    const long long g = idx ? (long long)idx[base + p] : base + p;
    sX[e] = x[g * NIN + (e - NIN * p)];
    if (e == NIN * p) TS.gidx[p] = g;
  }
  // order 2, until the eigensystems are dealt out: sK holds perm[SMF_TPB] (thread -> tile position of the matrix whose
  // J and H it computes) and part[2] (positions taken from the front, matrices without a cluster, and from the back)
  int *perm = reinterpret_cast<int *>(sK), *part = perm + (ORDER >= 2 ? SMF_TPB : 0);
  if (ORDER >= 2 && tid == 0) part[0] = part[1] = 0;
  __syncthreads();
  griddep_launch_dependents();  // the scratch of an ordered launch (idx: rows of the last matrices' H) has been read

  double lam[3], fl[3], V[3][3];
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
      if (!sym && asym) atomicAdd(asym, 1);  // counted for the host entry points (-3), NaN results either way
    } else {
#pragma unroll
      for (int k = 0; k < 6; k++) v[k] = xi[k];
    }
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
  }
  int mi = tid;  // the tile position whose J and H this thread computes
  if (ORDER >= 2) {
    double *stt = sG;  // the eigensystems, [15][SMF_TPB], until sG receives the results
    if (tid < cnt) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        stt[k * SMF_TPB + tid] = lam[k];
        stt[(3 + k) * SMF_TPB + tid] = fl[k];
#pragma unroll
        for (int b = 0; b < 3; b++) stt[(6 + 3 * k + b) * SMF_TPB + tid] = V[k][b];
      }
      const int pos = smf_any_cluster<KIND>(lam, C) ? cnt - 1 - atomicAdd(&part[1], 1) : atomicAdd(&part[0], 1);
      perm[pos] = tid;
    }
    __syncthreads();
    if (tid < cnt) {
      mi = perm[tid];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        lam[k] = stt[k * SMF_TPB + mi];
        fl[k] = stt[(3 + k) * SMF_TPB + mi];
#pragma unroll
        for (int b = 0; b < 3; b++) V[k][b] = stt[(6 + 3 * k + b) * SMF_TPB + mi];
      }
    }
    __syncthreads();  // every eigensystem and perm are read before sG and sK receive results
  }
  if (tid < cnt) {
    if (ORDER >= 1) {
      // divided differences D (smf_kernel.hpp:299-302)
      double D01 = smf_dd1<KIND>(lam[0], lam[1], fl[0], fl[1], C);
      double D02 = smf_dd1<KIND>(lam[0], lam[2], fl[0], fl[2], C);
      double D12 = smf_dd1<KIND>(lam[1], lam[2], fl[1], fl[2], C);
      double D00 = smf_deriv<KIND>(lam[0], fl[0], C), D11 = smf_deriv<KIND>(lam[1], fl[1], C);
      double D22 = smf_deriv<KIND>(lam[2], fl[2], C);
      // product vectors P_s[a] = V[k][a] V[l][a] of the Voigt pairs s = (k, l): with them
      //   K(I, p)     = B(P, P) sums,  B(x, y)    = sum_ab  D_ab  x_a y_b          (21 distinct values)
      //   G'(I, p, q) = 2 T(P, P, P) sums, T(x, y, z) = sum_amb D2_amb x_a y_m z_b  (56 distinct values)
      // because Et_p = V^T E_p V is a sum of one or two outer products of rows of V
      double P[6][3];
#pragma unroll
      for (int s6 = 0; s6 < 6; s6++)
#pragma unroll
        for (int a = 0; a < 3; a++) P[s6][a] = V[vk_(s6)][a] * V[vl_(s6)][a];
      const double Dm[3][3] = {{D00, D01, D02}, {D01, D11, D12}, {D02, D12, D22}};
      {
        double Bv[21];
#pragma unroll
        for (int g = 0; g < 6; g++) {
          double dy[3];
#pragma unroll
          for (int a = 0; a < 3; a++) dy[a] = Dm[a][0] * P[g][0] + Dm[a][1] * P[g][1] + Dm[a][2] * P[g][2];
#pragma unroll
          for (int b2 = 0; b2 <= g; b2++) Bv[sym2(b2, g)] = P[b2][0] * dy[0] + P[b2][1] * dy[1] + P[b2][2] * dy[2];
        }
        double *k_out = sK + mi * 21;
#pragma unroll
        for (int I = 0; I < 6; I++)
#pragma unroll
          for (int p = I; p < 6; p++) {
            // Et_I,ab Et_p,ab summed with D: the outer-product terms (s1, t1) of E_I and (s2, t2) of E_p give
            // B(P[s1 s2], P[t1 t2])
            double acc = 0.0;
            bool first = true;
#pragma unroll
            for (int u1 = 0; u1 < 2; u1++)
#pragma unroll
              for (int u2 = 0; u2 < 2; u2++) {
                if ((u1 && vk_(I) == vl_(I)) || (u2 && vk_(p) == vl_(p))) continue;
                const int s1 = u1 ? vl_(I) : vk_(I), t1 = u1 ? vk_(I) : vl_(I);
                const int s2 = u2 ? vl_(p) : vk_(p), t2 = u2 ? vk_(p) : vl_(p);
                const int pa = pidx(s1, s2), pb = pidx(t1, t2);
                const double v = Bv[sym2(min(pa, pb), max(pa, pb))];
                acc = first ? v : acc + v;
                first = false;
              }
            k_out[sym2(I, p)] = acc;
          }
      }
      if (ORDER >= 2) {
        // second divided differences over the 10 distinct triples (smf_kernel.hpp:328-338)
        double D2[3][3][3];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = i; j < 3; j++)
#pragma unroll
            for (int l = j; l < 3; l++) {
              const double d = (i == j && j == l)
                                   ? smf_dd2_same<KIND>(lam[i], fl[i], Dm[i][i], C)
                                   : smf_dd2<KIND>(lam[i], lam[j], lam[l], fl[i], fl[j], fl[l], Dm[i][j], Dm[i][l],
                                                   Dm[j][l], C);
              D2[i][j][l] = D2[i][l][j] = D2[j][i][l] = D2[j][l][i] = D2[l][i][j] = D2[l][j][i] = d;
            }
        // T over all sorted triples of product vectors: M_g[a][m] = sum_b D2_amb P_g[b], W_hg[a] = sum_m M_g[a][m]
        // P_h[m], T_fhg = sum_a P_f[a] W_hg[a]
        double Tv[56];
#pragma unroll
        for (int g = 0; g < 6; g++) {
          double M[3][3];
#pragma unroll
          for (int a = 0; a < 3; a++)
#pragma unroll
            for (int mm = a; mm < 3; mm++)
              M[a][mm] = M[mm][a] = D2[a][mm][0] * P[g][0] + D2[a][mm][1] * P[g][1] + D2[a][mm][2] * P[g][2];
#pragma unroll
          for (int h = 0; h <= g; h++) {
            double W[3];
#pragma unroll
            for (int a = 0; a < 3; a++) W[a] = M[a][0] * P[h][0] + M[a][1] * P[h][1] + M[a][2] * P[h][2];
#pragma unroll
            for (int f = 0; f <= h; f++) Tv[sym3(f, h, g)] = P[f][0] * W[0] + P[f][1] * W[1] + P[f][2] * W[2];
          }
        }
        // G'(I, y, z) / 2 = sum over the outer-product terms (s1, t1), (s2, t2), (s3, t3) of E_I, E_y, E_z of
        // T(P[s1 s2], P[t2 s3], P[t1 t3]); the factor 2 goes into the output weight
        double *g_out = sG + mi * 56;
#pragma unroll
        for (int z = 0; z < 6; z++)
#pragma unroll
          for (int y = 0; y <= z; y++)
#pragma unroll
            for (int I = 0; I <= y; I++) {
              double acc = 0.0;
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
                    const double v = Tv[sym3(a1, a2, a3)];
                    acc = first ? v : acc + v;
                    first = false;
                  }
              g_out[sym3(I, y, z)] = acc;
            }
      }
    }
  }
  __syncthreads();

  // ---- phase B: coalesced expansion into the output layout
  for (int e = tid; e < cnt * NF; e += NT) F[TS.gidx[e / NF] * NF + e % NF] = sF[e];
  if (ORDER >= 1) {
    constexpr int KJ = (NJ + NT - 1) / NT;
    int jidx[KJ], jexp[KJ];
#pragma unroll
    for (int k = 0; k < KJ; k++) {
      const int w = min(tid + NT * k, NJ - 1);
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
      double *o = J + TS.gidx[mi] * NJ;
      const double *s = sK + mi * 21;
#pragma unroll
      for (int k = 0; k < KJ; k++)
        if (tid + NT * k < NJ) o[tid + NT * k] = mulpow2(s[jidx[k]], jexp[k]);
    }
  }
  if (ORDER >= 2) {
    constexpr int KH = (NH + NT - 1) / NT;
    int hidx[KH], hexp[KH];
#pragma unroll
    for (int k = 0; k < KH; k++) {
      const int w = min(tid + NT * k, NH - 1);
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
      double *o = H + TS.gidx[mi] * NH;
      const double *s = sG + mi * 56;
#pragma unroll
      for (int k = 0; k < KH; k++)
        if (tid + NT * k < NH) o[tid + NT * k] = mulpow2(s[hidx[k]], hexp[k]);
    }
  }
}

}  // namespace mf
