// gmf_adjoint_tile.cuh -- one tile of the general adjoint kernels (gmf_cuda_adjoint, FP64; gmf_cuda_adjoint_f32,
// FP32 arrays): per thread the record of gmf_device.cuh, after a CTA-local ordering by class and series length, and
// its contraction with the directions W and V (the formulas are given in adjoint.cuh); coalesced load and store
// through shared memory.
#pragma once

#include "gmf_device.cuh"

namespace mf {

template <typename T>
MF_D void mm3(const T *X, const T *Y, T *Z) {  // Z = X Y
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Z[3 * i + j] = X[3 * i] * Y[j] + X[3 * i + 1] * Y[3 + j] + X[3 * i + 2] * Y[6 + j];
}
template <typename T>
MF_D void mmT3(const T *X, const T *Y, T *Z) {  // Z = X Y^T
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      Z[3 * i + j] = X[3 * i] * Y[3 * j] + X[3 * i + 1] * Y[3 * j + 1] + X[3 * i + 2] * Y[3 * j + 2];
}
template <typename T>
MF_D void mTm3(const T *X, const T *Y, T *Z) {  // Z = X^T Y
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Z[3 * i + j] = X[i] * Y[j] + X[3 + i] * Y[3 + j] + X[6 + i] * Y[6 + j];
}

// the output factor of a record, applied last as in the reference (NaN for a matrix outside the domain)
template <typename T>
MF_D T scale_out(T v, T sc) { return v * sc; }

// The contractions of one matrix's record (r_0 = I, r_1, r_2; D2' times s1, D3' times s2) with the directions, in the
// compute type TC (the record and directions rounded to TC first), ABS: of the absolute values of record and
// directions (the bound of the terms of each entry):
//   o[0] = Abar / sc1 = sum_m r_m^T (sum_n D2'_mn W r_n^T)
//   o[1] = JV / sc1   = sum_m r_m (sum_n D2'_mn V r_n)
//   o[2] = HWV / sc2  = sum_p (X_p^T W r_p^T + r_p^T W X_p^T),  X_p = sum_mn D3'_mnp r_m V r_n
// (only those asked for: dA, dJ, dH)
template <int ORDER, typename TC, bool ABS>
MF_D void gadj_contract(const GmfRec &R, double s1, double s2, const double *w, const double *v, bool dA, bool dJ,
                        bool dH, TC o[3][9]) {
  auto rd = [](double x) { return ABS ? (TC)fabs(x) : (TC)x; };
  TC r[3][9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    r[0][k] = k % 4 == 0 ? TC(1) : TC(0);
    r[1][k] = rd(R.r1[k]);
    r[2][k] = rd(R.r2[k]);
  }
  TC D2s[6], D3s[10];
#pragma unroll
  for (int k = 0; k < 6; k++) D2s[k] = rd(R.D2[k] * s1);
#pragma unroll
  for (int k = 0; k < 10; k++) D3s[k] = ORDER >= 2 ? rd(R.D3[k] * s2) : TC(0);
  const TC D2m[3][3] = {{D2s[0], D2s[3], D2s[4]}, {D2s[3], D2s[1], D2s[5]}, {D2s[4], D2s[5], D2s[2]}};
  TC Wl[9], Vl[9];
#pragma unroll
  for (int k = 0; k < 9; k++) { Wl[k] = dA | dH ? rd(w[k]) : TC(0); Vl[k] = dJ | dH ? rd(v[k]) : TC(0); }
  TC Gw[3][9];  // W r_n^T
  if (dA || dH) {
#pragma unroll
    for (int k = 0; k < 9; k++) Gw[0][k] = Wl[k];
    mmT3(Wl, r[1], Gw[1]);
    mmT3(Wl, r[2], Gw[2]);
  }
  if (dA) {
    TC acc[9];
#pragma unroll
    for (int k = 0; k < 9; k++) acc[k] = TC(0);
#pragma unroll
    for (int mm = 0; mm < 3; mm++) {
      TC Hm[9], Tm[9];
#pragma unroll
      for (int k = 0; k < 9; k++) Hm[k] = D2m[mm][0] * Gw[0][k] + D2m[mm][1] * Gw[1][k] + D2m[mm][2] * Gw[2][k];
      if (mm == 0) {
#pragma unroll
        for (int k = 0; k < 9; k++) acc[k] += Hm[k];
      } else {
        mTm3(r[mm], Hm, Tm);
#pragma unroll
        for (int k = 0; k < 9; k++) acc[k] += Tm[k];
      }
    }
#pragma unroll
    for (int k = 0; k < 9; k++) o[0][k] = acc[k];
  }
  TC Gv[3][9];  // V r_n
  if (dJ || dH) {
#pragma unroll
    for (int k = 0; k < 9; k++) Gv[0][k] = Vl[k];
    mm3(Vl, r[1], Gv[1]);
    mm3(Vl, r[2], Gv[2]);
  }
  if (dJ) {
    TC acc[9];
#pragma unroll
    for (int k = 0; k < 9; k++) acc[k] = TC(0);
#pragma unroll
    for (int mm = 0; mm < 3; mm++) {
      TC Hm[9], Tm[9];
#pragma unroll
      for (int k = 0; k < 9; k++) Hm[k] = D2m[mm][0] * Gv[0][k] + D2m[mm][1] * Gv[1][k] + D2m[mm][2] * Gv[2][k];
      if (mm == 0) {
#pragma unroll
        for (int k = 0; k < 9; k++) acc[k] += Hm[k];
      } else {
        mm3(r[mm], Hm, Tm);
#pragma unroll
        for (int k = 0; k < 9; k++) acc[k] += Tm[k];
      }
    }
#pragma unroll
    for (int k = 0; k < 9; k++) o[1][k] = acc[k];
  }
  if (ORDER >= 2 && dH) {
    TC X[3][9];
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
      for (int k = 0; k < 9; k++) X[p][k] = TC(0);
#pragma unroll
    for (int mm = 0; mm < 3; mm++)
#pragma unroll
      for (int nn = 0; nn < 3; nn++) {
        TC M[9];
        if (mm == 0) {
#pragma unroll
          for (int k = 0; k < 9; k++) M[k] = Gv[nn][k];
        } else {
          mm3(r[mm], Gv[nn], M);
        }
#pragma unroll
        for (int p = 0; p < 3; p++) {
          int i0 = mm, i1 = nn, i2 = p;
          sort3(i0, i1, i2);
          const TC d = D3s[sym3(i0, i1, i2)];
#pragma unroll
          for (int k = 0; k < 9; k++) X[p][k] += d * M[k];
        }
      }
    TC acc[9];
#pragma unroll
    for (int k = 0; k < 9; k++) acc[k] = TC(0);
#pragma unroll
    for (int p = 0; p < 3; p++) {
      TC T1[9], T2[9], T3[9];
      mTm3(X[p], Gw[p], T1);  // X_p^T (W r_p^T)
      mmT3(Wl, X[p], T2);     // W X_p^T
      if (p == 0) {
#pragma unroll
        for (int k = 0; k < 9; k++) T3[k] = T2[k];
      } else {
        mTm3(r[p], T2, T3);   // r_p^T W X_p^T
      }
#pragma unroll
      for (int k = 0; k < 9; k++) acc[k] += T1[k] + T3[k];
    }
#pragma unroll
    for (int k = 0; k < 9; k++) o[2][k] = acc[k];
  }
}

// FP32 adjoints: a matrix is recomputed from its FP64 record where an output's term bound exceeds this many times
// its largest |entry| (cancellation amplifies the FP32 rounding of the record by that ratio)
constexpr float GADJ_F32_AMP = 8.f;

// shared memory of one tile
template <int TPB>
struct GadjSmemT {
  double x[TPB * 9], w[TPB * 9], v[TPB * 9];
  double out[4][TPB * 9];  // F, Abar, JV, HWV staging
  GmfState state[TPB];
  unsigned key[TPB];
  int perm[TPB];
  long long gidx[TPB];  // tile position -> matrix index (the ordered launch)
};

// one tile: the matrices base .. base + cnt - 1 by a CTA of TPB threads; idx (optional): tile position p holds
// matrix idx[base + p] of the arrays (the ordered launch)
template <int KIND, int ORDER, typename T, int TPB>
MF_D void gmf_adjoint_tile(int64_t base, int cnt, const T *__restrict__ A, const T *__restrict__ W,
                           const T *__restrict__ V, T *__restrict__ F, T *__restrict__ Abar, T *__restrict__ JV,
                           T *__restrict__ HWV, const GmfCoef &C, const int *__restrict__ idx,
                           GadjSmemT<TPB> &S) {
  const int tid = threadIdx.x;
  for (int e = tid; e < cnt * 9; e += TPB) {  // (idx: position p holds matrix idx[base + p])
    const int p = e / 9;
    const long long g = idx ? (long long)idx[base + p] : base + p, ge = g * 9 + (e - 9 * p);
    S.x[e] = A[ge];
    if (W) S.w[e] = W[ge];
    if (V) S.v[e] = V[ge];
    if (e == 9 * p) S.gidx[p] = g;
  }
  __syncthreads();
  unsigned key = 0xFFFFFFFFu;
  if (tid < cnt) {
    double a[9];
#pragma unroll
    for (int k = 0; k < 9; k++) a[k] = S.x[tid * 9 + k];
    GmfState St;
    gmf_classify<KIND, ORDER>(a, C, St);
    S.state[tid] = St;
    key = gmf_finish_key(St);
  }
  S.key[tid] = key;
  __syncthreads();
  {
    int rank = 0;
    for (int j = 0; j < TPB; j++) {
      const unsigned kj = S.key[j];
      rank += (kj < key) | ((kj == key) & (j < tid));
    }
    S.perm[rank] = tid;
  }
  __syncthreads();
  const int mine = S.perm[tid];
  if (mine < cnt) {
    GmfRec R;
    gmf_finish<KIND, ORDER, sizeof(T) == 4>(S.state[mine], C, R);
    // FP32: fold the scale factors into D2', D3' in FP64 when finite and nonzero, then round the record once
    constexpr bool MIXED = sizeof(T) == 4;
    const double rsc2 = ORDER >= 2 ? R.sc2 : 1.0;
    const bool f1 = MIXED & isfinite(R.sc1) & (R.sc1 != 0.0), f2 = MIXED & isfinite(rsc2) & (rsc2 != 0.0);
    const double s1 = sel(f1, R.sc1, 1.0), s2 = sel(f2, rsc2, 1.0);
    const T sc1 = (T)sel(f1, 1.0, R.sc1), sc2 = (T)sel(f2, 1.0, rsc2);
    if (F) {
#pragma unroll
      for (int k = 0; k < 9; k++) S.out[0][mine * 9 + k] = R.F[k];
    }
    const double *w = S.w + mine * 9, *v = S.v + mine * 9;
    const bool dA = Abar != nullptr, dJ = JV != nullptr, dH = ORDER >= 2 && HWV != nullptr;
    double o[3][9];
    if constexpr (!MIXED) {
      gadj_contract<ORDER, double, false>(R, s1, s2, w, v, dA, dJ, dH, o);
    } else {
      // FP32: the record rounded once and contracted in FP32, and the same contraction of the absolute values (the
      // bound of the terms); an output whose bound exceeds GADJ_F32_AMP times its largest |entry| has cancelled, and
      // the matrix is contracted again from its FP64 record (near-defective matrices: nearly dependent r_0, r_1, r_2
      // against large divided differences)
      float of[3][9], bf[3][9];
      gadj_contract<ORDER, float, false>(R, s1, s2, w, v, dA, dJ, dH, of);
      gadj_contract<ORDER, float, true>(R, s1, s2, w, v, dA, dJ, dH, bf);
      bool wide = false;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        float mo = 0.f, mb = 0.f;
#pragma unroll
        for (int k = 0; k < 9; k++) { mo = fmaxf(mo, fabsf(of[q][k])); mb = fmaxf(mb, bf[q][k]); }
        wide = wide | (mb > GADJ_F32_AMP * mo);
      }
      if (wide) {
        gadj_contract<ORDER, double, false>(R, s1, s2, w, v, dA, dJ, dH, o);
      } else {
#pragma unroll
        for (int q = 0; q < 3; q++)
#pragma unroll
          for (int k = 0; k < 9; k++) o[q][k] = of[q][k];
      }
    }
#pragma unroll
    for (int k = 0; k < 9; k++) {
      if (dA) S.out[1][mine * 9 + k] = scale_out(o[0][k], (double)sc1);
      if (dJ) S.out[2][mine * 9 + k] = scale_out(o[1][k], (double)sc1);
      if (dH) S.out[3][mine * 9 + k] = scale_out(o[2][k], (double)sc2);
    }
  }
  __syncthreads();
  T *dst[4] = {F, Abar, JV, HWV};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (!dst[q]) continue;
    for (int e = tid; e < cnt * 9; e += TPB) dst[q][S.gidx[e / 9] * 9 + e % 9] = (T)S.out[q][e];
  }
}

}  // namespace mf
