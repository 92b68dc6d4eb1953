// adjoint.cuh -- adjoint kernels: contractions of J and H with given directions, without forming J or H.
//   VJP  Abar = J^T W     (Abar_cd = sum_ab W_ab J_abcd)           the gradient of <W, f(A)>
//   JVP  JV   = J V       ((JV)_ab = sum_cd J_abcd V_cd)            the derivative of f(A) along V
//   HVP  HWV  = W . H . V (HWV_ef = sum_abcd W_ab H_abcdef V_cd)   the derivative of the gradient along V
// (matrix layout, 3x3 row-major arrays, one matrix after another).
//
// General matrices, from the record of gmf_device.cuh (real basis r_0 = I, r_1, r_2; reduced D2', D3'):
//   Abar = sc1 sum_mn D2'_mn r_m^T W r_n^T,   JV = sc1 sum_mn D2'_mn r_m V r_n,
//   HWV  = sc2 sum_p (X_p^T W r_p^T + r_p^T W X_p^T),   X_p = sum_mn D3'_mnp r_m V r_n
// (the transposes of J_abcd = sc1 sum D2'_mn r_m[ac] r_n[db] and H_abcdef = sc2 (T6[ac,de,fb] + T6[ae,fc,db])).
// Symmetric matrices (derivatives of A -> f((A + A^T)/2)), with U the eigenvectors, D, D2 the divided differences,
// Wt = U^T sym(W) U, Vt = U^T sym(V) U:
//   Abar = U (D o Wt) U^T,   JV = U (D o Vt) U^T,   HWV = U (Q + Q^T) U^T,  Q_xy = sum_z D2_xyz Wt_xz Vt_yz
// (Daleckii-Krein and its second-order form; the first-order map is self-adjoint on symmetric directions).
//
// Mixed precision (FP32 arrays, T = float): gmf keeps its FP64 record (spectral analysis, series, residues), folds the
// scale factors into it in FP64 and rounds it to FP32 once for the contractions; smf takes the eigensystem and the
// divided differences of the mixed smf kernel (smf_mixed_math.cuh) and contracts in FP32.
#pragma once
#include "gmf_kernels.cuh"
#include "smf_kernels.cuh"
#include "smf_mixed.cuh"
#include "smf_adjoint_tile.cuh"

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

enum { ADJ_F = 1, ADJ_VJP = 2, ADJ_JVP = 4, ADJ_HVP = 8 };

// ------------------------------------------------------------------------------------------------ general
constexpr int GADJ_TPB = 128;

struct GadjSmem {
  double x[GADJ_TPB * 9], w[GADJ_TPB * 9], v[GADJ_TPB * 9];
  double out[4][GADJ_TPB * 9];  // F, Abar, JV, HWV staging
  GmfState state[GADJ_TPB];
  unsigned key[GADJ_TPB];
  int perm[GADJ_TPB];
  long long gidx[GADJ_TPB];  // tile position -> matrix index (the ordered launch)
};

template <int KIND, int ORDER, typename T>
__global__ void __launch_bounds__(GADJ_TPB) gmf_adjoint_kernel(int64_t n, const T *__restrict__ A,
                                                               const T *__restrict__ W, const T *__restrict__ V,
                                                               T *__restrict__ F, T *__restrict__ Abar,
                                                               T *__restrict__ JV, T *__restrict__ HWV,
                                                               const GmfCoef C, const int *__restrict__ idx) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GadjSmem &S = *reinterpret_cast<GadjSmem *>(smem_raw);
  const int tid = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * GADJ_TPB;
  const int cnt = (int)min((int64_t)GADJ_TPB, n - base);
  for (int e = tid; e < cnt * 9; e += GADJ_TPB) {  // (idx: position p holds matrix idx[base + p])
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
    const unsigned cls = St.K == 0 ? 0u : ((St.flags & 1024) ? 1u : 2u);
    key = (cls << 16) | ((unsigned)(255 - St.K) << 6) | (unsigned)((St.flags >> 3) & 63);
  }
  S.key[tid] = key;
  __syncthreads();
  {
    int rank = 0;
    for (int j = 0; j < GADJ_TPB; j++) {
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
    T r[3][9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
      r[0][k] = k % 4 == 0 ? T(1) : T(0);
      r[1][k] = (T)R.r1[k];
      r[2][k] = (T)R.r2[k];
    }
    T D2s[6], D3s[10];
#pragma unroll
    for (int k = 0; k < 6; k++) D2s[k] = (T)(R.D2[k] * s1);
#pragma unroll
    for (int k = 0; k < 10; k++) D3s[k] = ORDER >= 2 ? (T)(R.D3[k] * s2) : T(0);
    const T D2m[3][3] = {{D2s[0], D2s[3], D2s[4]}, {D2s[3], D2s[1], D2s[5]}, {D2s[4], D2s[5], D2s[2]}};
    if (F) {
#pragma unroll
      for (int k = 0; k < 9; k++) S.out[0][mine * 9 + k] = R.F[k];
    }
    const double *w = S.w + mine * 9, *v = S.v + mine * 9;
    T Wl[9], Vl[9];
#pragma unroll
    for (int k = 0; k < 9; k++) { Wl[k] = W ? (T)w[k] : T(0); Vl[k] = V ? (T)v[k] : T(0); }
    T Gw[3][9];  // W r_n^T
    if (Abar || HWV) {
#pragma unroll
      for (int k = 0; k < 9; k++) Gw[0][k] = Wl[k];
      mmT3(Wl, r[1], Gw[1]);
      mmT3(Wl, r[2], Gw[2]);
    }
    if (Abar) {  // sc1 sum_m r_m^T (sum_n D2'_mn W r_n^T)
      T acc[9];
#pragma unroll
      for (int k = 0; k < 9; k++) acc[k] = T(0);
#pragma unroll
      for (int mm = 0; mm < 3; mm++) {
        T Hm[9], Tm[9];
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
      for (int k = 0; k < 9; k++) S.out[1][mine * 9 + k] = scale_out(acc[k], sc1);
    }
    T Gv[3][9];  // V r_n
    if (JV || HWV) {
#pragma unroll
      for (int k = 0; k < 9; k++) Gv[0][k] = Vl[k];
      mm3(Vl, r[1], Gv[1]);
      mm3(Vl, r[2], Gv[2]);
    }
    if (JV) {  // sc1 sum_m r_m (sum_n D2'_mn V r_n)
      T acc[9];
#pragma unroll
      for (int k = 0; k < 9; k++) acc[k] = T(0);
#pragma unroll
      for (int mm = 0; mm < 3; mm++) {
        T Hm[9], Tm[9];
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
      for (int k = 0; k < 9; k++) S.out[2][mine * 9 + k] = scale_out(acc[k], sc1);
    }
    if (ORDER >= 2 && HWV) {
      // M_mn = r_m V r_n ; X_p = sum_mn D3'_mnp M_mn ; HWV = sc2 sum_p (X_p^T W r_p^T + r_p^T W X_p^T)
      T X[3][9];
#pragma unroll
      for (int p = 0; p < 3; p++)
#pragma unroll
        for (int k = 0; k < 9; k++) X[p][k] = T(0);
#pragma unroll
      for (int mm = 0; mm < 3; mm++)
#pragma unroll
        for (int nn = 0; nn < 3; nn++) {
          T M[9];
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
            const T d = D3s[sym3(i0, i1, i2)];
#pragma unroll
            for (int k = 0; k < 9; k++) X[p][k] += d * M[k];
          }
        }
      T acc[9];
#pragma unroll
      for (int k = 0; k < 9; k++) acc[k] = T(0);
#pragma unroll
      for (int p = 0; p < 3; p++) {
        T T1[9], T2[9], T3[9];
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
      for (int k = 0; k < 9; k++) S.out[3][mine * 9 + k] = scale_out(acc[k], sc2);
    }
  }
  __syncthreads();
  T *dst[4] = {F, Abar, JV, HWV};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (!dst[q]) continue;
    for (int e = tid; e < cnt * 9; e += GADJ_TPB) dst[q][S.gidx[e / 9] * 9 + e % 9] = (T)S.out[q][e];
  }
}

// ------------------------------------------------------------------------------------------------ symmetric
// the tiles and the contractions in the eigenbasis: smf_adjoint_tile.cuh
constexpr int SADJ_TPB = 64;

template <int KIND, int ORDER>
__global__ void __launch_bounds__(SADJ_TPB) smf_adjoint_kernel(int64_t n, const double *__restrict__ A,
                                                               const double *__restrict__ W,
                                                               const double *__restrict__ V, double *__restrict__ F,
                                                               double *__restrict__ Abar, double *__restrict__ JV,
                                                               double *__restrict__ HWV, const SmfCoef C) {
  __shared__ SadjSmem<double, SADJ_TPB> S;
  const int64_t base = (int64_t)blockIdx.x * SADJ_TPB;
  smf_adjoint_tile<KIND, ORDER, SADJ_TPB>(base, (int)min((int64_t)SADJ_TPB, n - base), A, W, V, F, Abar, JV, HWV, C,
                                          S);
}

// mixed precision: FP32 arrays, the eigensystem and divided differences of smf_mixed_math.cuh, FP32 contractions
template <int KIND, int ORDER>
__global__ void __launch_bounds__(SADJ_TPB) smf_adjoint_kernel_f32(int64_t n, const float *__restrict__ A,
                                                                   const float *__restrict__ W,
                                                                   const float *__restrict__ V, float *__restrict__ F,
                                                                   float *__restrict__ Abar, float *__restrict__ JV,
                                                                   float *__restrict__ HWV, const SmfCoefF C) {
  __shared__ SadjSmem<float, SADJ_TPB> S;
  const int64_t base = (int64_t)blockIdx.x * SADJ_TPB;
  smf_adjoint_tile_f32<KIND, ORDER, SADJ_TPB>(base, (int)min((int64_t)SADJ_TPB, n - base), A, W, V, F, Abar, JV,
                                              HWV, C, S);
}

// ------------------------------------------------------------------------------------------------ launchers
template <int KIND, int ORDER, typename T>
cudaError_t gmf_adjoint_one(unsigned blocks, int64_t n, const T *A, const T *W, const T *V, T *F, T *Abar, T *JV,
                            T *HWV, const GmfCoef &C, cudaStream_t st, const int *idx = nullptr) {
  static bool attr = false;  // per instantiation (idempotent)
  if (!attr) {
    const cudaError_t e = cudaFuncSetAttribute(gmf_adjoint_kernel<KIND, ORDER, T>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GadjSmem));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  gmf_adjoint_kernel<KIND, ORDER, T><<<blocks, GADJ_TPB, sizeof(GadjSmem), st>>>(n, A, W, V, F, Abar, JV, HWV, C,
                                                                                  idx);
  return cudaGetLastError();
}

// the batch ordering of gmf_kernels.cuh (log, pow; large batches): the adjoint outputs are too small to hold the
// scratch, so it comes from the stream-ordered allocator (cudaMallocAsync / cudaFreeAsync on the call's stream: no
// synchronisation, capturable, nothing shared between calls); without it the unordered launch runs
template <int KIND, typename T = double>
cudaError_t gmf_adjoint_t(double al, int64_t n, const T *A, const T *W, const T *V, T *F, T *Abar, T *JV, T *HWV,
                          cudaStream_t st) {
  const int order = HWV ? 2 : 1;
  GmfCoef C;
  gmf_coef(KIND, al, order, C);
  const unsigned blocks = (unsigned)((n + GADJ_TPB - 1) / GADJ_TPB);
  int *ord = nullptr;
  if ((KIND != EXP) & (n >= GMF_SORT_MIN) & (n <= INT_MAX)) {
    const int nblk = (int)((n + GKEY_TPB - 1) / GKEY_TPB);
    void *scr = nullptr;
    if (cudaMallocAsync(&scr, (size_t)(4 * n + 4 * (int64_t)GKEY_BINS * (nblk + 1) + n + 16), st) == cudaSuccess) {
      ord = static_cast<int *>(scr);
      int *counts = ord + n, *totals = counts + (int64_t)GKEY_BINS * nblk;
      unsigned char *keys = reinterpret_cast<unsigned char *>(totals + GKEY_BINS);
      gmf_key_kernel<KIND, T><<<nblk, GKEY_TPB, 0, st>>>((int)n, A, keys, counts, nblk, nullptr);
      gmf_scan_kernel<<<GKEY_BINS, 1024, 0, st>>>(counts, nblk, totals);
      gmf_scatter_kernel<<<nblk, GKEY_TPB, 0, st>>>((int)n, keys, counts, totals, nblk, ord);
    } else {
      cudaGetLastError();  // no pool memory: the unordered launch
    }
  }
  const cudaError_t e = order == 2 ? gmf_adjoint_one<KIND, 2, T>(blocks, n, A, W, V, F, Abar, JV, HWV, C, st, ord)
                                   : gmf_adjoint_one<KIND, 1, T>(blocks, n, A, W, V, F, Abar, JV, HWV, C, st, ord);
  if (ord) cudaFreeAsync(ord, st);
  return e;
}

template <int KIND>
cudaError_t smf_adjoint_t(double al, int64_t n, const double *A, const double *W, const double *V, double *F,
                          double *Abar, double *JV, double *HWV, cudaStream_t st) {
  SmfCoef C;
  smf_coef(KIND, al, C);
  const unsigned blocks = (unsigned)((n + SADJ_TPB - 1) / SADJ_TPB);
  if (HWV) smf_adjoint_kernel<KIND, 2><<<blocks, SADJ_TPB, 0, st>>>(n, A, W, V, F, Abar, JV, HWV, C);
  else smf_adjoint_kernel<KIND, 1><<<blocks, SADJ_TPB, 0, st>>>(n, A, W, V, F, Abar, JV, HWV, C);
  return cudaGetLastError();
}

template <int KIND>
cudaError_t smf_adjoint_f32_t(double al, int64_t n, const float *A, const float *W, const float *V, float *F,
                              float *Abar, float *JV, float *HWV, cudaStream_t st) {
  SmfCoefF C;
  smf_coef_f(KIND, al, C);
  const unsigned blocks = (unsigned)((n + SADJ_TPB - 1) / SADJ_TPB);
  if (HWV) smf_adjoint_kernel_f32<KIND, 2><<<blocks, SADJ_TPB, 0, st>>>(n, A, W, V, F, Abar, JV, HWV, C);
  else smf_adjoint_kernel_f32<KIND, 1><<<blocks, SADJ_TPB, 0, st>>>(n, A, W, V, F, Abar, JV, HWV, C);
  return cudaGetLastError();
}

}  // namespace mf
