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
#include "gmf_adjoint_tile.cuh"
#include "smf_adjoint_tile.cuh"

namespace mf {

enum { ADJ_F = 1, ADJ_VJP = 2, ADJ_JVP = 4, ADJ_HVP = 8 };

// ------------------------------------------------------------------------------------------------ general
constexpr int GADJ_TPB = 128;

using GadjSmem = GadjSmemT<GADJ_TPB>;

template <int KIND, int ORDER, typename T>
__global__ void __launch_bounds__(GADJ_TPB) gmf_adjoint_kernel(int64_t n, const T *__restrict__ A,
                                                               const T *__restrict__ W, const T *__restrict__ V,
                                                               T *__restrict__ F, T *__restrict__ Abar,
                                                               T *__restrict__ JV, T *__restrict__ HWV,
                                                               const GmfCoef C, const int *__restrict__ idx) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GadjSmem &S = *reinterpret_cast<GadjSmem *>(smem_raw);
  const int64_t base = (int64_t)blockIdx.x * GADJ_TPB;
  gmf_adjoint_tile<KIND, ORDER, T, GADJ_TPB>(base, (int)min((int64_t)GADJ_TPB, n - base), A, W, V, F, Abar, JV, HWV,
                                             C, idx, S);
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
  static std::atomic<unsigned long long> attr{0};  // per instantiation, one bit per device
  const cudaError_t e = smem_limit_per_device(gmf_adjoint_kernel<KIND, ORDER, T>, (int)sizeof(GadjSmem), attr);
  if (e != cudaSuccess) return e;
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
  gmf_coef(KIND, al, order, C, sizeof(T) == 4);
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
