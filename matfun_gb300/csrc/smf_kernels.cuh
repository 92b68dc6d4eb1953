// smf_kernels.cuh -- symmetric family (smf_cuda_eval / smf_cuda_eval_matrix): F, J, H of f(A) for symmetric 3x3
// matrices, FP64, Voigt or matrix layout.  Replaces smf_eval_kernel / smf_hess_kernel of the reference
// (cuda/src/matfun_cuda.cu:28-96).
//
// One CTA = 64 matrices (two warps) runs the tile of smf_tile.cuh.
// Order-2 batches of 2^17 matrices or more are first ordered by the predicted branch pattern of their second divided
// differences (smf_launch_sorted below).
#pragma once
#include <climits>

#include "batch_order.cuh"
#include "mf_launch.h"
#include "smf_tile.cuh"

namespace mf {

// (order 2: 228 registers and 46 KB of shared memory, 4 CTAs per SM.  A form with the inputs staged inside sG (43 KB,
// 166 registers, 5 CTAs per SM) ran 8 % slower on C0 -- n = 65536 then fills 1.35 waves of CTAs instead of 1.68 --
// and within +-4 % at n = 2^24.)
template <int KIND, int ORDER, bool MAT>
__global__ void __launch_bounds__(SMF_TPB) smf_kernel(int64_t n, const double *__restrict__ x,
                                                      double *__restrict__ F, double *__restrict__ J,
                                                      double *__restrict__ H, const SmfCoef C,
                                                      int *__restrict__ asym, const int *__restrict__ idx) {
  __shared__ SmfTileSmem<ORDER, MAT, SMF_TPB> TS;
  const int64_t base = (int64_t)blockIdx.x * SMF_TPB;
  smf_tile<KIND, ORDER, MAT, SMF_TPB>(base, (int)min((int64_t)SMF_TPB, n - base), x, F, J, H, C, asym, TS, idx);
}

// ---- batch-wide ordering (order 2).  The second divided differences take the cluster series or the difference
// formula per triple of eigenvalues, and a warp whose lanes split pays for both: on the C0 workload 19 of 32 lanes
// were active per FP64 instruction.  The key of a matrix is the pattern of those seven choices, predicted from FP32
// eigenvalues labelled as smf_eigsys labels them (lam[0] the root farthest from the other two, as Smith's formula
// picks it; lam[1] the larger of the remaining pair, as the Jacobi rotation orders it); a wrong prediction only
// costs time, the evaluation recomputes everything in FP64, and no result depends on the order.
template <int KIND, bool MAT>
__global__ void __launch_bounds__(GKEY_TPB) smf_key_kernel(int n, const double *__restrict__ x,
                                                           unsigned char *__restrict__ keys,
                                                           int *__restrict__ counts, int nblk, float tau) {
  __shared__ int hist[GKEY_BINS];
  for (int k = threadIdx.x; k < GKEY_BINS; k += GKEY_TPB) hist[k] = 0;
  __syncthreads();
  const int i = blockIdx.x * GKEY_TPB + threadIdx.x;
  if (i < n) {
    double v[6];
    if (MAT) {
      const double *a = x + (int64_t)i * 9;
      v[0] = a[0]; v[1] = a[4]; v[2] = a[8];
      v[3] = 0.5 * (a[1] + a[3]); v[4] = 0.5 * (a[2] + a[6]); v[5] = 0.5 * (a[5] + a[7]);
    } else {
#pragma unroll
      for (int k = 0; k < 6; k++) v[k] = x[(int64_t)i * 6 + k];
    }
    double mx = 0.0;
#pragma unroll
    for (int k = 0; k < 6; k++) mx = fmax(mx, fabs(v[k]));
    const double sc = (mx > 0.0) & (mx < 1e300) ? mx : 1.0;
    float a[6];
#pragma unroll
    for (int k = 0; k < 6; k++) a[k] = (float)(v[k] / sc);
    const float m = (a[0] + a[1] + a[2]) / 3.f, d0 = a[0] - m, d1 = a[1] - m, d2 = a[2] - m;
    const float p = d0 * d0 + d1 * d1 + d2 * d2 + 2.f * (a[3] * a[3] + a[4] * a[4] + a[5] * a[5]);
    const float q = d0 * (d1 * d2 - a[5] * a[5]) - a[3] * (a[3] * d2 - a[5] * a[4]) + a[4] * (a[3] * a[5] - d1 * a[4]);
    float l0 = m, l1 = m, l2 = m;
    if (p > 1e-30f) {
      const float r = fminf(1.f, fmaxf(-1.f, 7.3484692f * q / (p * sqrtf(p))));  // 3 sqrt(6) q / p^(3/2)
      const float t = sqrtf(2.f * p / 3.f), ph = acosf(r) / 3.f;
      const float x0 = t * cosf(ph), x1 = t * cosf(ph + 2.0943951f), x2 = t * cosf(ph + 4.1887902f);
      const bool rp = r >= 0.f;  // x0 >= x2 >= x1; Smith's root is x0 (r >= 0) or x1
      l0 = m + (rp ? x0 : x1);
      l1 = m + (rp ? x2 : x0);
      l2 = m + (rp ? x1 : x2);
    }
    double lam[3] = {l0 * sc, l1 * sc, l2 * sc};
    if (KIND == POW || KIND == SQRT) {
#pragma unroll
      for (int k = 0; k < 3; k++) lam[k] = lam[k] > 0 ? lam[k] : 0.0;
    }
    // the seven triples of smf_tile's loop order: 001 002 011 012 022 112 122
    constexpr int TI[7] = {0, 0, 0, 0, 0, 1, 1}, TJ[7] = {0, 0, 1, 1, 2, 1, 2}, TL[7] = {1, 2, 1, 2, 2, 2, 2};
    unsigned key = 0;
#pragma unroll
    for (int t7 = 0; t7 < 7; t7++) {
      const double li = lam[TI[t7]], lj = lam[TJ[t7]], lk = lam[TL[t7]];
      const double lo = fmin(li, fmin(lj, lk)), hi = fmax(li, fmax(lj, lk)), mid = li + lj + lk - lo - hi;
      const bool cl = KIND == EXP ? (mid - lo <= (double)tau) & (hi - mid <= (double)tau)
                                  : (mid > 0) & (mid - lo <= (double)tau * mid) & (hi - mid <= (double)tau * mid);
      key |= cl ? 1u << t7 : 0u;
    }
    keys[i] = (unsigned char)key;
    atomicAdd(&hist[key], 1);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < GKEY_BINS; k += GKEY_TPB) counts[k * nblk + blockIdx.x] = hist[k];
}

// below this the fixed cost of the ordering (three small launches and the tail launch, about one CTA's run time)
// outweighs its gain (C0, log order 2: 65536 matrices 0.50 -> 0.56 ms ordered; 2^17 0.93 -> 0.87 ms; 2^20 7.1 ->
// 5.3 ms)
constexpr int64_t SMF_SORT_MIN = 1 << 17;

// order 2 of a large batch: key, sort, ordered evaluation of the first nm matrices, plain evaluation of the last
// n - nm, whose rows of H held the scratch (order, block counts, totals, keys: ~9 B per matrix, 0.5 % of H's rows)
template <int KIND, bool MAT>
cudaError_t smf_launch_sorted(cudaStream_t st, int64_t n, const double *x, double *F, double *J, double *H,
                              const SmfCoef &C, int *asym) {
  constexpr int64_t NIN = MAT ? 9 : 6, NF = NIN, NJ = NF * NF, NH = NJ * NF;
  const int64_t nblk_n = (n + GKEY_TPB - 1) / GKEY_TPB;
  const int64_t need = 4 * n + 4 * (int64_t)GKEY_BINS * (nblk_n + 1) + n + 64;
  const int64_t tail = (need + NH * 8 - 1) / (NH * 8) + 1;
  const int64_t nm = n - tail;
  const int nblk = (int)((nm + GKEY_TPB - 1) / GKEY_TPB);
  int *order = reinterpret_cast<int *>(H + nm * NH);
  int *counts = order + nm, *totals = counts + (int64_t)GKEY_BINS * nblk;
  unsigned char *keys = reinterpret_cast<unsigned char *>(totals + GKEY_BINS);
  smf_key_kernel<KIND, MAT><<<nblk, GKEY_TPB, 0, st>>>((int)nm, x, keys, counts, nblk, (float)C.tau);
  gmf_scan_kernel<<<GKEY_BINS, 1024, 0, st>>>(counts, nblk, totals);
  gmf_scatter_kernel<<<nblk, GKEY_TPB, 0, st>>>((int)nm, keys, counts, totals, nblk, order);
  smf_kernel<KIND, 2, MAT><<<(unsigned)((nm + SMF_TPB - 1) / SMF_TPB), SMF_TPB, 0, st>>>(nm, x, F, J, H, C, asym,
                                                                                         order);
  // the tail overwrites the scratch only: launched with programmatic stream serialisation, it may start as soon as
  // every CTA of the ordered launch has read its part of the order (griddep_launch_dependents in smf_tile)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)((tail + SMF_TPB - 1) / SMF_TPB));
  cfg.blockDim = dim3(SMF_TPB);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, smf_kernel<KIND, 2, MAT>, (int64_t)tail, x + nm * NIN, F + nm * NF,
                                           J + nm * NJ, H + nm * NH, C, asym, (const int *)nullptr);
  return e != cudaSuccess ? e : cudaGetLastError();
}

template <int KIND, bool MAT>
cudaError_t smf_launch_kind(int order, cudaStream_t st, unsigned blocks, int64_t n, const double *x,
                                   double *F, double *J, double *H, const SmfCoef &C, int *asym, bool reorder) {
  if ((order == 2) & reorder & (n >= SMF_SORT_MIN) & (n <= INT_MAX))
    return smf_launch_sorted<KIND, MAT>(st, n, x, F, J, H, C, asym);
  if (order == 2) smf_kernel<KIND, 2, MAT><<<blocks, SMF_TPB, 0, st>>>(n, x, F, J, H, C, asym, nullptr);
  else if (order == 1) smf_kernel<KIND, 1, MAT><<<blocks, SMF_TPB, 0, st>>>(n, x, F, J, H, C, asym, nullptr);
  else smf_kernel<KIND, 0, MAT><<<blocks, SMF_TPB, 0, st>>>(n, x, F, J, H, C, asym, nullptr);
  return cudaGetLastError();
}

// one kind (instantiated in smf_<kind>.cu so that the kinds compile in parallel)
template <int KIND>
cudaError_t smf_launch_t(double al, int64_t n, const double *x, bool mat, double *F, double *J, double *H,
                         cudaStream_t st, int *asym, bool reorder = true) {
  SmfCoef C;
  smf_coef(KIND, al, C);
  const int order = H ? 2 : (J ? 1 : 0);
  const unsigned blocks = (unsigned)((n + SMF_TPB - 1) / SMF_TPB);
  return mat ? smf_launch_kind<KIND, true>(order, st, blocks, n, x, F, J, H, C, asym, reorder)
             : smf_launch_kind<KIND, false>(order, st, blocks, n, x, F, J, H, C, nullptr, reorder);
}

}  // namespace mf
