// gmf_kernels.cu -- general family (gmf_cuda_eval): F, J, H of f(A) for general real 3x3 matrices, FP64, matrix
// layout.  Replaces gmf_eval_kernel of the reference (cuda/src/matfun_cuda.cu:144-190).
//
// One CTA = 64 matrices.  Phase A: one thread per matrix computes the record of gmf_device.cuh (F, the real basis
// r_1, r_2 and the symmetric reduced divided differences D2', D3').  Phase B contracts them per thread into
//   T4[P1, P2]     = sum_mn  D2'_mn  r_m[P1] r_n[P2]            (symmetric: 45 distinct of 81)
//   T6[P1, P2, P3] = sum_mnp D3'_mnp r_m[P1] r_n[P2] r_p[P3]    (symmetric: 165 distinct of 729)
// (P = 3a + c a matrix entry, r_0 = I) into shared memory, and the CTA writes
//   J_abcd   = sc1 T4[ac, db]
//   H_abcdef = sc2 (T6[ac, de, fb] + T6[ae, fc, db])
// with fully coalesced stores.  The reference forms Y (27), Z (81) and Yh (243) per matrix and evaluates all 729 H
// entries with 6 multiply-adds each from every thread (gmf_kernel.hpp:636-691); the symmetric form needs about a
// third of the FP64 instructions, which on GB300 (FP64 at 1/74 of the FP32 rate) is what bounds this kernel.
#pragma once
#include "gmf_device.cuh"
#include "mf_launch.h"

namespace mf {

constexpr int GMF_TPB = 64;

// r_m[P] with r_0 = I (known per P at compile time after unrolling)
#define MF_R0(P) ((P) % 4 == 0 ? 1.0 : 0.0)

template <int KIND, int ORDER>
__global__ void __launch_bounds__(GMF_TPB) gmf_kernel(int64_t n, const double *__restrict__ A, double *__restrict__ F,
                                                      double *__restrict__ J, double *__restrict__ H,
                                                      const GmfCoef C) {
  extern __shared__ double smem[];
  double *sX = smem;                        // 64 x 9: input, then F
  double *sS = smem + GMF_TPB * 9;          // 64 x 2: output scale of J / H (1 when folded into T4 / T6)
  double *sT = smem + GMF_TPB * 11;         // 64 x 45 (T4) or 64 x 165 (T6)
  const int tid = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * GMF_TPB;
  const int cnt = (int)min((int64_t)GMF_TPB, n - base);

  for (int e = tid; e < cnt * 9; e += GMF_TPB) sX[e] = A[base * 9 + e];
  __syncthreads();
  GmfRec R;
  const bool active = tid < cnt;
  if (active) {
    double a[9];
#pragma unroll
    for (int k = 0; k < 9; k++) a[k] = sX[tid * 9 + k];
    gmf_record<KIND, ORDER>(a, C, R);
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int k = 0; k < 9; k++) sX[tid * 9 + k] = R.F[k];
  }
  __syncthreads();
  for (int e = tid; e < cnt * 9; e += GMF_TPB) F[base * 9 + e] = sX[e];
  if (ORDER < 1) return;

  // ---- J: T4 per thread, then the coalesced gather
  if (active) {
    const bool fold = isfinite(R.sc1) & (R.sc1 != 0.0);
    const double s = sel(fold, R.sc1, 1.0);
    sS[tid * 2] = sel(fold, 1.0, R.sc1);
    const double D00 = R.D2[0] * s, D11 = R.D2[1] * s, D22 = R.D2[2] * s, D01 = R.D2[3] * s, D02 = R.D2[4] * s,
                 D12 = R.D2[5] * s;
    double *t4 = sT + tid * 45;
#pragma unroll
    for (int y = 0; y < 9; y++) {
      // Y2[m] = sum_n D2'_mn r_n[y]
      const double y0 = (y % 4 == 0 ? D00 : 0.0) + D01 * R.r1[y] + D02 * R.r2[y];
      const double y1 = (y % 4 == 0 ? D01 : 0.0) + D11 * R.r1[y] + D12 * R.r2[y];
      const double y2 = (y % 4 == 0 ? D02 : 0.0) + D12 * R.r1[y] + D22 * R.r2[y];
#pragma unroll
      for (int xx = 0; xx <= y; xx++) t4[sym2(xx, y)] = (xx % 4 == 0 ? y0 : 0.0) + R.r1[xx] * y1 + R.r2[xx] * y2;
    }
  }
  __syncthreads();
  {
    constexpr int KJ = (81 + GMF_TPB - 1) / GMF_TPB;
    int jidx[KJ];
#pragma unroll
    for (int k = 0; k < KJ; k++) {
      const int w = min(tid + GMF_TPB * k, 80);
      const int a = w / 27, b = (w / 9) % 3, c = (w / 3) % 3, d = w % 3;
      const int p1 = 3 * a + c, p2 = 3 * d + b;
      jidx[k] = sym2(min(p1, p2), max(p1, p2));
    }
    for (int mi = 0; mi < cnt; mi++) {
      double *o = J + (base + mi) * 81;
      const double *t = sT + mi * 45;
      const double sc = sS[mi * 2];
      const bool plain = sc == 1.0;
#pragma unroll
      for (int k = 0; k < KJ; k++) {
        if (tid + GMF_TPB * k < 81) {
          const double v = t[jidx[k]];
          o[tid + GMF_TPB * k] = plain ? v : v * sc;
        }
      }
    }
  }
  if (ORDER < 2) return;
  __syncthreads();

  // ---- H: T6 per thread, then the coalesced gather
  if (active) {
    const bool fold = isfinite(R.sc2) & (R.sc2 != 0.0);
    const double s = sel(fold, R.sc2, 1.0);
    sS[tid * 2 + 1] = sel(fold, 1.0, R.sc2);
    double d3[10];
#pragma unroll
    for (int k = 0; k < 10; k++) d3[k] = R.D3[k] * s;
    double *t6 = sT + tid * 165;
#pragma unroll
    for (int z = 0; z < 9; z++) {
      // Zz[m][n] = sum_p D3'_mnp r_p[z]   (m <= n)
      double Zz[3][3];
      // sorted index of the triple (m, n, p) for p = 0, 1, 2 (m <= n)
#pragma unroll
      for (int mm = 0; mm < 3; mm++)
#pragma unroll
        for (int nn = mm; nn < 3; nn++) {
          const int i0 = sym3(0, mm, nn);
          const int i1 = nn <= 1 ? sym3(mm, nn, 1) : (mm <= 1 ? sym3(mm, 1, nn) : sym3(1, mm, nn));
          const int i2 = sym3(mm, nn, 2);
          Zz[mm][nn] = (z % 4 == 0 ? d3[i0] : 0.0) + d3[i1] * R.r1[z] + d3[i2] * R.r2[z];
          Zz[nn][mm] = Zz[mm][nn];
        }
#pragma unroll
      for (int y = 0; y <= z; y++) {
        const double Y0 = (y % 4 == 0 ? Zz[0][0] : 0.0) + Zz[0][1] * R.r1[y] + Zz[0][2] * R.r2[y];
        const double Y1 = (y % 4 == 0 ? Zz[1][0] : 0.0) + Zz[1][1] * R.r1[y] + Zz[1][2] * R.r2[y];
        const double Y2 = (y % 4 == 0 ? Zz[2][0] : 0.0) + Zz[2][1] * R.r1[y] + Zz[2][2] * R.r2[y];
#pragma unroll
        for (int xx = 0; xx <= y; xx++)
          t6[sym3(xx, y, z)] = (xx % 4 == 0 ? Y0 : 0.0) + R.r1[xx] * Y1 + R.r2[xx] * Y2;
      }
    }
  }
  __syncthreads();
  {
    constexpr int KH = (729 + GMF_TPB - 1) / GMF_TPB;
    int h1[KH], h2[KH];
#pragma unroll
    for (int k = 0; k < KH; k++) {
      const int w = min(tid + GMF_TPB * k, 728);
      const int a = w / 243, b = (w / 81) % 3, c = (w / 27) % 3, d = (w / 9) % 3, e = (w / 3) % 3, f = w % 3;
      int x1 = 3 * a + c, y1 = 3 * d + e, z1 = 3 * f + b;
      int x2 = 3 * a + e, y2 = 3 * f + c, z2 = 3 * d + b;
      sort3(x1, y1, z1);
      sort3(x2, y2, z2);
      h1[k] = sym3(x1, y1, z1);
      h2[k] = sym3(x2, y2, z2);
    }
    for (int mi = 0; mi < cnt; mi++) {
      double *o = H + (base + mi) * 729;
      const double *t = sT + mi * 165;
      const double sc = sS[mi * 2 + 1];
      const bool plain = sc == 1.0;
#pragma unroll
      for (int k = 0; k < KH; k++) {
        if (tid + GMF_TPB * k < 729) {
          const double v = t[h1[k]] + t[h2[k]];
          o[tid + GMF_TPB * k] = plain ? v : v * sc;
        }
      }
    }
  }
}
#undef MF_R0

inline size_t gmf_smem(int order) {
  return sizeof(double) * GMF_TPB * (11 + (order == 2 ? 165 : (order == 1 ? 45 : 0)));
}

template <int KIND, int ORDER>
cudaError_t gmf_launch_one(cudaStream_t st, unsigned blocks, int64_t n, const double *A, double *F, double *J,
                                  double *H, const GmfCoef &C) {
  static bool attr_done = false;  // per instantiation; setting the attribute twice is harmless
  const size_t smem = gmf_smem(ORDER);
  if (!attr_done) {
    const cudaError_t e = cudaFuncSetAttribute(gmf_kernel<KIND, ORDER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
    if (e != cudaSuccess) return e;
    attr_done = true;
  }
  gmf_kernel<KIND, ORDER><<<blocks, GMF_TPB, smem, st>>>(n, A, F, J, H, C);
  return cudaGetLastError();
}

template <int KIND>
cudaError_t gmf_launch_kind(int order, cudaStream_t st, unsigned blocks, int64_t n, const double *A, double *F,
                                   double *J, double *H, const GmfCoef &C) {
  if (order == 2) return gmf_launch_one<KIND, 2>(st, blocks, n, A, F, J, H, C);
  if (order == 1) return gmf_launch_one<KIND, 1>(st, blocks, n, A, F, J, H, C);
  return gmf_launch_one<KIND, 0>(st, blocks, n, A, F, J, H, C);
}

// host: launch constants (gmf_kernel.hpp:48-53 series coefficients, :84 binomial recurrence)
inline void gmf_coef(int kind, double al, int order, GmfCoef &C) {
  C.al = al;
  C.rho_f = (kind == POW && 3.0 / al < G_RHO) ? 3.0 / al : G_RHO;
  for (int k = 0; k < 3; k++) {
    const double bh = al - k, bb = bh - al;
    C.bh[k] = bh;
    C.bl[k] = (al - (bh - bb)) + (-k - bb);
  }
  C.bt[0] = 1.0;
  for (int j = 1; j < G_KMAX; j++)
    C.bt[j] = kind == EXP ? C.bt[j - 1] / j : (kind == LOG ? (j % 2 ? 1.0 : -1.0) / j : C.bt[j - 1] * (al - j + 1) / j);
  const int nn = 3 * (order + 1) - 1;
  double c = 1.0;
  for (int k = 0; k < G_KMAX; k++) {
    C.bin[k] = c;
    c = c * (k + nn + 1) / (k + 1);
  }
}

// one kind (instantiated in gmf_<kind>.cu so that the kinds compile in parallel)
template <int KIND>
cudaError_t gmf_launch_t(double al, int64_t n, const double *A, double *F, double *J, double *H, cudaStream_t st) {
  const int order = H ? 2 : (J ? 1 : 0);
  GmfCoef C;
  gmf_coef(KIND, al, order, C);
  const unsigned blocks = (unsigned)((n + GMF_TPB - 1) / GMF_TPB);
  return gmf_launch_kind<KIND>(order, st, blocks, n, A, F, J, H, C);
}

}  // namespace mf
