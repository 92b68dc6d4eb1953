// gmf_kernels.cuh -- general family (gmf_cuda_eval): F, J, H of f(A) for general real 3x3 matrices, FP64, matrix
// layout.  Replaces gmf_eval_kernel of the reference (cuda/src/matfun_cuda.cu:144-190).  The same tile with float
// storage is the mixed-precision form (gmf_cuda_eval_f32): phase A in FP64, phase B and the arrays in FP32.
//
// One CTA = 128 matrices (four warps).
// Phase A: one thread per matrix computes the record of gmf_device.cuh -- F, the real basis r_1, r_2 (r_0 = I) and
//   the symmetric reduced divided differences D2' (6), D3' (10) -- into shared memory (36 doubles per matrix), in three
//   parts with a CTA-local ordering of the matrices before the second and the third, so that a warp's lanes take the
//   same branches: the closed-form roots (gmf_roots), ordered by the branches of the spectral analysis that follow
//   (complex pair, pair refinement, branch-cut pair); the rest of the spectral analysis (gmf_classify_from), ordered
//   by class (no group / real series / complex series) and series length; then gmf_finish.  Unordered, about half
//   of the lanes idled.
// Phase B: each warp walks the 32 matrices it finished; for one matrix the 32 lanes build, through shared memory,
//   Y2[y][m]      = sum_n D2'_mn r_n[y]                       (27)
//   T4[x, y]      = sum_m r_m[x] Y2[y][m]                      (symmetric: 45 distinct of 81)
//   Z[z][m, n]    = sum_p D3'_mnp r_p[z]                       (54)
//   Y[y, z][m]    = sum_n Z[z][m, n] r_n[y]                    (135)
//   T6[x, y, z]   = sum_m r_m[x] Y[y, z][m]                    (symmetric: 165 distinct of 729)
// (x, y, z = 3a + c index matrix entries) and writes, 32 consecutive doubles per store,
//   J_abcd   = sc1 T4[ac, db]
//   H_abcdef = sc2 (T6[ac, de, fb] + T6[ae, fc, db])   (405 distinct sums: H is symmetric under (cd) <-> (ef)).
// The reference forms Y (27), Z (81) and Yh (243) per matrix and evaluates each of the 729 H entries with 6
// multiply-adds in every thread (gmf_kernel.hpp:636-691); the symmetric form needs about a third of the FP64
// instructions, which bound this kernel on GB300 (FP64 at 1/74 of the FP32 rate).  Spreading one matrix over the
// warp keeps phase B's work area at 4.5 KB per warp; the CTA's ~106 KB of shared memory (states and records of its
// 128 matrices) and phase A's 255 registers per thread both allow two CTAs per SM.
// Large batches (log, pow at orders 1 and 2, exp at order 2, n >= 2^15) are first ordered batch-wide by spectral
// class (gmf_launch_sorted below), so that a CTA's matrices share their branches before the CTA-local orderings.
#pragma once
#include <climits>

#include "batch_order.cuh"
#include "gmf_device.cuh"
#include "mf_launch.h"

namespace mf {

constexpr int GMF_TPB = 128;
constexpr int GMF_WARPS = GMF_TPB / 32;
constexpr int GMF_MIN_CTAS = 3;  // CTAs per SM the register allocation of gmf_kernel is bounded for (3: 168 registers,
                                 // C1 gmf log order 2 12.3 ms against 13.3 ms at 2 CTAs with 255 registers)
constexpr int GMF_REC = 36;  // r1 (9), r2 (9), D2' (6), D3' (10), sc1, sc2

// shared memory layout of one CTA (doubles unless noted)
struct GmfSmem {
  double x[GMF_TPB * 9];          // input, then F
  GmfState state[GMF_TPB];        // the first half's results by matrix, then the matrix's record (GMF_REC doubles)
  unsigned key[GMF_TPB];          // sort key of each matrix
  int perm[GMF_TPB];              // processing slot -> matrix
  double work[GMF_WARPS][165 + 405];  // per warp: T6, then Z and Y, then the 405 distinct H values over Z and Y
                                      // (J: Y2 at 0, T4 at 54)
  unsigned short umap[405];       // distinct H value -> (T6 index of the first term) | (second) << 8
  unsigned short hkey[729];       // H entry -> its distinct value (H is symmetric under (cd) <-> (ef))
  long long gidx[GMF_TPB];        // tile position -> matrix index in the arrays
  unsigned short t6map[165];      // T6 item -> x | y << 4 | z << 8
  unsigned short ymap[135];       // Y item  -> y | z << 4 | m << 8
};

// a T6 index pair of an H entry w = 243 a + 81 b + 27 c + 9 d + 3 e + f
MF_D unsigned short hmap_entry(int w) {
  const int a = w / 243, b = (w / 81) % 3, c = (w / 27) % 3, d = (w / 9) % 3, e = (w / 3) % 3, f = w % 3;
  int x1 = 3 * a + c, y1 = 3 * d + e, z1 = 3 * f + b;
  int x2 = 3 * a + e, y2 = 3 * f + c, z2 = 3 * d + b;
  sort3(x1, y1, z1);
  sort3(x2, y2, z2);
  return (unsigned short)(sym3(x1, y1, z1) | (sym3(x2, y2, z2) << 8));
}

// the tangent of psi(A) = |f(A)|^2 / 2 for one matrix, by the 32 lanes of a warp from its record rc (r1, r2, D2', D3'
// and the factors sc1, sc2 left to apply) and F = f(A): the gradient G = J^T F (9) and the tangent K = J^T J + F : H
// (81, symmetric), with J and H never formed.  With L_m = sum_n D2'_mn r_n (the Y2 of the J assembly),
// J_{ab,cd} = sc1 sum_m (r_m)_ac (L_m)_db and H as in the J / H assembly:
//   G_cd       = sc1 sum_m (r_m^T F L_m^T)_cd
//   (J^T J)_{cd,ef} = sc1^2 sum_mk (r_m^T r_k)_ce (L_m L_k^T)_df
//   (F : H)_{cd,ef} = sc2 sum_q ((r_q)_de N_q,cf + (r_q)_fc N_q,ed),  N_q = sum_mp D3'_mqp r_m^T F r_p^T
// wk: 351 doubles of the warp's work area; G, K: this matrix's rows of the outputs (G may be null)
MF_D double gmf_rm(const double *r1, const double *r2, int m, int x) {
  return m == 0 ? (x % 4 == 0 ? 1.0 : 0.0) : (m == 1 ? r1[x] : r2[x]);
}

MF_D void gmf_tangent_warp(const double *rc, const double *Fm, double *wk, int lane, double *G, double *K) {
  const double *r1 = rc, *r2 = rc + 9, *d3 = rc + 24;
  const double sc1 = rc[34], sc2 = rc[35];
  double *L = wk, *P = wk + 27, *Q = P + 81, *FR = Q + 81, *M = FR + 27, *N = M + 81, *FL = N + 27;
  if (lane < 27) {  // L_m[y] at 3 y + m; FR_p[af] = (F r_p^T)_af
    const int y = lane / 3, m = lane % 3;
    const int i0 = m == 0 ? 0 : (m == 1 ? 3 : 4), i1 = m == 0 ? 3 : (m == 1 ? 1 : 5), i2 = m == 0 ? 4 : (m == 1 ? 5 : 2);
    L[lane] = (y % 4 == 0 ? rc[18 + i0] : 0.0) + rc[18 + i1] * r1[y] + rc[18 + i2] * r2[y];
    const int p = lane / 9, a = (lane % 9) / 3, f = lane % 3;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) s += Fm[3 * a + k] * gmf_rm(r1, r2, p, 3 * f + k);
    FR[lane] = s;
  }
  __syncwarp();
  for (int t = lane; t < 81; t += 32) {  // P, Q, M by (m k | m p) * 9 + (c e | d f | c f)
    const int m = t / 27, k = (t / 9) % 3, u = (t % 9) / 3, v = t % 3;
    double sp = 0.0, sq = 0.0, sm = 0.0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const double rma = gmf_rm(r1, r2, m, 3 * a + u);
      sp += rma * gmf_rm(r1, r2, k, 3 * a + v);
      sq += L[3 * (3 * u + a) + m] * L[3 * (3 * v + a) + k];
      sm += rma * FR[9 * k + 3 * a + v];
    }
    P[t] = sp;
    Q[t] = sq;
    M[t] = sm;
  }
  if (lane < 27) {  // FL_m[ad] = (F L_m^T)_ad
    const int m = lane / 9, a = (lane % 9) / 3, d = lane % 3;
    double s = 0.0;
#pragma unroll
    for (int b = 0; b < 3; b++) s += Fm[3 * a + b] * L[3 * (3 * d + b) + m];
    FL[lane] = s;
  }
  __syncwarp();
  if (lane < 27) {  // N_q[cf] = sum_mp D3'_mqp M_mp[cf]
    const int q = lane / 9, cf = lane % 9;
    double s = 0.0;
#pragma unroll
    for (int m = 0; m < 3; m++)
#pragma unroll
      for (int p = 0; p < 3; p++) {
        int i0 = m, i1 = q, i2 = p;
        sort3(i0, i1, i2);
        s += d3[sym3(i0, i1, i2)] * M[9 * (3 * m + p) + cf];
      }
    N[lane] = s;
  }
  __syncwarp();
  for (int t = lane; t < 45; t += 32) {  // K[9 x + y] = K[9 y + x], x = 3c + d <= y = 3e + f (K is symmetric)
    int y = 0;
    while (sym2(0, y + 1) <= t) y++;
    const int x = t - sym2(0, y);
    const int c = x / 3, d = x % 3, e = y / 3, f = y % 3;
    double k1 = 0.0, k2 = 0.0;
#pragma unroll
    for (int mk = 0; mk < 9; mk++) k1 += P[9 * mk + 3 * c + e] * Q[9 * mk + 3 * d + f];
#pragma unroll
    for (int q = 0; q < 3; q++)
      k2 += gmf_rm(r1, r2, q, 3 * d + e) * N[9 * q + 3 * c + f] + gmf_rm(r1, r2, q, 3 * f + c) * N[9 * q + 3 * e + d];
    const double v = (sc1 == 1.0 ? k1 : sc1 * sc1 * k1) + (sc2 == 1.0 ? k2 : sc2 * k2);
    K[9 * x + y] = v;
    K[9 * y + x] = v;
  }
  if (G && lane < 9) {
    const int c = lane / 3, d = lane % 3;
    double s = 0.0;
#pragma unroll
    for (int m = 0; m < 3; m++)
#pragma unroll
      for (int a = 0; a < 3; a++) s += gmf_rm(r1, r2, m, 3 * a + c) * FL[9 * m + 3 * a + d];
    G[lane] = sc1 == 1.0 ? s : sc1 * s;
  }
  __syncwarp();
}

// ---- phase B for one matrix by the 32 lanes of a warp, in the compute type TC (double: the FP64 path, and the
// FP32 path's recomputation of a matrix whose contraction cancels; float: the FP32 path).  rc: the record (r1, r2,
// D2', D3', then the factors sc1, sc2 left to apply); wk: the warp's work area.

// J: Y2[y][m] = sum_n D2'_mn r_n[y] (27, at wk[0]), then T4[x, y] = sum_m r_m[x] Y2[y][m], x <= y (45, at wk[54])
template <typename TC>
MF_D void gmfb_t4(const TC *rc, TC *wk, int lane) {
  const TC *r1 = rc, *r2 = rc + 9;
  if (lane < 27) {
    const int y = lane / 3, m = lane % 3;
    const int i0 = m == 0 ? 0 : (m == 1 ? 3 : 4), i1 = m == 0 ? 3 : (m == 1 ? 1 : 5), i2 = m == 0 ? 4 : (m == 1 ? 5 : 2);
    const TC d0 = rc[18 + i0], d1 = rc[18 + i1], d2 = rc[18 + i2];
    wk[lane] = (y % 4 == 0 ? d0 : TC(0)) + d1 * r1[y] + d2 * r2[y];
  }
  __syncwarp();
  for (int t = lane; t < 45; t += 32) {
    int y = 0;
    while (sym2(0, y + 1) <= t) y++;
    const int x = t - sym2(0, y);
    const TC *yv = wk + 3 * y;
    wk[54 + t] = (x % 4 == 0 ? yv[0] : TC(0)) + r1[x] * yv[1] + r2[x] * yv[2];
  }
  __syncwarp();
}

MF_D float warp_max_abs(float v) {  // max |v| over the warp (non-negative floats order as their bit patterns; NaN wins)
  return __uint_as_float(__reduce_max_sync(0xFFFFFFFFu, __float_as_uint(fabsf(v))));
}

// J_abcd = sc1 T4[ac, db] (81 entries, consecutive lanes on consecutive entries); MAX: returns the largest |T4| of
// the matrix (the same in every lane)
template <typename TC, typename T, bool MAX = false>
MF_D float gmfb_store_j(const TC *wk, TC sc1, T *o, int lane) {
  const bool one1 = sc1 == TC(1);  // folded (the common case): no multiply per entry; uniform in the warp
  float mx = 0.f;
  for (int w = lane; w < 81; w += 32) {
    const int a = w / 27, b = (w / 9) % 3, c = (w / 3) % 3, d = w % 3;
    const int p1 = 3 * a + c, p2 = 3 * d + b;
    const TC v = wk[54 + sym2(min(p1, p2), max(p1, p2))];
    o[w] = (T)(one1 ? v : v * sc1);
    if (MAX) mx = fmaxf(mx, fabsf((float)v));
  }
  __syncwarp();
  return MAX ? warp_max_abs(mx) : 0.f;
}

// H: Z[z][mn] = sum_p D3'_mnp r_p[z] (54), Y[y, z][m] = sum_n Z[z][m, n] r_n[y] (135), T6[x, y, z] =
// sum_m r_m[x] Y[y, z][m] (165, at wk[0]), then the 405 distinct H values T6 + T6 (at wk[165], over Z and Y)
template <typename TC>
MF_D void gmfb_u(const TC *rc, TC *wk, const GmfSmem &S, int lane) {
  const TC *r1 = rc, *r2 = rc + 9, *d3 = rc + 24;
  TC *T6 = wk, *Zs = wk + 165, *Ys = wk + 165 + 54, *U = wk + 165;
  for (int t = lane; t < 54; t += 32) {  // (mn: 00 01 02 11 12 22)
    const int z = t / 6, mn = t % 6;
    const int mm = mn < 3 ? 0 : (mn < 5 ? 1 : 2), nn = mn < 3 ? mn : (mn < 5 ? mn - 2 : 2);
    const int i0 = sym3(0, mm, nn);
    const int i1 = nn <= 1 ? sym3(mm, nn, 1) : (mm <= 1 ? sym3(mm, 1, nn) : sym3(1, mm, nn));
    const int i2 = sym3(mm, nn, 2);
    Zs[t] = (z % 4 == 0 ? d3[i0] : TC(0)) + d3[i1] * r1[z] + d3[i2] * r2[z];
  }
  __syncwarp();
  for (int t = lane; t < 135; t += 32) {
    const unsigned short e = S.ymap[t];
    const int y = e & 15, z = (e >> 4) & 15, m = e >> 8;
    const TC *zz = Zs + 6 * z;
    const int k0 = m == 0 ? 0 : (m == 1 ? 1 : 2), k1 = m == 0 ? 1 : (m == 1 ? 3 : 4), k2 = m == 0 ? 2 : (m == 1 ? 4 : 5);
    Ys[t] = (y % 4 == 0 ? zz[k0] : TC(0)) + zz[k1] * r1[y] + zz[k2] * r2[y];
  }
  __syncwarp();
  for (int t = lane; t < 165; t += 32) {
    const unsigned short e = S.t6map[t];
    const int x = e & 15, y = (e >> 4) & 15, z = e >> 8;
    const TC *yv = Ys + 3 * sym2(y, z);
    T6[t] = (x % 4 == 0 ? yv[0] : TC(0)) + r1[x] * yv[1] + r2[x] * yv[2];
  }
  __syncwarp();
  for (int t = lane; t < 405; t += 32) {
    const unsigned short e = S.umap[t];
    U[t] = T6[e & 255] + T6[e >> 8];
  }
  __syncwarp();
}

// H_abcdef = sc2 U[hkey] (729 entries, consecutive lanes on consecutive entries); MAX: returns the largest |U| of the
// matrix (the same in every lane)
template <typename TC, typename T, bool MAX = false>
MF_D float gmfb_store_h(const TC *wk, TC sc2, const GmfSmem &S, T *o, int lane) {
  const TC *U = wk + 165;
  float mx = 0.f;
  if (sc2 == TC(1)) {
    for (int w = lane; w < 729; w += 32) {
      const TC v = U[S.hkey[w]];
      o[w] = (T)v;
      if (MAX) mx = fmaxf(mx, fabsf((float)v));
    }
  } else {
    for (int w = lane; w < 729; w += 32) {
      const TC v = U[S.hkey[w]];
      o[w] = (T)(v * sc2);
      if (MAX) mx = fmaxf(mx, fabsf((float)v));
    }
  }
  __syncwarp();
  return MAX ? warp_max_abs(mx) : 0.f;
}

// The FP32 path rounds the record to FP32 and contracts it in FP32.  Where the terms of the contraction cancel
// (near-defective matrices: large divided differences against nearly dependent r_0 = I, r_1, r_2), that rounding is
// amplified by the ratio of the terms' bound to the result, and the matrix is recomputed from the FP64 record.  The
// bound of the J entries is B_J = sum_mn |D2'_mn| rho_m rho_n, of the H entries 2 sum_mnp |D3'_mnp| rho_m rho_n rho_p
// (rho_0 = 1, rho_m = max |r_m|); a matrix whose bound exceeds GMF_F32_AMP times the largest |entry| of its FP32
// result is recomputed and its J (H) stored again (about 0.5 % (J) and 6 % (H) of random general matrices, under
// 1 % of the benchmark's).
constexpr float GMF_F32_AMP = 8.f;
// the FP32 record in a warp's work area (float offset, past the 570 floats of the FP32 phase B)
constexpr int GMF_RECF = 1100;
static_assert(GMF_RECF + GMF_REC <= 2 * (165 + 405), "the FP32 record fits the warp's work area");

// the bounds B_J, B_H of a record rounded to FP32
MF_D void gmfb_bounds(const float *rc, float &bj, float &bh) {
  float p1 = 0.f, p2 = 0.f;
#pragma unroll
  for (int k = 0; k < 9; k++) { p1 = fmaxf(p1, fabsf(rc[k])); p2 = fmaxf(p2, fabsf(rc[9 + k])); }
  const float *d2 = rc + 18, *d3 = rc + 24;
  bj = fabsf(d2[0]) + p1 * (fabsf(d2[1]) * p1 + 2.f * fabsf(d2[3])) + p2 * (fabsf(d2[2]) * p2 + 2.f * fabsf(d2[4])) +
       2.f * p1 * p2 * fabsf(d2[5]);
  // sym3 order 000 001 011 111 002 012 112 022 122 222, with the number of index orderings of each
  const float q[10] = {1.f, p1, p1 * p1, p1 * p1 * p1, p2, p1 * p2, p1 * p1 * p2, p2 * p2, p1 * p2 * p2, p2 * p2 * p2};
  const float mult[10] = {1.f, 3.f, 3.f, 1.f, 3.f, 6.f, 3.f, 3.f, 3.f, 1.f};
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 10; k++) s += mult[k] * q[k] * fabsf(d3[k]);
  bh = 2.f * s;
}

// one tile: matrices base .. base + cnt - 1 by a CTA of GMF_TPB threads (the standalone kernel and the batched
// persistent kernel run the same code).  T is the type of the arrays in HBM and of phase B: double for the FP64
// path; float for the mixed-precision path, where phase A (spectral analysis, series, residues: the FP64 steps of
// the method) stays in FP64 and its record -- with the scale factors folded in, in FP64 -- is rounded to FP32 once.
// idx (optional): tile position p holds matrix idx[base + p] of the arrays instead of base + p (the reordered launch);
// roots, keys (optional, by matrix): the closed-form roots and their key, already computed by gmf_key_kernel.
template <int KIND, int ORDER, typename T = double>
MF_D void gmf_tile(int64_t base, int cnt, const T *__restrict__ A, T *__restrict__ F, T *__restrict__ J,
                   T *__restrict__ H, const GmfCoef &C, GmfSmem &S, const int *__restrict__ idx = nullptr,
                   const double *__restrict__ roots = nullptr, const unsigned char *__restrict__ keys = nullptr) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int e = tid; e < cnt * 9; e += GMF_TPB) {
    const int p = e / 9;
    const long long g = idx ? (long long)idx[base + p] : base + p;
    S.x[e] = (double)A[g * 9 + (e - 9 * p)];
    if (e == 9 * p) S.gidx[p] = g;
  }
  static_assert(ORDER < 3 || sizeof(T) == 8, "the tangent form is FP64");
  static_assert(sizeof(GmfState) >= GMF_REC * sizeof(double), "a record fits its matrix's state slot");
  constexpr int OD = ORDER == 3 ? 2 : ORDER;  // the order of the derivatives the record holds
  if (ORDER == 2) {  // index tables of phase B
    for (int t = tid; t < 405; t += GMF_TPB) {  // t = 45 (ab) + sym2(cd, ef), cd <= ef
      const int p = t % 45;
      int ef = 0;
      while (sym2(0, ef + 1) <= p) ef++;
      S.umap[t] = hmap_entry(81 * (t / 45) + 9 * (p - sym2(0, ef)) + ef);
    }
    for (int w = tid; w < 729; w += GMF_TPB) {
      const int cd = (w / 9) % 9, ef = w % 9;
      S.hkey[w] = (unsigned short)(45 * (w / 81) + sym2(min(cd, ef), max(cd, ef)));
    }
    for (int t = tid; t < 165; t += GMF_TPB) {
      int z = 0;
      while (sym3(0, 0, z + 1) <= t) z++;
      int y = 0;
      while (sym3(0, y + 1, z) <= t && y + 1 <= z) y++;
      S.t6map[t] = (unsigned short)((t - sym3(0, y, z)) | (y << 4) | (z << 8));
    }
    for (int t = tid; t < 135; t += GMF_TPB) {
      const int pr = t / 3, m = t % 3;
      int z = 0;
      while (sym2(0, z + 1) <= pr) z++;
      S.ymap[t] = (unsigned short)((pr - sym2(0, z)) | (z << 4) | (m << 8));
    }
  }
  __syncthreads();

  // ---- phase A, first part: the closed-form roots of matrix tid and the key of the branches the spectral analysis
  // takes next (complex pair, pair refinement, branch-cut pair); the roots wait in the matrix's state slot
  unsigned key = 0xFFFFFFFFu;
  if (tid < cnt) {
    double *xs = reinterpret_cast<double *>(&S.state[tid]);
    if (roots) {
      const long long g = S.gidx[tid];
#pragma unroll
      for (int k = 0; k < 6; k++) xs[k] = roots[g * 6 + k];
      key = keys[g];
    } else {
      double a[9];
#pragma unroll
      for (int k = 0; k < 9; k++) a[k] = S.x[tid * 9 + k];
      cx x[3];
      key = gmf_roots<KIND>(a, x);
#pragma unroll
      for (int i = 0; i < 3; i++) { xs[2 * i] = x[i].re; xs[2 * i + 1] = x[i].im; }
    }
  }
  S.key[tid] = key;
  __syncthreads();
  // the scratch of an ordered launch (idx, roots, keys: rows of the last matrices' H) has been read by this CTA
  griddep_launch_dependents();
  {
    int rank = 0;
    for (int j = 0; j < GMF_TPB; j++) {
      const unsigned kj = S.key[j];
      rank += (kj < key) | ((kj == key) & (j < tid));
    }
    S.perm[rank] = tid;
  }
  __syncthreads();

  // ---- phase A, second part, in that order (the lanes of a warp take the same branches): the rest of the spectral
  // analysis, and the key of the finish: class (no group < real series < complex series), longer series first, then
  // the group's node pattern
  {
    const int mi = S.perm[tid];
    unsigned key2 = 0xFFFFFFFFu;
    if (mi < cnt) {
      double a[9];
#pragma unroll
      for (int k = 0; k < 9; k++) a[k] = S.x[mi * 9 + k];
      const double *xs = reinterpret_cast<const double *>(&S.state[mi]);
      cx x[3];
#pragma unroll
      for (int i = 0; i < 3; i++) x[i] = cmk(xs[2 * i], xs[2 * i + 1]);
      GmfState St;
      gmf_classify_from<KIND, OD>(a, x, C, St);
      S.state[mi] = St;
      key2 = gmf_finish_key(St);
    }
    S.key[mi] = key2;  // (every thread finished reading the first keys before the last barrier)
  }
  __syncthreads();
  {
    key = S.key[tid];
    int rank = 0;
    for (int j = 0; j < GMF_TPB; j++) {
      const unsigned kj = S.key[j];
      rank += (kj < key) | ((kj == key) & (j < tid));
    }
    S.perm[rank] = tid;
  }
  __syncthreads();

  // ---- phase A, finish, in the order of the second key: slot tid takes the matrix of rank tid; F goes straight to
  // HBM, the record takes the place of the matrix's state (read by gmf_finish and no longer needed)
  const int mine = S.perm[tid];
  if (mine < cnt) {
    GmfRec R;
    gmf_finish<KIND, OD, sizeof(T) == 4>(S.state[mine], C, R);
    if (F) {
#pragma unroll
      for (int k = 0; k < 9; k++) F[S.gidx[mine] * 9 + k] = (T)R.F[k];
    }
    if (ORDER == 3) {  // the tangent contracts with F: F stays in the matrix's input slot
#pragma unroll
      for (int k = 0; k < 9; k++) S.x[mine * 9 + k] = R.F[k];
    }
    if (OD >= 1) {
      // the scale factors sc1 / sc2 are folded into D2' / D3' when finite and nonzero; otherwise each output entry
      // is multiplied by them (keeping the reference's NaN / Inf); rc[34] / rc[35] hold the factor left to apply.
      // The record stays in FP64 for both storage types (the FP32 path rounds it in phase B).
      double *rc = reinterpret_cast<double *>(&S.state[mine]);
#pragma unroll
      for (int k = 0; k < 9; k++) { rc[k] = R.r1[k]; rc[9 + k] = R.r2[k]; }
      const bool f1 = isfinite(R.sc1) & (R.sc1 != 0.0);
      const double s1 = sel(f1, R.sc1, 1.0);
#pragma unroll
      for (int k = 0; k < 6; k++) rc[18 + k] = R.D2[k] * s1;
      rc[34] = sel(f1, 1.0, R.sc1);
      if (OD >= 2) {
        const bool f2 = isfinite(R.sc2) & (R.sc2 != 0.0);
        const double s2 = sel(f2, R.sc2, 1.0);
#pragma unroll
        for (int k = 0; k < 10; k++) rc[24 + k] = R.D3[k] * s2;
        rc[35] = sel(f2, 1.0, R.sc2);
      }
      if (OD < 2) {
#pragma unroll
        for (int k = 24; k < 34; k++) rc[k] = 0.0;
        rc[35] = 1.0;
      }
    }
  }
  if (ORDER < 1) return;
  __syncwarp();

  // ---- phase B: each warp assembles the matrices it finished (its 32 slots), so no CTA barrier separates the two
  // phases: a warp with short series assembles while the others still run theirs
  double *wkd = S.work[warp];
  float *wkf = reinterpret_cast<float *>(S.work[warp]);
  for (int sl = warp * 32; sl < warp * 32 + 32; sl++) {
    const int mi = S.perm[sl];
    if (mi >= cnt) break;  // the padding slots sort last
    const double *rcd = reinterpret_cast<const double *>(&S.state[mi]);
    if constexpr (ORDER == 3) {
      gmf_tangent_warp(rcd, S.x + mi * 9, wkd, lane, J ? J + S.gidx[mi] * 9 : nullptr, H + S.gidx[mi] * 81);
      continue;
    }
    T *oj = J + S.gidx[mi] * 81;
    T *oh = ORDER >= 2 ? H + S.gidx[mi] * 729 : nullptr;
    if constexpr (sizeof(T) == 8) {
      gmfb_t4<double>(rcd, wkd, lane);
      gmfb_store_j<double, T>(wkd, rcd[34], oj, lane);
      if (ORDER >= 2) {
        gmfb_u<double>(rcd, wkd, S, lane);
        gmfb_store_h<double, T>(wkd, rcd[35], S, oh, lane);
      }
    } else {
      // FP32: the record rounded once (past the FP32 work area) and the bounds of its contractions; contract and store
      // it; where its bound exceeds GMF_F32_AMP times the largest entry (uniform in the warp), contract the FP64
      // record and store the matrix's J (H) again
      float *rcf = wkf + GMF_RECF;
      for (int k = lane; k < GMF_REC; k += 32) rcf[k] = (float)rcd[k];
      __syncwarp();
      float bj, bh;  // (every lane, from the shared copy)
      gmfb_bounds(rcf, bj, bh);
      gmfb_t4<float>(rcf, wkf, lane);
      const float mj = gmfb_store_j<float, T, true>(wkf, rcf[34], oj, lane);
      if (bj > GMF_F32_AMP * mj) {
        gmfb_t4<double>(rcd, wkd, lane);
        gmfb_store_j<double, T>(wkd, rcd[34], oj, lane);
      }
      if (ORDER >= 2) {
        gmfb_u<float>(rcf, wkf, S, lane);
        const float mh = gmfb_store_h<float, T, true>(wkf, rcf[35], S, oh, lane);
        if (bh > GMF_F32_AMP * mh) {
          gmfb_u<double>(rcd, wkd, S, lane);
          gmfb_store_h<double, T>(wkd, rcd[35], S, oh, lane);
        }
      }
    }
  }
}

template <int KIND, int ORDER, typename T>
__global__ void __launch_bounds__(GMF_TPB, GMF_MIN_CTAS) gmf_kernel(int64_t n, const T *__restrict__ A, T *__restrict__ F,
                                                      T *__restrict__ J, T *__restrict__ H, const GmfCoef C,
                                                      const int *__restrict__ idx, const double *__restrict__ roots,
                                                      const unsigned char *__restrict__ keys) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GmfSmem &S = *reinterpret_cast<GmfSmem *>(smem_raw);
  const int64_t base = (int64_t)blockIdx.x * GMF_TPB;
  gmf_tile<KIND, ORDER, T>(base, (int)min((int64_t)GMF_TPB, n - base), A, F, J, H, C, S, idx, roots, keys);
}

// ---- batch-wide reordering.  The work of a matrix depends on its spectrum (real roots or a complex pair, pair
// refinement, branch-cut pair, the geometry of the roots); a CTA's 128 matrices of a random batch span many such
// classes, and a warp of one class runs up to twice as fast as a mixed one.  So the standalone launch first computes
// the class key of every matrix (gmf_roots), orders the batch by it with a stable counting sort, and evaluates the
// matrices in that order (results written at their own indices).  The scratch of the sort -- the order, the keys and
// per-block counts, about 9 bytes per matrix, and for order 2 the roots (48 bytes), which the evaluation then reads
// instead of recomputing them -- lies in the caller's own largest output array (H, or J for order 1), in the part
// that belongs to the last few matrices; those are evaluated afterwards by a plain launch, which overwrites it.
// Nothing is allocated, and concurrent calls share nothing.

template <int KIND, typename T>
__global__ void __launch_bounds__(GKEY_TPB) gmf_key_kernel(int n, const T *__restrict__ A,
                                                           unsigned char *__restrict__ keys,
                                                           int *__restrict__ counts, int nblk,
                                                           double *__restrict__ roots) {
  __shared__ int hist[GKEY_BINS];
  for (int k = threadIdx.x; k < GKEY_BINS; k += GKEY_TPB) hist[k] = 0;
  __syncthreads();
  const int i = blockIdx.x * GKEY_TPB + threadIdx.x;
  if (i < n) {
    double a[9];
#pragma unroll
    for (int k = 0; k < 9; k++) a[k] = (double)A[(int64_t)i * 9 + k];
    cx x[3];
    const unsigned key0 = gmf_roots<KIND>(a, x) & (GKEY_BINS - 1);
    // log, powers: the classes in descending key order, so that the launch starts with the complex pairs, the pairs
    // refined from A and the branch-cut pairs and ends with the real spectra of the smallest spread (equal
    // eigenvalues: the shortest work), and fewer SMs idle behind its last CTAs (C1 order 2: log 11.36 -> 10.84 ms,
    // sqrt 15.54 -> 14.82 ms); exp keeps the ascending order (7.74 ms against 7.78 ms descending)
    const unsigned key = KIND == EXP ? key0 : (GKEY_BINS - 1) - key0;
    keys[i] = (unsigned char)key;
    if (roots) {
#pragma unroll
      for (int k = 0; k < 3; k++) { roots[(int64_t)i * 6 + 2 * k] = x[k].re; roots[(int64_t)i * 6 + 2 * k + 1] = x[k].im; }
    }
    atomicAdd(&hist[key], 1);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < GKEY_BINS; k += GKEY_TPB) counts[k * nblk + blockIdx.x] = hist[k];
}

// (early: launched with programmatic stream serialisation, so that it may start once every CTA of the preceding
// gmf_kernel launch has read its scratch -- griddep_launch_dependents in gmf_tile -- instead of after its last CTA)
template <int KIND, int ORDER, typename T>
cudaError_t gmf_launch_one(cudaStream_t st, unsigned blocks, int64_t n, const T *A, T *F, T *J, T *H,
                           const GmfCoef &C, const int *idx = nullptr, const double *roots = nullptr,
                           const unsigned char *keys = nullptr, bool early = false) {
  static std::atomic<unsigned long long> attr{0};  // per instantiation, one bit per device
  cudaError_t e = smem_limit_per_device(gmf_kernel<KIND, ORDER, T>, (int)sizeof(GmfSmem), attr);
  if (e != cudaSuccess) return e;
  if (!early) {
    gmf_kernel<KIND, ORDER, T><<<blocks, GMF_TPB, sizeof(GmfSmem), st>>>(n, A, F, J, H, C, idx, roots, keys);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(GMF_TPB);
  cfg.dynamicSmemBytes = sizeof(GmfSmem);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, gmf_kernel<KIND, ORDER, T>, n, A, F, J, H, C, idx, roots, keys);
  return e != cudaSuccess ? e : cudaGetLastError();
}

// orders 1 and 2 of a large batch: key, sort, reordered evaluation of the first nm matrices, plain evaluation of the
// last n - nm (whose share of the largest output array held the scratch)
template <int KIND, int ORDER, typename T>
cudaError_t gmf_launch_sorted(cudaStream_t st, int64_t n, const T *A, T *F, T *J, T *H, const GmfCoef &C) {
  T *big = ORDER >= 2 ? H : J;
  const int64_t per = ORDER == 2 ? 729 : 81;  // elements of the largest output per matrix (ORDER 3: the tangent K)
  const int64_t nblk_n = (n + GKEY_TPB - 1) / GKEY_TPB;
  // order, counts, totals, keys (bytes) and, for order 2, the roots (48 bytes per matrix; the tail stays ~1 % of the
  // batch)
  const int64_t need = 4 * n + 4 * (int64_t)GKEY_BINS * (nblk_n + 1) + n + (ORDER == 2 ? 48 * n + 8 : 0) + 64;
  const int64_t tail = (need + per * (int64_t)sizeof(T) - 1) / (per * (int64_t)sizeof(T)) + 1;
  const int64_t nm = n - tail;
  const int nblk = (int)((nm + GKEY_TPB - 1) / GKEY_TPB);
  char *scr = reinterpret_cast<char *>(big + nm * per);
  int *order = reinterpret_cast<int *>(scr);
  int *counts = order + nm, *totals = counts + (int64_t)GKEY_BINS * nblk;
  unsigned char *keys = reinterpret_cast<unsigned char *>(totals + GKEY_BINS);
  double *roots = nullptr;
  if (ORDER == 2) {
    const uintptr_t r = reinterpret_cast<uintptr_t>(keys + nm);
    roots = reinterpret_cast<double *>((r + 7) & ~(uintptr_t)7);
  }
  gmf_key_kernel<KIND, T><<<nblk, GKEY_TPB, 0, st>>>((int)nm, A, keys, counts, nblk, roots);
  gmf_scan_kernel<<<GKEY_BINS, 1024, 0, st>>>(counts, nblk, totals);
  gmf_scatter_kernel<<<nblk, GKEY_TPB, 0, st>>>((int)nm, keys, counts, totals, nblk, order);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = gmf_launch_one<KIND, ORDER, T>(st, (unsigned)((nm + GMF_TPB - 1) / GMF_TPB), nm, A, F, J, H, C, order, roots,
                                     roots ? keys : nullptr);
  if (e != cudaSuccess) return e;
  // the tail's rows of the outputs: F (9 per matrix; optional for ORDER 3), J (81) and H (729) for orders 1, 2,
  // G (9, optional) and K (81) for the tangent
  T *Ft = F ? F + nm * 9 : nullptr;
  T *Jt = ORDER == 3 ? (J ? J + nm * 9 : nullptr) : J + nm * 81;
  T *Ht = ORDER == 3 ? H + nm * 81 : (ORDER == 2 ? H + nm * 729 : nullptr);
  // the tail overwrites the scratch only: it may start as soon as every CTA of the ordered launch has read it
  return gmf_launch_one<KIND, ORDER, T>(st, (unsigned)((tail + GMF_TPB - 1) / GMF_TPB), tail, A + nm * 9, Ft, Jt, Ht,
                                        C, nullptr, nullptr, nullptr, true);
}

constexpr int64_t GMF_SORT_MIN = 1 << 15;  // below this the reordering does not pay for its launches

template <int KIND, typename T>
cudaError_t gmf_launch_kind(int order, cudaStream_t st, unsigned blocks, int64_t n, const T *A, T *F, T *J, T *H,
                            const GmfCoef &C, bool reorder = true) {
  // log and pow (the branch-cut pair and the wider spread of work); exp only at order 2 (measured at n = 2^20:
  // order 2 10.2 -> 9.6 ms ordered, order 1 4.7 -> 5.0 ms, so order 1 keeps the plain launch)
  const bool sorted = reorder & ((KIND != EXP) | (order == 2)) & (n >= GMF_SORT_MIN) & (n <= INT_MAX);
  if (order == 2) return sorted ? gmf_launch_sorted<KIND, 2, T>(st, n, A, F, J, H, C)
                                : gmf_launch_one<KIND, 2, T>(st, blocks, n, A, F, J, H, C);
  if (order == 1) return sorted ? gmf_launch_sorted<KIND, 1, T>(st, n, A, F, J, H, C)
                                : gmf_launch_one<KIND, 1, T>(st, blocks, n, A, F, J, H, C);
  return gmf_launch_one<KIND, 0, T>(st, blocks, n, A, F, J, H, C);
}

// the tangent form (ORDER 3): F (optional), G = J^T F (optional), K = J^T J + F : H of a batch, in the order of the
// batch-wide sort like the order-2 evaluation (without the reuse of the roots, whose scratch would not fit K's tail)
template <int KIND>
cudaError_t gmf_launch_tangent_kind(cudaStream_t st, int64_t n, const double *A, double *F, double *G, double *K,
                                    const GmfCoef &C) {
  const bool sorted = (n >= GMF_SORT_MIN) & (n <= INT_MAX);
  return sorted ? gmf_launch_sorted<KIND, 3, double>(st, n, A, F, G, K, C)
                : gmf_launch_one<KIND, 3, double>(st, (unsigned)((n + GMF_TPB - 1) / GMF_TPB), n, A, F, G, K, C);
}

// one kind (instantiated in gmf_<kind>.cu and gmf_mixed_<kind>.cu so that they compile in parallel)
template <int KIND, typename T = double>
cudaError_t gmf_launch_t(double al, int64_t n, const T *A, T *F, T *J, T *H, cudaStream_t st, bool reorder = true) {
  const int order = H ? 2 : (J ? 1 : 0);
  GmfCoef C;
  gmf_coef(KIND, al, order, C, sizeof(T) == 4);
  const unsigned blocks = (unsigned)((n + GMF_TPB - 1) / GMF_TPB);
  return gmf_launch_kind<KIND, T>(order, st, blocks, n, A, F, J, H, C, reorder);
}

template <int KIND>
cudaError_t gmf_tangent_t(double al, int64_t n, const double *A, double *F, double *G, double *K, cudaStream_t st) {
  GmfCoef C;
  gmf_coef(KIND, al, 2, C);
  return gmf_launch_tangent_kind<KIND>(st, n, A, F, G, K, C);
}

}  // namespace mf
