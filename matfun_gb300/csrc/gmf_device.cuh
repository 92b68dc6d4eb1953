// gmf_device.cuh -- per-matrix device math of the general family (FP64, one thread per matrix): F, J, H of f(A) for
// a general real 3x3 A through the confluent Newton-Hermite form over its eigenvalues (the method of the reference's
// c/include/matfun/gmf_kernel.hpp:251-692 and theory.md, "General matrices"):
//   * the eigenvalues mu_i = m + x_i of A / sig (sig a power of two, m the shift), the x_i of the deviator in closed
//     form, refined against A where the closed form loses accuracy (a pair from det A and the principal minors after
//     Newton on the separated root; the pair near the branch cut from the 2x2 block on the complement of the left
//     eigenvector; Newton on single real nodes far from m)
//   * the nodes ordered and grouped (all three, the closest pair, or none); the 19 confluent divided differences
//     f[x0^a x1^b x2^c]: a group's by its Taylor series streamed over the series index, a single node's beside a
//     pair by its residue, and three single nodes by the Hermite recursion
//   * the real basis r_0 = I, r_1, r_2 and T = I + iN, giving F and the real-reduced divided differences
//     D2' = Re(T^T D T) (symmetric, 6 distinct) and D3' (T on all three indices; symmetric, 10 distinct).
// The decisions and their thresholds are the method's (they define the result to which the parity tests hold this
// code); the evaluation is this file's own: one thread per matrix takes only its branch, the CTA-local and batch-wide
// orderings of the kernels give a warp's lanes the same branches.  The kernels then contract D2' and D3' with r into
// J and H through symmetric tensors (gmf_kernels.cuh).
#pragma once
#include "ffloat.cuh"

namespace mf {

constexpr double G_RHO = 0.7, G_R_EXP = 4.0, G_RHO_POLE = 0.6;  // gmf_kernel.hpp:30
// log forms its series groups only within 0.5 of the centre instead of the reference's 0.7: nodes spread wider are
// taken as a closer pair group and a single node, or as single nodes (dd_three_single, the residues), so that the
// longest series (40-100 terms at radii 0.5-0.7) are not run: C1 log order 2 12.03 -> 11.37 ms on GB300.  Measured
// against the oracle on the host build of this header: C1 within 5e-14 per matrix, the stress sets within 8e-15 per
// call, every golden case of the reference within 0.17 of its tolerance (the same as at 0.7).  Powers keep 0.7:
// there the single-node forms lost up to 7e-11 per matrix at 0.5.
constexpr double G_RHO_LOG = 0.5;
// The FP32-storage kernels (results to about 1e-7) take their series groups only within 0.35 of the centre and end
// their series 2^-44 below the largest term instead of 1e-17: on GB300 C1 order 2 log 7.40 -> 6.92 ms, sqrt 10.59 ->
// 9.77, pow 0.3 11.84 -> 10.90 (exp unchanged, so it keeps its radius of 4), with the per-matrix errors of 6000
// random general matrices unchanged (3.5e-7 at most).  At 0.25 with a stop at 2^-34 the single-node forms of
// near-defective matrices lost up to 3e-4.
constexpr double G_RHO_F32 = 0.35, G_R_EXP_F32 = 4.0;
constexpr float G_LSTOP = -56.5237f - 0.05f, G_LSTOP_F32 = -44.f;  // log2(1e-17) less a margin; 2^-44
constexpr int G_KMAX = 200;                                      // gmf_kernel.hpp:31

// launch constants of the gmf kernels (host-computed once per call)
struct GmfCoef {
  double al;              // exponent (pow; sqrt arrives as pow 0.5), 0 otherwise
  double rho_f;           // group radius ratio: 0.5 for log, 0.7 or min(0.7, 3 / al) for pow
  double bh[3], bl[3];    // al - k split exactly (k = 0, 1, 2)
  double bt[G_KMAX];      // series coefficients b_j of f(c (1 + u)) (gmf_kernel.hpp:48-53)
  float lterm[G_KMAX];    // log2(|b_(n+k)| C(k + n, n)), n = 3 (order + 1) - 1: the term bound of gmf_kernel.hpp:73-97
  float bth[G_KMAX], btl[G_KMAX];  // bt as float-float (hi + lo)
  int ffser;              // 1: the group series may run on the FP32 pipe (every |bth[j]| <= 2^100)
  int tsh;                // bth, btl hold b_j 2^(tsh j) and group_tail takes the offsets times 2^-tsh (exp: 2, so
                          // that 4^j / j! stays in FP32's range; log, pow: 0)
  double rexp;            // exp: the group radius (offsets from the group's centre)
  float lstop;            // log2 of the last series term's size relative to the largest
};

// host: launch constants (series coefficients gmf_kernel.hpp:48-53; the binomial factors of the term bound by the
// recurrence of gmf_kernel.hpp:84, as log2 values); fp32: those of the FP32-storage kernels
inline void gmf_coef(int kind, double al, int order, GmfCoef &C, bool fp32 = false) {
  C.al = al;
  C.rho_f = kind == LOG ? G_RHO_LOG : ((kind == POW && 3.0 / al < G_RHO) ? 3.0 / al : G_RHO);
  C.rexp = G_R_EXP;
  C.lstop = G_LSTOP;
  if (fp32) {
    C.rho_f = C.rho_f < G_RHO_F32 ? C.rho_f : G_RHO_F32;
    C.rexp = G_R_EXP_F32;
    C.lstop = G_LSTOP_F32;
  }
  for (int k = 0; k < 3; k++) {
    const double bh = al - k, bb = bh - al;
    C.bh[k] = bh;
    C.bl[k] = (al - (bh - bb)) + (-k - bb);
  }
  C.bt[0] = 1.0;
  for (int j = 1; j < G_KMAX; j++)
    C.bt[j] = kind == EXP ? C.bt[j - 1] / j : (kind == LOG ? (j % 2 ? 1.0 : -1.0) / j : C.bt[j - 1] * (al - j + 1) / j);
  C.tsh = kind == EXP ? 2 : 0;
  C.ffser = 1;
  for (int j = 0; j < G_KMAX; j++) {
    const double bs = std::ldexp(C.bt[j], C.tsh * j);
    C.ffser &= std::fabs(bs) <= 0x1p100;  // (false for a NaN)
    C.bth[j] = (float)bs;
  }
  for (int j = 0; j < G_KMAX; j++)
    C.btl[j] = C.ffser ? (float)(std::ldexp(C.bt[j], C.tsh * j) - (double)C.bth[j]) : 0.f;
  const int nn = 3 * (order + 1) - 1;
  double c = 1.0;
  for (int k = 0; k < G_KMAX; k++) {
    const double t = nn + k < G_KMAX ? std::fabs(C.bt[nn + k]) * c : 0.0;
    C.lterm[k] = t > 0 ? (float)std::log2(t) : -INFINITY;
    c = c * (k + nn + 1) / (k + 1);
  }
}

// the 19 divided differences f[x0^a x1^b x2^c], a >= b >= c, a >= 1, in lexicographic order of (a, b, c); each is
// its parent with one node added (node 0 if a - 1 >= b, else node 1 if b - 1 >= c, else node 2)
MF_D constexpr int gpos(int a, int b, int c) { return (a == 1 ? 0 : (a == 2 ? 3 : 9)) + b * (b + 1) / 2 + c; }
MF_D constexpr int gms(int t, int i) {  // multiplicity of node i in entry t
  return i == 0 ? (t < 3 ? 1 : (t < 9 ? 2 : 3))
                : (i == 1 ? (t < 3 ? (t >= 1) : (t < 9 ? (t >= 6 ? 2 : (t >= 4)) : (t >= 15 ? 3 : (t >= 12 ? 2 : (t >= 10)))))
                          : (t < 3 ? (t == 2) : (t < 9 ? (t == 5 || t == 7 ? 1 : (t == 8 ? 2 : 0))
                                                      : (t == 11 || t == 13 || t == 16 ? 1 : (t == 14 || t == 17 ? 2 : (t == 18 ? 3 : 0))))));
}
MF_D constexpr int gnode(int t) {
  return t == 0 ? 0 : (gms(t, 0) - 1 >= gms(t, 1) ? 0 : (gms(t, 1) - 1 >= gms(t, 2) ? 1 : 2));
}
MF_D constexpr int gpar(int t) {
  return t == 0 ? -1
                : (gnode(t) == 0 ? gpos(gms(t, 0) - 1, gms(t, 1), gms(t, 2))
                                 : (gnode(t) == 1 ? gpos(gms(t, 0), gms(t, 1) - 1, gms(t, 2))
                                                  : gpos(gms(t, 0), gms(t, 1), gms(t, 2) - 1)));
}
MF_D constexpr int gpos2(int j, int k) { return gpos(2, (j >= 1) + (k >= 1), (j >= 2) + (k >= 2)); }
MF_D constexpr int gpos3(int j, int k, int l) {
  return gpos(3, (j >= 1) + (k >= 1) + (l >= 1), (j >= 2) + (k >= 2) + (l >= 2));
}

// number of series terms (gmf_kernel.hpp:73-97): the group series needs terms until |b_(n+k)| C(k+n, n) r^k drops
// below 1e-17 of the largest, the pole series until C(k+2, 2) q^k <= 1e-17 (2^-44 for the FP32-storage kernels,
// C.lstop).  Evaluated on log2 values in FP32 (the
// FP64 pipe is the bottleneck of this kernel) with a threshold 2^-0.05 below 1e-17, so that the count is never
// smaller than the FP64 bound's; one term more changes a result by less than 1e-17 relative.
//
// Also the term indices j1, j2 from which on every term is 2^-6 (j1) and 2^-30 (j2) below the largest term bound (the
// bound is unimodal in k): group_series sums the terms from j1 on in float-float and from j2 on in FP32, whose
// rounding errors (2^-48 and 2^-24 of the term) then stay below 2^-54 of the largest term, under the FP64 rounding of
// the leading terms (2^-53 of the largest).
MF_D int nterms(const GmfCoef &C, int n, double r, double q, int &j1, int &j2) {
  const float L17 = C.lstop;  // log2(1e-17) less a margin (FP64 results), 2^-34 (FP32 results)
  int M = 1, k1 = G_KMAX, k2 = G_KMAX;
  if (r > 0) {
    const float lr = log2f((float)r);
    float best = -INFINITY;
    for (int k = 0; n + k < G_KMAX; k++) {
      const float lk = (float)k * lr;
      const float t = C.lterm[k] + lk;
      best = fmaxf(best, t);
      M = k;
      k1 = (k1 == G_KMAX) & (t <= best - 6.0f) ? k : k1;
      k2 = (k2 == G_KMAX) & (t <= best - 30.0f) ? k : k2;
      if (((k > 2) & (t <= best + L17)) | (lk < -1074.0f)) break;
    }
  }
  j1 = n + k1 < G_KMAX ? n + k1 : G_KMAX;
  j2 = n + k2 < G_KMAX ? n + k2 : G_KMAX;
  if (q > 0) {
    const float lq = log2f((float)q);
    for (int k = 0; n + k < G_KMAX; k++) {
      if ((k > M) & (log2f((k + 1.0f) * (k + 2.0f) * 0.5f) + (float)k * lq <= L17)) break;
      M = k > M ? k : M;
    }
  }
  return n + M + 1 < G_KMAX ? n + M + 1 : G_KMAX;
}

// the group-series constant of log, f(c) at the real group centre (the real part of coef0<LOG>, without the
// arguments of the complex logarithm, which it does not need)
MF_D double log_b0(double sig, double m, double cxg, double cmu) {
  bool near = (m > 0) & (fabs(cxg) <= 0.5 * m);
  double ms = sel(m > 0, m, 1.0), zr = cxg / ms;
  return near ? log(sig * ms) + 0.5 * log1p(zr * (2.0 + zr)) : log(sig * fabs(cmu));
}

// an exact power of two, -1022 <= e <= 1023
MF_D double pow2i(int e) { return __longlong_as_double((long long)(1023 + e) << 52); }
// d_c of group_tail: the in-group multiplicity of entry c less one (0 for an entry without in-group nodes)
MF_D int gdeg(int c, const bool *inG) {
  const int d = (inG[0] ? gms(c, 0) : 0) + (inG[1] ? gms(c, 1) : 0) + (inG[2] ? gms(c, 2) : 0) - 1;
  return d < 0 ? 0 : d;
}

// the terms j1 <= j < K of group_series without a pole node (every entry's coefficient is b_j): float-float up to
// j2, FP32 from there on (see nterms), added to D at the end; Ep0 is the FP64 recursion state after term j1 - 1.
// With tsh > 0 (exp) the tail runs on u~ = u 2^-tsh and b~_j = b_j 2^(tsh j): entry c at step j is homogeneous of
// degree j - d_c in u (d_c = its in-group multiplicity - 1), so its state enters as Ep0 2^(-tsh (j1 - 1 - d_c)) and
// its tail sum leaves times 2^(-tsh d_c), all exact powers of two.
template <int ND, bool REAL>
MF_D void group_tail(int K, int j1, int j2, const GmfCoef &C, const bool *inG, const cx *u, const cx *Ep0, cx *D) {
  const ffl zero = {0.f, 0.f};
  const int sh = C.tsh;
  const double us = pow2i(-sh);
  ffl ur[3], ui[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    ur[i] = ff_of(u[i].re * us);
    ui[i] = REAL ? zero : ff_of(u[i].im * us);
  }
  ffl Er[ND], Ei[ND], Sr[ND], Si[ND];  // (the state updated in place, as in group_series)
#pragma unroll
  for (int c = 0; c < ND; c++) {
    const double es = pow2i(-sh * (j1 - 1 - gdeg(c, inG)));
    Er[c] = ff_of(Ep0[c].re * es);
    Ei[c] = REAL ? zero : ff_of(Ep0[c].im * es);
    Sr[c] = zero;
    Si[c] = zero;
  }
  const int jb = K < j2 ? K : j2;
  for (int j = j1; j < jb; j++) {
    const ffl bj = {C.bth[j], C.btl[j]};
#pragma unroll
    for (int c = ND - 1; c >= 0; c--) {
      const int par = gpar(c), i = gnode(c);
      const ffl eppr = par < 0 ? zero : Er[par < 0 ? 0 : par];
      if (REAL) {
        Er[c] = ff_sel(inG[i], ff_add_s(eppr, ff_prod(ur[i], Er[c])), Er[c]);
      } else {
        const ffl eppi = par < 0 ? zero : Ei[par < 0 ? 0 : par];
        const ffl tr = ff_add3(eppr, ff_prod(ur[i], Er[c]), ff_neg(ff_prod(ui[i], Ei[c])));
        const ffl ti = ff_add3(eppi, ff_prod(ur[i], Ei[c]), ff_prod(ui[i], Er[c]));
        Er[c] = ff_sel(inG[i], tr, Er[c]);
        Ei[c] = ff_sel(inG[i], ti, Ei[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < ND; c++) {
      const int par = gpar(c), i = gnode(c);
      Er[c] = ff_sel(inG[i], Er[c], par < 0 ? zero : Er[par < 0 ? 0 : par]);
      acc_ff_add(Sr[c], ff_prod(Er[c], bj));
      if (!REAL) {
        Ei[c] = ff_sel(inG[i], Ei[c], par < 0 ? zero : Ei[par < 0 ? 0 : par]);
        acc_ff_add(Si[c], ff_prod(Ei[c], bj));
      }
    }
  }
  float er[ND], ei[ND], sr[ND], si[ND], vr[3], vi[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    vr[i] = ur[i].hi;
    vi[i] = ui[i].hi;
  }
#pragma unroll
  for (int c = 0; c < ND; c++) {
    er[c] = Er[c].hi;
    ei[c] = REAL ? 0.f : Ei[c].hi;
    sr[c] = 0.f;
    si[c] = 0.f;
  }
  for (int j = jb > j1 ? jb : j1; j < K; j++) {
    const float bj = C.bth[j];
#pragma unroll
    for (int c = ND - 1; c >= 0; c--) {
      const int par = gpar(c), i = gnode(c);
      const float eppr = par < 0 ? 0.f : er[par < 0 ? 0 : par];
      if (REAL) {
        er[c] = inG[i] ? fmaf(vr[i], er[c], eppr) : er[c];
      } else {
        const float eppi = par < 0 ? 0.f : ei[par < 0 ? 0 : par];
        const float tr = fmaf(-vi[i], ei[c], fmaf(vr[i], er[c], eppr)), ti = fmaf(vi[i], er[c], fmaf(vr[i], ei[c], eppi));
        er[c] = inG[i] ? tr : er[c];
        ei[c] = inG[i] ? ti : ei[c];
      }
    }
#pragma unroll
    for (int c = 0; c < ND; c++) {
      const int par = gpar(c), i = gnode(c);
      er[c] = inG[i] ? er[c] : (par < 0 ? 0.f : er[par < 0 ? 0 : par]);
      sr[c] = fmaf(er[c], bj, sr[c]);
      if (!REAL) {
        ei[c] = inG[i] ? ei[c] : (par < 0 ? 0.f : ei[par < 0 ? 0 : par]);
        si[c] = fmaf(ei[c], bj, si[c]);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < ND; c++) {
    const double os = pow2i(-sh * gdeg(c, inG));
    D[c].re = D[c].re + (ff_dbl(Sr[c]) + (double)sr[c]) * os;
    if (!REAL) D[c].im = D[c].im + (ff_dbl(Si[c]) + (double)si[c]) * os;
  }
}

// the streamed group series (gmf_kernel.hpp:493-519) of the ND divided differences; REAL: every in-group offset
// and hence every term is real (half the FP64 instructions of the complex recursion).  FP64 terms up to j1, the tail
// by group_tail (j1 >= K: all in FP64)
//
// The recursion state is updated in place: a term of entry c is its parent's previous term plus u_i times its own
// previous term (entries with an in-group node i), or its parent's new term (the others).  So the in-group entries
// are updated from the last to the first (a parent has the lower index and still holds its previous term), then the
// others from the first to the last (their parent already holds its new term): one state array instead of two, the
// same arithmetic.
template <int ND, bool REAL>
MF_D void group_series(int K, double b0, const GmfCoef &C, const bool *inG, const bool *pk, const cx *u, double iap,
                       cx *D, int j1 = G_KMAX, int j2 = G_KMAX) {
  cx Ep[ND];
#pragma unroll
  for (int c = 0; c < ND; c++)
    Ep[c] = csel(inG[gnode(c)], cmk(0.0, 0.0), gpar(c) < 0 ? cmk(1.0, 0.0) : Ep[gpar(c) < 0 ? 0 : gpar(c)]);
  double q1 = 0.0, q2 = 0.0, q3 = 0.0;
  const int ja = K < j1 ? K : j1;
  for (int j = 0; j < ja; j++) {
    double bj = j == 0 ? b0 : C.bt[j];
    double g1 = (bj - q1) * iap, g2 = (g1 - q2) * iap, g3 = (g2 - q3) * iap;
    q1 = g1; q2 = g2; q3 = g3;
    double qv[4] = {bj, g1, g2, g3};
#pragma unroll
    for (int c = ND - 1; c >= 0; c--) {
      const int par = gpar(c), i = gnode(c);
      const cx epp = par < 0 ? cmk(sel(j == 0, 1.0, 0.0), 0.0) : Ep[par < 0 ? 0 : par];
      if (REAL) Ep[c].re = sel(inG[i], epp.re + u[i].re * Ep[c].re, Ep[c].re);
      else Ep[c] = csel(inG[i], cadd(epp, cmul(u[i], Ep[c])), Ep[c]);
    }
#pragma unroll
    for (int c = 0; c < ND; c++) {
      const int par = gpar(c), i = gnode(c);
      const cx epc = par < 0 ? cmk(0.0, 0.0) : Ep[par < 0 ? 0 : par];
      const double g = sel(pk[0], qv[gms(c, 0)], sel(pk[1], qv[gms(c, 1)], sel(pk[2], qv[gms(c, 2)], qv[0])));
      if (REAL) {
        Ep[c].re = sel(inG[i], Ep[c].re, epc.re);
        D[c].re = D[c].re + Ep[c].re * g;
      } else {
        Ep[c] = csel(inG[i], Ep[c], epc);
        D[c] = cadd(D[c], cscl(Ep[c], g));
      }
    }
  }
  if (K > ja) group_tail<ND, REAL>(K, ja, j2, C, inG, u, Ep, D);
}

// group_series entirely in float-float arithmetic on the FP32 pipe, for the FP32-storage kernels (about 48
// significant bits: 2^-48 of the largest term, amplified by the cancellation of the series, stays far below their
// FP32 results' rounding, but not below that of FP64 results, hence the split of group_tail there).  The same recursion
// and terms, rescaled by S = 2^-e (2^e > |iap|, e <= 8) so that every intermediate stays inside FP32's exponent
// range: offsets u/S, coefficients b_j S^j, pole recursion with the factor S iap (|S iap| < 1, so the pole
// coefficients no longer grow like iap^j); then D[c] = S^-d D~[c] with d = (multiplicity of c's in-group and pole
// nodes) - 1, exact powers of two.  The terms are summed with Sum2 (two_sum per term, errors collected).
template <int ND, bool REAL>
MF_D void group_series_ff(int K, double b0, const GmfCoef &C, const bool *inG, const bool *pk, const cx *u,
                          double iap, int e, cx *D) {
  const double up = __longlong_as_double((long long)(1023 + e) << 52);  // 2^e
  const float S = __int_as_float((127 - e) << 23);                      // 2^-e
  ffl ur[3], ui[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    ur[i] = ff_of(u[i].re * up);
    ui[i] = REAL ? ffl{0.f, 0.f} : ff_of(u[i].im * up);
  }
  const ffl qh = ff_of(iap / up), zero = {0.f, 0.f}, one = {1.f, 0.f}, b0f = ff_of(b0);
  ffl Epr[ND], Epi[ND], Dr[ND], Di[ND];  // (the state updated in place, as in group_series)
#pragma unroll
  for (int c = 0; c < ND; c++) {
    Epr[c] = ff_sel(inG[gnode(c)], zero, gpar(c) < 0 ? one : Epr[gpar(c) < 0 ? 0 : gpar(c)]);
    Epi[c] = zero;
    Dr[c] = zero;
    Di[c] = zero;
  }
  ffl q1 = zero, q2 = zero, q3 = zero;
  float sp = 1.f;
  for (int j = 0; j < K; j++) {
    ffl bj = {C.bth[j] * sp, C.btl[j] * sp};
    bj = ff_sel(j == 0, b0f, bj);
    sp *= S;
    ffl g1 = ff_mul(ff_add_s(bj, ff_neg(q1)), qh), g2 = ff_mul(ff_add_s(g1, ff_neg(q2)), qh),
        g3 = ff_mul(ff_add_s(g2, ff_neg(q3)), qh);
    q1 = g1; q2 = g2; q3 = g3;
    ffl qv[4] = {bj, g1, g2, g3};
#pragma unroll
    for (int c = ND - 1; c >= 0; c--) {
      const int par = gpar(c), i = gnode(c);
      const ffl eppr = par < 0 ? ff_sel(j == 0, one, zero) : Epr[par < 0 ? 0 : par];
      if (REAL) {
        Epr[c] = ff_sel(inG[i], ff_add_s(eppr, ff_prod(ur[i], Epr[c])), Epr[c]);
      } else {
        const ffl eppi = par < 0 ? zero : Epi[par < 0 ? 0 : par];
        const ffl tr = ff_add3(eppr, ff_prod(ur[i], Epr[c]), ff_neg(ff_prod(ui[i], Epi[c])));
        const ffl ti = ff_add3(eppi, ff_prod(ur[i], Epi[c]), ff_prod(ui[i], Epr[c]));
        Epr[c] = ff_sel(inG[i], tr, Epr[c]);
        Epi[c] = ff_sel(inG[i], ti, Epi[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < ND; c++) {
      const int par = gpar(c), i = gnode(c);
      const ffl g = ff_sel(pk[0], qv[gms(c, 0)], ff_sel(pk[1], qv[gms(c, 1)], ff_sel(pk[2], qv[gms(c, 2)], qv[0])));
      Epr[c] = ff_sel(inG[i], Epr[c], par < 0 ? zero : Epr[par < 0 ? 0 : par]);
      acc_ff_add(Dr[c], ff_prod(Epr[c], g));
      if (!REAL) {
        Epi[c] = ff_sel(inG[i], Epi[c], par < 0 ? zero : Epi[par < 0 ? 0 : par]);
        acc_ff_add(Di[c], ff_prod(Epi[c], g));
      }
    }
  }
#pragma unroll
  for (int c = 0; c < ND; c++) {
    int d = -1;
#pragma unroll
    for (int i = 0; i < 3; i++) d += (inG[i] | pk[i]) ? gms(c, i) : 0;
    d = d < 0 ? 0 : e * d;
    const double sc = __longlong_as_double((long long)(1023 + d) << 52);
    D[c] = cmk(ff_dbl(Dr[c]) * sc, REAL ? 0.0 : ff_dbl(Di[c]) * sc);
  }
}

// the state after the spectral analysis (eigenvalues, refinement, node order, groups, offsets, series length):
// everything the divided differences and the basis need.  Between the two halves the kernel sorts the matrices of a
// CTA by class and series length, so that the lanes of a warp do the same amount of the same work.
struct GmfState {
  double As[9];                     // A scaled by 1 / sig
  double sig, m, cxg, cmu, xshift, iap, L, iL;
  cx x[3], mu[3], u[3];
  int K;                            // series terms; 0 without a group
  int flags;  // ab (bits 0-2), inG (3-5), pk (6-8), bad (9), real offsets (10), series split j1 (12-19), j2 (20-27)
};
constexpr int GMF_STATE_D = 9 + 8 + 18;  // doubles of a packed state (K and flags in two ints apart)

// the per-matrix record the kernels contract into F, J, H
struct GmfRec {
  double F[9];
  double r1[9], r2[9];   // real basis (r_0 = I)
  double D2[6];          // Re(T^T D T) at (00, 11, 22, 01, 02, 12)
  double D3[10];         // D3' at the sorted triples (000, 001, 011, 111, 002, 012, 112, 022, 122, 222) = sym3 order
  double sc1, sc2;       // output factors of J and H (NaN for a matrix outside the domain)
};

MF_D void cross3(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
MF_D double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
MF_D void matvec3(const double *M, const double *v, double *o) {
#pragma unroll
  for (int r = 0; r < 3; r++) o[r] = M[3 * r] * v[0] + M[3 * r + 1] * v[1] + M[3 * r + 2] * v[2];
}

// ------------------------------------------------------------------------------------------------ spectral analysis
// One thread per matrix, and only the branch a matrix takes is evaluated (the CTA-local and batch-wide orderings of
// the kernels give the lanes of a warp the same branches).  The decisions -- which roots are refined against A, the
// branch-cut pair, the node order, the groups -- and their thresholds are those of the method (theory: confluent
// Newton-Hermite form over the eigenvalues): they define the result, to which the parity tests hold this code.

// det M by the cofactors of its first row
MF_D double det_cof(const double *M) {
  return M[0] * (M[4] * M[8] - M[5] * M[7]) + M[1] * (M[5] * M[6] - M[3] * M[8]) + M[2] * (M[3] * M[7] - M[4] * M[6]);
}

// det M by Gaussian elimination with partial pivoting (backward stable; exact pivots for a diagonal M), in the
// textbook order: the pivot row P (the largest |M_i0|, the first of equal ones) above the other two rows R, Q, the
// multipliers R_0 / P_0 and Q_0 / P_0, the 2 x 2 remainder [[b, c], [d, e]] eliminated the same way on its larger
// first-column entry.  Newton on det(As - mu I) converges, for an ill-conditioned eigenvalue, to a point of the
// rounding-noise band that this order of operations decides; the parity tests hold ill-conditioned matrices to the
// oracle at 1e-12, so the plain expressions (no explicit fused forms) matter here.
MF_D double det_elim(const double *M) {
  const double a0 = fabs(M[0]), a1 = fabs(M[3]), a2 = fabs(M[6]);
  const bool on1 = (a1 > a0) & (a1 >= a2), on2 = (a2 > a0) & (a2 > a1);
  double P[3], R[3], Q[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    P[k] = on1 ? M[3 + k] : (on2 ? M[6 + k] : M[k]);
    R[k] = (on1 | on2) ? M[k] : M[3 + k];
    Q[k] = on2 ? M[3 + k] : M[6 + k];
  }
  if (P[0] == 0.0) return 0.0;  // the first column vanishes
  const double lr = R[0] / P[0], lq = Q[0] / P[0];
  const double b = R[1] - lr * P[1], c = R[2] - lr * P[2], d = Q[1] - lq * P[1], e = Q[2] - lq * P[2];
  const bool sw = fabs(d) > fabs(b);  // the 2 x 2 pivot
  const double p2 = sw ? d : b, o2 = sw ? c : e, s2 = sw ? b : d, t2 = sw ? e : c;
  if (p2 == 0.0) return 0.0;
  const double sgn = (on1 != sw) ? -1.0 : 1.0;  // parity of the row order
  return sgn * P[0] * p2 * (o2 - s2 / p2 * t2);
}

// the sum of the principal 2 x 2 minors of M (the second invariant), its six products summed in order
MF_D double minors_sum(const double *M) {
  return M[0] * M[4] - M[1] * M[3] + M[0] * M[8] - M[2] * M[6] + M[4] * M[8] - M[5] * M[7];
}

// three Newton steps on p(mu) = det(As - mu I) for the real eigenvalue mu, the other two (a1 + i b1, a2 + i b2: both
// real or a conjugate pair) held fixed: -p'(mu) = (a1 - mu + i b1)(a2 - mu + i b2) = (a1 - mu)(a2 - mu) - b1 b2, real;
// the step p(mu) (1 / -p'(mu)); no step where p' vanishes
MF_D double newton_real(const double *As, double mu, cx o1, cx o2) {
#pragma unroll 1
  for (int it = 0; it < 3; it++) {
    const double d1 = o1.re - mu, d2 = o2.re - mu;
    const double dp = d1 * d2 - o1.im * o2.im;
    if (dp != 0.0) {
      const double B[9] = {As[0] - mu, As[1], As[2], As[3], As[4] - mu, As[5], As[6], As[7], As[8] - mu};
      mu = mu + det_elim(B) * (1.0 / dp);
    }
  }
  return mu;
}

// The eigenvalues of the deviator S (traceless up to rounding) in closed form: x[0] the real root farthest from the
// other two, x[1], x[2] the other two (a real pair, larger magnitude first, or a conjugate pair).  The rounding
// residue tau = tr S / 3 is removed; the traceless d = S - tau I is scaled by a power of two s0 ~ max |d| and its
// characteristic polynomial x^3 - p x - q (p = tr(d^2) / 2, q = det d) by s1 ~ max(sqrt |p|, cbrt |q|), so that p
// and q are O(1).  Three real roots (p > 0, 4 p^3 >= 27 q^2): the trigonometric form, x = 2 sqrt(p / 3) cos(phi),
// phi = acos(q (3 / p)^(3/2) / 2) / 3 (+ 2 pi / 3 for q < 0, the root farthest from the others); otherwise
// Cardano's real root w + p / (3 w), w^3 = q / 2 + sign(q) sqrt(q^2 / 4 - p^3 / 27).  The other two solve
// x^2 + r x + (r^2 - p) = 0: for a discriminant p - 3 r^2 / 4 >= 0 the larger one without cancellation and the other
// from the product q / r, else the conjugate pair.
MF_D void deviator_roots(const double *S, cx *x) {
  constexpr double TWO_PI_3 = 2.0943951023931957;
  const double tau = (S[0] + S[4] + S[8]) / 3.0;
  double d[9];
#pragma unroll
  for (int k = 0; k < 9; k++) d[k] = k % 4 == 0 ? S[k] - tau : S[k];
  double big = fabs(d[0]);
#pragma unroll
  for (int k = 1; k < 9; k++) big = tmax(big, fabs(d[k]));
  const double s0 = pow2safe(big), i0 = 1.0 / s0;
#pragma unroll
  for (int k = 0; k < 9; k++) d[k] *= i0;
  double p = 0.5 * (d[0] * d[0] + d[4] * d[4] + d[8] * d[8]) + d[1] * d[3] + d[2] * d[6] + d[5] * d[7];
  double q = det_cof(d);
  const double s1 = pow2safe(tmax(sqrt(fabs(p)), cbrt(fabs(q)))), i1 = 1.0 / s1;
  p *= i1 * i1;
  q *= i1 * i1 * i1;
  const double sc = s0 * s1;  // the roots of the cubic times sc are those of d
  double r;
  if ((p > 0) & (4.0 * p * p * p >= 27.0 * q * q)) {
    const double p3 = p / 3.0, rt = sqrt(p3);
    double c = 0.5 * q / (p3 * rt);
    c = c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c);
    const double phi = acos(c) / 3.0;
    r = 2.0 * rt * cos(c >= 0 ? phi : phi + TWO_PI_3);
  } else {
    const double disc = 0.25 * q * q - p * p * p / 27.0;
    const double w = cbrt(0.5 * q + copysgn(sqrt(disc > 0 ? disc : 0.0), q));
    r = w != 0 ? w + p / (3.0 * w) : 0.0;
  }
  const double dp = p - 0.75 * r * r, h = sqrt(fabs(dp));
  x[0] = cmk(r * sc + tau, 0.0);
  if (dp >= 0) {
    const double a = -0.5 * r - copysgn(h, r);
    const double prod = r != 0 ? q / r : -p;
    const double b = a != 0 ? prod / a : 0.0;
    x[1] = cmk(a * sc + tau, 0.0);
    x[2] = cmk(b * sc + tau, 0.0);
  } else {
    const double c = -0.5 * r * sc + tau;
    x[1] = cmk(c, h * sc);
    x[2] = cmk(c, -h * sc);
  }
}

// scaling by a power of two sig ~ max |a_ij| (exp: none), shift m = tr As / 3, deviator S = As - m I
template <int KIND>
MF_D void gmf_scale(const double *a, double &sig, double *As, double &m, double *S) {
  double amax = fabs(a[0]);
#pragma unroll
  for (int k = 1; k < 9; k++) amax = tmax(amax, fabs(a[k]));
  sig = KIND == EXP ? 1.0 : pow2safe(amax);
  const double is = 1.0 / sig;
#pragma unroll
  for (int k = 0; k < 9; k++) As[k] = a[k] * is;
  m = (As[0] + As[4] + As[8]) / 3.0;
#pragma unroll
  for (int k = 0; k < 9; k++) S[k] = k % 4 == 0 ? As[k] - m : As[k];
}

// The closed-form pair x[1], x[2] is replaced by one computed from A itself, after Newton on the separated root, when
// the closed form is not the accurate one: the pair small against mu0 (|mid| + R <= mu0 / 4), or the deviator not
// dominated by the shift with mu0 apart from the pair (|m| <= max |S|, R <= |mid - mu0| / 4); mid, R: the pair's
// centre and half-distance.  A real pair's half-distance is half its difference, a conjugate pair's its |imaginary|.
MF_D bool pair_from_A(const double *S, double m, double mu0, cx x1, cx x2, double &mid, double &R) {
  double smax = fabs(S[0]);
#pragma unroll
  for (int k = 1; k < 9; k++) smax = tmax(smax, fabs(S[k]));
  mid = 0.5 * ((m + x1.re) + (m + x2.re));
  R = x1.im != 0 ? fabs(x1.im) : 0.5 * fabs((m + x1.re) - (m + x2.re));
  const bool small = fabs(mid) + R <= 0.25 * fabs(mu0);
  const bool apart = (fabs(m) <= smax) & (R <= 0.25 * fabs(mid - mu0));
  return (mu0 != 0) & (small | apart);
}

// the branches the spectral analysis of a matrix takes, from its closed-form roots: a key for ordering a batch or a
// CTA so that neighbouring matrices take the same ones (complex pair, pair from A, branch-cut pair, and a 16-level
// geometry bucket: the argument of the pair, or the spread of three real roots relative to their mean)
template <int KIND>
MF_D unsigned gmf_roots(const double *a, cx *x) {
  double sig, As[9], m, S[9];
  gmf_scale<KIND>(a, sig, As, m, S);
  deviator_roots(S, x);
  double mid, R;
  const bool pc = pair_from_A(S, m, m + x[0].re, x[1], x[2], mid, R);
  const bool cut = (KIND != EXP) & ((m + x[1].re) + (m + x[2].re) < 0);
  const bool cplx = x[1].im != 0;
  const float argp = fabsf(atan2f((float)x[1].im, (float)(m + x[1].re))) * (16.0f / 3.1415927f);
  const float spread = (float)((tmax(tmax(x[0].re, x[1].re), x[2].re) - tmin(tmin(x[0].re, x[1].re), x[2].re)) /
                               tmax(fabs(m), 1e-300)) * 8.0f;
  const unsigned geo = (unsigned)fminf(cplx ? argp : spread, 15.0f);
  return (cplx ? 128u : 0u) | (pc ? 64u : 0u) | (cut ? 32u : 0u) | geo;
}

// a node of the divided differences during the analysis
struct GNode {
  cx x;          // relative to the shift m
  cx mu;         // the eigenvalue of As
  bool refined;  // mu was computed from As itself: differences to this node are taken between the mu
  bool pairpos;  // one of the closed form's deflated pair (positions 1, 2 before ordering)
};

MF_D void gswap(GNode &a, GNode &b) {
  const GNode t = a;
  a = b;
  b = t;
}

// the rest of the spectral analysis, from the closed-form roots xr of gmf_roots: refinement against A, node order,
// groups, offsets, series length
template <int KIND, int ORDER>
MF_D void gmf_classify_from(const double *a, const cx *xr, const GmfCoef &C, GmfState &St) {
  double sig, As[9], m, S[9];
  gmf_scale<KIND>(a, sig, As, m, S);
  GNode nd[3];
#pragma unroll
  for (int i = 0; i < 3; i++) nd[i] = {xr[i], cmk(m + xr[i].re, xr[i].im), false, i > 0};

  // ---- the pair from det A and the principal minors, after Newton on the separated root
  double mid, Rp;
  bool fromA = pair_from_A(S, m, nd[0].mu.re, nd[1].x, nd[2].x, mid, Rp);
  double pcen = 0.0, ps = 0.0;  // centre and half-width of the pair computed from A
  bool preal = true;
  bool mu0_newton = false;
  if (fromA) {
    const double m0 = newton_real(As, nd[0].mu.re, nd[1].mu, nd[2].mu);
    nd[0].mu.re = m0;
    mu0_newton = true;
    // product pi and sum sg of the pair: pi = det As / mu0, sg = (c2 - pi) / mu0 for mu0 the largest; otherwise
    // sg = tr As - mu0, pi = c2 - mu0 sg
    const double c2 = minors_sum(As);
    double sg, pi;
    if (fabs(m0) >= fabs(mid) + Rp) {
      pi = det_elim(As) / m0;
      sg = (c2 - pi) / m0;
    } else {
      sg = As[0] + As[4] + As[8] - m0;
      pi = c2 - m0 * sg;
    }
    const double disc = 0.25 * sg * sg - pi;
    pcen = 0.5 * sg;
    ps = sqrt(fabs(disc));
    preal = disc >= 0;
    if (preal) {
      const double r1 = pcen + copysgn(ps, pcen);
      nd[1].mu = cmk(r1, 0.0);
      nd[2].mu = cmk(r1 != 0 ? pi / r1 : pcen - copysgn(ps, pcen), 0.0);
    } else {
      nd[1].mu = cmk(pcen, ps);
      nd[2].mu = cmk(pcen, -ps);
    }
  }
  // ---- log, powers: a pair whose real parts sum below zero lies near the branch cut; f jumps between its nodes, so
  // the result needs the pair's imaginary part beta itself: from the 2 x 2 block B = Q^T S Q of the deviator on the
  // complement of mu0's left eigenvector u (u^T (As - mu0 I) = 0, the longest cross product of two columns),
  // beta^2 = -(((b11 - b22) / 2)^2 + b12 b21), centre m + tr B / 2
  const bool cut = (KIND != EXP) & (nd[1].mu.re + nd[2].mu.re < 0);
  if (cut) {
    if (!mu0_newton) nd[0].mu.re = newton_real(As, nd[0].mu.re, nd[1].mu, nd[2].mu);
    const double l0 = nd[0].mu.re;
    const double c0[3] = {As[0] - l0, As[3], As[6]}, c1[3] = {As[1], As[4] - l0, As[7]}, c2[3] = {As[2], As[5], As[8] - l0};
    double u[3], nu;
    {
      double w01[3], w02[3], w12[3];
      cross3(c0, c1, w01);
      cross3(c0, c2, w02);
      cross3(c1, c2, w12);
      const double n01 = dot3(w01, w01), n02 = dot3(w02, w02), n12 = dot3(w12, w12);
      const bool t02 = n02 > n01;
      nu = t02 ? n02 : n01;
      const bool t12 = n12 > nu;
      nu = t12 ? n12 : nu;
#pragma unroll
      for (int k = 0; k < 3; k++) u[k] = t12 ? w12[k] : (t02 ? w02[k] : w01[k]);
    }
    if (nu > 0) {
      const double iu = 1.0 / sqrt(nu);
#pragma unroll
      for (int k = 0; k < 3; k++) u[k] *= iu;
      // q1: the coordinate axis least aligned with u, less its u component, normalised; q2 = u x q1
      const double b0 = fabs(u[0]), b1 = fabs(u[1]), b2 = fabs(u[2]);
      const bool y1 = b1 < b0, z2 = b2 < (y1 ? b1 : b0);
      const int ax = z2 ? 2 : (y1 ? 1 : 0);
      const double ua = ax == 0 ? u[0] : (ax == 1 ? u[1] : u[2]);
      double q1[3] = {(ax == 0 ? 1.0 : 0.0) - ua * u[0], (ax == 1 ? 1.0 : 0.0) - ua * u[1],
                      (ax == 2 ? 1.0 : 0.0) - ua * u[2]};
      const double iq = 1.0 / sqrt(dot3(q1, q1));
#pragma unroll
      for (int k = 0; k < 3; k++) q1[k] *= iq;
      double q2[3], Sq1[3], Sq2[3];
      cross3(u, q1, q2);
      matvec3(S, q1, Sq1);
      matvec3(S, q2, Sq2);
      const double b11 = dot3(q1, Sq1), b12 = dot3(q1, Sq2), b21 = dot3(q2, Sq1), b22 = dot3(q2, Sq2);
      const double hd = 0.5 * (b11 - b22), beta2 = -(hd * hd + b12 * b21), cc = m + 0.5 * (b11 + b22);
      const double bt = sqrt(fabs(beta2));
      preal = beta2 <= 0;
      nd[1].mu = preal ? cmk(cc + bt, 0.0) : cmk(cc, bt);
      nd[2].mu = preal ? cmk(cc - bt, 0.0) : cmk(cc, -bt);
      pcen = cc;
      ps = bt;
      fromA = true;
    }
  }
  if (fromA) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      nd[i].refined = true;
      nd[i].x = cmk(nd[i].mu.re - m, nd[i].mu.im);
    }
  }

  // ---- node order: the node with the largest high derivatives last (exp: the largest real part; log, powers: the
  // smallest modulus); a conjugate pair stays adjacent, the real node first when it comes first by that order or the
  // pair lies near the cut (whose large divided differences then only multiply w_2), else last
  auto key = [&](cx v) { return KIND == EXP ? v.re : (v.im == 0 ? -fabs(v.re) : -cabs_s(v)); };
  if (nd[1].x.im != 0) {
    if (!((key(nd[0].mu) <= key(nd[1].mu)) | cut)) {  // (real, pair) -> (pair, real)
      gswap(nd[0], nd[1]);
      gswap(nd[1], nd[2]);
    }
  } else {  // three real nodes: a stable sort
    if (key(nd[0].mu) > key(nd[1].mu)) gswap(nd[0], nd[1]);
    if (key(nd[1].mu) > key(nd[2].mu)) gswap(nd[1], nd[2]);
    if (key(nd[0].mu) > key(nd[1].mu)) gswap(nd[0], nd[1]);
  }

  // ---- groups: all three nodes when their radius about the mean is within reach of the series (exp: radius <= 4;
  // log, powers: radius <= rho (m + centre), centre right of the singularity), else the closest eligible pair (both
  // real or conjugate) within reach whose radius is <= 0.6 of its distance to the third node (the series' pole), else
  // none
  auto reach = [&](double c, double R) -> bool {
    if (KIND == EXP) return R <= C.rexp;
    return (m + c > 0) & (R <= C.rho_f * (m + c));
  };
  const bool cplx = nd[1].x.im != 0 || nd[0].x.im != 0;
  const double cs = (nd[0].x.re + nd[1].x.re + nd[2].x.re) / 3.0;
  double R3;
  if (!cplx) {
    R3 = tmax(tmax(fabs(nd[0].x.re - cs), fabs(nd[1].x.re - cs)), fabs(nd[2].x.re - cs));
  } else {
    const bool real_first = nd[0].x.im == 0;  // the real node first (the pair at 1, 2) or last (the pair at 0, 1)
    const cx xc = real_first ? nd[1].x : nd[0].x;
    const double rc = cabs_s(cmk(xc.re - cs, xc.im));  // (the same for both members of the pair)
    R3 = real_first ? tmax(tmax(fabs(nd[0].x.re - cs), rc), rc) : tmax(tmax(rc, rc), fabs(nd[2].x.re - cs));
  }
  const bool triple = reach(cs, R3);
  bool inG[3] = {triple, triple, triple}, pk[3] = {false, false, false};
  if (!triple) {
    double bestR = __longlong_as_double(0x7FF0000000000000ll);
    int best = -1;
#pragma unroll
    for (int pr = 0; pr < 3; pr++) {  // pairs (0, 1), (0, 2), (1, 2); the third node k is the pole
      const int i = pr == 2 ? 1 : 0, j = pr == 0 ? 1 : 2, k = 3 - i - j;
      const cx xi = nd[i].x, xj = nd[j].x, xk = nd[k].x;
      const bool both_real = (xi.im == 0) & (xj.im == 0);
      if (!(both_real | ((xi.re == xj.re) & (xi.im == -xj.im)))) continue;
      const double c = 0.5 * (xi.re + xj.re);
      const double R = both_real ? 0.5 * fabs(xi.re - xj.re) : fabs(xi.im);
      const double pole = xk.im == 0 ? fabs(c - xk.re) : cabs_s(cmk(c - xk.re, -xk.im));
      if (reach(c, R) & (R <= G_RHO_POLE * pole) & (R < bestR)) {
        bestR = R;
        best = pr;
      }
    }
    // pair (0, 1): pole node 2; (0, 2): node 1; (1, 2): node 0
#pragma unroll
    for (int q = 0; q < 3; q++) {
      pk[q] = best == 2 - q;
      inG[q] = (best >= 0) & (best != 2 - q);
    }
  }

  // ---- group centre and offsets; the pair computed from A, when it is the group, keeps its own symmetric offsets
  const int gn = (int)inG[0] + (int)inG[1] + (int)inG[2];
  double cxg = gn > 0 ? ((inG[0] ? nd[0].x.re : 0.0) + (inG[1] ? nd[1].x.re : 0.0) + (inG[2] ? nd[2].x.re : 0.0)) /
                            (double)gn : 0.0;
  double cmu = m + cxg;
  const bool own_pair = fromA & (gn == 2) & ((!inG[0] | nd[0].pairpos) & (!inG[1] | nd[1].pairpos) &
                                             (!inG[2] | nd[2].pairpos));
  if (own_pair) {
    cxg = pcen - m;
    cmu = pcen;
  }
  cx off[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    off[i] = cmk(0.0, 0.0);
    if (!inG[i]) continue;
    if (own_pair) {  // +-ps (real pair) or +-i ps (conjugate pair) about pcen, in the nodes' own order
      const bool lower = (nd[i].mu.re - pcen < 0) | (nd[i].mu.im < 0);
      const double sgn = lower ? -1.0 : 1.0;
      off[i] = preal ? cmk(sgn * ps, 0.0) : cmk(0.0, sgn * ps);
      nd[i].mu = cmk(pcen + off[i].re, off[i].im);
      nd[i].x = cmk(nd[i].mu.re - m, nd[i].mu.im);
    } else {
      off[i] = cmk(nd[i].x.re - cxg, nd[i].x.im);
    }
  }

  // ---- single real nodes far from the shift (|x| > |m| / 2): Newton on det(As - mu I)
#pragma unroll
  for (int i = 0; i < 3; i++) {
    if (inG[i] | nd[i].refined | (nd[i].x.im != 0) | !(fabs(nd[i].x.re) > 0.5 * fabs(m))) continue;
    const int j = i == 0 ? 1 : 0, k = i == 2 ? 1 : 2;
    nd[i].mu.re = newton_real(As, nd[i].mu.re, nd[j].mu, nd[k].mu);
    nd[i].refined = true;
    nd[i].x = cmk(nd[i].mu.re - m, nd[i].mu.im);
  }
  // the series' pole: the outside node of a pair group, at its distance from the centre
  const bool grp_refined = (inG[0] & nd[0].refined) | (inG[1] & nd[1].refined) | (inG[2] & nd[2].refined);
  double apole = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (pk[k]) apole = (grp_refined | nd[k].refined) ? cmu - nd[k].mu.re : cxg - nd[k].x.re;
  const double xshift = KIND == EXP ? tmax(tmax(nd[0].x.re, nd[1].x.re), nd[2].x.re) : 0.0;
  // log, powers: a real eigenvalue <= 0 lies outside the domain (NaN results)
  bool bad = false;
  if (KIND != EXP) {
#pragma unroll
    for (int i = 0; i < 3; i++) bad = bad | ((nd[i].x.im == 0) & (nd[i].mu.re <= 0));
  }

  // ---- the series variable u = offset / L (L = the group centre for log and powers), its pole, the number of terms
  const bool hasg = gn > 0;
  const double L = KIND == EXP ? 1.0 : ((hasg & (cmu > 0)) ? cmu : 1.0), iL = 1.0 / L;
  cx u[3];
#pragma unroll
  for (int i = 0; i < 3; i++) u[i] = cscl(off[i], iL);
  const double ap = fabs(apole) > 0 ? apole * iL : 1.0, iap = 1.0 / ap;
  double rr = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++) rr = tmax(rr, u[i].im == 0 ? fabs(u[i].re) : cabs_s(u[i]));
  const bool anypk = pk[0] | pk[1] | pk[2];
  const double rq = (anypk & (rr * fabs(iap) <= 1.0)) ? rr * fabs(iap) : 0.0;
  rr = (hasg & (rr <= C.rexp + 0.5)) ? rr : 0.0;
  int j1 = G_KMAX, j2 = G_KMAX;
  St.K = hasg ? nterms(C, 3 * (ORDER + 1) - 1, rr, rq, j1, j2) : 0;
  // the float-float / FP32 tail of the series: groups without a pole node, coefficients within FP32's range
  const bool tail = (C.ffser != 0) & !anypk & (rr <= 4.0);
  j1 = tail ? j1 : G_KMAX;
  j2 = tail ? j2 : G_KMAX;
  const bool real = (u[0].im == 0) & (u[1].im == 0) & (u[2].im == 0);
#pragma unroll
  for (int k = 0; k < 9; k++) St.As[k] = As[k];
  St.sig = sig; St.m = m; St.cxg = cxg; St.cmu = cmu; St.xshift = xshift; St.iap = iap; St.L = L; St.iL = iL;
  int fl = (bad ? 512 : 0) | (real ? 1024 : 0) | (j1 << 12) | (j2 << 20);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    St.x[i] = nd[i].x;
    St.mu[i] = nd[i].mu;
    St.u[i] = u[i];
    fl |= (nd[i].refined ? 1 << i : 0) | (inG[i] ? 8 << i : 0) | (pk[i] ? 64 << i : 0);
  }
  St.flags = fl;
}

// the key by which a CTA orders its matrices before gmf_finish, so that a warp's lanes do the same work: the class
// (no group: real or complex nodes; real series; complex series), longer series first, then the group's node pattern
MF_D unsigned gmf_finish_key(const GmfState &St) {
  const bool allreal = (St.x[0].im == 0) & (St.x[1].im == 0) & (St.x[2].im == 0);
  const unsigned cls = St.K == 0 ? (allreal ? 0u : 1u) : ((St.flags & 1024) ? 2u : 3u);
  return (cls << 16) | ((unsigned)(255 - St.K) << 6) | (unsigned)((St.flags >> 3) & 63);
}

template <int KIND, int ORDER>
MF_D void gmf_classify(const double *a, const GmfCoef &C, GmfState &St) {
  cx x[3];
  gmf_roots<KIND>(a, x);
  gmf_classify_from<KIND, ORDER>(a, x, C, St);
}

// ---- single nodes.  The arithmetic is real where every node is real (V = double), complex otherwise (V = cx).
MF_D double vsub(double a, double b) { return a - b; }
MF_D cx vsub(cx a, cx b) { return csub(a, b); }
MF_D double vadd(double a, double b) { return a + b; }
MF_D cx vadd(cx a, cx b) { return cadd(a, b); }
MF_D double vmul(double a, double b) { return a * b; }
MF_D cx vmul(cx a, cx b) { return cmul(a, b); }
MF_D double vscl(double a, double s) { return a * s; }
MF_D cx vscl(cx a, double s) { return cscl(a, s); }
MF_D double vinv(double a) { return 1.0 / a; }
MF_D cx vinv(cx a) { return cinv_s(a); }
MF_D void vset(double &v, cx a) { v = a.re; }
MF_D void vset(cx &v, cx a) { v = a; }
MF_D cx vcx(double a) { return cmk(a, 0.0); }
MF_D cx vcx(cx a) { return a; }
MF_D double vzero(double) { return 0.0; }
MF_D cx vzero(cx) { return cmk(0.0, 0.0); }

// Taylor coefficients t = (f, f', f''/2) at the node z (the eigenvalue of As; x = z - m, relative to the shift) of
// the function whose divided differences the kernel forms: exp e^(x - xshift) (times e^(m + xshift) at the end); log
// log(sig z), as log(sig m) + log1p(x / m) for |x| <= m / 2; powers (z / rho)^al, rho a power of two near the largest
// |node| (the blocks of output order k are multiplied by (sig rho)^(al - k) rho^k afterwards).  Real z: real
// arithmetic (z > 0 for log and powers; a real node <= 0 makes every result of the matrix NaN in any case).
template <int KIND, typename V>
MF_D void node_taylor(const GmfCoef &C, double sig, double m, double xshift, double rho, cx x, cx z, V *t) {
  if (KIND == EXP) {
    const double e = exp(x.re - xshift);
    cx f0 = cmk(e, 0.0);
    if (x.im != 0) f0 = cmk(e * cos(x.im), e * sin(x.im));
    vset(t[0], f0);
    t[1] = t[0];
    t[2] = vscl(t[0], 0.5);
    return;
  }
  V iz;
  vset(iz, z.im == 0 ? cmk(1.0 / z.re, 0.0) : cinv_s(z));
  if (KIND == LOG) {
    const double ax = x.im == 0 ? fabs(x.re) : cabs_s(x);
    cx f0;
    if ((m > 0) & (ax <= 0.5 * m)) {  // near the shift: log(sig m) + log1p(x / m)
      const double zr = x.re / m, zi = x.im / m;
      f0 = cmk(log(sig * m) + 0.5 * log1p(zr * (2.0 + zr) + zi * zi), x.im == 0 ? 0.0 : atan2(zi, 1.0 + zr));
    } else {
      f0 = z.im == 0 ? cmk(log(sig * fabs(z.re)), atan2(0.0, z.re)) : cmk(log(sig * cabs_s(z)), atan2(z.im, z.re));
    }
    vset(t[0], f0);
    t[1] = iz;
    t[2] = vscl(vmul(iz, iz), -0.5);
    return;
  }
  cx f0;
  if (z.im == 0) {
    f0 = cmk(pow_split(fabs(z.re) / rho, C.bh[0], C.bl[0]), 0.0);
  } else {
    const double mag = pow_split(cabs_s(z) / rho, C.bh[0], C.bl[0]), ph = C.al * atan2(z.im, z.re);
    f0 = cmk(mag * cos(ph), mag * sin(ph));
  }
  vset(t[0], f0);
  t[1] = vscl(vmul(t[0], iz), C.al);
  t[2] = vscl(vmul(t[1], iz), 0.5 * (C.al - 1.0));
}

// the difference of nodes p and q: between the refined eigenvalues where either was refined against A, else between
// the deviator's roots
template <typename V>
MF_D V node_diff(const cx *x, const cx *mu, const bool *ab, int p, int q) {
  V d;
  vset(d, (ab[p] | ab[q]) ? csub(mu[p], mu[q]) : csub(x[p], x[q]));
  return d;
}

// No group (three single nodes, pairwise apart): the divided differences over multiplicity vectors (a, b, c), each at
// most ORDER + 1, by the Hermite recursion
//   f[z0^a z1^b z2^c] = (f[N - z_q] - f[N - z_p]) / (z_p - z_q),   p < q the first two nodes with nonzero multiplicity
// from f[z^k] = f^(k-1)(z) / (k-1)!: 54 steps of one difference and one product at order 2.
template <int KIND, int ORDER, typename V>
MF_D void dd_three_single(const GmfCoef &C, double sig, double m, double xshift, double rho, const cx *x,
                          const cx *mu, const bool *ab, const double *bs, cx *D) {
  constexpr int M = ORDER + 1, ND = ORDER == 0 ? 3 : (ORDER == 1 ? 9 : 19);
  V t[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++) node_taylor<KIND, V>(C, sig, m, xshift, rho, x[i], mu[i], t[i]);
  const V i01 = vinv(node_diff<V>(x, mu, ab, 0, 1)), i02 = vinv(node_diff<V>(x, mu, ab, 0, 2)),
          i12 = vinv(node_diff<V>(x, mu, ab, 1, 2));
  V G[M + 1][M + 1][M + 1];
#pragma unroll
  for (int k = 1; k <= M; k++) {
    G[k][0][0] = t[0][k - 1];
    G[0][k][0] = t[1][k - 1];
    G[0][0][k] = t[2][k - 1];
  }
#pragma unroll
  for (int s = 2; s <= 3 * M; s++)
#pragma unroll
    for (int a = 0; a <= M; a++)
#pragma unroll
      for (int b = 0; b <= M; b++) {
        const int c = s - a - b;
        if (c < 0 || c > M || (int)(a > 0) + (int)(b > 0) + (int)(c > 0) < 2) continue;
        if (a > 0 && b > 0) {         // nodes 0, 1
          G[a][b][c] = vmul(vsub(G[a][b - 1][c], G[a - 1][b][c]), i01);
        } else if (a > 0) {           // nodes 0, 2
          G[a][b][c] = vmul(vsub(G[a][b][c - 1], G[a - 1][b][c]), i02);
        } else {                      // nodes 1, 2
          G[a][b][c] = vmul(vsub(G[a][b][c - 1], G[a][b - 1][c]), i12);
        }
      }
#pragma unroll
  for (int e = 0; e < ND; e++) D[e] = cscl(vcx(G[gms(e, 0)][gms(e, 1)][gms(e, 2)]), bs[gms(e, 0) - 1]);
}

// Beside a pair group: the residue of the single node I, the coefficient of tau^(m_I - 1) in
// f(z_I + tau) prod_(z != I) (z_I - z + tau)^(-m_z), with (d + tau)^(-n) = d^(-n) (1 - n tau / d + n (n+1) / 2 tau^2 / d^2
// - ...), added to each entry with m_I > 0
template <int KIND, int ORDER, typename V, int I>
MF_D void dd_residue(const GmfCoef &C, double sig, double m, double xshift, double rho, const cx *x, const cx *mu,
                     const bool *ab, const double *bs, cx *D) {
  constexpr int ND = ORDER == 0 ? 3 : (ORDER == 1 ? 9 : 19);
  constexpr int A = I == 0 ? 1 : 0, B = I == 2 ? 1 : 2;  // the other two nodes
  V t[3];
  node_taylor<KIND, V>(C, sig, m, xshift, rho, x[I], mu[I], t);
  V wa[ORDER + 4], wb[ORDER + 4];  // powers 0 .. ORDER + 3 of 1 / (z_I - z_A), 1 / (z_I - z_B)
  wa[1] = vinv(node_diff<V>(x, mu, ab, I, A));
  wb[1] = vinv(node_diff<V>(x, mu, ab, I, B));
  vset(wa[0], cmk(1.0, 0.0));
  wb[0] = wa[0];
#pragma unroll
  for (int e = 2; e < ORDER + 4; e++) { wa[e] = vmul(wa[e - 1], wa[1]); wb[e] = vmul(wb[e - 1], wb[1]); }
#pragma unroll
  for (int e = 0; e < ND; e++) {
    const int mi = gms(e, I), ma = gms(e, A), mb = gms(e, B);
    if (mi == 0) continue;
    // coefficients of the two expansions up to tau^(mi - 1)
    V pa[3], pb[3];
#pragma unroll
    for (int k = 0; k < mi; k++) {
      const double ca = k == 0 ? 1.0 : (k == 1 ? -(double)ma : 0.5 * ma * (ma + 1));
      const double cb = k == 0 ? 1.0 : (k == 1 ? -(double)mb : 0.5 * mb * (mb + 1));
      pa[k] = ma == 0 ? (k == 0 ? wa[0] : vzero(wa[0])) : vscl(wa[ma + k], ca);
      pb[k] = mb == 0 ? (k == 0 ? wb[0] : vzero(wb[0])) : vscl(wb[mb + k], cb);
    }
    V r = vzero(t[0]);
#pragma unroll
    for (int j = 0; j < mi; j++) {  // t_j * (pa pb)_(mi - 1 - j)
      const int d = mi - 1 - j;
      V q = vzero(t[0]);
#pragma unroll
      for (int k = 0; k <= d; k++) {
        if (ma == 0 && k > 0) continue;
        if (mb == 0 && d - k > 0) continue;
        q = vadd(q, ma == 0 ? pb[d - k] : (mb == 0 ? pa[k] : vmul(pa[k], pb[d - k])));
      }
      r = vadd(r, vmul(t[j], q));
    }
    D[e] = cadd(D[e], cscl(vcx(r), bs[gms(e, 0) - 1]));
  }
}

// the second half: divided differences (series, residues), real basis, F and the reduced D2', D3'
template <int KIND, int ORDER, bool FF = false>
MF_D void gmf_finish(const GmfState &St, const GmfCoef &C, GmfRec &R) {
  constexpr int ND = ORDER == 0 ? 3 : (ORDER == 1 ? 9 : 19);
  double As[9], S[9];
#pragma unroll
  for (int k = 0; k < 9; k++) As[k] = St.As[k];
  const double sig = St.sig, isig = 1.0 / sig, m = St.m, cxg = St.cxg, cmu = St.cmu, xshift = St.xshift;
  const double iap = St.iap, L = St.L, iL = St.iL;
#pragma unroll
  for (int k = 0; k < 9; k++) S[k] = k % 4 == 0 ? As[k] - m : As[k];
  cx x[3], mu[3], u[3];
#pragma unroll
  for (int i = 0; i < 3; i++) { x[i] = St.x[i]; mu[i] = St.mu[i]; u[i] = St.u[i]; }
  const int fl = St.flags;
  bool ab[3] = {(fl & 1) != 0, (fl & 2) != 0, (fl & 4) != 0};
  bool inG[3] = {(fl & 8) != 0, (fl & 16) != 0, (fl & 32) != 0};
  bool pk[3] = {(fl & 64) != 0, (fl & 128) != 0, (fl & 256) != 0};
  const bool bad = (fl & 512) != 0, hasg = St.K > 0;
  double b0 = 1.0;
  if (KIND == LOG) b0 = log_b0(sig, m, cxg, cmu);
  cx D[ND];
#pragma unroll
  for (int c = 0; c < ND; c++) D[c] = cmk(0.0, 0.0);
  if (hasg) {
    const bool real = (fl & 1024) != 0;
    const unsigned am = __activemask();
    // FP32 storage: the whole series in float-float where coefficients, offsets and pole factor fit FP32's range
    const double aiap = fabs(iap);
    const int e = aiap > 1.0 ? (int)((__double_as_longlong(aiap) >> 52) & 0x7FF) - 1022 : 0;
    const bool ffok = FF & (KIND != EXP) & (C.ffser != 0) & (aiap < 256.0) & (fabs(b0) < 1e30) &
                      (cabs_s(u[0]) <= 4.0) & (cabs_s(u[1]) <= 4.0) & (cabs_s(u[2]) <= 4.0);
    if (FF && KIND != EXP && __all_sync(am, ffok)) {
      if (__all_sync(am, real)) group_series_ff<ND, true>(St.K, b0, C, inG, pk, u, iap, e, D);
      else group_series_ff<ND, false>(St.K, b0, C, inG, pk, u, iap, e, D);
    } else {
      // FP64 leading terms, float-float / FP32 tail from this matrix's own split points (so that its result does
      // not depend on the matrices beside it in the warp)
      const int j1 = (fl >> 12) & 255, j2 = (fl >> 20) & 255;
      if (__all_sync(am, real)) group_series<ND, true>(St.K, b0, C, inG, pk, u, iap, D, j1, j2);
      else group_series<ND, false>(St.K, b0, C, inG, pk, u, iap, D, j1, j2);
    }
#pragma unroll
    for (int c = 0; c < ND; c++) {
      const int nn = gms(c, 0) + gms(c, 1) + gms(c, 2) - 1, k = gms(c, 0) - 1;
      double fac;
      if (KIND == EXP) {
        fac = exp(cxg - xshift);
      } else {
        double iLn = 1.0;
#pragma unroll
        for (int r = 0; r < nn - (KIND == POW ? k : 0); r++) iLn = iLn * iL;
        fac = KIND == LOG ? iLn : pow_split(sig * L, C.bh[k], C.bl[k]) * iLn;
      }
      D[c] = cscl(D[c], fac);
    }
  }
  // ---- single nodes: with no group the divided differences of all three by the Hermite recursion, beside a pair
  // group the residue of the one outside node; powers rescaled per output order (node_taylor)
  const double rho = KIND == POW ? pow2safe(tmax(tmax(cabs_s(mu[0]), cabs_s(mu[1])), cabs_s(mu[2]))) : 1.0;
  double bs[3] = {1.0, 1.0, 1.0};  // the scale of each output order's block
  if (KIND == POW) {
#pragma unroll
    for (int k = 0; k <= ORDER; k++) bs[k] = pow_split(sig * rho, C.bh[k], C.bl[k]) * (k == 0 ? 1.0 : (k == 1 ? rho : rho * rho));
  }
  const bool allreal = (x[0].im == 0) & (x[1].im == 0) & (x[2].im == 0);
  if (!hasg) {
    if (allreal) dd_three_single<KIND, ORDER, double>(C, sig, m, xshift, rho, x, mu, ab, bs, D);
    else dd_three_single<KIND, ORDER, cx>(C, sig, m, xshift, rho, x, mu, ab, bs, D);
  } else {
    // (a pair group leaves one single node)
    if (allreal) {
      if (!inG[0]) dd_residue<KIND, ORDER, double, 0>(C, sig, m, xshift, rho, x, mu, ab, bs, D);
      else if (!inG[1]) dd_residue<KIND, ORDER, double, 1>(C, sig, m, xshift, rho, x, mu, ab, bs, D);
      else if (!inG[2]) dd_residue<KIND, ORDER, double, 2>(C, sig, m, xshift, rho, x, mu, ab, bs, D);
    } else {
      if (!inG[0]) dd_residue<KIND, ORDER, cx, 0>(C, sig, m, xshift, rho, x, mu, ab, bs, D);
      else if (!inG[1]) dd_residue<KIND, ORDER, cx, 1>(C, sig, m, xshift, rho, x, mu, ab, bs, D);
      else if (!inG[2]) dd_residue<KIND, ORDER, cx, 2>(C, sig, m, xshift, rho, x, mu, ab, bs, D);
    }
  }

  // ---- real basis and T = I + iN (gmf_kernel.hpp:578-599)
  double b0i = x[0].im, b1i = x[1].im;
  double B1[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const bool dg = k % 4 == 0;
    R.r1[k] = dg ? sel(ab[0], As[k] - mu[0].re, S[k] - x[0].re) : S[k];
    B1[k] = dg ? sel(ab[1], As[k] - mu[1].re, S[k] - x[1].re) : S[k];
  }
#pragma unroll
  for (int i2 = 0; i2 < 3; i2++)
#pragma unroll
    for (int j2 = 0; j2 < 3; j2++)
      R.r2[3 * i2 + j2] = R.r1[3 * i2] * B1[j2] + R.r1[3 * i2 + 1] * B1[3 + j2] + R.r1[3 * i2 + 2] * B1[6 + j2] -
                          (i2 == j2 ? b0i * b1i : 0.0);
  double a01 = sel(ab[0] | ab[1], mu[0].re - mu[1].re, x[0].re - x[1].re);
  double N10 = -b0i, N20 = -b0i * a01, N21 = -(b0i + b1i);
  double nanf = sel(bad, __longlong_as_double(0x7FF8000000000000ll), 1.0);
  {  // F = sum_m Re(T^T D)_m r_m
    double Dr0 = D[0].re - (N10 * D[1].im + N20 * D[2].im), Dr1 = D[1].re - N21 * D[2].im, Dr2 = D[2].re;
    double e = KIND == EXP ? exp(m + xshift) : 1.0;
#pragma unroll
    for (int k = 0; k < 9; k++)
      R.F[k] = ((k % 4 == 0 ? Dr0 : 0.0) + Dr1 * R.r1[k] + Dr2 * R.r2[k]) * e * nanf;
  }
  if (ORDER < 1) return;
  R.sc1 = (KIND == EXP ? exp(m + xshift) : (KIND == LOG ? isig : 1.0)) * nanf;
  {  // D2' = Re(T^T D T): T on index 0 (complex), then the real part after T on index 1
    double Dr[9], Di[9];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) { Dr[3 * j + k] = D[gpos2(j, k)].re; Di[3 * j + k] = D[gpos2(j, k)].im; }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      double vr0 = Dr[k], vr1 = Dr[3 + k], vr2 = Dr[6 + k], vi0 = Di[k], vi1 = Di[3 + k], vi2 = Di[6 + k];
      Dr[k] = vr0 - (N10 * vi1 + N20 * vi2); Di[k] = vi0 + (N10 * vr1 + N20 * vr2);
      Dr[3 + k] = vr1 - N21 * vi2;           Di[3 + k] = vi1 + N21 * vr2;
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Dr[3 * j] = Dr[3 * j] - (N10 * Di[3 * j + 1] + N20 * Di[3 * j + 2]);
      Dr[3 * j + 1] = Dr[3 * j + 1] - N21 * Di[3 * j + 2];
    }
    R.D2[0] = Dr[0]; R.D2[1] = Dr[4]; R.D2[2] = Dr[8]; R.D2[3] = Dr[1]; R.D2[4] = Dr[2]; R.D2[5] = Dr[5];
  }
  if (ORDER < 2) return;
  R.sc2 = (KIND == EXP ? exp(m + xshift) : (KIND == LOG ? isig * isig : 1.0)) * nanf;
  {  // D3': T on each of the three indices, real part
    double Dr[27], Di[27];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = 0; l < 3; l++) {
          Dr[9 * j + 3 * k + l] = D[gpos3(j, k, l)].re;
          Di[9 * j + 3 * k + l] = D[gpos3(j, k, l)].im;
        }
#pragma unroll
    for (int axis = 0; axis < 3; axis++) {
      const int s = axis == 0 ? 9 : (axis == 1 ? 3 : 1);
#pragma unroll
      for (int base = 0; base < 27; base++) {
        if ((base / s) % 3 != 0) continue;
        double vr0 = Dr[base], vr1 = Dr[base + s], vr2 = Dr[base + 2 * s];
        double vi0 = Di[base], vi1 = Di[base + s], vi2 = Di[base + 2 * s];
        Dr[base] = vr0 - (N10 * vi1 + N20 * vi2); Di[base] = vi0 + (N10 * vr1 + N20 * vr2);
        Dr[base + s] = vr1 - N21 * vi2;           Di[base + s] = vi1 + N21 * vr2;
      }
    }
#pragma unroll
    for (int z = 0; z < 3; z++)
#pragma unroll
      for (int y = 0; y <= z; y++)
#pragma unroll
        for (int xx = 0; xx <= y; xx++) R.D3[sym3(xx, y, z)] = Dr[9 * xx + 3 * y + z];
  }
}

template <int KIND, int ORDER>
MF_D void gmf_record(const double *a, const GmfCoef &C, GmfRec &R) {
  GmfState St;
  gmf_classify<KIND, ORDER>(a, C, St);
  gmf_finish<KIND, ORDER>(St, C, R);
}

}  // namespace mf
