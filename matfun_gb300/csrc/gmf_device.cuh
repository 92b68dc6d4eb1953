// gmf_device.cuh -- per-matrix device math of the general family (FP64, one thread per matrix).
// Algorithm of c/include/matfun/gmf_kernel.hpp:251-692 (theory: confluent Newton-Hermite form over the eigenvalues):
//   * eigenvalues of the deviator in closed form, refined against A itself where the closed form loses accuracy
//     (Newton on det(A - mu I), a pair from det A and the principal minors, the branch-cut pair from the 2x2 block
//     on the complement of the left eigenvector)
//   * node order, groups (triple / closest pair / none), the 19 confluent divided differences by the streamed group
//     series and the residues of single nodes
//   * the real basis r_0 = I, r_1, r_2 and T = I + iN, giving F and the real-reduced divided differences
//     D2' = Re(T^T D T) (symmetric, 6 distinct) and D3' (T on all three indices; symmetric, 10 distinct).
// Same branch thresholds and the same evaluation order of the series as the reference.  The kernels then contract
// D2' and D3' with r into J and H through symmetric tensors (gmf_kernels.cu).
// Written with sel() and non-short-circuit &, | (see mf_common.cuh) instead of long ?: / && chains.
#pragma once
#include "ffloat.cuh"

namespace mf {

constexpr double G_RHO = 0.7, G_R_EXP = 4.0, G_RHO_POLE = 0.6;  // gmf_kernel.hpp:30
constexpr int G_KMAX = 200;                                      // gmf_kernel.hpp:31

// launch constants of the gmf kernels (host-computed once per call)
struct GmfCoef {
  double al;              // exponent (pow; sqrt arrives as pow 0.5), 0 otherwise
  double rho_f;           // group radius ratio: 0.7, or min(0.7, 3 / al) for pow
  double bh[3], bl[3];    // al - k split exactly (k = 0, 1, 2)
  double bt[G_KMAX];      // series coefficients b_j of f(c (1 + u)) (gmf_kernel.hpp:48-53)
  float lterm[G_KMAX];    // log2(|b_(n+k)| C(k + n, n)), n = 3 (order + 1) - 1: the term bound of gmf_kernel.hpp:73-97
  float bth[G_KMAX], btl[G_KMAX];  // bt as float-float (hi + lo)
  int ffser;              // 1: the group series may run on the FP32 pipe (every |bth[j]| <= 2^100)
  int tsh;                // bth, btl hold b_j 2^(tsh j) and group_tail takes the offsets times 2^-tsh (exp: 2, so
                          // that 4^j / j! stays in FP32's range; log, pow: 0)
};

// host: launch constants (series coefficients gmf_kernel.hpp:48-53; the binomial factors of the term bound by the
// recurrence of gmf_kernel.hpp:84, as log2 values)
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

MF_D double det3(const double *M) {
  return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) + M[2] * (M[3] * M[7] - M[4] * M[6]);
}

// det by elimination with partial pivoting (gmf_kernel.hpp:138-159)
MF_D double det_lu(const double *M) {
  double a0 = fabs(M[0]), a1 = fabs(M[3]), a2 = fabs(M[6]);
  bool p1 = (a1 > a0) & (a1 >= a2), p2 = (a2 > a0) & (a2 > a1);
  double P[3], R1[3], R2[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    P[c] = sel(p1, M[3 + c], sel(p2, M[6 + c], M[c]));
    R1[c] = sel(p1 | p2, M[c], M[3 + c]);
    R2[c] = sel(p2, M[3 + c], M[6 + c]);
  }
  double sgn = sel(p1, -1.0, 1.0);
  double piv = sel(P[0] != 0, P[0], 1.0);
  double l1 = R1[0] / piv, l2 = R2[0] / piv;
  double b = R1[1] - l1 * P[1], c = R1[2] - l1 * P[2], d = R2[1] - l2 * P[1], e = R2[2] - l2 * P[2];
  bool sw = fabs(d) > fabs(b);
  double bb = sel(sw, d, b), cc = sel(sw, e, c), dd = sel(sw, b, d), ee = sel(sw, c, e);
  sgn = sel(sw, -sgn, sgn);
  double det = sgn * P[0] * bb * (ee - dd / sel(bb != 0, bb, 1.0) * cc);
  return sel((P[0] != 0) & (bb != 0), det, 0.0);
}

MF_D double minors2(const double *M) {
  return M[0] * M[4] - M[1] * M[3] + M[0] * M[8] - M[2] * M[6] + M[4] * M[8] - M[5] * M[7];
}

// eigenvalues of the deviator S (gmf_kernel.hpp:166-208)
MF_D void roots3(const double *S, cx *x) {
  constexpr double TWO_PI_3 = 2.0943951023931957;
  double tau = (S[0] + S[4] + S[8]) / 3.0;
  double Sp[9];
#pragma unroll
  for (int k = 0; k < 9; k++) Sp[k] = k % 4 == 0 ? S[k] - tau : S[k];
  double s = fabs(Sp[0]);
#pragma unroll
  for (int k = 1; k < 9; k++) s = tmax(s, fabs(Sp[k]));
  double t = pow2safe(s), it = 1.0 / t;
#pragma unroll
  for (int k = 0; k < 9; k++) Sp[k] = Sp[k] * it;
  double P = 0.5 * (Sp[0] * Sp[0] + Sp[4] * Sp[4] + Sp[8] * Sp[8]) + Sp[1] * Sp[3] + Sp[2] * Sp[6] + Sp[5] * Sp[7];
  double Q = det3(Sp);
  double u = pow2safe(tmax(sqrt(fabs(P)), cbrt(fabs(Q)))), iu = 1.0 / u;
  P = P * iu * iu;
  Q = Q * iu * iu * iu;
  t = t * u;
  bool trig = (P > 0) & (4.0 * P * P * P >= 27.0 * Q * Q);
  double s1;
  if (trig) {
    double p3 = P / 3.0;
    double r = 0.5 * Q / (p3 * sqrt(p3));
    r = sel(r > 1.0, 1.0, sel(r < -1.0, -1.0, r));
    double ph = acos(r) / 3.0;
    s1 = 2.0 * sqrt(p3) * cos(sel(r >= 0, ph, ph + TWO_PI_3));
  } else {
    double D = 0.25 * Q * Q - P * P * P / 27.0;
    double uc = cbrt(0.5 * Q + copysgn(sqrt(sel(D > 0, D, 0.0)), Q));
    s1 = uc + sel(uc != 0, P / (3.0 * sel(uc != 0, uc, 1.0)), 0.0);
  }
  double d = P - 0.75 * s1 * s1;
  bool real = d >= 0;
  double sq = sqrt(fabs(d));
  double sa = -0.5 * s1 - copysgn(sq, s1);
  double prod = sel(s1 != 0, Q / sel(s1 != 0, s1, 1.0), -P);
  double sb = sel(sa != 0, prod / sel(sa != 0, sa, 1.0), 0.0);
  double im = sel(real, 0.0, sq) * t;
  x[0] = cmk(s1 * t + tau, 0.0 * t);
  x[1] = cmk(sel(real, sa, -0.5 * s1) * t + tau, im);
  x[2] = cmk(sel(real, sb, -0.5 * s1) * t + tau, -im);
}

// 3 Newton steps on det(A - mu_j I), derivative from the other nodes (gmf_kernel.hpp:210-226)
template <int J>
MF_D void newton(const double *As, cx *mu) {
#pragma unroll
  for (int it = 0; it < 3; it++) {
    cx den = cmk(1.0, 0.0);
#pragma unroll
    for (int k = 0; k < 3; k++)
      if (k != J) den = cmul(den, csub(mu[k], mu[J]));
    bool ok = (den.re != 0) | (den.im != 0);
    double B[9];
#pragma unroll
    for (int k = 0; k < 9; k++) B[k] = k % 4 == 0 ? As[k] - mu[J].re : As[k];
    double step = det_lu(B) * cinv_s(den).re;
    mu[J].re = sel(ok, mu[J].re + step, mu[J].re);
  }
}

// f of a node (k: output order; pow times sig^(al - k)) (gmf_kernel.hpp:228-248)
template <int KIND>
MF_D cx coef0(const GmfCoef &C, double sig, double m, cx x, cx mu, int k) {
  if (KIND == EXP) {
    double e = exp(x.re);
    return cmk(e * cos(x.im), e * sin(x.im));
  }
  double th = atan2(mu.im, mu.re);
  if (KIND == LOG) {
    bool near = (m > 0) & (cabs_s(x) <= 0.5 * m);
    double ms = sel(m > 0, m, 1.0), zr = x.re / ms, zi = x.im / ms;
    double l1r = 0.5 * log1p(zr * (2.0 + zr) + zi * zi), l1i = atan2(zi, 1.0 + zr);
    double lr = near ? log(sig * ms) + l1r : log(sig * cabs_s(mu));
    return cmk(lr, sel(near, l1i, th));
  }
  double mag = pow_split(sig * cabs_s(mu), C.bh[k], C.bl[k]);
  double ph = (C.al - k) * th;
  cx out = cmk(mag * cos(ph), mag * sin(ph));
  for (int i = 0; i < k; i++) out = cmul(out, mu);
  return out;
}

// number of series terms (gmf_kernel.hpp:73-97): the group series needs terms until |b_(n+k)| C(k+n, n) r^k drops
// below 1e-17 of the largest, the pole series until C(k+2, 2) q^k <= 1e-17.  Evaluated on log2 values in FP32 (the
// FP64 pipe is the bottleneck of this kernel) with a threshold 2^-0.05 below 1e-17, so that the count is never
// smaller than the FP64 bound's; one term more changes a result by less than 1e-17 relative.
//
// Also the term indices j1, j2 from which on every term is 2^-6 (j1) and 2^-30 (j2) below the largest term bound (the
// bound is unimodal in k): group_series sums the terms from j1 on in float-float and from j2 on in FP32, whose
// rounding errors (2^-48 and 2^-24 of the term) then stay below 2^-54 of the largest term, under the FP64 rounding of
// the leading terms (2^-53 of the largest).
MF_D int nterms(const GmfCoef &C, int n, double r, double q, int &j1, int &j2) {
  constexpr float L17 = -56.5237f - 0.05f;  // log2(1e-17) less a margin
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
  ffl Er[ND], Ei[ND], Fr[ND], Fi[ND], Sr[ND], Si[ND];
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
    for (int c = 0; c < ND; c++) {
      const int par = gpar(c), i = gnode(c);
      ffl eppr = par < 0 ? zero : Er[par < 0 ? 0 : par];
      ffl epcr = par < 0 ? zero : Fr[par < 0 ? 0 : par];
      if (REAL) {
        Fr[c] = ff_sel(inG[i], ff_add_s(eppr, ff_prod(ur[i], Er[c])), epcr);
        acc_ff_add(Sr[c], ff_prod(Fr[c], bj));
      } else {
        ffl eppi = par < 0 ? zero : Ei[par < 0 ? 0 : par];
        ffl epci = par < 0 ? zero : Fi[par < 0 ? 0 : par];
        ffl tr = ff_add3(eppr, ff_prod(ur[i], Er[c]), ff_neg(ff_prod(ui[i], Ei[c])));
        ffl ti = ff_add3(eppi, ff_prod(ur[i], Ei[c]), ff_prod(ui[i], Er[c]));
        Fr[c] = ff_sel(inG[i], tr, epcr);
        Fi[c] = ff_sel(inG[i], ti, epci);
        acc_ff_add(Sr[c], ff_prod(Fr[c], bj));
        acc_ff_add(Si[c], ff_prod(Fi[c], bj));
      }
    }
#pragma unroll
    for (int c = 0; c < ND; c++) {
      Er[c] = Fr[c];
      if (!REAL) Ei[c] = Fi[c];
    }
  }
  float er[ND], ei[ND], fr[ND], fi[ND], sr[ND], si[ND], vr[3], vi[3];
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
    for (int c = 0; c < ND; c++) {
      const int par = gpar(c), i = gnode(c);
      float eppr = par < 0 ? 0.f : er[par < 0 ? 0 : par], epcr = par < 0 ? 0.f : fr[par < 0 ? 0 : par];
      if (REAL) {
        fr[c] = inG[i] ? fmaf(vr[i], er[c], eppr) : epcr;
        sr[c] = fmaf(fr[c], bj, sr[c]);
      } else {
        float eppi = par < 0 ? 0.f : ei[par < 0 ? 0 : par], epci = par < 0 ? 0.f : fi[par < 0 ? 0 : par];
        float tr = fmaf(-vi[i], ei[c], fmaf(vr[i], er[c], eppr)), ti = fmaf(vi[i], er[c], fmaf(vr[i], ei[c], eppi));
        fr[c] = inG[i] ? tr : epcr;
        fi[c] = inG[i] ? ti : epci;
        sr[c] = fmaf(fr[c], bj, sr[c]);
        si[c] = fmaf(fi[c], bj, si[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < ND; c++) {
      er[c] = fr[c];
      if (!REAL) ei[c] = fi[c];
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
template <int ND, bool REAL>
MF_D void group_series(int K, double b0, const GmfCoef &C, const bool *inG, const bool *pk, const cx *u, double iap,
                       cx *D, int j1 = G_KMAX, int j2 = G_KMAX) {
  cx Ep[ND], Ec[ND];
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
    for (int c = 0; c < ND; c++) {
      const int par = gpar(c), i = gnode(c);
      cx epp = par < 0 ? cmk(sel(j == 0, 1.0, 0.0), 0.0) : Ep[par < 0 ? 0 : par];
      cx epc = par < 0 ? cmk(0.0, 0.0) : Ec[par < 0 ? 0 : par];
      double g = sel(pk[0], qv[gms(c, 0)], sel(pk[1], qv[gms(c, 1)], sel(pk[2], qv[gms(c, 2)], qv[0])));
      if (REAL) {
        Ec[c].re = sel(inG[i], epp.re + u[i].re * Ep[c].re, epc.re);
        Ec[c].im = 0.0;
        D[c].re = D[c].re + Ec[c].re * g;
      } else {
        Ec[c] = csel(inG[i], cadd(epp, cmul(u[i], Ep[c])), epc);
        D[c] = cadd(D[c], cscl(Ec[c], g));
      }
    }
#pragma unroll
    for (int c = 0; c < ND; c++) Ep[c] = Ec[c];
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
  ffl Epr[ND], Epi[ND], Ecr[ND], Eci[ND], Dr[ND], Di[ND];
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
    for (int c = 0; c < ND; c++) {
      const int par = gpar(c), i = gnode(c);
      ffl eppr = par < 0 ? ff_sel(j == 0, one, zero) : Epr[par < 0 ? 0 : par];
      ffl epcr = par < 0 ? zero : Ecr[par < 0 ? 0 : par];
      ffl g = ff_sel(pk[0], qv[gms(c, 0)], ff_sel(pk[1], qv[gms(c, 1)], ff_sel(pk[2], qv[gms(c, 2)], qv[0])));
      if (REAL) {
        Ecr[c] = ff_sel(inG[i], ff_add_s(eppr, ff_prod(ur[i], Epr[c])), epcr);
        acc_ff_add(Dr[c], ff_prod(Ecr[c], g));
      } else {
        ffl eppi = par < 0 ? zero : Epi[par < 0 ? 0 : par];
        ffl epci = par < 0 ? zero : Eci[par < 0 ? 0 : par];
        ffl tr = ff_add3(eppr, ff_prod(ur[i], Epr[c]), ff_neg(ff_prod(ui[i], Epi[c])));
        ffl ti = ff_add3(eppi, ff_prod(ur[i], Epi[c]), ff_prod(ui[i], Epr[c]));
        Ecr[c] = ff_sel(inG[i], tr, epcr);
        Eci[c] = ff_sel(inG[i], ti, epci);
        acc_ff_add(Dr[c], ff_prod(Ecr[c], g));
        acc_ff_add(Di[c], ff_prod(Eci[c], g));
      }
    }
#pragma unroll
    for (int c = 0; c < ND; c++) {
      Epr[c] = Ecr[c];
      if (!REAL) Epi[c] = Eci[c];
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

// scaling by a power of two (exp: none), shift m, deviator S (gmf_kernel.hpp:262-275)
template <int KIND>
MF_D void gmf_scale(const double *a, double &sig, double *As, double &m, double *S) {
  double amax = fabs(a[0]);
#pragma unroll
  for (int k = 1; k < 9; k++) amax = tmax(amax, fabs(a[k]));
  sig = KIND == EXP ? 1.0 : pow2safe(amax);
  const double isig = 1.0 / sig;
#pragma unroll
  for (int k = 0; k < 9; k++) As[k] = a[k] * isig;
  m = (As[0] + As[4] + As[8]) / 3.0;
#pragma unroll
  for (int k = 0; k < 9; k++) S[k] = k % 4 == 0 ? As[k] - m : As[k];
}

// the pair-refinement test (gmf_kernel.hpp:277-284)
MF_D bool gmf_pair_check(const double *S, double m, const cx *mu, double &mid, double &Rp) {
  double smax = fabs(S[0]);
#pragma unroll
  for (int k = 1; k < 9; k++) smax = tmax(smax, fabs(S[k]));
  mid = 0.5 * (mu[1].re + mu[2].re);
  Rp = 0.5 * cabs_s(csub(mu[1], mu[2]));
  bool small = fabs(mid) + Rp <= 0.25 * fabs(mu[0].re);
  bool aniso = (fabs(m) <= smax) & (Rp <= 0.25 * fabs(mid - mu[0].re));
  return (mu[0].re != 0) & (small | aniso);
}

// first part of the spectral analysis: the closed-form roots x of the deviator, and a key of the branches the rest
// takes (complex pair, pair refinement, branch-cut pair), so that a CTA can order its matrices by it before the rest
template <int KIND>
MF_D unsigned gmf_roots(const double *a, cx *x) {
  double sig, As[9], m, S[9];
  gmf_scale<KIND>(a, sig, As, m, S);
  roots3(S, x);
  cx mu[3];
#pragma unroll
  for (int i = 0; i < 3; i++) mu[i] = cmk(m + x[i].re, x[i].im);
  double mid, Rp;
  const bool pc = gmf_pair_check(S, m, mu, mid, Rp);
  const bool cut = (KIND != EXP) & (mu[1].re + mu[2].re < 0);
  const bool cplx = (x[0].im != 0) | (x[1].im != 0) | (x[2].im != 0);
  // geometry bucket (16 levels): the argument of the complex pair, or the spread of three real roots relative to their
  // mean; neighbours in it take the same groups, Newton steps and series lengths in the rest
  const int ip = x[1].im != 0 ? 1 : (x[2].im != 0 ? 2 : 0);
  const cx mp = mu[ip];
  const float argp = fabsf(atan2f((float)mp.im, (float)mp.re)) * (16.0f / 3.1415927f);
  const float spread = (float)((tmax(tmax(x[0].re, x[1].re), x[2].re) - tmin(tmin(x[0].re, x[1].re), x[2].re)) /
                               tmax(fabs(m), 1e-300)) * 8.0f;
  const unsigned geo = (unsigned)fminf(cplx ? argp : spread, 15.0f);
  return (cplx ? 128u : 0u) | (pc ? 64u : 0u) | (cut ? 32u : 0u) | geo;
}

// the rest of the spectral analysis, from the roots x of gmf_roots
template <int KIND, int ORDER>
MF_D void gmf_classify_from(const double *a, const cx *xr, const GmfCoef &C, GmfState &St) {
  double sig, As[9], m, S[9];
  gmf_scale<KIND>(a, sig, As, m, S);
  cx x[3], mu[3];
#pragma unroll
  for (int i = 0; i < 3; i++) { x[i] = xr[i]; mu[i] = cmk(m + x[i].re, x[i].im); }

  // ---- pair refinement (gmf_kernel.hpp:277-304)
  double mid, Rp;
  bool pc = gmf_pair_check(S, m, mu, mid, Rp);
  double pcen = 0.0, ps = 0.0;
  bool preal = true;
  if (pc) {
    newton<0>(As, mu);
    double m0 = mu[0].re;
    bool big = fabs(m0) >= fabs(mid) + Rp;
    double pid = det_lu(As) / m0, c2 = minors2(As);
    double sgt = As[0] + As[4] + As[8] - m0;
    double sg = sel(big, (c2 - pid) / m0, sgt), pi = sel(big, pid, c2 - m0 * sgt);
    double disc = 0.25 * sg * sg - pi;
    pcen = 0.5 * sg;
    ps = sqrt(fabs(disc));
    preal = disc >= 0;
    double r1 = pcen + copysgn(ps, pcen);
    double r2 = sel(r1 != 0, pi / sel(r1 != 0, r1, 1.0), pcen - copysgn(ps, pcen));
    mu[1] = csel(preal, cmk(r1, 0.0), cmk(pcen, ps));
    mu[2] = csel(preal, cmk(r2, 0.0), cmk(pcen, -ps));
  }
  // ---- branch-cut pair (log, pow) (gmf_kernel.hpp:305-367)
  bool cut = (KIND != EXP) & (mu[1].re + mu[2].re < 0);
  if (cut) {
    if (!pc) newton<0>(As, mu);
    double l0 = mu[0].re;
    double Mc[9];
#pragma unroll
    for (int k = 0; k < 9; k++) Mc[k] = k % 4 == 0 ? As[k] - l0 : As[k];
    double c01[3] = {Mc[3] * Mc[7] - Mc[6] * Mc[4], Mc[6] * Mc[1] - Mc[0] * Mc[7], Mc[0] * Mc[4] - Mc[3] * Mc[1]};
    double c02[3] = {Mc[3] * Mc[8] - Mc[6] * Mc[5], Mc[6] * Mc[2] - Mc[0] * Mc[8], Mc[0] * Mc[5] - Mc[3] * Mc[2]};
    double c12[3] = {Mc[4] * Mc[8] - Mc[7] * Mc[5], Mc[7] * Mc[2] - Mc[1] * Mc[8], Mc[1] * Mc[5] - Mc[4] * Mc[2]};
    double n01 = c01[0] * c01[0] + c01[1] * c01[1] + c01[2] * c01[2];
    double n02 = c02[0] * c02[0] + c02[1] * c02[1] + c02[2] * c02[2];
    double n12 = c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2];
    bool s1 = n02 > n01;
    double u[3], nn = sel(s1, n02, n01);
#pragma unroll
    for (int k = 0; k < 3; k++) u[k] = sel(s1, c02[k], c01[k]);
    bool s2 = n12 > nn;
#pragma unroll
    for (int k = 0; k < 3; k++) u[k] = sel(s2, c12[k], u[k]);
    nn = sel(s2, n12, nn);
    bool okd = nn > 0;
    double iu = 1.0 / sqrt(sel(okd, nn, 1.0));
#pragma unroll
    for (int k = 0; k < 3; k++) u[k] = u[k] * iu;
    double au0 = fabs(u[0]), au1 = fabs(u[1]), au2 = fabs(u[2]);
    bool k1 = au1 < au0, k2 = au2 < sel(k1, au1, au0);
    double ex = sel(k1 | k2, 0.0, 1.0), ey = sel(k1 & !k2, 1.0, 0.0), ez = sel(k2, 1.0, 0.0);
    double eu = ex * u[0] + ey * u[1] + ez * u[2];
    double q1[3] = {ex - eu * u[0], ey - eu * u[1], ez - eu * u[2]};
    double iq = 1.0 / sqrt(q1[0] * q1[0] + q1[1] * q1[1] + q1[2] * q1[2]);
#pragma unroll
    for (int k = 0; k < 3; k++) q1[k] = q1[k] * iq;
    double q2[3] = {u[1] * q1[2] - u[2] * q1[1], u[2] * q1[0] - u[0] * q1[2], u[0] * q1[1] - u[1] * q1[0]};
    double Sq1[3], Sq2[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
      Sq1[r] = S[3 * r] * q1[0] + S[3 * r + 1] * q1[1] + S[3 * r + 2] * q1[2];
      Sq2[r] = S[3 * r] * q2[0] + S[3 * r + 1] * q2[1] + S[3 * r + 2] * q2[2];
    }
    double b11 = q1[0] * Sq1[0] + q1[1] * Sq1[1] + q1[2] * Sq1[2];
    double b12 = q1[0] * Sq2[0] + q1[1] * Sq2[1] + q1[2] * Sq2[2];
    double b21 = q2[0] * Sq1[0] + q2[1] * Sq1[1] + q2[2] * Sq1[2];
    double b22 = q2[0] * Sq2[0] + q2[1] * Sq2[1] + q2[2] * Sq2[2];
    double dd = 0.5 * (b11 - b22), beta2 = -(dd * dd + b12 * b21), cc = m + 0.5 * (b11 + b22);
    double bb = sqrt(fabs(beta2));
    bool creal = beta2 <= 0;
    mu[1] = csel(okd, csel(creal, cmk(cc + bb, 0.0), cmk(cc, bb)), mu[1]);
    mu[2] = csel(okd, csel(creal, cmk(cc - bb, 0.0), cmk(cc, -bb)), mu[2]);
    pcen = sel(okd, cc, pcen);
    ps = sel(okd, bb, ps);
    preal = (okd & creal) | (!okd & preal);
    pc = pc | okd;
  }
  bool ab[3] = {pc, pc, pc};
  double og[3] = {0.0, 1.0, 2.0};
#pragma unroll
  for (int i = 0; i < 3; i++) x[i] = csel(pc, cmk(mu[i].re - m, mu[i].im), x[i]);

  // ---- node order (gmf_kernel.hpp:373-410)
  {
    auto key = [&](cx v) { return KIND == EXP ? v.re : -cabs_s(v); };
    bool cplxp = x[1].im != 0;
    if (cplxp) {
      bool first = (key(mu[0]) <= key(mu[1])) | cut;
      if (!first) {  // rotate to (pair, real node)
        cx tx = x[0], tm = mu[0];
        bool ta = ab[0];
        double to = og[0];
        x[0] = x[1]; mu[0] = mu[1]; ab[0] = ab[1]; og[0] = og[1];
        x[1] = x[2]; mu[1] = mu[2]; ab[1] = ab[2]; og[1] = og[2];
        x[2] = tx; mu[2] = tm; ab[2] = ta; og[2] = to;
      }
    } else {
#pragma unroll
      for (int s = 0; s < 3; s++) {
        const int i = s == 1 ? 1 : 0, j = i + 1;
        bool sw = key(mu[i]) > key(mu[j]);
        cx tx = x[i], tm = mu[i];
        bool ta = ab[i];
        double to = og[i];
        x[i] = csel(sw, x[j], x[i]); x[j] = csel(sw, tx, x[j]);
        mu[i] = csel(sw, mu[j], mu[i]); mu[j] = csel(sw, tm, mu[j]);
        ab[i] = (sw & ab[j]) | (!sw & ab[i]); ab[j] = (sw & ta) | (!sw & ab[j]);
        og[i] = sel(sw, og[j], og[i]); og[j] = sel(sw, to, og[j]);
      }
    }
  }

  // ---- groups (gmf_kernel.hpp:412-437)
  auto okf = [&](double c, double R) -> bool {
    if (KIND == EXP) return R <= G_R_EXP;
    return (m + c > 0) & (R <= C.rho_f * (m + c));
  };
  double cs3 = (x[0].re + x[1].re + x[2].re) / 3.0;
  double R3 = tmax(tmax(cabs_s(cmk(x[0].re - cs3, x[0].im)), cabs_s(cmk(x[1].re - cs3, x[1].im))),
                   cabs_s(cmk(x[2].re - cs3, x[2].im)));
  bool triple = okf(cs3, R3);
  bool psel[3] = {false, false, false};
  double bestR = __longlong_as_double(0x7FF0000000000000ll);
#pragma unroll
  for (int p = 0; p < 3; p++) {
    const int i = p == 2 ? 1 : 0, j = p == 0 ? 1 : 2, k = 3 - i - j;
    bool elig = ((x[i].im == 0) & (x[j].im == 0)) | ((x[i].re == x[j].re) & (x[i].im == -x[j].im));
    double c = 0.5 * (x[i].re + x[j].re), R = 0.5 * cabs_s(csub(x[i], x[j]));
    bool okp = elig & okf(c, R) & (R <= G_RHO_POLE * cabs_s(cmk(c - x[k].re, -x[k].im))) & !triple;
    bool better = okp & (R < bestR);
    bestR = sel(better, R, bestR);
#pragma unroll
    for (int q = 0; q < p; q++) psel[q] = psel[q] & !better;
    psel[p] = better;
  }
  bool inG[3] = {bool(triple | psel[0] | psel[1]), bool(triple | psel[0] | psel[2]), bool(triple | psel[1] | psel[2])};
  bool pk[3] = {psel[2], psel[1], psel[0]};

  // ---- group centre and offsets (gmf_kernel.hpp:439-460)
  double gsum = sel(inG[0], 1.0, 0.0) + sel(inG[1], 1.0, 0.0) + sel(inG[2], 1.0, 0.0);
  double cxg = (sel(inG[0], x[0].re, 0.0) + sel(inG[1], x[1].re, 0.0) + sel(inG[2], x[2].re, 0.0)) /
               sel(gsum > 0, gsum, 1.0);
  double cmu = m + cxg;
  bool is12[3] = {og[0] > 0.5, og[1] > 0.5, og[2] > 0.5};
  bool ovr = pc & (gsum == 2.0) &
             ((inG[0] & inG[1] & is12[0] & is12[1]) | (inG[0] & inG[2] & is12[0] & is12[2]) |
              (inG[1] & inG[2] & is12[1] & is12[2]));
  cxg = sel(ovr, pcen - m, cxg);
  cmu = sel(ovr, pcen, cmu);
  cx dpair = cmk(sel(preal, ps, 0.0), sel(preal, 0.0, ps));
  cx off[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    bool neg = (mu[i].re - pcen < 0) | (mu[i].im < 0);
    cx di = csel(neg, cmk(-dpair.re, -dpair.im), dpair);
    bool ovi = ovr & inG[i];
    mu[i] = csel(ovi, cmk(pcen + di.re, di.im), mu[i]);
    x[i] = csel(ovi, cmk(mu[i].re - m, mu[i].im), x[i]);
    off[i] = csel(inG[i], csel(ovi, di, cmk(x[i].re - cxg, x[i].im)), cmk(0.0, 0.0));
  }

  // ---- single real nodes far from m: Newton (gmf_kernel.hpp:462-476)
#define MF_FAR_NEWTON(I)                                                                           \
  {                                                                                                \
    bool mask = !inG[I] & !ab[I] & (x[I].im == 0) & (fabs(x[I].re) > 0.5 * fabs(m));              \
    if (mask) {                                                                                    \
      newton<I>(As, mu);                                                                           \
      ab[I] = true;                                                                                \
      x[I] = cmk(mu[I].re - m, mu[I].im);                                                          \
    }                                                                                              \
  }
  MF_FAR_NEWTON(0)
  MF_FAR_NEWTON(1)
  MF_FAR_NEWTON(2)
#undef MF_FAR_NEWTON
  bool absc = (inG[0] & ab[0]) | (inG[1] & ab[1]) | (inG[2] & ab[2]);
  double apole = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) apole = sel(pk[k], sel(absc | ab[k], cmu - mu[k].re, cxg - x[k].re), apole);
  double xshift = KIND == EXP ? tmax(tmax(x[0].re, x[1].re), x[2].re) : 0.0;
  bool bad = KIND == EXP ? false
                         : (((x[0].im == 0) & (mu[0].re <= 0)) | ((x[1].im == 0) & (mu[1].re <= 0)) |
                            ((x[2].im == 0) & (mu[2].re <= 0)));

  // ---- group series (gmf_kernel.hpp:478-533)
  bool hasg = inG[0] | inG[1] | inG[2];
  double L = KIND == EXP ? 1.0 : sel(hasg & (cmu > 0), cmu, 1.0), iL = 1.0 / L;
  cx u[3];
#pragma unroll
  for (int i = 0; i < 3; i++) u[i] = cscl(off[i], iL);
  double ap = sel(fabs(apole) > 0, apole * iL, 1.0), iap = 1.0 / ap;
  double rr = tmax(cabs_s(u[0]), tmax(cabs_s(u[1]), cabs_s(u[2])));
  double rq = sel((pk[0] | pk[1] | pk[2]) & (rr * fabs(iap) <= 1.0), rr * fabs(iap), 0.0);
  rr = sel(hasg & (rr <= G_R_EXP + 0.5), rr, 0.0);
  int j1 = G_KMAX, j2 = G_KMAX;  // (no group: nterms is not called and the split points are not used)
  St.K = hasg ? nterms(C, 3 * (ORDER + 1) - 1, rr, rq, j1, j2) : 0;
  // the float-float / FP32 tail of the series: log and pow without a pole node, coefficients within FP32's range
  const bool tail = (C.ffser != 0) & !(pk[0] | pk[1] | pk[2]) & (rr <= 4.0);
  j1 = tail ? j1 : G_KMAX;
  j2 = tail ? j2 : G_KMAX;
  bool real = (u[0].im == 0) & (u[1].im == 0) & (u[2].im == 0);
#pragma unroll
  for (int k = 0; k < 9; k++) St.As[k] = As[k];
  St.sig = sig; St.m = m; St.cxg = cxg; St.cmu = cmu; St.xshift = xshift; St.iap = iap; St.L = L; St.iL = iL;
#pragma unroll
  for (int i = 0; i < 3; i++) { St.x[i] = x[i]; St.mu[i] = mu[i]; St.u[i] = u[i]; }
  St.flags = (ab[0] ? 1 : 0) | (ab[1] ? 2 : 0) | (ab[2] ? 4 : 0) | (inG[0] ? 8 : 0) | (inG[1] ? 16 : 0) |
             (inG[2] ? 32 : 0) | (pk[0] ? 64 : 0) | (pk[1] ? 128 : 0) | (pk[2] ? 256 : 0) | (bad ? 512 : 0) |
             (real ? 1024 : 0) | (j1 << 12) | (j2 << 20);
}

template <int KIND, int ORDER>
MF_D void gmf_classify(const double *a, const GmfCoef &C, GmfState &St) {
  cx x[3];
  gmf_roots<KIND>(a, x);
  gmf_classify_from<KIND, ORDER>(a, x, C, St);
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
  // ---- residues of the single nodes (gmf_kernel.hpp:534-576)
#pragma unroll
  for (int i = 0; i < 3; i++) {
    if (inG[i]) continue;
    cx xs = KIND == EXP ? cmk(x[i].re - xshift, x[i].im) : x[i];
    cx f0[3];
    f0[0] = coef0<KIND>(C, sig, m, xs, mu[i], 0);
    if (KIND == POW && ORDER >= 1) f0[1] = coef0<KIND>(C, sig, m, xs, mu[i], 1);
    if (KIND == POW && ORDER >= 2) f0[2] = coef0<KIND>(C, sig, m, xs, mu[i], 2);
    cx imu = cinv_s(mu[i]);
    // powers w_z^e (e = 1..5) of 1 / (mu_i - mu_z) for the two other nodes z: the Taylor coefficients of
    // 1 / (t - mu_z)^mz at mu_i are (w^mz, -mz w^(mz+1), mz (mz+1)/2 w^(mz+2))
    const int za = i == 0 ? 1 : 0, zb = i == 2 ? 1 : 2;
    cx wa[6], wb[6];
    wa[0] = cmk(1.0, 0.0);
    wb[0] = cmk(1.0, 0.0);
    wa[1] = cinv_s(csel(ab[i] | ab[za], csub(mu[i], mu[za]), csub(x[i], x[za])));
    wb[1] = cinv_s(csel(ab[i] | ab[zb], csub(mu[i], mu[zb]), csub(x[i], x[zb])));
#pragma unroll
    for (int e = 2; e < 6; e++) { wa[e] = cmul(wa[e - 1], wa[1]); wb[e] = cmul(wb[e - 1], wb[1]); }
#pragma unroll
    for (int c = 0; c < ND; c++) {
      const int mi = gms(c, i);
      if (mi == 0) continue;
      const int k = gms(c, 0) - 1, ma = gms(c, za), mb = gms(c, zb);
      cx fb = KIND == POW ? f0[k] : f0[0], ser[3];
      if (KIND == EXP) {
        ser[0] = fb; ser[1] = fb; ser[2] = cscl(fb, 0.5);
      } else if (KIND == LOG) {
        ser[0] = fb; ser[1] = imu; ser[2] = cscl(cmul(imu, imu), -0.5);
      } else {
        ser[0] = fb;
        ser[1] = cscl(cmul(fb, imu), C.al);
        ser[2] = cscl(cmul(ser[1], imu), (C.al - 1.0) / 2.0);
      }
      // coefficient mi - 1 of ser * Pa * Pb (truncated products, only the terms that are needed)
      cx pa[3], pb[3];
      pa[0] = wa[ma];
      pb[0] = wb[mb];
      if (mi >= 2) {
        pa[1] = ma ? cscl(wa[ma + 1], (double)-ma) : cmk(0.0, 0.0);
        pb[1] = mb ? cscl(wb[mb + 1], (double)-mb) : cmk(0.0, 0.0);
      }
      if (mi >= 3) {
        pa[2] = ma ? cscl(wa[ma + 2], ma * (ma + 1) / 2.0) : cmk(0.0, 0.0);
        pb[2] = mb ? cscl(wb[mb + 2], mb * (mb + 1) / 2.0) : cmk(0.0, 0.0);
      }
      cx q[3];
      q[0] = ma ? (mb ? cmul(pa[0], pb[0]) : pa[0]) : pb[0];
      if (mi >= 2) q[1] = cadd(ma ? (mb ? cmul(pa[0], pb[1]) : cmk(0.0, 0.0)) : pb[1],
                               mb ? (ma ? cmul(pa[1], pb[0]) : cmk(0.0, 0.0)) : pa[1]);
      if (mi >= 3) q[2] = cadd(cadd(ma ? (mb ? cmul(pa[0], pb[2]) : cmk(0.0, 0.0)) : pb[2],
                                    (ma && mb) ? cmul(pa[1], pb[1]) : cmk(0.0, 0.0)),
                               mb ? (ma ? cmul(pa[2], pb[0]) : cmk(0.0, 0.0)) : pa[2]);
      cx r = cmul(ser[0], q[mi - 1]);
      if (mi >= 2) r = cadd(r, cmul(ser[1], q[mi - 2]));
      if (mi >= 3) r = cadd(r, cmul(ser[2], q[0]));
      D[c] = cadd(D[c], r);
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
