// smf_mixed_math.cuh -- mixed-precision symmetric family, the per-matrix device math: FP32 input and output, FP32
// for the bulk of the arithmetic.
//
// Beyond FP32 precision (float-float, ffloat.cuh, on the FP32 pipe) only where FP32 would lose the result:
//   * the Rayleigh quotients that give the eigenvalues and the Gram matrix of the eigenvectors: with condition
//     numbers up to 1e6 and eigenvalue gaps down to 1e-12 FP32 quotients lose the small eigenvalues and the
//     near-degenerate pairs entirely;
//   * the differences of eigenvalues that feed the near-coalescent branches of the divided differences (z, u, w and
//     the denominators of the difference formulas), taken from the float-float eigenvalues before rounding to FP32.
// f(lambda), the first and second divided differences (stable forms, cluster series), the product vectors and the
// J / H forms of smf_tile.cuh run in FP32.  The kernel executes no FP64 instruction (the FP64 kernel: ~2.5k per
// matrix, at 1/74 of the FP32 rate on GB300), so it moves towards the HBM roofline, and FP32 storage halves the bytes.
// Accuracy against the FP64 oracle is stated per kind and order in the tests (<= 1e-6 relative, max-norm).
#pragma once
#include "ffloat.cuh"
#include "smf_device.cuh"

namespace mf {

// terms of the cluster series of the second divided difference in FP32.  log: the offsets are at most tau = 0.25 of
// the centre, so term k is below (k + 1) 0.25^k |c2[0]| and 16 terms reach 1e-8 relative (exp: offsets up to 1 in
// absolute terms, factorial coefficients).  Powers (and sqrt) take tau = 0.5 (or 3 / alpha, below it) and 30 terms
// (31 0.5^30 < 3e-8): outside the cluster the difference formula (D_jk - D_ij) / d subtracts first divided
// differences that differ by (1 - alpha) d / l_j of their size, so their FP32 rounding is amplified by about
// 1 / ((1 - alpha) tau); at tau = 0.25 that put H of pow 0.7 at 1.3e-6 .. 1.7e-6 of its maximum on near-double
// eigenvalues.  (The FP64 form, whose difference formula loses less, takes the series only within 2^-6.)
constexpr int DD2_TERMS_F = 16, DD2_TERMS_F_POW = 30;
constexpr double DD2_TAU_F_POW = 0.5;

constexpr int G1_TERMS_F = 16;  // terms of the series of g(z) below

struct SmfCoefF {
  float al, alm1;   // exponent and exponent - 1
  float zp1, z2;    // 0^(al - 1), f''(0)/2 for powers
  float tau;        // cluster radius of the second divided difference
  float c2[DD2_TERMS];
  // powers, f[a, b] = s^(al - 1) g(z) for s = (a + b) / 2, z = (b - a) / (2 s), |z| < 1/2:
  // g(z) = ((1 + z)^al - (1 - z)^al) / (2 z) = sum_m binom(al, 2m + 1) z^(2m); g1ser = 1 where that series, with
  // G1_TERMS_F terms, is summed without cancellation and truncated below 1e-9 (small exponents)
  int g1ser;
  float g1[G1_TERMS_F];
};

MF_D float self(bool m, float a, float b) { return m ? a : b; }

template <int KIND>
MF_D float fun_f(float x, float al) {
  if (KIND == EXP) return expf(x);
  if (KIND == LOG) return logf(x);
  if (!(x > 0.f)) return 0.f;
  return KIND == SQRT ? sqrtf(x) : powf(x, al);
}

// Divided differences on eigenvalues sorted ascending, in FP32.  The eigenvalue differences are taken in FP64 and
// rounded once (dab = b - a >= 0 and friends), so the near-coalescent branches see the same relative precision as
// the FP64 kernel; with the order known, the choice of difference formula and of the cluster midpoint of the FP64
// kernel becomes static.
// f[a, b], a <= b, dab = b - a, rdab = 1 / dab (1 where dab = 0), ra = 1 / a (log and powers) -- smf_kernel.hpp:84-115.
// Quotients by dab and a are products with the matrix's shared reciprocals (smf_rec_f): a correctly rounded
// division costs about as much as the reciprocal it is built on, and the three eigenvalues and three differences
// serve every first and second divided difference of the matrix.
template <int KIND>
MF_D float dd1s_f(float a, float b, float dab, float rdab, float ra, float fa, float fb, const SmfCoefF &C) {
  if (KIND == EXP) return fb * self(dab > 0.f, -expm1f(-dab) * rdab, 1.f);
  if (KIND == LOG) {
    const float rs = 1.f / (a + b), z = dab * rs, az = fabsf(z), z2 = z * z;
    if (az < 1e-3f) return (1.f + z2 * (1.f / 3.f) + z2 * z2 * 0.2f + z2 * z2 * z2 * (1.f / 7.f)) * (2.f * rs);
    // log(b / a) as log1p(dab / a), free of log |A| (whose ulp a difference of two logs would carry) and within a few
    // ulp for every ratio, so one form serves the near and the far pairs (the FP64 form's atanh branch for
    // 1e-3 <= |z| < 0.5 would be a third divergent path); a <= 0 keeps the difference of logs, with its infinities
    // and NaNs (fa, fb: log a, log b)
    return (a > 0.f ? log1pf(dab * ra) : fb - fa) * rdab;
  }
  if (KIND == SQRT) return 1.f / (fa + fb);  // (fa, fb: the square roots of a, b >= 0)
  float s = 0.5f * (a + b), ss = self(s > 0.f, s, 1.f);
  float z = dab * (s > 0.f ? 1.f / (a + b) : 0.5f), az = fabsf(z);
  bool zero = az == 0.f, near = !zero & (az < 0.5f);
  if (!zero & !near) return (fb - fa) * rdab;
  float g;
  if (C.g1ser) {  // (uniform: a launch constant) the series of g in z^2, Horner
    const float zz = z * z;
    g = C.g1[G1_TERMS_F - 1];
#pragma unroll
    for (int k = G1_TERMS_F - 2; k >= 0; k--) g = fmaf(g, zz, C.g1[k]);
  } else {
    g = zero ? C.al : (expm1f(C.al * log1pf(z)) - expm1f(C.al * log1pf(-z))) / (2.f * z);
  }
  return (s > 0.f ? powf(ss, C.alm1) : C.zp1) * g;
}

// f'(x) from fx = f(x) and rx = 1 / x (log and powers)
template <int KIND>
MF_D float deriv_f(float x, float fx, float rx, const SmfCoefF &C) {
  if (KIND == EXP) return fx;
  if (KIND == LOG) return rx;
  float xf = self(x > 0.f, x, 0.f);
  if (KIND == SQRT) return 1.f / (2.f * fx);  // (fx = sqrt(x), x >= 0)
  return xf > 0.f ? C.al * (fx / xf) : C.al * C.zp1;  // al x^(al - 1) from fx = x^al at hand
}

// f[li, lj, lk] for li <= lj <= lk; dji = lj - li, dkj = lk - lj, dki = lk - li, rlj = 1 / lj (log and powers),
// rdki = 1 / dki (1 where dki = 0) -- smf_kernel.hpp:148-192 (the widest difference is the denominator, the middle
// eigenvalue the cluster centre).  SHAPE is what the caller knows statically: 0 three distinct indices, 1 li = lj
// (dji = 0), 2 lj = lk (dkj = 0).  With one offset zero, the complete homogeneous polynomials h_k(u, w) of the
// cluster series are powers of the other, and the series is one Horner sum (one FMA a term instead of three).
template <int KIND, int SHAPE>
MF_D float dd2s_f(float lj, float lk, float fj, float rlj, float Dij, float Djk, float dji, float dkj, float rdki,
                  const SmfCoefF &C) {
  bool cluster;
  if (KIND == EXP) cluster = (dkj + dji) <= 1.f;
  else cluster = (lj > 0.f) & (dji <= C.tau * lj) & (dkj <= C.tau * lj);
  float out;
  if (cluster) {
    float u, w, scale;
    if (KIND == EXP) {
      u = -dji; w = dkj; scale = fj;
    } else {
      u = -dji * rlj; w = dkj * rlj;
      scale = (KIND == LOG ? rlj : fj * rlj) * rlj;
    }
    constexpr int NT = (KIND == POW || KIND == SQRT) ? DD2_TERMS_F_POW : DD2_TERMS_F;
    float sm;
    if (SHAPE == 0) {
      float h = 1.f, wk = 1.f;
      sm = C.c2[0];
#pragma unroll
      for (int k = 1; k < NT; k++) {
        wk = wk * w;
        h = fmaf(u, h, wk);
        sm = fmaf(C.c2[k], h, sm);
      }
    } else {
      const float x = SHAPE == 1 ? w : u;
      sm = C.c2[NT - 1];
#pragma unroll
      for (int k = NT - 2; k >= 0; k--) sm = fmaf(sm, x, C.c2[k]);
    }
    out = scale * sm;
  } else {
    out = (Djk - Dij) * rdki;
  }
  if (KIND == POW || KIND == SQRT) out = self(lk > 0.f, out, C.z2);
  return out;
}

template <int KIND>
MF_D float dd2_same_f(float lf, float fl, float rl, float Dll, const SmfCoefF &C) {
  bool cluster = KIND == EXP ? true : (lf > 0.f);
  float out = KIND == EXP ? self(cluster, fl * C.c2[0], Dll - Dll)
                          : self(cluster, ((KIND == LOG ? rl : fl * rl) * rl) * C.c2[0], Dll - Dll);
  if (KIND == POW || KIND == SQRT) out = self(lf > 0.f, out, C.z2);
  return out;
}

MF_D float nrm3(float &x, float &y, float &z) {
  float n = __fsqrt_rn(x * x + y * y + z * z), i = __fdiv_rn(1.f, n);
  x *= i; y *= i; z *= i;
  return n;
}

// The symmetric input of the mixed path: FP32 diagonal, float-float off-diagonal (the exact average of a_ij and a_ji
// for the matrix layout; LO = false for Voigt input, whose off-diagonal entries are FP32 values)
struct SmfInF {
  float d[3];
  ffl o[3];  // (0,1), (0,2), (1,2)
};

// x^T A x with the diagonal shifted by a float-float (A - mu I), compensated (Dot2) to float-float accuracy
template <bool LO>
MF_D ffl quad_ff(const ffl *dg, const ffl *o, float x0, float x1, float x2) {
  const float x[3] = {x0, x1, x2};
  ffacc A = {0.f, 0.f};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    ffl p = two_prod(x[i], x[i]);
    ffl t = two_prod(dg[i].hi, p.hi);
    acc_add(A, t.hi);
    A.e += fmaf(dg[i].hi, p.lo, fmaf(dg[i].lo, p.hi, t.lo));
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int i = k == 2 ? 1 : 0, j = k == 0 ? 1 : 2;
    ffl p = two_prod(2.f * x[i], x[j]);
    ffl t = two_prod(o[k].hi, p.hi);
    acc_add(A, t.hi);
    A.e += LO ? fmaf(o[k].hi, p.lo, fmaf(o[k].lo, p.hi, t.lo)) : fmaf(o[k].hi, p.lo, t.lo);
  }
  return acc_ff(A);
}

// x^T A y (A as above)
template <bool LO>
MF_D ffl bil_ff(const ffl *dg, const ffl *o, const float *x, const float *y) {
  ffacc A = {0.f, 0.f};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    ffl p = two_prod(x[i], y[i]);
    ffl t = two_prod(dg[i].hi, p.hi);
    acc_add(A, t.hi);
    A.e += fmaf(dg[i].hi, p.lo, fmaf(dg[i].lo, p.hi, t.lo));
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int i = k == 2 ? 1 : 0, j = k == 0 ? 1 : 2;
    ffl p1 = two_prod(x[i], y[j]), p2 = two_prod(x[j], y[i]);
    ffl s = two_sum(p1.hi, p2.hi);
    float sl = s.lo + (p1.lo + p2.lo);
    ffl t = two_prod(o[k].hi, s.hi);
    acc_add(A, t.hi);
    A.e += LO ? fmaf(o[k].hi, sl, fmaf(o[k].lo, s.hi, t.lo)) : fmaf(o[k].hi, sl, t.lo);
  }
  return acc_ff(A);
}

MF_D ffl dot_ff(const float *x, const float *y) {
  ffacc A = {0.f, 0.f};
#pragma unroll
  for (int i = 0; i < 3; i++) acc_prod(A, x[i], y[i]);
  return acc_ff(A);
}

// q / n for n = 1 + e close to 1: q (1 - e + e^2), float-float
MF_D ffl div_norm(ffl q, ffl n) {
  float e = (n.hi - 1.f) + n.lo;
  return ff_mul(q, fast_two_sum(1.f, e * e - e));
}

// The eigensystem of the mixed path, with no FP64: FP32 for the cubic's trigonometric root (on the deviator normalised
// to max 1, where the root of the separated eigenvalue is insensitive to rounding of r), its eigenvector (largest
// cross product of two rows of G - root I), the orthonormal complement and the 2x2 Jacobi rotation; float-float
// (ffloat.cuh) for the deviator, the Rayleigh quotients of the FP32 vectors and their Gram matrix.  The quotients
// are taken in A - mu I, mu the centre of the remaining pair, so that the pair's block is of the size of its own gap:
// the rotation angle is accurate relative to the gap, and the quotients divided by the vectors' squared norms give
// the eigenvalues to ~1e-14 relative to |A| (an FP32 vector error d moves a quotient by O(d^2)).  One Newton-Schulz
// step V (3 I - V^T V) / 2 with the float-float Gram matrix leaves the FP32 vectors orthonormal to the rounding of
// their components.  Input scaled by a power of two; eigenvalues and the deviator's eigenvalues (xd, for log near
// the mean) in the units of the input.
struct SmfEigF {
  ffl lam[3], xd[3];
  float m;
  float V[3][3];
};

template <int KIND, bool LO>
MF_D void smf_eigsys_ff(const SmfInF &in, SmfEigF &E) {
  constexpr float SQRT6 = 2.4494897f, TWO_PI_3 = 2.0943951f;
  // power-of-two scaling from the largest magnitude (integer compare of the bit patterns: NaN sorts above Inf)
  int kb = 0;
#pragma unroll
  for (int i = 0; i < 3; i++) kb = max(kb, __float_as_int(in.d[i]) & 0x7FFFFFFF);
#pragma unroll
  for (int k = 0; k < 3; k++) kb = max(kb, __float_as_int(in.o[k].hi) & 0x7FFFFFFF);
  const bool bad = kb >= 0x7F800000;  // NaN or infinite input: NaN vectors and results
  int ex = min(max((kb >> 23) & 0xFF, 1), 253);
  const float sig = __int_as_float(ex << 23), isig = __int_as_float((254 - ex) << 23);
  float a[3];
  ffl o[3];
#pragma unroll
  for (int i = 0; i < 3; i++) a[i] = in.d[i] * isig;
#pragma unroll
  for (int k = 0; k < 3; k++) o[k] = {in.o[k].hi * isig, LO ? in.o[k].lo * isig : 0.f};
  // mean of the diagonal and deviator, float-float
  ffl s01 = two_sum(a[0], a[1]), s = two_sum(s01.hi, a[2]);
  s = fast_two_sum(s.hi, s.lo + s01.lo);
  // (q1 within an ulp of s.hi / 3; the residue s.hi - 3 q1 is exact, so q1 + q2 is the mean to float-float accuracy)
  float q1 = s.hi * (1.f / 3.f);
  float q2 = (fmaf(-q1, 3.f, s.hi) + s.lo) * (1.f / 3.f);
  const ffl m = fast_two_sum(q1, q2);
  // deviator in FP32 (the input of the trigonometric root only), from the float-float mean: a - m.hi is exact near
  // the mean, and subtracting m.lo too leaves it traceless to FP32 rounding, as the root formula assumes (the
  // trace residue 3 m.lo alone is a few percent of a deviator of 1e-6 |A|, and skews the root and its vector)
  float dv[3];
#pragma unroll
  for (int i = 0; i < 3; i++) dv[i] = (a[i] - m.hi) - m.lo;
  // FP32: normalised deviator, trigonometric root, eigenvector, complement
  int kd = 0;
#pragma unroll
  for (int i = 0; i < 3; i++) kd = max(kd, __float_as_int(dv[i]) & 0x7FFFFFFF);
#pragma unroll
  for (int k = 0; k < 3; k++) kd = max(kd, __float_as_int(o[k].hi) & 0x7FFFFFFF);
  const bool iso = (kd == 0) | bad;
  const int ed = min(max((kd >> 23) & 0xFF, 1), 253);
  const float dsc = __int_as_float(ed << 23), ids = __int_as_float((254 - ed) << 23);
  float g0 = dv[0] * ids, g1 = dv[1] * ids, g2 = dv[2] * ids;
  float g3 = o[0].hi * ids, g4 = o[1].hi * ids, g5 = o[2].hi * ids;
  float p = g0 * g0 + g1 * g1 + g2 * g2 + 2.f * (g3 * g3 + g4 * g4 + g5 * g5);
  float q = g0 * (g1 * g2 - g5 * g5) - g3 * (g3 * g2 - g5 * g4) + g4 * (g3 * g5 - g1 * g4);
  float pg = self(iso, 1.f, p), qg = self(iso, 0.f, q);
  float r = 3.f * SQRT6 * qg / (pg * sqrtf(pg));
  r = self(r > 1.f, 1.f, self(r < -1.f, -1.f, r));
  float t = sqrtf(pg * (2.f / 3.f)), ph = acosf(r) * (1.f / 3.f);
  float sh = t * cosf(self(r >= 0.f, ph, ph + TWO_PI_3));
  float m00 = g0 - sh, m11 = g1 - sh, m22 = g2 - sh;
  float cxv = g3 * g5 - g4 * m11, cyv = g4 * g3 - m00 * g5, czv = m00 * m11 - g3 * g3;
  float nn = cxv * cxv + cyv * cyv + czv * czv;
  {
    float bx = g3 * m22 - g4 * g5, by = g4 * g4 - m00 * m22, bz = m00 * g5 - g3 * g4;
    float nb = bx * bx + by * by + bz * bz;
    bool s1 = nb > nn;
    cxv = self(s1, bx, cxv); cyv = self(s1, by, cyv); czv = self(s1, bz, czv); nn = self(s1, nb, nn);
    float ex2 = m11 * m22 - g5 * g5, ey2 = g5 * g4 - g3 * m22, ez2 = g3 * g5 - m11 * g4;
    float ne = ex2 * ex2 + ey2 * ey2 + ez2 * ez2;
    bool s2 = ne > nn;
    cxv = self(s2, ex2, cxv); cyv = self(s2, ey2, cyv); czv = self(s2, ez2, czv); nn = self(s2, ne, nn);
  }
  bool ok = (nn > 1e-30f) & !iso;
  float v[3] = {self(ok, cxv, 1.f), self(ok, cyv, 0.f), self(ok, czv, 0.f)};
  nrm3(v[0], v[1], v[2]);
  float ax = fabsf(v[0]), ay = fabsf(v[1]), az = fabsf(v[2]);
  bool k1 = ay < ax, k2 = az < self(k1, ay, ax);
  float ex1 = self(k1 | k2, 0.f, 1.f), ey1 = self(k1 & !k2, 1.f, 0.f), ez1 = self(k2, 1.f, 0.f);
  float vk = ex1 * v[0] + ey1 * v[1] + ez1 * v[2];
  float u[3] = {ex1 - vk * v[0], ey1 - vk * v[1], ez1 - vk * v[2]};
  nrm3(u[0], u[1], u[2]);
  float w[3] = {v[1] * u[2] - v[2] * u[1], v[2] * u[0] - v[0] * u[2], v[0] * u[1] - v[1] * u[0]};
  // float-float: quotients in A - mu I, mu = mean - root / 2 (the centre of the remaining pair)
  const float mu = self(iso, m.hi, m.hi - 0.5f * (sh * dsc));
  ffl dg[3];
#pragma unroll
  for (int i = 0; i < 3; i++) dg[i] = two_sum(a[i], -mu);
  const ffl qv = quad_ff<LO>(dg, o, v[0], v[1], v[2]), nv = dot_ff(v, v);
  const ffl b11 = quad_ff<LO>(dg, o, u[0], u[1], u[2]), b22 = quad_ff<LO>(dg, o, w[0], w[1], w[2]);
  const ffl b12 = bil_ff<LO>(dg, o, u, w);
  // FP32 Jacobi rotation of the pair from the block (its entries are of the size of the pair's gap).  The angle
  // depends on jy / jx only, so both are scaled by a power of two into [1, 2) before they are squared: a gap below
  // ~1e-19 of |A| would otherwise square into FP32's subnormal range, and the rounded jr would leave cos^2 + sin^2
  // away from 1 by more than the Newton-Schulz step below repairs (1e-5 at a gap of 1e-22).  Where the squares are
  // normal the scaling is exact and changes no bit of cos and sin.
  ffl jd = ff_sub(b11, b22);
  float jx = jd.hi + jd.lo, jy = 2.f * (b12.hi + b12.lo);
  {
    const int kj = max(__float_as_int(jx) & 0x7FFFFFFF, __float_as_int(jy) & 0x7FFFFFFF);
    const float js = __int_as_float((254 - min(max((kj >> 23) & 0xFF, 1), 253)) << 23);
    jx *= js;
    jy *= js;
  }
  float jr = sqrtf(jx * jx + jy * jy);
  bool jz = !(jr > 0.f), jpos = jx >= 0.f;
  float jrs = self(jz, 1.f, jr);
  float big = sqrtf((jrs + fabsf(jx)) / (2.f * jrs)), sml = jy / (2.f * jrs * big);
  float sgn = self(jy >= 0.f, 1.f, -1.f);
  float cs = self(jz, 1.f, self(jpos, big, sgn * sml)), sn = self(jz, 0.f, self(jpos, sml, sgn * big));
  float r1[3] = {cs * u[0] + sn * w[0], cs * u[1] + sn * w[1], cs * u[2] + sn * w[2]};
  float r2[3] = {cs * w[0] - sn * u[0], cs * w[1] - sn * u[1], cs * w[2] - sn * u[2]};
  const ffl n1 = dot_ff(r1, r1), n2 = dot_ff(r2, r2);
  const ffl q1f = quad_ff<LO>(dg, o, r1[0], r1[1], r1[2]), q2f = quad_ff<LO>(dg, o, r2[0], r2[1], r2[2]);
  const ffl th[3] = {div_norm(qv, nv), div_norm(q1f, n1), div_norm(q2f, n2)};
  const ffl mum = ff_sub(ff_from(mu), m);  // mu - mean
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const ffl lam = ff_add(th[i], ff_from(mu));
    E.lam[i] = {lam.hi * sig, lam.lo * sig};
    const ffl xd = ff_add(th[i], mum);
    E.xd[i] = {xd.hi * sig, xd.lo * sig};
  }
  E.m = m.hi * sig;
  // The FP32 cross products leave v a few ulp off its eigenvector, towards the pair's plane; H carries six factors of
  // it (an error of 2.5 ulp there put H of condition-1e6 matrices at 1.2e-6 of its maximum).  First-order correction
  // of that coupling: c_i = v^T (A - mu I) r_i in float-float is (the angle of v towards r_i) (th_v - th_i), so
  // v += sum_i r_i c_i / (th_v - th_i) and r_i -= v c_i / (th_v - th_i), taken where the angle is below 2^-10 (v
  // and the pair then well apart; near a triple eigenvalue the split does not matter).  The pair's own rotation is
  // accurate relative to its gap already.
  {
    const ffl c1 = bil_ff<LO>(dg, o, v, r1), c2 = bil_ff<LO>(dg, o, v, r2);
    const float t1 = (c1.hi + c1.lo) / ((th[0].hi - th[1].hi) + (th[0].lo - th[1].lo));
    const float t2 = (c2.hi + c2.lo) / ((th[0].hi - th[2].hi) + (th[0].lo - th[2].lo));
    const float a1 = fabsf(t1) <= 0x1p-10f ? t1 : 0.f, a2 = fabsf(t2) <= 0x1p-10f ? t2 : 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const float vi = v[i];
      v[i] = fmaf(r1[i], a1, fmaf(r2[i], a2, vi));
      r1[i] = fmaf(-vi, a1, r1[i]);
      r2[i] = fmaf(-vi, a2, r2[i]);
    }
  }
  // Newton-Schulz step with the float-float Gram matrix
  const ffl nv2 = dot_ff(v, v), n12 = dot_ff(r1, r1), n22 = dot_ff(r2, r2);
  const ffl g01 = dot_ff(v, r1), g02 = dot_ff(v, r2), g12 = dot_ff(r1, r2);
  float e00 = 0.5f * ((nv2.hi - 1.f) + nv2.lo), e11 = 0.5f * ((n12.hi - 1.f) + n12.lo);
  float e22 = 0.5f * ((n22.hi - 1.f) + n22.lo);
  float e01 = 0.5f * (g01.hi + g01.lo), e02 = 0.5f * (g02.hi + g02.lo), e12 = 0.5f * (g12.hi + g12.lo);
  float nanv = __int_as_float(0x7FC00000);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    E.V[i][0] = self(bad, nanv, v[i] - (v[i] * e00 + r1[i] * e01 + r2[i] * e02));
    E.V[i][1] = self(bad, nanv, r1[i] - (v[i] * e01 + r1[i] * e11 + r2[i] * e12));
    E.V[i][2] = self(bad, nanv, r2[i] - (v[i] * e02 + r1[i] * e12 + r2[i] * e22));
  }
  if (bad) {
#pragma unroll
    for (int i = 0; i < 3; i++) E.lam[i] = E.xd[i] = {nanv, nanv};
  }
}

// Voigt input (FP32 values)
MF_D void voigt_in_f(const float *xi, SmfInF &in) {
#pragma unroll
  for (int i = 0; i < 3; i++) in.d[i] = xi[i];
#pragma unroll
  for (int k = 0; k < 3; k++) in.o[k] = {xi[3 + k], 0.f};
}

// symmetric part of an FP32 3x3 matrix: the off-diagonal averages exactly as float-float; all NaN if
// |a_ij - a_ji| > 1e-8 max |a_kl| (smf_kernel.hpp:408-421)
MF_D void sym_in_f(const float *xi, SmfInF &in) {
  float mx = 0.f;
#pragma unroll
  for (int k = 0; k < 9; k++) mx = fmaxf(mx, fabsf(xi[k]));
  const float tol = 1e-8f * mx;
  const bool sym = !(fabsf(xi[1] - xi[3]) > tol) & !(fabsf(xi[2] - xi[6]) > tol) & !(fabsf(xi[5] - xi[7]) > tol);
  const float nanv = __int_as_float(0x7FC00000);
  in.d[0] = self(sym, xi[0], nanv); in.d[1] = self(sym, xi[4], nanv); in.d[2] = self(sym, xi[8], nanv);
  const int ia[3] = {1, 2, 5}, ib[3] = {3, 6, 7};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    ffl t = two_sum(xi[ia[k]], xi[ib[k]]);
    in.o[k] = {self(sym, 0.5f * t.hi, nanv), self(sym, 0.5f * t.lo, nanv)};
  }
}

// the spectrum of the mixed path, eigenvalues sorted ascending: FP32 eigenvectors V (columns), eigenvalues lf,
// their differences taken in float-float and rounded once (d10 = l1 - l0, d21, d20), and f(lambda) (log near the
// mean through log1p of the deviator's eigenvalue, smf_kernel.hpp:283-290); powers see max(lambda, 0)
struct SmfSpecF {
  float lf[3], fl[3], V[3][3], d10, d21, d20;
};

MF_D bool ff_less(ffl a, ffl b) { return (a.hi < b.hi) | ((a.hi == b.hi) & (a.lo < b.lo)); }

template <int KIND, bool LO>
MF_D void smf_spectrum_f(const SmfInF &in, const SmfCoefF &C, SmfSpecF &Sp) {
  SmfEigF E;
  smf_eigsys_ff<KIND, LO>(in, E);
  ffl lam[3] = {E.lam[0], E.lam[1], E.lam[2]}, xd[3] = {E.xd[0], E.xd[1], E.xd[2]};
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Sp.V[i][j] = E.V[i][j];
#pragma unroll
  for (int st = 0; st < 3; st++) {  // sort ascending: a static order for every divided difference
    const int a = st == 1 ? 1 : 0, b = a + 1;
    bool sw = ff_less(lam[b], lam[a]);
    ffl la = lam[a], lb = lam[b], xa = xd[a], xb = xd[b];
    lam[a] = ff_sel(sw, lb, la); lam[b] = ff_sel(sw, la, lb);
    xd[a] = ff_sel(sw, xb, xa); xd[b] = ff_sel(sw, xa, xb);
#pragma unroll
    for (int r = 0; r < 3; r++) {
      float va = Sp.V[r][a], vb = Sp.V[r][b];
      Sp.V[r][a] = self(sw, vb, va); Sp.V[r][b] = self(sw, va, vb);
    }
  }
  if (KIND == POW || KIND == SQRT) {
#pragma unroll
    for (int i = 0; i < 3; i++) lam[i] = ff_sel(ff_less(ffl{0.f, 0.f}, lam[i]), lam[i], ffl{0.f, 0.f});
  }
#pragma unroll
  for (int i = 0; i < 3; i++) Sp.lf[i] = lam[i].hi;
  ffl t10 = ff_sub(lam[1], lam[0]), t21 = ff_sub(lam[2], lam[1]), t20 = ff_sub(lam[2], lam[0]);
  Sp.d10 = t10.hi + t10.lo; Sp.d21 = t21.hi + t21.lo; Sp.d20 = t20.hi + t20.lo;
#pragma unroll
  for (int i = 0; i < 3; i++) Sp.fl[i] = fun_f<KIND>(Sp.lf[i], C.al);
  if (KIND == LOG) {
    const float mf = E.m, lms = logf(mf), imf = 1.f / mf;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      // near 1 (the log strain of a small deformation): log1p of lambda - 1, taken in float-float from the
      // float-float eigenvalue, keeps FP32 relative accuracy in log lambda, where log m + log1p(x / m) would lose
      // the rounding of m to FP32 against a result of the size of the strain; one log1p serves both forms
      const float x = xd[i].hi + xd[i].lo;
      const float tt = (lam[i].hi - 1.f) + lam[i].lo;  // lam.hi - 1 is exact where |tt| <= 0.25 (Sterbenz)
      const bool near1 = fabsf(tt) <= 0.25f, nearm = fabsf(x) <= 0.5f * mf;
      const float l1 = log1pf(self(near1, tt, x * imf));
      Sp.fl[i] = self(near1, l1, self(nearm, lms + l1, Sp.fl[i]));
    }
  }
}

// the reciprocals a matrix's divided differences share: of the eigenvalue differences (1 where one is 0) and, for
// log and powers, of the eigenvalues
struct SmfRecF {
  float rd10, rd20, rd21, rl[3];
};

template <int KIND>
MF_D SmfRecF smf_rec_f(const SmfSpecF &Sp) {
  SmfRecF R;
  R.rd10 = 1.f / self(Sp.d10 != 0.f, Sp.d10, 1.f);
  R.rd20 = 1.f / self(Sp.d20 != 0.f, Sp.d20, 1.f);
  R.rd21 = 1.f / self(Sp.d21 != 0.f, Sp.d21, 1.f);
#pragma unroll
  for (int i = 0; i < 3; i++) R.rl[i] = (KIND == LOG || KIND == POW) ? 1.f / Sp.lf[i] : 0.f;
  return R;
}

// first divided differences D_ij = f[l_i, l_j] (D_ii = f'(l_i)) in FP32
template <int KIND>
MF_D void smf_dm_f(const SmfSpecF &Sp, const SmfCoefF &C, float Dm[3][3]) {
  const SmfRecF R = smf_rec_f<KIND>(Sp);
  const float D01 = dd1s_f<KIND>(Sp.lf[0], Sp.lf[1], Sp.d10, R.rd10, R.rl[0], Sp.fl[0], Sp.fl[1], C);
  const float D02 = dd1s_f<KIND>(Sp.lf[0], Sp.lf[2], Sp.d20, R.rd20, R.rl[0], Sp.fl[0], Sp.fl[2], C);
  const float D12 = dd1s_f<KIND>(Sp.lf[1], Sp.lf[2], Sp.d21, R.rd21, R.rl[1], Sp.fl[1], Sp.fl[2], C);
#pragma unroll
  for (int i = 0; i < 3; i++) Dm[i][i] = deriv_f<KIND>(Sp.lf[i], Sp.fl[i], R.rl[i], C);
  Dm[0][1] = Dm[1][0] = D01; Dm[0][2] = Dm[2][0] = D02; Dm[1][2] = Dm[2][1] = D12;
}

// second divided differences D2_ijl = f[l_i, l_j, l_l] (symmetric) in FP32
template <int KIND>
MF_D void smf_d2_f(const SmfSpecF &Sp, const float Dm[3][3], const SmfCoefF &C, float D2[3][3][3]) {
  if (KIND == SQRT) {
    // sqrt: f[a, b, c] = -1 / ((sa + sb)(sa + sc)(sb + sc)) with s = sqrt, exactly (f''(a) / 2 = -1 / (8 a^(3/2))
    // where points coincide): sums of non-negative terms, free of cancellation at every spacing, so neither the
    // cluster series nor the difference formula is needed (a zero eigenvalue pair gives -inf, as f''(0) / 2)
    const float *sq = Sp.fl;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = i; j < 3; j++)
#pragma unroll
        for (int l = j; l < 3; l++) {
          const float d = -1.f / ((sq[i] + sq[j]) * (sq[i] + sq[l]) * (sq[j] + sq[l]));
          D2[i][j][l] = D2[i][l][j] = D2[j][i][l] = D2[j][l][i] = D2[l][i][j] = D2[l][j][i] = d;
        }
    return;
  }
  const SmfRecF R = smf_rec_f<KIND>(Sp);
  const float dd[3][3] = {{0.f, Sp.d10, Sp.d20}, {0.f, 0.f, Sp.d21}, {0.f, 0.f, 0.f}};
  const float rd[3][3] = {{1.f, R.rd10, R.rd20}, {1.f, 1.f, R.rd21}, {1.f, 1.f, 1.f}};
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++)
#pragma unroll
      for (int l = j; l < 3; l++) {
        float d;
        if (i == j && j == l) {
          d = dd2_same_f<KIND>(Sp.lf[i], Sp.fl[i], R.rl[i], Dm[i][i], C);
        } else {
          d = i == j ? dd2s_f<KIND, 1>(Sp.lf[j], Sp.lf[l], Sp.fl[j], R.rl[j], Dm[i][j], Dm[j][l], 0.f, dd[j][l],
                                       rd[i][l], C)
              : j == l ? dd2s_f<KIND, 2>(Sp.lf[j], Sp.lf[l], Sp.fl[j], R.rl[j], Dm[i][j], Dm[j][l], dd[i][j], 0.f,
                                         rd[i][l], C)
                       : dd2s_f<KIND, 0>(Sp.lf[j], Sp.lf[l], Sp.fl[j], R.rl[j], Dm[i][j], Dm[j][l], dd[i][j],
                                         dd[j][l], rd[i][l], C);
        }
        D2[i][j][l] = D2[i][l][j] = D2[j][i][l] = D2[j][l][i] = D2[l][i][j] = D2[l][j][i] = d;
      }
}

// host: the FP32 launch constants of a call, from the FP64 ones
inline void smf_coef_f(int kind, double al, SmfCoefF &C) {
  SmfCoef D;
  smf_coef(kind, al, D);
  C.al = (float)al;
  C.alm1 = (float)(al - 1.0);
  C.zp1 = (float)D.zp1;
  C.z2 = (float)D.z2;
  const bool pw = kind == POW || kind == SQRT;
  // (the FP32 form keeps its own cluster radius: 0.25 for exp / log (exp: the spread of the three points <= 1), 0.5
  // or 3 / al for powers, with its own term count)
  C.tau = (float)(pw ? (3.0 / al < DD2_TAU_F_POW ? 3.0 / al : DD2_TAU_F_POW) : DD2_TAU);
  for (int k = 0; k < DD2_TERMS; k++) C.c2[k] = (float)D.c2[k];
  // g1: binom(al, 2m + 1); the series is used where the magnitudes of its terms at |z| = 1/2 add up to at most 4 al
  // (its sum, g, is al at z = 0) and its last term is below 1e-9 al: exponents up to about 7, not al = 60.5
  double b = al, tot = 0.0;  // binom(al, 1)
  bool ok = kind == POW && al > 0.0;
  for (int m = 0; m < G1_TERMS_F; m++) {
    C.g1[m] = (float)b;
    tot += std::fabs(b) * std::pow(0.25, m);
    if (m == G1_TERMS_F - 1) ok &= std::fabs(b) * std::pow(0.25, m) <= 1e-9 * al;
    b = b * (al - (2 * m + 1)) * (al - (2 * m + 2)) / ((2.0 * m + 2) * (2.0 * m + 3));  // binom(al, 2m + 3)
  }
  C.g1ser = ok && tot <= 4.0 * al ? 1 : 0;
}

}  // namespace mf
