// smf_device.cuh -- per-matrix device math of the symmetric family (FP64, one thread per matrix), the method of the
// reference's c/include/matfun/smf_kernel.hpp (Daleckii-Krein forms over a closed-form eigensystem):
//   * the eigensystem of a symmetric 3x3 matrix: its deviator's eigenvalue farthest from the other two by the
//     trigonometric formula (Smith), that eigenvalue's eigenvector as the longest cross product of two rows of the
//     shifted deviator, an orthonormal complement, and the remaining pair by a Jacobi rotation of the 2x2 block;
//     eigenvalues as Rayleigh quotients of A (and of the deviator, for log near the mean)
//   * f of the eigenvalues (log through log1p near the mean)
//   * the first and second divided differences f[a, b], f[x, y, z] with their stable forms for close arguments
// and the eigen-basis quantities the kernels contract into J and H:
//   Et_p = V^T E_p V for the six Voigt basis matrices E_p,
//   J_{I,p}   = w_I  K(I, p),       K(X, Y)    = sum_ab D_ab X_ab Y_ab                       (21 distinct)
//   H_{I,p,q} = w_I  G'(I, p, q),   G'(X, Y, Z) = 2 sum_amb D2_amb X_ab Y_am Z_mb           (56 distinct)
// with w_I = 1 for a diagonal and 1/2 for an off-diagonal Voigt index I.  K and G' are symmetric in all their
// arguments (D and D2 are symmetric, the Et are symmetric matrices), so only the sorted index tuples are computed;
// the reference assembles all 36 / 126 entries (smf_kernel.hpp:297-381).  The branch thresholds of the divided
// differences and of the eigensystem are the method's (they define the result the parity tests hold this code to).
#pragma once
#include "mf_common.cuh"

namespace mf {

constexpr int DD2_TERMS = 30;  // smf_kernel.hpp:132
constexpr double DD2_TAU = 0.25;

// launch constants of the smf kernels (computed on the host once per call)
struct SmfCoef {
  double al;                // exponent (pow), 0.5 (sqrt), 0 otherwise
  double bh1, bl1;          // al - 1 split exactly (TwoSum)
  double zp1;               // 0^(al - 1)
  double z2;                // f''(0)/2 for powers: 0 (al == 1) or binom(al, 2) 0^(al - 2)
  double tau;               // cluster radius of the second divided difference (exp: absolute, else relative)
  int nterms;               // terms of its cluster series (<= DD2_TERMS)
  double c2[DD2_TERMS];     // Taylor coefficients f^(k+2)/(k+2)! without the m-dependent factor (smf_kernel.hpp:135-146)
};

// host: the launch constants of a call (kind already normalised: sqrt has al = 0.5)
inline void smf_coef(int kind, double al, SmfCoef &C) {
  C.al = al;
  double bh = al - 1.0, bb = bh - al;
  C.bh1 = bh;
  C.bl1 = (al - (bh - bb)) + (-1.0 - bb);
  auto zpow = [](double e) { return e < 0 ? HUGE_VAL : (e == 0 ? 1.0 : 0.0); };
  C.zp1 = zpow(al - 1.0);
  C.z2 = al == 1.0 ? 0.0 : al * (al - 1.0) / 2.0 * zpow(al - 2.0);
  C.tau = (kind == POW && 3.0 / al < DD2_TAU) ? 3.0 / al : DD2_TAU;
  if (kind == EXP) {
    double f = 0.5;
    for (int k = 0; k < DD2_TERMS; k++) { C.c2[k] = f; f /= (k + 3.0); }
  } else if (kind == LOG) {
    for (int k = 0; k < DD2_TERMS; k++) C.c2[k] = (k % 2 ? 1.0 : -1.0) / (k + 2.0);
  } else {
    double b = al * (al - 1.0) / 2.0;
    for (int k = 0; k < DD2_TERMS; k++) { C.c2[k] = b; b *= (al - k - 2.0) / (k + 3.0); }
  }
  // The cluster series is needed only where the difference formula (f[md, hi] - f[lo, md]) / (hi - lo) cancels: its
  // relative error is about 2 eps f' / ((hi - lo) f''), i.e. 2 eps lambda / (hi - lo) for log, eps / (hi - lo) for exp
  // and 2 eps lambda / (|al - 1| (hi - lo)) for powers.  So the FP64 path takes the series only within 2^-6 of the
  // middle point (exp: absolute 2^-4), where about 10 terms reach 1e-17 of the first (the difference formula is then
  // within 150 eps beyond it), instead of within 0.25 with 30 terms; powers with |al - 1| < 1/4 (f'' small) or al > 12
  // (growing binomial coefficients) keep 0.25 (3 / al for al > 12) and 30 terms.
  const bool narrow = kind == EXP || kind == LOG || (std::fabs(al - 1.0) >= 0.25 && al <= 12.0);
  if (narrow) {
    C.tau = kind == EXP ? 0.0625 : 0.015625;
    // the terms of sum_k c2[k] h_k(u, w), |h_k| <= (k + 1) tau^k: stop where the bound of every later term is below
    // 2^-57 of |c2[0]| (the bound decreases from there on for these coefficients)
    int n = DD2_TERMS;
    for (int k = 1; k < DD2_TERMS; k++) {
      const double bnd = std::fabs(C.c2[k]) * (k + 1) * std::pow(C.tau, k);
      if (bnd <= 0x1p-57 * std::fabs(C.c2[0]) || C.c2[0] == 0.0) { n = k; break; }
    }
    C.nterms = n;
  } else {
    C.nterms = DD2_TERMS;
  }
}

template <int KIND>
MF_D double smf_fun(double x, double al) {
  if (KIND == EXP) return exp(x);
  if (KIND == LOG) return log(x);
  if (!(x > 0)) return 0.0;
  return KIND == SQRT ? sqrt(x) : pow(x, al);
}

// eigenvalues lam and eigenvectors V (columns) of the symmetric matrix with Voigt vector v; for log also the
// deviator's Rayleigh quotients xd[i] = lam[i] / sig - m and m, sig (the log1p form near the mean)
struct SmfEig {
  double lam[3], V[3][3], xd[3], m, sig;
};

// y = M x for the symmetric M with diagonal (d0, d1, d2) and off-diagonal (o01, o02, o12)
MF_D void symv3(double d0, double d1, double d2, double o01, double o02, double o12, const double *x, double *y) {
  y[0] = d0 * x[0] + o01 * x[1] + o02 * x[2];
  y[1] = o01 * x[0] + d1 * x[1] + o12 * x[2];
  y[2] = o02 * x[0] + o12 * x[1] + d2 * x[2];
}
MF_D double sdot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
MF_D void scross3(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

template <int KIND>
MF_D void smf_eigsys(const double *v, SmfEig &E) {
  constexpr double SQRT6 = 2.449489742783178, TWO_PI_3 = 2.0943951023931957;
  // 1. an exact power-of-two scale sig ~ max |v| (products up to |A|^4 below then neither overflow nor underflow)
  const double sig = pow2floor(tmax(tmax(tmax(fabs(v[0]), fabs(v[1])), tmax(fabs(v[2]), fabs(v[3]))),
                                    tmax(fabs(v[4]), fabs(v[5]))) + 1e-300);
  const double is = 1.0 / sig;
  double a[6];
#pragma unroll
  for (int k = 0; k < 6; k++) a[k] = v[k] * is;
  // 2. the deviator d = A - m I, and its traceless part (the rounding residue of m removed) normalised by a power of
  //    two: g = (d - tr(d) / 3 I) / 2^k, so that the closed form sees a traceless matrix of magnitude ~1
  const double m = (a[0] + a[1] + a[2]) / 3.0;
  const double d[3] = {a[0] - m, a[1] - m, a[2] - m};
  const double res = (d[0] + d[1] + d[2]) / 3.0;
  const double e[3] = {d[0] - res, d[1] - res, d[2] - res};
  const double dmax = tmax(tmax(tmax(fabs(e[0]), fabs(e[1])), tmax(fabs(e[2]), fabs(a[3]))),
                           tmax(fabs(a[4]), fabs(a[5])));
  const bool iso = dmax <= 1e-300;  // A = m I: every vector is an eigenvector
  const double ig = iso ? 1.0 : 1.0 / pow2floor(dmax);
  const double g0 = e[0] * ig, g1 = e[1] * ig, g2 = e[2] * ig, g3 = a[3] * ig, g4 = a[4] * ig, g5 = a[5] * ig;
  // 3. the root of the normalised deviator farthest from the other two: with p = tr g^2, q = det g, cos(3 phi) =
  //    3 sqrt(6) q / p^(3/2), root = sqrt(2 p / 3) cos(phi) (phi + 2 pi / 3 for a negative cosine)
  double p = g0 * g0 + g1 * g1 + g2 * g2 + 2.0 * (g3 * g3 + g4 * g4 + g5 * g5);
  double q = g0 * (g1 * g2 - g5 * g5) - g3 * (g3 * g2 - g5 * g4) + g4 * (g3 * g5 - g1 * g4);
  if (iso) { p = 1.0; q = 0.0; }
  double c3 = 3.0 * SQRT6 * q / (p * sqrt(p));
  c3 = c3 > 1.0 ? 1.0 : (c3 < -1.0 ? -1.0 : c3);
  const double phi = acos(c3) / 3.0;
  const double root = sqrt(2.0 * p / 3.0) * cos(c3 >= 0 ? phi : phi + TWO_PI_3);
  // 4. its eigenvector: the longest cross product of two rows of g - root I
  const double r0[3] = {g0 - root, g3, g4}, r1[3] = {g3, g1 - root, g5}, r2[3] = {g4, g5, g2 - root};
  double c[3][3];
  scross3(r0, r1, c[0]);
  scross3(r0, r2, c[1]);
  scross3(r1, r2, c[2]);
  double vv[3] = {c[0][0], c[0][1], c[0][2]}, nn = sdot3(c[0], c[0]);
#pragma unroll
  for (int t = 1; t < 3; t++) {
    const double nt = sdot3(c[t], c[t]);
    if (nt > nn) {
      nn = nt;
      vv[0] = c[t][0]; vv[1] = c[t][1]; vv[2] = c[t][2];
    }
  }
  const double nrm = sqrt(nn);
  double vx[3] = {1.0, 0.0, 0.0};
  if ((nrm > 1e-300) & !iso) {
    const double in = 1.0 / nrm;
    vx[0] = vv[0] * in; vx[1] = vv[1] * in; vx[2] = vv[2] * in;
  }
  // 5. an orthonormal complement: u from the coordinate axis least aligned with v (less its v component), w = v x u
  const double b0 = fabs(vx[0]), b1 = fabs(vx[1]), b2 = fabs(vx[2]);
  const bool ay = b1 < b0, az = b2 < (ay ? b1 : b0);
  const int ax = az ? 2 : (ay ? 1 : 0);
  const double va = ax == 0 ? vx[0] : (ax == 1 ? vx[1] : vx[2]);
  double u[3] = {(ax == 0 ? 1.0 : 0.0) - va * vx[0], (ax == 1 ? 1.0 : 0.0) - va * vx[1],
                 (ax == 2 ? 1.0 : 0.0) - va * vx[2]};
  const double nu = sqrt(sdot3(u, u));
  if (nu > 1e-300) {
    const double in = 1.0 / nu;
    u[0] *= in; u[1] *= in; u[2] *= in;
  } else {
    u[0] = u[1] = u[2] = 0.0;
  }
  double w[3];
  scross3(vx, u, w);
  // 6. Rayleigh quotients: of A (the eigenvalues, accurate over spectra of many orders of magnitude) and of the
  //    deviator d (its 2x2 block gives the Jacobi angle without the cancellation of A's near I)
  double Au[3], Aw[3], Av[3], Du[3], Dw[3];
  symv3(a[0], a[1], a[2], a[3], a[4], a[5], u, Au);
  symv3(a[0], a[1], a[2], a[3], a[4], a[5], w, Aw);
  symv3(a[0], a[1], a[2], a[3], a[4], a[5], vx, Av);
  symv3(d[0], d[1], d[2], a[3], a[4], a[5], u, Du);
  symv3(d[0], d[1], d[2], a[3], a[4], a[5], w, Dw);
  const double a11 = sdot3(u, Au), a12 = sdot3(u, Aw), a22 = sdot3(w, Aw), lv = sdot3(vx, Av);
  const double b11 = sdot3(u, Du), b12 = sdot3(u, Dw), b22 = sdot3(w, Dw);
  // 7. the Jacobi rotation (cos, sin of half the angle atan2(2 b12, b11 - b22)) by the half-angle formulas, the larger
  //    eigenvalue of the block first
  const double jx = b11 - b22, jy = 2.0 * b12, jr = sqrt(jx * jx + jy * jy);
  double cs = 1.0, sn = 0.0;
  if (jr != 0) {
    const double big = sqrt((jr + fabs(jx)) / (2.0 * jr)), sml = jy / (2.0 * jr * big);
    const double sg = ((jy > 0) | ((jy == 0) & (__double_as_longlong(jy) >= 0))) ? 1.0 : -1.0;
    if (jx >= 0) { cs = big; sn = sml; }
    else { cs = sg * sml; sn = sg * big; }
  }
  E.lam[0] = lv * sig;
  E.lam[1] = (cs * cs * a11 + 2.0 * cs * sn * a12 + sn * sn * a22) * sig;
  E.lam[2] = (sn * sn * a11 - 2.0 * cs * sn * a12 + cs * cs * a22) * sig;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    E.V[k][0] = vx[k];
    E.V[k][1] = cs * u[k] + sn * w[k];
    E.V[k][2] = cs * w[k] - sn * u[k];
  }
  E.m = m;
  E.sig = sig;
  if (KIND == LOG) {
    double Dv[3];
    symv3(d[0], d[1], d[2], a[3], a[4], a[5], vx, Dv);
    E.xd[0] = sdot3(vx, Dv);
    E.xd[1] = cs * cs * b11 + 2.0 * cs * sn * b12 + sn * sn * b22;
    E.xd[2] = sn * sn * b11 - 2.0 * cs * sn * b12 + cs * cs * b22;
  }
}

// eigenvalues lam, f(lam), eigenvectors V (columns) of the symmetric matrix with Voigt vector v (FP64)
template <int KIND>
MF_D void smf_eigen(const double *v, double al, double lam[3], double fl[3], double V[3][3]) {
  SmfEig E;
  smf_eigsys<KIND>(v, E);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    lam[i] = E.lam[i];
#pragma unroll
    for (int j = 0; j < 3; j++) V[i][j] = E.V[i][j];
    if (KIND != LOG) fl[i] = smf_fun<KIND>(lam[i], al);
  }
  if (KIND == LOG) {
    // near m (|x| <= m / 2, x = lam - m from the deviator): log(m sig) + log1p(x / m); else log(lam).  One logarithm
    // per eigenvalue serves both: u = 1 + x / m near m (then log1p(x / m) = log(u) (x / m) / (u - 1), exact u - 1 by
    // Sterbenz, x / m where u rounds to 1 -- Goldberg's form of log1p, a few ulps), u = lam otherwise.
    const double lms = log(E.m * E.sig);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const bool near = fabs(E.xd[i]) <= 0.5 * E.m;
      const double y = E.xd[i] / E.m, u = near ? 1.0 + y : lam[i], L = log(u), um1 = u - 1.0;
      fl[i] = near ? lms + (um1 == 0.0 ? y : L * (y / um1)) : L;
    }
  }
}

// ---- first divided differences f[a, b] (f[a, a] = f'(a)) in forms stable for close arguments
// exp: e^max(a, b) (1 - e^-d) / d, d = |a - b| (no overflow, no cancellation)
// log: with s = (a + b) / 2, z = (a - b) / (a + b): log a - log b = 2 atanh z, so f[a, b] = 2 atanh(z) / (a - b)
//      = atanh(z) / (z s) for |z| < 0.5 (1 / s at z = 0; z's rounding reaches the result at about an ulp, and no
//      separate series is needed near z = 0), and the plain quotient (fa - fb) / (a - b)
//      of the logarithms already at hand for |z| >= 0.5 (a / b >= 3: their difference is >= log 3, so it is as
//      accurate as log a - log b evaluated anew).  Two forms instead of three: the lanes of a warp split between them,
//      and the warp pays for every form one of its lanes takes.
// sqrt: 1 / (sqrt a + sqrt b) (arguments clamped at 0: PSD round-off)
// powers: with s the mean and z = (a - b) / (2 s): a^al - b^al = s^al ((1 + z)^al - (1 - z)^al), so
//      f[a, b] = s^(al - 1) (expm1(al log1p z) - expm1(al log1p(-z))) / (2 z) for 0 < |z| < 0.5, al s^(al - 1) at
//      z = 0, the plain quotient beyond
template <int KIND>
MF_D double smf_dd1(double a, double b, double fa, double fb, const SmfCoef &C) {
  if (KIND == EXP) {
    const double d = fabs(a - b);
    const double fmax = a > b ? fa : fb;
    return d > 0 ? fmax * (-expm1(-d) / d) : fmax;
  }
  if (KIND == LOG) {
    // (atanh(z) / z) / s = 2 atanh(z) / (a - b): both forms are products with 1 / (a - b), the quotient's only
    // division (an FP64 division costs several FP64 instructions; z = 0: 1 / s)
    const double r = 1.0 / (a + b), z = (a - b) * r, az = fabs(z);
    const double dab = a - b, rd = 1.0 / (dab != 0.0 ? dab : 1.0);
    if (az >= 0.5) return (fa - fb) * rd;
    return z != 0.0 ? 2.0 * atanh(z) * rd : 2.0 * r;
  }
  a = a > 0 ? a : 0.0;
  b = b > 0 ? b : 0.0;
  if (KIND == SQRT) return 1.0 / (sqrt(a) + sqrt(b));
  const double s = 0.5 * (a + b), sp = s > 0 ? s : 1.0;
  const double dab = a - b, rd = 1.0 / (dab != 0.0 ? dab : 1.0);  // (1 / (2 z) = sp / (a - b))
  const double z = dab * (s > 0 ? 1.0 / (a + b) : 0.5), az = fabs(z);
  if (az >= 0.5) return (fa - fb) * rd;
  const double g = az == 0 ? C.al : (expm1(C.al * log1p(z)) - expm1(C.al * log1p(-z))) * (sp * rd);
  return (s > 0 ? pow_split(sp, C.bh1, C.bl1) : C.zp1) * g;
}

// f'(x) = f[x, x]
template <int KIND>
MF_D double smf_deriv(double x, double fx, const SmfCoef &C) {
  if (KIND == EXP) return fx;
  if (KIND == LOG) return 1.0 / x;
  x = x > 0 ? x : 0.0;
  if (KIND == SQRT) return 1.0 / (2.0 * sqrt(x));
  return C.al * (x > 0 ? pow_split(x, C.bh1, C.bl1) : C.zp1);
}

// ---- second divided differences f[x, y, z] (symmetric; f[x, x, x] = f''(x) / 2).  With the three points sorted,
// lo <= md <= hi: a cluster (exp: hi - lo <= 1; log, powers: lo and hi within tau md of md > 0) by the Taylor series
// about md, f[x, y, z] = sum_k f^(k+2)(md) / (k+2)! h_k(lo - md, hi - md), h_k(u, w) = sum_i u^i w^(k-i) (30 terms:
// the coefficients c2 without their md-dependent factor e^md, 1 / md^2 or md^(al - 2) = f(md) / md^2); otherwise the
// difference over the most distant pair, (f[md, hi] - f[lo, md]) / (hi - lo).  Powers: arguments clamped at 0, and
// f''(0) / 2 where all three are 0.
template <int KIND>
MF_D double smf_dd2(double li, double lj, double lk, double fi, double fj, double fk, double Dij, double Dik,
                    double Djk, const SmfCoef &C) {
  if (KIND == POW || KIND == SQRT) {
    li = li > 0 ? li : 0.0; lj = lj > 0 ? lj : 0.0; lk = lk > 0 ? lk : 0.0;
  }
  // sort (i, j, k) into (lo, md, hi), carrying f and the first differences of the pairs
  double x0 = li, x1 = lj, x2 = lk, f0 = fi, f1 = fj, f2 = fk, d01 = Dij, d02 = Dik, d12 = Djk, t;
  if (x1 < x0) { t = x0; x0 = x1; x1 = t; t = f0; f0 = f1; f1 = t; t = d02; d02 = d12; d12 = t; }
  if (x2 < x1) { t = x1; x1 = x2; x2 = t; t = f1; f1 = f2; f2 = t; t = d01; d01 = d02; d02 = t; }
  if (x1 < x0) { t = x0; x0 = x1; x1 = t; t = f0; f0 = f1; f1 = t; t = d02; d02 = d12; d12 = t; }
  const double lo = x0, md = x1, hi = x2;
  bool cluster;
  double u, w, scale;
  if (KIND == EXP) {
    cluster = (md - lo <= C.tau) & (hi - md <= C.tau);
    u = lo - md; w = hi - md; scale = f1;
  } else {
    cluster = (md > 0) & (md - lo <= C.tau * md) & (hi - md <= C.tau * md);
    const double im = 1.0 / md;  // (one division for the offsets and the scale)
    u = (lo - md) * im; w = (hi - md) * im;
    scale = (KIND == LOG ? im : f1 * im) * im;
  }
  double out;
  if (cluster) {
    double h = 1.0, wk = 1.0, acc = C.c2[0];
#pragma unroll 4
    for (int k = 1; k < C.nterms; k++) {  // h_k = u h_(k-1) + w^k
      wk = wk * w;
      h = u * h + wk;
      acc = acc + C.c2[k] * h;
    }
    out = scale * acc;
  } else {
    const double span = hi - lo;
    out = (d12 - d01) / (span != 0 ? span : 1.0);
  }
  if (KIND == POW || KIND == SQRT) out = hi > 0 ? out : C.z2;
  return out;
}

// f[l, l, l] = f''(l) / 2: the cluster series at u = w = 0 is its first coefficient times the scale; where l lies
// outside the cluster test (log, powers at l <= 0) the difference form gives (D_ll - D_ll) / 1
template <int KIND>
MF_D double smf_dd2_same(double l, double fl, double Dll, const SmfCoef &C) {
  if (KIND == POW || KIND == SQRT) l = l > 0 ? l : 0.0;
  double out;
  if (KIND == EXP) out = fl * C.c2[0];
  else out = l > 0 ? ((KIND == LOG ? 1.0 : fl) / (l * l)) * C.c2[0] : Dll - Dll;  // (l > 0: always in the cluster)
  if (KIND == POW || KIND == SQRT) out = l > 0 ? out : C.z2;
  return out;
}

// Voigt basis pair (k, l) of component p
MF_D constexpr int vk_(int p) { return p < 3 ? p : (p == 5 ? 1 : 0); }
MF_D constexpr int vl_(int p) { return p < 3 ? p : (p == 3 ? 1 : 2); }

// Et_p = V^T E_p V as the 6 entries (00, 11, 22, 01, 02, 12) of a symmetric matrix
MF_D void smf_et(double V[3][3], double Et[6][6]) {
#pragma unroll
  for (int p = 0; p < 6; p++) {
    const int k = vk_(p), l = vl_(p);
#pragma unroll
    for (int s = 0; s < 6; s++) {
      const int a = vk_(s), b = vl_(s);
      double e = V[k][a] * V[l][b];
      if (k != l) e += V[l][a] * V[k][b];
      Et[p][s] = e;
    }
  }
}

}  // namespace mf
