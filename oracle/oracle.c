/* oracle.c -- CPU restatement of matfun's batched 3x3 matrix functions (exp, log, sqrt, x^alpha; F, J, H) for
 * symmetric (smf, Voigt or matrix layout) and general (gmf) matrices.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker of the CUDA library and the scalar CPU baseline of the
 * benchmark; the product path never calls it.  It restates, in plain scalar C, the algorithm of
 *   c/include/matfun/smf_kernel.hpp   (symmetric: closed-form eigensystem, Daleckii-Krein divided differences)
 *   c/include/matfun/gmf_kernel.hpp   (general: cubic roots + refinement, confluent Newton-Hermite form)
 *   c/src/matfun.cc                   (argument checks, return codes, OpenMP over chunks)
 * with the same branch thresholds, so that results agree with the reference to rounding.  Where the reference
 * computes both sides of a branch and selects (it is written for SIMD lanes), this file evaluates only the taken side.
 * It is pinned against the reference's golden vectors (testdata/cases.txt, testdata/cases_general.txt, converted to
 * tests/golden/) and, where the reference library can be compiled (oracle/Makefile.ref), against it directly.
 *
 * C ABI (same signatures, layouts and codes as the reference's c/include/matfun/matfun.h:28-41):
 *   int orc_smf_eval(int kind, double alpha, int64_t n, const double *v, double *F, double *J, double *H);
 *   int orc_smf_eval_matrix(...);   -3 if a matrix is not symmetric (its results NaN)
 *   int orc_gmf_eval(...);
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { K_EXP = 0, K_LOG = 1, K_POW = 2, K_SQRT = 3 };

/* ------------------------------------------------------------------------------------------------ scalar helpers */
static inline double maxd(double a, double b) { return a > b ? a : b; } /* NaN in a: b (select semantics) */
static inline double mind(double a, double b) { return a < b ? a : b; }
/* largest power of two <= x (x > 0 normal): smf_kernel.hpp:53-54 */
static inline double pow2floor(double x) { return ldexp(1.0, ilogb(x)); }
/* 0^e: smf_kernel.hpp:57-58 */
static inline double zero_pow(double e) { return e < 0 ? INFINITY : (e == 0 ? 1.0 : 0.0); }
/* x^(al-k) with al-k split exactly into bh + bl (TwoSum), x^bh (1 + bl log x): smf_kernel.hpp:66-73 */
static double pow_split(double x, double al, double k) {
  const double bh = al - k, bb = bh - al, bl = (al - (bh - bb)) + (-k - bb);
  const double p = pow(x, bh);
  return bl == 0 ? p : p * (1.0 + bl * log(x));
}

/* ====================================================================================================== smf */
/* f(x): smf_kernel.hpp:75-82 (powers: negative round-off clamped to 0) */
static double fun(int kind, double x, double al) {
  if (kind == K_EXP) return exp(x);
  if (kind == K_LOG) return log(x);
  if (!(x > 0)) return 0.0;
  return kind == K_SQRT ? sqrt(x) : pow(x, al);
}

/* first divided difference f[a, b], stable forms: smf_kernel.hpp:84-115 */
static double divdiff(int kind, double a, double b, double fa, double fb, double al) {
  if (kind == K_EXP) {
    const double d = fabs(a - b);
    return (a > b ? fa : fb) * (d > 0 ? -expm1(-d) / d : 1.0);
  }
  if (kind == K_LOG) {
    const double s = 0.5 * (a + b), z = (a - b) / (a + b), az = fabs(z), z2 = z * z;
    if (az < 1e-3) return (1.0 + z2 / 3.0 + z2 * z2 / 5.0 + z2 * z2 * z2 / 7.0) / s;
    if (az >= 0.5) return (log(a) - log(b)) / (a - b);
    return atanh(z) / z / s;
  }
  a = a > 0 ? a : 0.0;
  b = b > 0 ? b : 0.0;
  if (kind == K_SQRT) return 1.0 / (sqrt(a) + sqrt(b));
  const double s = 0.5 * (a + b), ss = s > 0 ? s : 1.0;
  const double z = (a - b) / (2.0 * ss), az = fabs(z);
  const int zero = az == 0, near = !zero && az < 0.5;
  if (!zero && !near) return (fa - fb) / (a - b);
  const double g = zero ? al : (expm1(al * log1p(z)) - expm1(al * log1p(-z))) / (2.0 * z);
  return (s > 0 ? pow_split(ss, al, 1.0) : zero_pow(al - 1.0)) * g;
}

/* f'(x): smf_kernel.hpp:117-126 */
static double deriv(int kind, double x, double fx, double al) {
  if (kind == K_EXP) return fx;
  if (kind == K_LOG) return 1.0 / x;
  x = x > 0 ? x : 0.0;
  if (kind == K_SQRT) return 1.0 / (2.0 * sqrt(x));
  return x > 0 ? al * pow_split(x, al, 1.0) : al * zero_pow(al - 1.0);
}

#define DD2_TERMS 30  /* smf_kernel.hpp:132 */
#define DD2_TAU 0.25  /* smf_kernel.hpp:133 */
/* Taylor coefficients f^(k+2)(m)/(k+2)! without the m-dependent factor: smf_kernel.hpp:135-146 */
static void dd2_coef(int kind, double al, double *c) {
  if (kind == K_EXP) {
    double f = 0.5;
    for (int k = 0; k < DD2_TERMS; k++) { c[k] = f; f /= (k + 3.0); }
  } else if (kind == K_LOG) {
    for (int k = 0; k < DD2_TERMS; k++) c[k] = (k % 2 ? 1.0 : -1.0) / (k + 2.0);
  } else {
    double b = al * (al - 1.0) / 2.0;
    for (int k = 0; k < DD2_TERMS; k++) { c[k] = b; b *= (al - k - 2.0) / (k + 3.0); }
  }
}

/* second divided difference f[x, y, z]: recursion over the most distant pair, or the Taylor series around the middle
 * point inside a cluster: smf_kernel.hpp:148-192 */
static double divdiff2(int kind, double li, double lj, double lk, double fi, double fj, double fk, double Dij,
                       double Dik, double Djk, double al, const double *c) {
  if (kind == K_POW || kind == K_SQRT) {
    li = li > 0 ? li : 0.0; lj = lj > 0 ? lj : 0.0; lk = lk > 0 ? lk : 0.0;
  }
  const double dA = lk - li, dB = lj - li, dC = lk - lj, aA = fabs(dA), aB = fabs(dB), aC = fabs(dC);
  const int useA = aA >= aB && aA >= aC, useB = !useA && aB >= aC;
  const double num = useA ? Djk - Dij : (useB ? Djk - Dik : Dik - Dij);
  const double den = useA ? dA : (useB ? dB : dC);
  const double direct = num / (den != 0 ? den : 1.0);
  const double mn = li < lj ? li : lj, mx = li < lj ? lj : li;
  const double lo = mn < lk ? mn : lk, hi = mx > lk ? mx : lk, t = mx < lk ? mx : lk, mid = mn > t ? mn : t;
  const double fm = mid == li ? fi : (mid == lj ? fj : fk);
  int cluster;
  double u, w, scale;
  if (kind == K_EXP) {
    cluster = (hi - lo) <= 1.0;
    u = lo - mid; w = hi - mid; scale = fm;
  } else {
    const double tau = (kind == K_POW && 3.0 / al < DD2_TAU) ? 3.0 / al : DD2_TAU;
    cluster = (mid > 0) && (mid - lo <= tau * mid) && (hi - mid <= tau * mid);
    const double ms = cluster ? mid : 1.0;
    u = (lo - mid) / ms; w = (hi - mid) / ms;
    scale = (kind == K_LOG ? 1.0 : (cluster ? fm : 1.0)) / (ms * ms);
  }
  double out = direct;
  if (cluster) {
    double h = 1.0, wk = 1.0, s = c[0];
    for (int k = 1; k < DD2_TERMS; k++) { wk = wk * w; h = u * h + wk; s = s + c[k] * h; }
    out = scale * s;
  }
  if (kind == K_POW || kind == K_SQRT) {
    const double z2 = al == 1.0 ? 0.0 : al * (al - 1.0) / 2.0 * zero_pow(al - 2.0);
    out = hi > 0 ? out : z2;
  }
  return out;
}

/* Voigt index of (a, b), a <= b, and the Voigt pair of index p: smf_kernel.hpp:198, 316 */
static inline int vix(int a, int b) { return a == b ? a : a + b + 2; }
static const int VA[6] = {0, 1, 2, 0, 0, 1}, VB[6] = {0, 1, 2, 1, 2, 2};

/* one symmetric matrix (Voigt v) -> F[6], J[36] (or NULL), H[216] (or NULL): smf_kernel.hpp:200-382 */
static void smf_one(int kind, const double *v, double *F, double *J, double *H, double al, const double *c2) {
  const double SQRT6 = 2.449489742783178, TWO_PI_3 = 2.0943951023931957;
  /* power-of-two scaling (:203-211) */
  double sc = 0.0;
  for (int k = 0; k < 6; k++) sc = maxd(sc, fabs(v[k]));
  {  /* the reference's pairwise maximum tree, to keep NaN behaviour (:207-209) */
    const double s01 = maxd(fabs(v[0]), fabs(v[1])), s23 = maxd(fabs(v[2]), fabs(v[3]));
    const double s45 = maxd(fabs(v[4]), fabs(v[5])), s03 = maxd(s01, s23);
    sc = maxd(s03, s45) + 1e-300;
  }
  const double sig = pow2floor(sc), isig = 1.0 / sig;
  const double a0 = v[0] * isig, a1 = v[1] * isig, a2 = v[2] * isig, a3 = v[3] * isig, a4 = v[4] * isig,
               a5 = v[5] * isig;
  /* deviator less its trace residue, normalized by a power of two (:216-224) */
  const double m = (a0 + a1 + a2) / 3.0, d0 = a0 - m, d1 = a1 - m, d2 = a2 - m;
  const double tr3 = (d0 + d1 + d2) / 3.0, e0 = d0 - tr3, e1 = d1 - tr3, e2 = d2 - tr3;
  const double z01 = maxd(fabs(e0), fabs(e1)), z23 = maxd(fabs(e2), fabs(a3)), z45 = maxd(fabs(a4), fabs(a5));
  const double dmax = maxd(maxd(z01, z23), z45);
  const int iso = dmax <= 1e-300;
  const double ids = 1.0 / (iso ? 1.0 : pow2floor(dmax));
  const double g0 = e0 * ids, g1 = e1 * ids, g2 = e2 * ids, g3 = a3 * ids, g4 = a4 * ids, g5 = a5 * ids;
  /* the simple eigenvalue by Smith's trigonometric formula (:225-231) */
  const double p = g0 * g0 + g1 * g1 + g2 * g2 + 2.0 * (g3 * g3 + g4 * g4 + g5 * g5);
  const double q = g0 * (g1 * g2 - g5 * g5) - g3 * (g3 * g2 - g5 * g4) + g4 * (g3 * g5 - g1 * g4);
  const double pg = iso ? 1.0 : p, qg = iso ? 0.0 : q;
  double r = 3.0 * SQRT6 * qg / (pg * sqrt(pg));
  r = r > 1.0 ? 1.0 : (r < -1.0 ? -1.0 : r);
  const double t = sqrt(2.0 * pg / 3.0), ph = acos(r) / 3.0;
  const double sh = t * cos(r >= 0 ? ph : ph + TWO_PI_3);
  /* its eigenvector: the largest cross product of two rows of the shifted deviator (:232-244) */
  const double m00 = g0 - sh, m11 = g1 - sh, m22 = g2 - sh;
  const double cr[3][3] = {{g3 * g5 - g4 * m11, g4 * g3 - m00 * g5, m00 * m11 - g3 * g3},
                           {g3 * m22 - g4 * g5, g4 * g4 - m00 * m22, m00 * g5 - g3 * g4},
                           {m11 * m22 - g5 * g5, g5 * g4 - g3 * m22, g3 * g5 - m11 * g4}};
  double nr[3];
  for (int k = 0; k < 3; k++) nr[k] = cr[k][0] * cr[k][0] + cr[k][1] * cr[k][1] + cr[k][2] * cr[k][2];
  int best = 0;
  if (nr[1] > nr[0]) best = 1;
  if (nr[2] > nr[best]) best = 2;
  const double nrm = sqrt(nr[best]);
  const int ok = (nrm > 1e-300) && !iso;
  const double inv = 1.0 / (ok ? nrm : 1.0);
  const double vx = ok ? cr[best][0] * inv : 1.0, vy = ok ? cr[best][1] * inv : 0.0, vz = ok ? cr[best][2] * inv : 0.0;
  /* orthonormal complement u, w of v (:246-256) */
  const double ax = fabs(vx), ay = fabs(vy), az = fabs(vz);
  const int k1 = ay < ax, k2 = az < (k1 ? ay : ax);
  const double ex = (k1 || k2) ? 0.0 : 1.0, ey = (k1 && !k2) ? 1.0 : 0.0, ez = k2 ? 1.0 : 0.0;
  const double vk = ex * vx + ey * vy + ez * vz;
  double ux = ex - vk * vx, uy = ey - vk * vy, uz = ez - vk * vz;
  const double nu = sqrt(ux * ux + uy * uy + uz * uz);
  const int oku = nu > 1e-300;
  const double iu = 1.0 / (oku ? nu : 1.0);
  ux = oku ? ux * iu : 0.0; uy = oku ? uy * iu : 0.0; uz = oku ? uz * iu : 0.0;
  const double wx = vy * uz - vz * uy, wy = vz * ux - vx * uz, wz = vx * uy - vy * ux;
  /* Rayleigh quotients of A and of the deviator in the basis (v, u, w) (:259-266) */
  const double Aux = a0 * ux + a3 * uy + a4 * uz, Auy = a3 * ux + a1 * uy + a5 * uz, Auz = a4 * ux + a5 * uy + a2 * uz;
  const double Awx = a0 * wx + a3 * wy + a4 * wz, Awy = a3 * wx + a1 * wy + a5 * wz, Awz = a4 * wx + a5 * wy + a2 * wz;
  const double Avx = a0 * vx + a3 * vy + a4 * vz, Avy = a3 * vx + a1 * vy + a5 * vz, Avz = a4 * vx + a5 * vy + a2 * vz;
  const double a11 = ux * Aux + uy * Auy + uz * Auz, a12 = ux * Awx + uy * Awy + uz * Awz;
  const double a22 = wx * Awx + wy * Awy + wz * Awz, lv = vx * Avx + vy * Avy + vz * Avz;
  const double Dux = d0 * ux + a3 * uy + a4 * uz, Duy = a3 * ux + d1 * uy + a5 * uz, Duz = a4 * ux + a5 * uy + d2 * uz;
  const double Dwx = d0 * wx + a3 * wy + a4 * wz, Dwy = a3 * wx + d1 * wy + a5 * wz, Dwz = a4 * wx + a5 * wy + d2 * wz;
  const double b11 = ux * Dux + uy * Duy + uz * Duz, b12 = ux * Dwx + uy * Dwy + uz * Dwz;
  const double b22 = wx * Dwx + wy * Dwy + wz * Dwz;
  /* Jacobi rotation in span(u, w) by half-angle formulas (:268-275) */
  const double jx = b11 - b22, jy = 2.0 * b12, jr = sqrt(jx * jx + jy * jy);
  const int jz = jr == 0, jpos = jx >= 0;
  const double jrs = jz ? 1.0 : jr;
  const double big = sqrt((jrs + fabs(jx)) / (2.0 * jrs)), sml = jy / (2.0 * jrs * big);
  const double sgn = ((jy > 0) || (jy == 0 && !signbit(jy))) ? 1.0 : -1.0;
  const double cs = jz ? 1.0 : (jpos ? big : sgn * sml), sn = jz ? 0.0 : (jpos ? sml : sgn * big);
  const double lam[3] = {lv * sig, (cs * cs * a11 + 2.0 * cs * sn * a12 + sn * sn * a22) * sig,
                         (sn * sn * a11 - 2.0 * cs * sn * a12 + cs * cs * a22) * sig};
  const double V[3][3] = {{vx, cs * ux + sn * wx, cs * wx - sn * ux},
                          {vy, cs * uy + sn * wy, cs * wy - sn * uy},
                          {vz, cs * uz + sn * wz, cs * wz - sn * uz}};
  /* f of the eigenvalues; log near m from the deviator's Rayleigh quotients (:281-290) */
  double fl[3];
  for (int i = 0; i < 3; i++) fl[i] = fun(kind, lam[i], al);
  if (kind == K_LOG) {
    const double bv = vx * (d0 * vx + a3 * vy + a4 * vz) + vy * (a3 * vx + d1 * vy + a5 * vz) +
                      vz * (a4 * vx + a5 * vy + d2 * vz);
    const double xd[3] = {bv, cs * cs * b11 + 2.0 * cs * sn * b12 + sn * sn * b22,
                          sn * sn * b11 - 2.0 * cs * sn * b12 + cs * cs * b22};
    const double lms = log(m * sig);
    for (int i = 0; i < 3; i++)
      if (fabs(xd[i]) <= 0.5 * m) fl[i] = lms + log1p(xd[i] / m);
  }
  /* F = V diag(f) V^T (:291-295) */
  for (int x = 0; x < 3; x++)
    for (int y = x; y < 3; y++)
      F[vix(x, y)] = V[x][0] * fl[0] * V[y][0] + V[x][1] * fl[1] * V[y][1] + V[x][2] * fl[2] * V[y][2];
  if (!J) return;
  /* Daleckii-Krein (:297-327) */
  const double D01 = divdiff(kind, lam[0], lam[1], fl[0], fl[1], al);
  const double D02 = divdiff(kind, lam[0], lam[2], fl[0], fl[2], al);
  const double D12 = divdiff(kind, lam[1], lam[2], fl[1], fl[2], al);
  const double D[3][3] = {{deriv(kind, lam[0], fl[0], al), D01, D02},
                          {D01, deriv(kind, lam[1], fl[1], al), D12},
                          {D02, D12, deriv(kind, lam[2], fl[2], al)}};
  double P[3][3][3], Q[3][3][3];
  for (int i = 0; i < 3; i++)
    for (int x = 0; x < 3; x++)
      for (int y = 0; y < 3; y++) P[i][x][y] = V[x][i] * V[y][i];
  for (int i = 0; i < 3; i++)
    for (int x = 0; x < 3; x++)
      for (int y = 0; y < 3; y++) Q[i][x][y] = D[i][0] * P[0][x][y] + D[i][1] * P[1][x][y] + D[i][2] * P[2][x][y];
  for (int x = 0; x < 3; x++)
    for (int y = x; y < 3; y++)
      for (int k = 0; k < 6; k++) {
        const int pp = VA[k], qq = VB[k];
        double s = P[0][x][pp] * Q[0][y][qq] + P[1][x][pp] * Q[1][y][qq] + P[2][x][pp] * Q[2][y][qq];
        if (pp != qq) s += P[0][x][qq] * Q[0][y][pp] + P[1][x][qq] * Q[1][y][pp] + P[2][x][qq] * Q[2][y][pp];
        J[6 * vix(x, y) + k] = s;
      }
  if (!H) return;
  /* second order: D2 over the 10 distinct index triples, Et^p = V^T E_p V, S = X + X^T, H^pq = V S V^T (:328-381) */
  double D2[3][3][3];
  for (int i = 0; i < 3; i++)
    for (int j = i; j < 3; j++)
      for (int l = j; l < 3; l++) {
        const double d = divdiff2(kind, lam[i], lam[j], lam[l], fl[i], fl[j], fl[l], D[i][j], D[i][l], D[j][l], al, c2);
        D2[i][j][l] = D2[i][l][j] = D2[j][i][l] = D2[j][l][i] = D2[l][i][j] = D2[l][j][i] = d;
      }
  double Et[6][3][3];
  for (int pq = 0; pq < 6; pq++)
    for (int a = 0; a < 3; a++)
      for (int mm = a; mm < 3; mm++) {
        const int k = VA[pq], l = VB[pq];
        double e = V[k][a] * V[l][mm];
        if (k != l) e += V[l][a] * V[k][mm];
        Et[pq][a][mm] = Et[pq][mm][a] = e;
      }
  for (int pp = 0; pp < 6; pp++)
    for (int qq = pp; qq < 6; qq++) {
      double S[3][3], W[3][3];
      for (int a = 0; a < 3; a++)
        for (int b = a; b < 3; b++) {
          const double xab = D2[a][0][b] * Et[pp][a][0] * Et[qq][0][b] + D2[a][1][b] * Et[pp][a][1] * Et[qq][1][b] +
                             D2[a][2][b] * Et[pp][a][2] * Et[qq][2][b];
          const double xba = D2[b][0][a] * Et[pp][b][0] * Et[qq][0][a] + D2[b][1][a] * Et[pp][b][1] * Et[qq][1][a] +
                             D2[b][2][a] * Et[pp][b][2] * Et[qq][2][a];
          S[a][b] = S[b][a] = xab + xba;
        }
      for (int a = 0; a < 3; a++)
        for (int j = 0; j < 3; j++) W[a][j] = S[a][0] * V[j][0] + S[a][1] * V[j][1] + S[a][2] * V[j][2];
      for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
          const double h = V[i][0] * W[0][j] + V[i][1] * W[1][j] + V[i][2] * W[2][j];
          H[(6 * vix(i, j) + pp) * 6 + qq] = H[(6 * vix(i, j) + qq) * 6 + pp] = h;
        }
    }
}

/* matrix layout: Voigt index of matrix entry m = 3a + b and the derivative weight dv/dA_m: smf_kernel.hpp:384-389 */
static inline int mvix(int m) { return m % 4 == 0 ? m / 4 : (m == 1 || m == 3 ? 3 : (m == 2 || m == 6 ? 4 : 5)); }
static inline double mwt(int m) { return m % 4 == 0 ? 1.0 : 0.5; }

/* Voigt layout -> matrix layout of one matrix: smf_kernel.hpp:391-406 */
static void to_matrix(const double *Fv, const double *Jv, const double *Hv, double *F, double *J, double *H) {
  for (int m = 0; m < 9; m++) F[m] = Fv[mvix(m)];
  if (J)
    for (int m = 0; m < 9; m++)
      for (int c = 0; c < 9; c++) J[9 * m + c] = Jv[6 * mvix(m) + mvix(c)] * mwt(c);
  if (H)
    for (int m = 0; m < 9; m++)
      for (int c = 0; c < 9; c++)
        for (int e = 0; e < 9; e++) H[(9 * m + c) * 9 + e] = Hv[(6 * mvix(m) + mvix(c)) * 6 + mvix(e)] * (mwt(c) * mwt(e));
}

/* symmetric part of a full matrix as a Voigt vector; 0 and NaN if |a_ij - a_ji| > 1e-8 max|a|: smf_kernel.hpp:408-421 */
static int from_matrix(const double *a, double *v) {
  double mx = 0.0;
  for (int k = 0; k < 9; k++) mx = fabs(a[k]) > mx ? fabs(a[k]) : mx;
  const double tol = 1e-8 * mx;
  const int sym = !(fabs(a[1] - a[3]) > tol) && !(fabs(a[2] - a[6]) > tol) && !(fabs(a[5] - a[7]) > tol);
  v[0] = a[0]; v[1] = a[4]; v[2] = a[8];
  v[3] = 0.5 * (a[1] + a[3]); v[4] = 0.5 * (a[2] + a[6]); v[5] = 0.5 * (a[5] + a[7]);
  if (!sym)
    for (int k = 0; k < 6; k++) v[k] = NAN;
  return sym;
}

/* ====================================================================================================== gmf */
#define G_RHO 0.7        /* gmf_kernel.hpp:30 */
#define G_R_EXP 4.0
#define G_RHO_POLE 0.6
#define G_KMAX 200       /* gmf_kernel.hpp:31 */

typedef struct { double re, im; } cplx;
static inline cplx cmk(double re, double im) { cplx z = {re, im}; return z; }
static inline cplx cadd(cplx a, cplx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cplx csub(cplx a, cplx b) { return cmk(a.re - b.re, a.im - b.im); }
static inline cplx cmul(cplx a, cplx b) { return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cplx cscl(cplx a, double s) { return cmk(a.re * s, a.im * s); }
/* |a| without overflow of the squares: gmf_kernel.hpp:112-117 */
static double cabs_s(cplx a) {
  const double ar = fabs(a.re), ai = fabs(a.im), big = maxd(ar, ai), sml = mind(ar, ai);
  if (!(big > 0)) return 0.0;
  const double q = sml / big;
  return big * sqrt(1.0 + q * q);
}
/* 1 / b (Smith): gmf_kernel.hpp:118-125 */
static cplx cinv_s(cplx b) {
  const int sw = fabs(b.im) > fabs(b.re);
  const double p = sw ? b.im : b.re, q = sw ? b.re : b.im;
  const double r = q / (p != 0 ? p : 1.0), den = p + q * r;
  const double re = 1.0 / den, im = -r / den;
  return sw ? cmk(-im, -re) : cmk(re, im);
}
static inline double copysgn(double x, double y) { return y < 0 ? -fabs(x) : fabs(x); }
/* a power of two within a factor 2 of x (1 outside (1e-300, 1e300)): gmf_kernel.hpp:126-131 */
static inline double pow2safe(double x) { return (x > 1e-300 && x < 1e300) ? pow2floor(x) : 1.0; }

/* the 19 divided differences f[x0^a x1^b x2^c] (a >= b >= c, a >= 1) in lexicographic order of (a, b, c); each is
 * its parent with one node added (node 0 if a - 1 >= b, else node 1 if b - 1 >= c, else node 2); the first 3, 9, 19
 * serve orders 0, 1, 2 (gmf_kernel.hpp:34-37, 254-258) */
static int G_MS[19][3], G_PAR[19], G_NODE[19];
static int g_pos(int a, int b, int c) { return (a == 1 ? 0 : (a == 2 ? 3 : 9)) + b * (b + 1) / 2 + c; }
static void g_tables(void) {
  int idx = 0;
  for (int a = 1; a <= 3; a++)
    for (int b = 0; b <= a; b++)
      for (int c = 0; c <= b; c++) { G_MS[idx][0] = a; G_MS[idx][1] = b; G_MS[idx][2] = c; idx++; }
  for (int t = 0; t < 19; t++) {
    const int a = G_MS[t][0], b = G_MS[t][1], c = G_MS[t][2];
    if (t == 0) { G_PAR[t] = -1; G_NODE[t] = 0; continue; }
    if (a - 1 >= b) { G_PAR[t] = g_pos(a - 1, b, c); G_NODE[t] = 0; }
    else if (b - 1 >= c) { G_PAR[t] = g_pos(a, b - 1, c); G_NODE[t] = 1; }
    else { G_PAR[t] = g_pos(a, b, c - 1); G_NODE[t] = 2; }
  }
}
static inline int g_pos2(int j, int k) { return g_pos(2, (j >= 1) + (k >= 1), (j >= 2) + (k >= 2)); }
static inline int g_pos3(int j, int k, int l) {
  return g_pos(3, (j >= 1) + (k >= 1) + (l >= 1), (j >= 2) + (k >= 2) + (l >= 2));
}

/* series coefficients of f(c (1 + u)) / scale: gmf_kernel.hpp:48-53 */
static void series_coef(int kind, double al, double *b) {
  b[0] = 1.0;
  for (int j = 1; j < G_KMAX; j++)
    b[j] = kind == K_EXP ? b[j - 1] / j : (kind == K_LOG ? (j % 2 ? 1.0 : -1.0) / j : b[j - 1] * (al - j + 1) / j);
}

/* number of series terms from the term bound 1e-17: gmf_kernel.hpp:73-97 */
static int nterms(const double *b, int n, double r, double q) {
  int M = 1;
  if (r > 0) {
    double best = 0.0, c = 1.0, rk = 1.0;
    for (int k = 0; n + k < G_KMAX; k++) {
      const double t = fabs(b[n + k]) * c * rk;
      best = t > best ? t : best;
      M = k;
      if ((k > 2 && t <= 1e-17 * best) || !(rk > 0)) break;
      c = c * (k + n + 1) / (k + 1);
      rk *= r;
    }
  }
  if (q > 0) {
    double qk = 1.0;
    for (int k = 0; n + k < G_KMAX; k++) {
      if (k > M && (k + 1.0) * (k + 2.0) / 2.0 * qk <= 1e-17) break;
      M = k > M ? k : M;
      qk *= q;
    }
  }
  return n + M + 1 < G_KMAX ? n + M + 1 : G_KMAX;
}

static double det3(const double *M) {
  return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) + M[2] * (M[3] * M[7] - M[4] * M[6]);
}
/* det by elimination with partial pivoting: gmf_kernel.hpp:138-159 */
static double det_lu(const double *M) {
  const double a0 = fabs(M[0]), a1 = fabs(M[3]), a2 = fabs(M[6]);
  const int p1 = (a1 > a0) && (a1 >= a2), p2 = (a2 > a0) && (a2 > a1);
  double P[3], R1[3], R2[3];
  for (int c = 0; c < 3; c++) {
    P[c] = p1 ? M[3 + c] : (p2 ? M[6 + c] : M[c]);
    R1[c] = (p1 || p2) ? M[c] : M[3 + c];
    R2[c] = p2 ? M[3 + c] : M[6 + c];
  }
  double sgn = p1 ? -1.0 : 1.0;
  if (P[0] == 0) return 0.0;
  const double l1 = R1[0] / P[0], l2 = R2[0] / P[0];
  const double b = R1[1] - l1 * P[1], c = R1[2] - l1 * P[2], d = R2[1] - l2 * P[1], e = R2[2] - l2 * P[2];
  const int sw = fabs(d) > fabs(b);
  const double bb = sw ? d : b, cc = sw ? e : c, dd = sw ? b : d, ee = sw ? c : e;
  if (sw) sgn = -sgn;
  if (bb == 0) return 0.0;
  return sgn * P[0] * bb * (ee - dd / bb * cc);
}
/* sum of the principal 2x2 minors: gmf_kernel.hpp:161-164 */
static double minors2(const double *M) {
  return M[0] * M[4] - M[1] * M[3] + M[0] * M[8] - M[2] * M[6] + M[4] * M[8] - M[5] * M[7];
}

/* eigenvalues of the deviator S from x^3 - P x - Q (trigonometric / Cardano), normalized twice: gmf_kernel.hpp:166-208 */
static void roots3(const double *S, cplx *x) {
  const double TWO_PI_3 = 2.0943951023931957;
  const double tau = (S[0] + S[4] + S[8]) / 3.0;
  double Sp[9];
  for (int k = 0; k < 9; k++) Sp[k] = k % 4 == 0 ? S[k] - tau : S[k];
  double s = fabs(Sp[0]);
  for (int k = 1; k < 9; k++) s = maxd(s, fabs(Sp[k]));
  double t = pow2safe(s);
  const double it = 1.0 / t;
  for (int k = 0; k < 9; k++) Sp[k] = Sp[k] * it;
  double P = 0.5 * (Sp[0] * Sp[0] + Sp[4] * Sp[4] + Sp[8] * Sp[8]) + Sp[1] * Sp[3] + Sp[2] * Sp[6] + Sp[5] * Sp[7];
  double Q = det3(Sp);
  const double u = pow2safe(maxd(sqrt(fabs(P)), cbrt(fabs(Q)))), iu = 1.0 / u;
  P = P * iu * iu;
  Q = Q * iu * iu * iu;
  t = t * u;
  const int trig = (P > 0) && (4.0 * P * P * P >= 27.0 * Q * Q);
  double s1;
  if (trig) {
    const double p3 = P / 3.0;
    double r = 0.5 * Q / (p3 * sqrt(p3));
    r = r > 1.0 ? 1.0 : (r < -1.0 ? -1.0 : r);
    const double ph = acos(r) / 3.0;
    s1 = 2.0 * sqrt(p3) * cos(r >= 0 ? ph : ph + TWO_PI_3);
  } else {
    const double D = 0.25 * Q * Q - P * P * P / 27.0;
    const double uc = cbrt(0.5 * Q + copysgn(sqrt(D > 0 ? D : 0.0), Q));
    s1 = uc + (uc != 0 ? P / (3.0 * uc) : 0.0);
  }
  const double d = P - 0.75 * s1 * s1;  /* x^2 + s1 x + (s1^2 - P) = 0 */
  const int real = d >= 0;
  const double sq = sqrt(fabs(d));
  const double sa = -0.5 * s1 - copysgn(sq, s1);
  const double prod = s1 != 0 ? Q / s1 : -P;
  const double sb = sa != 0 ? prod / sa : 0.0;
  const double im = (real ? 0.0 : sq) * t;
  x[0] = cmk(s1 * t + tau, 0.0 * t);
  x[1] = cmk((real ? sa : -0.5 * s1) * t + tau, im);
  x[2] = cmk((real ? sb : -0.5 * s1) * t + tau, -im);
}

/* 3 Newton steps on det(A - mu_j I) for real node j, derivative from the other nodes: gmf_kernel.hpp:210-226 */
static void newton(const double *As, cplx *mu, int j) {
  for (int it = 0; it < 3; it++) {
    cplx den = cmk(1.0, 0.0);
    for (int k = 0; k < 3; k++)
      if (k != j) den = cmul(den, csub(mu[k], mu[j]));
    if (!(den.re != 0 || den.im != 0)) continue;
    double B[9];
    for (int k = 0; k < 9; k++) B[k] = k % 4 == 0 ? As[k] - mu[j].re : As[k];
    mu[j].re = mu[j].re + det_lu(B) * cinv_s(den).re;
  }
}

/* f(mu) of a node (k: output order; pow times sig^(al - k)): gmf_kernel.hpp:228-248 */
static cplx coef0(int kind, double al, double sig, double m, cplx x, cplx mu, int k) {
  if (kind == K_EXP) {
    const double e = exp(x.re);
    return cmk(e * cos(x.im), e * sin(x.im));
  }
  const double th = atan2(mu.im, mu.re);
  if (kind == K_LOG) {
    if (m > 0 && cabs_s(x) <= 0.5 * m) {
      const double zr = x.re / m, zi = x.im / m;
      return cmk(log(sig * m) + 0.5 * log1p(zr * (2.0 + zr) + zi * zi), atan2(zi, 1.0 + zr));
    }
    return cmk(log(sig * cabs_s(mu)), th);
  }
  const double mag = pow_split(sig * cabs_s(mu), al, (double)k), ph = (al - k) * th;
  cplx out = cmk(mag * cos(ph), mag * sin(ph));
  for (int i = 0; i < k; i++) out = cmul(out, mu);
  return out;
}

/* (N^T v) on one index of stride s: (N^T v)_0 = N10 v_1 + N20 v_2, (N^T v)_1 = N21 v_2, (N^T v)_2 = 0 (T = I + iN):
 * gmf_kernel.hpp:596-599 */
static inline void nt3(double N10, double N20, double N21, const double *v, double *o) {
  o[0] = N10 * v[1] + N20 * v[2];
  o[1] = N21 * v[2];
  o[2] = 0.0;
}

/* one general matrix: gmf_kernel.hpp:251-692 (order 0: F; 1: + J; 2: + H) */
static void gmf_one(int kind, int order, const double *a, double *F, double *J, double *H, double al,
                    const double *bt) {
  const int ND = order == 0 ? 3 : (order == 1 ? 9 : 19);
  /* scaling (exp: none), shift m, deviator S (:261-271) */
  double amax = fabs(a[0]);
  for (int k = 1; k < 9; k++) amax = maxd(amax, fabs(a[k]));
  const double sig = kind == K_EXP ? 1.0 : pow2safe(amax), isig = 1.0 / sig;
  double As[9], S[9];
  for (int k = 0; k < 9; k++) As[k] = a[k] * isig;
  const double m = (As[0] + As[4] + As[8]) / 3.0;
  for (int k = 0; k < 9; k++) S[k] = k % 4 == 0 ? As[k] - m : As[k];
  cplx x[3], mu[3];
  roots3(S, x);
  for (int i = 0; i < 3; i++) mu[i] = cmk(m + x[i].re, x[i].im);

  /* pair refinement from det A and the principal minors after Newton on mu0 (:277-304) */
  double smax = fabs(S[0]);
  for (int k = 1; k < 9; k++) smax = maxd(smax, fabs(S[k]));
  const double mid = 0.5 * (mu[1].re + mu[2].re), Rp = 0.5 * cabs_s(csub(mu[1], mu[2]));
  const int small = fabs(mid) + Rp <= 0.25 * fabs(mu[0].re);
  const int aniso = (fabs(m) <= smax) && (Rp <= 0.25 * fabs(mid - mu[0].re));
  int pc = (mu[0].re != 0) && (small || aniso);
  double pcen = 0.0, ps = 0.0;
  int preal = 1;
  if (pc) {
    newton(As, mu, 0);
    const double m0 = mu[0].re;
    const int big = fabs(m0) >= fabs(mid) + Rp;
    const double pid = det_lu(As) / m0, c2 = minors2(As);
    const double sgt = As[0] + As[4] + As[8] - m0;
    const double sg = big ? (c2 - pid) / m0 : sgt, pi = big ? pid : c2 - m0 * sgt;
    const double disc = 0.25 * sg * sg - pi;
    pcen = 0.5 * sg;
    ps = sqrt(fabs(disc));
    preal = disc >= 0;
    const double r1 = pcen + copysgn(ps, pcen);
    const double r2 = r1 != 0 ? pi / r1 : pcen - copysgn(ps, pcen);
    mu[1] = preal ? cmk(r1, 0.0) : cmk(pcen, ps);
    mu[2] = preal ? cmk(r2, 0.0) : cmk(pcen, -ps);
  }
  /* a pair near the negative real axis (log, pow): from the 2x2 block of the deviator on the complement of the left
   * eigenvector of mu0 (:305-367) */
  const int cut = kind != K_EXP && (mu[1].re + mu[2].re < 0);
  if (cut) {
    if (!pc) newton(As, mu, 0);
    const double l0 = mu[0].re;
    double Mc[9];
    for (int k = 0; k < 9; k++) Mc[k] = k % 4 == 0 ? As[k] - l0 : As[k];
    /* cross products of the columns (c0 x c1, c0 x c2, c1 x c2) */
    const double c01[3] = {Mc[3] * Mc[7] - Mc[6] * Mc[4], Mc[6] * Mc[1] - Mc[0] * Mc[7], Mc[0] * Mc[4] - Mc[3] * Mc[1]};
    const double c02[3] = {Mc[3] * Mc[8] - Mc[6] * Mc[5], Mc[6] * Mc[2] - Mc[0] * Mc[8], Mc[0] * Mc[5] - Mc[3] * Mc[2]};
    const double c12[3] = {Mc[4] * Mc[8] - Mc[7] * Mc[5], Mc[7] * Mc[2] - Mc[1] * Mc[8], Mc[1] * Mc[5] - Mc[4] * Mc[2]};
    const double n01 = c01[0] * c01[0] + c01[1] * c01[1] + c01[2] * c01[2];
    const double n02 = c02[0] * c02[0] + c02[1] * c02[1] + c02[2] * c02[2];
    const double n12 = c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2];
    double u[3], nn;
    if (n02 > n01) { memcpy(u, c02, sizeof u); nn = n02; } else { memcpy(u, c01, sizeof u); nn = n01; }
    if (n12 > nn) { memcpy(u, c12, sizeof u); nn = n12; }
    const int okd = nn > 0;
    const double iu = 1.0 / sqrt(okd ? nn : 1.0);
    for (int k = 0; k < 3; k++) u[k] *= iu;
    const double au0 = fabs(u[0]), au1 = fabs(u[1]), au2 = fabs(u[2]);
    const int k1 = au1 < au0, k2 = au2 < (k1 ? au1 : au0);
    const double ex = (k1 || k2) ? 0.0 : 1.0, ey = (k1 && !k2) ? 1.0 : 0.0, ez = k2 ? 1.0 : 0.0;
    const double eu = ex * u[0] + ey * u[1] + ez * u[2];
    double q1[3] = {ex - eu * u[0], ey - eu * u[1], ez - eu * u[2]};
    const double iq = 1.0 / sqrt(q1[0] * q1[0] + q1[1] * q1[1] + q1[2] * q1[2]);
    for (int k = 0; k < 3; k++) q1[k] *= iq;
    const double q2[3] = {u[1] * q1[2] - u[2] * q1[1], u[2] * q1[0] - u[0] * q1[2], u[0] * q1[1] - u[1] * q1[0]};
    double Sq1[3], Sq2[3];
    for (int r = 0; r < 3; r++) {
      Sq1[r] = S[3 * r] * q1[0] + S[3 * r + 1] * q1[1] + S[3 * r + 2] * q1[2];
      Sq2[r] = S[3 * r] * q2[0] + S[3 * r + 1] * q2[1] + S[3 * r + 2] * q2[2];
    }
    const double b11 = q1[0] * Sq1[0] + q1[1] * Sq1[1] + q1[2] * Sq1[2];
    const double b12 = q1[0] * Sq2[0] + q1[1] * Sq2[1] + q1[2] * Sq2[2];
    const double b21 = q2[0] * Sq1[0] + q2[1] * Sq1[1] + q2[2] * Sq1[2];
    const double b22 = q2[0] * Sq2[0] + q2[1] * Sq2[1] + q2[2] * Sq2[2];
    const double dd = 0.5 * (b11 - b22), beta2 = -(dd * dd + b12 * b21), cc = m + 0.5 * (b11 + b22);
    const double bb = sqrt(fabs(beta2));
    const int creal = beta2 <= 0;
    if (okd) {
      mu[1] = creal ? cmk(cc + bb, 0.0) : cmk(cc, bb);
      mu[2] = creal ? cmk(cc - bb, 0.0) : cmk(cc, -bb);
      pcen = cc;
      ps = bb;
      preal = creal;
      pc = 1;
    }
  }
  int ab[3] = {pc, pc, pc};
  double og[3] = {0.0, 1.0, 2.0};
  if (pc)
    for (int i = 0; i < 3; i++) x[i] = cmk(mu[i].re - m, mu[i].im);

  /* node order: largest high derivatives last (exp: largest real part; log, pow: smallest modulus); a complex pair
   * stays adjacent, after the real node if near the cut (:373-410) */
#define GKEY(v) (kind == K_EXP ? (v).re : -cabs_s(v))
  {
    const int cplxp = x[1].im != 0;
    if (cplxp) {
      const int first = (GKEY(mu[0]) <= GKEY(mu[1])) || cut;
      if (!first) {  /* rotate: (pair, real node) */
        cplx tx = x[0], tm = mu[0];
        int ta = ab[0];
        double to = og[0];
        for (int k = 0; k < 2; k++) { x[k] = x[k + 1]; mu[k] = mu[k + 1]; ab[k] = ab[k + 1]; og[k] = og[k + 1]; }
        x[2] = tx; mu[2] = tm; ab[2] = ta; og[2] = to;
      }
    } else {
      static const int NET[3][2] = {{0, 1}, {1, 2}, {0, 1}};
      for (int s = 0; s < 3; s++) {
        const int i = NET[s][0], j = NET[s][1];
        if (GKEY(mu[i]) > GKEY(mu[j])) {
          cplx tx = x[i], tm = mu[i];
          int ta = ab[i];
          double to = og[i];
          x[i] = x[j]; mu[i] = mu[j]; ab[i] = ab[j]; og[i] = og[j];
          x[j] = tx; mu[j] = tm; ab[j] = ta; og[j] = to;
        }
      }
    }
  }
#undef GKEY

  /* groups: all three nodes, else the closest eligible pair, else none (:412-437) */
  const double rho_f = (kind == K_POW && 3.0 / al < G_RHO) ? 3.0 / al : G_RHO;
#define GOK(c, R) (kind == K_EXP ? ((R) <= G_R_EXP) : ((m + (c) > 0) && ((R) <= rho_f * (m + (c)))))
  const double cs3 = (x[0].re + x[1].re + x[2].re) / 3.0;
  const double R3 = maxd(maxd(cabs_s(cmk(x[0].re - cs3, x[0].im)), cabs_s(cmk(x[1].re - cs3, x[1].im))),
                         cabs_s(cmk(x[2].re - cs3, x[2].im)));
  const int triple = GOK(cs3, R3);
  int psel[3] = {0, 0, 0};
  double bestR = INFINITY;
  static const int PI_[3] = {0, 0, 1}, PJ_[3] = {1, 2, 2};
  for (int p = 0; p < 3; p++) {
    const int i = PI_[p], j = PJ_[p], k = 3 - i - j;
    const int elig = (x[i].im == 0 && x[j].im == 0) || (x[i].re == x[j].re && x[i].im == -x[j].im);
    const double c = 0.5 * (x[i].re + x[j].re), R = 0.5 * cabs_s(csub(x[i], x[j]));
    const int okp = elig && GOK(c, R) && (R <= G_RHO_POLE * cabs_s(cmk(c - x[k].re, -x[k].im))) && !triple;
    const int better = okp && (R < bestR);
    if (better) {
      bestR = R;
      for (int q = 0; q < p; q++) psel[q] = 0;
    }
    psel[p] = better;
  }
#undef GOK
  const int inG[3] = {triple || psel[0] || psel[1], triple || psel[0] || psel[2], triple || psel[1] || psel[2]};
  const int pk[3] = {psel[2], psel[1], psel[0]};  /* the node outside a pair group */

  /* group centre and offsets; the refined pair as a group: symmetric offsets (:439-460) */
  const int gsum = inG[0] + inG[1] + inG[2];
  double cxg = ((inG[0] ? x[0].re : 0.0) + (inG[1] ? x[1].re : 0.0) + (inG[2] ? x[2].re : 0.0)) /
               (gsum > 0 ? (double)gsum : 1.0);
  double cmu = m + cxg;
  int is12[3];
  for (int i = 0; i < 3; i++) is12[i] = og[i] > 0.5;
  const int ovr = pc && gsum == 2 &&
                  ((inG[0] && inG[1] && is12[0] && is12[1]) || (inG[0] && inG[2] && is12[0] && is12[2]) ||
                   (inG[1] && inG[2] && is12[1] && is12[2]));
  if (ovr) { cxg = pcen - m; cmu = pcen; }
  const cplx dpair = preal ? cmk(ps, 0.0) : cmk(0.0, ps);
  cplx off[3];
  for (int i = 0; i < 3; i++) {
    const int neg = (mu[i].re - pcen < 0) || (mu[i].im < 0);
    const cplx di = neg ? cmk(-dpair.re, -dpair.im) : dpair;
    const int ovi = ovr && inG[i];
    if (ovi) {
      mu[i] = cmk(pcen + di.re, di.im);
      x[i] = cmk(mu[i].re - m, mu[i].im);
    }
    off[i] = inG[i] ? (ovi ? di : cmk(x[i].re - cxg, x[i].im)) : cmk(0.0, 0.0);
  }

  /* single real nodes far from m: Newton (:462-476) */
  for (int i = 0; i < 3; i++) {
    const int mask = !inG[i] && !ab[i] && x[i].im == 0 && fabs(x[i].re) > 0.5 * fabs(m);
    if (mask) {
      newton(As, mu, i);
      ab[i] = 1;
      x[i] = cmk(mu[i].re - m, mu[i].im);
    }
  }
  const int absc = (inG[0] && ab[0]) || (inG[1] && ab[1]) || (inG[2] && ab[2]);
  double apole = 0.0;
  for (int k = 0; k < 3; k++)
    if (pk[k]) apole = (absc || ab[k]) ? cmu - mu[k].re : cxg - x[k].re;
  const double xshift = kind == K_EXP ? maxd(maxd(x[0].re, x[1].re), x[2].re) : 0.0;
  const int bad = kind != K_EXP && ((x[0].im == 0 && mu[0].re <= 0) || (x[1].im == 0 && mu[1].re <= 0) ||
                                    (x[2].im == 0 && mu[2].re <= 0));

  /* group part of the divided differences: the Taylor series streamed over the series index (:478-533) */
  const int hasg = inG[0] || inG[1] || inG[2];
  const double L = kind == K_EXP ? 1.0 : ((hasg && cmu > 0) ? cmu : 1.0), iL = 1.0 / L;
  cplx u[3];
  for (int i = 0; i < 3; i++) u[i] = cscl(off[i], iL);
  const double ap = fabs(apole) > 0 ? apole * iL : 1.0, iap = 1.0 / ap;
  double rr = maxd(cabs_s(u[0]), maxd(cabs_s(u[1]), cabs_s(u[2])));
  const double rq = ((pk[0] || pk[1] || pk[2]) && rr * fabs(iap) <= 1.0) ? rr * fabs(iap) : 0.0;
  rr = (hasg && rr <= G_R_EXP + 0.5) ? rr : 0.0;
  const int K = nterms(bt, 3 * (order + 1) - 1, rr, rq);
  double b0 = 1.0;
  if (kind == K_LOG) b0 = coef0(K_LOG, al, sig, m, cmk(cxg, 0.0), cmk(cmu, 0.0), 0).re;
  cplx Ep[19], Ec[19], acc[19], D[19];
  for (int c = 0; c < ND; c++) {
    Ep[c] = inG[G_NODE[c]] ? cmk(0.0, 0.0) : (G_PAR[c] < 0 ? cmk(1.0, 0.0) : Ep[G_PAR[c]]);
    acc[c] = cmk(0.0, 0.0);
  }
  if (hasg) {
    double q1 = 0.0, q2 = 0.0, q3 = 0.0;
    for (int j = 0; j < K; j++) {
      const double bj = j == 0 ? b0 : bt[j];
      const double g1 = (bj - q1) * iap, g2 = (g1 - q2) * iap, g3 = (g2 - q3) * iap;
      q1 = g1; q2 = g2; q3 = g3;
      const double q[4] = {bj, g1, g2, g3};
      for (int c = 0; c < ND; c++) {
        const int par = G_PAR[c], i = G_NODE[c];
        const cplx epp = par < 0 ? cmk(j == 0 ? 1.0 : 0.0, 0.0) : Ep[par];
        const cplx epc = par < 0 ? cmk(0.0, 0.0) : Ec[par];
        Ec[c] = inG[i] ? cadd(epp, cmul(u[i], Ep[c])) : epc;
        const double g = pk[0] ? q[G_MS[c][0]] : (pk[1] ? q[G_MS[c][1]] : (pk[2] ? q[G_MS[c][2]] : q[0]));
        acc[c] = cadd(acc[c], cscl(Ec[c], g));
      }
      for (int c = 0; c < ND; c++) Ep[c] = Ec[c];
    }
  }
  for (int c = 0; c < ND; c++) {
    const int n = G_MS[c][0] + G_MS[c][1] + G_MS[c][2] - 1, k = G_MS[c][0] - 1;
    double fac;
    if (kind == K_EXP) {
      fac = exp(cxg - xshift);
    } else {
      double iLn = 1.0;
      for (int r = 0; r < n - (kind == K_POW ? k : 0); r++) iLn = iLn * iL;
      fac = kind == K_LOG ? iLn : pow_split(sig * L, al, (double)k) * iLn;
    }
    D[c] = hasg ? cscl(acc[c], fac) : cmk(0.0, 0.0);
  }
  /* residues of the single nodes (:534-576) */
  for (int i = 0; i < 3; i++) {
    if (inG[i]) continue;
    const cplx xs = kind == K_EXP ? cmk(x[i].re - xshift, x[i].im) : x[i];
    cplx f0[3];
    f0[0] = coef0(kind, al, sig, m, xs, mu[i], 0);
    if (kind == K_POW && order >= 1) f0[1] = coef0(kind, al, sig, m, xs, mu[i], 1);
    if (kind == K_POW && order >= 2) f0[2] = coef0(kind, al, sig, m, xs, mu[i], 2);
    const cplx imu = cinv_s(mu[i]);
    cplx w[3];
    for (int z = 0; z < 3; z++)
      if (z != i) w[z] = cinv_s((ab[i] || ab[z]) ? csub(mu[i], mu[z]) : csub(x[i], x[z]));
    for (int c = 0; c < ND; c++) {
      const int mi = G_MS[c][i];
      if (mi == 0) continue;
      const int k = G_MS[c][0] - 1;
      const cplx fb = kind == K_POW ? f0[k] : f0[0];
      cplx ser[3];
      if (kind == K_EXP) {
        ser[0] = fb; ser[1] = fb; ser[2] = cscl(fb, 0.5);
      } else if (kind == K_LOG) {
        ser[0] = fb; ser[1] = imu; ser[2] = cscl(cmul(imu, imu), -0.5);
      } else {
        ser[0] = fb;
        ser[1] = cscl(cmul(fb, imu), al);
        ser[2] = cscl(cmul(ser[1], imu), (al - 1.0) / 2.0);
      }
      for (int z = 0; z < 3; z++) {  /* times the series of 1 / (d + t)^mz */
        const int mz = G_MS[c][z];
        if (z == i || mz == 0) continue;
        cplx wp = cmk(1.0, 0.0);
        for (int r = 0; r < mz; r++) wp = cmul(wp, w[z]);
        const cplx p1 = cscl(cmul(wp, w[z]), (double)-mz);
        const cplx p2 = cscl(cmul(cmul(wp, w[z]), w[z]), mz * (mz + 1) / 2.0);
        const cplx n0 = cmul(ser[0], wp), n1 = cadd(cmul(ser[1], wp), cmul(ser[0], p1));
        const cplx n2 = cadd(cadd(cmul(ser[2], wp), cmul(ser[1], p1)), cmul(ser[0], p2));
        ser[0] = n0; ser[1] = n1; ser[2] = n2;
      }
      D[c] = cadd(D[c], ser[mi - 1]);
    }
  }

  /* real basis r_0 = I, r_1 = B_0, r_2 = B_0 B_1 - b0 b1 I and T = I + iN (:578-599) */
  const double b0i = x[0].im, b1i = x[1].im;
  double B0[9], B1[9], r[3][9];
  for (int k = 0; k < 9; k++) {
    const int dg = k % 4 == 0;
    B0[k] = dg ? (ab[0] ? As[k] - mu[0].re : S[k] - x[0].re) : S[k];
    B1[k] = dg ? (ab[1] ? As[k] - mu[1].re : S[k] - x[1].re) : S[k];
    r[0][k] = dg ? 1.0 : 0.0;
    r[1][k] = B0[k];
  }
  for (int i2 = 0; i2 < 3; i2++)
    for (int j2 = 0; j2 < 3; j2++)
      r[2][3 * i2 + j2] = B0[3 * i2] * B1[j2] + B0[3 * i2 + 1] * B1[3 + j2] + B0[3 * i2 + 2] * B1[6 + j2] -
                          (i2 == j2 ? b0i * b1i : 0.0);
  const double a01 = (ab[0] || ab[1]) ? mu[0].re - mu[1].re : x[0].re - x[1].re;
  const double N10 = -b0i, N20 = -b0i * a01, N21 = -(b0i + b1i);
  const double nanf = bad ? NAN : 1.0;
  { /* F = sum_m Re(T^T D)_m r_m (:600-609) */
    double Dr[3], Di[3], Ni[3];
    for (int j = 0; j < 3; j++) { Dr[j] = D[j].re; Di[j] = D[j].im; }
    nt3(N10, N20, N21, Di, Ni);
    const double e = kind == K_EXP ? exp(m + xshift) : 1.0;
    for (int k = 0; k < 9; k++)
      F[k] = ((Dr[0] - Ni[0]) * r[0][k] + (Dr[1] - Ni[1]) * r[1][k] + (Dr[2] - Ni[2]) * r[2][k]) * e * nanf;
  }
  if (order < 1) return;
  /* J_abcd = sum_mn Re(T^T D T)_mn r_m[a][c] r_n[d][b] (:610-647) */
  const double sc1 = (kind == K_EXP ? exp(m + xshift) : (kind == K_LOG ? isig : 1.0)) * nanf;
  double D2[9];
  {
    double Dr[9], Di[9];
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) { Dr[3 * j + k] = D[g_pos2(j, k)].re; Di[3 * j + k] = D[g_pos2(j, k)].im; }
    for (int k = 0; k < 3; k++) {  /* T on index 0 */
      const double vr[3] = {Dr[k], Dr[3 + k], Dr[6 + k]}, vi[3] = {Di[k], Di[3 + k], Di[6 + k]};
      double nr[3], ni[3];
      nt3(N10, N20, N21, vr, nr);
      nt3(N10, N20, N21, vi, ni);
      for (int j = 0; j < 3; j++) { Dr[3 * j + k] = vr[j] - ni[j]; Di[3 * j + k] = vi[j] + nr[j]; }
    }
    for (int j = 0; j < 3; j++) {  /* real part after T on index 1 */
      double ni[3];
      nt3(N10, N20, N21, Di + 3 * j, ni);
      for (int k = 0; k < 3; k++) D2[3 * j + k] = Dr[3 * j + k] - ni[k];
    }
  }
  double Y[3][9];
  for (int mm = 0; mm < 3; mm++)
    for (int k = 0; k < 9; k++) Y[mm][k] = D2[3 * mm] * r[0][k] + D2[3 * mm + 1] * r[1][k] + D2[3 * mm + 2] * r[2][k];
  for (int aa = 0; aa < 3; aa++)
    for (int bb = 0; bb < 3; bb++)
      for (int cc = 0; cc < 3; cc++)
        for (int dd = 0; dd < 3; dd++)
          J[((3 * aa + bb) * 3 + cc) * 3 + dd] = (r[0][3 * aa + cc] * Y[0][3 * dd + bb] +
                                                  r[1][3 * aa + cc] * Y[1][3 * dd + bb] +
                                                  r[2][3 * aa + cc] * Y[2][3 * dd + bb]) * sc1;
  if (order < 2) return;
  /* H_abcdef = T6_acdefb + T6_aefcdb, T6_acdefb = sum_mnp Re(D with T on each index)_mnp r_m[ac] r_n[de] r_p[fb]
   * (:648-691) */
  const double sc2 = (kind == K_EXP ? exp(m + xshift) : (kind == K_LOG ? isig * isig : 1.0)) * nanf;
  double D3[27];
  {
    double Dr[27], Di[27];
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) {
          Dr[9 * j + 3 * k + l] = D[g_pos3(j, k, l)].re;
          Di[9 * j + 3 * k + l] = D[g_pos3(j, k, l)].im;
        }
    static const int STR[3] = {9, 3, 1};
    for (int axis = 0; axis < 3; axis++) {
      const int s = STR[axis];
      for (int base = 0; base < 27; base++) {
        if ((base / s) % 3 != 0) continue;
        const double vr[3] = {Dr[base], Dr[base + s], Dr[base + 2 * s]};
        const double vi[3] = {Di[base], Di[base + s], Di[base + 2 * s]};
        double nr[3], ni[3];
        nt3(N10, N20, N21, vr, nr);
        nt3(N10, N20, N21, vi, ni);
        for (int j = 0; j < 3; j++) { Dr[base + j * s] = vr[j] - ni[j]; Di[base + j * s] = vi[j] + nr[j]; }
      }
    }
    memcpy(D3, Dr, sizeof D3);
  }
  double Z[9][9], Yh[3][81];
  for (int mn = 0; mn < 9; mn++)
    for (int k = 0; k < 9; k++) Z[mn][k] = D3[3 * mn] * r[0][k] + D3[3 * mn + 1] * r[1][k] + D3[3 * mn + 2] * r[2][k];
  for (int mm = 0; mm < 3; mm++)
    for (int de = 0; de < 9; de++)
      for (int fb = 0; fb < 9; fb++)
        Yh[mm][9 * de + fb] = r[0][de] * Z[3 * mm][fb] + r[1][de] * Z[3 * mm + 1][fb] + r[2][de] * Z[3 * mm + 2][fb];
  for (int aa = 0; aa < 3; aa++)
    for (int bb = 0; bb < 3; bb++)
      for (int cc = 0; cc < 3; cc++)
        for (int dd = 0; dd < 3; dd++)
          for (int ee = 0; ee < 3; ee++)
            for (int ff = 0; ff < 3; ff++) {
              const int i1 = 9 * (3 * dd + ee) + 3 * ff + bb, i2 = 9 * (3 * ff + cc) + 3 * dd + bb;
              const double h = r[0][3 * aa + cc] * Yh[0][i1] + r[1][3 * aa + cc] * Yh[1][i1] +
                               r[2][3 * aa + cc] * Yh[2][i1] + r[0][3 * aa + ee] * Yh[0][i2] +
                               r[1][3 * aa + ee] * Yh[1][i2] + r[2][3 * aa + ee] * Yh[2][i2];
              H[((((3 * aa + bb) * 3 + cc) * 3 + dd) * 3 + ee) * 3 + ff] = h * sc2;
            }
}

/* ================================================================================================ C ABI driver */
enum { FAM_VOIGT = 0, FAM_MATRIX = 1, FAM_GENERAL = 2 };

/* argument check and normalisation: c/src/matfun.cc:23-32 */
static int prepare(int fam, int *kind, double *alpha, int64_t n, const double *J, const double *H) {
  if (*kind < K_EXP || *kind > K_SQRT || n < 0 || (H && !J) || (*kind == K_POW && !(*alpha > 0))) return 0;
  if (fam == FAM_GENERAL && *kind == K_SQRT) { *kind = K_POW; *alpha = 0.5; }
  if (*kind != K_POW) *alpha = *kind == K_SQRT ? 0.5 : 0.0;
  return 1;
}

static int g_tables_ready = 0;

/* matrices lo..hi-1; returns 0 if one of them is not symmetric (matrix family): c/src/matfun.cc:34-53 */
static int run_range(int fam, int kind, double al, const double *x, double *F, double *J, double *H, int64_t lo,
                     int64_t hi, const double *c2, const double *bt) {
  int sym = 1;
  for (int64_t i = lo; i < hi; i++) {
    if (fam == FAM_GENERAL) {
      const int order = H ? 2 : (J ? 1 : 0);
      gmf_one(kind, order, x + 9 * i, F + 9 * i, J ? J + 81 * i : NULL, H ? H + 729 * i : NULL, al, bt);
    } else if (fam == FAM_VOIGT) {
      smf_one(kind, x + 6 * i, F + 6 * i, J ? J + 36 * i : NULL, H ? H + 216 * i : NULL, al, c2);
    } else {
      double v[6], fv[6], jv[36], hv[216];
      sym &= from_matrix(x + 9 * i, v);
      smf_one(kind, v, fv, J ? jv : NULL, H ? hv : NULL, al, c2);
      to_matrix(fv, jv, hv, F + 9 * i, J ? J + 81 * i : NULL, H ? H + 729 * i : NULL);
    }
  }
  return sym;
}

static int eval_family(int fam, int kind, double alpha, int64_t n, const double *x, double *F, double *J, double *H) {
  if (!prepare(fam, &kind, &alpha, n, J, H)) return -1;
  if (!g_tables_ready) {  /* idempotent; racing first calls write identical values */
    g_tables();
    g_tables_ready = 1;
  }
  double c2[DD2_TERMS], bt[G_KMAX];
  dd2_coef(kind, alpha, c2);
  series_coef(kind, alpha, bt);
  /* tasks of a few hundred matrices, dynamically scheduled (c/src/matfun.cc:55-83) */
  const int64_t ch = H ? 256 : 1024, nch = (n + ch - 1) / ch;
  int asym = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : asym)
  for (int64_t k = 0; k < nch; k++) {
    const int64_t lo = k * ch, hi = lo + ch < n ? lo + ch : n;
    asym |= !run_range(fam, kind, alpha, x, F, J, H, lo, hi, c2, bt);
  }
  return asym ? -3 : 0;
}

int orc_smf_eval(int kind, double alpha, int64_t n, const double *v, double *F, double *J, double *H) {
  return eval_family(FAM_VOIGT, kind, alpha, n, v, F, J, H);
}
int orc_smf_eval_matrix(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H) {
  return eval_family(FAM_MATRIX, kind, alpha, n, A, F, J, H);
}
int orc_gmf_eval(int kind, double alpha, int64_t n, const double *A, double *F, double *J, double *H) {
  return eval_family(FAM_GENERAL, kind, alpha, n, A, F, J, H);
}
int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
const char *orc_version(void) { return "matfun-oracle 0.1.3 (scalar C restatement)"; }
