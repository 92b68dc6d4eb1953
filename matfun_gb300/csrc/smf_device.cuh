// smf_device.cuh -- per-matrix device math of the symmetric family (FP64, one thread per matrix):
//   * closed-form eigensystem of a symmetric 3x3 matrix (deviator + Smith's trigonometric formula, cross-product
//     eigenvector, Jacobi rotation by half-angle formulas) -- c/include/matfun/smf_kernel.hpp:200-280
//   * f of the eigenvalues with the log1p form near the mean -- smf_kernel.hpp:75-82, 281-290
//   * stable first / second divided differences -- smf_kernel.hpp:84-192
// and the eigen-basis quantities the kernels contract into J and H:
//   Et_p = V^T E_p V for the six Voigt basis matrices E_p,
//   J_{I,p}   = w_I  K(I, p),       K(X, Y)    = sum_ab D_ab X_ab Y_ab                       (21 distinct)
//   H_{I,p,q} = w_I  G'(I, p, q),   G'(X, Y, Z) = 2 sum_amb D2_amb X_ab Y_am Z_mb           (56 distinct)
// with w_I = 1 for a diagonal and 1/2 for an off-diagonal Voigt index I.  K and G' are symmetric in all their
// arguments (D and D2 are symmetric, the Et are symmetric matrices), so only the sorted index tuples are computed;
// the reference assembles all 36 / 126 entries (smf_kernel.hpp:297-381).  Same branch thresholds as the reference.
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
  double tau;               // cluster radius of the second divided difference
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

template <int KIND>
MF_D void smf_eigsys(const double *v, SmfEig &E) {
  constexpr double SQRT6 = 2.449489742783178, TWO_PI_3 = 2.0943951023931957;
  // power-of-two scale sig ~ max|v| (exact; the pairwise select tree keeps the reference's NaN behaviour)
  double s01 = tmax(fabs(v[0]), fabs(v[1])), s23 = tmax(fabs(v[2]), fabs(v[3]));
  double s45 = tmax(fabs(v[4]), fabs(v[5]));
  double sig = pow2floor(tmax(tmax(s01, s23), s45) + 1e-300), isig = 1.0 / sig;
  double a0 = v[0] * isig, a1 = v[1] * isig, a2 = v[2] * isig, a3 = v[3] * isig, a4 = v[4] * isig,
               a5 = v[5] * isig;
  // deviator, its trace residue removed, normalised by a power of two
  double m = (a0 + a1 + a2) / 3.0, d0 = a0 - m, d1 = a1 - m, d2 = a2 - m;
  double tr3 = (d0 + d1 + d2) / 3.0, e0 = d0 - tr3, e1 = d1 - tr3, e2 = d2 - tr3;
  double z01 = tmax(fabs(e0), fabs(e1)), z23 = tmax(fabs(e2), fabs(a3)), z45 = tmax(fabs(a4), fabs(a5));
  double dmax = tmax(tmax(z01, z23), z45);
  bool iso = dmax <= 1e-300;
  double ids = 1.0 / sel(iso, 1.0, pow2floor(dmax));
  double g0 = e0 * ids, g1 = e1 * ids, g2 = e2 * ids, g3 = a3 * ids, g4 = a4 * ids, g5 = a5 * ids;
  // the eigenvalue farthest from the other two (Smith)
  double p = g0 * g0 + g1 * g1 + g2 * g2 + 2.0 * (g3 * g3 + g4 * g4 + g5 * g5);
  double q = g0 * (g1 * g2 - g5 * g5) - g3 * (g3 * g2 - g5 * g4) + g4 * (g3 * g5 - g1 * g4);
  double pg = sel(iso, 1.0, p), qg = sel(iso, 0.0, q);
  double r = 3.0 * SQRT6 * qg / (pg * sqrt(pg));
  r = sel(r > 1.0, 1.0, sel(r < -1.0, -1.0, r));
  double t = sqrt(2.0 * pg / 3.0), ph = acos(r) / 3.0;
  double sh = t * cos(sel(r >= 0, ph, ph + TWO_PI_3));
  // its eigenvector: the longest cross product of two rows of the shifted deviator
  double m00 = g0 - sh, m11 = g1 - sh, m22 = g2 - sh;
  double cxv = g3 * g5 - g4 * m11, cyv = g4 * g3 - m00 * g5, czv = m00 * m11 - g3 * g3;
  double nn = cxv * cxv + cyv * cyv + czv * czv;
  {
    double bx = g3 * m22 - g4 * g5, by = g4 * g4 - m00 * m22, bz = m00 * g5 - g3 * g4;
    double nb = bx * bx + by * by + bz * bz;
    bool s1 = nb > nn;
    cxv = sel(s1, bx, cxv); cyv = sel(s1, by, cyv); czv = sel(s1, bz, czv); nn = sel(s1, nb, nn);
    double ex = m11 * m22 - g5 * g5, ey = g5 * g4 - g3 * m22, ez = g3 * g5 - m11 * g4;
    double ne = ex * ex + ey * ey + ez * ez;
    bool s2 = ne > nn;
    cxv = sel(s2, ex, cxv); cyv = sel(s2, ey, cyv); czv = sel(s2, ez, czv); nn = sel(s2, ne, nn);
  }
  double nrm = sqrt(nn);
  bool ok = (nrm > 1e-300) & !iso;
  double inv = 1.0 / sel(ok, nrm, 1.0);
  double vx = sel(ok, cxv * inv, 1.0), vy = sel(ok, cyv * inv, 0.0), vz = sel(ok, czv * inv, 0.0);
  // orthonormal complement (u, w)
  double ax = fabs(vx), ay = fabs(vy), az = fabs(vz);
  bool k1 = ay < ax, k2 = az < sel(k1, ay, ax);
  double ex = sel(k1 | k2, 0.0, 1.0), ey = sel(k1 & !k2, 1.0, 0.0), ez = sel(k2, 1.0, 0.0);
  double vk = ex * vx + ey * vy + ez * vz;
  double ux = ex - vk * vx, uy = ey - vk * vy, uz = ez - vk * vz;
  double nu = sqrt(ux * ux + uy * uy + uz * uz);
  bool oku = nu > 1e-300;
  double iu = 1.0 / sel(oku, nu, 1.0);
  ux = sel(oku, ux * iu, 0.0); uy = sel(oku, uy * iu, 0.0); uz = sel(oku, uz * iu, 0.0);
  double wx = vy * uz - vz * uy, wy = vz * ux - vx * uz, wz = vx * uy - vy * ux;
  // Rayleigh quotients of A (eigenvalues) and of the deviator (rotation angle; log near m)
  double Aux = a0 * ux + a3 * uy + a4 * uz, Auy = a3 * ux + a1 * uy + a5 * uz, Auz = a4 * ux + a5 * uy + a2 * uz;
  double Awx = a0 * wx + a3 * wy + a4 * wz, Awy = a3 * wx + a1 * wy + a5 * wz, Awz = a4 * wx + a5 * wy + a2 * wz;
  double Avx = a0 * vx + a3 * vy + a4 * vz, Avy = a3 * vx + a1 * vy + a5 * vz, Avz = a4 * vx + a5 * vy + a2 * vz;
  double a11 = ux * Aux + uy * Auy + uz * Auz, a12 = ux * Awx + uy * Awy + uz * Awz;
  double a22 = wx * Awx + wy * Awy + wz * Awz, lv = vx * Avx + vy * Avy + vz * Avz;
  double Dux = d0 * ux + a3 * uy + a4 * uz, Duy = a3 * ux + d1 * uy + a5 * uz, Duz = a4 * ux + a5 * uy + d2 * uz;
  double Dwx = d0 * wx + a3 * wy + a4 * wz, Dwy = a3 * wx + d1 * wy + a5 * wz, Dwz = a4 * wx + a5 * wy + d2 * wz;
  double b11 = ux * Dux + uy * Duy + uz * Duz, b12 = ux * Dwx + uy * Dwy + uz * Dwz;
  double b22 = wx * Dwx + wy * Dwy + wz * Dwz;
  // Jacobi rotation (cos, sin of half the angle atan2(2 b12, b11 - b22))
  double jx = b11 - b22, jy = 2.0 * b12, jr = sqrt(jx * jx + jy * jy);
  bool jz = jr == 0, jpos = jx >= 0;
  double jrs = sel(jz, 1.0, jr);
  double big = sqrt((jrs + fabs(jx)) / (2.0 * jrs)), sml = jy / (2.0 * jrs * big);
  double sgn = sel((jy > 0) | ((jy == 0) & (__double_as_longlong(jy) >= 0)), 1.0, -1.0);
  double cs = sel(jz, 1.0, sel(jpos, big, sgn * sml)), sn = sel(jz, 0.0, sel(jpos, sml, sgn * big));
  E.lam[0] = lv * sig;
  E.lam[1] = (cs * cs * a11 + 2.0 * cs * sn * a12 + sn * sn * a22) * sig;
  E.lam[2] = (sn * sn * a11 - 2.0 * cs * sn * a12 + cs * cs * a22) * sig;
  E.V[0][0] = vx; E.V[0][1] = cs * ux + sn * wx; E.V[0][2] = cs * wx - sn * ux;
  E.V[1][0] = vy; E.V[1][1] = cs * uy + sn * wy; E.V[1][2] = cs * wy - sn * uy;
  E.V[2][0] = vz; E.V[2][1] = cs * uz + sn * wz; E.V[2][2] = cs * wz - sn * uz;
  E.m = m;
  E.sig = sig;
  if (KIND == LOG) {
    E.xd[0] = vx * (d0 * vx + a3 * vy + a4 * vz) + vy * (a3 * vx + d1 * vy + a5 * vz) + vz * (a4 * vx + a5 * vy + d2 * vz);
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
    fl[i] = smf_fun<KIND>(lam[i], al);
  }
  if (KIND == LOG) {  // near m: log(m sig) + log1p(x / m), x from the deviator
    double lms = log(E.m * E.sig);
#pragma unroll
    for (int i = 0; i < 3; i++)
      fl[i] = sel(fabs(E.xd[i]) <= 0.5 * E.m, lms + log1p(E.xd[i] / E.m), fl[i]);
  }
}

// first divided difference f[a, b] (smf_kernel.hpp:84-115)
template <int KIND>
MF_D double smf_dd1(double a, double b, double fa, double fb, const SmfCoef &C) {
  if (KIND == EXP) {
    double d = fabs(a - b);
    return sel(a > b, fa, fb) * sel(d > 0, -expm1(-d) / d, 1.0);
  }
  if (KIND == LOG) {
    double s = 0.5 * (a + b), z = (a - b) / (a + b), az = fabs(z), z2 = z * z;
    if (az < 1e-3) return (1.0 + z2 / 3.0 + z2 * z2 / 5.0 + z2 * z2 * z2 / 7.0) / s;
    if (az >= 0.5) return (log(a) - log(b)) / (a - b);
    return atanh(z) / z / s;
  }
  a = sel(a > 0, a, 0.0);
  b = sel(b > 0, b, 0.0);
  if (KIND == SQRT) return 1.0 / (sqrt(a) + sqrt(b));
  double s = 0.5 * (a + b), ss = sel(s > 0, s, 1.0);
  double z = (a - b) / (2.0 * ss), az = fabs(z);
  bool zero = az == 0, near = !zero & (az < 0.5);
  if (!zero & !near) return (fa - fb) / (a - b);
  double al = C.al;
  double g = zero ? al : (expm1(al * log1p(z)) - expm1(al * log1p(-z))) / (2.0 * z);
  return (s > 0 ? pow_split(ss, C.bh1, C.bl1) : C.zp1) * g;
}

// f'(x) (smf_kernel.hpp:117-126)
template <int KIND>
MF_D double smf_deriv(double x, double fx, const SmfCoef &C) {
  if (KIND == EXP) return fx;
  if (KIND == LOG) return 1.0 / x;
  x = sel(x > 0, x, 0.0);
  if (KIND == SQRT) return 1.0 / (2.0 * sqrt(x));
  return x > 0 ? C.al * pow_split(x, C.bh1, C.bl1) : C.al * C.zp1;
}

// second divided difference f[li, lj, lk] (smf_kernel.hpp:148-192)
template <int KIND>
MF_D double smf_dd2(double li, double lj, double lk, double fi, double fj, double fk, double Dij, double Dik,
                    double Djk, const SmfCoef &C) {
  if (KIND == POW || KIND == SQRT) {
    li = sel(li > 0, li, 0.0); lj = sel(lj > 0, lj, 0.0); lk = sel(lk > 0, lk, 0.0);
  }
  double dA = lk - li, dB = lj - li, dC = lk - lj, aA = fabs(dA), aB = fabs(dB), aC = fabs(dC);
  bool useA = (aA >= aB) & (aA >= aC), useB = !useA & (aB >= aC);
  double num = sel(useA, Djk - Dij, sel(useB, Djk - Dik, Dik - Dij));
  double den = sel(useA, dA, sel(useB, dB, dC));
  double mn = sel(li < lj, li, lj), mx = sel(li < lj, lj, li);
  double lo = sel(mn < lk, mn, lk), hi = sel(mx > lk, mx, lk), t = sel(mx < lk, mx, lk), mid = sel(mn > t, mn, t);
  bool cluster;
  if (KIND == EXP) {
    cluster = (hi - lo) <= 1.0;
  } else {
    cluster = (mid > 0) & (mid - lo <= C.tau * mid) & (hi - mid <= C.tau * mid);
  }
  double out;
  if (cluster) {
    double fm = sel(mid == li, fi, sel(mid == lj, fj, fk));
    double u, w, scale;
    if (KIND == EXP) {
      u = lo - mid; w = hi - mid; scale = fm;
    } else {
      u = (lo - mid) / mid; w = (hi - mid) / mid;
      scale = (KIND == LOG ? 1.0 : fm) / (mid * mid);
    }
    double h = 1.0, wk = 1.0, s = C.c2[0];
#pragma unroll
    for (int k = 1; k < DD2_TERMS; k++) {
      wk = wk * w;
      h = u * h + wk;
      s = s + C.c2[k] * h;
    }
    out = scale * s;
  } else {
    out = num / sel(den != 0, den, 1.0);
  }
  if (KIND == POW || KIND == SQRT) out = sel(hi > 0, out, C.z2);
  return out;
}

// f[l, l, l] = f''(l) / 2: the reference's cluster series at u = w = 0 is exactly scale * c2[0]; outside the
// cluster its difference formula gives (D_ll - D_ll) / 1 (smf_kernel.hpp:148-192, specialised to three equal points)
template <int KIND>
MF_D double smf_dd2_same(double l, double fl, double Dll, const SmfCoef &C) {
  if (KIND == POW || KIND == SQRT) l = sel(l > 0, l, 0.0);
  bool cluster;
  if (KIND == EXP) cluster = (l - l) <= 1.0;
  else cluster = (l > 0) & (l - l <= C.tau * l) & (l - l <= C.tau * l);
  double out;
  if (KIND == EXP) out = sel(cluster, fl * C.c2[0], Dll - Dll);
  else out = sel(cluster, ((KIND == LOG ? 1.0 : fl) / (l * l)) * C.c2[0], Dll - Dll);
  if (KIND == POW || KIND == SQRT) out = sel(l > 0, out, C.z2);
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
