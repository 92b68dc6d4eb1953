// smf_mixed.cuh -- mixed-precision symmetric family: FP32 input and output, FP32 for the bulk of the arithmetic.
//
// FP64 is kept only where FP32 would lose the result:
//   * the eigensystem (deviator, the cubic's trigonometric root, cross-product eigenvector, Jacobi rotation, Rayleigh
//     quotients): with condition numbers up to 1e6 and eigenvalue gaps down to 1e-12 an FP32 eigensolve loses the
//     small eigenvalues and the near-degenerate pairs entirely;
//   * the differences of eigenvalues that feed the near-coalescent branches of the divided differences (z, u, w and
//     the denominators of the difference formulas), taken from the FP64 eigenvalues before rounding to FP32.
// f(lambda), the first and second divided differences (stable forms, cluster series), the product vectors and the
// J / H forms of smf_kernels.cuh run in FP32.  The FP64 share per matrix drops from ~2.5k to ~0.4k operations, so
// on GB300 (FP64 at 1/74 of FP32) the kernel moves towards the HBM roofline, and FP32 storage halves the bytes.
// Accuracy against the FP64 oracle is stated per kind and order in the tests (<= 1e-6 relative, max-norm).
#pragma once
#include "smf_kernels.cuh"

namespace mf {

struct SmfCoefF {
  float al, alm1;   // exponent and exponent - 1
  float zp1, z2;    // 0^(al - 1), f''(0)/2 for powers
  float tau;        // cluster radius of the second divided difference
  float c2[DD2_TERMS];
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
// f[a, b], a <= b, dab = b - a -- smf_kernel.hpp:84-115
template <int KIND>
MF_D float dd1s_f(float a, float b, float dab, float fa, float fb, const SmfCoefF &C) {
  if (KIND == EXP) return fb * self(dab > 0.f, -expm1f(-dab) / dab, 1.f);
  if (KIND == LOG) {
    float s = 0.5f * (a + b), z = dab / (a + b), az = fabsf(z), z2 = z * z;
    if (az < 1e-3f) return (1.f + z2 / 3.f + z2 * z2 / 5.f + z2 * z2 * z2 / 7.f) / s;
    if (az >= 0.5f) return (logf(b) - logf(a)) / dab;
    return atanhf(z) / z / s;
  }
  if (KIND == SQRT) return 1.f / (sqrtf(a) + sqrtf(b));
  float s = 0.5f * (a + b), ss = self(s > 0.f, s, 1.f);
  float z = dab / (2.f * ss), az = fabsf(z);
  bool zero = az == 0.f, near = !zero & (az < 0.5f);
  if (!zero & !near) return (fb - fa) / dab;
  float g = zero ? C.al : (expm1f(C.al * log1pf(z)) - expm1f(C.al * log1pf(-z))) / (2.f * z);
  return (s > 0.f ? powf(ss, C.alm1) : C.zp1) * g;
}

template <int KIND>
MF_D float deriv_f(float x, float fx, const SmfCoefF &C) {
  if (KIND == EXP) return fx;
  if (KIND == LOG) return 1.f / x;
  float xf = self(x > 0.f, x, 0.f);
  if (KIND == SQRT) return 1.f / (2.f * sqrtf(xf));
  return xf > 0.f ? C.al * powf(xf, C.alm1) : C.al * C.zp1;
}

// f[li, lj, lk] for li <= lj <= lk; dji = lj - li, dkj = lk - lj, dki = lk - li -- smf_kernel.hpp:148-192 (the widest
// difference is the denominator, the middle eigenvalue the cluster centre)
template <int KIND>
MF_D float dd2s_f(float lj, float lk, float fj, float Dij, float Djk, float dji, float dkj, float dki,
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
      u = -dji / lj; w = dkj / lj;
      scale = (KIND == LOG ? 1.f : fj) / (lj * lj);
    }
    float h = 1.f, wk = 1.f, sm = C.c2[0];
#pragma unroll
    for (int k = 1; k < DD2_TERMS; k++) {
      wk = wk * w;
      h = fmaf(u, h, wk);
      sm = fmaf(C.c2[k], h, sm);
    }
    out = scale * sm;
  } else {
    out = (Djk - Dij) / self(dki != 0.f, dki, 1.f);
  }
  if (KIND == POW || KIND == SQRT) out = self(lk > 0.f, out, C.z2);
  return out;
}

template <int KIND>
MF_D float dd2_same_f(float lf, float fl, float Dll, const SmfCoefF &C) {
  bool cluster = KIND == EXP ? true : (lf > 0.f);
  float out = KIND == EXP ? self(cluster, fl * C.c2[0], Dll - Dll)
                          : self(cluster, ((KIND == LOG ? 1.f : fl) / (lf * lf)) * C.c2[0], Dll - Dll);
  if (KIND == POW || KIND == SQRT) out = self(lf > 0.f, out, C.z2);
  return out;
}

// |x| of a double as an ordered integer key (max of magnitudes on the integer pipe)
MF_D long long absbits(double x) { return __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFll; }
MF_D long long kmax(long long a, long long b) { return a > b ? a : b; }

// 2^-e for a power of two 2^e of normal range (exponent arithmetic, no division)
MF_D double pow2inv(double p) {
  long long e = (__double_as_longlong(p) >> 52) & 0x7FF;
  return __longlong_as_double((2046ll - e) << 52);
}

MF_D float nrm3(float &x, float &y, float &z) {
  float n = __fsqrt_rn(x * x + y * y + z * z), i = __fdiv_rn(1.f, n);
  x *= i; y *= i; z *= i;
  return n;
}

// The eigensystem of the mixed path.  FP32: the cubic's trigonometric root (on the deviator normalised to max 1, where
// the root of the separated eigenvalue is insensitive to rounding of r), its eigenvector (largest cross product of
// two rows of G - root I), the orthonormal complement and the 2x2 Jacobi rotation.  FP64: the deviator and the
// Rayleigh quotients of the FP32 vectors in the deviator shifted by minus half the root (the centre of the remaining
// pair), so that the pair's block is of the size of its own gap: the rotation angle is then accurate relative to the
// gap, and the quotients, divided by the vectors' FP64 squared norms (1 - e + e^2 with e = |x|^2 - 1), give the
// eigenvalues to ~1e-14 relative to |A| (an FP32 vector error d moves a quotient by O(d^2)).  Eigenvalues and the
// deviator's eigenvalues (xd, for log near the mean) are in the units of the input.
struct SmfEigM {
  double lam[3], xd[3], m;
  float V[3][3];
};

template <int KIND>
MF_D void smf_eigsys_mixed(const double *v, SmfEigM &E) {
  constexpr float SQRT6 = 2.4494897f, TWO_PI_3 = 2.0943951f;
  double m = (v[0] + v[1] + v[2]) * (1.0 / 3.0);
  double d0 = v[0] - m, d1 = v[1] - m, d2 = v[2] - m;
  long long k01 = kmax(absbits(d0), absbits(d1)), k23 = kmax(absbits(d2), absbits(v[3]));
  long long k45 = kmax(absbits(v[4]), absbits(v[5]));
  double dmax = __longlong_as_double(kmax(kmax(k01, k23), k45));
  bool bad = !(dmax < 1e300), iso = !(dmax > 0.0) | bad;  // bad: NaN or infinite input (NaN vectors and results)
  double dsc = sel(iso, 1.0, pow2floor(dmax)), ids = pow2inv(dsc);
  float g0 = (float)(d0 * ids), g1 = (float)(d1 * ids), g2 = (float)(d2 * ids);
  float g3 = (float)(v[3] * ids), g4 = (float)(v[4] * ids), g5 = (float)(v[5] * ids);
  float p = g0 * g0 + g1 * g1 + g2 * g2 + 2.f * (g3 * g3 + g4 * g4 + g5 * g5);
  float q = g0 * (g1 * g2 - g5 * g5) - g3 * (g3 * g2 - g5 * g4) + g4 * (g3 * g5 - g1 * g4);
  float pg = self(iso, 1.f, p), qg = self(iso, 0.f, q);
  float r = 3.f * SQRT6 * qg / (pg * sqrtf(pg));
  r = self(r > 1.f, 1.f, self(r < -1.f, -1.f, r));
  float t = sqrtf(2.f * pg / 3.f), ph = acosf(r) / 3.f;
  float sh = t * cosf(self(r >= 0.f, ph, ph + TWO_PI_3));
  float m00 = g0 - sh, m11 = g1 - sh, m22 = g2 - sh;
  float cxv = g3 * g5 - g4 * m11, cyv = g4 * g3 - m00 * g5, czv = m00 * m11 - g3 * g3;
  float nn = cxv * cxv + cyv * cyv + czv * czv;
  {
    float bx = g3 * m22 - g4 * g5, by = g4 * g4 - m00 * m22, bz = m00 * g5 - g3 * g4;
    float nb = bx * bx + by * by + bz * bz;
    bool s1 = nb > nn;
    cxv = self(s1, bx, cxv); cyv = self(s1, by, cyv); czv = self(s1, bz, czv); nn = self(s1, nb, nn);
    float ex = m11 * m22 - g5 * g5, ey = g5 * g4 - g3 * m22, ez = g3 * g5 - m11 * g4;
    float ne = ex * ex + ey * ey + ez * ez;
    bool s2 = ne > nn;
    cxv = self(s2, ex, cxv); cyv = self(s2, ey, cyv); czv = self(s2, ez, czv); nn = self(s2, ne, nn);
  }
  bool ok = (nn > 1e-30f) & !iso;
  float vx = self(ok, cxv, 1.f), vy = self(ok, cyv, 0.f), vz = self(ok, czv, 0.f);
  nrm3(vx, vy, vz);
  float ax = fabsf(vx), ay = fabsf(vy), az = fabsf(vz);
  bool k1 = ay < ax, k2 = az < self(k1, ay, ax);
  float ex = self(k1 | k2, 0.f, 1.f), ey = self(k1 & !k2, 1.f, 0.f), ez = self(k2, 1.f, 0.f);
  float vk = ex * vx + ey * vy + ez * vz;
  float ux = ex - vk * vx, uy = ey - vk * vy, uz = ez - vk * vz;
  nrm3(ux, uy, uz);
  float wx = vy * uz - vz * uy, wy = vz * ux - vx * uz, wz = vx * uy - vy * ux;
  // FP64: quotients in the shifted deviator Ds = D + s I, s = root * dsc / 2
  double s = sel(iso, 0.0, (double)sh * dsc * 0.5);
  double e0 = d0 + s, e1 = d1 + s, e2 = d2 + s, o3 = v[3], o4 = v[4], o5 = v[5];
  double Vx = vx, Vy = vy, Vz = vz, Ux = ux, Uy = uy, Uz = uz, Wx = wx, Wy = wy, Wz = wz;
  double Dvx = e0 * Vx + o3 * Vy + o4 * Vz, Dvy = o3 * Vx + e1 * Vy + o5 * Vz, Dvz = o4 * Vx + o5 * Vy + e2 * Vz;
  double Dux = e0 * Ux + o3 * Uy + o4 * Uz, Duy = o3 * Ux + e1 * Uy + o5 * Uz, Duz = o4 * Ux + o5 * Uy + e2 * Uz;
  double Dwx = e0 * Wx + o3 * Wy + o4 * Wz, Dwy = o3 * Wx + e1 * Wy + o5 * Wz, Dwz = o4 * Wx + o5 * Wy + e2 * Wz;
  double qv = Vx * Dvx + Vy * Dvy + Vz * Dvz, nv = Vx * Vx + Vy * Vy + Vz * Vz;
  double b11 = Ux * Dux + Uy * Duy + Uz * Duz, b12 = Ux * Dwx + Uy * Dwy + Uz * Dwz;
  double b22 = Wx * Dwx + Wy * Dwy + Wz * Dwz;
  double uu = Ux * Ux + Uy * Uy + Uz * Uz, uw = Ux * Wx + Uy * Wy + Uz * Wz, ww = Wx * Wx + Wy * Wy + Wz * Wz;
  // FP32 Jacobi rotation of the pair from the FP64 block (its entries are of the size of the pair's gap)
  float jx = (float)(b11 - b22), jy = (float)(b12 + b12), jr = sqrtf(jx * jx + jy * jy);
  bool jz = !(jr > 0.f), jpos = jx >= 0.f;
  float jrs = self(jz, 1.f, jr);
  float big = sqrtf((jrs + fabsf(jx)) / (2.f * jrs)), sml = jy / (2.f * jrs * big);
  float sgn = self(jy >= 0.f, 1.f, -1.f);
  float cs = self(jz, 1.f, self(jpos, big, sgn * sml)), sn = self(jz, 0.f, self(jpos, sml, sgn * big));
  double C = cs, S = sn, CC = C * C, SS = S * S, CS2 = 2.0 * (C * S);
  double n1 = CC * uu + CS2 * uw + SS * ww - 1.0, n2 = SS * uu - CS2 * uw + CC * ww - 1.0, n0 = nv - 1.0;
  double t0 = qv * (1.0 - n0 + n0 * n0);
  double t1 = (CC * b11 + CS2 * b12 + SS * b22) * (1.0 - n1 + n1 * n1);
  double t2 = (SS * b11 - CS2 * b12 + CC * b22) * (1.0 - n2 + n2 * n2);
  E.xd[0] = t0 - s; E.xd[1] = t1 - s; E.xd[2] = t2 - s;
  E.lam[0] = m + E.xd[0]; E.lam[1] = m + E.xd[1]; E.lam[2] = m + E.xd[2];
  E.m = m;
  float r1x = cs * ux + sn * wx, r1y = cs * uy + sn * wy, r1z = cs * uz + sn * wz;
  float r2x = cs * wx - sn * ux, r2y = cs * wy - sn * uy, r2z = cs * wz - sn * uz;
  // one Newton-Schulz step V <- V (3 I - V^T V) / 2 with the Gram matrix in FP64: the FP32 vectors come out
  // orthonormal to the rounding of their components (an FP32 Gram matrix would leave its own rounding in them)
  double R1x = r1x, R1y = r1y, R1z = r1z, R2x = r2x, R2y = r2y, R2z = r2z;
  float e00 = (float)(n0 * 0.5), e11 = (float)((R1x * R1x + R1y * R1y + R1z * R1z - 1.0) * 0.5);
  float e22 = (float)((R2x * R2x + R2y * R2y + R2z * R2z - 1.0) * 0.5);
  float e01 = (float)((Vx * R1x + Vy * R1y + Vz * R1z) * 0.5), e02 = (float)((Vx * R2x + Vy * R2y + Vz * R2z) * 0.5);
  float e12 = (float)((R1x * R2x + R1y * R2y + R1z * R2z) * 0.5);
  float c0[3] = {vx, vy, vz}, c1[3] = {r1x, r1y, r1z}, c2[3] = {r2x, r2y, r2z};
  float nanv = __int_as_float(0x7FC00000);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    E.V[i][0] = self(bad, nanv, c0[i] - (c0[i] * e00 + c1[i] * e01 + c2[i] * e02));
    E.V[i][1] = self(bad, nanv, c1[i] - (c0[i] * e01 + c1[i] * e11 + c2[i] * e12));
    E.V[i][2] = self(bad, nanv, c2[i] - (c0[i] * e02 + c1[i] * e12 + c2[i] * e22));
  }
}

// symmetric part of an FP32 3x3 matrix as Voigt values in FP64; all NaN if |a_ij - a_ji| > 1e-8 max |a_kl|
// (smf_kernel.hpp:408-421), checked in FP64 on the FP32 values
MF_D void sym_voigt_f(const float *xi, double *v) {
  double a9[9], mx = 0.0;
#pragma unroll
  for (int k = 0; k < 9; k++) { a9[k] = xi[k]; mx = sel(fabs(a9[k]) > mx, fabs(a9[k]), mx); }
  const double tol = 1e-8 * mx;
  bool sym = !(fabs(a9[1] - a9[3]) > tol) & !(fabs(a9[2] - a9[6]) > tol) & !(fabs(a9[5] - a9[7]) > tol);
  v[0] = a9[0]; v[1] = a9[4]; v[2] = a9[8];
  v[3] = 0.5 * (a9[1] + a9[3]); v[4] = 0.5 * (a9[2] + a9[6]); v[5] = 0.5 * (a9[5] + a9[7]);
#pragma unroll
  for (int k = 0; k < 6; k++) v[k] = sel(sym, v[k], __longlong_as_double(0x7FF8000000000000ll));
}

// the spectrum of the mixed path, eigenvalues sorted ascending: FP32 eigenvectors V (columns), eigenvalues lf,
// their differences taken in FP64 and rounded once (d10 = l1 - l0, d21, d20), and f(lambda) (log near the mean
// through log1p of the deviator's eigenvalue, smf_kernel.hpp:283-290); powers see max(lambda, 0)
struct SmfSpecF {
  float lf[3], fl[3], V[3][3], d10, d21, d20;
};

template <int KIND>
MF_D void smf_spectrum_f(const double *v, const SmfCoefF &C, SmfSpecF &Sp) {
  SmfEigM E;
  smf_eigsys_mixed<KIND>(v, E);
  double lam[3] = {E.lam[0], E.lam[1], E.lam[2]}, xd[3] = {E.xd[0], E.xd[1], E.xd[2]};
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Sp.V[i][j] = E.V[i][j];
#pragma unroll
  for (int st = 0; st < 3; st++) {  // sort ascending (FP64 keys): a static order for every divided difference
    const int a = st == 1 ? 1 : 0, b = a + 1;
    bool sw = lam[b] < lam[a];
    double la = lam[a], lb = lam[b], xa = xd[a], xb = xd[b];
    lam[a] = sel(sw, lb, la); lam[b] = sel(sw, la, lb);
    xd[a] = sel(sw, xb, xa); xd[b] = sel(sw, xa, xb);
#pragma unroll
    for (int r = 0; r < 3; r++) {
      float va = Sp.V[r][a], vb = Sp.V[r][b];
      Sp.V[r][a] = self(sw, vb, va); Sp.V[r][b] = self(sw, va, vb);
    }
  }
  if (KIND == POW || KIND == SQRT) {
#pragma unroll
    for (int i = 0; i < 3; i++) lam[i] = sel(lam[i] > 0.0, lam[i], 0.0);
  }
#pragma unroll
  for (int i = 0; i < 3; i++) Sp.lf[i] = (float)lam[i];
  Sp.d10 = (float)(lam[1] - lam[0]); Sp.d21 = (float)(lam[2] - lam[1]); Sp.d20 = (float)(lam[2] - lam[0]);
#pragma unroll
  for (int i = 0; i < 3; i++) Sp.fl[i] = fun_f<KIND>(Sp.lf[i], C.al);
  if (KIND == LOG) {
    float mf = (float)E.m, lms = logf(mf);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      float x = (float)xd[i];
      Sp.fl[i] = self(fabsf(x) <= 0.5f * mf, lms + log1pf(x / mf), Sp.fl[i]);
    }
  }
}

// first divided differences D_ij = f[l_i, l_j] (D_ii = f'(l_i)) in FP32
template <int KIND>
MF_D void smf_dm_f(const SmfSpecF &Sp, const SmfCoefF &C, float Dm[3][3]) {
  const float D01 = dd1s_f<KIND>(Sp.lf[0], Sp.lf[1], Sp.d10, Sp.fl[0], Sp.fl[1], C);
  const float D02 = dd1s_f<KIND>(Sp.lf[0], Sp.lf[2], Sp.d20, Sp.fl[0], Sp.fl[2], C);
  const float D12 = dd1s_f<KIND>(Sp.lf[1], Sp.lf[2], Sp.d21, Sp.fl[1], Sp.fl[2], C);
  Dm[0][0] = deriv_f<KIND>(Sp.lf[0], Sp.fl[0], C); Dm[1][1] = deriv_f<KIND>(Sp.lf[1], Sp.fl[1], C);
  Dm[2][2] = deriv_f<KIND>(Sp.lf[2], Sp.fl[2], C);
  Dm[0][1] = Dm[1][0] = D01; Dm[0][2] = Dm[2][0] = D02; Dm[1][2] = Dm[2][1] = D12;
}

// second divided differences D2_ijl = f[l_i, l_j, l_l] (symmetric) in FP32
template <int KIND>
MF_D void smf_d2_f(const SmfSpecF &Sp, const float Dm[3][3], const SmfCoefF &C, float D2[3][3][3]) {
  const float dd[3][3] = {{0.f, Sp.d10, Sp.d20}, {0.f, 0.f, Sp.d21}, {0.f, 0.f, 0.f}};
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++)
#pragma unroll
      for (int l = j; l < 3; l++) {
        const float d = (i == j && j == l)
                            ? dd2_same_f<KIND>(Sp.lf[i], Sp.fl[i], Dm[i][i], C)
                            : dd2s_f<KIND>(Sp.lf[j], Sp.lf[l], Sp.fl[j], Dm[i][j], Dm[j][l], dd[i][j], dd[j][l],
                                           dd[i][l], C);
        D2[i][j][l] = D2[i][l][j] = D2[j][i][l] = D2[j][l][i] = D2[l][i][j] = D2[l][j][i] = d;
      }
}

constexpr int SMFX_TPB = 64;  // matrices per CTA of the standalone kernel

template <int ORDER, bool MAT, int TPB>
struct SmfxTileSmem {
  static constexpr int NIN = MAT ? 9 : 6, NF = MAT ? 9 : 6;
  float sX[TPB * NIN];
  float sF[TPB * NF];
  float sK[ORDER >= 1 ? TPB * 21 : 1];
  float sG[ORDER >= 2 ? TPB * 56 : 1];
};

template <int KIND, int ORDER, bool MAT, int SMFX_TPB>
MF_D void smf_mixed_tile(int64_t base, int cnt, const float *__restrict__ x, float *__restrict__ F,
                         float *__restrict__ J, float *__restrict__ H, const SmfCoefF &C,
                         SmfxTileSmem<ORDER, MAT, SMFX_TPB> &TS) {
  constexpr int NIN = MAT ? 9 : 6, NF = MAT ? 9 : 6, NJ = NF * NF, NH = NJ * NF;
  float *sX = TS.sX, *sF = TS.sF, *sK = TS.sK, *sG = TS.sG;
  const int tid = threadIdx.x;
  for (int e = tid; e < cnt * NIN; e += SMFX_TPB) sX[e] = x[base * NIN + e];
  __syncthreads();
  if (tid < cnt) {
    double v[6];
    const float *xi = sX + tid * NIN;
    if (MAT) {
      sym_voigt_f(xi, v);
    } else {
#pragma unroll
      for (int k = 0; k < 6; k++) v[k] = xi[k];
    }
    SmfSpecF Sp;
    smf_spectrum_f<KIND>(v, C, Sp);
    const float(&V)[3][3] = Sp.V;
    const float *fl = Sp.fl;
    float Fv[6];
#pragma unroll
    for (int s = 0; s < 6; s++) {
      const int a = vk_(s), b = vl_(s);
      Fv[s] = V[a][0] * fl[0] * V[b][0] + V[a][1] * fl[1] * V[b][1] + V[a][2] * fl[2] * V[b][2];
    }
    if (MAT) {
#pragma unroll
      for (int m = 0; m < 9; m++) sF[tid * 9 + m] = Fv[m % 4 == 0 ? m / 4 : (m == 1 || m == 3 ? 3 : (m == 2 || m == 6 ? 4 : 5))];
    } else {
#pragma unroll
      for (int s = 0; s < 6; s++) sF[tid * 6 + s] = Fv[s];
    }
    if (ORDER >= 1) {
      float Dm[3][3];
      smf_dm_f<KIND>(Sp, C, Dm);
      float P[6][3];
#pragma unroll
      for (int s6 = 0; s6 < 6; s6++)
#pragma unroll
        for (int a = 0; a < 3; a++) P[s6][a] = V[vk_(s6)][a] * V[vl_(s6)][a];
      {
        float Bv[21];
#pragma unroll
        for (int g = 0; g < 6; g++) {
          float dy[3];
#pragma unroll
          for (int a = 0; a < 3; a++) dy[a] = Dm[a][0] * P[g][0] + Dm[a][1] * P[g][1] + Dm[a][2] * P[g][2];
#pragma unroll
          for (int b2 = 0; b2 <= g; b2++) Bv[sym2(b2, g)] = P[b2][0] * dy[0] + P[b2][1] * dy[1] + P[b2][2] * dy[2];
        }
        float *k_out = sK + tid * 21;
#pragma unroll
        for (int I = 0; I < 6; I++)
#pragma unroll
          for (int p = I; p < 6; p++) {
            float acc = 0.f;
            bool first = true;
#pragma unroll
            for (int u1 = 0; u1 < 2; u1++)
#pragma unroll
              for (int u2 = 0; u2 < 2; u2++) {
                if ((u1 && vk_(I) == vl_(I)) || (u2 && vk_(p) == vl_(p))) continue;
                const int s1 = u1 ? vl_(I) : vk_(I), t1 = u1 ? vk_(I) : vl_(I);
                const int s2 = u2 ? vl_(p) : vk_(p), t2 = u2 ? vk_(p) : vl_(p);
                const int pa = pidx(s1, s2), pb = pidx(t1, t2);
                const float v2 = Bv[sym2(min(pa, pb), max(pa, pb))];
                acc = first ? v2 : acc + v2;
                first = false;
              }
            k_out[sym2(I, p)] = acc;
          }
      }
      if (ORDER >= 2) {
        float D2[3][3][3];
        smf_d2_f<KIND>(Sp, Dm, C, D2);
        float Tv[56];
#pragma unroll
        for (int g = 0; g < 6; g++) {
          float M[3][3];
#pragma unroll
          for (int a = 0; a < 3; a++)
#pragma unroll
            for (int mm = a; mm < 3; mm++)
              M[a][mm] = M[mm][a] = D2[a][mm][0] * P[g][0] + D2[a][mm][1] * P[g][1] + D2[a][mm][2] * P[g][2];
#pragma unroll
          for (int h = 0; h <= g; h++) {
            float W[3];
#pragma unroll
            for (int a = 0; a < 3; a++) W[a] = M[a][0] * P[h][0] + M[a][1] * P[h][1] + M[a][2] * P[h][2];
#pragma unroll
            for (int f = 0; f <= h; f++) Tv[sym3(f, h, g)] = P[f][0] * W[0] + P[f][1] * W[1] + P[f][2] * W[2];
          }
        }
        float *g_out = sG + tid * 56;
#pragma unroll
        for (int z = 0; z < 6; z++)
#pragma unroll
          for (int y = 0; y <= z; y++)
#pragma unroll
            for (int I = 0; I <= y; I++) {
              float acc = 0.f;
              bool first = true;
#pragma unroll
              for (int u1 = 0; u1 < 2; u1++)
#pragma unroll
                for (int u2 = 0; u2 < 2; u2++)
#pragma unroll
                  for (int u3 = 0; u3 < 2; u3++) {
                    if ((u1 && vk_(I) == vl_(I)) || (u2 && vk_(y) == vl_(y)) || (u3 && vk_(z) == vl_(z))) continue;
                    const int s1 = u1 ? vl_(I) : vk_(I), t1 = u1 ? vk_(I) : vl_(I);
                    const int s2 = u2 ? vl_(y) : vk_(y), t2 = u2 ? vk_(y) : vl_(y);
                    const int s3 = u3 ? vl_(z) : vk_(z), t3 = u3 ? vk_(z) : vl_(z);
                    int a1 = pidx(s1, s2), a2 = pidx(t2, s3), a3 = pidx(t1, t3);
                    sort3(a1, a2, a3);
                    const float v3 = Tv[sym3(a1, a2, a3)];
                    acc = first ? v3 : acc + v3;
                    first = false;
                  }
              g_out[sym3(I, y, z)] = acc;
            }
      }
    }
  }
  __syncthreads();
  for (int e = tid; e < cnt * NF; e += SMFX_TPB) F[base * NF + e] = sF[e];
  if (ORDER >= 1) {
    constexpr int KJ = (NJ + SMFX_TPB - 1) / SMFX_TPB;
    int jidx[KJ];
    float jw[KJ];  // layout weight 2^ex (an FP32 multiplication by a power of two is exact)
#pragma unroll
    for (int k = 0; k < KJ; k++) {
      const int w = min(tid + SMFX_TPB * k, NJ - 1);
      int I, p, ex;
      if (MAT) {
        I = midx(w / 9); p = midx(w % 9);
        ex = (I >= 3 ? -1 : 0) + mwt_log2(w % 9);
      } else {
        I = w / 6; p = w % 6;
        ex = I >= 3 ? -1 : 0;
      }
      jidx[k] = sym2(min(I, p), max(I, p));
      jw[k] = __int_as_float((127 + ex) << 23);
    }
    for (int mi = 0; mi < cnt; mi++) {
      float *o = J + (base + mi) * NJ;
      const float *s = sK + mi * 21;
#pragma unroll
      for (int k = 0; k < KJ; k++)
        if (tid + SMFX_TPB * k < NJ) o[tid + SMFX_TPB * k] = s[jidx[k]] * jw[k];
    }
  }
  if (ORDER >= 2) {
    constexpr int KH = (NH + SMFX_TPB - 1) / SMFX_TPB;
    int hidx[KH];
    float hw[KH];
#pragma unroll
    for (int k = 0; k < KH; k++) {
      const int w = min(tid + SMFX_TPB * k, NH - 1);
      int I, p, q, ex;
      if (MAT) {
        const int m = w / 81, c = (w / 9) % 9, e = w % 9;
        I = midx(m); p = midx(c); q = midx(e);
        ex = 1 + (I >= 3 ? -1 : 0) + mwt_log2(c) + mwt_log2(e);
      } else {
        I = w / 36; p = (w / 6) % 6; q = w % 6;
        ex = 1 + (I >= 3 ? -1 : 0);
      }
      sort3(I, p, q);
      hidx[k] = sym3(I, p, q);
      hw[k] = __int_as_float((127 + ex) << 23);
    }
    for (int mi = 0; mi < cnt; mi++) {
      float *o = H + (base + mi) * NH;
      const float *s = sG + mi * 56;
#pragma unroll
      for (int k = 0; k < KH; k++)
        if (tid + SMFX_TPB * k < NH) o[tid + SMFX_TPB * k] = s[hidx[k]] * hw[k];
    }
  }
}

template <int KIND, int ORDER, bool MAT>
__global__ void __launch_bounds__(SMFX_TPB) smf_mixed_kernel(int64_t n, const float *__restrict__ x,
                                                             float *__restrict__ F, float *__restrict__ J,
                                                             float *__restrict__ H, const SmfCoefF C) {
  __shared__ SmfxTileSmem<ORDER, MAT, SMFX_TPB> TS;
  const int64_t base = (int64_t)blockIdx.x * SMFX_TPB;
  smf_mixed_tile<KIND, ORDER, MAT, SMFX_TPB>(base, (int)min((int64_t)SMFX_TPB, n - base), x, F, J, H, C, TS);
}

inline void smf_coef_f(int kind, double al, SmfCoefF &C) {
  SmfCoef D;
  smf_coef(kind, al, D);
  C.al = (float)al;
  C.alm1 = (float)(al - 1.0);
  C.zp1 = (float)D.zp1;
  C.z2 = (float)D.z2;
  C.tau = (float)D.tau;
  for (int k = 0; k < DD2_TERMS; k++) C.c2[k] = (float)D.c2[k];
}

template <int KIND>
cudaError_t smf_mixed_launch_t(double al, int64_t n, const float *x, bool mat, float *F, float *J, float *H,
                               cudaStream_t st) {
  SmfCoefF C;
  smf_coef_f(KIND, al, C);
  const int order = H ? 2 : (J ? 1 : 0);
  const unsigned blocks = (unsigned)((n + SMFX_TPB - 1) / SMFX_TPB);
  if (mat) {
    if (order == 2) smf_mixed_kernel<KIND, 2, true><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else if (order == 1) smf_mixed_kernel<KIND, 1, true><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else smf_mixed_kernel<KIND, 0, true><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
  } else {
    if (order == 2) smf_mixed_kernel<KIND, 2, false><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else if (order == 1) smf_mixed_kernel<KIND, 1, false><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else smf_mixed_kernel<KIND, 0, false><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
  }
  return cudaGetLastError();
}

}  // namespace mf
