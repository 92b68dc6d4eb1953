// mf_common.cuh -- device helpers shared by the smf and gmf kernels (sm_103a, FP64).
//
// On GB300 the FP64 pipe runs at 1/74 of the FP32 rate (measured: 1.0 vs 74.6 TFLOP/s), so every helper here avoids
// FP64 instructions where an exact integer or select form exists: powers of two are made by masking exponent bits,
// maxima of non-negative values are taken on their bit patterns, and selects are plain register moves.
#pragma once
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace mf {

enum Kind { EXP = 0, LOG = 1, POW = 2, SQRT = 3 };

#define MF_D __device__ __forceinline__

// largest power of two <= x for a positive normal x (also +inf -> +inf): the exponent bits of x alone.  Equals
// ldexp(1, ilogb(x)) of the reference (c/include/matfun/smf_kernel.hpp:53-54) wherever the reference calls it on a
// normal number (it guards against zero and subnormals before every call).
MF_D double pow2floor(double x) {
  return __longlong_as_double(__double_as_longlong(x) & 0x7FF0000000000000ll);
}

// a power of two within a factor 2 of x, 1 outside (1e-300, 1e300) (NaN -> 1): gmf_kernel.hpp:126-131
MF_D double pow2safe(double x) { return (x > 1e-300 && x < 1e300) ? pow2floor(x) : 1.0; }

// select (the front end is slow on long chains of ?: and short-circuit operators in one function body, so the
// device math is written with sel() and the non-short-circuit & and | on bools)
MF_D double sel(bool m, double a, double b) { return m ? a : b; }

// select-based max / min with the reference's NaN behaviour (a NaN in the first argument yields the second)
MF_D double tmax(double a, double b) { return a > b ? a : b; }
MF_D double tmin(double a, double b) { return a < b ? a : b; }

// 0^e: inf for e < 0, 1 for e = 0, 0 for e > 0 (smf_kernel.hpp:57-58)
MF_D double zero_pow(double e) { return e < 0 ? __longlong_as_double(0x7FF0000000000000ll) : (e == 0 ? 1.0 : 0.0); }

// x^(al - k), x > 0, with the exponent al - k = bh + bl split exactly (TwoSum): x^bh (1 + bl log x)
// (smf_kernel.hpp:66-73).  bh, bl depend only on al and k and are computed once on the host when possible.
MF_D double pow_split(double x, double bh, double bl) {
  const double p = pow(x, bh);
  return bl == 0 ? p : p * (1.0 + bl * log(x));
}
MF_D void split_exponent(double al, double k, double &bh, double &bl) {
  bh = al - k;
  const double bb = bh - al;
  bl = (al - (bh - bb)) + (-k - bb);
}

MF_D double copysgn(double x, double y) { return y < 0 ? -fabs(x) : fabs(x); }

// Programmatic dependent launch: this CTA no longer needs what a dependent grid launched with programmatic stream
// serialisation will overwrite, so that grid may start once every CTA of this one has said so or exited.  Without
// such a dependent (a plain launch) it has no effect.  (Host builds of the tile code: nothing to signal.)
MF_D void griddep_launch_dependents() {
#if defined(__CUDA_ARCH__)
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// ------------------------------------------------------------------------------------------- complex (re, im)
struct cx {
  double re, im;
};
MF_D cx cmk(double re, double im) { return cx{re, im}; }
MF_D cx cadd(cx a, cx b) { return cx{a.re + b.re, a.im + b.im}; }
MF_D cx csub(cx a, cx b) { return cx{a.re - b.re, a.im - b.im}; }
MF_D cx cmul(cx a, cx b) { return cx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
MF_D cx cscl(cx a, double s) { return cx{a.re * s, a.im * s}; }
MF_D cx csel(bool m, cx a, cx b) { return cx{m ? a.re : b.re, m ? a.im : b.im}; }
// |a| without overflow of the squares (gmf_kernel.hpp:112-117)
MF_D double cabs_s(cx a) {
  const double ar = fabs(a.re), ai = fabs(a.im), big = tmax(ar, ai), sml = tmin(ar, ai);
  if (!(big > 0)) return 0.0;
  const double q = sml / big;
  return big * sqrt(1.0 + q * q);
}
// 1 / b by Smith's method (gmf_kernel.hpp:118-125)
MF_D cx cinv_s(cx b) {
  const bool sw = fabs(b.im) > fabs(b.re);
  const double p = sw ? b.im : b.re, q = sw ? b.re : b.im;
  const double r = q / (p != 0 ? p : 1.0), den = p + q * r;
  const double re = 1.0 / den, im = -r / den;
  return sw ? cx{-im, -re} : cx{re, im};
}

// ------------------------------------------------------------------------------ symmetric index bookkeeping
// sorted pair (x <= y) of 0..8 -> 0..44 ; sorted triple (x <= y <= z) -> 0..164 (combinatorial number system)
MF_D constexpr int sym2(int x, int y) { return y * (y + 1) / 2 + x; }
MF_D constexpr int sym3(int x, int y, int z) { return z * (z + 1) * (z + 2) / 6 + y * (y + 1) / 2 + x; }
MF_D void sort3(int &a, int &b, int &c) {
  int t;
  if (a > b) { t = a; a = b; b = t; }
  if (b > c) { t = b; b = c; c = t; }
  if (a > b) { t = a; a = b; b = t; }
}

}  // namespace mf
