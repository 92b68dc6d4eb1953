// ffloat.cuh -- float-float arithmetic on the FP32 pipe: a value x = hi + lo with |lo| <= ulp(hi) / 2 (about 48
// significant bits, relative 2^-48 ~ 3.6e-15), built on the error-free transformations
//   two_sum  (Knuth, TAOCP vol. 2, 4.2.2):       a + b = s + e exactly, s = fl(a + b)
//   two_prod (with a fused multiply-add):        a * b = p + e exactly, p = fl(a * b)
// and the compensated dot product Dot2 of Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput.
// 26 (2005)), whose result is as accurate as if computed in twice the working precision and then rounded.
// On GB300 an FP64 instruction costs about 80 FP32 instruction slots, so a handful of these FP32 operations replaces
// one FP64 operation at a fraction of its cost.  The code relies on IEEE FP32 semantics without reassociation (no
// fast-math); products that must stay exact are written with fmaf explicitly.
#pragma once
#include "mf_common.cuh"

namespace mf {

struct ffl {
  float hi, lo;
};

MF_D ffl two_sum(float a, float b) {
  float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
MF_D ffl fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
  float s = a + b;
  return {s, b - (s - a)};
}
MF_D ffl two_prod(float a, float b) {
  float p = a * b;
  return {p, fmaf(a, b, -p)};
}
MF_D ffl ff_add(ffl x, ffl y) {  // accurate under cancellation of the high parts
  ffl s = two_sum(x.hi, y.hi), t = two_sum(x.lo, y.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
MF_D ffl ff_neg(ffl x) { return {-x.hi, -x.lo}; }
MF_D ffl ff_sub(ffl x, ffl y) { return ff_add(x, ff_neg(y)); }
MF_D ffl ff_mul_f(ffl x, float b) {
  ffl p = two_prod(x.hi, b);
  p.lo = fmaf(x.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
MF_D ffl ff_mul(ffl x, ffl y) {
  ffl p = two_prod(x.hi, y.hi);
  p.lo = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, p.lo));
  return fast_two_sum(p.hi, p.lo);
}
MF_D ffl ff_from(float a) { return {a, 0.f}; }
MF_D ffl ff_of(double x) {  // a double rounded to float-float (48 bits; x within FP32's range)
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
MF_D double ff_dbl(ffl x) { return (double)x.hi + (double)x.lo; }
MF_D ffl ff_prod(ffl x, ffl y) {  // x * y, not renormalised (hi = fl(x.hi y.hi), lo the remainder)
  const float p = x.hi * y.hi;
  return {p, fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, fmaf(x.hi, y.hi, -p)))};
}
MF_D ffl ff_add_s(ffl x, ffl y) {  // x + y with one two_sum (error relative to |x| + |y|), renormalised
  const ffl s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
MF_D ffl ff_add3(ffl x, ffl y, ffl z) {  // x + y + z, renormalised
  const ffl s = two_sum(x.hi, y.hi), t = two_sum(s.hi, z.hi);
  return fast_two_sum(t.hi, ((x.lo + y.lo) + (z.lo + s.lo)) + t.lo);
}
MF_D ffl ff_sel(bool m, ffl a, ffl b) { return {m ? a.hi : b.hi, m ? a.lo : b.lo}; }
MF_D void acc_ff_add(ffl &A, ffl p) {  // Sum2 accumulator (A.hi = running sum, A.lo = collected errors) += p
  const ffl t = two_sum(A.hi, p.hi);
  A.hi = t.hi;
  A.lo += t.lo + p.lo;
}

// running compensated sum (Sum2 / Dot2 of Ogita-Rump-Oishi): S + E, every term added through two_sum
struct ffacc {
  float s, e;
};
MF_D void acc_add(ffacc &A, float t) {
  ffl r = two_sum(A.s, t);
  A.s = r.hi;
  A.e += r.lo;
}
MF_D void acc_prod(ffacc &A, float a, float b) {  // += a * b (exact product)
  ffl p = two_prod(a, b);
  acc_add(A, p.hi);
  A.e += p.lo;
}
MF_D void acc_ffprod(ffacc &A, ffl a, float b) {  // += a * b for a float-float a
  ffl p = two_prod(a.hi, b);
  acc_add(A, p.hi);
  A.e = fmaf(a.lo, b, A.e + p.lo);
}
MF_D ffl acc_ff(const ffacc &A) { return two_sum(A.s, A.e); }

}  // namespace mf
