// host_intrinsics.h -- the few CUDA device intrinsics that the per-matrix math headers of the smf and gmf kernels use,
// written for a host compiler, so that a CPU test can compile those headers (which include <cuda_runtime.h>, whose
// __device__ / __forceinline__ expand to host-compatible qualifiers under gcc) and run their math on the CPU.  Each
// is the exact host counterpart: bit casts by memcpy, IEEE sqrt and division (the device forms are the correctly
// rounded __fsqrt_rn / __fdiv_rn), integer min / max.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

inline int __float_as_int(float x) {
  int i;
  std::memcpy(&i, &x, sizeof i);
  return i;
}
inline float __int_as_float(int i) {
  float x;
  std::memcpy(&x, &i, sizeof x);
  return x;
}
inline long long __double_as_longlong(double x) {
  long long i;
  std::memcpy(&i, &x, sizeof i);
  return i;
}
inline double __longlong_as_double(long long i) {
  double x;
  std::memcpy(&x, &i, sizeof x);
  return x;
}
using std::isfinite;  // a global function in device code
inline float __fsqrt_rn(float x) { return std::sqrt(x); }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
// warp votes for a warp of one lane (the gmf series picks its recursion uniformly per warp): the lane's own predicate
inline unsigned __activemask() { return 1u; }
inline bool __all_sync(unsigned, bool p) { return p; }
