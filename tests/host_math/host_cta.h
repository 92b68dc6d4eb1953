// host_cta.h -- a CTA of one thread for a host build of the kernels' tile functions: threadIdx is thread 0, a barrier
// has nothing to wait for, and an atomic is a plain update.  With TPB = 1 every cooperative loop of a tile runs in its
// one thread.
#pragma once

struct HostDim3 {
  unsigned x = 0, y = 0, z = 0;
};
static HostDim3 threadIdx;
inline void __syncthreads() {}
inline int atomicAdd(int *p, int v) {
  const int o = *p;
  *p += v;
  return o;
}
