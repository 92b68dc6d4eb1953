// batch_order.cuh -- the family-independent part of the batch-wide ordering of the gmf and smf launches: a key of at
// most GKEY_BINS values per matrix (the family's key kernel writes it with per-block histograms counts[key * nblk +
// block]), one CTA per key scanning its row of block counts, and a stable scatter of the matrix indices into the
// order of the keys.
#pragma once
#include "mf_common.cuh"

namespace mf {

constexpr int GKEY_TPB = 256, GKEY_BINS = 256;

// exclusive prefix sums of the rows counts[k nblk .. (k + 1) nblk) in place (one CTA of 1024 threads per key k,
// coalesced; warp shuffles, then the 32 warp sums) and the row totals
static __global__ void __launch_bounds__(1024) gmf_scan_kernel(int *__restrict__ counts, int nblk,
                                                                int *__restrict__ totals) {
  __shared__ int wsum[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int *row = counts + (int64_t)blockIdx.x * nblk;
  int carry = 0;
  for (int base = 0; base < nblk; base += 1024) {
    const int i = base + (int)threadIdx.x;
    const int v = i < nblk ? row[i] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      x += lane >= o ? y : 0;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, w, o);
        w += lane >= o ? y : 0;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    if (i < nblk) row[i] = carry + (warp ? wsum[warp - 1] : 0) + x - v;
    carry += wsum[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

// order[start(key) + offset(key, block) + rank among the equal keys before it in its block] = i: a stable sort by
// key; start(key) = the exclusive prefix sum of the row totals (GKEY_BINS = GKEY_TPB entries, scanned here)
static __global__ void __launch_bounds__(GKEY_TPB) gmf_scatter_kernel(int n, const unsigned char *__restrict__ keys,
                                                                      const int *__restrict__ offs,
                                                                      const int *__restrict__ totals, int nblk,
                                                                      int *__restrict__ order) {
  __shared__ int sk[GKEY_TPB], start[GKEY_BINS];
  static_assert(GKEY_BINS == GKEY_TPB, "one key per thread in the scan of the totals");
  const int i = blockIdx.x * GKEY_TPB + threadIdx.x;
  sk[threadIdx.x] = i < n ? (int)keys[i] : -1;
  start[threadIdx.x] = totals[threadIdx.x];
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int k = 0; k < GKEY_BINS; k++) {
      const int v = start[k];
      start[k] = acc;
      acc += v;
    }
  }
  __syncthreads();
  if (i < n) {
    const int key = sk[threadIdx.x];
    int r = 0;
    for (int j = 0; j < (int)threadIdx.x; j++) r += sk[j] == key;
    order[start[key] + offs[key * nblk + blockIdx.x] + r] = i;
  }
}

}  // namespace mf
