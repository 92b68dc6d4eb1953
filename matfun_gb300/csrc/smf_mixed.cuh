// smf_mixed.cuh -- mixed-precision symmetric family: the standalone kernel over the tile of smf_mixed_tile.cuh and
// its launch.
#pragma once
#include "smf_kernels.cuh"
#include "smf_mixed_tile.cuh"

namespace mf {

template <int KIND, int ORDER, bool MAT>
__global__ void __launch_bounds__(SMFX_TPB) smf_mixed_kernel(int64_t n, const float *__restrict__ x,
                                                             float *__restrict__ F, float *__restrict__ J,
                                                             float *__restrict__ H, const SmfCoefF C) {
  __shared__ SmfxTileSmem<ORDER, MAT, SMFX_TPB> TS;
  const int64_t base = (int64_t)blockIdx.x * SMFX_TPB;
  smf_mixed_tile<KIND, ORDER, MAT, SMFX_TPB>(base, (int)min((int64_t)SMFX_TPB, n - base), x, F, J, H, C, TS);
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
