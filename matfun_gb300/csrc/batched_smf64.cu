// batched_smf64.cu -- smf FP64 tile routines of the batched kernel (relocatable device code, batched_tiles.cuh).
#include "batched_tiles.cuh"

namespace mf {
// (SUF v / m: 128 matrices per tile; v64 / m64: 64 matrices per tile; both by the 128 threads of the CTA)
#define MF_DEF(K, O, M, SUF, TM)                                                                                 \
  __device__ __noinline__ void bt_smf64_##K##_##O##_##SUF MF_BT_SIG {                                           \
    smf_tile<K, O, M, TM, BT_TPB>(base, cnt, (const double *)R.x, (double *)R.F, (double *)R.J, (double *)R.H,          \
                                  *(const SmfCoef *)coef, nullptr, *(SmfS<O, M, TM> *)smem);                       \
  }
#define MF_DEF_S(K, O) MF_DEF(K, O, false, v, BT_TPB) MF_DEF(K, O, true, m, BT_TPB) \
                       MF_DEF(K, O, false, v64, 64) MF_DEF(K, O, true, m64, 64)
#define MF_DEF_K(K) MF_DEF_S(K, 0) MF_DEF_S(K, 1) MF_DEF_S(K, 2)
MF_DEF_K(0) MF_DEF_K(1) MF_DEF_K(2) MF_DEF_K(3)
}  // namespace mf
