// batched_smf64.cu -- smf FP64 tile routines of the batched kernel (relocatable device code, batched_tiles.cuh).
#include "batched_tiles.cuh"

namespace mf {
#define MF_DEF(K, O, M, SUF)                                                                                      \
  __device__ __noinline__ void bt_smf64_##K##_##O##_##SUF MF_BT_SIG {                                             \
    smf_tile<K, O, M, BT_TPB>(base, cnt, (const double *)R.x, (double *)R.F, (double *)R.J, (double *)R.H,        \
                              *(const SmfCoef *)coef, nullptr, *(SmfS<O, M> *)smem);                             \
  }
#define MF_DEF_K(K) MF_DEF(K, 0, false, v) MF_DEF(K, 1, false, v) MF_DEF(K, 2, false, v) \
                    MF_DEF(K, 0, true, m) MF_DEF(K, 1, true, m) MF_DEF(K, 2, true, m)
MF_DEF_K(0) MF_DEF_K(1) MF_DEF_K(2) MF_DEF_K(3)
}  // namespace mf
