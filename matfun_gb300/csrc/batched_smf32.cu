// batched_smf32.cu -- mixed-precision smf tile routines of the batched kernel (relocatable device code).
#include "batched_tiles.cuh"

namespace mf {
#define MF_DEF(K, O, M, SUF)                                                                                       \
  __device__ __noinline__ void bt_smf32_##K##_##O##_##SUF MF_BT_SIG {                                              \
    smf_mixed_tile<K, O, M, BT_TPB>(base, cnt, (const float *)R.x, (float *)R.F, (float *)R.J, (float *)R.H,       \
                                    *(const SmfCoefF *)coef, *(SmfxS<O, M> *)smem);                               \
  }
#define MF_DEF_K(K) MF_DEF(K, 0, false, v) MF_DEF(K, 1, false, v) MF_DEF(K, 2, false, v) \
                    MF_DEF(K, 0, true, m) MF_DEF(K, 1, true, m) MF_DEF(K, 2, true, m)
MF_DEF_K(0) MF_DEF_K(1) MF_DEF_K(2) MF_DEF_K(3)
}  // namespace mf
