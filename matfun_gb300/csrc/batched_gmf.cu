// batched_gmf.cu -- gmf tile routines of the batched kernel (relocatable device code, batched_tiles.cuh).
#include "batched_tiles.cuh"

namespace mf {
#define MF_DEF(K, O)                                                                                              \
  __device__ __noinline__ void bt_gmf_##K##_##O MF_BT_SIG {                                                       \
    gmf_tile<K, O>(base, cnt, (const double *)R.x, (double *)R.F, (double *)R.J, (double *)R.H,                  \
                   *(const GmfCoef *)coef, *(GmfSmem *)smem, R.idx);                                                 \
  }
MF_DEF(0, 0) MF_DEF(0, 1) MF_DEF(0, 2) MF_DEF(1, 0) MF_DEF(1, 1) MF_DEF(1, 2) MF_DEF(2, 0) MF_DEF(2, 1) MF_DEF(2, 2)
}  // namespace mf
