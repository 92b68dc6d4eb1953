// batched_tiles.cuh -- the tile routines of the batched persistent kernel, one non-inlined device function per
// variant.  They are compiled in three translation units (batched_smf64.cu, batched_smf32.cu, batched_gmf.cu) with
// relocatable device code and linked to the kernel in batched.cu, so that the variants compile in parallel.
#pragma once
#include "gmf_kernels.cuh"
#include "smf_mixed.cuh"

namespace mf {

constexpr int BT_TPB = 128;  // threads per CTA; matrices per tile: gmf 128, smf 64 or 128 (chosen per plan)

struct DevReq {
  int family, kind, order, dtype;
  double alpha;
  long long n;
  const void *x;
  void *F, *J, *H;
  long long coef_off;  // byte offset of the coefficient block
  const int *idx;      // gmf: position p of the request holds matrix idx[p] (the batch order by spectral class), or null
  int tile;            // matrices per tile of this request
};

template <int ORDER, bool MAT, int TM = BT_TPB>
using SmfS = SmfTileSmem<ORDER, MAT, TM>;
template <int ORDER, bool MAT, int TM = BT_TPB>
using SmfxS = SmfxTileSmem<ORDER, MAT, TM>;

#define MF_BT_SIG (long long base, int cnt, const DevReq &R, const unsigned char *coef, unsigned char *smem)
// smf FP64 / FP32 (kind 0..3, order 0..2, layout V / M) and gmf FP64 / FP32 (kind 0..2, order 0..2)
#define MF_BT_DECL(name) extern __device__ __noinline__ void name MF_BT_SIG;
#define MF_BT_SMF(pfx, K, O) MF_BT_DECL(pfx##_##K##_##O##_v) MF_BT_DECL(pfx##_##K##_##O##_m) \
                             MF_BT_DECL(pfx##_##K##_##O##_v64) MF_BT_DECL(pfx##_##K##_##O##_m64)
#define MF_BT_SMF_K(pfx, K) MF_BT_SMF(pfx, K, 0) MF_BT_SMF(pfx, K, 1) MF_BT_SMF(pfx, K, 2)
MF_BT_SMF_K(bt_smf64, 0) MF_BT_SMF_K(bt_smf64, 1) MF_BT_SMF_K(bt_smf64, 2) MF_BT_SMF_K(bt_smf64, 3)
MF_BT_SMF_K(bt_smf32, 0) MF_BT_SMF_K(bt_smf32, 1) MF_BT_SMF_K(bt_smf32, 2) MF_BT_SMF_K(bt_smf32, 3)
#define MF_BT_GMF_K(pfx, K) MF_BT_DECL(pfx##_##K##_0) MF_BT_DECL(pfx##_##K##_1) MF_BT_DECL(pfx##_##K##_2)
MF_BT_GMF_K(bt_gmf, 0) MF_BT_GMF_K(bt_gmf, 1) MF_BT_GMF_K(bt_gmf, 2)
MF_BT_GMF_K(bt_gmf32, 0) MF_BT_GMF_K(bt_gmf32, 1) MF_BT_GMF_K(bt_gmf32, 2)

}  // namespace mf
