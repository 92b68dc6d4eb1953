// tma_store.cuh -- row blocks of an output array written by the tensor memory accelerator: a warp stages a box of
// 32 rows x 64 or 128 bytes in shared memory (swizzled, so that 32 lanes writing one 16-byte chunk of their own rows
// hit every bank once per quarter warp) and one lane hands it to the TMA unit (cp.async.bulk.tensor, bulk-group
// completion).  The unit clips rows and columns beyond the array's extent, so partial tiles need no special case.
//
// Host side: a 2-D tensor map over a row-major FP32 array of `rows` x `cols` (cols * 4 a multiple of 16, base
// address 16-byte aligned), boxes of 32 rows; encoded through the driver entry point
// cuTensorMapEncodeTiled, looked up once through the runtime (the library does not link the driver library).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "mf_common.cuh"

namespace mf {

constexpr int TMA_BOX_ROWS = 32;  // rows of a box (one per lane of a warp)

// ---- device
MF_D uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// generic-proxy writes to shared memory become visible to the bulk copies this thread (after __syncwarp: its warp)
// issues next
MF_D void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// store the box at `box` (shared, aligned to its swizzle's period) to columns x ... of rows y .. y + 31
MF_D void tma_store_box(const CUtensorMap *map, const void *box, int x, int y) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(smem_u32(box))
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// wait until at most N of this thread's bulk groups still read shared memory
template <int N>
MF_D void tma_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

// ---- host
inline PFN_cuTensorMapEncodeTiled_v12000 tma_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// a tensor map of `rows` x `cols` floats at `base` for boxes of 32 rows x `bw` floats (32: 128-byte swizzle, 16:
// 64-byte swizzle); false when the array does not qualify (misaligned base or row stride, more rows than a 32-bit
// coordinate reaches) or the driver entry point is missing
inline bool tma_map_rows(CUtensorMap *map, const float *base, int64_t rows, int cols, int bw = 32) {
  if (!base || rows < 1 || rows > INT32_MAX || (reinterpret_cast<uintptr_t>(base) & 15) || ((cols * 4) & 15))
    return false;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tma_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 4};
  const cuuint32_t box[2] = {(cuuint32_t)bw, TMA_BOX_ROWS}, es[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, bw == 32 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
             CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace mf
