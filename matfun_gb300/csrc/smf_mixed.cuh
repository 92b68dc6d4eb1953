// smf_mixed.cuh -- mixed-precision symmetric family: the standalone kernels and their launch.  The matrix layout,
// order 0 and store path 0 run the tile of smf_mixed_tile.cuh (per-entry stores of the expanded rows); the Voigt
// layout at orders 1 and 2 runs smf_mixed_voigt_kernel below, whose J and H rows the TMA unit writes.
#pragma once
#include "smf_kernels.cuh"
#include "smf_mixed_tile.cuh"
#include "tma_store.cuh"

#include <atomic>

namespace mf {

template <int KIND, int ORDER, bool MAT>
__global__ void __launch_bounds__(SMFX_TPB) smf_mixed_kernel(int64_t n, const float *__restrict__ x,
                                                             float *__restrict__ F, float *__restrict__ J,
                                                             float *__restrict__ H, const SmfCoefF C) {
  __shared__ SmfxTileSmem<ORDER, MAT, SMFX_TPB> TS;
  const int64_t base = (int64_t)blockIdx.x * SMFX_TPB;
  smf_mixed_tile<KIND, ORDER, MAT, SMFX_TPB>(base, (int)min((int64_t)SMFX_TPB, n - base), x, F, J, H, C, TS);
}


// ---- Voigt layout: J and H rows written by the TMA unit (orders 1 and 2), F by each lane (every order).  Each warp
// takes 32 consecutive matrices, one per lane, and each lane reads its own input row: no staging, no CTA barrier, so
// a warp starts when its own loads arrive and the warps of a CTA drift apart (boxes drain while other warps
// compute).  A lane keeps its matrix's distinct J (21) and H (56) values in registers and writes its own row
// chunks, weighted, as 16-byte shared-memory stores into a swizzled box of 32 rows x BW floats; one lane hands each
// box to the TMA unit (columns and rows past the array are clipped by the unit), two boxes per warp in flight.  This
// replaces the CTA-wide expansion through per-entry gathers and 4-byte stores.  Variants (the box width and the CTAs
// per SM the registers are bounded for) trade registers and shared memory against resident warps; which one runs is
// a tuning choice (smf_voigt_variant).
constexpr int SMFV_TPB = 64;  // matrices (threads) per CTA

// chunk c (entries 4c .. 4c + 3) of a Voigt J row: J[I][p] = K[I, p] / (1 + [I >= 3])
MF_D float4 smfv_jchunk(const float (&K)[21], int c) {
  float v[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int w = min(4 * c + k, 35), I = w / 6, p = w % 6;
    const float e = K[sym2(min(I, p), max(I, p))];
    v[k] = I >= 3 ? 0.5f * e : e;
  }
  return make_float4(v[0], v[1], v[2], v[3]);
}

// chunk c of a Voigt H row: H[I][p][q] = G[sort(I, p, q)] (2 for I < 3, 1 for I >= 3)
MF_D float4 smfv_hchunk(const float (&G)[56], int c) {
  float v[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int w = min(4 * c + k, 215);
    int I = w / 36, p = (w / 6) % 6, q = w % 6;
    const bool dbl = I < 3;
    sort3(I, p, q);
    const float e = G[sym3(I, p, q)];
    v[k] = dbl ? 2.f * e : e;
  }
  return make_float4(v[0], v[1], v[2], v[3]);
}

// box geometry: BW = 32 floats (128-byte rows, 128-byte swizzle) or 16 (64-byte rows, 64-byte swizzle); the 16-byte
// chunk c of row r lies at r * 4 BW + 16 (c ^ phase(r)), so that the 8 lanes of a quarter warp storing one chunk of
// their own rows cover every bank once
template <int BW>
struct SmfvBox {
  static_assert(BW == 32 || BW == 16, "128- or 64-byte box rows");
  static constexpr int CH = BW / 4;                 // chunks per box row
  static constexpr int BYTES = 32 * BW * 4;         // one box
  static constexpr int ALIGN = BW == 32 ? 1024 : 512;  // the swizzle's period
  MF_D static void put(unsigned char *box, int r, int c, float4 v) {
    const int ph = BW == 32 ? (r & 7) : ((r >> 1) & 3);
    *reinterpret_cast<float4 *>(box + r * (BW * 4) + ((c ^ ph) << 4)) = v;
  }
};

// the chunks [CH q, CH q + CH) of the rows of this warp's lanes, chunk(c) for c < NC, into the box at b; then stored
// to columns 4 CH q ... of rows row0 ... by lane 0
template <int BW, typename Chunk>
MF_D void smfv_box(unsigned char *b, int q, int NC, int lane, const CUtensorMap *map, int row0, Chunk chunk) {
  using B = SmfvBox<BW>;
#pragma unroll
  for (int c = 0; c < B::CH; c++)
    if (B::CH * q + c < NC) B::put(b, lane, c, chunk(B::CH * q + c));
  fence_async_smem();
  __syncwarp();
  if (lane == 0) tma_store_box(map, b, BW * q, row0);
}

template <int KIND, int ORDER, int MINB, int BW>
__global__ void __launch_bounds__(SMFV_TPB, MINB)
    smf_mixed_voigt_kernel(int64_t n, const float *__restrict__ x, float *__restrict__ F,
                           const __grid_constant__ CUtensorMap mJ, const __grid_constant__ CUtensorMap mH,
                           const SmfCoefF C) {
  static_assert(ORDER >= 0 && ORDER <= 2, "F, J and H");
  using B = SmfvBox<BW>;
  constexpr int NJB = (9 + B::CH - 1) / B::CH, NHB = (54 + B::CH - 1) / B::CH;  // boxes of a J and an H row
  // two boxes per warp, at the swizzle's period (none at order 0): the CTA's only shared memory
  __shared__ __align__(B::ALIGN) unsigned char raw[ORDER == 0 ? 16 : SMFV_TPB / 32 * 2 * B::BYTES];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * SMFV_TPB;
  const int cnt = (int)min((int64_t)SMFV_TPB, n - base);
  const int64_t row0 = base + warp * 32;
  // (a box off the swizzle's period would be written in the wrong order: such a CTA writes nothing)
  if (row0 >= n || (ORDER > 0 && (smem_u32(raw) & (B::ALIGN - 1)) != 0)) return;
  const bool live = tid < cnt;
  unsigned char *bufs[2];
  bufs[0] = raw + warp * 2 * B::BYTES;
  bufs[1] = bufs[0] + B::BYTES;

  // each lane reads its own matrix (the warp's 32 rows are 768 contiguous bytes); lanes past the end evaluate the
  // identity (rows the TMA unit clips), so that the warp stays converged
  float xin[6];
#pragma unroll
  for (int k = 0; k < 6; k++) xin[k] = live ? x[(base + tid) * 6 + k] : (k < 3 ? 1.f : 0.f);
  SmfInF in;
  voigt_in_f(xin, in);
  SmfSpecF Sp;
  smf_spectrum_f<KIND, false>(in, C, Sp);
  const float(&V)[3][3] = Sp.V;
  if (live) {
    float *o = F + (base + tid) * 6;
#pragma unroll
    for (int s = 0; s < 6; s++) {
      const int a = vk_(s), b = vl_(s);
      o[s] = V[a][0] * Sp.fl[0] * V[b][0] + V[a][1] * Sp.fl[1] * V[b][1] + V[a][2] * Sp.fl[2] * V[b][2];
    }
  }
  if (ORDER == 0) return;
  float Dm[3][3];
  smf_dm_f<KIND>(Sp, C, Dm);
  // the second divided differences before the J boxes: their 10 values stay live across them instead of the spectrum
  float D2[3][3][3];
  if (ORDER >= 2) smf_d2_f<KIND>(Sp, Dm, C, D2);
  float P[6][3];
  smfx_pvec(V, P);
  int nb = 0;  // boxes issued by this warp; box k uses buffer k & 1
  {
    float K[21];
    smfx_jform(P, Dm, K);
#pragma unroll
    for (int q = 0; q < NJB; q++, nb++) {
      if (nb >= 2) {
        if (lane == 0) tma_wait_read<1>();  // the box stored from this buffer two boxes ago has been read
        __syncwarp();
      }
      smfv_box<BW>(bufs[nb & 1], q, 9, lane, &mJ, (int)row0, [&](int c) { return smfv_jchunk(K, c); });
    }
  }
  if (ORDER >= 2) {
    float G[56];
    smfx_hform(P, D2, G);
#pragma unroll
    for (int q = 0; q < NHB; q++, nb++) {
      if (nb >= 2) {
        if (lane == 0) tma_wait_read<1>();
        __syncwarp();
      }
      smfv_box<BW>(bufs[nb & 1], q, 54, lane, &mH, (int)row0, [&](int c) { return smfv_hchunk(G, c); });
    }
  }
  if (lane == 0) tma_wait_read<0>();  // shared memory stays until the unit has read it
}

// the store path of the Voigt FP32 kernels at orders 1-2: 0 = per-entry stores (smf_mixed_kernel), 1 = TMA boxes of
// 128-byte rows (registers bounded for 8 CTAs per SM at order 2, 12 at order 1), 2 = TMA boxes of 64-byte rows
// (12 CTAs per SM at order 2, 16 at order 1), 3 = TMA boxes of 64-byte rows at 14 CTAs per SM (order 2; 12 at order 1)
extern std::atomic<int> smf_voigt_variant[2];  // (by order - 1)

template <int KIND, int ORDER>
cudaError_t smfv_launch(int variant, int64_t n, const float *x, float *F, float *J, float *H, const SmfCoefF &C,
                        cudaStream_t st) {
  const int bw = variant == 1 ? 32 : 16;
  CUtensorMap mJ, mH;
  if (!tma_map_rows(&mJ, J, n, 36, bw) || (ORDER == 2 && !tma_map_rows(&mH, H, n, 216, bw)))
    return cudaErrorNotSupported;
  if (ORDER == 1) mH = mJ;
  const unsigned vb = (unsigned)((n + SMFV_TPB - 1) / SMFV_TPB);
  if (variant == 1) smf_mixed_voigt_kernel<KIND, ORDER, ORDER == 2 ? 8 : 12, 32><<<vb, SMFV_TPB, 0, st>>>(n, x, F, mJ, mH, C);
  else if (variant == 3) smf_mixed_voigt_kernel<KIND, ORDER, ORDER == 2 ? 14 : 12, 16><<<vb, SMFV_TPB, 0, st>>>(n, x, F, mJ, mH, C);
  else smf_mixed_voigt_kernel<KIND, ORDER, ORDER == 2 ? 12 : 16, 16><<<vb, SMFV_TPB, 0, st>>>(n, x, F, mJ, mH, C);
  return cudaGetLastError();
}

template <int KIND>
cudaError_t smf_mixed_launch_t(double al, int64_t n, const float *x, bool mat, float *F, float *J, float *H,
                               cudaStream_t st) {
  SmfCoefF C;
  smf_coef_f(KIND, al, C);
  const int order = H ? 2 : (J ? 1 : 0);
  const int variant = order >= 1 ? smf_voigt_variant[order - 1].load() : 0;
  if (!mat && order == 0) {  // F only: the per-lane kernel without boxes (no tensor maps; its map arguments unused)
    CUtensorMap none{};
    smf_mixed_voigt_kernel<KIND, 0, 16, 16>
        <<<(unsigned)((n + SMFV_TPB - 1) / SMFV_TPB), SMFV_TPB, 0, st>>>(n, x, F, none, none, C);
    return cudaGetLastError();
  }
  if (!mat && variant != 0) {
    const cudaError_t e = order == 2 ? smfv_launch<KIND, 2>(variant, n, x, F, J, H, C, st)
                                     : smfv_launch<KIND, 1>(variant, n, x, F, J, H, C, st);
    if (e != cudaErrorNotSupported) return e;  // (else: J or H does not qualify for the TMA unit)
  }
  const unsigned blocks = (unsigned)((n + SMFX_TPB - 1) / SMFX_TPB);
  if (mat) {
    if (order == 2) smf_mixed_kernel<KIND, 2, true><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else if (order == 1) smf_mixed_kernel<KIND, 1, true><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else smf_mixed_kernel<KIND, 0, true><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
  } else {
    if (order == 2) smf_mixed_kernel<KIND, 2, false><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
    else smf_mixed_kernel<KIND, 1, false><<<blocks, SMFX_TPB, 0, st>>>(n, x, F, J, H, C);
  }
  return cudaGetLastError();
}

}  // namespace mf
