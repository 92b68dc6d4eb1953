// smf_mixed_tile.cuh -- one tile of the mixed-precision symmetric family: coalesced FP32 input, the eigensystem and
// divided differences of smf_mixed_math.cuh per thread, the J / H forms of smf_tile.cuh in FP32 (smfx_jform,
// smfx_hform, which the TMA-store kernel of smf_mixed.cuh shares), coalesced FP32 output; the code a CTA of the
// standalone kernel and of the batched persistent kernel runs.
#pragma once

#include "smf_mixed_math.cuh"
#include "smf_tile.cuh"

namespace mf {

constexpr int SMFX_TPB = 64;  // matrices per CTA of the standalone kernel

// (order 2: the inputs are staged in the last TPB * NIN floats of sG, read before sG receives results -- 21 KB per
// 64 Voigt matrices, 10 CTAs per SM)
template <int ORDER, bool MAT, int TPB>
struct SmfxTileSmem {
  static constexpr int NIN = MAT ? 9 : 6, NF = MAT ? 9 : 6;
  float sX[ORDER >= 2 ? 1 : TPB * NIN];
  float sF[TPB * NF];
  float sK[ORDER >= 1 ? TPB * 21 : 1];
  float sG[ORDER >= 2 ? TPB * 56 : 1];
};

// product vectors of the Voigt pairs s = (k, l): P[s][a] = V[k][a] V[l][a]
MF_D void smfx_pvec(const float (&V)[3][3], float (&P)[6][3]) {
#pragma unroll
  for (int s6 = 0; s6 < 6; s6++)
#pragma unroll
    for (int a = 0; a < 3; a++) P[s6][a] = V[vk_(s6)][a] * V[vl_(s6)][a];
}

// the 21 distinct values of J's symmetric form, K[sym2(I, p)] (I <= p, Voigt indices), through the 21 values of
// B(x, y) = sum_ab Dm_ab x_a y_b on the product vectors
MF_D void smfx_jform(const float (&P)[6][3], const float (&Dm)[3][3], float (&K)[21]) {
  float Bv[21];
#pragma unroll
  for (int g = 0; g < 6; g++) {
    float dy[3];
#pragma unroll
    for (int a = 0; a < 3; a++) dy[a] = Dm[a][0] * P[g][0] + Dm[a][1] * P[g][1] + Dm[a][2] * P[g][2];
#pragma unroll
    for (int b2 = 0; b2 <= g; b2++) Bv[sym2(b2, g)] = P[b2][0] * dy[0] + P[b2][1] * dy[1] + P[b2][2] * dy[2];
  }
#pragma unroll
  for (int I = 0; I < 6; I++)
#pragma unroll
    for (int p = I; p < 6; p++) {
      float acc = 0.f;
      bool first = true;
#pragma unroll
      for (int u1 = 0; u1 < 2; u1++)
#pragma unroll
        for (int u2 = 0; u2 < 2; u2++) {
          if ((u1 && vk_(I) == vl_(I)) || (u2 && vk_(p) == vl_(p))) continue;
          const int s1 = u1 ? vl_(I) : vk_(I), t1 = u1 ? vk_(I) : vl_(I);
          const int s2 = u2 ? vl_(p) : vk_(p), t2 = u2 ? vk_(p) : vl_(p);
          const int pa = pidx(s1, s2), pb = pidx(t1, t2);
          const float v2 = Bv[sym2(min(pa, pb), max(pa, pb))];
          acc = first ? v2 : acc + v2;
          first = false;
        }
      K[sym2(I, p)] = acc;
    }
}

// the 56 distinct values of H's symmetric form, G[sym3(I, y, z)] (I <= y <= z), through the 56 values of
// T(x, y, z) = sum_amb D2_amb x_a y_m z_b on the product vectors
MF_D void smfx_hform(const float (&P)[6][3], const float (&D2)[3][3][3], float (&G)[56]) {
  float Tv[56];
#pragma unroll
  for (int g = 0; g < 6; g++) {
    float M[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int mm = a; mm < 3; mm++)
        M[a][mm] = M[mm][a] = D2[a][mm][0] * P[g][0] + D2[a][mm][1] * P[g][1] + D2[a][mm][2] * P[g][2];
#pragma unroll
    for (int h = 0; h <= g; h++) {
      float W[3];
#pragma unroll
      for (int a = 0; a < 3; a++) W[a] = M[a][0] * P[h][0] + M[a][1] * P[h][1] + M[a][2] * P[h][2];
#pragma unroll
      for (int f = 0; f <= h; f++) Tv[sym3(f, h, g)] = P[f][0] * W[0] + P[f][1] * W[1] + P[f][2] * W[2];
    }
  }
#pragma unroll
  for (int z = 0; z < 6; z++)
#pragma unroll
    for (int y = 0; y <= z; y++)
#pragma unroll
      for (int I = 0; I <= y; I++) {
        float acc = 0.f;
        bool first = true;
#pragma unroll
        for (int u1 = 0; u1 < 2; u1++)
#pragma unroll
          for (int u2 = 0; u2 < 2; u2++)
#pragma unroll
            for (int u3 = 0; u3 < 2; u3++) {
              if ((u1 && vk_(I) == vl_(I)) || (u2 && vk_(y) == vl_(y)) || (u3 && vk_(z) == vl_(z))) continue;
              const int s1 = u1 ? vl_(I) : vk_(I), t1 = u1 ? vk_(I) : vl_(I);
              const int s2 = u2 ? vl_(y) : vk_(y), t2 = u2 ? vk_(y) : vl_(y);
              const int s3 = u3 ? vl_(z) : vk_(z), t3 = u3 ? vk_(z) : vl_(z);
              int a1 = pidx(s1, s2), a2 = pidx(t2, s3), a3 = pidx(t1, t3);
              sort3(a1, a2, a3);
              const float v3 = Tv[sym3(a1, a2, a3)];
              acc = first ? v3 : acc + v3;
              first = false;
            }
        G[sym3(I, y, z)] = acc;
      }
}

// (cnt <= SMFX_TPB matrices by a CTA of NT >= SMFX_TPB threads: phase A by the first cnt threads, the cooperative
// loads and stores by all NT)
template <int KIND, int ORDER, bool MAT, int SMFX_TPB, int NT = SMFX_TPB>
MF_D void smf_mixed_tile(int64_t base, int cnt, const float *__restrict__ x, float *__restrict__ F,
                         float *__restrict__ J, float *__restrict__ H, const SmfCoefF &C,
                         SmfxTileSmem<ORDER, MAT, SMFX_TPB> &TS) {
  constexpr int NIN = MAT ? 9 : 6, NF = MAT ? 9 : 6, NJ = NF * NF, NH = NJ * NF;
  float *sF = TS.sF, *sK = TS.sK, *sG = TS.sG;
  float *sX = ORDER >= 2 ? sG + SMFX_TPB * (56 - NIN) : TS.sX;
  const int tid = threadIdx.x;
  for (int e = tid; e < cnt * NIN; e += NT) sX[e] = x[base * NIN + e];
  __syncthreads();
  SmfInF in;
  if (tid < cnt) {
    const float *xi = sX + tid * NIN;
    if (MAT) sym_in_f(xi, in);
    else voigt_in_f(xi, in);
  }
  if (ORDER >= 2) __syncthreads();  // every staged input is read before sG receives results
  if (tid < cnt) {
    SmfSpecF Sp;
    smf_spectrum_f<KIND, MAT>(in, C, Sp);
    const float(&V)[3][3] = Sp.V;
    const float *fl = Sp.fl;
    float Fv[6];
#pragma unroll
    for (int s = 0; s < 6; s++) {
      const int a = vk_(s), b = vl_(s);
      Fv[s] = V[a][0] * fl[0] * V[b][0] + V[a][1] * fl[1] * V[b][1] + V[a][2] * fl[2] * V[b][2];
    }
    if (MAT) {
#pragma unroll
      for (int m = 0; m < 9; m++) sF[tid * 9 + m] = Fv[m % 4 == 0 ? m / 4 : (m == 1 || m == 3 ? 3 : (m == 2 || m == 6 ? 4 : 5))];
    } else {
#pragma unroll
      for (int s = 0; s < 6; s++) sF[tid * 6 + s] = Fv[s];
    }
    if (ORDER >= 1) {
      float Dm[3][3];
      smf_dm_f<KIND>(Sp, C, Dm);
      float P[6][3];
      smfx_pvec(V, P);
      {
        float K[21];
        smfx_jform(P, Dm, K);
        float *k_out = sK + tid * 21;
#pragma unroll
        for (int k = 0; k < 21; k++) k_out[k] = K[k];
      }
      if (ORDER >= 2) {
        float D2[3][3][3];
        smf_d2_f<KIND>(Sp, Dm, C, D2);
        float G[56];
        smfx_hform(P, D2, G);
        float *g_out = sG + tid * 56;
#pragma unroll
        for (int k = 0; k < 56; k++) g_out[k] = G[k];
      }
    }
  }
  __syncthreads();
  for (int e = tid; e < cnt * NF; e += NT) F[base * NF + e] = sF[e];
  if (ORDER >= 1) {
    constexpr int KJ = (NJ + NT - 1) / NT;
    int jidx[KJ];
    float jw[KJ];  // layout weight 2^ex (an FP32 multiplication by a power of two is exact)
#pragma unroll
    for (int k = 0; k < KJ; k++) {
      const int w = min(tid + NT * k, NJ - 1);
      int I, p, ex;
      if (MAT) {
        I = midx(w / 9); p = midx(w % 9);
        ex = (I >= 3 ? -1 : 0) + mwt_log2(w % 9);
      } else {
        I = w / 6; p = w % 6;
        ex = I >= 3 ? -1 : 0;
      }
      jidx[k] = sym2(min(I, p), max(I, p));
      jw[k] = __int_as_float((127 + ex) << 23);
    }
    for (int mi = 0; mi < cnt; mi++) {
      float *o = J + (base + mi) * NJ;
      const float *s = sK + mi * 21;
#pragma unroll
      for (int k = 0; k < KJ; k++)
        if (tid + NT * k < NJ) o[tid + NT * k] = s[jidx[k]] * jw[k];
    }
  }
  if (ORDER >= 2) {
    constexpr int KH = (NH + NT - 1) / NT;
    int hidx[KH];
    float hw[KH];
#pragma unroll
    for (int k = 0; k < KH; k++) {
      const int w = min(tid + NT * k, NH - 1);
      int I, p, q, ex;
      if (MAT) {
        const int m = w / 81, c = (w / 9) % 9, e = w % 9;
        I = midx(m); p = midx(c); q = midx(e);
        ex = 1 + (I >= 3 ? -1 : 0) + mwt_log2(c) + mwt_log2(e);
      } else {
        I = w / 36; p = (w / 6) % 6; q = w % 6;
        ex = 1 + (I >= 3 ? -1 : 0);
      }
      sort3(I, p, q);
      hidx[k] = sym3(I, p, q);
      hw[k] = __int_as_float((127 + ex) << 23);
    }
    for (int mi = 0; mi < cnt; mi++) {
      float *o = H + (base + mi) * NH;
      const float *s = sG + mi * 56;
#pragma unroll
      for (int k = 0; k < KH; k++)
        if (tid + NT * k < NH) o[tid + NT * k] = s[hidx[k]] * hw[k];
    }
  }
}

}  // namespace mf
