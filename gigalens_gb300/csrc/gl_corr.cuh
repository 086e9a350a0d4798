// Register-blocked 1-D correlation rows: the building block of the
// PSF + supersample-binning correlations (forward and transposed) of the
// fused and least-squares kernels.  A parity plane row segment and one
// sub-kernel row are held in registers; each thread produces CB adjacent
// outputs (kFusedCB in the fused kernel, kColBlock in the least-squares one).
#pragma once
#include "gl_internal.cuh"

namespace gl {

// ---------------------------------------------------------------- correlation
// acc[c] += sum_l k[l] * seg[c + l]  (REV: k[KS-1-l]); seg and krow 16-byte aligned.
// The segment is held in registers; the kernel row is read four taps at a
// time (a broadcast 16-byte load), which keeps the live set near CB + SEGN.
template <int KS, bool REV, int CB = kColBlock>
__device__ __forceinline__ void corr_row(const float* __restrict__ seg,
                                         const float* __restrict__ krow, float (&acc)[CB]) {
  constexpr int SEGN = (CB + KS - 1 + 3) & ~3;
  constexpr int NG = (KS + 3) / 4;   // 16-byte groups of the kernel row
  float s[SEGN];
#pragma unroll
  for (int i = 0; i < SEGN / 4; ++i) {
    float4 t = reinterpret_cast<const float4*>(seg)[i];
    s[4 * i] = t.x;
    s[4 * i + 1] = t.y;
    s[4 * i + 2] = t.z;
    s[4 * i + 3] = t.w;
  }
#pragma unroll
  for (int gi = 0; gi < NG; ++gi) {
    const int g = REV ? NG - 1 - gi : gi;
    const float4 t = reinterpret_cast<const float4*>(krow)[g];
    const float kq[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
    for (int ei = 0; ei < 4; ++ei) {
      const int e = REV ? 3 - ei : ei;
      const int kidx = 4 * g + e;
      if (kidx < KS) {
        const int l = REV ? KS - 1 - kidx : kidx;
#pragma unroll
        for (int c = 0; c < CB; ++c) acc[c] = fmaf(kq[e], s[c + l], acc[c]);
      }
    }
  }
}

// n consecutive rows: acc[c] += sum_r sum_l k_r[l] * seg_r[c + l + SHIFT],
// with seg_r = seg + r * seg_pitch (16-byte aligned; SHIFT < 4 skips the
// first floats of the aligned segment) and k_r = krow + r * k_step (REV: taps
// reversed).  The next row's segment is loaded while the current one is
// consumed.  The prefetch of row n (one past the last) must stay inside
// shared memory; its values are not used.
template <int KS, bool REV, int CB, int SHIFT = 0>
__device__ __forceinline__ void corr_rows(const float* __restrict__ seg, int seg_pitch,
                                          const float* __restrict__ krow, int k_step, int n,
                                          float (&acc)[CB]) {
  constexpr int SEGN = (CB + KS - 1 + SHIFT + 3) & ~3;
  constexpr int NG = (KS + 3) / 4;
  float4 cur[SEGN / 4];
#pragma unroll
  for (int i = 0; i < SEGN / 4; ++i) cur[i] = reinterpret_cast<const float4*>(seg)[i];
#pragma unroll 2
  for (int r = 0; r < n; ++r) {
    float4 nxt[SEGN / 4];
    const float4* sn = reinterpret_cast<const float4*>(seg + (r + 1) * seg_pitch);
#pragma unroll
    for (int i = 0; i < SEGN / 4; ++i) nxt[i] = sn[i];
    float s[SEGN];
#pragma unroll
    for (int i = 0; i < SEGN / 4; ++i) {
      s[4 * i] = cur[i].x;
      s[4 * i + 1] = cur[i].y;
      s[4 * i + 2] = cur[i].z;
      s[4 * i + 3] = cur[i].w;
    }
    const float* kr = krow + r * k_step;
#pragma unroll
    for (int gi = 0; gi < NG; ++gi) {
      const int g = REV ? NG - 1 - gi : gi;
      const float4 t = reinterpret_cast<const float4*>(kr)[g];
      const float kq[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
      for (int ei = 0; ei < 4; ++ei) {
        const int e = REV ? 3 - ei : ei;
        const int kidx = 4 * g + e;
        if (kidx < KS) {
          const int l = REV ? KS - 1 - kidx : kidx;
#pragma unroll
          for (int c = 0; c < CB; ++c) acc[c] = fmaf(kq[e], s[c + l + SHIFT], acc[c]);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < SEGN / 4; ++i) cur[i] = nxt[i];
  }
}

// Sub-kernel sides 1..25: odd for every PSF at ss = 1 and for PSF sizes
// k = 1 mod 4 at ss = 2, even for k = 3 mod 4 at ss = 2.
#define GL_KS_DISPATCH(KSVAL, CALL) \
  switch (KSVAL) {                  \
    case 1: CALL(1); break; \
    case 2: CALL(2); break; \
    case 3: CALL(3); break; \
    case 4: CALL(4); break; \
    case 5: CALL(5); break; \
    case 6: CALL(6); break; \
    case 7: CALL(7); break; \
    case 8: CALL(8); break; \
    case 9: CALL(9); break; \
    case 10: CALL(10); break; \
    case 11: CALL(11); break; \
    case 12: CALL(12); break; \
    case 13: CALL(13); break; \
    case 14: CALL(14); break; \
    case 15: CALL(15); break; \
    case 16: CALL(16); break; \
    case 17: CALL(17); break; \
    case 18: CALL(18); break; \
    case 19: CALL(19); break; \
    case 20: CALL(20); break; \
    case 21: CALL(21); break; \
    case 22: CALL(22); break; \
    case 23: CALL(23); break; \
    case 24: CALL(24); break; \
    case 25: CALL(25); break; \
    default: break;                 \
  }

}  // namespace gl
