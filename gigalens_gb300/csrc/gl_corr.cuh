// Register-blocked 1-D correlation rows: the building block of the
// PSF + supersample-binning correlations (forward and transposed) of the
// fused and least-squares kernels.  A parity plane row segment and one
// sub-kernel row are held in registers; each thread produces kColBlock
// adjacent outputs.
#pragma once
#include "gl_internal.cuh"

namespace gl {

// ---------------------------------------------------------------- correlation
// acc[c] += sum_l k[l] * seg[c + l]  (REV: k[KS-1-l]); seg and krow 16-byte aligned.
template <int KS, bool REV>
__device__ __forceinline__ void corr_row(const float* __restrict__ seg,
                                         const float* __restrict__ krow, float (&acc)[kColBlock]) {
  constexpr int SEGN = (kColBlock + KS - 1 + 3) & ~3;
  constexpr int KSP = (KS + 3) & ~3;
  float s[SEGN];
  float k[KSP];
#pragma unroll
  for (int i = 0; i < SEGN / 4; ++i) {
    float4 t = reinterpret_cast<const float4*>(seg)[i];
    s[4 * i] = t.x;
    s[4 * i + 1] = t.y;
    s[4 * i + 2] = t.z;
    s[4 * i + 3] = t.w;
  }
#pragma unroll
  for (int i = 0; i < KSP / 4; ++i) {
    float4 t = reinterpret_cast<const float4*>(krow)[i];
    k[4 * i] = t.x;
    k[4 * i + 1] = t.y;
    k[4 * i + 2] = t.z;
    k[4 * i + 3] = t.w;
  }
#pragma unroll
  for (int l = 0; l < KS; ++l) {
    const float kv = REV ? k[KS - 1 - l] : k[l];
#pragma unroll
    for (int c = 0; c < kColBlock; ++c) acc[c] = fmaf(kv, s[c + l], acc[c]);
  }
}

#define GL_KS_DISPATCH(KSVAL, CALL) \
  switch (KSVAL) {                  \
    case 1: CALL(1); break;         \
    case 3: CALL(3); break;         \
    case 5: CALL(5); break;         \
    case 7: CALL(7); break;         \
    case 9: CALL(9); break;         \
    case 11: CALL(11); break;       \
    case 13: CALL(13); break;       \
    case 15: CALL(15); break;       \
    case 17: CALL(17); break;       \
    case 19: CALL(19); break;       \
    case 21: CALL(21); break;       \
    case 23: CALL(23); break;       \
    case 25: CALL(25); break;       \
    default: break;                 \
  }

}  // namespace gl
