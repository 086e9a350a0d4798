// Register-blocked 1-D correlation rows: the building block of the
// PSF + supersample-binning correlations (forward and transposed) of the
// fused and least-squares kernels.  A parity plane row segment is held in
// registers and the sub-kernel row is read four taps at a time (a broadcast
// 16-byte load); each thread produces CB adjacent outputs (kFusedCB in the
// fused kernel, 16 or 20 in the least-squares one).
#pragma once
#include "gl_internal.cuh"

namespace gl {

// ---------------------------------------------------------------- correlation
// One row of corr_rows: acc[c] += sum_l k[l] * seg[c + l + SHIFT] with the
// segment already in registers.
template <int KS, bool REV, int CB, int SHIFT, int NV>
__device__ __forceinline__ void corr_row_regs(const float4 (&v)[NV], const float* __restrict__ kr,
                                              float (&acc)[CB]) {
  constexpr int NG = (KS + 3) / 4;
  float s[4 * NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    s[4 * i] = v[i].x;
    s[4 * i + 1] = v[i].y;
    s[4 * i + 2] = v[i].z;
    s[4 * i + 3] = v[i].w;
  }
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
}

// n consecutive rows: acc[c] += sum_r sum_l k_r[l] * seg_r[c + l + SHIFT],
// with seg_r = seg + r * seg_pitch (16-byte aligned; SHIFT < 4 skips the
// first floats of the aligned segment) and k_r = krow + r * k_step (REV: taps
// reversed).  Two register buffers alternate: the next row's segment loads
// while the current one is consumed, with no copies between them.  The
// prefetch may read row n (one past the last), which must stay inside shared
// memory; its values are not used.
template <int KS, bool REV, int CB, int SHIFT = 0>
__device__ __forceinline__ void corr_rows(const float* __restrict__ seg, int seg_pitch,
                                          const float* __restrict__ krow, int k_step, int n,
                                          float (&acc)[CB]) {
  constexpr int NV = ((CB + KS - 1 + SHIFT + 3) & ~3) / 4;
  float4 a[NV], b[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) a[i] = reinterpret_cast<const float4*>(seg)[i];
  int r = 0;
#pragma unroll 1
  for (; r + 1 < n; r += 2) {
    const float4* s1 = reinterpret_cast<const float4*>(seg + (r + 1) * seg_pitch);
#pragma unroll
    for (int i = 0; i < NV; ++i) b[i] = s1[i];
    corr_row_regs<KS, REV, CB, SHIFT>(a, krow + r * k_step, acc);
    const float4* s2 = reinterpret_cast<const float4*>(seg + (r + 2) * seg_pitch);
#pragma unroll
    for (int i = 0; i < NV; ++i) a[i] = s2[i];
    corr_row_regs<KS, REV, CB, SHIFT>(b, krow + (r + 1) * k_step, acc);
  }
  if (r < n) corr_row_regs<KS, REV, CB, SHIFT>(a, krow + r * k_step, acc);
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

namespace gl {

// ---------------------------------------------------------------- packed FFMA2
// The same correlation as corr_rows with Blackwell's two-wide FP32 FMA
// (__ffma2_rn: one instruction, two FMAs).  With t_l the taps in order (REV:
// reversed), acc[c] += sum_l t_l seg[c + l + SHIFT] is split by the parity of
// l + SHIFT so that every pair of segment values an FMA2 reads is an aligned
// half (x, y or z, w) of a 16-byte load, with no register moves:
//   l + SHIFT even: outputs (2m, 2m+1)   += (t_l, t_l) * (s[2m+l+S], s[2m+l+S+1])
//   l + SHIFT odd:  outputs (2m+1, 2m+2) += (t_l, t_l) * (s[2m+1+l+S], s[2m+2+l+S]),
//                   outputs 0 and CB-1 with one scalar FMA each.
// The two classes accumulate separately and are added at the end, so the
// rounding differs from corr_rows (each output is still a float32 sum of the
// same products).  The segment of a row is loaded into registers once
// (single-buffered: the warps of a CTA hide the shared-memory latency).
template <int KS, bool REV, int CB, int SHIFT, int NV>
__device__ __forceinline__ void corr_row_x2(const float4 (&v)[NV], const float* __restrict__ kr,
                                            float2 (&aE)[CB / 2], float2 (&aO)[CB / 2 - 1], float& o0,
                                            float& oL) {
  constexpr int NG = (KS + 3) / 4;
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const float4 t4 = reinterpret_cast<const float4*>(kr)[g];
    const float kq[4] = {t4.x, t4.y, t4.z, t4.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int kidx = 4 * g + e;
      if (kidx < KS) {
        const int l = REV ? KS - 1 - kidx : kidx;   // tap position
        const float t = kq[e];
        const float2 tt = make_float2(t, t);
        if (((l + SHIFT) & 1) == 0) {
#pragma unroll
          for (int m = 0; m < CB / 2; ++m) {
            const int j = 2 * m + l + SHIFT;   // even
            const float4 q = v[j >> 2];
            const float2 sp = (j & 2) ? make_float2(q.z, q.w) : make_float2(q.x, q.y);
            aE[m] = __ffma2_rn(tt, sp, aE[m]);
          }
        } else {
#pragma unroll
          for (int m = 0; m < CB / 2 - 1; ++m) {
            const int j = 2 * m + 1 + l + SHIFT;   // even
            const float4 q = v[j >> 2];
            const float2 sp = (j & 2) ? make_float2(q.z, q.w) : make_float2(q.x, q.y);
            aO[m] = __ffma2_rn(tt, sp, aO[m]);
          }
          {
            const int j0 = l + SHIFT;   // odd
            const float4 q = v[j0 >> 2];
            o0 = fmaf(t, (j0 & 2) ? q.w : q.y, o0);
            const int j1 = CB - 1 + l + SHIFT;   // even
            const float4 r = v[j1 >> 2];
            oL = fmaf(t, (j1 & 2) ? r.z : r.x, oL);
          }
        }
      }
    }
  }
}

// Accumulators of the FFMA2 correlation: output pairs of the even-tap class,
// of the odd-tap class, and the odd class's two end outputs.
template <int CB>
struct CorrX2Acc {
  float2 aE[CB / 2], aO[CB / 2 - 1];
  float o0, oL;
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int m = 0; m < CB / 2; ++m) aE[m] = make_float2(0.f, 0.f);
#pragma unroll
    for (int m = 0; m < CB / 2 - 1; ++m) aO[m] = make_float2(0.f, 0.f);
    o0 = oL = 0.f;
  }
  // out[c] = the sum of both classes for output c
  __device__ __forceinline__ void finish(float (&out)[CB]) const {
#pragma unroll
    for (int m = 0; m < CB / 2; ++m) {
      out[2 * m] = aE[m].x + (m == 0 ? o0 : aO[m - 1].y);
      out[2 * m + 1] = aE[m].y + (m == CB / 2 - 1 ? oL : aO[m].x);
    }
  }
};

// corr_rows with FFMA2 (see corr_row_x2): n rows of seg (16-byte aligned,
// seg_pitch floats apart) against kernel rows krow + r * k_step, added into
// the accumulators.  Reads exactly the segments of rows 0 .. n-1.
template <int KS, bool REV, int CB, int SHIFT = 0>
__device__ __forceinline__ void corr_rows_x2(const float* __restrict__ seg, int seg_pitch,
                                             const float* __restrict__ krow, int k_step, int n,
                                             CorrX2Acc<CB>& A) {
  static_assert(CB % 2 == 0 && CB >= 4, "even column blocks");
  constexpr int NV = ((CB + KS - 1 + SHIFT + 3) & ~3) / 4;
#pragma unroll 1
  for (int r = 0; r < n; ++r) {
    float4 v[NV];
    const float4* s = reinterpret_cast<const float4*>(seg + r * seg_pitch);
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = s[i];
    corr_row_x2<KS, REV, CB, SHIFT>(v, krow + r * k_step, A.aE, A.aO, A.o0, A.oL);
  }
}

}  // namespace gl
