// Fused forward model + likelihood (+ adjoint) kernel.
//
// One CTA evaluates one sample at a time (persistent grid-stride loop over the
// batch).  Per sample, nothing round-trips HBM except the 22 parameters in and
// logL, chi^2 and the gradient out:
//   phase 1  ray-trace every supersampled pixel through the mass profiles and
//            evaluate the light (gigalens/tf/simulator.py:57-81); the image is
//            written to shared memory as ss*ss parity planes with zero halos
//   phase 2  PSF convolution + supersample binning as one strided correlation
//            with the combined kernel (PSF (x) ss*ss box), evaluated only at the
//            N*N output pixels (tf/simulator.py:83-97), fused with the
//            Gaussian log-likelihood, chi^2 (tf/model.py:77-86) and the
//            likelihood adjoint dlogL/dimage
//   phase 3  transposed correlation of the adjoint image back to the
//            supersampled grid (overwrites the parity planes)
//   phase 4  per pixel, recompute the forward (the EPL series once, with the
//            running sums its derivatives need) and run the hand-written
//            reverse mode, accumulating d logL / d(profile parameters)
// then a block reduction and the per-sample chain rule to the flat
// parameter vector (and, for log_prob, the prior and bijector terms).
#pragma once
#include <cstdio>

#include "gl_internal.cuh"
#include "gl_fused_ops.cuh"
#include "gl_corr.cuh"
#include "gl_profiles.cuh"
#include "gl_profiles_gen.cuh"

namespace gl {

template <int FAM>
struct FamTraits;
template <>
struct FamTraits<FAM_EPL_SHEAR_SE_SE> {
  static constexpr bool kShear = true, kLensLight = true;
};
template <>
struct FamTraits<FAM_EPL_SHEAR_SE> {
  static constexpr bool kShear = true, kLensLight = false;
};
template <>
struct FamTraits<FAM_EPL_SE_SE> {
  static constexpr bool kShear = false, kLensLight = true;
};
template <>
struct FamTraits<FAM_EPL_SE> {
  static constexpr bool kShear = false, kLensLight = false;
};
template <>
struct FamTraits<FAM_GENERIC> {
  static constexpr bool kShear = false, kLensLight = false;   // unused: runtime lists
};

// Model signature of the general-path kernels: the mass and light profile
// types, the light groups and the shear.  FAM_GENERIC reads them from GenArgs
// at run time and keeps the per-profile reverse code out of line; the
// compiled signatures (FAM_SIG_*) fix them at compile time, so the profile
// code is inlined per slot and the gradient accumulators stay in registers.
// Column maps, amplitudes and every other per-profile setting still come from
// GenArgs.
template <int FAM>
struct GenSig {
  static constexpr bool kStatic = false;
  static constexpr bool kShear = false;
  static constexpr int kNMass = 0, kNLight = 0;
  __device__ static constexpr int mass(int) { return GL_PROF_NONE; }
  __device__ static constexpr int light(int) { return GL_PROF_NONE; }
  __device__ static constexpr bool src(int) { return false; }
};
template <>
struct GenSig<FAM_SIG_SIE_SHEAR_SE_SE> {   // SIE + shear ; SersicEllipse ; SersicEllipse
  static constexpr bool kStatic = true, kShear = true;
  static constexpr int kNMass = 1, kNLight = 2;
  __device__ static constexpr int mass(int s) { return s == 0 ? GL_PROF_SIE : GL_PROF_NONE; }
  __device__ static constexpr int light(int l) { return l < 2 ? GL_PROF_SERSIC_ELLIPSE : GL_PROF_NONE; }
  __device__ static constexpr bool src(int l) { return l == 1; }
};
template <>
struct GenSig<FAM_SIG_SIS_SHEAR_SE_SE> {   // SIS + shear ; SersicEllipse ; SersicEllipse
  static constexpr bool kStatic = true, kShear = true;
  static constexpr int kNMass = 1, kNLight = 2;
  __device__ static constexpr int mass(int s) { return s == 0 ? GL_PROF_SIS : GL_PROF_NONE; }
  __device__ static constexpr int light(int l) { return l < 2 ? GL_PROF_SERSIC_ELLIPSE : GL_PROF_NONE; }
  __device__ static constexpr bool src(int l) { return l == 1; }
};
template <>
struct GenSig<FAM_SIG_EPL_SHEAR_SHP> {     // EPL + shear ; no lens light ; Shapelets
  static constexpr bool kStatic = true, kShear = true;
  static constexpr int kNMass = 1, kNLight = 1;
  __device__ static constexpr int mass(int s) { return s == 0 ? GL_PROF_EPL : GL_PROF_NONE; }
  __device__ static constexpr int light(int l) { return l == 0 ? GL_PROF_SHAPELETS : GL_PROF_NONE; }
  __device__ static constexpr bool src(int l) { return l == 0; }
};
template <int FAM>
constexpr bool kGenFamily = FAM >= FAM_GENERIC;

// Signature accessors: compile-time for the compiled signatures.
template <class S>
__device__ __forceinline__ int gs_n_mass(const GenArgs& g) {
  if constexpr (S::kStatic) return S::kNMass; else return g.n_mass;
}
template <class S>
__device__ __forceinline__ int gs_mass(const GenArgs& g, int s) {
  if constexpr (S::kStatic) return S::mass(s); else return g.mass[s].type;
}
template <class S>
__device__ __forceinline__ bool gs_shear(const GenArgs& g) {
  if constexpr (S::kStatic) return S::kShear; else return g.has_shear != 0;
}
template <class S>
__device__ __forceinline__ int gs_n_light(const GenArgs& g) {
  if constexpr (S::kStatic) return S::kNLight; else return g.n_light;
}
template <class S>
__device__ __forceinline__ int gs_light(const GenArgs& g, int l) {
  if constexpr (S::kStatic) return S::light(l); else return g.light[l].type;
}
template <class S>
__device__ __forceinline__ bool gs_src(const GenArgs& g, int l) {
  if constexpr (S::kStatic) return S::src(l); else return g.light[l].group == GL_GROUP_SOURCE;
}

// Pixels per thread whose series recurrences interleave (phase 1, phase 4).
constexpr int kPixF = 4;
constexpr int kPixR = 2;

struct SmemStatic {
  float x[GL_MAX_PARAMS];          // physical parameters of the current sample
  float z[GL_MAX_PARAMS];          // unconstrained parameters (z mode)
  float gx[GL_MAX_PARAMS];         // d logL / d x
  float4 tab[kMaxTerms + 2];       // EPL series table (A_n, n A_n, s_n A_n, 0), n = 0..K
  float red[kThreads / 32][kRedSlots];
  float out[kRedSlots];
  int K[GL_MAX_IMAGES];
  // general path
  SerC gser[kGenLight];            // Sersic constants of the light slots
  SieC gsie[kGenMass];             // SIE constants of the mass slots
  float amp[kMaxAmps];             // external amplitudes of the current sample
  float ampg[64];                  // d logL / d (explicit shapelet amplitudes)
  float pref[kMaxShapeletN + 1];   // shapelet normalisations 1/sqrt(2^n sqrt(pi) n!)
};

__device__ __forceinline__ float pget(const float* sx, int col, float dflt) {
  return col >= 0 ? sx[col] : dflt;
}

// ---------------------------------------------------------------- prior
__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + expf(-z)); }
__device__ __forceinline__ float softplusf_(float z) {
  return fmaxf(z, 0.f) + log1pf(expf(-fabsf(z)));
}

__device__ __forceinline__ float bij_forward(const DevPriorLeaf& L, float z) {
  switch (L.dist) {
    case GL_DIST_LOGNORMAL:
      return expf(z);
    case GL_DIST_UNIFORM:
    case GL_DIST_TRUNCNORMAL:
      return L.lo + (L.hi - L.lo) * sigmoidf_(z);
    default:
      return z;
  }
}

// log prior of x, fldj(z); and, if want, d/dz of (logprior + fldj) plus the
// Jacobian dx/dz that multiplies the likelihood gradient.
__device__ __forceinline__ void prior_terms(const DevPriorLeaf& L, float z, float x, float& lp,
                                            float& fldj, float& dxdz, float& dlp_dx,
                                            float& dfldj_dz) {
  const float inf = __int_as_float(0x7f800000);
  switch (L.dist) {
    case GL_DIST_NORMAL: {
      float u = (x - L.loc) / L.scale;
      lp = -0.5f * u * u - logf(L.scale) - kHalfLog2Pi;
      fldj = 0.f;
      dxdz = 1.f;
      dlp_dx = -u / L.scale;
      dfldj_dz = 0.f;
      break;
    }
    case GL_DIST_LOGNORMAL: {
      float y = logf(x);
      float u = (y - L.loc) / L.scale;
      lp = -0.5f * u * u - logf(L.scale) - kHalfLog2Pi - y;
      fldj = z;
      dxdz = x;
      dlp_dx = (-u / L.scale - 1.f) / x;
      dfldj_dz = 1.f;
      break;
    }
    case GL_DIST_UNIFORM: {
      lp = (x >= L.lo && x < L.hi) ? -L.lognorm : -inf;
      float s = sigmoidf_(z), sm = sigmoidf_(-z);
      fldj = L.loglen - softplusf_(-z) - softplusf_(z);
      dxdz = (L.hi - L.lo) * s * sm;
      dlp_dx = 0.f;
      dfldj_dz = sm - s;
      break;
    }
    case GL_DIST_TRUNCNORMAL: {
      float u = (x - L.loc) / L.scale;
      lp = (x >= L.lo && x <= L.hi) ? (-0.5f * u * u - logf(L.scale) - kHalfLog2Pi - L.lognorm) : -inf;
      float s = sigmoidf_(z), sm = sigmoidf_(-z);
      fldj = L.loglen - softplusf_(-z) - softplusf_(z);
      dxdz = (L.hi - L.lo) * s * sm;
      dlp_dx = -u / L.scale;
      dfldj_dz = sm - s;
      break;
    }
    default:
      lp = 0.f;
      fldj = 0.f;
      dxdz = 1.f;
      dlp_dx = 0.f;
      dfldj_dz = 0.f;
  }
}

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Reduce n per-thread values (n <= kRedSlots) across the block into s.out.
template <int NV>
__device__ __forceinline__ void block_reduce(float (&v)[NV], SmemStatic& s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    float r = warp_sum(v[i]);
    if (lane == 0) s.red[warp][i] = r;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    float t = 0.f;
#pragma unroll 1
    for (int w = 0; w < kThreads / 32; ++w) t += s.red[w][threadIdx.x];
    s.out[threadIdx.x] = t;
  }
  __syncthreads();
}

// Correlation work items (phases 2 and 3).  An item is one warp's work: its
// four quarter-warps take the four parity planes (ss = 2) of one group of 8
// units, or four groups of the single plane (ss = 1).  A group is 4 rows x 2
// column blocks of kFusedCB outputs, so the 16-byte shared loads of a
// quarter-warp are conflict-free when the plane pitch is an odd multiple of
// four floats.  Items go to warps round-robin: with 16 warps every SM
// sub-partition receives the same number of items to within one.
__device__ __forceinline__ int conv_items(const DevImage& I) {
  const int groups = ((I.N + 3) >> 2) * (I.ncb >> 1);
  return I.nplanes == 1 ? (groups + 3) >> 2 : groups;
}

__device__ __forceinline__ bool conv_unit(const DevImage& I, int item, int lane, int& i, int& j0,
                                          int& pq) {
  const int qtr = lane >> 3, l8 = lane & 7;
  const int pairs = I.ncb >> 1;
  const int groups = ((I.N + 3) >> 2) * pairs;
  int g;
  if (I.nplanes == 1) {
    g = 4 * item + qtr;
    pq = 0;
  } else {
    g = item;
    pq = qtr;
  }
  const int quad = g / pairs;
  i = 4 * quad + (l8 >> 1);
  j0 = kFusedCB * (2 * (g - quad * pairs) + (l8 & 1));
  return g < groups && i < I.N && j0 < I.N;
}

// Phase 2: PSF + binning + likelihood.  Returns per-thread partial sums.
// With four planes the quarter-warps' partial outputs are combined by a
// reduce-scatter in a fixed order: quarter j ends with outputs 4j..4j+3 of
// its 16-column block, (a_j + a_{j^2}) + (a_{j^1} + a_{j^3}).
template <int KS, bool X2>
static __device__ void phase_conv_forward(const DevImage& I, float* sm, float* img_out, bool want_w,
                                   const float* err_map, float cf, float& lsum, float& csum) {
  const int lane = threadIdx.x & 31, qtr = lane >> 3;
  const int items = conv_items(I);
  auto emit = [&](int i, int j, float conv) {
    if (j >= I.N) return;
    const float im = conv * cf;
    if (img_out) img_out[i * I.N + j] = im;
    if (I.obs) {
      const float o = __ldg(I.obs + i * I.N + j);
      if (err_map) {
        // data noise (tf/model.py:112-116,157-158): sigma fixed
        const float err = __ldg(err_map + i * I.N + j);
        const float zz = (o - im) / err;
        lsum += -0.5f * zz * zz - logf(err) - kHalfLog2Pi;
        csum += zz * zz;
        if (want_w) sm[I.offW + i * I.pitchW + I.padW + j] = zz / err * cf;
      } else {
        // model noise (tf/model.py:76-80): sigma^2 = bg^2 + clip(im, 0)/t
        const float e2 = I.bg2 + fmaxf(im, 0.f) * I.inv_t;
        const float err = sqrtf(e2);
        const float zz = (o - im) / err;
        lsum += -0.5f * zz * zz - logf(err) - kHalfLog2Pi;
        csum += zz * zz;
        if (want_w) {
          const float inv_e = 1.f / err;
          float w = zz * inv_e;
          if (im >= 0.f) w += (zz * zz - 1.f) * 0.5f * inv_e * inv_e * I.inv_t;
          sm[I.offW + i * I.pitchW + I.padW + j] = w * cf;
        }
      }
    }
  };
  for (int it = threadIdx.x >> 5; it < items; it += kWarps) {
    int i, j0, pq;
    const bool valid = conv_unit(I, it, lane, i, j0, pq);
    float acc[kFusedCB];
#pragma unroll
    for (int c = 0; c < kFusedCB; ++c) acc[c] = 0.f;
    if (valid) {
      const int p = pq / I.ss, q = pq - p * I.ss;
      const float* plane = sm + I.offI + pq * I.N * I.pitchI + I.padI[q] - I.d[q] + j0;
      const float* kp = sm + I.offK + pq * KS * I.ksp;
      const int mlo = max(0, I.d[p] - i), mhi = min(KS, I.N + I.d[p] - i);
      if constexpr (X2) {
        CorrX2Acc<kFusedCB> A;
        A.zero();
        corr_rows_x2<KS, false, kFusedCB>(plane + (i + mlo - I.d[p]) * I.pitchI, I.pitchI, kp + mlo * I.ksp,
                                          I.ksp, mhi - mlo, A);
        A.finish(acc);
      } else {
        // the prefetch one row past mhi reads the next plane, the likelihood
        // plane or the sub-kernels: all inside shared memory
        corr_rows<KS, false, kFusedCB>(plane + (i + mlo - I.d[p]) * I.pitchI, I.pitchI, kp + mlo * I.ksp,
                                       I.ksp, mhi - mlo, acc);
      }
    }
    if (I.nplanes == 4) {
      float r8[8], r4[4];
      const bool hi1 = qtr >= 2, hi2 = (qtr & 1) != 0;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const float send = hi1 ? acc[c] : acc[c + 8];
        const float keep = hi1 ? acc[c + 8] : acc[c];
        r8[c] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float send = hi2 ? r8[c] : r8[c + 4];
        const float keep = hi2 ? r8[c + 4] : r8[c];
        r4[c] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
      }
      if (valid) {
#pragma unroll
        for (int c = 0; c < 4; ++c) emit(i, j0 + 4 * qtr + c, r4[c]);
      }
    } else if (valid) {
#pragma unroll
      for (int c = 0; c < kFusedCB; ++c) emit(i, j0 + c, acc[c]);
    }
  }
}

// Items of the transposed correlation.  With four planes a warp takes one
// column parity q and two groups: quarter j handles row parity j & 1 of group
// 2 gp + (j >> 1).  Every lane of the warp then reads the likelihood plane at
// the same offset d[q] - d[0] past a 16-byte boundary (0, or 1 for PSF sizes
// k = 3 mod 4), which the correlation takes as a compile-time shift.
static __device__ __forceinline__ int adj_items(const DevImage& I) {
  const int groups = ((I.N + 3) >> 2) * (I.ncb >> 1);
  return I.nplanes == 1 ? (groups + 3) >> 2 : 2 * ((groups + 1) >> 1);
}

static __device__ __forceinline__ bool adj_unit(const DevImage& I, int item, int lane, int& i,
                                                int& j0, int& pq) {
  const int qtr = lane >> 3, l8 = lane & 7;
  const int pairs = I.ncb >> 1;
  const int groups = ((I.N + 3) >> 2) * pairs;
  int g;
  if (I.nplanes == 1) {
    g = 4 * item + qtr;
    pq = 0;
  } else {
    g = 2 * (item >> 1) + (qtr >> 1);
    pq = (qtr & 1) * I.ss + (item & 1);
  }
  const int quad = g / pairs;
  i = 4 * quad + (l8 >> 1);
  j0 = kFusedCB * (2 * (g - quad * pairs) + (l8 & 1));
  return g < groups && i < I.N && j0 < I.N;
}

// Phase 3: transposed correlation, adjoint image -> supersampled parity planes.
template <int KS, bool X2>
static __device__ void phase_conv_adjoint(const DevImage& I, float* sm) {
  const int lane = threadIdx.x & 31;
  const int items = adj_items(I);
  for (int it = threadIdx.x >> 5; it < items; it += kWarps) {
    int Y, j0, pq;
    if (!adj_unit(I, it, lane, Y, j0, pq)) continue;
    const int p = pq / I.ss, q = pq - p * I.ss;
    const int ep = KS - 1 - I.d[p], eq = KS - 1 - I.d[q];
    float acc[kFusedCB];
#pragma unroll
    for (int c = 0; c < kFusedCB; ++c) acc[c] = 0.f;
    // wb = plane start + (d[q] - d[0]) + j0
    const float* wb = sm + I.offW + I.padW - eq + j0;
    const float* kp = sm + I.offK + pq * KS * I.ksp;
    const int mlo = max(0, ep - Y), mhi = min(KS, I.N + ep - Y);
    const float* row0 = wb + (Y + mlo - ep) * I.pitchW;
    const float* k0 = kp + (KS - 1 - mlo) * I.ksp;
    if constexpr (X2) {
      CorrX2Acc<kFusedCB> A;
      A.zero();
      if constexpr (KS % 2 == 0) {
        if (I.d[q] != I.d[0]) {
          corr_rows_x2<KS, true, kFusedCB, 1>(row0 - 1, I.pitchW, k0, -I.ksp, mhi - mlo, A);
        } else {
          corr_rows_x2<KS, true, kFusedCB, 0>(row0, I.pitchW, k0, -I.ksp, mhi - mlo, A);
        }
      } else {
        corr_rows_x2<KS, true, kFusedCB, 0>(row0, I.pitchW, k0, -I.ksp, mhi - mlo, A);
      }
      A.finish(acc);
    } else {
      // the prefetch one row past mhi reads the spare row after the plane
      if constexpr (KS % 2 == 0) {
        if (I.d[q] != I.d[0]) {
          corr_rows<KS, true, kFusedCB, 1>(row0 - 1, I.pitchW, k0, -I.ksp, mhi - mlo, acc);
        } else {
          corr_rows<KS, true, kFusedCB, 0>(row0, I.pitchW, k0, -I.ksp, mhi - mlo, acc);
        }
      } else {
        corr_rows<KS, true, kFusedCB, 0>(row0, I.pitchW, k0, -I.ksp, mhi - mlo, acc);
      }
    }
    float* dst = sm + I.offI + pq * I.N * I.pitchI + Y * I.pitchI + I.padI[q] + j0;
#pragma unroll
    for (int c = 0; c < kFusedCB; ++c)
      if (j0 + c < I.N) dst[c] = acc[c];
  }
}

// ---------------------------------------------------------------- per-sample consts
template <int FAM>
struct SampleConsts {
  EplC epl;
  float g1, g2;
  SerC ll, src;
  SerC2 lls;   // (lens light, source) packed, families with a lens light
};

template <int FAM>
__device__ __forceinline__ SampleConsts<FAM> make_consts(const FusedArgs& a, const float* sx, int K) {
  using T = FamTraits<FAM>;
  SampleConsts<FAM> c;
  const int* e = a.epl.col;
  c.epl = epl_consts(pget(sx, e[0], 0.f), pget(sx, e[1], 2.f), pget(sx, e[2], 0.f),
                     pget(sx, e[3], 0.f), pget(sx, e[4], 0.f), pget(sx, e[5], 0.f), K);
  if (T::kShear) {
    c.g1 = pget(sx, a.shear.col[0], 0.f);
    c.g2 = pget(sx, a.shear.col[1], 0.f);
  } else {
    c.g1 = c.g2 = 0.f;
  }
  if (T::kLensLight) {
    const int* l = a.llight.col;
    c.ll = sersic_consts(pget(sx, l[0], 1.f), pget(sx, l[1], 1.f), pget(sx, l[2], 0.f),
                         pget(sx, l[3], 0.f), pget(sx, l[4], 0.f), pget(sx, l[5], 0.f),
                         pget(sx, l[6], 1.f));
  }
  const int* s = a.source.col;
  c.src = sersic_consts(pget(sx, s[0], 1.f), pget(sx, s[1], 1.f), pget(sx, s[2], 0.f),
                        pget(sx, s[3], 0.f), pget(sx, s[4], 0.f), pget(sx, s[5], 0.f),
                        pget(sx, s[6], 1.f));
  if (T::kLensLight) c.lls = sersic_pack(c.ll, c.src);
  return c;
}

// Phase 1: light of every supersampled pixel into the parity planes.
template <int FAM>
static __device__ void phase_pixels_forward(const FusedArgs& a, const DevImage& I, float* sm,
                                     const SmemStatic& st, int K) {
  using T = FamTraits<FAM>;
  const SampleConsts<FAM> c = make_consts<FAM>(a, st.x, K);
  const int total = I.nplanes * I.N * I.N;
  const float4* grid = reinterpret_cast<const float4*>(I.grid);
  // light of one pixel from its coordinates and deflection, stored to its plane
  auto finish = [&](const float4& g, float ax, float ay) {
    float bx = g.x - ax, by = g.y - ay;
    if (T::kShear) {
      bx = bx - (c.g1 * g.x + c.g2 * g.y);
      by = by - (c.g2 * g.x - c.g1 * g.y);
    }
    float img;
    if constexpr (T::kLensLight) {   // lens light at theta and source at beta, packed
      const float2 r = sersic_light2(c.lls, make_float2(g.x, bx), make_float2(g.y, by));
      img = r.x + r.y;
    } else {
      img = sersic_light(c.src, bx, by);
    }
    if (isnan(img)) img = 0.f;
    sm[__float_as_int(g.z)] = img;
  };
  // kPixF pixels per iteration: their series evaluations interleave
  int v = threadIdx.x;
  for (; v + (kPixF - 1) * kThreads < total; v += kPixF * kThreads) {
    float4 g[kPixF];
    float x[kPixF], y[kPixF], ax[kPixF], ay[kPixF];
#pragma unroll
    for (int k = 0; k < kPixF; ++k) {
      g[k] = __ldg(grid + v + k * kThreads);
      x[k] = g[k].x;
      y[k] = g[k].y;
    }
    epl_deflect_n<kPixF>(c.epl, st.tab, x, y, ax, ay);
#pragma unroll
    for (int k = 0; k < kPixF; ++k) finish(g[k], ax[k], ay[k]);
  }
  for (; v < total; v += kThreads) {
    const float4 g = __ldg(grid + v);
    float x[1] = {g.x}, y[1] = {g.y}, ax[1], ay[1];
    epl_deflect_n<1>(c.epl, st.tab, x, y, ax, ay);
    finish(g, ax[0], ay[0]);
  }
}

// Slots of the reduced gradient accumulators.
enum : int {
  R_EPL = 0,        // 8: phi SP SPlnR FH FT q cx cy
  R_SH = 8,         // 2
  R_LL = 10,        // 9
  R_SRC = 19,       // 9
  R_NACC = 28
};

// Phase 4: reverse mode per pixel.
template <int FAM>
static __device__ void phase_pixels_reverse(const FusedArgs& a, const DevImage& I, const float* sm,
                                     SmemStatic& st, int K) {
  using T = FamTraits<FAM>;
  const SampleConsts<FAM> c = make_consts<FAM>(a, st.x, K);
  EplAcc ea;
  ea.zero();
  SerAcc la, sa;
  la.zero();
  sa.zero();
  SerAcc2 lsa;   // (lens light, source) accumulators, families with a lens light
  lsa.zero();
  float g1b = 0.f, g2b = 0.f;
  const int total = I.nplanes * I.N * I.N;
  const float4* grid = reinterpret_cast<const float4*>(I.grid);
  // light reverse and parameter accumulation of one pixel
  auto pixel = [&](const float4& xy, float gimg, const EplState& es) {
    float bx = xy.x - es.ax, by = xy.y - es.ay;
    if (T::kShear) {
      bx = bx - (c.g1 * xy.x + c.g2 * xy.y);
      by = by - (c.g2 * xy.x - c.g1 * xy.y);
    }
    float bxb, byb;
    if constexpr (T::kLensLight) {   // lens light at theta and source at beta, packed
      const SerFwd2 f = sersic_fwd2(c.lls, make_float2(xy.x, bx), make_float2(xy.y, by));
      const float img = f.I.x + f.I.y;
      if (isnan(img)) return;   // the reference zeroes NaN pixels: no gradient flows
      float2 Xb, Yb;
      sersic_reverse2(c.lls, f, gimg, lsa, Xb, Yb);
      bxb = Xb.y;
      byb = Yb.y;
    } else {
      const SerFwd sf = sersic_fwd(c.src, bx, by);
      if (isnan(sf.I)) return;
      sersic_reverse(c.src, sf, gimg, sa, bxb, byb);
    }
    const float abx = -bxb, aby = -byb;   // beta = theta - sum alpha
    if (T::kShear) {
      g1b += abx * xy.x - aby * xy.y;
      g2b += abx * xy.y + aby * xy.x;
    }
    epl_backprop(c.epl, es, abx, aby, ea);
  };
  // kPixR pixels per iteration: their series recurrences interleave
  int px = threadIdx.x;
  for (; px + (kPixR - 1) * kThreads < total; px += kPixR * kThreads) {
    float4 g[kPixR];
    float x[kPixR], y[kPixR], gi[kPixR];
#pragma unroll
    for (int k = 0; k < kPixR; ++k) {
      g[k] = __ldg(grid + px + k * kThreads);
      x[k] = g[k].x;
      y[k] = g[k].y;
      gi[k] = sm[__float_as_int(g[k].z)];
    }
    EplState es[kPixR];
    epl_state_n<kPixR>(c.epl, st.tab, x, y, es);
#pragma unroll
    for (int k = 0; k < kPixR; ++k) pixel(g[k], gi[k], es[k]);
  }
  for (; px < total; px += kThreads) {
    const float4 g = __ldg(grid + px);
    pixel(g, sm[__float_as_int(g.z)], epl_state(c.epl, st.tab, g.x, g.y));
  }
  if constexpr (T::kLensLight) {
    la.Ie = lsa.Ie.x; la.RsA = lsa.RsA.x; la.nA = lsa.nA.x; la.bnA = lsa.bnA.x; la.sq = lsa.sq.x;
    la.isq = lsa.isq.x; la.phi = lsa.phi.x; la.cx = lsa.cx.x; la.cy = lsa.cy.x;
    sa.Ie = lsa.Ie.y; sa.RsA = lsa.RsA.y; sa.nA = lsa.nA.y; sa.bnA = lsa.bnA.y; sa.sq = lsa.sq.y;
    sa.isq = lsa.isq.y; sa.phi = lsa.phi.y; sa.cx = lsa.cx.y; sa.cy = lsa.cy.y;
  }
  float v[R_NACC] = {ea.phi, ea.SP, ea.SPlnR, ea.FH, ea.FT, ea.q, ea.cx, ea.cy,
                     g1b, g2b,
                     la.Ie, la.RsA, la.nA, la.bnA, la.sq, la.isq, la.phi, la.cx, la.cy,
                     sa.Ie, sa.RsA, sa.nA, sa.bnA, sa.sq, sa.isq, sa.phi, sa.cx, sa.cy};
  block_reduce<R_NACC>(v, st);
}

__device__ __forceinline__ void scatter(float* gx, const int* cols, const float* vals, int n) {
  for (int i = 0; i < n; ++i)
    if (cols[i] >= 0) gx[cols[i]] += vals[i];
}

// Per-sample chain rule from the reduced accumulators to gx[d] (thread 0).
template <int FAM>
static __device__ void sample_chain(const FusedArgs& a, SmemStatic& st, int K) {
  using T = FamTraits<FAM>;
  const float* sx = st.x;
  const SampleConsts<FAM> c = make_consts<FAM>(a, sx, K);
  for (int i = 0; i < a.d; ++i) st.gx[i] = 0.f;
  const float* o = st.out;
  {
    EplAcc ea;
    ea.phi = o[0]; ea.SP = o[1]; ea.SPlnR = o[2]; ea.FH = o[3];
    ea.FT = o[4]; ea.q = o[5]; ea.cx = o[6]; ea.cy = o[7];
    const int* e = a.epl.col;
    float g[6];
    epl_chain(pget(sx, e[0], 0.f), pget(sx, e[1], 2.f), pget(sx, e[2], 0.f), pget(sx, e[3], 0.f),
              c.epl, ea, g);
    scatter(st.gx, e, g, 6);
  }
  if (T::kShear) {
    float g[2] = {o[R_SH], o[R_SH + 1]};
    scatter(st.gx, a.shear.col, g, 2);
  }
  auto ser = [&](const DevProfile& pr, const SerC& sc, int base) {
    SerAcc sa;
    sa.Ie = o[base]; sa.RsA = o[base + 1]; sa.nA = o[base + 2]; sa.bnA = o[base + 3];
    sa.sq = o[base + 4]; sa.isq = o[base + 5]; sa.phi = o[base + 6]; sa.cx = o[base + 7];
    sa.cy = o[base + 8];
    const int* l = pr.col;
    float g[7];
    sersic_chain(pget(sx, l[0], 1.f), pget(sx, l[1], 1.f), pget(sx, l[2], 0.f), pget(sx, l[3], 0.f),
                 sc, sa, g);
    scatter(st.gx, l, g, 7);
  };
  if (T::kLensLight) ser(a.llight, c.ll, R_LL);
  ser(a.source, c.src, R_SRC);
}


// ================================================================ general path
// Models outside the compiled families: up to kGenMass mass profiles (EPL,
// SIS, SIE, TNFW) plus SHEAR, and up to kGenLight light profiles (Sersic,
// SersicEllipse, CoreSersic, Shapelets), dispatched per pixel.  EPL and
// Sersic use the hand-written reverse mode of the fast path; SIS, SIE, TNFW
// and CoreSersic differentiate their templated formulas with dual numbers;
// shapelets use d phi_n / dt = sqrt(2n) phi_{n-1}.
//
// Reduced accumulators: mass slot s at 8 s (EPL: EplAcc; others: d/d of
// their canonical parameters), shear at 16, light slot l at 18 + 10 l
// (SersicEllipse: SerAcc; CoreSersic: d/d of its 10 parameters; Shapelets:
// d/d beta, center_x, center_y).
enum : int { G_MASS = 0, G_SH = 2 * 8, G_LIGHT = G_SH + 2, G_NACC = G_LIGHT + 10 * kGenLight };
static_assert(G_NACC <= kRedSlots, "general-path accumulators exceed the reduction slots");

__device__ __forceinline__ const DevProfile* gen_epl(const GenArgs& g) {
  for (int s = 0; s < g.n_mass; ++s)
    if (g.mass[s].type == GL_PROF_EPL) return &g.mass[s];
  return nullptr;
}

__device__ __forceinline__ EplC gen_epl_consts(const GenArgs& g, const float* sx, int K) {
  const DevProfile* e = gen_epl(g);
  if (!e) {
    EplC c;
    memset(&c, 0, sizeof(c));
    return c;
  }
  const int* ec = e->col;
  return epl_consts(pget(sx, ec[0], 0.f), pget(sx, ec[1], 2.f), pget(sx, ec[2], 0.f),
                    pget(sx, ec[3], 0.f), pget(sx, ec[4], 0.f), pget(sx, ec[5], 0.f), K);
}

// Amplitude (Ie) of light slot L for the current sample.
__device__ __forceinline__ float gen_amp(const GenLight& L, const SmemStatic& st, int ie_col) {
  return L.amp_ext ? st.amp[L.amp_idx] : pget(st.x, ie_col, 1.f);
}

// Deflection of a non-EPL mass slot (value only).
__device__ __forceinline__ void gen_mass_alpha(const DevProfile& m, int type, int slot, const SmemStatic& st,
                                               float x, float y, float& ax, float& ay) {
  const float* sx = st.x;
  const int* c = m.col;
  switch (type) {
    case GL_PROF_SIS:
      sis_alpha_t<float>(pget(sx, c[0], 0.f), pget(sx, c[1], 0.f), pget(sx, c[2], 0.f), x, y, ax, ay);
      break;
    case GL_PROF_SIE:
      sie_alpha(st.gsie[slot], x, y, ax, ay);
      break;
    case GL_PROF_TNFW:
      tnfw_alpha_t<float>(pget(sx, c[0], 1.f), pget(sx, c[1], 0.f), pget(sx, c[2], 1.f),
                          pget(sx, c[3], 0.f), pget(sx, c[4], 0.f), x, y, ax, ay);
      break;
    default:
      ax = ay = 0.f;
  }
}

// d(alpha)/d(parameters) of a non-EPL mass slot contracted with the
// deflection adjoint (abx, aby), added to acc[0..4].
__device__ __forceinline__ void gen_mass_reverse_body(const DevProfile& m, int type, int slot,
                                                      const SmemStatic& st, float x, float y, float abx,
                                                      float aby, float* acc) {
  using D5 = Dual<5>;
  const float* sx = st.x;
  const int* c = m.col;
  D5 ax, ay;
  int np = 0;
  if (type == GL_PROF_SIE) {   // hand-written reverse mode: adjoints of the per-sample intermediates
    sie_backprop(st.gsie[slot], x, y, abx, aby, acc);
    return;
  }
  switch (type) {
    case GL_PROF_SIS:
      np = 3;
      sis_alpha_t<D5>(D5::seed(pget(sx, c[0], 0.f), 0), D5::seed(pget(sx, c[1], 0.f), 1),
                      D5::seed(pget(sx, c[2], 0.f), 2), x, y, ax, ay);
      break;
    case GL_PROF_TNFW:
      np = 5;
      tnfw_alpha_t<D5>(D5::seed(pget(sx, c[0], 1.f), 0), D5::seed(pget(sx, c[1], 0.f), 1),
                       D5::seed(pget(sx, c[2], 1.f), 2), D5::seed(pget(sx, c[3], 0.f), 3),
                       D5::seed(pget(sx, c[4], 0.f), 4), x, y, ax, ay);
      break;
    default:
      return;
  }
#pragma unroll
  for (int k = 0; k < 5; ++k)
    if (k < np) acc[k] += abx * ax.d[k] + aby * ay.d[k];
}
// Out-of-line form for the run-time signature.
static __device__ __noinline__ void gen_mass_reverse(const DevProfile& m, int slot, const SmemStatic& st,
                                                 float x, float y, float abx, float aby, float* acc) {
  gen_mass_reverse_body(m, m.type, slot, st, x, y, abx, aby, acc);
}

// Value of light slot l at (X, Y).
__device__ __forceinline__ float gen_light(const GenLight& L, int type, int l, const SmemStatic& st,
                                           const float* tab, float X, float Y) {
  const float* sx = st.x;
  const int* c = L.col;
  switch (type) {
    case GL_PROF_SERSIC_ELLIPSE:
      return sersic_light(st.gser[l], X, Y);
    case GL_PROF_CORE_SERSIC:
      return gen_amp(L, st, c[9]) *
             core_sersic_t<float>(pget(sx, c[0], 1.f), pget(sx, c[1], 1.f), pget(sx, c[2], 0.f),
                                  pget(sx, c[3], 1.f), pget(sx, c[4], 0.f), pget(sx, c[5], 0.f),
                                  pget(sx, c[6], 0.f), pget(sx, c[7], 0.f), pget(sx, c[8], 0.f), X, Y);
    case GL_PROF_SHAPELETS: {
      const float beta = pget(sx, c[0], 1.f);
      const float u = (X - pget(sx, c[1], 0.f)) / beta, v = (Y - pget(sx, c[2], 0.f)) / beta;
      const float* amp = L.amp_ext ? st.amp + L.amp_idx : sx + (c[3] >= 0 ? c[3] : 0);
      if (L.interp) return shapelets_sum_interp(u, v, L.n_max, amp, tab, nullptr, nullptr);
      return shapelets_sum(u, v, L.n_max, amp, st.pref, nullptr, nullptr);
    }
    default:
      return 0.f;
  }
}

// Reverse of light slot l at (X, Y) with image adjoint gi: parameter adjoints
// into acc[0..9], evaluation-point adjoint into (Xb, Yb).
__device__ __forceinline__ void gen_light_reverse_body(const GenLight& L, int type, int l, const SmemStatic& st,
                                                       const float* tab, float X, float Y, float gi, float* acc,
                                                       float& Xb, float& Yb) {
  const float* sx = st.x;
  const int* c = L.col;
  switch (type) {
    case GL_PROF_SERSIC_ELLIPSE: {
      const SerFwd f = sersic_fwd(st.gser[l], X, Y);
      SerAcc a;
      a.zero();
      sersic_reverse(st.gser[l], f, gi, a, Xb, Yb);
      acc[0] += a.Ie;
      acc[1] += a.RsA;
      acc[2] += a.nA;
      acc[3] += a.bnA;
      acc[4] += a.sq;
      acc[5] += a.isq;
      acc[6] += a.phi;
      acc[7] += a.cx;
      acc[8] += a.cy;
      break;
    }
    case GL_PROF_CORE_SERSIC: {
      using D11 = Dual<11>;
      const D11 I0 = core_sersic_t<D11>(
          D11::seed(pget(sx, c[0], 1.f), 0), D11::seed(pget(sx, c[1], 1.f), 1),
          D11::seed(pget(sx, c[2], 0.f), 2), D11::seed(pget(sx, c[3], 1.f), 3),
          D11::seed(pget(sx, c[4], 0.f), 4), D11::seed(pget(sx, c[5], 0.f), 5),
          D11::seed(pget(sx, c[6], 0.f), 6), D11::seed(pget(sx, c[7], 0.f), 7),
          D11::seed(pget(sx, c[8], 0.f), 8), D11::seed(X, 9), D11::seed(Y, 10));
      const float ie = gen_amp(L, st, c[9]);
      const float g = gi * ie;
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[k] += g * I0.d[k];
      acc[9] += gi * I0.v;
      Xb = g * I0.d[9];
      Yb = g * I0.d[10];
      break;
    }
    case GL_PROF_SHAPELETS: {
      const float beta = pget(sx, c[0], 1.f);
      const float u = (X - pget(sx, c[1], 0.f)) / beta, v = (Y - pget(sx, c[2], 0.f)) / beta;
      const float* amp = L.amp_ext ? st.amp + L.amp_idx : sx + (c[3] >= 0 ? c[3] : 0);
      float du, dv;
      if (L.interp)
        shapelets_sum_interp(u, v, L.n_max, amp, tab, &du, &dv);
      else
        shapelets_sum(u, v, L.n_max, amp, st.pref, &du, &dv);
      const float ub = gi * du / beta, vb = gi * dv / beta;   // adjoints of X, Y
      acc[0] += -(ub * u + vb * v);                            // d/d beta
      acc[1] -= ub;
      acc[2] -= vb;
      Xb = ub;
      Yb = vb;
      break;
    }
    default:
      Xb = Yb = 0.f;
  }
}

// Out-of-line form for the run-time signature.
static __device__ __noinline__ void gen_light_reverse(const GenLight& L, int l, const SmemStatic& st,
                                                  const float* tab, float X, float Y, float gi, float* acc,
                                                  float& Xb, float& Yb) {
  gen_light_reverse_body(L, L.type, l, st, tab, X, Y, gi, acc, Xb, Yb);
}

// Phase 1 (general path), signature S.
template <class S>
static __device__ void phase_pixels_forward_gen(const FusedArgs& a, const DevImage& I, float* sm,
                                         const SmemStatic& st, int K) {
  const GenArgs& g = a.gen;
  const EplC ec = gen_epl_consts(g, st.x, K);
  const bool has_shear = gs_shear<S>(g);
  const float g1 = has_shear ? pget(st.x, a.shear.col[0], 0.f) : 0.f;
  const float g2 = has_shear ? pget(st.x, a.shear.col[1], 0.f) : 0.f;
  const int total = I.nplanes * I.N * I.N;
  const float4* grid = reinterpret_cast<const float4*>(I.grid);
  for (int px = threadIdx.x; px < total; px += kThreads) {
    const float4 xy = __ldg(grid + px);
    float ax = 0.f, ay = 0.f;
#pragma unroll
    for (int s = 0; s < kGenMass; ++s) {
      if (s < gs_n_mass<S>(g)) {
        float mx, my;
        const int mt = gs_mass<S>(g, s);
        if (mt == GL_PROF_EPL) {
          float xs[1] = {xy.x}, ys[1] = {xy.y}, ox[1], oy[1];
          epl_deflect_n<1>(ec, st.tab, xs, ys, ox, oy);
          mx = ox[0];
          my = oy[0];
        } else {
          gen_mass_alpha(g.mass[s], mt, s, st, xy.x, xy.y, mx, my);
        }
        ax += mx;
        ay += my;
      }
    }
    float bx = xy.x - ax, by = xy.y - ay;
    if (has_shear) {
      bx = bx - (g1 * xy.x + g2 * xy.y);
      by = by - (g2 * xy.x - g1 * xy.y);
    }
    float img = 0.f;
#pragma unroll
    for (int l = 0; l < kGenLight; ++l)
      if (l < gs_n_light<S>(g)) {
        const bool src = gs_src<S>(g, l);
        img += gen_light(g.light[l], gs_light<S>(g, l), l, st, g.shp_tab, src ? bx : xy.x, src ? by : xy.y);
      }
    if (isnan(img)) img = 0.f;
    sm[__float_as_int(xy.z)] = img;
  }
}

// (n1, n2) of shapelet basis function k in the reference's order
// (0,0), (1,0), (0,1), (2,0), (1,1), (0,2), ...
__host__ __device__ constexpr int shp_order(int k) {
  int m = 0;
  while ((m + 1) * (m + 2) / 2 <= k) ++m;
  return m;
}
__host__ __device__ constexpr int shp_n2(int k) { return k - shp_order(k) * (shp_order(k) + 1) / 2; }
__host__ __device__ constexpr int shp_n1(int k) { return shp_order(k) - shp_n2(k); }

// Adds one pixel's amplitude-gradient contributions g * basis_k(u, v) of an
// explicit shapelet profile to the warp's running sums: a reduce-scatter over
// the warp leaves lane l with the sums of amplitudes l and 32 + l.  Every
// lane of the warp calls it (g = 0 where a lane has no pixel).
static __device__ __forceinline__ void shapelet_amp_grad(float g, float u, float v, int nmax,
                                                         const float* pref, const float* tab,
                                                         float& acc_lo, float& acc_hi) {
  const int lane = threadIdx.x & 31;
  float pu[kMaxShapeletN + 1], pv[kMaxShapeletN + 1];
  float fg;
  if (tab) {   // interpolate=True: the tabulated functions carry the Gaussian
    const ShpLerp Lu = shp_lerp(u), Lv = shp_lerp(v);
#pragma unroll
    for (int k = 0; k <= kMaxShapeletN; ++k) {
      pu[k] = k <= nmax ? shp_tab_value(tab, k, Lu) : 0.f;
      pv[k] = k <= nmax ? shp_tab_value(tab, k, Lv) : 0.f;
    }
    fg = g;
  } else {
    shapelet_phis(u, nmax, pref, pu);
    shapelet_phis(v, nmax, pref, pv);
    fg = g * expf(-(u * u + v * v) / 2.f);
  }
  const int D = (nmax + 1) * (nmax + 2) / 2;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float w[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int k = 32 * h + j;
      constexpr int kMaxD = (kMaxShapeletN + 1) * (kMaxShapeletN + 2) / 2;
      w[j] = (k < kMaxD && k < D) ? fg * pu[k < kMaxD ? shp_n1(k) : 0] * pv[k < kMaxD ? shp_n2(k) : 0] : 0.f;
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      const bool up = (lane & off) != 0;
#pragma unroll
      for (int j = 0; j < off; ++j) {
        const float send = up ? w[j] : w[j + off];
        const float keep = up ? w[j + off] : w[j];
        w[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
      }
    }
    if (h == 0) acc_lo += w[0];
    else acc_hi += w[0];
  }
}

// Phase 4 (general path), signature S.
template <class S>
static __device__ void phase_pixels_reverse_gen(const FusedArgs& a, const DevImage& I, const float* sm,
                                         SmemStatic& st, int K) {
  const GenArgs& g = a.gen;
  const EplC ec = gen_epl_consts(g, st.x, K);
  const bool has_shear = gs_shear<S>(g);
  const float g1 = has_shear ? pget(st.x, a.shear.col[0], 0.f) : 0.f;
  const float g2 = has_shear ? pget(st.x, a.shear.col[1], 0.f) : 0.f;
  float acc[G_NACC];
#pragma unroll
  for (int k = 0; k < G_NACC; ++k) acc[k] = 0.f;
  EplAcc ea;
  ea.zero();
  const int total = I.nplanes * I.N * I.N;
  const float4* grid = reinterpret_cast<const float4*>(I.grid);
  const int lane = threadIdx.x & 31;
  const int as = g.amp_grad_slot;   // explicit shapelet slot, or -1
  float amp_lo = 0.f, amp_hi = 0.f;
  // the warp's lanes iterate together (the amplitude gradients reduce over the warp)
  for (int base = threadIdx.x - lane; base < total; base += kThreads) {
    const int px = base + lane;
    float ga = 0.f, su = 0.f, sv = 0.f;   // amplitude-gradient inputs of this pixel
    if (px < total) {
    const float4 xy = __ldg(grid + px);
    const float gimg = sm[__float_as_int(xy.z)];
    // deflection (the EPL keeps its series state for the reverse)
    EplState es;
    float ax = 0.f, ay = 0.f;
#pragma unroll
    for (int s = 0; s < kGenMass; ++s) {
      if (s < gs_n_mass<S>(g)) {
        float mx, my;
        const int mt = gs_mass<S>(g, s);
        if (mt == GL_PROF_EPL) {
          es = epl_state(ec, st.tab, xy.x, xy.y);
          mx = es.ax;
          my = es.ay;
        } else {
          gen_mass_alpha(g.mass[s], mt, s, st, xy.x, xy.y, mx, my);
        }
        ax += mx;
        ay += my;
      }
    }
    float bx = xy.x - ax, by = xy.y - ay;
    if (has_shear) {
      bx = bx - (g1 * xy.x + g2 * xy.y);
      by = by - (g2 * xy.x - g1 * xy.y);
    }
    float img = 0.f;
#pragma unroll
    for (int l = 0; l < kGenLight; ++l)
      if (l < gs_n_light<S>(g)) {
        const bool src = gs_src<S>(g, l);
        img += gen_light(g.light[l], gs_light<S>(g, l), l, st, g.shp_tab, src ? bx : xy.x, src ? by : xy.y);
      }
    if (!isnan(img)) {   // the reference zeroes NaN pixels: no gradient flows
    if (as >= 0) {
      const GenLight& L = g.light[as];
      const bool src = L.group == GL_GROUP_SOURCE;
      const float beta = pget(st.x, L.col[0], 1.f);
      su = ((src ? bx : xy.x) - pget(st.x, L.col[1], 0.f)) / beta;
      sv = ((src ? by : xy.y) - pget(st.x, L.col[2], 0.f)) / beta;
      ga = gimg;
    }
    // light reverse; the sources give the adjoint of beta
    float bxb = 0.f, byb = 0.f;
#pragma unroll
    for (int l = 0; l < kGenLight; ++l)
      if (l < gs_n_light<S>(g)) {
        const bool src = gs_src<S>(g, l);
        float Xb, Yb;
        if constexpr (S::kStatic)
          gen_light_reverse_body(g.light[l], S::light(l), l, st, g.shp_tab, src ? bx : xy.x, src ? by : xy.y,
                                 gimg, acc + G_LIGHT + 10 * l, Xb, Yb);
        else
          gen_light_reverse(g.light[l], l, st, g.shp_tab, src ? bx : xy.x, src ? by : xy.y, gimg,
                            acc + G_LIGHT + 10 * l, Xb, Yb);
        if (src) {
          bxb += Xb;
          byb += Yb;
        }
      }
    const float abx = -bxb, aby = -byb;   // beta = theta - sum alpha
    if (has_shear) {
      acc[G_SH] += abx * xy.x - aby * xy.y;
      acc[G_SH + 1] += abx * xy.y + aby * xy.x;
    }
#pragma unroll
    for (int s = 0; s < kGenMass; ++s)
      if (s < gs_n_mass<S>(g)) {
        if (gs_mass<S>(g, s) == GL_PROF_EPL)
          epl_backprop(ec, es, abx, aby, ea);
        else if constexpr (S::kStatic)
          gen_mass_reverse_body(g.mass[s], S::mass(s), s, st, xy.x, xy.y, abx, aby, acc + G_MASS + 8 * s);
        else
          gen_mass_reverse(g.mass[s], s, st, xy.x, xy.y, abx, aby, acc + G_MASS + 8 * s);
      }
    }   // !isnan(img)
    }   // px < total
    if (as >= 0)
      shapelet_amp_grad(ga, su, sv, g.light[as].n_max, st.pref, g.light[as].interp ? g.shp_tab : nullptr,
                        amp_lo, amp_hi);
  }
  // the EPL slot's accumulators
#pragma unroll
  for (int s = 0; s < kGenMass; ++s)
    if (s < gs_n_mass<S>(g) && gs_mass<S>(g, s) == GL_PROF_EPL) {
      float* e = acc + G_MASS + 8 * s;
      e[0] = ea.phi; e[1] = ea.SP; e[2] = ea.SPlnR; e[3] = ea.FH;
      e[4] = ea.FT; e[5] = ea.q; e[6] = ea.cx; e[7] = ea.cy;
    }
  block_reduce<G_NACC>(acc, st);   // ends with a barrier: st.red is free again
  if (as >= 0) {
    // amplitude gradients: the warps' lane sums, over the warps
    const int warp = threadIdx.x >> 5;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      st.red[warp][lane] = h == 0 ? amp_lo : amp_hi;
      __syncthreads();
      if (threadIdx.x < 32) {
        float s = 0.f;
        for (int w = 0; w < kWarps; ++w) s += st.red[w][threadIdx.x];
        st.ampg[32 * h + threadIdx.x] = s;
      }
      __syncthreads();
    }
  }
}

// Per-sample chain rule of the general path (thread 0).
static __device__ void sample_chain_gen(const FusedArgs& a, SmemStatic& st, int K) {
  const GenArgs& g = a.gen;
  const float* sx = st.x;
  const float* o = st.out;
  for (int i = 0; i < a.d; ++i) st.gx[i] = 0.f;
  for (int s = 0; s < g.n_mass; ++s) {
    const DevProfile& m = g.mass[s];
    const float* e = o + G_MASS + 8 * s;
    if (m.type == GL_PROF_EPL) {
      const EplC ec = gen_epl_consts(g, sx, K);
      EplAcc ea;
      ea.phi = e[0]; ea.SP = e[1]; ea.SPlnR = e[2]; ea.FH = e[3];
      ea.FT = e[4]; ea.q = e[5]; ea.cx = e[6]; ea.cy = e[7];
      float gr[6];
      epl_chain(pget(sx, m.col[0], 0.f), pget(sx, m.col[1], 2.f), pget(sx, m.col[2], 0.f),
                pget(sx, m.col[3], 0.f), ec, ea, gr);
      scatter(st.gx, m.col, gr, 6);
    } else if (m.type == GL_PROF_SIE) {
      float gr[5];
      sie_chain(pget(sx, m.col[0], 0.f), pget(sx, m.col[1], 0.f), pget(sx, m.col[2], 0.f), e, gr);
      scatter(st.gx, m.col, gr, 5);
    } else {
      const int np = m.type == GL_PROF_SIS ? 3 : 5;
      scatter(st.gx, m.col, e, np);
    }
  }
  if (g.has_shear) scatter(st.gx, a.shear.col, o + G_SH, 2);
  for (int l = 0; l < g.n_light; ++l) {
    const GenLight& L = g.light[l];
    const float* e = o + G_LIGHT + 10 * l;
    if (L.type == GL_PROF_SERSIC_ELLIPSE) {
      SerAcc sa;
      sa.Ie = e[0]; sa.RsA = e[1]; sa.nA = e[2]; sa.bnA = e[3]; sa.sq = e[4];
      sa.isq = e[5]; sa.phi = e[6]; sa.cx = e[7]; sa.cy = e[8];
      float gr[7];
      sersic_chain(pget(sx, L.col[0], 1.f), pget(sx, L.col[1], 1.f), pget(sx, L.col[2], 0.f),
                   pget(sx, L.col[3], 0.f), st.gser[l], sa, gr);
      int cols[7];
      for (int k = 0; k < 7; ++k) cols[k] = L.col[k];
      if (L.amp_ext) cols[6] = -1;
      scatter(st.gx, cols, gr, 7);
    } else if (L.type == GL_PROF_CORE_SERSIC) {
      int cols[10];
      for (int k = 0; k < 10; ++k) cols[k] = L.col[k];
      if (L.amp_ext) cols[9] = -1;
      scatter(st.gx, cols, e, 10);
    } else if (L.type == GL_PROF_SHAPELETS) {
      scatter(st.gx, L.col, e, 3);
      if (l == g.amp_grad_slot) {
        const int D = (L.n_max + 1) * (L.n_max + 2) / 2;
        for (int k = 0; k < D; ++k) st.gx[L.col[3] + k] += st.ampg[k];
      }
    }
  }
}

// Term counts of the EPL series per image: the reference's batch-max rule.
static __device__ void compute_term_counts(const FusedArgs& a, SmemStatic& st) {
  float mx[GL_MAX_IMAGES];
  for (int i = 0; i < GL_MAX_IMAGES; ++i) mx[i] = 0.f;
  const int c1 = a.epl.col[2], c2 = a.epl.col[3];
  for (int b = threadIdx.x; b < a.bs; b += kThreads) {
    const int im = a.img_id ? a.img_id[b] : 0;
    float e1 = c1 >= 0 ? a.x[(size_t)b * a.d + c1] : 0.f;
    float e2 = c2 >= 0 ? a.x[(size_t)b * a.d + c2] : 0.f;
    if (a.zmode) {
      if (c1 >= 0) e1 = bij_forward(a.prior[c1], e1);
      if (c2 >= 0) e2 = bij_forward(a.prior[c2], e2);
    }
    const float f = epl_f_of(e1, e2);
    for (int i = 0; i < GL_MAX_IMAGES; ++i)
      if (i == im) mx[i] = fmaxf(mx[i], f);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = 0; i < a.n_images; ++i) {
    float m = mx[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) st.red[warp][i] = m;
  }
  __syncthreads();
  if (threadIdx.x < a.n_images) {
    float m = 0.f;
    for (int w = 0; w < kThreads / 32; ++w) m = fmaxf(m, st.red[w][threadIdx.x]);
    st.K[threadIdx.x] = epl_terms_from_maxf(m, a.epl.niter);
  }
  __syncthreads();
}

// Set up shared memory for image I: zero the planes (their halos must be zero)
// and copy the parity sub-kernels.
static __device__ void setup_image(const DevImage& I, float* sm) {
  for (int i = threadIdx.x; i < I.offK; i += kThreads) sm[i] = 0.f;
  const int nk = I.nplanes * I.KS * I.ksp;
  for (int i = threadIdx.x; i < nk; i += kThreads) sm[I.offK + i] = __ldg(I.kern + i);
}

// X2: PSF correlations on packed FFMA2 (corr_rows_x2) or scalar FFMA (corr_rows).
template <int FAM, bool GMEM, bool X2>
__global__ void __launch_bounds__(kThreads, 1) fused_kernel(const __grid_constant__ FusedArgs a) {
  extern __shared__ float4 smem_dyn[];
  // the image planes: dynamic shared memory, or (GMEM) this CTA's slice of a
  // global, L2-resident scratch when the image does not fit in shared memory.
  // Separate instantiations, so the shared-memory kernels address shared
  // memory directly.
  float* sm;
  if constexpr (GMEM)
    sm = a.gscratch + (size_t)blockIdx.x * a.cta_floats;
  else
    sm = reinterpret_cast<float*>(smem_dyn);
  __shared__ SmemStatic st;
  const int tid = threadIdx.x;

  compute_term_counts(a, st);
  if (kGenFamily<FAM> && tid <= kMaxShapeletN) {
    double f = 1.0;
    for (int i = 2; i <= tid; ++i) f *= i;
    st.pref[tid] = (float)(1.0 / sqrt(pow(2.0, (double)tid) * sqrt(3.14159265358979323846) * f));
  }

  int cur = -1;
  for (int b = blockIdx.x; b < a.bs; b += gridDim.x) {
    const int im = a.img_id ? a.img_id[b] : 0;
    if (im < 0 || im >= a.n_images) {   // bad image index: flag the sample, touch nothing else
      if (tid == 0) {
        if (a.logL) a.logL[b] = __int_as_float(0x7fc00000);
        if (a.chi2) a.chi2[b] = __int_as_float(0x7fc00000);
        if (a.status) a.status[b] = 4;
      }
      continue;
    }
    const DevImage& I = a.img[im];
    if (im != cur) {
      setup_image(I, sm);
      cur = im;
    }
    // parameters (and the bijector in z mode)
    if (tid < a.d) {
      const float v = a.x[(size_t)b * a.d + tid];
      if (a.zmode) {
        st.z[tid] = v;
        st.x[tid] = bij_forward(a.prior[tid], v);
      } else {
        st.x[tid] = v;
      }
    }
    if (kGenFamily<FAM> && a.gen.amps && tid < a.gen.n_amp)
      st.amp[tid] = a.gen.amps[(size_t)b * a.gen.n_amp + tid];
    __syncthreads();
    if (kGenFamily<FAM> && tid >= 64 && tid < 64 + a.gen.n_mass) {
      // SIE constants of the general path's mass slots
      const DevProfile& m = a.gen.mass[tid - 64];
      if (m.type == GL_PROF_SIE)
        st.gsie[tid - 64] = sie_consts(pget(st.x, m.col[0], 0.f), pget(st.x, m.col[1], 0.f),
                                       pget(st.x, m.col[2], 0.f), pget(st.x, m.col[3], 0.f),
                                       pget(st.x, m.col[4], 0.f));
    }
    if (kGenFamily<FAM> && tid >= 32 && tid < 32 + a.gen.n_light) {
      // Sersic constants of the general path's light slots
      const GenLight& L = a.gen.light[tid - 32];
      if (L.type == GL_PROF_SERSIC_ELLIPSE) {
        const int* c = L.col;
        const float ie = L.amp_ext ? st.amp[L.amp_idx] : pget(st.x, c[6], 1.f);
        st.gser[tid - 32] = sersic_consts(pget(st.x, c[0], 1.f), pget(st.x, c[1], 1.f),
                                          pget(st.x, c[2], 0.f), pget(st.x, c[3], 0.f),
                                          pget(st.x, c[4], 0.f), pget(st.x, c[5], 0.f), ie);
      }
    }
    // EPL series coefficient table (warp 0)
    const int K = st.K[im];
    if (tid < 32) {
      const int* e = a.epl.col;
      const float e1 = pget(st.x, e[2], 0.f), e2 = pget(st.x, e[3], 0.f);
      epl_build_table(st.tab, epl_f_of(e1, e2), pget(st.x, e[1], 2.f) - 1.f, K, tid);
    }
    __syncthreads();

    if constexpr (kGenFamily<FAM>)
      phase_pixels_forward_gen<GenSig<FAM>>(a, I, sm, st, K);
    else
      phase_pixels_forward<FAM>(a, I, sm, st, K);
    __syncthreads();

    float lsum = 0.f, csum = 0.f;
    float* img_out = a.img_out ? a.img_out + (size_t)b * a.img_stride : nullptr;
    const float* err_map = (kGenFamily<FAM> && a.gen.noise_err) ? I.err : nullptr;
    const float cf = (kGenFamily<FAM> && a.gen.unit_cf) ? 1.f : I.cf;
#define GL_CALL_FWD(KSV) \
  phase_conv_forward<KSV, X2>(I, sm, img_out, a.want_grad != 0, err_map, cf, lsum, csum)
    GL_KS_DISPATCH(I.KS, GL_CALL_FWD)
#undef GL_CALL_FWD
    {
      float v2[2] = {lsum, csum};
      block_reduce<2>(v2, st);   // ends with __syncthreads: w plane complete
    }
    const float logL = st.out[0];
    const float chi2 = st.out[1] / (float)(I.N * I.N);
    __syncthreads();   // st.out is reused by the gradient reduction

    if (a.want_grad) {
#define GL_CALL_ADJ(KSV) phase_conv_adjoint<KSV, X2>(I, sm)
      GL_KS_DISPATCH(I.KS, GL_CALL_ADJ)
#undef GL_CALL_ADJ
      __syncthreads();
      if constexpr (kGenFamily<FAM>) {
        phase_pixels_reverse_gen<GenSig<FAM>>(a, I, sm, st, K);
        if (tid == 0) sample_chain_gen(a, st, K);
      } else {
        phase_pixels_reverse<FAM>(a, I, sm, st, K);
        if (tid == 0) sample_chain<FAM>(a, st, K);
      }
      __syncthreads();
    }

    // outputs
    if (a.zmode) {
      // log posterior = logL + sum_i (log prior_i + fldj_i)
      if (tid < 32) {
        float lp = 0.f;
        for (int i = tid; i < a.d; i += 32) {
          float plp, fl, dxdz, dlpdx, dfl;
          prior_terms(a.prior[i], st.z[i], st.x[i], plp, fl, dxdz, dlpdx, dfl);
          lp += plp + fl;
          if (a.want_grad && a.grad)
            a.grad[(size_t)b * a.d + i] = (st.gx[i] + dlpdx) * dxdz + dfl;
        }
        lp = warp_sum(lp);
        if (tid == 0) {
          const float logp = logL + lp;
          if (a.logL) a.logL[b] = logp;
          if (a.chi2) a.chi2[b] = chi2;
          if (a.status) a.status[b] = isfinite(logp) ? 0 : 1;
        }
      }
    } else {
      const float scale = a.dlogL ? a.dlogL[b] : 1.f;
      if (a.want_grad && a.grad && tid < a.d) a.grad[(size_t)b * a.d + tid] = st.gx[tid] * scale;
      if (tid == 0) {
        if (a.logL) a.logL[b] = logL;
        if (a.chi2) a.chi2[b] = chi2;
        if (a.status) {
          int s = isfinite(logL) ? 0 : 1;
          if (a.want_grad)
            for (int i = 0; i < a.d; ++i)
              if (!isfinite(st.gx[i])) s |= 2;
          a.status[b] = s;
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- host entries
// Defined here, instantiated once per family in gl_fused_fam*.cu so that the
// families compile as separate translation units (in parallel).
template <int FAM, bool GMEM, bool X2>
int fam_launch(const FusedArgs& a, int grid, int smem_bytes, cudaStream_t stream) {
  if constexpr (GMEM) {
    // no dynamic shared memory: give the SM's unified memory to L1, which
    // then holds the planes' working rows and the threads' local arrays
    static bool carveout_set[kMaxDevices];
    const int dev = current_device_slot();
    if (!carveout_set[dev])
      carveout_set[dev] = cudaFuncSetAttribute(fused_kernel<FAM, true, X2>,
                                               cudaFuncAttributePreferredSharedMemoryCarveout,
                                               (int)cudaSharedmemCarveoutMaxL1) == cudaSuccess;
  }
  fused_kernel<FAM, GMEM, X2><<<grid, kThreads, GMEM ? 0 : smem_bytes, stream>>>(a);
  return 0;
}

template <int FAM, bool X2>
cudaError_t fam_set_smem(int smem_bytes) {
  return cudaFuncSetAttribute(fused_kernel<FAM, false, X2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              smem_bytes);
}

// (the general path exists only with global planes)
template <int FAM>
int fam_static_smem() {
  cudaFuncAttributes at;
  if (cudaFuncGetAttributes(&at, fused_kernel<FAM, FAM == FAM_GENERIC, true>) != cudaSuccess) {
    cudaGetLastError();
    return (int)sizeof(SmemStatic);
  }
  return (int)at.sharedSizeBytes;
}

}  // namespace gl
