// Linear-amplitude path: LensSimulator.lstsq_simulate (tf/simulator.py:99-165).
//
//   basis kernel   per (sample, band of output rows; the whole image when
//                  one channel's parity planes fit in shared memory):
//                  ray-trace the band's supersampled pixels once into the
//                  CTA's slice of a global scratch (L2-resident), then for
//                  every basis channel (unit-amplitude lens-light Sersic,
//                  shapelet (n1, n2) functions of the source) evaluate the
//                  channel into the parity planes, apply PSF + binning with
//                  the register-blocked row correlation of the fused kernel,
//                  and store the binned basis X[b][c][pixel] (unweighted, as
//                  `ret`)
//   gram kernel    G_b = X^T W^2 X and h_b = X^T W^2 y, W = 1/err_map
//   solve kernel   coeffs = pinv(G, rcond=1e-6) h: cyclic Jacobi
//                  eigen-decomposition of the symmetric G (for a symmetric
//                  matrix the singular values are |eigenvalues|), eigenvalues
//                  with |lambda| <= rcond * max|lambda| dropped, as
//                  tf.linalg.pinv does
//   image kernel   img = sum_c coeffs_c X_c (no conversion factor, as the
//                  reference), Gaussian log-likelihood with the data-based
//                  error map and chi^2 (BackwardProbModel, tf/model.py:157-163)
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "gl_corr.cuh"
#include "gl_cpasync.cuh"
#include "gl_internal.cuh"
#include "gl_profiles.cuh"
#include "gl_profiles_gen.cuh"
#include "gl_lstsq.cuh"

namespace gl {

// ------------------------------------------------------------------ device helpers
__device__ __forceinline__ float lpget(const float* sx, int col, float dflt) {
  return col >= 0 ? sx[col] : dflt;
}

// Normalised Hermite function values phi_n(u) without the Gaussian,
// H_n(u) / sqrt(2^n sqrt(pi) n!), by the recursion H_n = 2 (u H_{n-1} -
// (n-1) H_{n-2}) (tf/profiles/light/shapelets.py:47-48,77-85), for U
// independent arguments of one order n (the basis kernel evaluates U pixels
// per thread so their chains interleave).
template <int U>
__device__ __forceinline__ void hermite_fn_n(int n, const float (&u)[U], float (&out)[U], const float* pref) {
  float h0[U], h1[U];
#pragma unroll
  for (int k = 0; k < U; ++k) {
    h0[k] = 1.f;
    h1[k] = 2.f * u[k];
  }
  if (n == 0) {
#pragma unroll
    for (int k = 0; k < U; ++k) out[k] = pref[0];
    return;
  }
  // H_i = (2u) H_{i-1} - 2(i-1) H_{i-2}: the factor 2 distributed (exact in
  // binary floating point), two operations per step
  float tu[U];
#pragma unroll
  for (int k = 0; k < U; ++k) tu[k] = 2.f * u[k];
  if constexpr (U % 2 == 0) {
    // pixel pairs on packed FP32 (FMUL2, FFMA2): the same roundings as the
    // scalar step, so the values are identical
    float2 p0[U / 2], p1[U / 2], pt[U / 2];
#pragma unroll
    for (int k = 0; k < U / 2; ++k) {
      p0[k] = make_float2(h0[2 * k], h0[2 * k + 1]);
      p1[k] = make_float2(h1[2 * k], h1[2 * k + 1]);
      pt[k] = make_float2(tu[2 * k], tu[2 * k + 1]);
    }
    for (int i = 2; i <= n; ++i) {
      const float c2 = -(float)(2 * (i - 1));
      const float2 nc = make_float2(c2, c2);
#pragma unroll
      for (int k = 0; k < U / 2; ++k) {
        const float2 h2 = __ffma2_rn(pt[k], p1[k], __fmul2_rn(nc, p0[k]));
        p0[k] = p1[k];
        p1[k] = h2;
      }
    }
#pragma unroll
    for (int k = 0; k < U / 2; ++k) {
      out[2 * k] = p1[k].x * pref[n];
      out[2 * k + 1] = p1[k].y * pref[n];
    }
    return;
  }
  for (int i = 2; i <= n; ++i) {
    const float c2 = (float)(2 * (i - 1));
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const float h2 = fmaf(tu[k], h1[k], -(c2 * h0[k]));
      h0[k] = h1[k];
      h1[k] = h2;
    }
  }
#pragma unroll
  for (int k = 0; k < U; ++k) out[k] = h1[k] * pref[n];
}


struct LsqShared {
  float x[GL_MAX_PARAMS];
  float4 tab[kMaxTerms + 2];
  float red[16][4];   // per warp (at most 16)
  int K[GL_MAX_IMAGES];
};

template <int NT>
__device__ void lsq_term_counts(const LsqArgs& a, LsqShared& st) {
  float mx[GL_MAX_IMAGES];
  for (int i = 0; i < GL_MAX_IMAGES; ++i) mx[i] = 0.f;
  const int c1 = a.epl.col[2], c2 = a.epl.col[3];
  for (int b = threadIdx.x; b < a.bs; b += NT) {
    const int im = a.img_id ? a.img_id[b] : 0;
    const float e1 = c1 >= 0 ? a.x[(size_t)b * a.d + c1] : 0.f;
    const float e2 = c2 >= 0 ? a.x[(size_t)b * a.d + c2] : 0.f;
    const float f = epl_f_of(e1, e2);
    for (int i = 0; i < GL_MAX_IMAGES; ++i)
      if (i == im) mx[i] = fmaxf(mx[i], f);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = 0; i < a.n_images; ++i) {
    float m = mx[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) st.red[warp][i & 3] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int w = 0; w < NT / 32; ++w) t = fmaxf(t, st.red[w][i & 3]);
      st.K[i] = epl_terms_from_maxf(t, a.epl.niter);
    }
    __syncthreads();
  }
}

// i / div for 0 <= i < 2^21 through the float reciprocal inv = 1/div: the
// quotient (i + 0.5) / div lies at least 0.5 / div from an integer, and the
// product's relative error (three roundings, < 2e-7) moves it by less than
// (i + 0.5) * 2e-7 / div < 0.5 / div.  The host checks the index bound.
__device__ __forceinline__ int small_div(int i, float inv) {
  return __float2int_rz(((float)i + 0.5f) * inv);
}

// PSF + binning of one pass: output rows [i0, i0 + nb) of the channels
// c0 .. c0 + CPn - 1 held in the planes.  A unit is (channel slot, column
// block, output row) with the row fastest, so the eight threads of a
// 16-byte load phase read eight consecutive plane rows of one column block:
// with pitch / 4 odd they fall into eight distinct bank groups.
template <int KS, int CB, int NT>
__device__ void lsq_pass_conv(const LsqImage& I, const float* sm, int c0, int nb, int i0,
                              float* __restrict__ Xout /* X[b][0] */) {
  const int units = I.CPn * I.ncbC * nb;
  const float* kern = sm + I.offK;
  for (int u = threadIdx.x; u < units; u += NT) {
    const int rest = u / nb;
    const int il = u - rest * nb;
    const int slot = rest / I.ncbC;
    const int cb = rest - slot * I.ncbC;
    if (c0 + slot >= I.cpass) continue;
    const int j0 = cb * CB;
    CorrX2Acc<CB> A;
    A.zero();
    const float* sbase = sm + (size_t)slot * I.nplanes * I.plane_floats + j0;
    for (int pq = 0; pq < I.nplanes; ++pq) {
      const int p = pq / I.ss;
      // output row i0 + il of parity p reads plane rows i0 + il - d[p] + m
      const float* seg = sbase + pq * I.plane_floats + (il + I.R0 - I.d[p]) * I.pitch;
      corr_rows_x2<KS, false, CB>(seg, I.pitch, kern + pq * KS * I.ksp, I.ksp, KS, A);
    }
    float acc[CB];
    A.finish(acc);
    float* dst = Xout + (size_t)(c0 + slot) * I.xcstride + (size_t)(i0 + il) * I.N + j0;
#pragma unroll
    for (int c = 0; c < CB; ++c)
      if (j0 + c < I.N) dst[c] = acc[c];
  }
}

// Channel evaluation loop over the pixels 0 <= i < per_plane of a plane set
// (i = (plane row - Ya) * N + column, the band's in-image rows from Ya) by
// NTH threads: a thread takes U2 positions i per step and at each position
// the pixel of every one of the NPL parity planes (NPL = ss^2; one index
// division for NPL pixels), so U2 * NPL evaluations and their coordinate
// loads interleave.  val(px, py, v) computes the basis values from their
// coordinates; NaN values are stored as 0 (the reference zeroes NaN pixels).
template <int NTH, int NPL, int U2, bool GF, class Val>
__device__ __forceinline__ void lsq_eval_loop(const LsqImage& I, float* sbase, const float2* bp,
                                              const float4* gp, const float* gfp, bool src, int per_plane,
                                              Val&& val) {
  constexpr int U = NPL * U2;
  const float inv_n = 1.f / (float)I.N;
  const size_t gstride = (size_t)I.N * I.N;   // the grid holds whole-image planes
  float* pb[NPL];                             // plane origins (column parity q = pq % ss)
#pragma unroll
  for (int pq = 0; pq < NPL; ++pq) pb[pq] = sbase + pq * I.plane_floats + I.padI[NPL == 4 ? (pq & 1) : 0];
  for (int i0 = threadIdx.x; i0 < per_plane; i0 += U2 * NTH) {
    float px[U], py[U], gf[U];
#pragma unroll
    for (int m = 0; m < U2; ++m) {
      const int i = min(i0 + m * NTH, per_plane - 1);
#pragma unroll
      for (int pq = 0; pq < NPL; ++pq) {
        if constexpr (GF) gf[m * NPL + pq] = gfp[(size_t)pq * per_plane + i];
        if (src) {
          const float2 bt = bp[(size_t)pq * per_plane + i];
          px[m * NPL + pq] = bt.x;
          py[m * NPL + pq] = bt.y;
        } else {
          const float4 xy = __ldg(gp + pq * gstride + i);
          px[m * NPL + pq] = xy.x;
          py[m * NPL + pq] = xy.y;
        }
      }
    }
    float v[U];
    val(px, py, gf, v);
#pragma unroll
    for (int m = 0; m < U2; ++m) {
      const int i = i0 + m * NTH;
      if (i < per_plane) {
        const int r = small_div(i, inv_n);
        const int off = r * I.pitch + (i - r * I.N);
#pragma unroll
        for (int pq = 0; pq < NPL; ++pq) {
          float x = v[m * NPL + pq];
          if (isnan(x)) x = 0.f;
          pb[pq][off] = x;
        }
      }
    }
  }
}

// Shapelet basis values phi_n1(u) phi_n2(w) exp(-(u^2 + w^2) / 2) of U
// pixels; GF: the Gaussian factors gf were computed once per sample with the
// same operations (lsq_basis_kernel's ray-trace pass).
template <int U, bool GF>
__device__ __forceinline__ void shapelet_vals(const float (&px)[U], const float (&py)[U], const float (&gf)[U],
                                              float cx, float cy, float ib, int n1, int n2, const float* pref,
                                              float (&v)[U]) {
  float u[U], w[U], hu[U], hw[U];
#pragma unroll
  for (int k = 0; k < U; ++k) {
    u[k] = (px[k] - cx) * ib;
    w[k] = (py[k] - cy) * ib;
  }
  hermite_fn_n<U>(n1, u, hu, pref);
  hermite_fn_n<U>(n2, w, hw, pref);
#pragma unroll
  for (int k = 0; k < U; ++k) {
    const float fac = GF ? gf[k] : expf(-(u[k] * u[k] + w[k] * w[k]) / 2.f);
    v[k] = fac * hu[k] * hw[k];
  }
}

// Basis values of one channel (see lsq_eval_loop).
template <int NTH, int NPL, int U2>
__device__ __forceinline__ void lsq_eval_channel(const LsqArgs& a, const LsqImage& I, const float* sx,
                                                 const float* pref, float* sbase, const float2* bp,
                                                 const float4* gp, const float* gfp, const LsqChannel& ch,
                                                 int per_plane) {
  constexpr int U = NPL * U2;
  const LsqProfile& pr = a.prof[ch.prof];
  const bool src = pr.group == GL_GROUP_SOURCE;
  if (ch.kind == 1 && pr.interp) {   // tabulated shapelet functions (interpolate=True)
    const float beta_s = lpget(sx, pr.col[0], 1.f);
    const float cx = lpget(sx, pr.col[1], 0.f), cy = lpget(sx, pr.col[2], 0.f);
    const float* tab = a.shp_tab;
    const int n1 = ch.n1, n2 = ch.n2;
    lsq_eval_loop<NTH, NPL, U2, false>(I, sbase, bp, gp, nullptr, src, per_plane,
                                [=](const float (&px)[U], const float (&py)[U], const float (&gf)[U], float (&v)[U]) {
#pragma unroll
                                  for (int k = 0; k < U; ++k) {
                                    const float u = (px[k] - cx) / beta_s, w = (py[k] - cy) / beta_s;
                                    v[k] = shp_tab_value(tab, n1, shp_lerp(u)) * shp_tab_value(tab, n2, shp_lerp(w));
                                  }
                                });
  } else if (ch.kind == 1) {   // shapelet basis function (unit amplitude)
    if (ch.prof != a.gfac_prof) gfp = nullptr;
    const float ib = 1.f / lpget(sx, pr.col[0], 1.f);
    const float cx = lpget(sx, pr.col[1], 0.f), cy = lpget(sx, pr.col[2], 0.f);
    const int n1 = ch.n1, n2 = ch.n2;
    if (gfp)
      lsq_eval_loop<NTH, NPL, U2, true>(I, sbase, bp, gp, gfp, src, per_plane,
                                        [=](const float (&px)[U], const float (&py)[U], const float (&gf)[U],
                                            float (&v)[U]) { shapelet_vals<U, true>(px, py, gf, cx, cy, ib, n1, n2, pref, v); });
    else
      lsq_eval_loop<NTH, NPL, U2, false>(I, sbase, bp, gp, nullptr, src, per_plane,
                                         [=](const float (&px)[U], const float (&py)[U], const float (&gf)[U],
                                             float (&v)[U]) { shapelet_vals<U, false>(px, py, gf, cx, cy, ib, n1, n2, pref, v); });
  } else {              // unit-amplitude Sersic
    const SerC sc = sersic_consts(lpget(sx, pr.col[0], 1.f), lpget(sx, pr.col[1], 1.f),
                                  lpget(sx, pr.col[2], 0.f), lpget(sx, pr.col[3], 0.f),
                                  lpget(sx, pr.col[4], 0.f), lpget(sx, pr.col[5], 0.f), 1.f);
    lsq_eval_loop<NTH, NPL, U2, false>(I, sbase, bp, gp, nullptr, src, per_plane,
                                [=](const float (&px)[U], const float (&py)[U], const float (&gf)[U], float (&v)[U]) {
#pragma unroll
                                  for (int k = 0; k < U; ++k) v[k] = sersic_light(sc, px[k], py[k]);
                                });
  }
}

// Channel evaluation: the basis images of channels c0 .. c0 + CPn - 1 (one
// plane set per slot) on the band's in-image rows Ya .. Ya + per_plane / N - 1
// (shared-memory row 0 is plane row Ybase).  Source channels read the
// ray-traced coordinates beta, lens-light channels the image-plane grid.
template <int NTH>
__device__ __forceinline__ void lsq_eval(const LsqArgs& a, const LsqImage& I, const float* sx,
                                         const float* pref, float* sm, const float2* beta,
                                         const float4* grid, int c0, int Ya, int Ybase, int per_plane) {
  const float4* gp = grid + (size_t)Ya * I.N;
  for (int slot = 0; slot < I.CPn && c0 + slot < a.D; ++slot) {
    const LsqChannel ch = a.ch[c0 + slot];
    float* sbase = sm + (size_t)slot * I.nplanes * I.plane_floats + (Ya - Ybase) * I.pitch;
    const float* gfp = a.gfac_prof >= 0 ? reinterpret_cast<const float*>(beta + (size_t)I.nplanes * per_plane)
                                         : nullptr;
    if (I.nplanes == 4)
      lsq_eval_channel<NTH, 4, 2>(a, I, sx, pref, sbase, beta, gp, gfp, ch, per_plane);
    else
      lsq_eval_channel<NTH, 1, 8>(a, I, sx, pref, sbase, beta, gp, gfp, ch, per_plane);
  }
}

// Column blocks of 20 for sub-kernels up to 15 taps (register budget), 16 otherwise.
#define GL_LSQ_CONV(KSV)                                                     \
  do {                                                                       \
    if constexpr (KSV <= 15) {                                               \
      if (I.CB == 20) {                                                      \
        lsq_pass_conv<KSV, 20, NT>(I, sm, c0, nb, i0, Xb);                   \
        break;                                                               \
      }                                                                      \
    }                                                                        \
    lsq_pass_conv<KSV, 16, NT>(I, sm, c0, nb, i0, Xb);                       \
  } while (0)

// NT = 512 (one CTA per SM, whole-image planes when they fit) or 256 (two
// CTAs per SM on row bands: one CTA's channel evaluation overlaps the other's
// correlation).
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) lsq_basis_kernel(const __grid_constant__ LsqArgs a) {
  extern __shared__ float4 smem_dyn[];
  float* sm = reinterpret_cast<float*>(smem_dyn);
  __shared__ LsqShared st;
  __shared__ float pref[kMaxShapeletN + 1];
  const int tid = threadIdx.x;
  if (tid <= kMaxShapeletN) {
    double f = 1.0;
    for (int i = 2; i <= tid; ++i) f *= i;
    pref[tid] = (float)(1.0 / sqrt(pow(2.0, tid) * sqrt(3.14159265358979323846) * f));
  }
  lsq_term_counts<NT>(a, st);
  float2* beta = a.beta + (size_t)blockIdx.x * a.beta_stride;
  const int total = a.bs * a.max_bands;
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    const int b = item / a.max_bands, band = item - b * a.max_bands;
    const int im = a.img_id ? a.img_id[b] : 0;
    if (im < 0 || im >= a.n_images) continue;
    const LsqImage& I = a.img[im];
    if (band >= I.nbands) continue;
    const int i0 = band * I.Bo;
    const int nb = min(I.Bo, I.N - i0);
    const int Ybase = i0 - I.R0;                        // plane row of shared-memory row 0
    const int Ya = max(0, Ybase), Yb = min(I.N, Ybase + I.brows);
    const int nrows = Yb - Ya;                          // plane rows inside the image
    const int per_plane = nrows * I.N;
    if (tid < a.d) st.x[tid] = a.x[(size_t)b * a.d + tid];
    // zero the planes (halo rows and columns stay zero), load the sub-kernels
    for (int i = tid; i < I.offK / 4; i += NT) smem_dyn[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = tid; i < I.nplanes * I.KS * I.ksp; i += NT) sm[I.offK + i] = __ldg(I.kern + i);
    __syncthreads();
    const int K = st.K[im];
    const int* e = a.epl.col;
    if (tid < 32)
      epl_build_table(st.tab, epl_f_of(lpget(st.x, e[2], 0.f), lpget(st.x, e[3], 0.f)),
                      lpget(st.x, e[1], 2.f) - 1.f, K, tid);
    __syncthreads();
    const float4* grid = reinterpret_cast<const float4*>(I.grid);
    // ray-trace the band's supersampled pixels once: beta[(pq, row, X)]
    {
      const EplC ec = epl_consts(lpget(st.x, e[0], 0.f), lpget(st.x, e[1], 2.f), lpget(st.x, e[2], 0.f),
                                 lpget(st.x, e[3], 0.f), lpget(st.x, e[4], 0.f), lpget(st.x, e[5], 0.f), K);
      const float g1 = a.has_shear ? lpget(st.x, a.shear.col[0], 0.f) : 0.f;
      const float g2 = a.has_shear ? lpget(st.x, a.shear.col[1], 0.f) : 0.f;
      // the Gaussian of the source shapelet profile (its channels' common factor)
      float gib = 0.f, gcx = 0.f, gcy = 0.f;
      if (a.gfac_prof >= 0) {
        const LsqProfile& gp = a.prof[a.gfac_prof];
        gib = 1.f / lpget(st.x, gp.col[0], 1.f);
        gcx = lpget(st.x, gp.col[1], 0.f);
        gcy = lpget(st.x, gp.col[2], 0.f);
      }
      float* gf = reinterpret_cast<float*>(beta + (size_t)I.nplanes * per_plane);
      for (int pq = 0; pq < I.nplanes; ++pq) {
        const float4* gp = grid + ((size_t)pq * I.N + Ya) * I.N;
        float2* bp = beta + (size_t)pq * per_plane;
        for (int i = tid; i < per_plane; i += NT) {
          const float4 xy = __ldg(gp + i);
          float ax, ay;
          epl_deflect(ec, st.tab, xy.x, xy.y, ax, ay);
          float2 bt = make_float2(xy.x - ax, xy.y - ay);
          if (a.has_shear) {
            bt.x = bt.x - (g1 * xy.x + g2 * xy.y);
            bt.y = bt.y - (g2 * xy.x - g1 * xy.y);
          }
          bp[i] = bt;
          if (a.gfac_prof >= 0) {
            const float u = (bt.x - gcx) * gib, w = (bt.y - gcy) * gib;
            gf[(size_t)pq * per_plane + i] = expf(-(u * u + w * w) / 2.f);
          }
        }
      }
    }
    __syncthreads();
    float* Xb = a.X + (size_t)b * a.xstride;
    for (int c0 = 0; c0 < a.D; c0 += I.CPn) {
      lsq_eval<NT>(a, I, st.x, pref, sm, beta, grid, c0, Ya, Ybase, per_plane);
      __syncthreads();
      GL_KS_DISPATCH(I.KS, GL_LSQ_CONV)
      __syncthreads();
    }
  }
}
#undef GL_LSQ_CONV

// pinv(G) h by cyclic Jacobi (round-robin parallel ordering), one CTA of
// kSolveThreads per sample.  A round rotates n/2 disjoint index pairs at once:
// their rotations are computed first, then every 2x2 block of the lower
// triangle (rows of pair P, columns of pair R) takes J_P^T B J_R in one pass
// (the block mirrored above the diagonal), and V takes V J in the same pass.
// A and V live in dynamic shared memory sized for n (row pitch n | 1, odd, so
// column accesses stay conflict-free), so many samples share an SM.
constexpr int kSolveThreads = 128;
size_t solve_smem_bytes(int D) {
  const int n = (D + 1) & ~1, ld = n | 1, np = n / 2;
  return (size_t)(2 * n * ld + n + n) * 4 + (size_t)np * (np + 1) / 2 * 2;
}
__global__ void __launch_bounds__(kSolveThreads) lsq_solve_kernel(int bs, int D, const float* __restrict__ G,
                                                        const float* __restrict__ h, float rcond,
                                                        float* __restrict__ coeffs, int max_sweeps,
                                                        float* __restrict__ Vout, float* __restrict__ ilam,
                                                        const int* __restrict__ status) {
  extern __shared__ float4 solve_dyn[];
  const int n = (D + 1) & ~1;   // even size; a padding index carries a zero row/column
  const int ld = n | 1;
  const int npair = n / 2;
  const int nblk = npair * (npair + 1) / 2;
  float* A = reinterpret_cast<float*>(solve_dyn);
  float* V = A + n * ld;
  float* hs = V + n * ld;
  float* proj = hs + n;
  unsigned char* blk = reinterpret_cast<unsigned char*>(proj + n);   // (k1, k2), k2 <= k1
  __shared__ float cs[kMaxLsqChannels / 2 + 1][2];
  __shared__ int pr[kMaxLsqChannels / 2 + 1][2];
  __shared__ float red[2];
  __shared__ float wred[2][kSolveThreads / 32];
  for (int b = threadIdx.x; b < nblk; b += kSolveThreads) {
    int k1 = 0;
    while ((k1 + 1) * (k1 + 2) / 2 <= b) ++k1;
    blk[2 * b] = (unsigned char)k1;
    blk[2 * b + 1] = (unsigned char)(b - k1 * (k1 + 1) / 2);
  }
  for (int b = blockIdx.x; b < bs; b += gridDim.x) {
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int i = t / n, j = t - i * n;
      A[i * ld + j] = (i < D && j < D) ? G[((size_t)b * D + i) * D + j] : 0.f;
      V[i * ld + j] = (i == j) ? 1.f : 0.f;
    }
    for (int t = threadIdx.x; t < n; t += blockDim.x) hs[t] = (t < D) ? h[(size_t)b * D + t] : 0.f;
    __syncthreads();
    float prev_off = INFINITY;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
      // convergence test: off-diagonal vs diagonal Frobenius norm (block reduction)
      {
        float off = 0.f, dg = 0.f;
        for (int t = threadIdx.x; t < n * n; t += kSolveThreads) {
          const int i = t / n, j = t - i * n;
          const float v = A[i * ld + j] * A[i * ld + j];
          if (i == j) dg += v;
          else off += v;
        }
        for (int o = 16; o > 0; o >>= 1) {
          off += __shfl_xor_sync(0xffffffffu, off, o);
          dg += __shfl_xor_sync(0xffffffffu, dg, o);
        }
        if ((threadIdx.x & 31) == 0) {
          wred[0][threadIdx.x >> 5] = off;
          wred[1][threadIdx.x >> 5] = dg;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          float o = 0.f, g = 0.f;
          for (int w = 0; w < kSolveThreads / 32; ++w) {
            o += wred[0][w];
            g += wred[1][w];
          }
          red[0] = o;
          red[1] = g;
        }
        __syncthreads();
      }
      // Converged when the off-diagonal part is below 1e-11 of the diagonal
      // (|off|_F < 3.2e-6 |diag|_F), or once a sweep near the float32 floor
      // (< 1e-8) no longer halves it: rounding alone leaves off-diagonal
      // entries of order eps |lambda|, whose sum over D^2 entries can stay
      // near 1e-12 for good.  NaN stops at once.
      const float off_now = red[0], dg_now = red[1];
      const bool done = !(off_now > 1e-11f * dg_now) ||
                        (off_now < 1e-8f * dg_now && off_now > 0.5f * prev_off);
      prev_off = off_now;
      __syncthreads();
      if (done) break;
      for (int round = 0; round < n - 1; ++round) {
        // tournament pairing: index 0 fixed, the others rotate
        for (int k = threadIdx.x; k < npair; k += kSolveThreads) {
          auto at = [&](int pos) {
            if (pos == 0) return 0;
            int v = pos - 1 + round;   // < 2 (n - 1)
            if (v >= n - 1) v -= n - 1;
            return 1 + v;
          };
          int p = at(k), q = at(n - 1 - k);
          if (p > q) {
            const int t = p;
            p = q;
            q = t;
          }
          const float apq = A[p * ld + q];
          float c = 1.f, s = 0.f;
          if (fabsf(apq) > 1e-30f) {
            const float theta = (A[q * ld + q] - A[p * ld + p]) / (2.f * apq);
            const float t = copysignf(1.f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.f));
            c = rsqrtf(t * t + 1.f);
            s = t * c;
          }
          cs[k][0] = c;
          cs[k][1] = s;
          pr[k][0] = p;
          pr[k][1] = q;
        }
        __syncthreads();
        // A <- J^T A J block by block (lower triangle, mirrored); V <- V J
        for (int t = threadIdx.x; t < nblk + n * npair; t += kSolveThreads) {
          if (t < nblk) {
            const int k1 = blk[2 * t], k2 = blk[2 * t + 1];
            const int p = pr[k1][0], q = pr[k1][1], r = pr[k2][0], u = pr[k2][1];
            const float cP = cs[k1][0], sP = cs[k1][1], cR = cs[k2][0], sR = cs[k2][1];
            const float b00 = A[p * ld + r], b01 = A[p * ld + u], b10 = A[q * ld + r], b11 = A[q * ld + u];
            const float t00 = cP * b00 - sP * b10, t01 = cP * b01 - sP * b11;
            const float t10 = sP * b00 + cP * b10, t11 = sP * b01 + cP * b11;
            const float n00 = cR * t00 - sR * t01, n01 = sR * t00 + cR * t01;
            const float n10 = cR * t10 - sR * t11, n11 = sR * t10 + cR * t11;
            A[p * ld + r] = n00;
            A[p * ld + u] = n01;
            A[q * ld + r] = n10;
            A[q * ld + u] = n11;
            if (k1 != k2) {
              A[r * ld + p] = n00;
              A[u * ld + p] = n01;
              A[r * ld + q] = n10;
              A[u * ld + q] = n11;
            }
          } else {
            const int e = t - nblk;
            const int k = e / n, i = e - k * n;
            const int p = pr[k][0], q = pr[k][1];
            const float c = cs[k][0], s = cs[k][1];
            const float vp = V[i * ld + p], vq = V[i * ld + q];
            V[i * ld + p] = c * vp - s * vq;
            V[i * ld + q] = s * vp + c * vq;
          }
        }
        __syncthreads();
      }
    }
    // pinv solve: coeffs = sum over kept eigenpairs of (v_i . h / lambda_i) v_i
    if (threadIdx.x == 0) {
      float m = 0.f;
      for (int i = 0; i < D; ++i) m = fmaxf(m, fabsf(A[i * ld + i]));
      red[0] = rcond * m;
    }
    __syncthreads();
    const float cutoff = red[0];
    // proj_i = (v_i . h) / lambda_i
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      float s = 0.f;
      for (int r = 0; r < n; ++r) s = fmaf(V[r * ld + i], hs[r], s);
      const float lam = A[i * ld + i];
      proj[i] = (i < D && fabsf(lam) > cutoff) ? s / lam : 0.f;
    }
    __syncthreads();
    // the pinv operator, kept for the refinement: V and the kept inverse eigenvalues
    const bool bad = status && *status;
    for (int t = threadIdx.x; t < D * D; t += blockDim.x) {
      const int r = t / D, i = t - r * D;
      Vout[(size_t)b * D * D + t] = V[r * ld + i];
    }
    for (int i = threadIdx.x; i < D; i += blockDim.x) {
      const float lam = A[i * ld + i];
      ilam[(size_t)b * D + i] = fabsf(lam) > cutoff ? 1.f / lam : 0.f;
    }
    for (int r = threadIdx.x; r < D; r += blockDim.x) {
      float s = 0.f;
      for (int i = 0; i < n; ++i) s = fmaf(V[r * ld + i], proj[i], s);
      coeffs[(size_t)b * D + r] = bad ? __int_as_float(0x7fc00000) : s;
    }
    __syncthreads();
  }
}

// Passes over the basis stack X after the normal equations, streamed from HBM
// through a shared-memory ring (cp.async, kXRing chunks of kXT pixels x D
// channels; one block per sample, persistent over the batch, the copies of
// the next chunks crossing into the next sample).  Per chunk:
//
//  RESID  projected residual of the weighted least-squares problem from the
//         basis itself (not from G): (1) thread t forms
//         e_p = W_p^2 (y_p - sum_c X_cp c_c) of pixel p = chunk + t, the
//         channel sum in float32 groups of 8 combined in float-float
//         (TwoSum); (2) warp w projects the chunk onto channels w, w + 8, ...:
//         r_c += sum_p X_cp e_p, lanes over pixels, float32 over a lane's 8
//         pixels and float-float across chunks, float64 only in the final
//         reduction over lanes.
//  IMAGE  img = sum_c coeffs_c X_c (no conversion factor, as the reference),
//         the Gaussian log-likelihood with the data error map and chi^2
//         (BackwardProbModel, tf/model.py:157-163).
constexpr int kXT = 256;      // threads = pixels per chunk
constexpr int kXRing = 2;     // chunks in the ring (two blocks per SM: their chunk barriers interleave)
constexpr int kXChPerWarp = (kMaxLsqChannels + (kXT / 32) - 1) / (kXT / 32);

size_t xpass_smem_bytes(int D) { return (size_t)kXRing * D * kXT * 4; }

template <bool IMAGE>
__global__ void __launch_bounds__(kXT, 2) lsq_xpass_kernel(const __grid_constant__ LsqArgs a,
                                                          const float* __restrict__ coeffs,
                                                          float* __restrict__ r_out, float* img_out,
                                                          float* logL, float* chi2) {
  extern __shared__ float4 xring4[];
  float* ring = reinterpret_cast<float*>(xring4);
  __shared__ float cf[kMaxLsqChannels];
  __shared__ float e_s[kXT];
  __shared__ float red[2][kXT / 32];
  const int D = a.D;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int items = D * (kXT / 4);   // 16-byte pieces of a chunk

  auto valid_sample = [&](int b) {
    const int im = a.img_id ? a.img_id[b] : 0;
    return im >= 0 && im < a.n_images;
  };
  auto next_sample = [&](int b) {
    for (b += gridDim.x; b < a.bs && !valid_sample(b); b += gridDim.x) {
    }
    return b;
  };
  int first = blockIdx.x;
  while (first < a.bs && !valid_sample(first)) first += gridDim.x;
  int pb = first, pch = 0;
  auto issue = [&](int slot) {
    if (pb < a.bs) {
      const LsqImage& I = a.img[a.img_id ? a.img_id[pb] : 0];
      const int P = I.N * I.N;
      const float* Xb = a.X + (size_t)pb * a.xstride;
      const int p0 = pch * kXT;
      float* dst = ring + (size_t)slot * D * kXT;
      for (int it = tid; it < items; it += kXT) {
        const int r = it / (kXT / 4), q = it - r * (kXT / 4);
        const int p = p0 + 4 * q;
        const float* row = Xb + (size_t)r * I.xcstride;
        const int left = P - p;
        const uint32_t bytes = left >= 4 ? 16u : (left > 0 ? 4u * left : 0u);
        cp_async16(dst + r * kXT + 4 * q, bytes ? row + p : row, bytes);
      }
      if (++pch == (P + kXT - 1) / kXT) {
        pb = next_sample(pb);
        pch = 0;
      }
    }
    cp_async_commit();
  };
  for (int s = 0; s < kXRing - 1; ++s) issue(s);

  uint32_t gchunk = 0;
  for (int b = first; b < a.bs; b = next_sample(b)) {
    const LsqImage& I = a.img[a.img_id ? a.img_id[b] : 0];
    const int P = I.N * I.N;
    const int nchunks = (P + kXT - 1) / kXT;
    for (int c = tid; c < D; c += kXT) cf[c] = coeffs[(size_t)b * D + c];
    float acc_h[kXChPerWarp], acc_l[kXChPerWarp];
#pragma unroll
    for (int k = 0; k < kXChPerWarp; ++k) acc_h[k] = acc_l[k] = 0.f;
    float ls = 0.f, cs2 = 0.f;
    for (int ch = 0; ch < nchunks; ++ch, ++gchunk) {
      issue((gchunk + kXRing - 1) % kXRing);
      cp_async_wait<kXRing - 1>();
      __syncthreads();   // every thread's pieces of this chunk (and cf) are visible
      const float* xs = ring + (size_t)(gchunk % kXRing) * D * kXT;
      const int p = ch * kXT + tid;
      if (IMAGE) {
        float v = 0.f;
        for (int c = 0; c < D; ++c) v = fmaf(xs[c * kXT + tid], cf[c], v);
        if (p < P) {
          if (img_out) img_out[(size_t)b * a.maxP + p] = v;
          if (I.obs) {
            const float err = __ldg(I.err + p);
            const float zz = (v - __ldg(I.obs + p)) / err;
            ls += -0.5f * zz * zz - logf(err) - kHalfLog2Pi;
            cs2 += zz * zz;
          }
        }
      } else {
        float mh = 0.f, ml = 0.f;
        if (coeffs) {
          for (int c0 = 0; c0 < D; c0 += 8) {
            float g = 0.f;
            const int c1 = min(D, c0 + 8);
            for (int c = c0; c < c1; ++c) g = fmaf(xs[c * kXT + tid], cf[c], g);
            ff_add(mh, ml, g);
          }
        }
        float e = 0.f;
        if (p < P) {
          const float w = __ldg(I.W + p);
          e = ((__ldg(I.obs + p) - mh) - ml) * (w * w);
        }
        e_s[tid] = e;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kXChPerWarp; ++k) {
          const int c = warp + k * (kXT / 32);
          if (c < D) {
            const float* xc = xs + c * kXT;
            float g = 0.f;
#pragma unroll
            for (int j = 0; j < kXT / 32; ++j) g = fmaf(xc[lane + 32 * j], e_s[lane + 32 * j], g);
            ff_add(acc_h[k], acc_l[k], g);
          }
        }
      }
      __syncthreads();   // the ring slot and e_s are reused next
    }
    if (IMAGE) {
      for (int o = 16; o > 0; o >>= 1) {
        ls += __shfl_xor_sync(0xffffffffu, ls, o);
        cs2 += __shfl_xor_sync(0xffffffffu, cs2, o);
      }
      if (lane == 0) {
        red[0][warp] = ls;
        red[1][warp] = cs2;
      }
      __syncthreads();
      if (tid == 0) {
        float l = 0.f, c = 0.f;
        for (int w = 0; w < kXT / 32; ++w) {
          l += red[0][w];
          c += red[1][w];
        }
        if (logL) logL[b] = l;
        if (chi2) chi2[b] = c / (float)P;
      }
      __syncthreads();
    } else {
#pragma unroll
      for (int k = 0; k < kXChPerWarp; ++k) {
        const int c = warp + k * (kXT / 32);
        double v = (double)acc_h[k] + (double)acc_l[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && c < D) r_out[(size_t)b * D + c] = (float)v;
      }
    }
  }
  cp_async_wait<0>();
}

// Refinement step: c += V diag(ilam) V^T r (the pinv of G applied to the residual).
__global__ void __launch_bounds__(64) lsq_update_kernel(int bs, int D, const float* __restrict__ V,
                                                       const float* __restrict__ ilam,
                                                       const float* __restrict__ r,
                                                       float* __restrict__ coeffs) {
  __shared__ float proj[kMaxLsqChannels];
  for (int b = blockIdx.x; b < bs; b += gridDim.x) {
    const float* Vb = V + (size_t)b * D * D;
    for (int i = threadIdx.x; i < D; i += blockDim.x) {
      float s = 0.f;
      for (int k = 0; k < D; ++k) s = fmaf(Vb[k * D + i], r[(size_t)b * D + k], s);
      proj[i] = s * ilam[(size_t)b * D + i];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < D; k += blockDim.x) {
      float s = 0.f;
      for (int i = 0; i < D; ++i) s = fmaf(Vb[k * D + i], proj[i], s);
      coeffs[(size_t)b * D + k] += s;
    }
    __syncthreads();
  }
}

// W = 1 / err and b = W * obs per image, zero beyond the N^2 pixels.
__global__ void lsq_weights_kernel(const float* __restrict__ err, const float* __restrict__ obs, int P,
                                   int padded, float* __restrict__ W, float* __restrict__ bw) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < padded; p += gridDim.x * blockDim.x) {
    const float w = p < P ? 1.f / err[p] : 0.f;
    W[p] = w;
    bw[p] = p < P && obs ? obs[p] * w : 0.f;
  }
}
// ------------------------------------------------------------------ host side
static int g_lsq_smem_set[kMaxDevices][2];   // basis kernel smem attribute set per device and variant

// Shared-memory layout and launch shape of the basis kernel for one tuning:
// ctas_per_sm = 1 (512 threads, up to the whole opt-in shared memory of a
// CTA) or 2 (256 threads, half the SM's shared memory each); col_block = 16
// or 20 columns per correlation unit, 0 for the planner's choice.
int lsq_plan_layout(LsqPlan* L, const gl_plan* plan, int ctas_per_sm, int col_block) {
  if (ctas_per_sm != 1 && ctas_per_sm != 2) {
    set_error("least squares: %d basis CTAs per SM (1 or 2)", ctas_per_sm);
    return GL_ERR_INVALID;
  }
  if (col_block != 0 && col_block != 16 && col_block != 20) {
    set_error("least squares: column block %d (16 or 20)", col_block);
    return GL_ERR_INVALID;
  }
  const int D = L->D;
  const int nt = ctas_per_sm == 1 ? 512 : 256;
  int dev_smem = 0, sm_smem = 0;
  cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, plan->device);
  cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, plan->device);
  const int static_bytes = 8 * 1024;
  // per CTA: 1 KB of every CTA's shared memory is reserved by the system
  const int cta_smem = ctas_per_sm == 1 ? dev_smem : std::min(dev_smem, sm_smem / 2 - 1024);
  int maxP = 0, maxXc = 0, smem = 0, max_bands = 0;
  size_t beta_per_cta = 0;
  LsqImage img[GL_MAX_IMAGES];
  for (int i = 0; i < plan->n_images; ++i) {
    const DevImage& F = plan->img[i];
    LsqImage I = L->img[i];
    I.N = F.N;
    I.ss = F.ss;
    I.nplanes = F.nplanes;
    I.KS = F.KS;
    I.ksp = F.ksp;
    for (int k = 0; k < kMaxPlanes; ++k) {
      I.d[k] = F.d[k];
      I.padI[k] = F.padI[k];
    }
    I.pitch = 0;
    I.xcstride = (F.N * F.N + 3) & ~3;   // 16-byte aligned channel rows (cp.async)
    I.cpass = D;
    int dmin = F.d[0], dmax = F.d[0];
    for (int p = 1; p < F.ss; ++p) {
      dmin = std::min(dmin, F.d[p]);
      dmax = std::max(dmax, F.d[p]);
    }
    I.R0 = dmax;
    // Layout: per channel slot, ss^2 parity planes of brows rows x pitch
    // floats (image rows with a top/bottom halo of the sub-kernel, columns
    // with a zero right halo), then the sub-kernels.  Prefer the whole image
    // in one band with as many channels per pass as fit; among column blocks
    // of 16 and 20 pick the one that keeps the most of the threads busy.
    const int kern_floats = F.nplanes * F.KS * F.ksp;
    const int avail = cta_smem - static_bytes - kern_floats * 4;
    double best_score = -1.0;
    for (int cb : {20, 16}) {
      if (cb == 20 && F.KS > 15) continue;
      if (col_block && cb != col_block) continue;
      const int ncbC = (F.N + cb - 1) / cb;
      const int segn = (cb + F.KS - 1 + 3) & ~3;
      int pitch = std::max(F.N + F.KS - 1, (ncbC - 1) * cb + segn);
      pitch = (pitch + 3) & ~3;
      if ((pitch / 4) % 2 == 0) pitch += 4;
      // band height: the whole image when one channel's planes fit
      int bo = F.N;
      while (bo >= 1 && F.nplanes * (bo + F.KS + dmax - dmin) * pitch * 4 > avail) --bo;
      if (bo < 1) continue;
      const int brows = bo + F.KS + dmax - dmin;
      const int set_bytes = F.nplanes * brows * pitch * 4;
      const int cp_max = std::max(1, std::min(std::min(avail / set_bytes, D), 4));
      for (int cp = 1; cp <= cp_max; ++cp) {
        const int units = cp * ncbC * bo;
        const int rounds = (units + nt - 1) / nt;
        const double util = (double)cp * bo * F.N / ((double)rounds * nt * cb);
        const double halo = (double)bo / std::min(brows, F.N);   // rows evaluated per output row
        const double score = util * std::min(1.0, halo) * (1.0 + 0.02 * cp);
        if (score > best_score) {
          best_score = score;
          I.CB = cb;
          I.ncbC = ncbC;
          I.pitch = pitch;
          I.Bo = bo;
          I.brows = brows;
          I.CPn = cp;
        }
      }
    }
    if (best_score < 0) {
      set_error("least squares: image %d does not fit in shared memory", i);
      return GL_ERR_UNSUPPORTED;
    }
    I.nbands = (F.N + I.Bo - 1) / I.Bo;
    I.plane_floats = I.brows * I.pitch;
    I.offK = I.CPn * F.nplanes * I.plane_floats;
    I.smem_floats = I.offK + kern_floats;
    // the per-pixel loops divide indices below 2^21 through float reciprocals
    if ((long long)F.nplanes * std::min(I.brows, F.N) * F.N >= (1 << 21)) {
      set_error("least squares: image %d too large (%d px)", i, F.N);
      return GL_ERR_UNSUPPORTED;
    }
    size_t beta_n = (size_t)F.nplanes * std::min(I.brows, F.N) * F.N;
    if (L->gfac_prof >= 0) beta_n += (beta_n + 1) / 2;   // and the Gaussian factors (floats)
    if (beta_n > beta_per_cta) beta_per_cta = beta_n;
    if (I.smem_floats * 4 > smem) smem = I.smem_floats * 4;
    if (F.N * F.N > maxP) maxP = F.N * F.N;
    if (I.xcstride > maxXc) maxXc = I.xcstride;
    if (I.nbands > max_bands) max_bands = I.nbands;
    img[i] = I;
  }
  const int dev_slot = current_device_slot();
  int* set = ctas_per_sm == 1 ? g_lsq_smem_set[dev_slot] + 0 : g_lsq_smem_set[dev_slot] + 1;
  if (smem > *set) {
    cudaError_t e = ctas_per_sm == 1
                        ? cudaFuncSetAttribute(lsq_basis_kernel<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
                        : cudaFuncSetAttribute(lsq_basis_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) {
      set_error("lsq smem attribute: %s", cudaGetErrorString(e));
      return GL_ERR_CUDA;
    }
    *set = smem;
  }
  for (int i = 0; i < plan->n_images; ++i) L->img[i] = img[i];
  L->smem_bytes = smem;
  L->maxP = maxP;
  L->maxXc = maxXc;
  L->max_bands = max_bands;
  L->beta_per_cta = beta_per_cta;
  L->nt = nt;
  L->ctas_per_sm = ctas_per_sm;
  L->col_block = col_block;
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, plan->device);
  L->n_sm = ctas_per_sm * sms;
  return GL_OK;
}

int lsq_prepare(gl_plan* plan, std::vector<std::vector<float>>& errs) {
  LsqPlan* L = new LsqPlan;
  memset(L, 0, sizeof(*L));
  L->gram = 2;
  const gl_model_desc& m = plan->model;
  int D = 0;
  for (int i = 0; i < m.n_profiles; ++i) {
    const gl_profile_desc& p = m.prof[i];
    if (p.group == GL_GROUP_LENS) {
      if (p.type == GL_PROF_EPL) {
        L->epl.type = p.type;
        L->epl.niter = p.niter;
        for (int k = 0; k < GL_MAX_PROFILE_PARAMS; ++k) L->epl.col[k] = p.col[k];
      } else if (p.type == GL_PROF_SHEAR) {
        L->has_shear = 1;
        for (int k = 0; k < GL_MAX_PROFILE_PARAMS; ++k) L->shear.col[k] = p.col[k];
      }
      continue;
    }
    if (L->n_prof >= kMaxLsqProfiles) {
      set_error("least squares: at most %d light profiles", kMaxLsqProfiles);
      delete L;
      return GL_ERR_UNSUPPORTED;
    }
    LsqProfile& pr = L->prof[L->n_prof];
    pr.group = p.group;
    pr.type = p.type;
    pr.interp = p.type == GL_PROF_SHAPELETS && p.interpolate ? 1 : 0;
    for (int k = 0; k < GL_MAX_PROFILE_PARAMS; ++k) pr.col[k] = -1;
    if (p.type == GL_PROF_SHAPELETS) {
      if (p.niter < 0 || p.niter > kMaxShapeletN) {
        set_error("shapelets n_max %d outside [0, %d]", p.niter, kMaxShapeletN);
        delete L;
        return GL_ERR_UNSUPPORTED;
      }
      for (int k = 0; k < 3; ++k) pr.col[k] = p.col[k];
      int n1 = 0, n2 = 0;
      const int nl = (p.niter + 1) * (p.niter + 2) / 2;
      for (int k = 0; k < nl; ++k) {
        if (D >= kMaxLsqChannels) {
          set_error("least squares: more than %d basis channels", kMaxLsqChannels);
          delete L;
          return GL_ERR_UNSUPPORTED;
        }
        L->ch[D].kind = 1;
        L->ch[D].prof = L->n_prof;
        L->ch[D].n1 = n1;
        L->ch[D].n2 = n2;
        ++D;
        if (n1 == 0) {
          n1 = n2 + 1;
          n2 = 0;
        } else {
          --n1;
          ++n2;
        }
      }
    } else if (p.type == GL_PROF_SERSIC_ELLIPSE || p.type == GL_PROF_SERSIC) {
      if (p.type == GL_PROF_SERSIC_ELLIPSE) {
        for (int k = 0; k < 6; ++k) pr.col[k] = p.col[k];
      } else {
        pr.col[0] = p.col[0];
        pr.col[1] = p.col[1];
        pr.col[4] = p.col[2];
        pr.col[5] = p.col[3];
      }
      if (D >= kMaxLsqChannels) {
        set_error("least squares: more than %d basis channels", kMaxLsqChannels);
        delete L;
        return GL_ERR_UNSUPPORTED;
      }
      L->ch[D].kind = 0;
      L->ch[D].prof = L->n_prof;
      ++D;
    } else {
      set_error("least squares: light type %d not supported", p.type);
      delete L;
      return GL_ERR_UNSUPPORTED;
    }
    if (!p.use_lstsq) {
      set_error("least squares needs every light profile with use_lstsq");
      delete L;
      return GL_ERR_UNSUPPORTED;
    }
    ++L->n_prof;
  }
  if (L->epl.type != GL_PROF_EPL || D < 1 || D > kMaxLsqChannels) {
    set_error("least squares needs an EPL lens and 1..%d basis channels (got %d)", kMaxLsqChannels, D);
    delete L;
    return GL_ERR_UNSUPPORTED;
  }
  L->D = D;
  // the first source shapelet profile (Hermite functions): its Gaussian is
  // computed once per pixel and sample in the ray-trace pass
  L->gfac_prof = -1;
  for (int i = 0; i < L->n_prof && L->gfac_prof < 0; ++i)
    if (L->prof[i].type == GL_PROF_SHAPELETS && !L->prof[i].interp && L->prof[i].group == GL_GROUP_SOURCE)
      L->gfac_prof = i;
  for (int i = 0; i < plan->n_images; ++i) {
    const DevImage& F = plan->img[i];
    LsqImage& I = L->img[i];
    I.grid = F.grid;
    I.kern = F.kern;
    I.obs = F.obs;
  }
  {
    int rc = lsq_plan_layout(L, plan, 1, 0);
    if (rc) {
      delete L;
      return rc;
    }
  }
  // error maps, W = 1/err and b = W * obs on the device (W and b zero-padded
  // to whole streaming chunks)
  auto up256 = [](size_t v) { return (v + 255) / 256 * 256; };
  auto padded = [](size_t P) { return (P + kPixPad - 1) / kPixPad * kPixPad; };
  size_t bytes = 0;
  for (int i = 0; i < plan->n_images; ++i)
    bytes += up256(errs[i].size() * 4) + 2 * up256(padded(errs[i].size()) * 4);
  if (cudaMalloc((void**)&L->dev_err, bytes) != cudaSuccess) {
    set_error("cudaMalloc(error maps) failed");
    delete L;
    return GL_ERR_NOMEM;
  }
  char* base = (char*)L->dev_err;
  for (int i = 0; i < plan->n_images; ++i) {
    const size_t P = errs[i].size(), Pp = padded(P);
    cudaMemcpy(base, errs[i].data(), P * 4, cudaMemcpyHostToDevice);
    LsqImage& I = L->img[i];
    I.err = (const float*)base;
    base += up256(P * 4);
    float* W = (float*)base;
    base += up256(Pp * 4);
    float* bw = (float*)base;
    base += up256(Pp * 4);
    lsq_weights_kernel<<<(int)((Pp + 255) / 256), 256>>>(I.err, I.obs, (int)P, (int)Pp, W, bw);
    I.W = W;
    I.bw = bw;
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    set_error("least squares weights: %s", cudaGetErrorString(cudaGetLastError()));
    cudaFree(L->dev_err);
    delete L;
    return GL_ERR_CUDA;
  }
  if (cudaFuncSetAttribute(lsq_xpass_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)xpass_smem_bytes(D)) != cudaSuccess ||
      cudaFuncSetAttribute(lsq_xpass_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)xpass_smem_bytes(D)) != cudaSuccess) {
    set_error("least squares pass kernels: shared memory attribute: %s", cudaGetErrorString(cudaGetLastError()));
    cudaFree(L->dev_err);
    delete L;
    return GL_ERR_CUDA;
  }
  plan->lsq = L;
  return GL_OK;
}

void lsq_destroy(gl_plan* plan) {
  if (!plan->lsq) return;
  LsqPlan* L = (LsqPlan*)plan->lsq;
  if (L->dev_err) cudaFree(L->dev_err);
  delete L;
  plan->lsq = nullptr;
}

// CTAs of the basis kernel: one per work item, at most one per SM.
static int basis_ctas(const LsqPlan* L, int bs) {
  const long long items = (long long)bs * L->max_bands;
  return (int)std::max(1LL, std::min(items, (long long)L->n_sm));
}

// Workspace: X [bs][D][maxXc], G [bs][D][D], V [bs][D][D], h, r, ilam [bs][D],
// beta [basis CTAs][beta_per_cta] (float2), status.
size_t lsq_status_offset(const LsqPlan* L, int bs) {
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  const size_t X = (size_t)bs * L->D * L->maxXc * 4;
  const size_t G = (size_t)bs * L->D * L->D * 4;
  const size_t h = (size_t)bs * L->D * 4;
  const size_t beta = (size_t)basis_ctas(L, bs) * L->beta_per_cta * 8;
  return up(X) + 2 * up(G) + 3 * up(h) + up(beta);
}

size_t lsq_workspace_bytes(const LsqPlan* L, int bs) { return lsq_status_offset(L, bs) + 256; }

int lsq_run(const gl_plan* plan, const float* x, const int* img_id, int bs, float* work,
            size_t work_bytes, float* coeffs, float* img_out, float* logL, float* chi2,
            cudaStream_t stream) {
  const LsqPlan* L = (const LsqPlan*)plan->lsq;
  if (work_bytes < lsq_workspace_bytes(L, bs)) {
    set_error("least squares workspace too small: %zu < %zu bytes", work_bytes, lsq_workspace_bytes(L, bs));
    return GL_ERR_INVALID;
  }
  if (bs == 0) return GL_OK;
  LsqArgs a;
  memset(&a, 0, sizeof(a));
  a.bs = bs;
  a.d = plan->model.n_params;
  a.D = L->D;
  a.n_images = plan->n_images;
  a.n_prof = L->n_prof;
  for (int i = 0; i < kMaxLsqProfiles; ++i) a.prof[i] = L->prof[i];
  for (int i = 0; i < kMaxLsqChannels; ++i) a.ch[i] = L->ch[i];
  a.epl = L->epl;
  a.shear = L->shear;
  a.shp_tab = plan->shp_tab;
  a.has_shear = L->has_shear;
  a.gfac_prof = L->gfac_prof;
  for (int i = 0; i < plan->n_images; ++i) a.img[i] = L->img[i];
  a.x = x;
  a.img_id = img_id;
  a.maxP = L->maxP;
  a.max_bands = L->max_bands;
  a.xstride = (size_t)L->D * L->maxXc;
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  char* base = (char*)work;
  a.X = (float*)base;
  base += up((size_t)bs * L->D * L->maxXc * 4);
  float* G = (float*)base;
  base += up((size_t)bs * L->D * L->D * 4);
  float* V = (float*)base;
  base += up((size_t)bs * L->D * L->D * 4);
  float* h = (float*)base;
  base += up((size_t)bs * L->D * 4);
  float* r = (float*)base;
  base += up((size_t)bs * L->D * 4);
  float* ilam = (float*)base;
  base += up((size_t)bs * L->D * 4);
  const int n_basis = basis_ctas(L, bs);
  a.beta = (float2*)base;
  a.beta_stride = L->beta_per_cta;
  base += up((size_t)n_basis * L->beta_per_cta * 8);
  int* status = (int*)base;
  if ((size_t)((char*)status - (char*)work) != lsq_status_offset(L, bs)) {
    set_error("least squares: workspace layout mismatch");
    return GL_ERR_INTERNAL;
  }
  float* co = coeffs;
  if (!co) {
    set_error("least squares: coeffs buffer required");
    return GL_ERR_INVALID;
  }
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, plan->device);
  cudaMemsetAsync(status, 0, sizeof(int), stream);
  // basis stack, then G = A^T A and h = A^T b (FP32 register tiles, or the
  // tensor cores in 3xTF32)
  if (L->nt == 512)
    lsq_basis_kernel<512><<<n_basis, 512, L->smem_bytes, stream>>>(a);
  else
    lsq_basis_kernel<256><<<n_basis, 256, L->smem_bytes, stream>>>(a);
  int rc;
  if (L->gram == 1)
    rc = launch_gram_tc(a, G, h, status, std::min(bs, gram_tc_ctas_per_sm(L->D) * sms), stream);
  else
    rc = launch_gram_fp32(a, G, h, std::min(bs, sms), stream);
  if (rc) return rc;
  // c0 = pinv(G) h, then two refinement steps against the residual of the
  // least-squares problem itself
  const int xpass_blocks = std::min(bs, 2 * sms);
  const size_t xsm = xpass_smem_bytes(L->D);
  lsq_solve_kernel<<<bs < 12 * sms ? bs : 12 * sms, kSolveThreads, solve_smem_bytes(L->D), stream>>>(
      bs, L->D, G, h, 1e-6f, co, 30, V, ilam, status);
  for (int it = 0; it < 2; ++it) {
    lsq_xpass_kernel<false><<<xpass_blocks, kXT, xsm, stream>>>(a, co, r, nullptr, nullptr, nullptr);
    lsq_update_kernel<<<bs < 8 * sms ? bs : 8 * sms, 64, 0, stream>>>(bs, L->D, V, ilam, r, co);
  }
  if (img_out || logL || chi2)
    lsq_xpass_kernel<true><<<xpass_blocks, kXT, xsm, stream>>>(a, co, nullptr, img_out, logL, chi2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("least squares launch: %s", cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}

// ------------------------------------------------------------------ allocation-free variant
// Fixed scratch for gl_lstsq_noalloc: a file-scope device array that every GPU
// loading this library holds until the process exits.  Its host-side name is
// only a stand-in for the symbol; the device address comes from
// cudaGetSymbolAddress, looked up once per device with that device current.
constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;   // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
static void* g_noalloc_addr[kNoAllocMaxDevices];
static std::mutex g_noalloc_mutex;

static int noalloc_scratch_address(int device, void** out) {
  if (device < 0 || device >= kNoAllocMaxDevices) {
    set_error("gl_lstsq_noalloc: device %d out of range", device);
    return GL_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error("gl_lstsq_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return GL_ERR_CUDA;
    }
    g_noalloc_addr[device] = p;
  }
  *out = g_noalloc_addr[device];
  return GL_OK;
}

}  // namespace gl

extern "C" int gl_lstsq_status(const gl_plan* plan, int bs, const void* work, int* status,
                               void* stream) {
  using namespace gl;
  if (!plan || !plan->lsq || bs < 0 || !status) {
    set_error("gl_lstsq_status: null plan or status, negative batch, or no least-squares profiles");
    return GL_ERR_INVALID;
  }
  const char* base = (const char*)work;
  if (!base) {
    int dev = -1;
    cudaGetDevice(&dev);
    void* p = nullptr;
    int rc = noalloc_scratch_address(dev, &p);
    if (rc) return rc;
    base = (const char*)p;
  }
  const size_t off = lsq_status_offset((const LsqPlan*)plan->lsq, bs);
  cudaError_t e = cudaMemcpyAsync(status, base + off, sizeof(int), cudaMemcpyDefault, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    set_error("gl_lstsq_status: %s", cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}

extern "C" int gl_test_set_wait_polls(int polls) {
  gl::set_gram_wait_polls(polls);
  return GL_OK;
}

extern "C" int gl_lstsq_noalloc(const gl_plan* plan, const float* x, const int* img_id, int bs,
                                float* coeffs, float* img_out, float* logL, float* chi2,
                                void* stream) {
  using namespace gl;
  if (!plan || bs < 0 || (bs > 0 && (!x || !coeffs))) {
    set_error("gl_lstsq_noalloc: null plan, input or coeffs, or negative batch");
    return GL_ERR_INVALID;
  }
  if (!plan->lsq) {
    set_error("the plan has no linear-amplitude light profiles");
    return GL_ERR_INVALID;
  }
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != plan->device) {
    set_error("plan was created on device %d but device %d is current", plan->device, dev);
    return GL_ERR_INVALID;
  }
  if (logL || chi2)
    for (int i = 0; i < plan->n_images; ++i)
      if (!plan->img[i].obs) {
        set_error("image %d has no observed data", i);
        return GL_ERR_INVALID;
      }
  const LsqPlan* L = (const LsqPlan*)plan->lsq;
  const size_t need = lsq_workspace_bytes(L, bs);
  if (need > kNoAllocScratchBytes) {
    // the workspace grows with the batch: bisect for the largest batch that fits
    int lo = 0, hi = bs;
    while (hi - lo > 1) {
      const int mid = lo + (hi - lo) / 2;
      if (lsq_workspace_bytes(L, mid) <= kNoAllocScratchBytes) lo = mid;
      else hi = mid;
    }
    set_error("gl_lstsq_noalloc: %d chains need %zu bytes of scratch, more than its fixed %zu bytes "
              "(at most %d chains for this plan); split the batch or use gl_lstsq",
              bs, need, kNoAllocScratchBytes, lo);
    return GL_ERR_INVALID;
  }
  void* scratch = nullptr;
  int rc = noalloc_scratch_address(dev, &scratch);
  if (rc) return rc;
  return lsq_run(plan, x, img_id, bs, (float*)scratch, kNoAllocScratchBytes, coeffs, img_out, logL,
                 chi2, (cudaStream_t)stream);
}


extern "C" int gl_plan_set_tuning(gl_plan* plan, const gl_tuning* t) {
  using namespace gl;
  if (!plan || !t) {
    set_error("gl_plan_set_tuning: null plan or tuning");
    return GL_ERR_INVALID;
  }
  if (t->fused_corr < 0 || t->fused_corr > 2) {
    set_error("gl_plan_set_tuning: fused_corr %d (1 FFMA2, 2 scalar FFMA)", t->fused_corr);
    return GL_ERR_INVALID;
  }
  if (t->lsq_gram < 0 || t->lsq_gram > 2) {
    set_error("gl_plan_set_tuning: lsq_gram %d (1 tensor cores, 2 FP32)", t->lsq_gram);
    return GL_ERR_INVALID;
  }
  if (t->fused_corr) plan->corr_scalar = t->fused_corr == 2;
  if (plan->lsq && t->lsq_gram) ((LsqPlan*)plan->lsq)->gram = t->lsq_gram;
  if (!plan->lsq || (t->lsq_ctas_per_sm == 0 && t->lsq_col_block == 0)) return GL_OK;
  LsqPlan* L = (LsqPlan*)plan->lsq;
  const int ctas = t->lsq_ctas_per_sm ? t->lsq_ctas_per_sm : L->ctas_per_sm;
  const int cb = t->lsq_col_block == 0 ? L->col_block : (t->lsq_col_block < 0 ? 0 : t->lsq_col_block);
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != plan->device) {
    set_error("plan was created on device %d but device %d is current", plan->device, dev);
    return GL_ERR_INVALID;
  }
  LsqPlan saved = *L;
  int rc = lsq_plan_layout(L, plan, ctas, cb);
  if (rc) *L = saved;   // keep the previous, valid layout
  return rc;
}

extern "C" int gl_plan_get_tuning(const gl_plan* plan, gl_tuning* t) {
  using namespace gl;
  if (!plan || !t) {
    set_error("gl_plan_get_tuning: null plan or tuning");
    return GL_ERR_INVALID;
  }
  memset(t, 0, sizeof(*t));
  t->fused_corr = plan->corr_scalar ? 2 : 1;
  if (plan->lsq) {
    const LsqPlan* L = (const LsqPlan*)plan->lsq;
    t->lsq_ctas_per_sm = L->ctas_per_sm;
    t->lsq_col_block = L->img[0].CB;
    t->lsq_gram = L->gram;
  }
  return GL_OK;
}
