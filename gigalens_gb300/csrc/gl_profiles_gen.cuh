// Closed-form profiles of the fused kernel's general path and of the
// elementwise profile kernels, each written once as a template over its
// scalar type: float gives the value, Dual<N> the value and its derivatives
// (see gl_dual.cuh).  Formulas follow the reference:
//   SIS         gigalens/tf/profiles/mass/sis.py:13-18
//   SIE         gigalens/tf/profiles/mass/sie.py:14-43 (s_scale = 0)
//   TNFW        gigalens/tf/profiles/mass/tnfw.py:14-58
//   CoreSersic  gigalens/tf/profiles/light/sersic.py:88-121, with the
//               reference's grouping kept as it is: the core term
//               (1 + (Rb/R)^alpha)^(gamma/alpha) times
//               exp(-bn ((R^alpha + Rb^alpha) / R_sersic^alpha / (alpha n)) - 1)
//   Shapelets   gigalens/tf/profiles/light/shapelets.py:53-85 (interpolate=False: the
//               Hermite recursion; True: the tabulated functions)
#pragma once
#include "gl_dual.cuh"

namespace gl {

constexpr float kPiF = 3.14159265358979f;

// sqrt with a zero derivative at 0 (the reference's sqrt gradient is infinite
// there; the profiles below only take sqrt(0) where the result is not used
// through its derivative, e.g. e1 = e2 = 0).
__device__ __forceinline__ float gsqrt0(float x) { return sqrtf(x); }
template <int N>
__device__ __forceinline__ Dual<N> gsqrt0(const Dual<N>& x) {
  const float s = sqrtf(x.v);
  return chain1(x, s, s > 0.f ? 0.5f / s : 0.f);
}

// ------------------------------------------------------------------ SIS
template <class T>
__device__ __forceinline__ void sis_alpha_t(const T& theta_E, const T& cx, const T& cy, float x,
                                            float y, T& ax, T& ay) {
  const T dx = x - cx, dy = y - cy;
  const T R = gsqrt0(dx * dx + dy * dy);
  const T a = (val(R) == 0.f) ? T(0.f) : theta_E / R;
  ax = a * dx;
  ay = a * dy;
}

// ------------------------------------------------------------------ SIE
template <class T>
__device__ __forceinline__ void sie_alpha_t(const T& theta_E, const T& e1, const T& e2, const T& cx,
                                            const T& cy, float x, float y, T& ax, T& ay) {
  const T phi = gatan2(e2, e1) * 0.5f;
  T c = gsqrt0(e1 * e1 + e2 * e2);
  if (val(c) > 0.9999f) c = T(0.9999f);   // tf.math.minimum(c, 0.9999)
  const T q = (1.f - c) / (1.f + c);
  const T q2 = q * q;
  const T theta_E_conv = theta_E / gsqrt((1.f + q2) / (2.f * q));
  const T b = theta_E_conv * gsqrt((1.f + q2) / 2.f);
  const T cp = gcos(phi), sp = gsin(phi);
  const T dx = x - cx, dy = y - cy;
  const T xr = dx * cp + dy * sp;
  const T yr = -dx * sp + dy * cp;
  const T psi = gsqrt(q2 * (xr * xr) + yr * yr);
  const T sq = gsqrt(1.f - q2);
  const T fx = b / sq * gatan(sq * xr / psi);
  const T fy = b / sq * gatanh(sq * yr / psi);
  ax = fx * cp - fy * sp;
  ay = fx * sp + fy * cp;
}

// SIE on the fused kernel's general path: the per-sample constants once
// (the same operations as sie_alpha_t), the deflection per pixel, and a
// hand-written reverse mode that accumulates the adjoints of the per-sample
// intermediates B = b / sqrt(1 - q^2), sq = sqrt(1 - q^2), q^2, phi and the
// centre; sie_chain maps them to (theta_E, e1, e2, center_x, center_y) once
// per sample.
struct SieC {
  float B, sq, q2, cp, sp, cx, cy;
};
__device__ __forceinline__ SieC sie_consts(float theta_E, float e1, float e2, float cx, float cy) {
  const float phi = atan2f(e2, e1) * 0.5f;
  float c = sqrtf(e1 * e1 + e2 * e2);
  if (c > 0.9999f) c = 0.9999f;
  const float q = (1.f - c) / (1.f + c);
  const float q2 = q * q;
  const float theta_E_conv = theta_E / sqrtf((1.f + q2) / (2.f * q));
  const float b = theta_E_conv * sqrtf((1.f + q2) / 2.f);
  SieC k;
  k.sq = sqrtf(1.f - q2);
  k.B = b / k.sq;
  k.q2 = q2;
  k.cp = cosf(phi);
  k.sp = sinf(phi);
  k.cx = cx;
  k.cy = cy;
  return k;
}
__device__ __forceinline__ void sie_alpha(const SieC& k, float x, float y, float& ax, float& ay) {
  const float dx = x - k.cx, dy = y - k.cy;
  const float xr = dx * k.cp + dy * k.sp;
  const float yr = -dx * k.sp + dy * k.cp;
  const float psi = sqrtf(k.q2 * (xr * xr) + yr * yr);
  const float fx = k.B * atanf(k.sq * xr / psi);
  const float fy = k.B * atanhf(k.sq * yr / psi);
  ax = fx * k.cp - fy * k.sp;
  ay = fx * k.sp + fy * k.cp;
}
// Adjoint slots: 0 B, 1 sq, 2 q^2, 3 phi, 4 center_x, 5 center_y.
constexpr int kSieAcc = 6;
__device__ __forceinline__ void sie_backprop(const SieC& k, float x, float y, float abx, float aby, float* acc) {
  const float dx = x - k.cx, dy = y - k.cy;
  const float xr = dx * k.cp + dy * k.sp;
  const float yr = -dx * k.sp + dy * k.cp;
  const float ipsi = 1.f / sqrtf(k.q2 * (xr * xr) + yr * yr);
  const float u = k.sq * xr * ipsi, v = k.sq * yr * ipsi;
  const float au = atanf(u), av = atanhf(v);
  const float fx = k.B * au, fy = k.B * av;
  // alpha = R(-phi) (fx, fy): the rotation's phi adjoint, then (fx, fy)
  acc[3] += abx * (-fx * k.sp - fy * k.cp) + aby * (fx * k.cp - fy * k.sp);
  const float fxb = abx * k.cp + aby * k.sp, fyb = -abx * k.sp + aby * k.cp;
  acc[0] += fxb * au + fyb * av;
  const float ub = fxb * k.B / (1.f + u * u), vb = fyb * k.B / (1.f - v * v);
  acc[1] += (ub * xr + vb * yr) * ipsi;
  // u = sq xr / psi, v = sq yr / psi, psi^2 = q^2 xr^2 + yr^2
  const float psib = -(ub * u + vb * v) * ipsi;
  acc[2] += psib * 0.5f * xr * xr * ipsi;
  const float xrb = (ub * k.sq + psib * k.q2 * xr) * ipsi;
  const float yrb = (vb * k.sq + psib * yr) * ipsi;
  // (xr, yr) = R(phi) (dx, dy)
  acc[3] += xrb * yr - yrb * xr;
  acc[4] -= xrb * k.cp - yrb * k.sp;
  acc[5] -= xrb * k.sp + yrb * k.cp;
}
// d logL / d(theta_E, e1, e2, center_x, center_y) from the adjoints (thread 0).
__device__ __forceinline__ void sie_chain(float theta_E, float e1, float e2, const float* acc, float out[5]) {
  using D3 = Dual<3>;
  const D3 tE = D3::seed(theta_E, 0), E1 = D3::seed(e1, 1), E2 = D3::seed(e2, 2);
  const D3 phi = gatan2(E2, E1) * 0.5f;
  D3 c = gsqrt0(E1 * E1 + E2 * E2);
  if (val(c) > 0.9999f) c = D3(0.9999f);
  const D3 q = (1.f - c) / (1.f + c);
  const D3 q2 = q * q;
  const D3 theta_E_conv = tE / gsqrt((1.f + q2) / (2.f * q));
  const D3 b = theta_E_conv * gsqrt((1.f + q2) / 2.f);
  const D3 sq = gsqrt(1.f - q2);
  const D3 B = b / sq;
#pragma unroll
  for (int i = 0; i < 3; ++i) out[i] = acc[0] * B.d[i] + acc[1] * sq.d[i] + acc[2] * q2.d[i] + acc[3] * phi.d[i];
  out[3] = acc[4];
  out[4] = acc[5];
}

// ------------------------------------------------------------------ TNFW
// F(x) of the NFW profile, tnfw.py:41-58 (exactly 1 at x == 1)
template <class T>
__device__ __forceinline__ T tnfw_F(const T& X) {
  const float xv = val(X);
  if (xv < 1.f) {
    const T s = gsqrt(1.f - X * X);
    return gatanh(s) / s;
  }
  if (xv > 1.f) {
    const T s = gsqrt(X * X - 1.f);
    return gatan(s) / s;
  }
  return T(1.f);
}

template <class T>
__device__ __forceinline__ void tnfw_alpha_t(const T& Rs, const T& alpha_Rs, const T& r_trunc,
                                             const T& cx, const T& cy, float x, float y, T& ax,
                                             T& ay) {
  const T rho0 = alpha_Rs / (4.f * (Rs * Rs) * (1.f + logf(0.5f)));
  const T dx = x - cx, dy = y - cy;
  T R = gsqrt0(dx * dx + dy * dy);
  const T Rmin = 0.001f * Rs;
  if (!(val(R) >= val(Rmin))) R = Rmin;   // tf.maximum(R, 0.001 Rs)
  const T X = R / Rs;
  const T tau = r_trunc / Rs;
  const T t2 = tau * tau;
  const T st = gsqrt(t2 + X * X);
  const T L = glog(X / (tau + st));
  const T F = tnfw_F(X);
  const T t21 = t2 + 1.f;
  const T gx = t2 / (t21 * t21) *
               ((t21 + 2.f * (X * X - 1.f)) * F + tau * kPiF + (t2 - 1.f) * glog(tau) +
                st * (-kPiF + L * (t2 - 1.f) / tau));
  const T a = 4.f * rho0 * Rs * gx / (X * X);
  ax = a * dx;
  ay = a * dy;
}

// ------------------------------------------------------------------ CoreSersic
// Sersic distance, tf/profiles/light/sersic.py:33-59
template <class T>
__device__ __forceinline__ T sersic_distance_t(const T& X, const T& Y, const T& cx, const T& cy,
                                               const T& e1, const T& e2) {
  const T phi = gatan2(e2, e1) * 0.5f;
  const T c = gsqrt0(e1 * e1 + e2 * e2);
  const T q = (1.f - c) / (1.f + c);
  const T dx = X - cx, dy = Y - cy;
  const T cp = gcos(phi), sp = gsin(phi);
  const T sq = gsqrt(q);
  const T xt1 = (cp * dx + sp * dy) * sq;
  const T xt2 = (-sp * dx + cp * dy) / sq;
  return gsqrt0(xt1 * xt1 + xt2 * xt2);
}

// unit-amplitude CoreSersic (the caller multiplies by Ie)
template <class T>
__device__ __forceinline__ T core_sersic_t(const T& Rs, const T& n, const T& Rb, const T& alpha,
                                           const T& gamma, const T& e1, const T& e2, const T& cx,
                                           const T& cy, const T& X, const T& Y) {
  const T R = sersic_distance_t(X, Y, cx, cy, e1, e2);
  const T bn = 1.9992f * n - 0.3271f;
  const T core = gpow(1.f + gpow(Rb / R, alpha), gamma / alpha);
  const T arg = -bn * ((gpow(R, alpha) + gpow(Rb, alpha)) / gpow(Rs, alpha) / (alpha * n)) - 1.f;
  return core * gexp(arg);
}

// ------------------------------------------------------------------ Shapelets
// phi_n(t) = H_n(t) / sqrt(2^n sqrt(pi) n!) for n = 0..nmax (physicists'
// Hermite polynomials, H_n = 2 (t H_{n-1} - (n-1) H_{n-2})).
__device__ __forceinline__ void shapelet_phis(float t, int nmax, const float* pref,
                                              float (&ph)[kMaxShapeletN + 1]) {
  float h0 = 1.f, h1 = 2.f * t;
  ph[0] = pref[0];
#pragma unroll
  for (int k = 1; k <= kMaxShapeletN; ++k) {
    if (k <= nmax) {
      if (k >= 2) {
        const float h2 = 2.f * (t * h1 - (float)(k - 1) * h0);
        h0 = h1;
        h1 = h2;
      }
      ph[k] = h1 * pref[k];
    } else {
      ph[k] = 0.f;
    }
  }
}

// Tabulated shapelet functions (Shapelets(interpolate=True),
// tf/profiles/light/shapelets.py:37-38,55-60): psi_n(t) = phi_n(t) e^{-t^2/2}
// at kShpTabN points on [kShpTabLo, kShpTabHi], row n of `tab`, linearly
// interpolated as tfp.math.interp_regular_1d_grid does -- fractional index
// (t - lo) / (hi - lo) (N - 1) clipped to the grid, the bracket [i0, i0 + 1]
// (the last bracket for the top point), value w y1 + (1 - w) y0 -- with 0
// outside [lo, hi] and NaN for NaN t.  The slope d psi / dt is the bracket's
// (y1 - y0) (N - 1) / (hi - lo), the derivative of that interpolant.
struct ShpLerp {
  int i0, i1;
  float w;
  int state;   // 0 inside, 1 outside (value 0), 2 NaN
};
__device__ __forceinline__ ShpLerp shp_lerp(float t) {
  ShpLerp L;
  L.state = isnan(t) ? 2 : ((t >= kShpTabLo && t <= kShpTabHi) ? 0 : 1);
  float fi = (t - kShpTabLo) / (kShpTabHi - kShpTabLo) * (float)(kShpTabN - 1);
  fi = fminf(fmaxf(fi, 0.f), (float)(kShpTabN - 1));   // a NaN index becomes 0
  float ib = floorf(fi);
  const float ia = fminf(ib + 1.f, (float)(kShpTabN - 1));
  ib = fmaxf(ia - 1.f, 0.f);
  L.w = fi - ib;
  L.i0 = (int)ib;
  L.i1 = (int)ia;
  return L;
}
__device__ __forceinline__ float shp_tab_value(const float* __restrict__ tab, int n, const ShpLerp& L) {
  if (L.state == 2) return __int_as_float(0x7fc00000);
  if (L.state == 1) return 0.f;
  const float* r = tab + n * kShpTabN;
  const float y0 = __ldg(r + L.i0), y1 = __ldg(r + L.i1);
  return L.w * y1 + (1.f - L.w) * y0;
}
__device__ __forceinline__ void shp_tab_value_slope(const float* __restrict__ tab, int n, const ShpLerp& L,
                                                    float& val, float& slope) {
  if (L.state != 0) {
    val = slope = L.state == 2 ? __int_as_float(0x7fc00000) : 0.f;
    return;
  }
  const float* r = tab + n * kShpTabN;
  const float y0 = __ldg(r + L.i0), y1 = __ldg(r + L.i1);
  val = L.w * y1 + (1.f - L.w) * y0;
  slope = (y1 - y0) * ((float)(kShpTabN - 1) / (kShpTabHi - kShpTabLo));
}

// sum_k amp_k psi_n1(u) psi_n2(v) from the table, and its u, v partials.
__device__ __forceinline__ float shapelets_sum_interp(float u, float v, int nmax, const float* amp,
                                                      const float* __restrict__ tab, float* du, float* dv) {
  float pu[kMaxShapeletN + 1], pv[kMaxShapeletN + 1], qu[kMaxShapeletN + 1], qv[kMaxShapeletN + 1];
  const ShpLerp Lu = shp_lerp(u), Lv = shp_lerp(v);
#pragma unroll
  for (int k = 0; k <= kMaxShapeletN; ++k) {
    if (k <= nmax) {
      shp_tab_value_slope(tab, k, Lu, pu[k], qu[k]);
      shp_tab_value_slope(tab, k, Lv, pv[k], qv[k]);
    } else {
      pu[k] = pv[k] = qu[k] = qv[k] = 0.f;
    }
  }
  float s = 0.f, su = 0.f, sv = 0.f;
#pragma unroll
  for (int m = 0; m <= kMaxShapeletN; ++m) {
    if (m <= nmax) {
#pragma unroll
      for (int j = 0; j <= m; ++j) {
        const int n1 = m - j, n2 = j;
        const float c = amp[m * (m + 1) / 2 + j];
        s = fmaf(c, pu[n1] * pv[n2], s);
        if (du) {
          su = fmaf(c, qu[n1] * pv[n2], su);
          sv = fmaf(c, pu[n1] * qv[n2], sv);
        }
      }
    }
  }
  if (du) {
    *du = su;
    *dv = sv;
  }
  return s;
}

// Value of sum_k amp_k e^{-(u^2+v^2)/2} phi_n1(u) phi_n2(v) (k in the
// reference's order (0,0), (1,0), (0,1), (2,0), ...), and its u, v partials.
__device__ __forceinline__ float shapelets_sum(float u, float v, int nmax, const float* amp,
                                               const float* pref, float* du, float* dv) {
  float pu[kMaxShapeletN + 1], pv[kMaxShapeletN + 1];
  shapelet_phis(u, nmax, pref, pu);
  shapelet_phis(v, nmax, pref, pv);
  const float fac = expf(-(u * u + v * v) / 2.f);
  float s = 0.f, su = 0.f, sv = 0.f;
#pragma unroll
  for (int m = 0; m <= kMaxShapeletN; ++m) {
    if (m <= nmax) {
#pragma unroll
      for (int j = 0; j <= m; ++j) {
        const int n1 = m - j, n2 = j;
        const float c = amp[m * (m + 1) / 2 + j];
        s = fmaf(c, pu[n1] * pv[n2], s);
        if (du) {
          // d/dt phi_n = sqrt(2n) phi_{n-1}
          const float dpu = n1 > 0 ? sqrtf(2.f * n1) * pu[n1 - 1] : 0.f;
          const float dpv = n2 > 0 ? sqrtf(2.f * n2) * pv[n2 - 1] : 0.f;
          su = fmaf(c, dpu * pv[n2], su);
          sv = fmaf(c, pu[n1] * dpv, sv);
        }
      }
    }
  }
  if (du) {
    *du = fac * (su - u * s);
    *dv = fac * (sv - v * s);
  }
  return fac * s;
}

}  // namespace gl
