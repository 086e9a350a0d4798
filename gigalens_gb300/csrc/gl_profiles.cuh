// Per-pixel profile arithmetic (forward and reverse mode) shared by the fused
// kernel and the elementwise profile kernels.
//
// Forward formulas follow the reference:
//   EPL    gigalens/tf/profiles/mass/epl.py:23-68  (Tessore-Metcalf series)
//   Shear  gigalens/tf/profiles/mass/shear.py:12-14
//   Sersic gigalens/tf/profiles/light/sersic.py:25-72
// The reverse mode is written by hand: it replaces TensorFlow autodiff and
// differentiates the same expressions.  The EPL series is not stored: its
// derivatives come from two extra sums of the recomputed series,
//   dF/da = i (2H + F),  H = sum_n n last_n     (last_n = A_n e^{i(2n+1)a})
//   dF/df = H / f                                (A_n is proportional to f^n)
//   dF/dt = sum_n s_n last_n, s_n = sum_{m<=n} d ln|p_m| / dt
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace gl {

constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLn2 = 0.6931471805599453f;
constexpr float kHalfLog2Pi = 0.91893853320467274f;

// ------------------------------------------------------------------ EPL
struct EplC {
  float cx, cy, cph, sph;   // centre, rotation by phi
  float q, t, tm1, f;       // axis ratio, t = gamma-1, f = (1-q)/(1+q)
  float A, log2b;           // A = 2b/(1+q), b = theta_E_conv*sqrt((1+q^2)/2)
  int K;                    // series iterations
};

__device__ __forceinline__ EplC epl_consts(float theta_E, float gamma, float e1, float e2, float cx,
                                           float cy, int K) {
  EplC c;
  float phi = atan2f(e2, e1) * 0.5f;
  float cr = sqrtf(e1 * e1 + e2 * e2);
  float cc = fminf(fmaxf(cr, 0.f), 1.f);
  float q = (1.f - cc) / (1.f + cc);
  float theta_E_conv = theta_E / sqrtf((1.f + q * q) / (2.f * q));
  float b = theta_E_conv * sqrtf((1.f + q * q) / 2.f);
  sincosf(phi, &c.sph, &c.cph);
  c.cx = cx;
  c.cy = cy;
  c.q = q;
  c.t = gamma - 1.f;
  c.tm1 = c.t - 1.f;
  c.f = (1.f - q) / (1.f + q);
  c.A = (2.f * b) / (1.f + q);
  c.log2b = log2f(b);
  c.K = K;
  return c;
}

// Term count rule, tf/profiles/mass/epl.py:41 and :51-56, float32 throughout.
__device__ __forceinline__ float epl_f_of(float e1, float e2) {
  float cc = fminf(fmaxf(sqrtf(e1 * e1 + e2 * e2), 0.f), 1.f);
  float q = (1.f - cc) / (1.f + cc);
  return (1.f - q) / (1.f + q);
}
__device__ __forceinline__ int epl_terms_from_maxf(float maxf, int cap) {
  float niter = logf(1e-12f) / logf(maxf) + 2.f;
  // iterations i = 1, 2, ... while i < niter, at most cap
  int k = 0;
  if (niter > 1.f) {                      // false for NaN
    float c = ceilf(niter) - 1.f;
    k = c >= (float)cap ? cap : (int)c;
  }
  return k;
}

// p_n = -f (2n - (2-t)) / (2n + (2-t)) with the reference's op order.
__device__ __forceinline__ float epl_prefac(float f, float t, int n) {
  float nn = (float)n;
  float tt = 2.f - t;
  return (-f * (2.f * nn - tt)) / (2.f * nn + tt);
}
// d ln|p_n| / dt
__device__ __forceinline__ float epl_dlnp_dt(float t, int n) {
  float nn = (float)n;
  return 1.f / (2.f * nn - 2.f + t) + 1.f / (2.f * nn + 2.f - t);
}

struct EplGeom {
  float dx, dy, xr, yr, qx, R2, invR, l2Rc, Cs, Ss, Cs2, Ss2;
  bool clipped;
};

__device__ __forceinline__ EplGeom epl_geom(const EplC& c, float x, float y) {
  EplGeom g;
  g.dx = x - c.cx;
  g.dy = y - c.cy;
  g.xr = g.dx * c.cph + g.dy * c.sph;
  g.yr = -g.dx * c.sph + g.dy * c.cph;
  g.qx = c.q * g.xr;
  g.R2 = g.qx * g.qx + g.yr * g.yr;
  float R = sqrtf(g.R2);
  float Rc = fminf(fmaxf(R, 1e-10f), 1e10f);
  g.clipped = !(R >= 1e-10f && R <= 1e10f);
  if (g.R2 > 0.f) {
    g.invR = rsqrtf(g.R2);
    g.Cs = g.qx * g.invR;
    g.Ss = g.yr * g.invR;
  } else {  // atan2(+-0, +-0): angle 0 or pi
    g.invR = 0.f;
    g.Cs = signbit(g.qx) ? -1.f : 1.f;
    g.Ss = 0.f;
  }
  g.l2Rc = __log2f(Rc);
  g.Cs2 = g.Cs * g.Cs - g.Ss * g.Ss;
  g.Ss2 = 2.f * g.Cs * g.Ss;
  return g;
}

// The series as a trigonometric sum: last_n = A_n z^(2n+1) with z = e^{ia},
// A_n = prod_{m<=n} p_m, so F = sum_{n<=K} last_n = z P(w), P(w) = sum A_n w^n,
// w = z^2 = e^{2ia}.  The coefficients are real and |w| = 1, so
//   Re P = A_0 + b_1 cos(2a) - b_2,  Im P = b_1 sin(2a),
//   b_n = A_n + 2 cos(2a) b_{n+1} - b_{n+2}  (n = K..1, b_{K+1} = b_{K+2} = 0),
// Clenshaw's recurrence: 2 FP32 operations per term and one dependent FMA.
// tab[n] = (A_n, n A_n, s_n A_n, s_n A_n), n = 0..K (A_0 = 1, s_0 = 0); the
// repeated last entry lets two pixels' third recurrence read an aligned pair.
__device__ __forceinline__ void epl_series_F(const EplGeom& g, const float4* __restrict__ tab, int K,
                                             float& Fx, float& Fy) {
  const float c2 = 2.f * g.Cs2;
  float b1 = 0.f, b2 = 0.f;
#pragma unroll 4
  for (int n = K; n >= 1; --n) {
    const float b0 = fmaf(c2, b1, tab[n].x - b2);
    b2 = b1;
    b1 = b0;
  }
  const float Px = fmaf(b1, g.Cs2, 1.f - b2), Py = b1 * g.Ss2;
  Fx = g.Cs * Px - g.Ss * Py;
  Fy = g.Cs * Py + g.Ss * Px;
}

// Forward deflection.
__device__ __forceinline__ void epl_deflect(const EplC& c, const float4* __restrict__ tab, float x,
                                            float y, float& ax, float& ay) {
  EplGeom g = epl_geom(c, x, y);
  float Fx, Fy;
  epl_series_F(g, tab, c.K, Fx, Fy);
  float P = c.A * exp2f(c.tm1 * (c.log2b - g.l2Rc));
  float arx = Fx * P, ary = Fy * P;
  ax = arx * c.cph - ary * c.sph;
  ay = arx * c.sph + ary * c.cph;
}

// NP pixels at once: their recurrences interleave for ILP.
template <int NP>
__device__ __forceinline__ void epl_deflect_n(const EplC& c, const float4* __restrict__ tab,
                                              const float (&x)[NP], const float (&y)[NP],
                                              float (&ax)[NP], float (&ay)[NP]) {
  EplGeom g[NP];
  float c2[NP], b1[NP], b2[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    g[k] = epl_geom(c, x[k], y[k]);
    c2[k] = 2.f * g[k].Cs2;
    b1[k] = 0.f;
    b2[k] = 0.f;
  }
  if constexpr (NP == 4) {
    // Packed FFMA2 over pixel pairs (0, 1) and (2, 3), the same roundings as
    // the scalar loop (t - b2 as fma(b2, -1, t)): identical results.
    const float2 neg = make_float2(-1.f, -1.f);
    const float2 ca = make_float2(c2[0], c2[1]), cb = make_float2(c2[2], c2[3]);
    float2 u1 = make_float2(0.f, 0.f), u2 = u1, v1 = u1, v2 = u1;
#pragma unroll 2
    for (int n = c.K; n >= 1; --n) {
      const float a = tab[n].x;
      const float2 aa = make_float2(a, a);
      const float2 u0 = __ffma2_rn(ca, u1, __ffma2_rn(u2, neg, aa));
      const float2 v0 = __ffma2_rn(cb, v1, __ffma2_rn(v2, neg, aa));
      u2 = u1;
      u1 = u0;
      v2 = v1;
      v1 = v0;
    }
    b1[0] = u1.x; b1[1] = u1.y; b2[0] = u2.x; b2[1] = u2.y;
    b1[2] = v1.x; b1[3] = v1.y; b2[2] = v2.x; b2[3] = v2.y;
  } else {
#pragma unroll 2
    for (int n = c.K; n >= 1; --n) {
      const float a = tab[n].x;
#pragma unroll
      for (int k = 0; k < NP; ++k) {
        const float b0 = fmaf(c2[k], b1[k], a - b2[k]);
        b2[k] = b1[k];
        b1[k] = b0;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    const float Px = fmaf(b1[k], g[k].Cs2, 1.f - b2[k]), Py = b1[k] * g[k].Ss2;
    const float Fx = g[k].Cs * Px - g[k].Ss * Py, Fy = g[k].Cs * Py + g[k].Ss * Px;
    const float P = c.A * exp2f(c.tm1 * (c.log2b - g[k].l2Rc));
    const float arx = Fx * P, ary = Fy * P;
    ax[k] = arx * c.cph - ary * c.sph;
    ay[k] = arx * c.sph + ary * c.cph;
  }
}

struct EplAcc {
  float phi, SP, SPlnR, FH, FT, q, cx, cy;
  __device__ __forceinline__ void zero() { phi = SP = SPlnR = FH = FT = q = cx = cy = 0.f; }
};

// Series state of one pixel: the deflection plus the sums that the reverse
// mode needs (H = sum n last_n, T = sum s_n last_n).
struct EplState {
  EplGeom g;
  float Fx, Fy, Hx, Hy, Tx, Ty, P, ax, ay;
};

// F = z P(w), H = z sum n A_n w^n, T = z sum s_n A_n w^n: three Clenshaw
// recurrences over the columns of the table, for NP pixels at once.
template <int NP>
__device__ __forceinline__ void epl_state_n(const EplC& c, const float4* __restrict__ tab,
                                            const float (&x)[NP], const float (&y)[NP],
                                            EplState (&s)[NP]) {
  float c2[NP], a1[NP], a2[NP], m1[NP], m2[NP], r1[NP], r2[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    s[k].g = epl_geom(c, x[k], y[k]);
    c2[k] = 2.f * s[k].g.Cs2;
    a1[k] = a2[k] = m1[k] = m2[k] = r1[k] = r2[k] = 0.f;
  }
  if constexpr (NP == 2) {
    // Packed FFMA2 (two FMAs per instruction, each rounded as fmaf): per
    // pixel the F and H recurrences share the table pair (A_n, n A_n); the T
    // recurrences of the two pixels share (s_n A_n, s_n A_n).  t - b2 is
    // fma(b2, -1, t), the same rounding as the subtraction, so the results
    // equal the scalar loop's bit for bit.
    const float2 neg = make_float2(-1.f, -1.f);
    const float2 cp0 = make_float2(c2[0], c2[0]), cp1 = make_float2(c2[1], c2[1]);
    const float2 cr = make_float2(c2[0], c2[1]);
    float2 p1 = make_float2(0.f, 0.f), p2 = p1, q1 = p1, q2 = p1, s1 = p1, s2 = p1;
#pragma unroll 2
    for (int n = c.K; n >= 1; --n) {
      const float4 t = tab[n];
      const float2 tam = make_float2(t.x, t.y), tss = make_float2(t.z, t.w);
      const float2 p0 = __ffma2_rn(cp0, p1, __ffma2_rn(p2, neg, tam));
      const float2 q0 = __ffma2_rn(cp1, q1, __ffma2_rn(q2, neg, tam));
      const float2 s0 = __ffma2_rn(cr, s1, __ffma2_rn(s2, neg, tss));
      p2 = p1;
      p1 = p0;
      q2 = q1;
      q1 = q0;
      s2 = s1;
      s1 = s0;
    }
    a1[0] = p1.x; m1[0] = p1.y; a2[0] = p2.x; m2[0] = p2.y;
    a1[1] = q1.x; m1[1] = q1.y; a2[1] = q2.x; m2[1] = q2.y;
    r1[0] = s1.x; r1[1] = s1.y; r2[0] = s2.x; r2[1] = s2.y;
  } else {
#pragma unroll 2
    for (int n = c.K; n >= 1; --n) {
      const float4 t = tab[n];
#pragma unroll
      for (int k = 0; k < NP; ++k) {
        const float a0 = fmaf(c2[k], a1[k], t.x - a2[k]);
        const float m0 = fmaf(c2[k], m1[k], t.y - m2[k]);
        const float r0 = fmaf(c2[k], r1[k], t.z - r2[k]);
        a2[k] = a1[k];
        a1[k] = a0;
        m2[k] = m1[k];
        m1[k] = m0;
        r2[k] = r1[k];
        r1[k] = r0;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    const float wx = s[k].g.Cs2, wy = s[k].g.Ss2;
    // n = 0 coefficients: A_0 = 1, 0 * A_0 = 0, s_0 A_0 = 0
    const float Px = fmaf(a1[k], wx, 1.f - a2[k]), Py = a1[k] * wy;
    const float Nx = fmaf(m1[k], wx, -m2[k]), Ny = m1[k] * wy;
    const float Qx = fmaf(r1[k], wx, -r2[k]), Qy = r1[k] * wy;
    const float zx = s[k].g.Cs, zy = s[k].g.Ss;
    s[k].Fx = zx * Px - zy * Py;
    s[k].Fy = zx * Py + zy * Px;
    s[k].Hx = zx * Nx - zy * Ny;
    s[k].Hy = zx * Ny + zy * Nx;
    s[k].Tx = zx * Qx - zy * Qy;
    s[k].Ty = zx * Qy + zy * Qx;
    s[k].P = c.A * exp2f(c.tm1 * (c.log2b - s[k].g.l2Rc));
    const float arx = s[k].Fx * s[k].P, ary = s[k].Fy * s[k].P;
    s[k].ax = arx * c.cph - ary * c.sph;
    s[k].ay = arx * c.sph + ary * c.cph;
  }
}

__device__ __forceinline__ EplState epl_state(const EplC& c, const float4* __restrict__ tab, float x,
                                              float y) {
  const float xs[1] = {x}, ys[1] = {y};
  EplState s[1];
  epl_state_n<1>(c, tab, xs, ys, s);
  return s[0];
}

// Per-chain series table, built by one warp: tab[n] = (A_n, n A_n, s_n A_n, 0),
// n = 0..K, with A_n = prod_{m<=n} p_m (p_m with the reference's op order) and
// s_n = sum_{m<=n} d ln|p_m| / dt, both as warp scans.
__device__ __forceinline__ void epl_build_table(float4* tab, float f, float t, int K, int lane) {
  float carry_p = 1.f, carry_s = 0.f;
  for (int base = 0; base <= K; base += 32) {
    const int n = base + lane;
    const bool term = n >= 1 && n <= K;
    float p = term ? epl_prefac(f, t, n) : 1.f;
    float dl = term ? epl_dlnp_dt(t, n) : 0.f;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float yp = __shfl_up_sync(0xffffffffu, p, o);
      const float yd = __shfl_up_sync(0xffffffffu, dl, o);
      if (lane >= o) {
        p *= yp;
        dl += yd;
      }
    }
    const float A = carry_p * p, S = carry_s + dl;
    if (n <= K) tab[n] = make_float4(A, (float)n * A, S * A, S * A);
    carry_p *= __shfl_sync(0xffffffffu, p, 31);
    carry_s += __shfl_sync(0xffffffffu, dl, 31);
  }
}

// Accumulate the contribution of the deflection adjoint (abx, aby).
__device__ __forceinline__ void epl_backprop(const EplC& c, const EplState& s, float abx, float aby,
                                             EplAcc& acc) {
  const EplGeom& g = s.g;
  // rotate back by -phi
  acc.phi += -abx * s.ay + aby * s.ax;
  float arbx = abx * c.cph + aby * c.sph;
  float arby = -abx * c.sph + aby * c.cph;
  // alpha_r = P * F
  float Pb = arbx * s.Fx + arby * s.Fy;
  float PbP = Pb * s.P;
  acc.SP += PbP;
  acc.SPlnR += PbP * (kLn2 * g.l2Rc);
  float Fbx = s.P * arbx, Fby = s.P * arby;
  float Dx = 2.f * s.Hx + s.Fx, Dy = 2.f * s.Hy + s.Fy;
  float ab = -Fbx * Dy + Fby * Dx;          // adjoint of the angle a
  acc.FH += Fbx * s.Hx + Fby * s.Hy;
  acc.FT += Fbx * s.Tx + Fby * s.Ty;
  float Rb = g.clipped ? 0.f : -PbP * c.tm1 * g.invR;   // dP/dR = P (1-t) / R
  float inv2 = g.invR * g.invR;
  float qxb = Rb * g.qx * g.invR - ab * g.yr * inv2;
  float yrb = Rb * g.yr * g.invR + ab * g.qx * inv2;
  float xrb = qxb * c.q;
  acc.q += qxb * g.xr;
  float dxb = xrb * c.cph - yrb * c.sph;
  float dyb = xrb * c.sph + yrb * c.cph;
  acc.phi += xrb * g.yr - yrb * g.xr;
  acc.cx -= dxb;
  acc.cy -= dyb;
}

// Per-sample chain rule of the EPL accumulators to d/d(theta_E, gamma, e1, e2, cx, cy).
__device__ __forceinline__ void epl_chain(float theta_E, float gamma, float e1, float e2,
                                          const EplC& c, const EplAcc& a, float out[6]) {
  float cr = sqrtf(e1 * e1 + e2 * e2);
  float cc = fminf(fmaxf(cr, 0.f), 1.f);
  float q = c.q;
  float b = exp2f(c.log2b);
  float lnb = kLn2 * c.log2b;
  float tb = a.SP * lnb - a.SPlnR + a.FT;          // d/dt
  float bb = (b != 0.f) ? a.SP * c.tm1 / b : 0.f;  // d/db via P
  float Ab = (c.A != 0.f) ? a.SP / c.A : 0.f;       // d/dA
  bb += Ab * 2.f / (1.f + q);
  float qb = a.q - Ab * 2.f * b / ((1.f + q) * (1.f + q));
  if (c.f != 0.f) qb += (a.FH / c.f) * (-2.f / ((1.f + q) * (1.f + q)));
  // b = theta_E * sqrt(q) (the reference's two-factor form, simplified)
  float thb = bb * sqrtf(q);
  if (q != 0.f) qb += bb * b / (2.f * q);
  float cb = qb * (-2.f / ((1.f + cc) * (1.f + cc)));
  float e1b = 0.f, e2b = 0.f;
  if (cr > 0.f && cr <= 1.f) {
    e1b += cb * e1 / cr;
    e2b += cb * e2 / cr;
  }
  float r2 = e1 * e1 + e2 * e2;
  if (r2 > 0.f) {
    e1b += a.phi * (-0.5f * e2 / r2);
    e2b += a.phi * (0.5f * e1 / r2);
  }
  out[0] = thb;
  out[1] = tb;
  out[2] = e1b;
  out[3] = e2b;
  out[4] = a.cx;
  out[5] = a.cy;
}

// ------------------------------------------------------------------ Sersic
struct SerC {
  float cx, cy, cph, sph, sq, isq;
  float a1, a0;     // rho = (R/Rs)^(1/n) = exp2(a1*log2(R^2) - a0)
  float nb;         // -bn*log2(e)
  float bn, Ie;
};

__device__ __forceinline__ SerC sersic_consts(float Rs, float n, float e1, float e2, float cx,
                                              float cy, float Ie) {
  SerC s;
  float phi = atan2f(e2, e1) * 0.5f;
  float c = sqrtf(e1 * e1 + e2 * e2);
  float q = (1.f - c) / (1.f + c);
  sincosf(phi, &s.sph, &s.cph);
  s.sq = sqrtf(q);
  s.isq = 1.f / s.sq;
  s.cx = cx;
  s.cy = cy;
  s.a1 = 0.5f / n;
  s.a0 = log2f(Rs) / n;
  s.bn = 1.9992f * n - 0.3271f;
  s.nb = -s.bn * kLog2e;
  s.Ie = Ie;
  return s;
}

__device__ __forceinline__ float sersic_light(const SerC& s, float X, float Y) {
  float dX = X - s.cx, dY = Y - s.cy;
  float u = s.cph * dX + s.sph * dY;
  float v = -s.sph * dX + s.cph * dY;
  float xt1 = u * s.sq, xt2 = v * s.isq;
  float R2 = xt1 * xt1 + xt2 * xt2;
  float rho = exp2f(s.a1 * __log2f(R2) - s.a0);
  return s.Ie * exp2f(s.nb * (rho - 1.f));
}

struct SerAcc {
  float Ie, RsA, nA, bnA, sq, isq, phi, cx, cy;
  __device__ __forceinline__ void zero() { Ie = RsA = nA = bnA = sq = isq = phi = cx = cy = 0.f; }
};

struct SerFwd {
  float dX, dY, u, v, xt1, xt2, R2, l2, rho, E, I;
};

__device__ __forceinline__ SerFwd sersic_fwd(const SerC& s, float X, float Y) {
  SerFwd f;
  f.dX = X - s.cx;
  f.dY = Y - s.cy;
  f.u = s.cph * f.dX + s.sph * f.dY;
  f.v = -s.sph * f.dX + s.cph * f.dY;
  f.xt1 = f.u * s.sq;
  f.xt2 = f.v * s.isq;
  f.R2 = f.xt1 * f.xt1 + f.xt2 * f.xt2;
  f.l2 = __log2f(f.R2);
  f.rho = exp2f(s.a1 * f.l2 - s.a0);
  f.E = exp2f(s.nb * (f.rho - 1.f));
  f.I = s.Ie * f.E;
  return f;
}

// Reverse of one Sersic evaluation with image adjoint Ib; returns the
// adjoint of the evaluation coordinates in (Xb, Yb).
__device__ __forceinline__ void sersic_reverse(const SerC& s, const SerFwd& f, float Ib,
                                               SerAcc& a, float& Xb, float& Yb) {
  a.Ie += Ib * f.E;
  float rb = Ib * (-s.bn * f.I);          // adjoint of rho
  float rr = rb * f.rho;
  a.RsA += rr;
  float lnrho = kLn2 * (s.a1 * f.l2 - s.a0);
  a.nA += rr * lnrho;
  a.bnA += Ib * f.I * (f.rho - 1.f);
  float R2b = (f.R2 > 0.f) ? rr * s.a1 / f.R2 : 0.f;
  float xt1b = 2.f * R2b * f.xt1, xt2b = 2.f * R2b * f.xt2;
  float ub = xt1b * s.sq, vb = xt2b * s.isq;
  a.sq += xt1b * f.u;
  a.isq += xt2b * f.v;
  float dXb = ub * s.cph - vb * s.sph;
  float dYb = ub * s.sph + vb * s.cph;
  a.phi += ub * f.v - vb * f.u;
  a.cx -= dXb;
  a.cy -= dYb;
  Xb = dXb;
  Yb = dYb;
}

// Per-sample chain to d/d(R_sersic, n_sersic, e1, e2, cx, cy, Ie).
// Two Sersic profiles evaluated together on packed FP32 pairs (component x:
// profile a, y: profile b; a pixel's lens light at theta and source at
// beta).  Each packed operation rounds as its scalar counterpart (fused
// multiply-adds where the scalar code contracts), the transcendentals run per
// component: the values agree with sersic_light / sersic_fwd / sersic_reverse
// to float32 rounding.
struct SerC2 {
  float2 ncx, ncy, cph, sph, nsph, sq, isq, a1, na0, nb, Ie, nbn;
};
__device__ __forceinline__ SerC2 sersic_pack(const SerC& a, const SerC& b) {
  SerC2 p;
  p.ncx = make_float2(-a.cx, -b.cx);
  p.ncy = make_float2(-a.cy, -b.cy);
  p.cph = make_float2(a.cph, b.cph);
  p.sph = make_float2(a.sph, b.sph);
  p.nsph = make_float2(-a.sph, -b.sph);
  p.sq = make_float2(a.sq, b.sq);
  p.isq = make_float2(a.isq, b.isq);
  p.a1 = make_float2(a.a1, b.a1);
  p.na0 = make_float2(-a.a0, -b.a0);
  p.nb = make_float2(a.nb, b.nb);
  p.Ie = make_float2(a.Ie, b.Ie);
  p.nbn = make_float2(-a.bn, -b.bn);
  return p;
}
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }

__device__ __forceinline__ float2 sersic_light2(const SerC2& s, float2 X, float2 Y) {
  const float2 dX = __fadd2_rn(X, s.ncx), dY = __fadd2_rn(Y, s.ncy);
  const float2 u = __ffma2_rn(s.cph, dX, __fmul2_rn(s.sph, dY));
  const float2 v = __ffma2_rn(s.cph, dY, __fmul2_rn(s.nsph, dX));
  const float2 xt1 = __fmul2_rn(u, s.sq), xt2 = __fmul2_rn(v, s.isq);
  const float2 R2 = __ffma2_rn(xt1, xt1, __fmul2_rn(xt2, xt2));
  const float2 t = __ffma2_rn(s.a1, make_float2(__log2f(R2.x), __log2f(R2.y)), s.na0);
  const float2 e = __fmul2_rn(s.nb, __fadd2_rn(make_float2(exp2f(t.x), exp2f(t.y)), f2(-1.f)));
  return __fmul2_rn(s.Ie, make_float2(exp2f(e.x), exp2f(e.y)));
}

struct SerFwd2 {
  float2 dX, dY, u, v, xt1, xt2, R2, l2, rho, E, I;
};
struct SerAcc2 {
  float2 Ie, RsA, nA, bnA, sq, isq, phi, cx, cy;
  __device__ __forceinline__ void zero() {
    Ie = RsA = nA = bnA = sq = isq = phi = cx = cy = make_float2(0.f, 0.f);
  }
};
__device__ __forceinline__ SerFwd2 sersic_fwd2(const SerC2& s, float2 X, float2 Y) {
  SerFwd2 f;
  f.dX = __fadd2_rn(X, s.ncx);
  f.dY = __fadd2_rn(Y, s.ncy);
  f.u = __ffma2_rn(s.cph, f.dX, __fmul2_rn(s.sph, f.dY));
  f.v = __ffma2_rn(s.cph, f.dY, __fmul2_rn(s.nsph, f.dX));
  f.xt1 = __fmul2_rn(f.u, s.sq);
  f.xt2 = __fmul2_rn(f.v, s.isq);
  f.R2 = __ffma2_rn(f.xt1, f.xt1, __fmul2_rn(f.xt2, f.xt2));
  f.l2 = make_float2(__log2f(f.R2.x), __log2f(f.R2.y));
  const float2 t = __ffma2_rn(s.a1, f.l2, s.na0);
  f.rho = make_float2(exp2f(t.x), exp2f(t.y));
  const float2 e = __fmul2_rn(s.nb, __fadd2_rn(f.rho, f2(-1.f)));
  f.E = make_float2(exp2f(e.x), exp2f(e.y));
  f.I = __fmul2_rn(s.Ie, f.E);
  return f;
}
__device__ __forceinline__ void sersic_reverse2(const SerC2& s, const SerFwd2& f, float Ib, SerAcc2& a,
                                                float2& Xb, float2& Yb) {
  const float2 ib = f2(Ib);
  a.Ie = __ffma2_rn(ib, f.E, a.Ie);
  const float2 rb = __fmul2_rn(ib, __fmul2_rn(s.nbn, f.I));   // adjoint of rho
  const float2 rr = __fmul2_rn(rb, f.rho);
  a.RsA = __fadd2_rn(a.RsA, rr);
  const float2 lnrho = __fmul2_rn(f2(kLn2), __ffma2_rn(s.a1, f.l2, s.na0));
  a.nA = __ffma2_rn(rr, lnrho, a.nA);
  a.bnA = __ffma2_rn(__fmul2_rn(ib, f.I), __fadd2_rn(f.rho, f2(-1.f)), a.bnA);
  const float2 ra = __fmul2_rn(rr, s.a1);
  const float2 R2b = make_float2(f.R2.x > 0.f ? ra.x / f.R2.x : 0.f, f.R2.y > 0.f ? ra.y / f.R2.y : 0.f);
  const float2 R2b2 = __fmul2_rn(f2(2.f), R2b);
  const float2 xt1b = __fmul2_rn(R2b2, f.xt1), xt2b = __fmul2_rn(R2b2, f.xt2);
  const float2 ub = __fmul2_rn(xt1b, s.sq), vb = __fmul2_rn(xt2b, s.isq);
  a.sq = __ffma2_rn(xt1b, f.u, a.sq);
  a.isq = __ffma2_rn(xt2b, f.v, a.isq);
  const float2 dXb = __ffma2_rn(ub, s.cph, __fmul2_rn(vb, s.nsph));
  const float2 dYb = __ffma2_rn(ub, s.sph, __fmul2_rn(vb, s.cph));
  a.phi = __ffma2_rn(ub, f.v, __ffma2_rn(__fmul2_rn(vb, f2(-1.f)), f.u, a.phi));
  a.cx = __ffma2_rn(dXb, f2(-1.f), a.cx);
  a.cy = __ffma2_rn(dYb, f2(-1.f), a.cy);
  Xb = dXb;
  Yb = dYb;
}

__device__ __forceinline__ void sersic_chain(float Rs, float n, float e1, float e2, const SerC& s,
                                             const SerAcc& a, float out[7]) {
  float c = sqrtf(e1 * e1 + e2 * e2);
  float q = s.sq * s.sq;
  out[0] = a.RsA * (-1.f / (n * Rs));
  out[1] = a.nA * (-1.f / n) - a.bnA * 1.9992f;
  float qb = a.sq * 0.5f / s.sq + a.isq * (-0.5f * s.isq / q);
  float cb = qb * (-2.f / ((1.f + c) * (1.f + c)));
  float e1b = 0.f, e2b = 0.f;
  if (c > 0.f) {
    e1b = cb * e1 / c + a.phi * (-0.5f * e2 / (c * c));
    e2b = cb * e2 / c + a.phi * (0.5f * e1 / (c * c));
  }
  out[2] = e1b;
  out[3] = e2b;
  out[4] = a.cx;
  out[5] = a.cy;
  out[6] = a.Ie;
}

}  // namespace gl
