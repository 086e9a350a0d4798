// Forward-mode dual numbers for the reverse mode of the closed-form profiles
// on the fused kernel's general path (SIS, SIE, TNFW, CoreSersic).
//
// A profile formula is written once as a template over its scalar type: with
// float it is the forward evaluation, with Dual<N> (value + N partial
// derivatives, seeded with one direction per parameter) the same code yields
// the value and its gradient with respect to the N seeded inputs.  The reverse
// mode of a pixel then contracts that gradient with the pixel's adjoint.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace gl {

template <int N>
struct Dual {
  float v;
  float d[N];
  __device__ __forceinline__ Dual() {}
  __device__ __forceinline__ Dual(float c) : v(c) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.f;
  }
  // input number k of the N seeded directions
  __device__ __forceinline__ static Dual seed(float c, int k) {
    Dual r(c);
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = (i == k) ? 1.f : 0.f;
    return r;
  }
};

// ---- value access (float and Dual alike)
__device__ __forceinline__ float val(float x) { return x; }
template <int N>
__device__ __forceinline__ float val(const Dual<N>& x) { return x.v; }

// r = f(x) with f'(x) = g: chain rule helper
template <int N>
__device__ __forceinline__ Dual<N> chain1(const Dual<N>& x, float f, float g) {
  Dual<N> r;
  r.v = f;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = g * x.d[i];
  return r;
}

// ---- arithmetic
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fmaf(a.d[i], b.v, a.v * b.d[i]);
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  const float ib = 1.f / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, float b) {
  Dual<N> r = a;
  r.v += b;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(float a, const Dual<N>& b) {
  return b + a;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, float b) {
  Dual<N> r = a;
  r.v -= b;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(float a, const Dual<N>& b) {
  Dual<N> r = -b;
  r.v += a;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, float b) {
  Dual<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(float a, const Dual<N>& b) {
  return b * a;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, float b) {
  Dual<N> r;
  r.v = a.v / b;
  const float ib = 1.f / b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * ib;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(float a, const Dual<N>& b) {
  return Dual<N>(a) / b;
}

// ---- elementary functions (float overloads call the CUDA functions)
__device__ __forceinline__ float gsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ float gexp(float x) { return expf(x); }
__device__ __forceinline__ float glog(float x) { return logf(x); }
__device__ __forceinline__ float gatan(float x) { return atanf(x); }
__device__ __forceinline__ float gatanh(float x) { return atanhf(x); }
__device__ __forceinline__ float gatan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ float gcos(float x) { return cosf(x); }
__device__ __forceinline__ float gsin(float x) { return sinf(x); }
__device__ __forceinline__ float gpow(float a, float b) { return powf(a, b); }

template <int N>
__device__ __forceinline__ Dual<N> gsqrt(const Dual<N>& x) {
  const float s = sqrtf(x.v);
  return chain1(x, s, 0.5f / s);
}
template <int N>
__device__ __forceinline__ Dual<N> gexp(const Dual<N>& x) {
  const float e = expf(x.v);
  return chain1(x, e, e);
}
template <int N>
__device__ __forceinline__ Dual<N> glog(const Dual<N>& x) {
  return chain1(x, logf(x.v), 1.f / x.v);
}
template <int N>
__device__ __forceinline__ Dual<N> gatan(const Dual<N>& x) {
  return chain1(x, atanf(x.v), 1.f / (1.f + x.v * x.v));
}
template <int N>
__device__ __forceinline__ Dual<N> gatanh(const Dual<N>& x) {
  return chain1(x, atanhf(x.v), 1.f / (1.f - x.v * x.v));
}
template <int N>
__device__ __forceinline__ Dual<N> gcos(const Dual<N>& x) {
  return chain1(x, cosf(x.v), -sinf(x.v));
}
template <int N>
__device__ __forceinline__ Dual<N> gsin(const Dual<N>& x) {
  return chain1(x, sinf(x.v), cosf(x.v));
}
// d atan2(y, x) = (x dy - y dx) / (x^2 + y^2)
template <int N>
__device__ __forceinline__ Dual<N> gatan2(const Dual<N>& y, const Dual<N>& x) {
  Dual<N> r;
  r.v = atan2f(y.v, x.v);
  const float r2 = x.v * x.v + y.v * y.v;
  const float ir = r2 > 0.f ? 1.f / r2 : 0.f;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (x.v * y.d[i] - y.v * x.d[i]) * ir;
  return r;
}
// a^b = exp(b log a) for a > 0; d = a^b (b' log a + b a'/a)
template <int N>
__device__ __forceinline__ Dual<N> gpow(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = powf(a.v, b.v);
  const float la = logf(a.v);
  const float ba = b.v / a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = r.v * fmaf(b.d[i], la, ba * a.d[i]);
  return r;
}

}  // namespace gl
