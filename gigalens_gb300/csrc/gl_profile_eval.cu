// Elementwise profile evaluation (the MassProfile.deriv / LightProfile.light
// API), the EPL term-count rule as a device reduction, and the unconstraining
// bijector.  These are the non-fused entry points; the fused kernel inlines
// the same arithmetic from gl_profiles.cuh.
#include <cmath>
#include <mutex>
#include <vector>

#include "gl_internal.cuh"
#include "gl_profiles.cuh"
#include "gl_profiles_gen.cuh"

namespace gl {

// params: [np][n], row p = canonical parameter p.
template <int TYPE>
__global__ void profile_eval_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                    int64_t n, const float* __restrict__ prm,
                                    const int* __restrict__ n_terms, float* __restrict__ out0,
                                    float* __restrict__ out1) {
  const int K = (TYPE == GL_PROF_EPL) ? *n_terms : 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float xi = x[i], yi = y[i];
    auto P = [&](int p) { return prm[(int64_t)p * n + i]; };
    if (TYPE == GL_PROF_EPL) {
      const float theta_E = P(0), gamma = P(1), e1 = P(2), e2 = P(3);
      EplC c = epl_consts(theta_E, gamma, e1, e2, P(4), P(5), K);
      EplGeom g = epl_geom(c, xi, yi);
      float lx = g.Cs, ly = g.Ss, Fx = g.Cs, Fy = g.Ss;
      for (int k = 1; k <= K; ++k) {
        const float p = epl_prefac(c.f, c.t, k);
        const float u = p * lx, v = p * ly;
        lx = fmaf(g.Cs2, u, -g.Ss2 * v);
        ly = fmaf(g.Ss2, u, g.Cs2 * v);
        Fx += lx;
        Fy += ly;
      }
      const float Pf = c.A * exp2f(c.tm1 * (c.log2b - g.l2Rc));
      const float arx = Fx * Pf, ary = Fy * Pf;
      out0[i] = arx * c.cph - ary * c.sph;
      out1[i] = arx * c.sph + ary * c.cph;
    } else if (TYPE == GL_PROF_SHEAR) {
      const float g1 = P(0), g2 = P(1);
      out0[i] = g1 * xi + g2 * yi;
      out1[i] = g2 * xi - g1 * yi;
    } else if (TYPE == GL_PROF_SIS) {
      float ax, ay;
      sis_alpha_t<float>(P(0), P(1), P(2), xi, yi, ax, ay);
      out0[i] = ax;
      out1[i] = ay;
    } else if (TYPE == GL_PROF_SIE) {
      float ax, ay;
      sie_alpha_t<float>(P(0), P(1), P(2), P(3), P(4), xi, yi, ax, ay);
      out0[i] = ax;
      out1[i] = ay;
    } else if (TYPE == GL_PROF_TNFW) {
      float ax, ay;
      tnfw_alpha_t<float>(P(0), P(1), P(2), P(3), P(4), xi, yi, ax, ay);
      out0[i] = ax;
      out1[i] = ay;
    } else if (TYPE == GL_PROF_CORE_SERSIC) {
      out0[i] = P(9) * core_sersic_t<float>(P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), xi, yi);
    } else if (TYPE == GL_PROF_SERSIC) {
      SerC s = sersic_consts(P(0), P(1), 0.f, 0.f, P(2), P(3), P(4));
      out0[i] = sersic_light(s, xi, yi);
    } else if (TYPE == GL_PROF_SERSIC_ELLIPSE) {
      SerC s = sersic_consts(P(0), P(1), P(2), P(3), P(4), P(5), P(6));
      out0[i] = sersic_light(s, xi, yi);
    }
  }
}

int launch_profile_eval(int type, const float* x, const float* y, int64_t n, const float* params,
                        const int* n_terms, float* out0, float* out1, cudaStream_t stream) {
  if (n == 0) return GL_OK;
  int sms = 1, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256;
  int64_t blocks = (n + threads - 1) / threads;
  if (blocks > (int64_t)sms * 8) blocks = (int64_t)sms * 8;
  switch (type) {
#define GL_CASE(T) \
  case T: profile_eval_kernel<T><<<(int)blocks, threads, 0, stream>>>(x, y, n, params, n_terms, out0, out1); break;
    GL_CASE(GL_PROF_EPL)
    GL_CASE(GL_PROF_SHEAR)
    GL_CASE(GL_PROF_SIS)
    GL_CASE(GL_PROF_SIE)
    GL_CASE(GL_PROF_TNFW)
    GL_CASE(GL_PROF_CORE_SERSIC)
    GL_CASE(GL_PROF_SERSIC)
    GL_CASE(GL_PROF_SERSIC_ELLIPSE)
#undef GL_CASE
    default:
      set_error("gl_profile_eval: type %d not supported", type);
      return GL_ERR_UNSUPPORTED;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("profile kernel launch: %s", cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}

// Shapelets at n points: Hermite recursion per point, all orders at once.
__global__ void shapelets_eval_kernel(int n_max, const float* __restrict__ tab, const float* __restrict__ x,
                                      const float* __restrict__ y, int64_t n, const float* __restrict__ prm,
                                      const float* __restrict__ amps, float* __restrict__ out) {
  __shared__ float pref[32];
  if (threadIdx.x <= n_max) {
    double f = 1.0;
    for (int i = 2; i <= (int)threadIdx.x; ++i) f *= i;
    pref[threadIdx.x] = (float)(1.0 / sqrt(pow(2.0, (double)threadIdx.x) * sqrt(3.14159265358979323846) * f));
  }
  __syncthreads();
  const int D = (n_max + 1) * (n_max + 2) / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float beta = prm[i], cx = prm[n + i], cy = prm[2 * n + i];
    const float u = (x[i] - cx) / beta, v = (y[i] - cy) / beta;
    if (tab) {   // interpolate=True: products of tabulated 1-D functions
      const ShpLerp Lu = shp_lerp(u), Lv = shp_lerp(v);
      float acc = 0.f;
      int n1 = 0, n2 = 0;
      for (int k = 0; k < D; ++k) {
        const float bk = shp_tab_value(tab, n1, Lu) * shp_tab_value(tab, n2, Lv);
        if (amps) acc = fmaf(amps[(int64_t)k * n + i], bk, acc);
        else out[(int64_t)k * n + i] = bk;
        if (n1 == 0) {
          n1 = n2 + 1;
          n2 = 0;
        } else {
          --n1;
          ++n2;
        }
      }
      if (amps) out[i] = acc;
      continue;
    }
    float hu[32], hv[32];
    hu[0] = 1.f;
    hv[0] = 1.f;
    if (n_max >= 1) {
      hu[1] = 2.f * u;
      hv[1] = 2.f * v;
    }
    for (int k = 2; k <= n_max; ++k) {
      hu[k] = 2.f * (u * hu[k - 1] - (float)(k - 1) * hu[k - 2]);
      hv[k] = 2.f * (v * hv[k - 1] - (float)(k - 1) * hv[k - 2]);
    }
    const float fac = expf(-(u * u + v * v) / 2.f);
    float acc = 0.f;
    int n1 = 0, n2 = 0;
    for (int k = 0; k < D; ++k) {
      const float bk = fac * (hu[n1] * pref[n1]) * (hv[n2] * pref[n2]);
      if (amps) acc = fmaf(amps[(int64_t)k * n + i], bk, acc);
      else out[(int64_t)k * n + i] = bk;
      if (n1 == 0) {
        n1 = n2 + 1;
        n2 = 0;
      } else {
        --n1;
        ++n2;
      }
    }
    if (amps) out[i] = acc;
  }
}

// One block: max over the batch of f, then the reference's term-count rule.
__global__ void epl_term_count_kernel(const float* __restrict__ e1, const float* __restrict__ e2,
                                      int64_t n, int cap, int* __restrict__ k_out) {
  __shared__ float red[32];
  float m = 0.f;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, epl_f_of(e1[i], e2[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmaxf(t, red[w]);
    *k_out = epl_terms_from_maxf(t, cap);
  }
}

int launch_shapelets_eval(int n_max, const float* tab, const float* x, const float* y, int64_t n,
                          const float* params, const float* amps, float* out, cudaStream_t stream) {
  if (n == 0) return GL_OK;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  shapelets_eval_kernel<<<(int)blocks, 256, 0, stream>>>(n_max, tab, x, y, n, params, amps, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("shapelets launch: %s", cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}

// ------------------------------------------------------------------ shapelet table
// psi_n(x_i) = phi_n(x_i) e^{-x_i^2/2}, x_i = lo + i (hi - lo) / (N - 1), the
// reference's tables of lenstronomy's 1-D shapelet functions
// (tf/profiles/light/shapelets.py:37-38: phi_n on linspace(-5, 5, 6000),
// stored as float32).  Computed in double with the normalised recurrence
// psi_0 = pi^{-1/4} e^{-x^2/2}, psi_1 = sqrt(2) x psi_0,
// psi_n = sqrt(2/n) x psi_{n-1} - sqrt((n-1)/n) psi_{n-2}, which equals
// H_n(x) e^{-x^2/2} / sqrt(2^n sqrt(pi) n!) without its large intermediates.
static __device__ float g_shp_table[kShpTabRows * kShpTabN];
constexpr int kShpMaxDevices = 64;
static const float* g_shp_addr[kShpMaxDevices];
static std::mutex g_shp_mutex;

int shapelet_table(int device, const float** out) {
  if (device < 0 || device >= kShpMaxDevices) {
    set_error("shapelet table: device %d out of range", device);
    return GL_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_shp_mutex);
  if (!g_shp_addr[device]) {
    std::vector<float> host((size_t)kShpTabRows * kShpTabN);
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < kShpTabN; ++i) {
      const double xv = (double)kShpTabLo + (double)i * ((double)kShpTabHi - (double)kShpTabLo) / (kShpTabN - 1);
      double p0 = std::pow(pi, -0.25) * std::exp(-0.5 * xv * xv);
      double p1 = std::sqrt(2.0) * xv * p0;
      host[i] = (float)p0;
      host[kShpTabN + i] = (float)p1;
      for (int k = 2; k < kShpTabRows; ++k) {
        const double p2 = std::sqrt(2.0 / k) * xv * p1 - std::sqrt((k - 1.0) / k) * p0;
        host[(size_t)k * kShpTabN + i] = (float)p2;
        p0 = p1;
        p1 = p2;
      }
    }
    cudaError_t e = cudaMemcpyToSymbol(g_shp_table, host.data(), host.size() * sizeof(float));
    void* p = nullptr;
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_shp_table);
    if (e != cudaSuccess || !p) {
      set_error("shapelet table: %s", cudaGetErrorString(e));
      return GL_ERR_CUDA;
    }
    g_shp_addr[device] = (const float*)p;
  }
  *out = g_shp_addr[device];
  return GL_OK;
}

int launch_epl_term_count(const float* e1, const float* e2, int64_t n, int cap, int* k_out,
                          cudaStream_t stream) {
  epl_term_count_kernel<<<1, 512, 0, stream>>>(e1, e2, n, cap, k_out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("term count launch: %s", cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}

struct PriorTable {
  DevPriorLeaf leaf[GL_MAX_PARAMS];
};

__global__ void bijector_forward_kernel(const __grid_constant__ PriorTable t, int d,
                                        const float* __restrict__ z, int64_t total,
                                        float* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const DevPriorLeaf& L = t.leaf[i % d];
    const float v = z[i];
    float r;
    switch (L.dist) {
      case GL_DIST_LOGNORMAL: r = expf(v); break;
      case GL_DIST_UNIFORM:
      case GL_DIST_TRUNCNORMAL: r = L.lo + (L.hi - L.lo) * (1.f / (1.f + expf(-v))); break;
      default: r = v;
    }
    x[i] = r;
  }
}

int launch_bijector_forward(const DevPriorLeaf* leaves, int d, const float* z, int bs, float* x,
                            cudaStream_t stream) {
  if (bs == 0) return GL_OK;
  PriorTable t;
  for (int i = 0; i < GL_MAX_PARAMS; ++i) t.leaf[i] = leaves[i];
  const int64_t total = (int64_t)bs * d;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  bijector_forward_kernel<<<blocks, 256, 0, stream>>>(t, d, z, total, x);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("bijector launch: %s", cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}

}  // namespace gl
