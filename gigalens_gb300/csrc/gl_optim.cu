// Adam step with Keras semantics and a device-side step counter, so the whole
// MAP iteration (fused log-prob+gradient kernel, then this) replays from one
// CUDA graph without host synchronisation.
#include "gl_internal.cuh"

namespace gl {

__device__ __forceinline__ float lr_at(const gl_adam_cfg& c, float s) {
  if (c.schedule == GL_LR_POLYNOMIAL) {
    const float ss = fminf(s, c.decay_steps);
    return (c.lr0 - c.lr_end) * powf(1.f - ss / c.decay_steps, c.power) + c.lr_end;
  }
  return c.lr0;
}

__global__ void adam_kernel(float* __restrict__ var, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ grad, int64_t n, float grad_scale,
                            const gl_adam_cfg c, const int* __restrict__ step) {
  const int s = *step;
  const float t = (float)(s + 1);
  const float lr = lr_at(c, (float)s);
  const float alpha = lr * sqrtf(1.f - powf(c.beta2, t)) / (1.f - powf(c.beta1, t));
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float g = grad[i] * grad_scale;
    float mi = m[i], vi = v[i];
    mi += (g - mi) * (1.f - c.beta1);
    vi += (g * g - vi) * (1.f - c.beta2);
    m[i] = mi;
    v[i] = vi;
    var[i] -= (mi * alpha) / (sqrtf(vi) + c.eps);
  }
}

__global__ void step_increment_kernel(int* step) { *step += 1; }

}  // namespace gl

extern "C" int gl_adam_step(float* var, float* m, float* v, const float* grad, int64_t n,
                            float grad_scale, const gl_adam_cfg* cfg, int* step, void* stream) {
  using namespace gl;
  if (!var || !m || !v || !grad || !cfg || !step || n < 0) {
    set_error("gl_adam_step: null pointer or negative size");
    return GL_ERR_INVALID;
  }
  if (cfg->schedule == GL_LR_POLYNOMIAL && !(cfg->decay_steps > 0.f)) {
    set_error("gl_adam_step: decay_steps must be > 0");
    return GL_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 1184) blocks = 1184;
  if (blocks < 1) blocks = 1;
  adam_kernel<<<blocks, 256, 0, s>>>(var, m, v, grad, n, grad_scale, *cfg, step);
  step_increment_kernel<<<1, 1, 0, s>>>(step);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("adam launch: %s", cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}
