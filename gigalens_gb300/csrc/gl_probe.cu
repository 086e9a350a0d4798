// Diagnostics: an FP32 FMA throughput probe.  The fused kernel is bound by
// the FP32 pipe, and the measured peak of this probe (at the clocks of the
// moment) is the denominator of its roofline fraction.
#include "gl_internal.cuh"

namespace gl {

// Eight independent FMA chains per thread; 2 flop per FMA.
__global__ void __launch_bounds__(256) fma_probe_kernel(float* out, int iters, float a, float b) {
  float r0 = threadIdx.x, r1 = r0 + 1.f, r2 = r0 + 2.f, r3 = r0 + 3.f;
  float r4 = r0 + 4.f, r5 = r0 + 5.f, r6 = r0 + 6.f, r7 = r0 + 7.f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      r0 = fmaf(r0, a, b);
      r1 = fmaf(r1, a, b);
      r2 = fmaf(r2, a, b);
      r3 = fmaf(r3, a, b);
      r4 = fmaf(r4, a, b);
      r5 = fmaf(r5, a, b);
      r6 = fmaf(r6, a, b);
      r7 = fmaf(r7, a, b);
    }
  }
  const float s = r0 + r1 + r2 + r3 + r4 + r5 + r6 + r7;
  if (s == 1234.5f) out[blockIdx.x] = s;   // keep the chains alive
}

}  // namespace gl

extern "C" int gl_probe_fp32_fma(float* out, int iters, int blocks_per_sm, double* flops,
                                 void* stream) {
  using namespace gl;
  if (!out || iters <= 0 || blocks_per_sm <= 0) {
    set_error("gl_probe_fp32_fma: bad arguments");
    return GL_ERR_INVALID;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * blocks_per_sm;
  fma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters, 0.999999f, 1e-7f);
  if (flops) *flops = 2.0 * 8.0 * 16.0 * (double)iters * 256.0 * (double)blocks;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("probe launch: %s", cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}
