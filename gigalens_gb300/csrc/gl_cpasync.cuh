// Asynchronous global -> shared copies (cp.async, 16 bytes per thread and
// copy, L2 only), used by the kernels that stream the least-squares basis
// stack X from HBM through a shared-memory ring: each thread issues its own
// copies of a chunk, commits them as one group and later waits until at most
// `n` of its groups are still in flight.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gl {

// Copy 16 bytes, of which the first `src_bytes` (0..16) are read from `src`
// and the rest are zero-filled.  Both addresses 16-byte aligned; with
// src_bytes == 0 nothing is read, and callers still pass an address inside
// the source buffer.
__device__ __forceinline__ void cp_async16(void* dst_smem, const void* src, uint32_t src_bytes) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes)
               : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Error-free transformation of a float sum (Knuth's TwoSum): s + e == a + b
// exactly, s = fl(a + b).  Used for float-float accumulators in place of
// float64, whose throughput is a small fraction of float32's on this GPU.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (hi, lo) += v, keeping hi + lo the float-float sum.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float v) {
  float s, e;
  two_sum(hi, v, s, e);
  hi = s;
  lo = __fadd_rn(lo, e);
}

}  // namespace gl
