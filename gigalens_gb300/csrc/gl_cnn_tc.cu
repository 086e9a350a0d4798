// Tensor-core (tcgen05, kind::tf32) GEMM of the learned initialiser's
// convolution layers: C(m, n) (+)= alpha * sum_k A(m, k) B(n, k) with
//   A(m, k) = A[m * a_sm + k * a_sk]   float32 activations or gradients
//   B(n, k) = B[n * b_sn + k * b_sk]   BF16 weights or float32 gradients
//   C(m, n) = C[m * c_sm + n * c_sn]
// The m side is the large output dimension (pixels of the batch, or the
// im2col rows of a weight gradient).  FP32-level accuracy from TF32 products:
// A is split into a TF32 head and tail, stored as ONE 128-row operand (heads
// rows 0-63, tails rows 64-127), so one MMA gives hi(A) B^T in TMEM lanes 0-63
// and lo(A) B^T in lanes 64-127.  BF16 weights are exact in TF32 (2xTF32);
// a float32 B is split as well and its tail rows follow its head rows in the
// N direction (3xTF32: hi hi + hi lo + lo hi).  Operands are staged through
// registers into the canonical K-major no-swizzle layout (8-row x 16-byte
// core matrices, K stride 144 bytes), two stages deep; one thread issues the
// MMAs and commits them to the stage's mbarrier (bounded waits: a timeout
// sets the status word and the CTA stops after draining).  K can be split
// over CTAs (ksplit): partial sums are added atomically into a zeroed C.
#include <cuda_bf16.h>

#include <cstdint>

#include "gl_internal.cuh"
#include "gl_tc.cuh"

namespace gl {

namespace {
constexpr int kTT = 256;                  // threads
constexpr int kTM = 64;                   // m rows per CTA (128 MMA rows: heads + tails)
constexpr int kTK = 32;                   // K per stage
constexpr uint32_t kTLBO = 144;           // bytes between K-adjacent core matrices
constexpr uint32_t kTSBO = kTLBO * (kTK / 4);
constexpr int kATile = 16 * kTSBO;        // 128 rows
constexpr uint32_t kTWait = 1u << 22;

__host__ __device__ constexpr int b_rows(int NS, bool split) { return split ? 2 * NS : NS; }
__host__ __device__ constexpr int b_tile_bytes(int NS, bool split) { return (b_rows(NS, split) / 8) * kTSBO; }
__host__ __device__ constexpr int tc_stage_bytes(int NS, bool split) { return kATile + b_tile_bytes(NS, split); }
__host__ __device__ constexpr int tc_smem_bytes(int NS, bool split) {
  return 1024 + 2 * tc_stage_bytes(NS, split) + 64 * 17 * 4;
}
__host__ __device__ constexpr uint32_t tmem_cols(int n) { return n <= 32 ? 32u : (n <= 64 ? 64u : (n <= 128 ? 128u : 256u)); }

__device__ __forceinline__ uint32_t koff(int row, int k) {
  return (uint32_t)(row >> 3) * kTSBO + (uint32_t)(k >> 2) * kTLBO + (uint32_t)(row & 7) * 16u +
         (uint32_t)(k & 3) * 4u;
}
}  // namespace

struct TcGemmArgs {
  int MA, NB, K;
  const float* A;
  long long a_sm, a_sk;
  const void* B;
  long long b_sn, b_sk;
  float* C;
  long long c_sm, c_sn;
  float alpha;
  int ksplit;
  int* status;
  uint32_t polls;
};

// A_MFAST: a_sm == 1 (consecutive threads along m); B_NFAST: b_sn == 1.
template <int NS, bool BSPLIT, bool BBF16, bool A_MFAST, bool B_NFAST>
__global__ void __launch_bounds__(kTT) cnn_gemm_tc_kernel(const __grid_constant__ TcGemmArgs a) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(tsm);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tsm + 64);
  unsigned char* stages = tsm + 1024;
  float* stage_out = reinterpret_cast<float*>(stages + 2 * tc_stage_bytes(NS, BSPLIT));   // [64][17]
  constexpr int NR = b_rows(NS, BSPLIT);   // MMA N
  constexpr uint32_t COLS = tmem_cols(NR);
  constexpr int A_PER = kTM * kTK / kTT;   // 8 elements of A per thread and stage
  constexpr int B_PER = (NS * kTK + kTT - 1) / kTT;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kTM, n0 = blockIdx.y * NS;
  // this CTA's K range
  const int kchunk = ((a.K + a.ksplit - 1) / a.ksplit + kTK - 1) / kTK * kTK;
  const int kbeg = blockIdx.z * kchunk, kend = min(a.K, kbeg + kchunk);
  const int nch = kend > kbeg ? (kend - kbeg + kTK - 1) / kTK : 0;
  const uint32_t idesc = idesc_tf32(128, NR);

  for (int i = tid; i < 2 * tc_stage_bytes(NS, BSPLIT) / 16; i += kTT)
    reinterpret_cast<float4*>(stages)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tc_alloc(tmem_slot, COLS);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  float ra[A_PER], rb[B_PER];
  auto a_idx = [&](int e, int& m, int& k) {
    const int t = tid + e * kTT;
    if (A_MFAST) {
      m = t % kTM;
      k = t / kTM;
    } else {
      k = t % kTK;
      m = t / kTK;
    }
  };
  auto b_idx = [&](int e, int& n, int& k) {
    const int t = tid + e * kTT;
    if (B_NFAST) {
      n = t % NS;
      k = t / NS;
    } else {
      k = t % kTK;
      n = t / kTK;
    }
  };
  auto load = [&](int ch) {
    const int k0 = kbeg + ch * kTK;
#pragma unroll
    for (int e = 0; e < A_PER; ++e) {
      int m, k;
      a_idx(e, m, k);
      const int gm = m0 + m, gk = k0 + k;
      ra[e] = (gm < a.MA && gk < kend) ? a.A[(long long)gm * a.a_sm + (long long)gk * a.a_sk] : 0.f;
    }
#pragma unroll
    for (int e = 0; e < B_PER; ++e) {
      int n, k;
      b_idx(e, n, k);
      const int gn = n0 + n, gk = k0 + k;
      float v = 0.f;
      if (tid + e * kTT < NS * kTK && gn < a.NB && gk < kend) {
        const long long idx = (long long)gn * a.b_sn + (long long)gk * a.b_sk;
        v = BBF16 ? __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(a.B)[idx])
                  : reinterpret_cast<const float*>(a.B)[idx];
      }
      rb[e] = v;
    }
  };
  auto store = [&](unsigned char* st) {
    unsigned char* tA = st;
    unsigned char* tB = st + kATile;
#pragma unroll
    for (int e = 0; e < A_PER; ++e) {
      int m, k;
      a_idx(e, m, k);
      const float hi = to_tf32(ra[e]);
      const float lo = to_tf32(ra[e] - hi);
      *reinterpret_cast<float*>(tA + koff(m, k)) = hi;
      *reinterpret_cast<float*>(tA + koff(m + 64, k)) = lo;
    }
#pragma unroll
    for (int e = 0; e < B_PER; ++e) {
      if (tid + e * kTT >= NS * kTK) continue;
      int n, k;
      b_idx(e, n, k);
      const float hi = BSPLIT ? to_tf32(rb[e]) : rb[e];   // BF16 values are exact in TF32
      *reinterpret_cast<float*>(tB + koff(n, k)) = hi;
      if (BSPLIT) *reinterpret_cast<float*>(tB + koff(n + NS, k)) = to_tf32(rb[e] - hi);
    }
  };

  bool failed = false;
  uint32_t committed = 0;
  if (nch > 0) load(0);
  for (int ch = 0; ch < nch; ++ch) {
    const int s = ch & 1;
    unsigned char* st = stages + s * tc_stage_bytes(NS, BSPLIT);
    bool ok = true;
    if (ch >= 2) ok = mbar_wait(&mbar[s], ((ch - 2) >> 1) & 1u, a.polls);
    if (ok) store(st);
    if (ch + 1 < nch) load(ch + 1);
    fence_proxy_async_smem();
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      const uint32_t ba = smem_u32(st), bb = smem_u32(st + kATile);
#pragma unroll
      for (int ks = 0; ks < kTK / 8; ++ks) {
        const uint64_t da = umma_desc_noswizzle(ba + (uint32_t)ks * 2u * kTLBO, kTLBO, kTSBO);
        const uint64_t db = umma_desc_noswizzle(bb + (uint32_t)ks * 2u * kTLBO, kTLBO, kTSBO);
        tc_mma_tf32(tmem, da, db, idesc, (ch == 0 && ks == 0) ? 0u : 1u);
      }
      tc_commit(&mbar[s]);
    }
    committed = ch + 1;
  }
  if (!failed && nch > 0) {
    const uint32_t last = nch - 1;
    const bool ok = mbar_wait(&mbar[last & 1], (last >> 1) & 1u, a.polls);
    if (__syncthreads_or(!ok)) failed = true;
  }
  if (failed) {
    if (tid == 0 && a.status) *a.status = 1;
    for (uint32_t k = 0; k < 2 && committed > k; ++k) {
      const uint32_t last = committed - 1 - k;
      mbar_wait(&mbar[last & 1], (last >> 1) & 1u, kTWait);
    }
  } else if (nch > 0) {
    tc_fence_after();
    // C(m, n) = D[m][n] (+ D[m][NS + n]) + D[64 + m][n], 16 columns at a time
    const int row = (warp & 1) * 32 + lane;
    for (int j0 = 0; j0 < NS; j0 += 16) {
      if (warp >= 2 && warp < 4) {
        float t[16];
        tc_ld_32x32b_x16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)j0, t);
#pragma unroll
        for (int i = 0; i < 16; ++i) stage_out[row * 17 + i] = t[i];
      }
      __syncthreads();
      if (warp < 2) {
        float hh[16], hl[16];
        tc_ld_32x32b_x16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)j0, hh);
        if (BSPLIT) tc_ld_32x32b_x16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(NS + j0), hl);
        const int gm = m0 + row;
        if (gm < a.MA) {
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int gn = n0 + j0 + i;
            if (gn >= a.NB) continue;
            float v = hh[i] + stage_out[row * 17 + i];
            if (BSPLIT) v += hl[i];
            float* c = a.C + (long long)gm * a.c_sm + (long long)gn * a.c_sn;
            if (a.ksplit > 1) atomicAdd(c, a.alpha * v);
            else *c = a.alpha * v;
          }
        }
      }
      __syncthreads();
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(tmem, COLS);
}

template <int NS, bool BSPLIT, bool BBF16, bool A_MFAST, bool B_NFAST>
static int launch_tc(const TcGemmArgs& a, cudaStream_t s) {
  static bool attr_set[kMaxDevices];
  const int dev = current_device_slot();
  constexpr int smem = tc_smem_bytes(NS, BSPLIT);
  if (!attr_set[dev]) {
    if (cudaFuncSetAttribute(cnn_gemm_tc_kernel<NS, BSPLIT, BBF16, A_MFAST, B_NFAST>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
      set_error("tensor-core GEMM: shared memory attribute");
      return GL_ERR_CUDA;
    }
    attr_set[dev] = true;
  }
  dim3 grid((a.MA + kTM - 1) / kTM, (a.NB + NS - 1) / NS, a.ksplit);
  cnn_gemm_tc_kernel<NS, BSPLIT, BBF16, A_MFAST, B_NFAST><<<grid, kTT, smem, s>>>(a);
  return GL_OK;
}

static int* g_tc_status[kMaxDevices];   // status word of the tensor-core GEMMs, per device

// The convolution GEMMs of gl_nn_gemm on the tensor cores; returns 1 when the
// call's shape is not one of them (the caller then uses its SIMT kernel).
//   forward     C[co][p]  = W[co][k] col[k][p]       (A bf16, no transposes)
//   input grad  C[k][p]   = W[co][k]^T dY[co][p]     (A bf16 transposed)
//   weight grad C[co][k]  = dY[co][p] col[k][p]^T    (float32, B transposed, K = pixels)
int nn_gemm_tc(int transA, int transB, int a_bf16, int M, int N, int K, float alpha, const void* A, int lda,
               const float* B, int ldb, float* C, int ldc, int ksplit, cudaStream_t s) {
  const int dev = current_device_slot();
  int dev_id = 0;
  cudaGetDevice(&dev_id);
  if (!g_tc_status[dev]) {
    if (cudaMalloc((void**)&g_tc_status[dev], sizeof(int)) != cudaSuccess ||
        cudaMemset(g_tc_status[dev], 0, sizeof(int)) != cudaSuccess) {
      set_error("tensor-core GEMM: status word");
      return GL_ERR_NOMEM;
    }
  }
  TcGemmArgs t{};
  t.alpha = alpha;
  t.ksplit = 1;
  t.status = g_tc_status[dev];
  t.polls = kTWait;
  if (!transA && !transB && a_bf16 && M <= 32 && N >= 4096) {
    // forward: m = pixel (N), n = output channel (M), k
    t.MA = N; t.NB = M; t.K = K;
    t.A = B; t.a_sm = 1; t.a_sk = ldb;
    t.B = A; t.b_sn = lda; t.b_sk = 1;
    t.C = C; t.c_sm = 1; t.c_sn = ldc;
    return launch_tc<32, false, true, true, false>(t, s);
  }
  if (transA && !transB && a_bf16 && K <= 32 && N >= 4096 && M <= 384) {
    // input gradient: m = pixel (N), n = im2col row (M), k = output channel
    t.MA = N; t.NB = M; t.K = K;
    t.A = B; t.a_sm = 1; t.a_sk = ldb;
    t.B = A; t.b_sn = 1; t.b_sk = lda;
    t.C = C; t.c_sm = 1; t.c_sn = ldc;
    return launch_tc<96, false, true, true, true>(t, s);
  }
  if (!transA && transB && !a_bf16 && M <= 32 && K >= 4096) {
    // weight gradient: m = im2col row (N), n = output channel (M), k = pixel (K); C zeroed by the caller
    t.MA = N; t.NB = M; t.K = K;
    t.A = B; t.a_sm = ldb; t.a_sk = 1;
    t.B = A; t.b_sn = lda; t.b_sk = 1;
    t.C = C; t.c_sm = 1; t.c_sn = ldc;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id);
    const int tiles = (N + kTM - 1) / kTM;
    int ks = (2 * sms + tiles - 1) / tiles;
    ks = ks > K / 1024 ? K / 1024 : ks;
    t.ksplit = ks < 1 ? 1 : ks;
    if (t.ksplit > 1 && ksplit <= 1) {   // partial sums need a zeroed C
      for (int r = 0; r < M; ++r)
        if (cudaMemsetAsync(C + (long long)r * ldc, 0, sizeof(float) * N, s) != cudaSuccess) {
          set_error("tensor-core GEMM: clearing C failed");
          return GL_ERR_CUDA;
        }
    }
    return launch_tc<32, true, false, false, false>(t, s);
  }
  return 1;
}

}  // namespace gl
