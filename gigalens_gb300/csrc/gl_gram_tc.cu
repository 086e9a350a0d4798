// Batched normal matrix G = A^T A of the least-squares path on the tensor
// cores (tcgen05), A = W X (basis stack X [D][P] of one sample, W = 1/err):
// the dense contraction of LensSimulator.lstsq_simulate
// (gigalens/tf/simulator.py:150-160, X^T W^2 X).
//
// One CTA per sample (persistent over the batch), 256 threads.  Pixels are
// consumed in chunks of 32: the threads load a chunk of A, split every value
// into a TF32 head and a TF32 tail (3xTF32: A^T A ~ hi^T hi + hi^T lo + lo^T
// hi, FP32-level accuracy), and store both into shared memory in the
// canonical K-major layout (8-row x 16-byte core matrices; the K stride of
// 144 bytes keeps the stores conflict-free).  One thread issues twelve
// tcgen05.mma.kind::tf32 (M = 128 rows of A, N = 64: the same tile's first 64
// rows act as B) into a TMEM accumulator and commits them to the stage's
// mbarrier; two stages overlap the fill of one chunk with the MMAs of the
// previous.  Every 32 chunks (1024 pixels) the accumulator is read back with
// tcgen05.ld and added into a float64 copy of G in shared memory, which keeps
// the accumulation error of long pixel sums out of G.  All mbarrier waits are
// bounded; a timeout sets *status, drains and frees TMEM, and the kernel
// returns.
#include <cstdint>

#include "gl_internal.cuh"
#include "gl_lstsq.cuh"
#include "gl_tc.cuh"

namespace gl {

namespace {
constexpr int kGT = 256;                   // threads
constexpr int kKC = 32;                    // pixels per chunk (K per stage)
constexpr int kM = 128, kN = 64;           // MMA shape; rows >= D are zero
constexpr uint32_t kLBO = 144;             // bytes between K-adjacent core matrices
constexpr uint32_t kSBO = kLBO * (kKC / 4);   // bytes between row groups (8 rows)
constexpr int kTileBytes = (kM / 8) * kSBO;   // one operand tile (hi or lo)
constexpr int kStageBytes = 2 * kTileBytes;   // hi + lo
constexpr int kSegChunks = 32;             // chunks per TMEM accumulation segment
constexpr uint32_t kTmemCols = 64;
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr int kG64Ld = kN + 1;              // float64 copy of G: padded rows (bank spread)
constexpr int kGramSmem = 1024 + 2 * kStageBytes + kN * kG64Ld * 8;
constexpr int kRowsPT = kN / (kGT / 32);   // rows of a chunk one thread loads (D <= 64)

__device__ __forceinline__ uint32_t elem_off(int row, int k) {
  return (uint32_t)(row >> 3) * kSBO + (uint32_t)(k >> 2) * kLBO + (uint32_t)(row & 7) * 16u +
         (uint32_t)(k & 3) * 4u;
}
}  // namespace

// Polls of the pipeline's mbarrier waits (0 = kWaitLimit).  Only the
// failure-detection test lowers it, to make those waits run out; the drain
// after a timeout always waits with kWaitLimit, so no MMA is in flight when
// the TMEM is freed.
static unsigned g_wait_polls_override = 0;

__global__ void __launch_bounds__(kGT) lsq_gram_tc_kernel(const __grid_constant__ LsqArgs a, float* G,
                                                          int* status, uint32_t wait_polls) {
  extern __shared__ __align__(1024) unsigned char gsm[];
  // layout: [0, 1024) control; stages; float64 G copy
  uint64_t* mbar = reinterpret_cast<uint64_t*>(gsm);          // 2 barriers
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gsm + 64);
  int* abort_flag = reinterpret_cast<int*>(gsm + 128);
  unsigned char* stages = gsm + 1024;
  double* G64 = reinterpret_cast<double*>(gsm + 1024 + 2 * kStageBytes);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int D = a.D;
  const uint32_t idesc = idesc_tf32(kM, kN);

  // zero both stages once: rows >= D stay zero for the whole kernel
  for (int i = tid; i < 2 * kStageBytes / 16; i += kGT)
    reinterpret_cast<float4*>(stages)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int i = tid; i < kN * kG64Ld; i += kGT) G64[i] = 0.0;
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 0) {
    tc_alloc(tmem_slot, kTmemCols);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  uint32_t gchunk = 0;      // chunks started by this CTA (stage = gchunk & 1)
  uint32_t committed = 0;   // chunks whose MMAs were committed
  bool failed = false;
  for (int b = blockIdx.x; b < a.bs && !failed; b += gridDim.x) {
    const int im = a.img_id ? a.img_id[b] : 0;
    if (im < 0 || im >= a.n_images) continue;
    const LsqImage& I = a.img[im];
    const int P = I.N * I.N;
    const float* Xb = a.X + (size_t)b * a.xstride;
    const int nchunks = (P + kKC - 1) / kKC;
    int seg_pos = 0;
    // a thread's values of the next chunk, loaded while the previous MMAs run
    float pre[kRowsPT];
    auto load_chunk = [&](int ch) {
      const int p = ch * kKC + lane;
      const float w = p < P ? 1.f / I.err[p] : 0.f;
#pragma unroll
      for (int k = 0; k < kRowsPT; ++k) {
        const int r = warp + k * (kGT / 32);
        pre[k] = (p < P && r < D) ? Xb[(size_t)r * I.xcstride + p] * w : 0.f;
      }
    };
    load_chunk(0);
    for (int ch = 0; ch < nchunks; ++ch, ++gchunk) {
      const int s = gchunk & 1;
      unsigned char* tile_hi = stages + s * kStageBytes;
      unsigned char* tile_lo = tile_hi + kTileBytes;
      // the stage's previous MMAs (chunk gchunk - 2) must be done before refilling
      if (gchunk >= 2) {
        const bool ok = mbar_wait(&mbar[s], ((gchunk - 2) >> 1) & 1u, wait_polls);
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
      }
      // fill: a warp covers one channel row, 32 consecutive pixels (coalesced)
#pragma unroll
      for (int k = 0; k < kRowsPT; ++k) {
        const int r = warp + k * (kGT / 32);
        if (r < D) {
          const float hi = to_tf32(pre[k]);
          const float lo = to_tf32(pre[k] - hi);
          const uint32_t off = elem_off(r, lane);
          *reinterpret_cast<float*>(tile_hi + off) = hi;
          *reinterpret_cast<float*>(tile_lo + off) = lo;
        }
      }
      if (ch + 1 < nchunks) load_chunk(ch + 1);
      fence_proxy_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t ahi = smem_u32(tile_hi), alo = smem_u32(tile_lo);
#pragma unroll
        for (int ks = 0; ks < kKC / 8; ++ks) {
          const uint32_t koff = (uint32_t)ks * 2u * kLBO;
          const uint64_t dhi = umma_desc_noswizzle(ahi + koff, kLBO, kSBO);
          const uint64_t dlo = umma_desc_noswizzle(alo + koff, kLBO, kSBO);
          const uint32_t acc0 = (seg_pos == 0 && ks == 0) ? 0u : 1u;
          tc_mma_tf32(tmem, dhi, dhi, idesc, acc0);
          tc_mma_tf32(tmem, dhi, dlo, idesc, 1u);
          tc_mma_tf32(tmem, dlo, dhi, idesc, 1u);
        }
        tc_commit(&mbar[s]);
      }
      committed = gchunk + 1;
      ++seg_pos;
      // end of a segment (or of the sample): add the accumulator into G64
      if (seg_pos == kSegChunks || ch == nchunks - 1) {
        const bool ok = mbar_wait(&mbar[s], (gchunk >> 1) & 1u, wait_polls);
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
        tc_fence_after();
        if (warp < 2) {
          const int row = warp * 32 + lane;   // TMEM lane = row of G
#pragma unroll
          for (int cb = 0; cb < kN / 16; ++cb) {
            float v[16];
            tc_ld_32x32b_x16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cb * 16), v);
            if (row < D) {
#pragma unroll
              for (int i = 0; i < 16; ++i) G64[row * kG64Ld + cb * 16 + i] += (double)v[i];
            }
          }
        }
        tc_fence_before();
        __syncthreads();
        seg_pos = 0;
      }
    }
    if (failed) break;
    // write G (float) and clear the float64 copy for the next sample
    for (int i = tid; i < D * D; i += kGT) {
      const int r = i / D, c = i - r * D;
      G[(size_t)b * D * D + i] = (float)G64[r * kG64Ld + c];
    }
    __syncthreads();
    for (int i = tid; i < kN * kG64Ld; i += kGT) G64[i] = 0.0;
    __syncthreads();
  }
  if (failed) {
    if (tid == 0) *status = 1;
    // drain: wait (bounded) for the last committed chunk of each stage
    for (uint32_t k = 0; k < 2 && committed > k; ++k) {
      const uint32_t last = committed - 1 - k;
      mbar_wait(&mbar[last & 1], (last >> 1) & 1u, kWaitLimit);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(tmem, kTmemCols);
}

int gram_tc_smem_bytes() { return kGramSmem; }

int launch_gram_tc(const LsqArgs& a, float* G, int* status, int grid, cudaStream_t stream) {
  static bool attr_set[kMaxDevices];   // per device
  const int dev = current_device_slot();
  if (!attr_set[dev]) {
    cudaError_t e = cudaFuncSetAttribute(lsq_gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kGramSmem);
    if (e != cudaSuccess) {
      set_error("Gram kernel shared memory attribute: %s", cudaGetErrorString(e));
      return GL_ERR_CUDA;
    }
    attr_set[dev] = true;
  }
  const uint32_t polls = g_wait_polls_override ? g_wait_polls_override - 1u : kWaitLimit;
  lsq_gram_tc_kernel<<<grid, kGT, kGramSmem, stream>>>(a, G, status, polls);
  return GL_OK;
}

void set_gram_wait_polls(int polls) { g_wait_polls_override = polls < 0 ? 0u : (unsigned)polls + 1u; }

}  // namespace gl
