// Batched normal equations of the least-squares path on the tensor cores
// (tcgen05): G = A^T A and h = A^T b with A = W X (basis stack X [D][P] of one
// sample, W = 1/err) and b = W y, the dense contraction of
// LensSimulator.lstsq_simulate (gigalens/tf/simulator.py:150-160,
// X^T W^2 X and X^T W^2 y).
//
// One CTA per SM (persistent over the batch), 256 threads.  The rows of the
// contraction are the D basis channels plus b (R = D + 1 <= 64).  Pixels are
// streamed from HBM in chunks of 64 through a ring of chunks in shared memory
// (cp.async; each thread copies and later converts the same 16-byte pieces,
// with its own copy of their weights, so it only waits for its own copy
// groups; up to seven chunks of copies in flight per SM hide the HBM
// latency).  A chunk is weighted, split into
// TF32 head and tail (3xTF32: a_i a_j ~ hi_i hi_j + hi_i lo_j + lo_i hi_j,
// FP32-level accuracy) and stored in the canonical K-major layout (8-row x
// 16-byte core matrices; a K stride of 144 bytes keeps the 16-byte stores
// conflict-free) as ONE 128-row operand: rows 0-63 hold the heads, rows 64-127
// the tails.  With the heads as the B operand (N = R rounded up to 16), one
// tcgen05.mma.kind::tf32 (M = 128, K = 8) gives HH = hi hi^T in TMEM lanes
// 0-63 and LH = lo hi^T in lanes 64-127, and G = HH + LH + LH^T.  Two operand
// stages keep one chunk's MMAs in flight while the next is filled.
// Every 1024 pixels the accumulation switches between two TMEM accumulators;
// the finished one is read back (tcgen05.ld) one segment later, when its MMAs
// are long complete, and added into float-float (TwoSum) sums of the lower
// triangle in shared memory, which keep the accumulation error of long pixel
// sums out of G without float64 arithmetic.  All mbarrier waits are bounded; a
// timeout sets *status, drains and frees TMEM, and the kernel returns.
#include <cstdint>

#include "gl_cpasync.cuh"
#include "gl_internal.cuh"
#include "gl_lstsq.cuh"
#include "gl_tc.cuh"

namespace gl {

namespace {
constexpr int kGT = 256;                   // threads
constexpr int kKC = 64;                    // pixels per chunk (K per operand stage)
constexpr int kQ = kKC / 4;                // 16-byte pieces per row of a chunk
constexpr int kM = 128;                    // MMA rows: heads 0..63, tails 64..127
constexpr int kRmax = 64;
constexpr uint32_t kLBO = 144;             // bytes between K-adjacent core matrices
constexpr uint32_t kSBO = kLBO * kQ;       // bytes between row groups (8 rows)
constexpr int kTileBytes = (kM / 8) * kSBO;   // one operand stage
constexpr int kStages = 2;                 // operand stages (the MMAs of one chunk take ~200 cycles)
constexpr int kRowBytes = kKC * 4;         // one row of a raw chunk
constexpr int kSegChunks = 16;             // chunks per TMEM accumulation segment (1024 px)
constexpr uint32_t kTmemCols = 128;        // two accumulators of 64 columns
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr int kCtrlBytes = 1024;
constexpr int kMaxRing = 8, kMinRing = 2;   // ring slots: up to 7 chunks in flight per SM
constexpr int kSmemLimit = 227 * 1024;

__host__ __device__ constexpr int tri_entries(int R) { return R * (R + 1) / 2; }
__host__ __device__ constexpr int fixed_bytes(int R) {
  return kCtrlBytes + kStages * kTileBytes + 2 * tri_entries(R) * 8;
}
// A ring slot: the chunk's R rows, then each thread's own copy of the 16 bytes
// of W for its pixel quad (every piece a thread converts lies in quad tid % kQ).
__host__ __device__ constexpr int slot_bytes(int R) { return R * kRowBytes + kGT * 16; }
__host__ __device__ constexpr int ring_depth(int R) {
  const int d = (kSmemLimit - fixed_bytes(R)) / slot_bytes(R);
  return d > kMaxRing ? kMaxRing : d;
}
__host__ __device__ constexpr int gram_smem_bytes(int R) { return fixed_bytes(R) + ring_depth(R) * slot_bytes(R); }

__device__ __forceinline__ uint32_t head_off(int row, int quad) {
  return (uint32_t)(row >> 3) * kSBO + (uint32_t)quad * kLBO + (uint32_t)(row & 7) * 16u;
}
__device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }   // i >= j

__device__ __forceinline__ void cp_wait_ring(int depth) {
  // at most depth - 1 groups still in flight
  switch (depth) {
    case 2: cp_async_wait<1>(); break;
    case 3: cp_async_wait<2>(); break;
    case 4: cp_async_wait<3>(); break;
    case 5: cp_async_wait<4>(); break;
    case 6: cp_async_wait<5>(); break;
    case 7: cp_async_wait<6>(); break;
    default: cp_async_wait<7>(); break;
  }
}

// A finished accumulation segment whose read-back is still due.
struct PendingSeg {
  int valid;
  int acc;          // TMEM accumulator (0 or 1)
  uint32_t glast;   // its last chunk (operand stage glast % kStages)
  int buf;          // float-float sums buffer (sample parity)
  int finish;       // the sample's last segment: write G and h afterwards
  int b;            // the sample
};
}  // namespace

// Polls of the pipeline's mbarrier waits (0 = kWaitLimit).  Only the
// failure-detection test lowers it, to make those waits run out; the drain
// after a timeout always waits with kWaitLimit, so no MMA is in flight when
// the TMEM is freed.
static unsigned g_wait_polls_override = 0;

__global__ void __launch_bounds__(kGT, 1) lsq_gram_tc_kernel(const __grid_constant__ LsqArgs a, float* G,
                                                             float* h, int* status, uint32_t wait_polls) {
  extern __shared__ __align__(1024) unsigned char gsm[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(gsm);          // kStages barriers
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gsm + 128);
  const int D = a.D, R = D + 1;
  const int NB = (R + 15) & ~15;   // B rows (MMA N)
  const int depth = ring_depth(R);
  unsigned char* stages = gsm + kCtrlBytes;
  float2* sums = reinterpret_cast<float2*>(stages + kStages * kTileBytes);   // [2][tri]
  unsigned char* ring = reinterpret_cast<unsigned char*>(sums + 2 * tri_entries(R));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t idesc = idesc_tf32(kM, NB);
  const int items = R * kQ;   // 16-byte pieces of a chunk (<= 1024: four per thread)
  const int ntri = tri_entries(R);

  for (int i = tid; i < kStages * kTileBytes / 16; i += kGT)
    reinterpret_cast<float4*>(stages)[i] = make_float4(0.f, 0.f, 0.f, 0.f);   // rows >= R stay zero
  for (int i = tid; i < 2 * ntri; i += kGT) sums[i] = make_float2(0.f, 0.f);
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&mbar[s], 1);
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

  // producer cursor: the next chunk to copy (sample pb, chunk pch)
  int pb = first, pch = 0;
  auto issue = [&](int slot) {
    if (pb < a.bs) {
      const LsqImage& I = a.img[a.img_id ? a.img_id[pb] : 0];
      const int P = I.N * I.N;
      const float* Xb = a.X + (size_t)pb * a.xstride;
      const int p0 = pch * kKC;
      unsigned char* dst = ring + slot * slot_bytes(R);
      for (int it = tid; it < items; it += kGT) {
        const int r = it / kQ, q = it - r * kQ;
        const int p = p0 + 4 * q;
        const float* row = r < D ? Xb + (size_t)r * I.xcstride : I.bw;
        const int left = P - p;
        const uint32_t bytes = left >= 4 ? 16u : (left > 0 ? 4u * left : 0u);
        cp_async16(dst + r * kRowBytes + q * 16, bytes ? row + p : row, bytes);
      }
      // W of this thread's quad (zero-padded past the image: always 16 bytes)
      cp_async16(dst + R * kRowBytes + tid * 16, I.W + p0 + 4 * (tid % kQ), 16u);
      if (++pch == (P + kKC - 1) / kKC) {
        pb = next_sample(pb);
        pch = 0;
      }
    }
    cp_async_commit();   // possibly empty: one group per ring slot
  };
  for (int s = 0; s < depth - 1; ++s) issue(s);

  bool failed = false;
  PendingSeg pend[2] = {{0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0}};
  // Read back a finished segment and add HH + LH + LH^T into the lower
  // triangle of its sums; `gnow` = chunks consumed so far.  Its MMAs are
  // complete once the fill of chunk glast + kStages waited for them;
  // otherwise wait here (its stage has not been refilled since).
  auto run_epilogue = [&](PendingSeg& ps, uint32_t gnow) -> bool {
    if (!ps.valid) return true;
    ps.valid = 0;
    if (gnow < ps.glast + 1 + kStages) {
      const bool ok = mbar_wait(&mbar[ps.glast % kStages], (ps.glast / kStages) & 1u, wait_polls);
      if (__syncthreads_or(!ok)) return false;
    }
    tc_fence_after();
    float v[kRmax];
    const int row = (warp & 1) * 32 + lane;   // row of HH (warps 0, 1) or LH (warps 2, 3)
    if (warp < 4) {
      const uint32_t base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(ps.acc * 64);
#pragma unroll
      for (int cb = 0; cb < kRmax / 16; ++cb) {
        if (cb * 16 < NB) {
          float t[16];
          tc_ld_32x32b_x16(base + (uint32_t)(cb * 16), t);
#pragma unroll
          for (int i = 0; i < 16; ++i) v[cb * 16 + i] = t[i];
        }
      }
    }
    float2* S = sums + ps.buf * ntri;
    // HH (symmetric; warps 0, 1), then LH (warps 2, 3), on and below the
    // diagonal of row `row`; the two touch the same entries, so in turn
    for (int part = 0; part < 2; ++part) {
      if ((warp >> 1) == part && warp < 4 && row < R) {
#pragma unroll
        for (int j = 0; j < kRmax; ++j)
          if (j <= row) {
            float2& e = S[tri(row, j)];
            ff_add(e.x, e.y, v[j]);
          }
      }
      __syncthreads();
    }
    if (warp >= 2 && warp < 4 && row < R) {   // LH^T: element (j, row) for j >= row
#pragma unroll
      for (int j = 0; j < kRmax; ++j)
        if (j >= row && j < R) {
          float2& e = S[tri(j, row)];
          ff_add(e.x, e.y, v[j]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (ps.finish) {   // the sample's sums are complete: write G (symmetric) and h, clear
      const int b = ps.b;
      for (int i = tid; i < D * D; i += kGT) {
        const int r = i / D, c = i - r * D;
        const float2 e = r >= c ? S[tri(r, c)] : S[tri(c, r)];
        G[(size_t)b * D * D + i] = e.x + e.y;
      }
      for (int i = tid; i < D; i += kGT) {
        const float2 e = S[tri(D, i)];
        h[(size_t)b * D + i] = e.x + e.y;
      }
      __syncthreads();
      for (int i = tid; i < ntri; i += kGT) S[i] = make_float2(0.f, 0.f);
      __syncthreads();
    }
    return true;
  };

  uint32_t gchunk = 0;      // chunks consumed by this CTA
  uint32_t segs = 0;        // segments started by this CTA (accumulator = segs & 1)
  uint32_t committed = 0;   // chunks whose MMAs were committed
  int sample_idx = 0;
  for (int b = first; b < a.bs && !failed; b = next_sample(b), ++sample_idx) {
    const LsqImage& I = a.img[a.img_id ? a.img_id[b] : 0];
    const int P = I.N * I.N;
    const int nchunks = (P + kKC - 1) / kKC;
    int seg_pos = 0;
    for (int ch = 0; ch < nchunks; ++ch, ++gchunk) {
      const int s = gchunk % kStages;
      const int slot = gchunk % depth;
      issue((gchunk + depth - 1) % depth);   // the slot this thread emptied last iteration
      cp_wait_ring(depth);                   // this thread's pieces of chunk gchunk landed
      unsigned char* tile = stages + s * kTileBytes;
      // a new segment reuses an accumulator: read back its previous segment first
      if (seg_pos == 0 && !run_epilogue(pend[segs & 1], gchunk)) {
        failed = true;
        break;
      }
      // the stage's previous MMAs (chunk gchunk - kStages) must be done before
      // refilling; each thread waits for itself, the barrier after the fill
      // then agrees on any timeout
      bool ok = true;
      if (gchunk >= kStages) ok = mbar_wait(&mbar[s], ((gchunk - kStages) / kStages) & 1u, wait_polls);
      // weight, split and store this thread's own pieces
      const unsigned char* src = ring + slot * slot_bytes(R);
      const float4 w = *reinterpret_cast<const float4*>(src + R * kRowBytes + tid * 16);
      for (int it = tid; it < items && ok; it += kGT) {
        const int r = it / kQ, q = it - r * kQ;
        float4 v = *reinterpret_cast<const float4*>(src + r * kRowBytes + q * 16);
        if (r < D) {
          v.x *= w.x;
          v.y *= w.y;
          v.z *= w.z;
          v.w *= w.w;
        }
        float4 hi, lo;
        hi.x = to_tf32(v.x);
        hi.y = to_tf32(v.y);
        hi.z = to_tf32(v.z);
        hi.w = to_tf32(v.w);
        lo.x = to_tf32(v.x - hi.x);
        lo.y = to_tf32(v.y - hi.y);
        lo.z = to_tf32(v.z - hi.z);
        lo.w = to_tf32(v.w - hi.w);
        const uint32_t off = head_off(r, q);
        *reinterpret_cast<float4*>(tile + off) = hi;
        *reinterpret_cast<float4*>(tile + off + 8 * kSBO) = lo;   // row r + 64
      }
      fence_proxy_async_smem();
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      const int acc = segs & 1;
      if (tid == 0) {
        tc_fence_after();
        const uint32_t base = smem_u32(tile);
#pragma unroll
        for (int ks = 0; ks < kKC / 8; ++ks) {
          const uint64_t d = umma_desc_noswizzle(base + (uint32_t)ks * 2u * kLBO, kLBO, kSBO);
          tc_mma_tf32(tmem + (uint32_t)(acc * 64), d, d, idesc, (seg_pos == 0 && ks == 0) ? 0u : 1u);
        }
        tc_commit(&mbar[s]);
      }
      committed = gchunk + 1;
      if (++seg_pos == kSegChunks || ch == nchunks - 1) {
        pend[acc] = PendingSeg{1, acc, gchunk, sample_idx & 1, ch == nchunks - 1, b};
        ++segs;
        seg_pos = 0;
      }
    }
  }
  // the last two segments' read-backs
  for (int k = 0; k < 2 && !failed; ++k)
    if (!run_epilogue(pend[(segs + k) & 1], gchunk)) failed = true;
  cp_async_wait<0>();
  if (failed) {
    if (tid == 0) *status = 1;
    // drain: wait (bounded) for the last committed chunk of every stage
    for (uint32_t k = 0; k < (uint32_t)kStages && committed > k; ++k) {
      const uint32_t last = committed - 1 - k;
      mbar_wait(&mbar[last % kStages], (last / kStages) & 1u, kWaitLimit);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(tmem, kTmemCols);
}

int gram_tc_ctas_per_sm(int) { return 1; }

int launch_gram_tc(const LsqArgs& a, float* G, float* h, int* status, int grid, cudaStream_t stream) {
  static int attr_set[kMaxDevices];   // per device: the largest size set so far
  const int dev = current_device_slot();
  const int R = a.D + 1;
  if (R > kRmax || ring_depth(R) < kMinRing) {
    set_error("Gram kernel: %d channels, at most %d", a.D, kRmax - 1);
    return GL_ERR_UNSUPPORTED;
  }
  const int smem = gram_smem_bytes(R);
  if (smem > attr_set[dev]) {
    cudaError_t e = cudaFuncSetAttribute(lsq_gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) {
      set_error("Gram kernel shared memory attribute: %s", cudaGetErrorString(e));
      return GL_ERR_CUDA;
    }
    attr_set[dev] = smem;
  }
  const uint32_t polls = g_wait_polls_override ? g_wait_polls_override - 1u : kWaitLimit;
  lsq_gram_tc_kernel<<<grid, kGT, smem, stream>>>(a, G, h, status, polls);
  return GL_OK;
}

void set_gram_wait_polls(int polls) { g_wait_polls_override = polls < 0 ? 0u : (unsigned)polls + 1u; }

}  // namespace gl
