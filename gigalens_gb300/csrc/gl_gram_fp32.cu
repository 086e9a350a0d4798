// Batched normal equations of the least-squares path on the FP32 pipes:
// G = A^T A and h = A^T b with A = W X (basis stack X [D][P] of one sample,
// W = 1/err) and b = W y, the dense contraction of
// LensSimulator.lstsq_simulate (gigalens/tf/simulator.py:150-160,
// X^T W^2 X and X^T W^2 y).  The same sums as lsq_gram_tc_kernel; this
// variant keeps them in registers instead of TMEM.
//
// The contraction is tall and thin: R = D + 1 <= 64 rows (the channels plus
// b) against 10^3..10^4 pixels per sample, so its arithmetic (R^2 / 2 FMAs a
// pixel) is small next to the stream of X, and a register-tiled SIMT kernel
// has no per-chunk hand-off to one MMA-issuing thread.
//
// One CTA per SM (persistent over the batch), 256 threads.  The R rows are
// padded to RP = 8 nT and cut into nT interleaved row sets {t + nT r : r < 8};
// a thread owns one 8 x 8 tile (ti <= tj) of G's upper block triangle, and
// the threads of one tile set ("group") take disjoint pixel ranges of every
// chunk.  Chunks of C pixels stream through a ring of shared-memory slots
// (cp.async).  A copying thread keeps one pixel quad of the chunk and takes
// every (256 / (C/4))-th row of it, so the pieces it copies share one quad of
// W: it copies that quad into its own 16 bytes of the slot in the same group
// and weights its pieces once they land, with no barrier and no global load
// on the way.  A chunk row has a pitch of an odd number of 16-byte units, so
// the 16-byte loads of the eight rows t + nT r (fixed r, consecutive t) hit
// distinct bank groups.  At
// the end of a sample the groups' partial sums are added in a fixed order
// (bitwise reproducible) and written as G (symmetric, D x D) and h.
#include <cstdint>

#include "gl_cpasync.cuh"
#include "gl_internal.cuh"
#include "gl_lstsq.cuh"

namespace gl {

namespace {
constexpr int kFT = 256;                 // threads
constexpr int kFRmax = 64;               // rows (D + 1) at most
constexpr int kFSmemLimit = 227 * 1024;
constexpr int kFMaxRing = 3;             // ring slots (two chunks in flight)

// The launch shape for NT row sets (R = D + 1 <= 8 NT); compile-time, so
// every shared-memory offset of the inner loops is an immediate.
template <int NT>
struct GShape {
  static constexpr int RP = 8 * NT;
  static constexpr int tiles = NT * (NT + 1) / 2;
  static constexpr int groups = kFT / tiles;
  static constexpr int m0 = (64 + groups / 2) / groups;   // quads per group and chunk: ~64 quads a chunk
  static constexpr int m = m0 < 1 ? 1 : m0;
  static constexpr int C = 4 * groups * m;
  static constexpr int cq = C / 4;                        // 16-byte pieces (pixel quads) per chunk row
  static constexpr int pitch = C + ((cq & 1) ? 0 : 4);
  static constexpr int slot_floats = RP * pitch + 4 * kFT;   // the rows, then each thread's W quad
  static constexpr int red_floats = groups * 64 * tiles;
  static constexpr int d0 = (kFSmemLimit / 4 - red_floats) / slot_floats;
  static constexpr int depth = d0 > kFMaxRing ? kFMaxRing : d0;
  static constexpr int nrs = kFT / cq;                    // rows a pass of the copying threads covers
  static constexpr int smem_bytes = (depth * slot_floats + red_floats) * 4;
  static_assert(depth >= 2 && smem_bytes <= kFSmemLimit, "Gram shape does not fit");
};

// tile k of the upper block triangle -> (ti, tj), ti <= tj
__device__ __forceinline__ void tile_rows(int nT, int k, int& ti, int& tj) {
  ti = 0;
  while (k >= nT - ti) {
    k -= nT - ti;
    ++ti;
  }
  tj = ti + k;
}
}  // namespace

template <int NT>
__global__ void __launch_bounds__(kFT, 1) lsq_gram_fp32_kernel(const __grid_constant__ LsqArgs a, float* G,
                                                               float* h) {
  using S = GShape<NT>;
  extern __shared__ __align__(16) float fsm[];
  const int D = a.D, R = D + 1;
  float* ring = fsm;
  float* red = fsm + S::depth * S::slot_floats;
  const int tid = threadIdx.x;
  const bool copier = tid < S::nrs * S::cq;
  const int cq_t = tid % S::cq, r_t = tid / S::cq;   // this thread's quad and first row

  // rows R..RP-1 of every slot are read as zeros and never copied into
  for (int i = tid; i < S::depth * S::slot_floats; i += kFT) ring[i] = 0.f;
  __syncthreads();

  const bool active = tid < S::groups * S::tiles;
  const int grp = active ? tid / S::tiles : 0;
  const int tile = active ? tid - grp * S::tiles : 0;
  int ti, tj;
  tile_rows(NT, tile, ti, tj);

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
      float* dst = ring + slot * S::slot_floats + 4 * cq_t;
      if (copier) {
        const int p = pch * S::C + 4 * cq_t;
        const int left = P - p;
        const uint32_t bytes = left >= 4 ? 16u : (left > 0 ? 4u * left : 0u);
        const float* row = Xb + (size_t)r_t * I.xcstride + (bytes ? p : 0);
        const size_t rstep = (size_t)S::nrs * I.xcstride;
        int r = r_t;
        for (; r < D; r += S::nrs, row += rstep) cp_async16(dst + r * S::pitch, row, bytes);
        if (r == D) cp_async16(dst + D * S::pitch, I.bw + (bytes ? p : 0), bytes);
        // W is zero-padded to a multiple of 4 floats past the image
        cp_async16(ring + slot * S::slot_floats + S::RP * S::pitch + 4 * tid, left > 0 ? I.W + p : I.W,
                   left > 0 ? 16u : 0u);
      }
      if (++pch == (P + S::C - 1) / S::C) {
        pb = next_sample(pb);
        pch = 0;
      }
    }
    cp_async_commit();   // possibly empty: one group per chunk
  };
  for (int s = 0; s < S::depth - 1; ++s) issue(s);

  uint32_t gchunk = 0;   // chunks consumed by this CTA
  for (int b = first; b < a.bs; b = next_sample(b)) {
    const LsqImage& I = a.img[a.img_id ? a.img_id[b] : 0];
    const int P = I.N * I.N;
    const int nchunks = (P + S::C - 1) / S::C;
    // (even pixels, odd pixels) partial sums of the tile's 64 entries
    float2 acc[8][8];
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
      for (int s = 0; s < 8; ++s) acc[r][s] = make_float2(0.f, 0.f);

    for (int ch = 0; ch < nchunks; ++ch, ++gchunk) {
      const int slot = gchunk % S::depth;
      // this thread's pieces of chunk gchunk have landed (the depth - 2
      // chunks issued after it may still be in flight)
      if constexpr (S::depth >= 3)
        cp_async_wait<1>();
      else
        cp_async_wait<0>();
      float* src = ring + slot * S::slot_floats;
      const int p0 = ch * S::C;
      // weight the basis rows of this thread's own pieces (b arrives weighted)
      if (copier && p0 + 4 * cq_t < P) {
        const float4 w = *reinterpret_cast<const float4*>(src + S::RP * S::pitch + 4 * tid);
        float* v = src + r_t * S::pitch + 4 * cq_t;
#pragma unroll 4
        for (int r = r_t; r < D; r += S::nrs, v += S::nrs * S::pitch) {
          float4 x = *reinterpret_cast<float4*>(v);
          x.x *= w.x;
          x.y *= w.y;
          x.z *= w.z;
          x.w *= w.w;
          *reinterpret_cast<float4*>(v) = x;
        }
      }
      __syncthreads();   // chunk gchunk complete; every thread is done with chunk gchunk - 1
      issue((gchunk + S::depth - 1) % S::depth);   // into the slot of chunk gchunk - 1
      if (active) {
        const int nq = min(S::cq, (P - p0 + 3) >> 2);   // quads of the chunk inside the image
        const int q0 = grp * S::m;
        const int qn = min(S::m, nq - q0);
        const float* pi = src + 4 * q0 + ti * S::pitch;
        const float* pj = src + 4 * q0 + tj * S::pitch;
#pragma unroll 1
        for (int k = 0; k < qn; ++k, pi += 4, pj += 4) {
          float4 xi[8];
#pragma unroll
          for (int r = 0; r < 8; ++r) xi[r] = *reinterpret_cast<const float4*>(pi + r * NT * S::pitch);
#pragma unroll
          for (int s = 0; s < 8; ++s) {
            const float4 xj = *reinterpret_cast<const float4*>(pj + s * NT * S::pitch);
            const float2 j01 = make_float2(xj.x, xj.y), j23 = make_float2(xj.z, xj.w);
            // pixels 0-1 of the quad into the column's eight accumulators, then
            // pixels 2-3: eight independent FFMA2 between dependent ones
#pragma unroll
            for (int r = 0; r < 8; ++r) acc[r][s] = __ffma2_rn(make_float2(xi[r].x, xi[r].y), j01, acc[r][s]);
#pragma unroll
            for (int r = 0; r < 8; ++r) acc[r][s] = __ffma2_rn(make_float2(xi[r].z, xi[r].w), j23, acc[r][s]);
          }
        }
      }
    }

    // the groups' partial sums, added in group order
    if (active) {
#pragma unroll
      for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int s = 0; s < 8; ++s) red[(grp * 64 + r * 8 + s) * S::tiles + tile] = acc[r][s].x + acc[r][s].y;
    }
    __syncthreads();
    for (int o = tid; o < S::tiles * 64; o += kFT) {
      const int t = o >> 6, e = o & 63;
      float v = 0.f;
#pragma unroll 4
      for (int g = 0; g < S::groups; ++g) v += red[(g * 64 + e) * S::tiles + t];
      int oi, oj;
      tile_rows(NT, t, oi, oj);
      const int i = oi + NT * (e >> 3), j = oj + NT * (e & 7);
      if (i >= R || j >= R || (oi == oj && i > j)) continue;   // padding, or a diagonal tile's mirror
      if (i < D && j < D) {
        G[(size_t)b * D * D + (size_t)i * D + j] = v;
        G[(size_t)b * D * D + (size_t)j * D + i] = v;
      } else if (i == D && j < D) {
        h[(size_t)b * D + j] = v;
      } else if (j == D && i < D) {
        h[(size_t)b * D + i] = v;
      }
    }
    // the next write of `red` follows at least one chunk barrier
  }
  cp_async_wait<0>();
}

template <int NT>
static int launch_nt(const LsqArgs& a, float* G, float* h, int grid, cudaStream_t stream) {
  static int attr_set[kMaxDevices];   // per device
  const int dev = current_device_slot();
  constexpr int smem = GShape<NT>::smem_bytes;
  if (!attr_set[dev]) {
    cudaError_t e = cudaFuncSetAttribute(lsq_gram_fp32_kernel<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) {
      set_error("Gram kernel shared memory attribute: %s", cudaGetErrorString(e));
      return GL_ERR_CUDA;
    }
    attr_set[dev] = 1;
  }
  lsq_gram_fp32_kernel<NT><<<grid, kFT, smem, stream>>>(a, G, h);
  return GL_OK;
}

int launch_gram_fp32(const LsqArgs& a, float* G, float* h, int grid, cudaStream_t stream) {
  switch ((a.D + 8) / 8) {   // NT = ceil((D + 1) / 8)
    case 1: return launch_nt<1>(a, G, h, grid, stream);
    case 2: return launch_nt<2>(a, G, h, grid, stream);
    case 3: return launch_nt<3>(a, G, h, grid, stream);
    case 4: return launch_nt<4>(a, G, h, grid, stream);
    case 5: return launch_nt<5>(a, G, h, grid, stream);
    case 6: return launch_nt<6>(a, G, h, grid, stream);
    case 7: return launch_nt<7>(a, G, h, grid, stream);
    case 8: return launch_nt<8>(a, G, h, grid, stream);
    default:
      set_error("Gram kernel: %d channels, at most %d", a.D, kFRmax - 1);
      return GL_ERR_UNSUPPORTED;
  }
}

}  // namespace gl
