// Kernels of the learned MAP initialiser (a small CNN that maps an observed
// image to a Gaussian over the unconstrained parameters; it proposes the
// starting ensemble of ModellingSequence.MAP, whose `start` argument is the
// hook, gigalens/inference.py:34-57).
//
// Convolutions are im2col + GEMM.  The GEMM reads its weight operand as BF16
// (the stored precision of the network's weights) and accumulates in FP32;
// activations, gradients and the optimizer's master weights are FP32.
#include <cuda_bf16.h>

#include "gl_internal.cuh"

namespace gl {

// gl_cnn_tc.cu: the convolution GEMMs on the tensor cores (1: shape not handled)
int nn_gemm_tc(int transA, int transB, int a_bf16, int M, int N, int K, float alpha, const void* A, int lda,
               const float* B, int ldb, float* C, int ldc, int ksplit, cudaStream_t s);

// ------------------------------------------------------------------ GEMM
// C[b] = alpha * op(A[b]) op(B[b]) + beta * C[b];  op(A) is M x K, op(B) K x N,
// row-major storage; TA/TB select transposed storage.  A may be BF16.
constexpr int GT_K = 16;

// BM x BN output tile per CTA, 256 threads in a (BM/4) x (BN/4) grid, 4 x 4 outputs each.
// ksplit > 1 splits K over blockIdx.z (with the batch): partial products are
// added atomically into C, which the caller zeroes first (beta must be 0).
template <int BM, int BN, bool TA, bool TB, bool ABF16>
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, float alpha, const void* __restrict__ Av,
                                                   int lda, long long sA, const float* __restrict__ B, int ldb,
                                                   long long sB, float beta, float* __restrict__ C, int ldc,
                                                   long long sC, int ksplit) {
  static_assert((BM / 4) * (BN / 4) == 256, "tile must map onto 256 threads");
  __shared__ float As[GT_K][BM + 4];
  __shared__ float Bs[GT_K][BN + 4];
  const int bz = blockIdx.z / ksplit, kz = blockIdx.z - bz * ksplit;
  const int kchunk = ((K + ksplit - 1) / ksplit + GT_K - 1) / GT_K * GT_K;
  const int kbeg = kz * kchunk, kend = min(K, kbeg + kchunk);
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int tx = threadIdx.x % (BN / 4), ty = threadIdx.x / (BN / 4);
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  const float* Af = reinterpret_cast<const float*>(Av) + bz * sA;
  const __nv_bfloat16* Ah = reinterpret_cast<const __nv_bfloat16*>(Av) + bz * sA;
  const float* Bb = B + bz * sB;
  for (int k0 = kbeg; k0 < kend; k0 += GT_K) {
    for (int t = threadIdx.x; t < BM * GT_K; t += 256) {
      int m, k;
      if (TA) {            // A stored K x M: consecutive threads along m
        m = t % BM;
        k = t / BM;
      } else {             // A stored M x K: consecutive threads along k
        k = t % GT_K;
        m = t / GT_K;
      }
      const int gm = m0 + m, gk = k0 + k;
      float v = 0.f;
      if (gm < M && gk < kend) {
        const long long idx = TA ? (long long)gk * lda + gm : (long long)gm * lda + gk;
        v = ABF16 ? __bfloat162float(Ah[idx]) : Af[idx];
      }
      As[k][m] = v;
    }
    for (int t = threadIdx.x; t < BN * GT_K; t += 256) {
      int n, k;
      if (TB) {            // B stored N x K
        k = t % GT_K;
        n = t / GT_K;
      } else {             // B stored K x N
        n = t % BN;
        k = t / BN;
      }
      const int gn = n0 + n, gk = k0 + k;
      float v = 0.f;
      if (gn < N && gk < kend) v = TB ? Bb[(long long)gn * ldb + gk] : Bb[(long long)gk * ldb + gn];
      Bs[k][n] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < GT_K; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  float* Cb = C + bz * sC;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float* c = Cb + (long long)gm * ldc + gn;
      if (ksplit > 1) atomicAdd(c, alpha * acc[i][j]);
      else *c = alpha * acc[i][j] + (beta != 0.f ? beta * *c : 0.f);
    }
  }
}

// ------------------------------------------------------------------ im2col / col2im (3x3, pad 1)
// Channel-major activations X [C][B][H][W]; col [C*9][B][Ho*Wo] with
// col[c*9 + ky*3 + kx][b][oy*Wo + ox] = X[c][b][oy*s + ky - 1][ox*s + kx - 1].
__global__ void im2col3x3_kernel(const float* __restrict__ X, int B, int C, int H, int W, int s, int Ho,
                                 int Wo, float* __restrict__ col) {
  const long long total = (long long)C * 9 * B * Ho * Wo;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int ox = (int)(i % Wo);
    long long r = i / Wo;
    const int oy = (int)(r % Ho);
    r /= Ho;
    const int b = (int)(r % B);
    r /= B;
    const int k = (int)(r % 9);
    const int c = (int)(r / 9);
    const int iy = oy * s + k / 3 - 1, ix = ox * s + k % 3 - 1;
    col[i] = (iy >= 0 && iy < H && ix >= 0 && ix < W) ? X[(((long long)c * B + b) * H + iy) * W + ix] : 0.f;
  }
}

// dX[c][b][iy][ix] = sum of the dcol entries that read (iy, ix)
__global__ void col2im3x3_kernel(const float* __restrict__ dcol, int B, int C, int H, int W, int s, int Ho,
                                 int Wo, float* __restrict__ dX) {
  const long long total = (long long)C * B * H * W;
  const long long plane = (long long)B * Ho * Wo;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % W);
    long long r = i / W;
    const int iy = (int)(r % H);
    r /= H;
    const int b = (int)(r % B);
    const int c = (int)(r / B);
    float acc = 0.f;
    for (int ky = 0; ky < 3; ++ky) {
      const int ty = iy + 1 - ky;
      if (ty < 0 || ty % s) continue;
      const int oy = ty / s;
      if (oy >= Ho) continue;
      for (int kx = 0; kx < 3; ++kx) {
        const int tx = ix + 1 - kx;
        if (tx < 0 || tx % s) continue;
        const int ox = tx / s;
        if (ox >= Wo) continue;
        acc += dcol[((long long)c * 9 + ky * 3 + kx) * plane + (long long)b * Ho * Wo + oy * Wo + ox];
      }
    }
    dX[i] = acc;
  }
}

// [A][B][C] -> [B][A][C]
__global__ void permute01_kernel(const float* __restrict__ src, int A, int B, int C, float* __restrict__ dst) {
  const long long total = (long long)A * B * C;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    long long r = i / C;
    const int a = (int)(r % A);
    const int b = (int)(r / A);
    dst[i] = src[((long long)a * B + b) * C + c];
  }
}

// ------------------------------------------------------------------ bias + ReLU
// Y[b][c][p] += bias[c], then ReLU if relu; layout [B][C][P] (P = 1 for dense layers
// stored [B][C]).
__global__ void bias_act_kernel(float* __restrict__ Y, const float* __restrict__ bias, int B, int C, int P,
                                int relu) {
  const long long total = (long long)B * C * P;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)((i / P) % C);
    float v = Y[i] + bias[c];
    Y[i] = relu ? fmaxf(v, 0.f) : v;
  }
}

// dY *= (Y > 0) when relu; dbias[c] += sum over this block's slice of dY
// (grid: channels x slices; dbias zeroed by the launcher).
__global__ void bias_act_backward_kernel(float* __restrict__ dY, const float* __restrict__ Y, int B, int C, int P,
                                         int relu, float* __restrict__ dbias) {
  const int c = blockIdx.x;
  const long long n = (long long)B * P;
  const long long chunk = (n + gridDim.y - 1) / gridDim.y;
  const long long beg = blockIdx.y * chunk, end = min(n, beg + chunk);
  float acc = 0.f;
  for (long long t = beg + threadIdx.x; t < end; t += blockDim.x) {
    const int b = (int)(t / P), p = (int)(t % P);
    const long long i = ((long long)b * C + c) * P + p;
    float g = dY[i];
    if (relu && !(Y[i] > 0.f)) g = 0.f;
    dY[i] = g;
    acc += g;
  }
  __shared__ float red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float sum = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += red[w];
    atomicAdd(dbias + c, sum);
  }
}

// ------------------------------------------------------------------ Gaussian NLL head
// Feature-major layouts: out [2d][B] = (mu rows, log-sigma rows), target t [d][B].
// log_sigma = clamp(raw, -12, 12) (no gradient outside the clamp); per entry
// loss = log_sigma + 0.5 ((t - mu) / sigma)^2; dout = d(mean of loss)/d out.
__global__ void gauss_nll_kernel(const float* __restrict__ out, const float* __restrict__ t, int B, int d,
                                 float* __restrict__ loss, float* __restrict__ dout) {
  const long long total = (long long)B * d;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(i / B), b = (int)(i % B);
    const float mu = out[(long long)j * B + b];
    const float raw = out[(long long)(d + j) * B + b];
    const float ls = fminf(fmaxf(raw, -12.f), 12.f);
    const float inv = expf(-ls);
    const float r = (t[i] - mu) * inv;
    if (loss) loss[i] = ls + 0.5f * r * r;
    if (dout) {
      const float scale = 1.f / (float)total;
      dout[(long long)j * B + b] = -r * inv * scale;
      dout[(long long)(d + j) * B + b] = (raw >= -12.f && raw <= 12.f) ? (1.f - r * r) * scale : 0.f;
    }
  }
}

// dst [cols][rows] = src [rows][cols]^T
__global__ void transpose_kernel(const float* __restrict__ src, int rows, int cols, float* __restrict__ dst) {
  __shared__ float tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + j, c = bx + threadIdx.x;
    tile[j][threadIdx.x] = (r < rows && c < cols) ? src[(long long)r * cols + c] : 0.f;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = bx + j, r = by + threadIdx.x;
    if (c < cols && r < rows) dst[(long long)c * rows + r] = tile[threadIdx.x][j];
  }
}

__global__ void cast_bf16_kernel(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16_rn(src[i]);
}

static int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 16384) b = 16384;
  if (b < 1) b = 1;
  return (int)b;
}

static int launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s launch: %s", what, cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}

}  // namespace gl

using namespace gl;

extern "C" {

int gl_nn_gemm(int transA, int transB, int a_bf16, int M, int N, int K, float alpha, const void* A, int lda,
               long long strideA, const float* B, int ldb, long long strideB, float beta, float* C, int ldc,
               long long strideC, int batch, int ksplit, void* stream) {
  if (M < 0 || N < 0 || K < 0 || batch < 1 || ksplit < 1 || (ksplit > 1 && beta != 0.f) ||
      (M * N > 0 && (!A || !B || !C))) {
    set_error("gl_nn_gemm: bad arguments");
    return GL_ERR_INVALID;
  }
  if (M == 0 || N == 0) return GL_OK;
  if (ksplit > 1) {   // partial sums accumulate atomically into a zeroed C
    const bool dense = ldc == N && (batch == 1 || strideC == (long long)M * N);
    cudaError_t e = cudaSuccess;
    if (dense) {
      e = cudaMemsetAsync(C, 0, sizeof(float) * (size_t)M * N * batch, (cudaStream_t)stream);
    } else {
      for (int bz = 0; bz < batch && e == cudaSuccess; ++bz)
        for (int r = 0; r < M && e == cudaSuccess; ++r)
          e = cudaMemsetAsync(C + bz * strideC + (long long)r * ldc, 0, sizeof(float) * N, (cudaStream_t)stream);
    }
    if (e != cudaSuccess) {
      set_error("gl_nn_gemm: clearing C failed");
      return GL_ERR_CUDA;
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (batch == 1 && beta == 0.f) {   // the convolution shapes run on the tensor cores
    const int rc = nn_gemm_tc(transA, transB, a_bf16, M, N, K, alpha, A, lda, B, ldb, C, ldc, ksplit, s);
    if (rc != 1) return rc == GL_OK ? launch_check("tensor-core gemm") : rc;
  }
  const bool narrow = M <= 32;    // 32-channel layers: 32 x 128 tiles instead of 64 x 64
  dim3 grid(narrow ? (N + 127) / 128 : (N + 63) / 64, narrow ? (M + 31) / 32 : (M + 63) / 64, batch * ksplit);
#define GL_GEMM(TA, TB, BF)                                                                                    \
  do {                                                                                                         \
    if (narrow)                                                                                                \
      gemm_kernel<32, 128, TA, TB, BF><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, strideA, B, ldb, strideB,  \
                                                           beta, C, ldc, strideC, ksplit);                     \
    else                                                                                                       \
      gemm_kernel<64, 64, TA, TB, BF><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, strideA, B, ldb, strideB,   \
                                                          beta, C, ldc, strideC, ksplit);                      \
  } while (0)
  const int code = (transA ? 4 : 0) | (transB ? 2 : 0) | (a_bf16 ? 1 : 0);
  switch (code) {
    case 0: GL_GEMM(false, false, false); break;
    case 1: GL_GEMM(false, false, true); break;
    case 2: GL_GEMM(false, true, false); break;
    case 3: GL_GEMM(false, true, true); break;
    case 4: GL_GEMM(true, false, false); break;
    case 5: GL_GEMM(true, false, true); break;
    case 6: GL_GEMM(true, true, false); break;
    default: GL_GEMM(true, true, true); break;
  }
#undef GL_GEMM
  return launch_check("gemm");
}

int gl_nn_im2col3x3(const float* X, int B, int C, int H, int W, int stride, float* col, void* stream) {
  if (!X || !col || B < 1 || C < 1 || H < 1 || W < 1 || stride < 1) {
    set_error("gl_nn_im2col3x3: bad arguments");
    return GL_ERR_INVALID;
  }
  const int Ho = (H - 1) / stride + 1, Wo = (W - 1) / stride + 1;
  const long long n = (long long)C * 9 * B * Ho * Wo;
  im2col3x3_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(X, B, C, H, W, stride, Ho, Wo, col);
  return launch_check("im2col");
}

int gl_nn_col2im3x3(const float* dcol, int B, int C, int H, int W, int stride, float* dX, void* stream) {
  if (!dcol || !dX || B < 1 || C < 1 || H < 1 || W < 1 || stride < 1) {
    set_error("gl_nn_col2im3x3: bad arguments");
    return GL_ERR_INVALID;
  }
  const int Ho = (H - 1) / stride + 1, Wo = (W - 1) / stride + 1;
  const long long n = (long long)B * C * H * W;
  col2im3x3_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(dcol, B, C, H, W, stride, Ho, Wo, dX);
  return launch_check("col2im");
}

int gl_nn_bias_act(float* Y, const float* bias, int B, int C, int P, int relu, void* stream) {
  if (!Y || !bias || B < 1 || C < 1 || P < 1) {
    set_error("gl_nn_bias_act: bad arguments");
    return GL_ERR_INVALID;
  }
  bias_act_kernel<<<grid_for((long long)B * C * P), 256, 0, (cudaStream_t)stream>>>(Y, bias, B, C, P, relu);
  return launch_check("bias_act");
}

int gl_nn_bias_act_backward(float* dY, const float* Y, int B, int C, int P, int relu, float* dbias, void* stream) {
  if (!dY || !Y || !dbias || B < 1 || C < 1 || P < 1) {
    set_error("gl_nn_bias_act_backward: bad arguments");
    return GL_ERR_INVALID;
  }
  if (cudaMemsetAsync(dbias, 0, sizeof(float) * C, (cudaStream_t)stream) != cudaSuccess) {
    set_error("gl_nn_bias_act_backward: clearing dbias failed");
    return GL_ERR_CUDA;
  }
  long long n = (long long)B * P;
  int slices = (int)((n + 4095) / 4096);
  if (slices > 256) slices = 256;
  if (slices < 1) slices = 1;
  bias_act_backward_kernel<<<dim3(C, slices), 256, 0, (cudaStream_t)stream>>>(dY, Y, B, C, P, relu, dbias);
  return launch_check("bias_act_backward");
}

int gl_nn_gauss_nll(const float* out, const float* target, int B, int d, float* loss, float* dout, void* stream) {
  if (!out || !target || B < 1 || d < 1) {
    set_error("gl_nn_gauss_nll: bad arguments");
    return GL_ERR_INVALID;
  }
  gauss_nll_kernel<<<grid_for((long long)B * d), 256, 0, (cudaStream_t)stream>>>(out, target, B, d, loss, dout);
  return launch_check("gauss_nll");
}

int gl_nn_transpose(const float* src, int rows, int cols, float* dst, void* stream) {
  if (!src || !dst || rows < 1 || cols < 1) {
    set_error("gl_nn_transpose: bad arguments");
    return GL_ERR_INVALID;
  }
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  transpose_kernel<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(src, rows, cols, dst);
  return launch_check("transpose");
}

int gl_nn_permute01(const float* src, int A, int B, int C, float* dst, void* stream) {
  if (!src || !dst || A < 1 || B < 1 || C < 1) {
    set_error("gl_nn_permute01: bad arguments");
    return GL_ERR_INVALID;
  }
  permute01_kernel<<<grid_for((long long)A * B * C), 256, 0, (cudaStream_t)stream>>>(src, A, B, C, dst);
  return launch_check("permute01");
}

int gl_nn_cast_bf16(const float* src, void* dst, long long n, void* stream) {
  if (!src || !dst || n < 0) {
    set_error("gl_nn_cast_bf16: bad arguments");
    return GL_ERR_INVALID;
  }
  if (n == 0) return GL_OK;
  cast_bf16_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(src, (__nv_bfloat16*)dst, n);
  return launch_check("cast_bf16");
}

}  // extern "C"
