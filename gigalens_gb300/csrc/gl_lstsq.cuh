// Structures of the linear-amplitude (least-squares) path; see gl_lstsq.cu.
#pragma once
#include <cstddef>
#include <vector>

#include "gl_internal.cuh"

namespace gl {

constexpr int kMaxLsqChannels = 63;   // basis images per sample (shapelets n_max <= 9 + lens light);
                                      // with the data row b the normal equations have <= 64 rows
constexpr int kMaxLsqProfiles = 4;

struct LsqChannel {
  int kind;    // 0: unit-amplitude Sersic, 1: shapelet basis function
  int prof;    // light-profile slot
  int n1, n2;  // shapelet orders
};

struct LsqProfile {
  int type, group;
  int interp;   // shapelets: tabulated functions (interpolate=True)
  int col[GL_MAX_PROFILE_PARAMS];  // SHAPELETS: beta, cx, cy; Sersic: SERSIC_ELLIPSE slots
};

struct LsqImage {
  int N, ss, nplanes, KS, ksp;
  int d[kMaxPlanes], padI[kMaxPlanes];
  int pitch;          // plane row pitch in floats (a multiple of 4 with pitch / 4 odd)
  int CB;             // output columns per correlation unit (16 or 20)
  int ncbC;           // column blocks of CB columns
  int Bo;             // output rows per band (N: the whole image in one band)
  int CPn;            // channels per pass
  int R0;             // max_p d[p]: shared-memory row 0 holds plane row i0 - R0
  int brows;          // plane rows held per band: Bo + KS + R0 - min_p d[p]
  int nbands;
  int cpass;          // number of channels (D)
  int xcstride;       // floats between channels in X (N*N rounded up to a multiple of 4)
  int plane_floats;   // brows * pitch
  int offK, smem_floats;
  const float* grid;
  const float* kern;
  const float* obs;
  const float* err;
  const float* W;     // 1 / err, zero-padded to a multiple of kPixPad floats
  const float* bw;    // b = W * obs, zero-padded likewise
};

constexpr int kPixPad = 256;   // pixel padding of W and bw (the streaming kernels' chunk)

struct LsqArgs {
  int bs, d, D, n_images, n_prof, has_shear;
  int maxP, max_bands;
  size_t xstride;   // floats per sample in X
  float2* beta;         // ray-traced source-plane coordinates, one slice per CTA
  size_t beta_stride;   // float2 per slice
  const float* shp_tab; // shapelet table (interpolating shapelet profiles), or null
  int gfac_prof;        // source shapelet profile whose Gaussian the ray-trace pass stores after
                        // beta in each slice (floats, same pixel order), or -1
  LsqProfile prof[kMaxLsqProfiles];
  LsqChannel ch[kMaxLsqChannels];
  DevProfile epl, shear;
  LsqImage img[GL_MAX_IMAGES];
  const float* x;
  const int* img_id;
  float* X;
};

struct LsqPlan {
  int D, n_prof, has_shear, maxP, max_bands, smem_bytes;
  int maxXc;            // largest per-channel stride of X (floats)
  int n_sm;             // CTAs of the basis kernel at most (ctas_per_sm per SM)
  int nt, ctas_per_sm;  // basis kernel: threads per CTA (512 or 256) and CTAs per SM
  int col_block;        // forced correlation column block (0: planner's choice)
  int gram;             // Gram kernel: 1 tensor cores (3xTF32), 2 FP32 register tiles
  size_t beta_per_cta;  // float2 of the largest band's ray-traced coordinates (and Gaussian factors)
  int gfac_prof;        // see LsqArgs
  LsqProfile prof[kMaxLsqProfiles];
  LsqChannel ch[kMaxLsqChannels];
  DevProfile epl, shear;
  LsqImage img[GL_MAX_IMAGES];
  float* dev_err;
};

int lsq_prepare(gl_plan* plan, std::vector<std::vector<float>>& errs);
int lsq_plan_layout(LsqPlan* L, const gl_plan* plan, int ctas_per_sm, int col_block);
// tensor-core Gram (gl_gram_tc.cu)
int launch_gram_tc(const LsqArgs& a, float* G, float* h, int* status, int grid, cudaStream_t stream);
int gram_tc_ctas_per_sm(int D);
void set_gram_wait_polls(int polls);   // < 0: the default limit
// FP32 register-tile Gram (gl_gram_fp32.cu): same G and h, no wait or status
int launch_gram_fp32(const LsqArgs& a, float* G, float* h, int grid, cudaStream_t stream);
size_t lsq_status_offset(const LsqPlan* L, int bs);
void lsq_destroy(gl_plan* plan);
size_t lsq_workspace_bytes(const LsqPlan* L, int bs);
int lsq_run(const gl_plan* plan, const float* x, const int* img_id, int bs, float* work,
            size_t work_bytes, float* coeffs, float* img_out, float* logL, float* chi2,
            cudaStream_t stream);

}  // namespace gl
