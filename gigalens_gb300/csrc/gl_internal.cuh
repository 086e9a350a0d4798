// Internal structures shared by the host side of the C ABI and the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "gigalens_cuda.h"

namespace gl {

constexpr int kThreads = 512;        // 16 warps: 4 per SM sub-partition, up to 128 registers
constexpr int kWarps = kThreads / 32;
constexpr int kFusedCB = 16;         // output columns per thread, fused-kernel PSF correlation
constexpr int kMaxTerms = 256;       // largest EPL iteration cap the fused kernel accepts
constexpr int kMaxKS = 25;           // largest parity sub-kernel side
constexpr int kMaxPlanes = 4;        // supersample <= 2 in the fused kernel
constexpr int kRedSlots = 48;        // reduced quantities per sample
constexpr int kMaxShapeletN = 9;     // shapelets n_max <= 9: at most 55 basis functions
// Shapelets(interpolate=True): phi_n(t) exp(-t^2/2) tabulated at kShpTabN
// points on [kShpTabLo, kShpTabHi] for n < kShpTabRows
constexpr int kShpTabN = 6000;
constexpr int kShpTabRows = 31;
constexpr float kShpTabLo = -5.f, kShpTabHi = 5.f;
constexpr int kGenMass = 2;          // general path: mass profiles besides SHEAR
constexpr int kGenLight = 3;         // general path: light profiles
constexpr int kMaxAmps = 64;         // general path: external amplitudes per sample
constexpr int kMaxDevices = 64;      // per-device caches of launch attributes

// Per-image constants, in device-ready form.
struct DevImage {
  int N;            // base pixels per side
  int ss;           // supersampling factor
  int nplanes;      // ss*ss parity planes of the supersampled image
  int KS;           // parity sub-kernel side
  int ksp;          // KS rounded up to a multiple of 4 (row pitch of a sub-kernel)
  int d[kMaxPlanes];      // correlation offset of parity p (rows) / q (cols)
  int pitchI;       // row pitch (floats) of an image-parity plane in shared memory
  int padI[kMaxPlanes];   // left zero pad of plane with column parity q
  int pitchW;       // row pitch of the likelihood-adjoint plane
  int padW;         // its left zero pad
  int ncb;          // column blocks of kFusedCB outputs (even)
  int units;        // correlation work units of one plane: N rows x ncb blocks
  float x0, y0, t00, t01, t10, t11;   // fine grid: x = t00*col + t01*row + x0
  float cf;         // det(transform_pix2angle), tf/simulator.py:24-26
  float bg2;        // background_rms^2
  float inv_t;      // 1/exp_time
  const float* obs; // device N*N (may be null)
  const float* grid;// device [nplanes][N][N] float4: (x, y, shared-memory offset of the pixel
                    // in the fused kernel's parity planes as int bits, 0), plane order
  const float* kern;// device [nplanes][KS][ksp] forward parity sub-kernels
  const float* err; // device N*N noise sigma (data-noise likelihood), or null
  // shared-memory layout (float offsets)
  int offI, offW, offK, smem_floats;
};

// Profile slot: columns of each canonical parameter in the flat vector.
struct DevProfile {
  int type;
  int niter;
  int col[GL_MAX_PROFILE_PARAMS];
};

struct DevPriorLeaf {
  int dist;           // GL_DIST_*
  float loc, scale;   // Normal / LogNormal / TruncatedNormal
  float lo, hi;       // support of Uniform / TruncatedNormal (Sigmoid bijector range)
  float lognorm;      // TruncatedNormal: log(Phi(beta)-Phi(alpha)); Uniform: log(high-low)
  float loglen;       // log(high-low) of the Sigmoid bijector
};

// Model family of the fused kernel (compile-time); see gl_fused.cu.
enum ModelFamily : int {
  FAM_EPL_SHEAR_SE_SE = 0,  // EPL + Shear ; SersicEllipse lens light ; SersicEllipse source
  FAM_EPL_SHEAR_SE = 1,     // EPL + Shear ; no lens light            ; SersicEllipse source
  FAM_EPL_SE_SE = 2,        // EPL         ; SersicEllipse            ; SersicEllipse
  FAM_EPL_SE = 3,           // EPL         ; no lens light            ; SersicEllipse
  FAM_GENERIC = 4,          // general path: the profile lists of GenArgs, dispatched per pixel
  // general path compiled for one model signature (profile code inlined)
  FAM_SIG_SIE_SHEAR_SE_SE = 5,   // SIE + Shear ; SersicEllipse ; SersicEllipse
  FAM_SIG_SIS_SHEAR_SE_SE = 6,   // SIS + Shear ; SersicEllipse ; SersicEllipse
  FAM_SIG_EPL_SHEAR_SHP = 7,     // EPL + Shear ; no lens light ; Shapelets (BackwardProbModel gradient)
  FAM_COUNT = 8
};
// Families that run the general path's code (FusedArgs::gen describes the model).
inline bool is_gen_family(int fam) { return fam >= FAM_GENERIC; }

// A light profile of the general path.
struct GenLight {
  int type;     // GL_PROF_SERSIC_ELLIPSE (SERSIC as e1 = e2 = 0), GL_PROF_CORE_SERSIC, GL_PROF_SHAPELETS
  int group;    // GL_GROUP_LENS_LIGHT (evaluated at theta) or GL_GROUP_SOURCE (at beta)
  int n_max;    // shapelets
  int amp_ext;  // amplitude(s) from the external per-sample vector (least-squares coefficients)
  int amp_idx;  // index of the (first) amplitude in that vector
  int interp;   // shapelets: tabulated functions (interpolate=True)
  int col[GL_MAX_PROFILE_PARAMS];   // SERSIC_ELLIPSE / CORE_SERSIC / SHAPELETS canonical columns
};

// Model of the general path.
struct GenArgs {
  int n_mass;
  DevProfile mass[kGenMass];   // EPL (at most one), SIS, SIE, TNFW
  int has_shear;
  int n_light;
  GenLight light[kGenLight];
  int n_amp;                   // external amplitudes per sample
  const float* amps;           // [bs, n_amp] or null
  int noise_err;               // data-noise likelihood with the image's error map
  int unit_cf;                 // images without the conversion factor (least-squares images)
  int explicit_shapelets;      // shapelet profiles with amplitude parameters
  int amp_grad_slot;           // the light slot whose amplitude gradients are reduced, or -1
  const float* shp_tab;        // shapelet table (interpolating profiles), or null
};

struct FusedArgs {
  int family;
  int d;                    // flat parameter count
  int bs;
  int n_images;
  DevImage img[GL_MAX_IMAGES];
  // slots of the compile-time family, resolved to columns
  DevProfile epl, shear, llight, source;
  GenArgs gen;              // FAM_GENERIC
  int has_prior;
  DevPriorLeaf prior[GL_MAX_PARAMS];
  // inputs / outputs
  const float* x;           // [bs,d] physical (mode x) or unconstrained z (mode z)
  const int* img_id;        // [bs] or null
  const float* dlogL;       // [bs] upstream weights (adjoint mode) or null
  float* logL;              // [bs] or null
  float* chi2;              // [bs] or null
  float* img_out;           // [bs, maxN*maxN] or null
  float* grad;              // [bs,d] or null
  int* status;              // [bs] or null
  int img_stride;           // floats per sample in img_out
  int zmode;                // 1: x holds z; apply bijector, add prior + fldj
  int want_grad;            // run the adjoint phases
  float* gscratch;          // images too large for shared memory: per-CTA planes in
  int cta_floats;           //   global memory (cta_floats per CTA), else null
  int n_cta;                //   slices in gscratch: the grid never exceeds it
  int corr_scalar;          // 1: the headline family's scalar-FFMA correlation variant
};

}  // namespace gl

struct gl_plan {
  int device;
  gl_model_desc model;
  int family;
  int n_images;
  gl_image_desc host_img[GL_MAX_IMAGES];
  gl::DevImage img[GL_MAX_IMAGES];
  float* dev_buf;           // owns obs + kernels for all images
  size_t dev_buf_bytes;
  int smem_bytes;
  int max_pix;              // largest N*N
  int has_prior;
  gl::DevPriorLeaf prior[GL_MAX_PARAMS];
  gl::DevProfile epl, shear, llight, source;
  gl::GenArgs gen;          // the model on the fused kernel's general path
  int gen_ok;               // gen describes the model
  int gen_family;           // FAM_GENERIC or the compiled signature that matches gen
  int fused_fits;           // the images fit the fused kernel's shared memory
  float* gscratch;          // otherwise: per-CTA plane storage in global memory
  int cta_floats;           // floats per CTA in gscratch
  int n_cta;                // CTAs gscratch holds (the device's SM count)
  void* lsq;                // gl::LsqPlan of the least-squares path, or null
  int corr_scalar;          // tuning: scalar-FFMA correlations in the headline family
  const float* shp_tab;     // shapelet table (interpolating shapelet profiles), or null
};

namespace gl {
// implemented in gl_fused.cu
int launch_fused(const FusedArgs& a, int smem_bytes, cudaStream_t stream);
int fused_kernel_prepare(int smem_bytes);
// The current device as an index into the per-device caches (ids at or
// above kMaxDevices share the last slot).
inline int current_device_slot() {
  int d = 0;
  cudaGetDevice(&d);
  return d < 0 ? 0 : (d < kMaxDevices ? d : kMaxDevices - 1);
}
int fused_static_smem_bytes();
// implemented in gl_profile_eval.cu
int launch_profile_eval(int type, const float* x, const float* y, int64_t n, const float* params,
                        const int* n_terms, float* out0, float* out1, cudaStream_t stream);
int launch_shapelets_eval(int n_max, const float* tab, const float* x, const float* y, int64_t n,
                          const float* params, const float* amps, float* out, cudaStream_t stream);
// Device address of the shapelet table on `device` (filled on first use).
int shapelet_table(int device, const float** out);
int launch_epl_term_count(const float* e1, const float* e2, int64_t n, int cap, int* k_out,
                          cudaStream_t stream);
int launch_bijector_forward(const DevPriorLeaf* leaves, int d, const float* z, int bs, float* x,
                            cudaStream_t stream);
void set_error(const char* fmt, ...);

// Host-side NVTX range around one C-ABI call (its checks and launches), in
// the "gigalens_gb300" domain.  NVTX v3 is header-only: without a profiler
// attached each push/pop is a null-pointer test.
struct NvtxRange {
  explicit NvtxRange(const char* name) {
    static nvtxDomainHandle_t dom = nvtxDomainCreateA("gigalens_gb300");
    nvtxEventAttributes_t ev = {};
    ev.version = NVTX_VERSION;
    ev.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
    ev.messageType = NVTX_MESSAGE_TYPE_ASCII;
    ev.message.ascii = name;
    domain = dom;
    nvtxDomainRangePushEx(domain, &ev);
  }
  ~NvtxRange() { nvtxDomainRangePop(domain); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
  nvtxDomainHandle_t domain;
};
#define GL_NVTX_RANGE(name) ::gl::NvtxRange gl_nvtx_range_(name)
}  // namespace gl
