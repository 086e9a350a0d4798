/*
 * gigalens_cuda.h - C ABI of libgigalens_cuda.so, the GB300 (sm_103a) device
 * library behind the gigalens_gb300.cuda substrate.
 *
 * The reference (GIGA-Lens, pure Python on TensorFlow/JAX) has no FFI: its
 * plug-in boundary is the Python class protocol of profiles, simulator and
 * probabilistic model.  Each entry point below replaces the device work of
 * one reference call; the replaced call is cited beside it.
 *
 * Conventions
 *  - extern "C", plain pointers and sizes.  Every array argument of a compute
 *    call is DEVICE memory of the current CUDA device unless marked "host".
 *  - float32, row-major.  A flat parameter vector per sample holds the
 *    physical parameters in the reference's packing order (leaves of the
 *    parameter structure: groups lens / lens light / source, profiles in
 *    order, keys sorted; gigalens/tf/model.py:42-49).
 *  - Stream-ordered: compute calls enqueue on `stream` (a cudaStream_t passed
 *    as void*, NULL = legacy default stream) and return without synchronising.
 *  - Return 0 on success, a negative GL_ERR_* code otherwise; gl_last_error()
 *    gives a message.  Bad values are never errors (NaN pixels are zeroed,
 *    like gigalens/tf/simulator.py:81); bad shapes, sizes and pointers are.
 *  - A plan is immutable after creation and may be used from several streams;
 *    the caller owns every output buffer.
 */
#ifndef GIGALENS_CUDA_H
#define GIGALENS_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GL_ABI_VERSION 4

/* ---- error codes ---------------------------------------------------- */
#define GL_OK 0
#define GL_ERR_INVALID (-1)      /* bad argument, shape or descriptor      */
#define GL_ERR_UNSUPPORTED (-2)  /* valid input this build does not cover   */
#define GL_ERR_CUDA (-3)         /* a CUDA runtime call failed              */
#define GL_ERR_NOMEM (-4)        /* device allocation failed                */
#define GL_ERR_INTERNAL (-5)     /* an internal consistency check failed    */

/* ---- profile types (reference class names in comments) --------------- */
#define GL_PROF_NONE 0
#define GL_PROF_EPL 1            /* tf/profiles/mass/epl.py:9    EPL        */
#define GL_PROF_SHEAR 2          /* tf/profiles/mass/shear.py:6  Shear      */
#define GL_PROF_SIS 3            /* tf/profiles/mass/sis.py:9    SIS        */
#define GL_PROF_SIE 4            /* tf/profiles/mass/sie.py:9    SIE        */
#define GL_PROF_TNFW 5           /* tf/profiles/mass/tnfw.py:10  TNFW       */
#define GL_PROF_SERSIC 10        /* tf/profiles/light/sersic.py:9   Sersic        */
#define GL_PROF_SERSIC_ELLIPSE 11 /* tf/profiles/light/sersic.py:62 SersicEllipse */
#define GL_PROF_SHAPELETS 12     /* tf/profiles/light/shapelets.py:11 Shapelets */
#define GL_PROF_CORE_SERSIC 13   /* tf/profiles/light/sersic.py:75 CoreSersic    */

#define GL_GROUP_LENS 0
#define GL_GROUP_LENS_LIGHT 1
#define GL_GROUP_SOURCE 2

#define GL_MAX_PROFILES 8
#define GL_MAX_PROFILE_PARAMS 12
#define GL_MAX_IMAGES 8
#define GL_MAX_PARAMS 64

/* Canonical parameter order per type (index into gl_profile_desc.col):
 *   EPL:            theta_E, gamma, e1, e2, center_x, center_y
 *   SHEAR:          gamma1, gamma2
 *   SIS:            theta_E, center_x, center_y
 *   SIE:            theta_E, e1, e2, center_x, center_y
 *   TNFW:           Rs, alpha_Rs, r_trunc, center_x, center_y
 *   SERSIC:         R_sersic, n_sersic, center_x, center_y, Ie
 *   SERSIC_ELLIPSE: R_sersic, n_sersic, e1, e2, center_x, center_y, Ie
 *   CORE_SERSIC:    R_sersic, n_sersic, Rb, alpha, gamma, e1, e2, center_x,
 *                   center_y, Ie
 *   SHAPELETS:      beta, center_x, center_y, amp0 (column of the first of
 *                   the D = (n_max+1)(n_max+2)/2 amplitudes, which are
 *                   consecutive in the reference's ordering amp00, amp01, ..)
 * A light profile with use_lstsq has no Ie / amplitude column (col = -1).
 *
 * The fused kernel has compiled fast paths for EPL [+ SHEAR] with
 * SERSIC / SERSIC_ELLIPSE lens light and source; every other model with at
 * most 2 mass profiles besides SHEAR (at most one EPL), at most one SHEAR
 * and at most 3 light profiles runs on its general path; three model
 * signatures of the general path are compiled with their profile code
 * inlined (SIE or SIS + SHEAR with SERSIC_ELLIPSE lens light and source;
 * EPL + SHEAR with one SHAPELETS source, explicit or solved linearly).
 * Gradients with respect to explicit shapelet amplitudes are computed for
 * one shapelet profile per model (more give GL_ERR_UNSUPPORTED).
 * Images whose supersampled planes exceed a CTA's shared memory (about 90 x 90
 * at ss = 2 with a 41-pixel PSF), and every image on the general path outside
 * those signatures, keep them in a per-CTA slice of a global scratch owned by
 * the plan: calls on one such plan must not overlap on the GPU (one stream,
 * or serialised).                                                          */
typedef struct {
  int type;                        /* GL_PROF_*                            */
  int group;                       /* GL_GROUP_*                           */
  int niter;                       /* EPL: iteration cap (EPL(niter));
                                      SHAPELETS: n_max                     */
  int use_lstsq;                   /* light: unit amplitude, solved linearly */
  int col[GL_MAX_PROFILE_PARAMS];  /* flat-vector column of each parameter */
  int interpolate;                 /* SHAPELETS: Shapelets(interpolate=True),
                                      the 1-D functions phi_n(t) exp(-t^2/2)
                                      tabulated at 6000 points on [-5, 5]
                                      and interpolated linearly, 0 outside
                                      (tf/profiles/light/shapelets.py:37-38,
                                      55-60); 0: exact Hermite recursion    */
} gl_profile_desc;

typedef struct {
  int n_profiles;
  int n_params;                    /* d, width of the flat parameter vector */
  gl_profile_desc prof[GL_MAX_PROFILES];
} gl_model_desc;

/* One camera/data configuration (SimulatorConfig + observed data).
 * gigalens/simulator.py:11-28, tf/simulator.py:11-56, tf/model.py:31-37.   */
typedef struct {
  int num_pix;                     /* N (image is N x N)                   */
  int supersample;                 /* ss                                   */
  float transform_pix2angle[4];    /* base-scale 2x2, row-major            */
  int kernel_size;                 /* k, odd, of the supersampled PSF; 0 = none */
  const float* kernel;             /* host, k*k: the supersampled PSF as the
                                      reference's subgrid_kernel returns it
                                      (not flipped); true convolution     */
  const float* observed;           /* host, N*N (may be NULL for simulate-only) */
  float background_rms;
  float exp_time;
  const float* err_map;            /* host, N*N noise sigma for the least-squares
                                      path; NULL = sqrt(bg^2 + clip(obs,0)/t),
                                      the BackwardProbModel map (tf/model.py:92-94) */
} gl_image_desc;

/* Prior leaf: a distribution and its default event-space bijector, one per
 * flat-vector column (tfp JointDistribution leaves,
 * tf/model.py:50 experimental_default_event_space_bijector).              */
#define GL_DIST_NORMAL 1           /* Normal(a=loc, b=scale), Identity          */
#define GL_DIST_LOGNORMAL 2        /* LogNormal(a=loc, b=scale), Exp            */
#define GL_DIST_UNIFORM 3          /* Uniform(a=low, b=high), Sigmoid(low,high) */
#define GL_DIST_TRUNCNORMAL 4      /* TruncatedNormal(a=loc,b=scale,c=low,d=high),
                                      Sigmoid(low, high)                       */
typedef struct {
  int dist;
  float a, b, c, d;
} gl_prior_leaf;

typedef struct gl_plan gl_plan;

/* ---- library ---------------------------------------------------------- */
int gl_abi_version(void);
/* sizeof of the public structs, for bindings to check their mirrors:
 * 0 gl_profile_desc, 1 gl_model_desc, 2 gl_image_desc, 3 gl_prior_leaf,
 * 4 gl_tune_result, 5 gl_adam_cfg, 6 gl_tuning; -1 for any other index.  */
int gl_struct_size(int which);
const char* gl_last_error(void);
/* Number of SMs and the opt-in shared memory per block of the current device. */
int gl_device_info(int* sm_count, int* smem_optin_bytes);

/* ---- plans ------------------------------------------------------------ */
/* Replaces LensSimulator.__init__ (tf/simulator.py:11-56) and the constant
 * part of ForwardProbModel.__init__ (tf/model.py:31-37): validates the model,
 * builds the PSF+binning sub-kernels, copies observed images to the device. */
int gl_plan_create(const gl_model_desc* model, const gl_image_desc* images, int n_images,
                   gl_plan** out);
/* Attach the prior (one leaf per column) for gl_log_prob / gl_log_prob_grad. */
int gl_plan_set_prior(gl_plan* plan, const gl_prior_leaf* leaves, int n_leaves);
int gl_plan_destroy(gl_plan* plan);
/* Shared memory per block and threads per block the fused kernel uses. */
int gl_plan_query(const gl_plan* plan, int* smem_bytes, int* threads_per_block, int* max_img_pix);

/* ---- fused forward model + likelihood -------------------------------- */
/* img_id: [bs] image index per sample, or NULL (all samples use image 0).
 * status: [bs] per-sample flags (bit0 non-finite logL, bit1 non-finite
 * gradient) or NULL.                                                      */

/* LensSimulator.simulate + ForwardProbModel likelihood
 * (tf/simulator.py:65-97, tf/model.py:76-86): x[bs,d] physical parameters ->
 * logL[bs] (sum over pixels of the Normal log density, model-based noise),
 * chi2[bs] (mean squared normalised residual), optional img_out[bs,N,N]
 * (simulated image; for mixed image sizes each sample's slot is max_N^2,
 * row-major N x N at the start).  logL/chi2 may be NULL when the image has no
 * observed data.                                                         */
int gl_forward(const gl_plan* plan, const float* x, const int* img_id, int bs,
               float* logL, float* chi2, float* img_out, int* status, void* stream);

/* Fused value and gradient: as gl_forward plus dlogL_dx[bs,d] = d logL / d x
 * (hand-written adjoint of tf/model.py:76-80 through tf/simulator.py:65-97
 * and the profiles; replaces TF GradientTape, tf/inference.py:30-33).    */
int gl_forward_grad(const gl_plan* plan, const float* x, const int* img_id, int bs,
                    float* logL, float* chi2, float* dlogL_dx, int* status, void* stream);

/* Vector-Jacobian product: dx[b,:] = dlogL[b] * d logL_b / d x_b.          */
int gl_adjoint(const gl_plan* plan, const float* x, const int* img_id, int bs,
               const float* dlogL, float* dx, int* status, void* stream);

/* ForwardProbModel.log_prob (tf/model.py:53-86) on unconstrained z[bs,d]:
 * logp = logL + prior.log_prob(x) + fldj(z) with x = bijector(z); chi2 as
 * above; dlogp_dz[bs,d] (NULL = value only).  Needs gl_plan_set_prior.    */
int gl_log_prob(const gl_plan* plan, const float* z, const int* img_id, int bs,
                float* logp, float* chi2, float* dlogp_dz, int* status, void* stream);

/* Unconstraining bijector forward: x = bij(z) per column (tf/model.py:75).  */
int gl_bijector_forward(const gl_plan* plan, const float* z, int bs, float* x, void* stream);

/* ---- profile evaluation (the MassProfile.deriv / LightProfile.light API) */
/* Evaluate one profile at n points.  params: [n_params_of_type, n] device
 * (row p = canonical parameter p, one value per point).  EPL uses n_terms
 * series iterations; gl_epl_term_count computes the reference's rule.
 * MassProfile.deriv -> (out0, out1) = deflection; LightProfile.light -> out0
 * (SERSIC, SERSIC_ELLIPSE, CORE_SERSIC rows include Ie as the last row).
 * (tf/profiles/mass/*.py deriv, tf/profiles/light/sersic.py light.)        */
int gl_profile_eval(int type, const float* x, const float* y, int64_t n, const float* params,
                    const int* n_terms, float* out0, float* out1, void* stream);
/* Shapelets.light (tf/profiles/light/shapelets.py:53-85): params [3, n] =
 * (beta, center_x, center_y) per point.  amps [D, n] with
 * D = (n_max+1)(n_max+2)/2 gives out [n] = sum_k amps_k basis_k; amps NULL
 * gives the unit-amplitude basis stack out [D, n] (use_lstsq).
 * interpolate: 1 for the tabulated functions (interpolate=True), 0 for the
 * exact recursion (interpolate=False).                                     */
int gl_shapelets_eval(int n_max, int interpolate, const float* x, const float* y, int64_t n,
                      const float* params, const float* amps, float* out, void* stream);
/* tf/profiles/mass/epl.py:41,51-56: K = min(cap, #{i=1,2,..: i < log(1e-12)/log(max f)+2})
 * over n ellipticity pairs; writes the int K to *k_out (device).           */
int gl_epl_term_count(const float* e1, const float* e2, int64_t n, int cap, int* k_out, void* stream);

/* ---- linear amplitudes (least squares) -------------------------------- */
/* LensSimulator.lstsq_simulate (tf/simulator.py:99-165) for a plan whose
 * light profiles all have use_lstsq (unit-amplitude Sersic, Shapelets with
 * either interpolate setting): basis stack -> PSF + binning -> weighted normal
 * equations G = X^T W^2 X, h = X^T W^2 y (W = 1/err_map) -> coeffs =
 * pinv(G, rcond=1e-6) h -> img = sum_c coeffs_c X_c (no conversion factor,
 * as the reference) -> BackwardProbModel likelihood with the error map
 * (tf/model.py:157-163).  work: caller-allocated device scratch of
 * gl_lstsq_workspace() bytes.  coeffs [bs, D] is required; img_out
 * [bs, max_N^2], logL [bs], chi2 [bs] may be NULL.                        */
int gl_lstsq_workspace(const gl_plan* plan, int bs, size_t* bytes, int* n_channels);
int gl_lstsq(const gl_plan* plan, const float* x, const int* img_id, int bs, void* work,
             size_t work_bytes, float* coeffs, float* img_out, float* logL, float* chi2,
             void* stream);

/* Allocation-free variant of gl_lstsq (no counterpart in the reference).
 * Some callers cannot call cudaMalloc: a host framework whose own allocator
 * has already reserved the GPU's memory, a serving loop that must not pay the
 * device-wide synchronisation of cudaMalloc/cudaFree, or a plug-in callback
 * that is not allowed to allocate.  This entry point takes the same inputs
 * and outputs as gl_lstsq but no workspace: its scratch is a fixed 64 MiB
 * array inside the library, which every GPU that loads the library keeps
 * until the process exits.  It allocates nothing itself.
 *  - Batches whose gl_lstsq_workspace() exceeds 64 MiB are rejected with
 *    GL_ERR_INVALID and a message giving the largest batch that fits.
 *  - The first call on a device looks up the array's device address (with
 *    that device current); make that first call before any stream capture.
 *  - Every call shares the one array and it keeps the last call's contents;
 *    each call writes every scratch element it reads, so nothing needs
 *    clearing.  Calls that overlap on the GPU (other streams, other host
 *    threads) race on the array: serialise them.                          */
int gl_lstsq_noalloc(const gl_plan* plan, const float* x, const int* img_id, int bs,
                     float* coeffs, float* img_out, float* logL, float* chi2, void* stream);

/* Status word of the last gl_lstsq / gl_lstsq_noalloc call of bs chains on
 * this plan (no reference counterpart: TF raises no error for this).  The
 * tensor-core Gram kernel's waits (gl_tuning.lsq_gram = 1) are bounded; a
 * wait that runs out sets the word to 1, the kernel drains its MMAs, frees
 * its tensor memory and returns, and the solve writes NaN coefficients.  The
 * default FP32 Gram kernel has no waits and leaves the word 0.  work: the workspace given
 * to gl_lstsq, or NULL for gl_lstsq_noalloc's fixed scratch.  *status
 * (device or host memory) receives the word, stream-ordered: 0 = ok.       */
int gl_lstsq_status(const gl_plan* plan, int bs, const void* work, int* status, void* stream);

/* Failure-detection test hook (no reference counterpart): the number of
 * polls of the Gram kernel's pipeline waits for the following launches;
 * polls < 0 restores the default limit.  0 makes every such wait run out at
 * once.  Not for production use.                                          */
int gl_test_set_wait_polls(int polls);

/* Launch configuration of the fused kernel for a batch of bs samples
 * (no reference counterpart: TensorFlow/XLA choose the reference's kernels).
 * The correlation tile (16 outputs per lane, quarter-warp groups of 4 rows x
 * 2 blocks), the block size (512 threads, 16 warps) and the interleave depth
 * are compiled for sm_103a and the grid is persistent (one CTA per SM, at
 * most bs); the least-squares basis kernel's shape is the plan's tuning
 * (gl_plan_set_tuning, chosen by timing in gigalens_gb300.cuda.autotune and
 * cached per plan shape).  The result is the configuration the plan's
 * launches use.                                                            */
typedef struct {
  int threads_per_block;
  int blocks;              /* CTAs of a launch of bs samples            */
  int samples_per_cta;     /* ceil(bs / blocks)                          */
  int smem_bytes;          /* dynamic shared memory per CTA             */
  int family;              /* 0..3 compiled fast paths, 4 general path,
                              5..7 general path compiled for one model
                              signature: 5 SIE + shear, 6 SIS + shear (each
                              with SersicEllipse lens light and source),
                              7 EPL + shear with a shapelet source          */
  int global_planes;       /* 1: the image planes live in global memory */
  int subkernel_side;      /* largest parity sub-kernel side            */
  int col_block;           /* correlation outputs per lane              */
} gl_tune_result;
int gl_autotune(const gl_plan* plan, int bs, gl_tune_result* out);

/* Tunable launch shape of a plan (no reference counterpart).  The timing
 * search over these values lives on the host side (cuda/autotune.py): it
 * times each candidate on the caller's inputs, keeps the fastest and caches
 * it per plan shape.  Changing the least-squares fields re-plans the basis
 * kernel's shared-memory layout, which changes gl_lstsq_workspace(): query
 * it again afterwards.  Fields left 0 keep the current value.
 *   lsq_ctas_per_sm  1: 512 threads per CTA, whole-image parity planes when
 *                    they fit; 2: two CTAs of 256 threads per SM on row bands,
 *                    so one CTA's channel evaluation overlaps the other's
 *                    correlation
 *   lsq_col_block    output columns per correlation unit: 16 or 20, or -1
 *                    for the planner's choice
 *   fused_corr       the fused kernel's PSF correlations (EPL + shear +
 *                    Sersic lens light + Sersic source, image planes in
 *                    shared memory): 1 packed FFMA2, 2 scalar FFMA; other
 *                    models always use FFMA2
 *   lsq_gram         the normal equations A^T A, A^T b: 1 tcgen05 tensor
 *                    cores in 3xTF32 (its pipeline waits are bounded and set
 *                    the status word), 2 FP32 register tiles (the default)  */
typedef struct {
  int lsq_ctas_per_sm;
  int lsq_col_block;
  int fused_corr;
  int lsq_gram;
  int reserved[4];
} gl_tuning;
int gl_plan_set_tuning(gl_plan* plan, const gl_tuning* t);
int gl_plan_get_tuning(const gl_plan* plan, gl_tuning* t);

/* Gradient of the BackwardProbModel likelihood (tf/model.py:152-158: the
 * least-squares image scored with the data-based error map) with respect to
 * the nonlinear parameters x, at the coefficients gl_lstsq returned for the
 * same x.  The coefficients minimise chi^2 for the fixed noise map, so by the
 * envelope theorem d logL/dx = (partial d logL/dx at fixed coefficients);
 * TensorFlow's derivative through pinv reduces to the same value where the
 * normal equations are solved exactly.  logL [bs], chi2 [bs] (may be NULL)
 * are recomputed from the same image; grad [bs, d] is written.            */
int gl_lstsq_grad(const gl_plan* plan, const float* x, const int* img_id, int bs,
                  const float* coeffs, float* logL, float* chi2, float* grad, void* stream);

/* ---- optimizer step (graph-capturable) ------------------------------- */
/* Keras Adam as used by ModellingSequence.MAP (tf/inference.py:34,
 * optimizer.apply_gradients): with t = *step + 1 and lr = schedule(*step),
 *   alpha = lr*sqrt(1-b2^t)/(1-b1^t); m += (g-m)(1-b1); v += (g^2-v)(1-b2);
 *   var -= alpha*m/(sqrt(v)+eps),  g = grad_scale * grad,
 * then *step += 1.  step is a device int so the call can be replayed from a
 * CUDA graph.  Schedules: constant, or Keras PolynomialDecay
 * lr(s) = (lr0-lr_end)(1-min(s,decay_steps)/decay_steps)^power + lr_end.  */
#define GL_LR_CONSTANT 0
#define GL_LR_POLYNOMIAL 1
typedef struct {
  int schedule;      /* GL_LR_* */
  float lr0, lr_end, decay_steps, power;
  float beta1, beta2, eps;
} gl_adam_cfg;
int gl_adam_step(float* var, float* m, float* v, const float* grad, int64_t n, float grad_scale,
                 const gl_adam_cfg* cfg, int* step, void* stream);

/* ---- learned MAP initialiser (no reference counterpart) ----------------
 * Building blocks of the CNN that proposes ModellingSequence.MAP's starting
 * ensemble (the `start` hook, gigalens/inference.py:34-57); orchestrated by
 * gigalens_gb300/cuda/initializer.py.  Row-major float32 unless noted.     */
/* C[b] = alpha op(A[b]) op(B[b]) + beta C[b] for b < batch; op(A) M x K,
 * op(B) K x N; trans* = operand stored transposed; a_bf16: A is bfloat16
 * (weights stored in BF16), accumulation is float32.  ksplit > 1 splits K
 * across CTAs and adds the partial products atomically (beta must be 0;
 * C is cleared first).                                                    */
int gl_nn_gemm(int transA, int transB, int a_bf16, int M, int N, int K, float alpha, const void* A,
               int lda, long long strideA, const float* B, int ldb, long long strideB, float beta,
               float* C, int ldc, long long strideC, int batch, int ksplit, void* stream);
/* 3x3, padding 1, channel-major activations: col [C*9][B][Ho*Wo] from
 * X [C][B][H][W]; Ho = (H-1)/stride + 1.                                  */
int gl_nn_im2col3x3(const float* X, int B, int C, int H, int W, int stride, float* col, void* stream);
/* adjoint of im2col: dX [C][B][H][W] from dcol [C*9][B][Ho*Wo].            */
int gl_nn_col2im3x3(const float* dcol, int B, int C, int H, int W, int stride, float* dX, void* stream);
/* dst [B][A][C] = src [A][B][C] with the first two axes swapped.           */
int gl_nn_permute01(const float* src, int A, int B, int C, float* dst, void* stream);
/* Y [B][C][P] += bias[c]; ReLU when relu.                                  */
int gl_nn_bias_act(float* Y, const float* bias, int B, int C, int P, int relu, void* stream);
/* dY *= (Y > 0) when relu; dbias[c] = sum over b, p of dY.                 */
int gl_nn_bias_act_backward(float* dY, const float* Y, int B, int C, int P, int relu, float* dbias,
                            void* stream);
/* Gaussian negative log-likelihood head: out [2d][B] (means, log-sigma
 * clamped to [-12, 12]), target [d][B]; loss [d][B] and dout [2d][B] =
 * gradient of the mean loss (either may be NULL).                          */
int gl_nn_gauss_nll(const float* out, const float* target, int B, int d, float* loss, float* dout,
                    void* stream);
int gl_nn_transpose(const float* src, int rows, int cols, float* dst, void* stream);
/* dst (bfloat16) = round-to-nearest(src), n elements.                      */
int gl_nn_cast_bf16(const float* src, void* dst, long long n, void* stream);

/* ---- diagnostics (no reference counterpart) --------------------------- */
/* FP32 FMA throughput probe: blocks_per_sm*SMs blocks of 256 threads run
 * 8 independent FMA chains for iters*16 steps; *flops receives the flop
 * count of one launch (out: device scratch of >= blocks floats).  Time it
 * with events to get the FP32 peak that the fused kernel's roofline uses. */
int gl_probe_fp32_fma(float* out, int iters, int blocks_per_sm, double* flops, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GIGALENS_CUDA_H */
