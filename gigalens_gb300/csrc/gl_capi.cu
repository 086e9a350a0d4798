// Host side of the C ABI: plan construction (validation, PSF+binning
// sub-kernels, coordinate grid, device constants) and the compute entry
// points.  No compute happens here; every entry point enqueues kernels.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gl_internal.cuh"
#include "gl_lstsq.cuh"

namespace gl {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

static int cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? GL_ERR_NOMEM : GL_ERR_CUDA;
  }
  return GL_OK;
}

static int param_count(int type) {
  switch (type) {
    case GL_PROF_EPL: return 6;
    case GL_PROF_SHEAR: return 2;
    case GL_PROF_SIS: return 3;
    case GL_PROF_SIE: return 5;
    case GL_PROF_TNFW: return 5;
    case GL_PROF_SERSIC: return 5;
    case GL_PROF_SERSIC_ELLIPSE: return 7;
    case GL_PROF_CORE_SERSIC: return 10;
    case GL_PROF_SHAPELETS: return 4;
    default: return -1;
  }
}

// Map the model descriptor to a compiled fast-path family of the fused kernel
// and resolve every slot to flat-vector columns.  SERSIC (spherical) runs as
// SERSIC_ELLIPSE with e1 = e2 = 0.  Returns false (no error) when the model
// is not one of the fast-path families.
static bool resolve_family(const gl_model_desc* m, int* family, DevProfile* epl, DevProfile* shear,
                           DevProfile* llight, DevProfile* source) {
  int n_epl = 0, n_shear = 0, n_ll = 0, n_src = 0;
  for (auto* p : {epl, shear, llight, source}) {
    p->type = GL_PROF_NONE;
    p->niter = 0;
    for (int i = 0; i < GL_MAX_PROFILE_PARAMS; ++i) p->col[i] = -1;
  }
  for (int i = 0; i < m->n_profiles; ++i) {
    const gl_profile_desc& p = m->prof[i];
    if (p.group == GL_GROUP_LENS) {
      if (p.type == GL_PROF_EPL) {
        ++n_epl;
        epl->type = p.type;
        epl->niter = p.niter;
        for (int k = 0; k < 6; ++k) epl->col[k] = p.col[k];
      } else if (p.type == GL_PROF_SHEAR) {
        ++n_shear;
        shear->type = p.type;
        for (int k = 0; k < 2; ++k) shear->col[k] = p.col[k];
      } else {
        return false;
      }
    } else {
      DevProfile* dst = p.group == GL_GROUP_LENS_LIGHT ? llight : source;
      int* cnt = p.group == GL_GROUP_LENS_LIGHT ? &n_ll : &n_src;
      ++*cnt;
      dst->type = GL_PROF_SERSIC_ELLIPSE;
      if (p.use_lstsq) return false;
      if (p.type == GL_PROF_SERSIC_ELLIPSE) {
        for (int k = 0; k < 7; ++k) dst->col[k] = p.col[k];
      } else if (p.type == GL_PROF_SERSIC) {
        // R_sersic, n_sersic, center_x, center_y, Ie -> SE slots 0,1,4,5,6
        dst->col[0] = p.col[0];
        dst->col[1] = p.col[1];
        dst->col[4] = p.col[2];
        dst->col[5] = p.col[3];
        dst->col[6] = p.col[4];
      } else {
        return false;
      }
    }
  }
  if (n_epl != 1 || n_shear > 1 || n_ll > 1 || n_src != 1) return false;
  if (n_shear) *family = n_ll ? FAM_EPL_SHEAR_SE_SE : FAM_EPL_SHEAR_SE;
  else *family = n_ll ? FAM_EPL_SE_SE : FAM_EPL_SE;
  return true;
}

// The model on the fused kernel's general path.  With lsq, light profiles
// with use_lstsq take their amplitudes from the least-squares coefficient
// vector, in the channel order of the least-squares planner (light profiles
// in descriptor order; one channel per Sersic, D per shapelet set).
static int resolve_generic(const gl_model_desc* m, bool lsq, GenArgs* g, DevProfile* epl,
                           DevProfile* shear) {
  memset(g, 0, sizeof(*g));
  g->amp_grad_slot = -1;
  for (auto* p : {epl, shear}) {
    p->type = GL_PROF_NONE;
    p->niter = 0;
    for (int i = 0; i < GL_MAX_PROFILE_PARAMS; ++i) p->col[i] = -1;
  }
  int n_amp = 0;
  for (int i = 0; i < m->n_profiles; ++i) {
    const gl_profile_desc& p = m->prof[i];
    if (p.group == GL_GROUP_LENS) {
      if (p.type == GL_PROF_SHEAR) {
        if (g->has_shear) {
          set_error("at most one SHEAR profile");
          return GL_ERR_UNSUPPORTED;
        }
        g->has_shear = 1;
        shear->type = p.type;
        for (int k = 0; k < 2; ++k) shear->col[k] = p.col[k];
        continue;
      }
      if (p.type != GL_PROF_EPL && p.type != GL_PROF_SIS && p.type != GL_PROF_SIE &&
          p.type != GL_PROF_TNFW) {
        set_error("lens profile type %d is not a mass profile", p.type);
        return GL_ERR_INVALID;
      }
      if (g->n_mass >= kGenMass) {
        set_error("at most %d mass profiles besides SHEAR", kGenMass);
        return GL_ERR_UNSUPPORTED;
      }
      DevProfile& d = g->mass[g->n_mass++];
      d.type = p.type;
      d.niter = p.niter;
      for (int k = 0; k < GL_MAX_PROFILE_PARAMS; ++k) d.col[k] = p.col[k];
      if (p.type == GL_PROF_EPL) {
        if (epl->type == GL_PROF_EPL) {
          set_error("at most one EPL profile");
          return GL_ERR_UNSUPPORTED;
        }
        if (p.niter < 0 || p.niter > kMaxTerms) {
          set_error("EPL niter %d outside [0, %d]", p.niter, kMaxTerms);
          return GL_ERR_UNSUPPORTED;
        }
        *epl = d;
      }
    } else if (p.group == GL_GROUP_LENS_LIGHT || p.group == GL_GROUP_SOURCE) {
      if (g->n_light >= kGenLight) {
        set_error("at most %d light profiles", kGenLight);
        return GL_ERR_UNSUPPORTED;
      }
      GenLight& L = g->light[g->n_light++];
      L.group = p.group;
      for (int k = 0; k < GL_MAX_PROFILE_PARAMS; ++k) L.col[k] = -1;
      const bool ext = lsq && p.use_lstsq;
      L.amp_ext = ext ? 1 : 0;
      L.amp_idx = n_amp;
      if (p.type == GL_PROF_SERSIC_ELLIPSE || p.type == GL_PROF_SERSIC) {
        L.type = GL_PROF_SERSIC_ELLIPSE;
        if (p.type == GL_PROF_SERSIC_ELLIPSE) {
          for (int k = 0; k < 7; ++k) L.col[k] = p.col[k];
        } else {
          L.col[0] = p.col[0];
          L.col[1] = p.col[1];
          L.col[4] = p.col[2];
          L.col[5] = p.col[3];
          L.col[6] = p.col[4];
        }
        if (p.use_lstsq) L.col[6] = -1;   // unit amplitude (or the coefficient)
        if (ext) n_amp += 1;
      } else if (p.type == GL_PROF_CORE_SERSIC) {
        L.type = p.type;
        for (int k = 0; k < 10; ++k) L.col[k] = p.col[k];
        if (p.use_lstsq) L.col[9] = -1;
        if (ext) n_amp += 1;
      } else if (p.type == GL_PROF_SHAPELETS) {
        L.type = p.type;
        if (p.niter < 0 || p.niter > kMaxShapeletN) {
          set_error("shapelets n_max %d outside [0, %d]", p.niter, kMaxShapeletN);
          return GL_ERR_UNSUPPORTED;
        }
        L.n_max = p.niter;
        L.interp = p.interpolate ? 1 : 0;
        for (int k = 0; k < 3; ++k) L.col[k] = p.col[k];
        const int D = (p.niter + 1) * (p.niter + 2) / 2;
        if (ext) {
          n_amp += D;
        } else if (p.use_lstsq) {
          set_error("shapelets with use_lstsq need the least-squares coefficients (gl_lstsq)");
          return GL_ERR_UNSUPPORTED;
        } else {
          if (p.col[3] < 0 || p.col[3] + D > m->n_params) {
            set_error("shapelets: amplitude columns %d..%d outside the parameter vector", p.col[3],
                      p.col[3] + D - 1);
            return GL_ERR_INVALID;
          }
          L.col[3] = p.col[3];
          if (g->explicit_shapelets++ == 0) g->amp_grad_slot = g->n_light - 1;
        }
      } else {
        set_error("light profile type %d is not a light profile", p.type);
        return GL_ERR_INVALID;
      }
    } else {
      set_error("profile %d: bad group %d", i, p.group);
      return GL_ERR_INVALID;
    }
  }
  if (g->n_light < 1) {
    set_error("the model needs at least one light profile");
    return GL_ERR_INVALID;
  }
  if (n_amp > kMaxAmps) {
    set_error("%d linear amplitudes exceed %d", n_amp, kMaxAmps);
    return GL_ERR_UNSUPPORTED;
  }
  g->n_amp = n_amp;
  return GL_OK;
}

// The compiled general-path signature matching the model of g (the profile
// types, counts, light groups and the shear), or FAM_GENERIC.
static int gen_signature(const GenArgs& g) {
  if (!g.has_shear || g.n_mass != 1) return FAM_GENERIC;
  const int m = g.mass[0].type;
  if (g.n_light == 2 && g.light[0].type == GL_PROF_SERSIC_ELLIPSE && g.light[0].group == GL_GROUP_LENS_LIGHT &&
      g.light[1].type == GL_PROF_SERSIC_ELLIPSE && g.light[1].group == GL_GROUP_SOURCE) {
    if (m == GL_PROF_SIE) return FAM_SIG_SIE_SHEAR_SE_SE;
    if (m == GL_PROF_SIS) return FAM_SIG_SIS_SHEAR_SE_SE;
  }
  if (g.n_light == 1 && m == GL_PROF_EPL && g.light[0].type == GL_PROF_SHAPELETS &&
      g.light[0].group == GL_GROUP_SOURCE)
    return FAM_SIG_EPL_SHEAR_SHP;
  return FAM_GENERIC;
}

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct HostImage {
  std::vector<float> obs, grid, kern, err;
};

// Fill the device-ready description of one image; host arrays go to hi.
static int build_image(const gl_image_desc& g, DevImage& I, HostImage& hi) {
  const int N = g.num_pix, ss = g.supersample;
  if (N <= 0 || N > 4096) {
    set_error("num_pix %d out of range", N);
    return GL_ERR_INVALID;
  }
  if (ss < 1 || ss > 2) {
    set_error("supersample %d: the fused kernel supports 1 and 2", ss);
    return GL_ERR_UNSUPPORTED;
  }
  if (g.kernel_size < 0 || (g.kernel_size > 0 && (g.kernel_size % 2 == 0 || !g.kernel))) {
    set_error("kernel_size %d must be 0 or odd with a kernel pointer", g.kernel_size);
    return GL_ERR_INVALID;
  }
  if (!(g.exp_time > 0.f) || !(g.background_rms >= 0.f)) {
    set_error("exp_time must be > 0 and background_rms >= 0");
    return GL_ERR_INVALID;
  }
  memset(&I, 0, sizeof(I));
  I.N = N;
  I.ss = ss;
  I.nplanes = ss * ss;
  // flipped PSF (the reference correlates with kernel[::-1, ::-1])
  const int k = g.kernel_size > 0 ? g.kernel_size : 1;
  std::vector<double> flat(k * k, 1.0);
  if (g.kernel_size > 0)
    for (int m = 0; m < k; ++m)
      for (int n = 0; n < k; ++n) flat[m * k + n] = g.kernel[(k - 1 - m) * k + (k - 1 - n)];
  const int pad = (k - 1) / 2;
  const int kc = k + ss - 1;
  // combined kernel: correlation with PSF then ss x ss average pooling
  std::vector<double> Kc(kc * kc, 0.0);
  for (int u = 0; u < kc; ++u)
    for (int v = 0; v < kc; ++v) {
      double s = 0.0;
      for (int a = 0; a < ss; ++a)
        for (int b = 0; b < ss; ++b) {
          int m = u - a, n = v - b;
          if (m >= 0 && m < k && n >= 0 && n < k) s += flat[m * k + n];
        }
      Kc[u * kc + v] = s / (ss * ss);
    }
  const int KS = (kc + ss - 1) / ss;
  if (KS > kMaxKS) {
    set_error("PSF too large for the fused kernel: sub-kernel side %d > %d", KS, kMaxKS);
    return GL_ERR_UNSUPPORTED;
  }
  I.KS = KS;
  I.ksp = (KS + 3) & ~3;
  for (int p = 0; p < ss; ++p) I.d[p] = (p + pad) / ss;
  for (int p = 1; p < ss; ++p)
    if (I.d[p] - I.d[0] < 0 || I.d[p] - I.d[0] > 1 || (I.d[p] != I.d[0] && KS % 2)) {
      set_error("PSF size %d with supersample %d: parity offsets %d, %d not supported", k, ss, I.d[0],
                I.d[p]);
      return GL_ERR_UNSUPPORTED;
    }
  hi.kern.assign(I.nplanes * KS * I.ksp, 0.f);
  for (int p = 0; p < ss; ++p)
    for (int q = 0; q < ss; ++q)
      for (int m = 0; m < KS; ++m)
        for (int l = 0; l < KS; ++l) {
          int u = ss * m + (p + pad) % ss, v = ss * l + (q + pad) % ss;
          double val = (u < kc && v < kc) ? Kc[u * kc + v] : 0.0;
          hi.kern[((p * ss + q) * KS + m) * I.ksp + l] = (float)val;
        }
  // shared-memory layout
  // The pitch covers the segments read by the fused kernel (kFusedCB columns
  // per unit, plus one when the transposed correlation of column parity 1
  // starts one float past a 16-byte boundary: PSF sizes k = 3 mod 4 at ss = 2).
  const int max_shift = I.d[ss - 1] - I.d[0];
  I.ncb = ((N + kFusedCB - 1) / kFusedCB + 1) & ~1;
  I.units = N * I.ncb;
  const int seg_f = (kFusedCB + KS - 1 + max_shift + 3) & ~3;
  int pitch = (int)align_up(kFusedCB * (I.ncb - 1) + seg_f, 4);
  if ((pitch / 4) % 2 == 0) pitch += 4;
  for (int q = 0; q < ss; ++q) I.padI[q] = I.d[q];
  I.pitchI = pitch;
  I.padW = KS - 1 - I.d[0];
  I.pitchW = pitch;
  I.offI = 0;
  I.offW = I.nplanes * N * I.pitchI;
  // one spare row after the likelihood-adjoint plane: the row prefetch of the
  // transposed correlation reads one row past the plane's last
  I.offK = I.offW + (N + 1) * I.pitchW;
  I.smem_floats = I.offK + I.nplanes * KS * I.ksp;
  // coordinate grid, gigalens/simulator.py:91-125 (float64 then float32)
  const int S = ss * N;
  double T[4];
  for (int i = 0; i < 4; ++i) T[i] = (double)g.transform_pix2angle[i] / ss;
  // lo = min(arange(S) - mean) and the origin T @ [lo, lo] are float32 in the reference
  const float lo = 0.f - (float)((double)(S - 1) / 2.0);
  const double ra0 = (double)(float)((float)((float)T[0] * lo) + (float)((float)T[1] * lo));
  const double dec0 = (double)(float)((float)((float)T[2] * lo) + (float)((float)T[3] * lo));
  hi.grid.assign((size_t)I.nplanes * N * N * 4, 0.f);
  for (int p = 0; p < ss; ++p)
    for (int q = 0; q < ss; ++q)
      for (int Y = 0; Y < N; ++Y)
        for (int X = 0; X < N; ++X) {
          const double row = ss * Y + p, col = ss * X + q;
          const int pq = p * ss + q;
          const size_t v = (((size_t)pq * N + Y) * N + X) * 4;
          hi.grid[v] = (float)(T[0] * col + T[1] * row + ra0);
          hi.grid[v + 1] = (float)(T[2] * col + T[3] * row + dec0);
          const int off = I.offI + (pq * N + Y) * I.pitchI + I.padI[q] + X;
          memcpy(&hi.grid[v + 2], &off, sizeof(int));
        }
  I.t00 = (float)T[0];
  I.t01 = (float)T[1];
  I.t10 = (float)T[2];
  I.t11 = (float)T[3];
  I.x0 = (float)ra0;
  I.y0 = (float)dec0;
  I.cf = (float)((double)g.transform_pix2angle[0] * g.transform_pix2angle[3] -
                 (double)g.transform_pix2angle[1] * g.transform_pix2angle[2]);
  I.bg2 = g.background_rms * g.background_rms;
  I.inv_t = 1.f / g.exp_time;
  if (g.observed) hi.obs.assign(g.observed, g.observed + (size_t)N * N);
  // noise map of the least-squares path: given, or the BackwardProbModel
  // data-based map sqrt(bg^2 + clip(obs, 0, inf) / t) in float32
  if (g.err_map) {
    hi.err.assign(g.err_map, g.err_map + (size_t)N * N);
  } else if (g.observed) {
    hi.err.resize((size_t)N * N);
    const float bg2 = g.background_rms * g.background_rms;
    for (size_t p = 0; p < hi.err.size(); ++p)
      hi.err[p] = sqrtf(bg2 + fmaxf(g.observed[p], 0.f) / g.exp_time);
  }
  return GL_OK;
}

static int check_device(const gl_plan* plan) {
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != plan->device) {
    set_error("plan was created on device %d but device %d is current", plan->device, dev);
    return GL_ERR_INVALID;
  }
  return GL_OK;
}

static DevPriorLeaf make_leaf(const gl_prior_leaf& l) {
  DevPriorLeaf d;
  memset(&d, 0, sizeof(d));
  d.dist = l.dist;
  switch (l.dist) {
    case GL_DIST_NORMAL:
    case GL_DIST_LOGNORMAL:
      d.loc = l.a;
      d.scale = l.b;
      break;
    case GL_DIST_UNIFORM:
      d.lo = l.a;
      d.hi = l.b;
      d.lognorm = (float)std::log((double)l.b - (double)l.a);
      d.loglen = d.lognorm;
      break;
    case GL_DIST_TRUNCNORMAL: {
      d.loc = l.a;
      d.scale = l.b;
      d.lo = l.c;
      d.hi = l.d;
      const double al = ((double)l.c - l.a) / l.b, be = ((double)l.d - l.a) / l.b;
      const double Z = 0.5 * (std::erfc(-be / std::sqrt(2.0)) - std::erfc(-al / std::sqrt(2.0)));
      d.lognorm = (float)std::log(Z);
      d.loglen = (float)std::log((double)l.d - (double)l.c);
      break;
    }
    default:
      break;
  }
  return d;
}

static void fill_args(const gl_plan* plan, FusedArgs& a) {
  memset(&a, 0, sizeof(a));
  a.family = plan->family;
  a.corr_scalar = plan->corr_scalar;
  a.d = plan->model.n_params;
  a.n_images = plan->n_images;
  for (int i = 0; i < plan->n_images; ++i) a.img[i] = plan->img[i];
  a.epl = plan->epl;
  a.shear = plan->shear;
  a.llight = plan->llight;
  a.source = plan->source;
  a.gen = plan->gen;
  a.gscratch = plan->gscratch;
  a.cta_floats = plan->cta_floats;
  a.n_cta = plan->n_cta;
  a.has_prior = plan->has_prior;
  for (int i = 0; i < GL_MAX_PARAMS; ++i) a.prior[i] = plan->prior[i];
  a.img_stride = plan->max_pix;
}

}  // namespace gl

using namespace gl;

extern "C" {

int gl_abi_version(void) { return GL_ABI_VERSION; }

int gl_struct_size(int which) {
  switch (which) {
    case 0: return (int)sizeof(gl_profile_desc);
    case 1: return (int)sizeof(gl_model_desc);
    case 2: return (int)sizeof(gl_image_desc);
    case 3: return (int)sizeof(gl_prior_leaf);
    case 4: return (int)sizeof(gl_tune_result);
    case 5: return (int)sizeof(gl_adam_cfg);
    case 6: return (int)sizeof(gl_tuning);
    default: return -1;
  }
}

const char* gl_last_error(void) { return g_err; }

int gl_device_info(int* sm_count, int* smem_optin_bytes) {
  int dev = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (sm_count) cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (smem_optin_bytes)
    cudaDeviceGetAttribute(smem_optin_bytes, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return GL_OK;
}

int gl_plan_create(const gl_model_desc* model, const gl_image_desc* images, int n_images,
                   gl_plan** out) {
  GL_NVTX_RANGE("gl_plan_create");
  if (!model || !images || !out || n_images < 1 || n_images > GL_MAX_IMAGES) {
    set_error("gl_plan_create: bad arguments (n_images %d)", n_images);
    return GL_ERR_INVALID;
  }
  *out = nullptr;
  if (model->n_profiles < 1 || model->n_profiles > GL_MAX_PROFILES || model->n_params < 1 ||
      model->n_params > GL_MAX_PARAMS) {
    set_error("gl_plan_create: bad model (n_profiles %d, n_params %d)", model->n_profiles,
              model->n_params);
    return GL_ERR_INVALID;
  }
  for (int i = 0; i < model->n_profiles; ++i) {
    const gl_profile_desc& p = model->prof[i];
    const int np = param_count(p.type);
    if (np < 0) {
      set_error("profile %d: unknown type %d", i, p.type);
      return GL_ERR_INVALID;
    }
    for (int k = 0; k < np; ++k)
      if (p.col[k] < -1 || p.col[k] >= model->n_params) {
        set_error("profile %d parameter %d: column %d out of range", i, k, p.col[k]);
        return GL_ERR_INVALID;
      }
  }
  gl_plan* plan = new gl_plan;
  memset(plan, 0, sizeof(*plan));
  plan->model = *model;
  plan->n_images = n_images;
  // a model whose light is solved linearly runs on the least-squares kernels
  bool lsq_model = false;
  for (int i = 0; i < model->n_profiles; ++i)
    if (model->prof[i].group != GL_GROUP_LENS && model->prof[i].use_lstsq) lsq_model = true;
  int rc = GL_OK;
  if (lsq_model) {
    plan->family = -1;
    // the general path with the coefficients as amplitudes (gl_lstsq_grad)
    DevProfile e, sh;
    plan->gen_ok = resolve_generic(model, true, &plan->gen, &e, &sh) == GL_OK;
    plan->gen_family = FAM_GENERIC;
    if (plan->gen_ok) {
      plan->epl = e;
      plan->shear = sh;
      plan->gen_family = gen_signature(plan->gen);
    }
    set_error("");
  } else if (!resolve_family(model, &plan->family, &plan->epl, &plan->shear, &plan->llight,
                             &plan->source)) {
    rc = resolve_generic(model, false, &plan->gen, &plan->epl, &plan->shear);
    plan->gen_ok = rc == GL_OK;
    plan->family = plan->gen_ok ? gen_signature(plan->gen) : FAM_GENERIC;
    plan->gen_family = plan->family;
  }
  if (!rc && plan->epl.type == GL_PROF_EPL && (plan->epl.niter < 0 || plan->epl.niter > kMaxTerms)) {
    set_error("EPL niter %d outside [0, %d]", plan->epl.niter, kMaxTerms);
    rc = GL_ERR_UNSUPPORTED;
  }
  if (rc) {
    delete plan;
    return rc;
  }
  rc = cuda_check(cudaGetDevice(&plan->device), "cudaGetDevice");
  if (rc) {
    delete plan;
    return rc;
  }
  std::vector<HostImage> hi(n_images);
  size_t bytes = 0;
  int smem_floats = 0;
  for (int i = 0; i < n_images; ++i) {
    plan->host_img[i] = images[i];
    rc = build_image(images[i], plan->img[i], hi[i]);
    if (rc) {
      delete plan;
      return rc;
    }
    bytes += align_up(hi[i].obs.size() * 4, 256) + align_up(hi[i].grid.size() * 4, 256) +
             align_up(hi[i].kern.size() * 4, 256) + align_up(hi[i].err.size() * 4, 256);
    if (plan->img[i].smem_floats > smem_floats) smem_floats = plan->img[i].smem_floats;
    const int pix = images[i].num_pix * images[i].num_pix;
    if (pix > plan->max_pix) plan->max_pix = pix;
  }
  int dev_smem = 0;
  cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, plan->device);
  plan->smem_bytes = smem_floats * 4;
  const int static_smem = lsq_model ? 0 : fused_static_smem_bytes();
  (void)static_smem;
  plan->fused_fits = plan->smem_bytes + fused_static_smem_bytes() <= dev_smem;
  // The general path keeps its planes in global memory at every size: its
  // per-thread accumulator arrays live in local memory, which hits L1 only
  // when shared memory is not carved out for the planes (90^2 px: 262 k ->
  // 288 k evals/s).
  // The compiled signatures keep them in shared memory when they fit.
  if (plan->family == FAM_GENERIC || (lsq_model && plan->gen_ok && plan->gen_family == FAM_GENERIC))
    plan->fused_fits = 0;
  rc = cuda_check(cudaMalloc((void**)&plan->dev_buf, bytes), "cudaMalloc(plan)");
  if (rc) {
    delete plan;
    return rc;
  }
  if (!plan->fused_fits && !lsq_model && !is_gen_family(plan->family) &&
      plan->family != FAM_EPL_SHEAR_SE_SE) {
    // planes in global memory: the headline family and the general path
    rc = resolve_generic(model, false, &plan->gen, &plan->epl, &plan->shear);
    if (rc) {
      cudaFree(plan->dev_buf);
      delete plan;
      return rc;
    }
    plan->family = gen_signature(plan->gen);
    plan->gen_family = plan->family;
    plan->gen_ok = 1;
  }
  if (!plan->fused_fits && (!lsq_model || plan->gen_ok)) {
    // the image planes of one CTA exceed shared memory: give every CTA a
    // slice of global memory (it stays in L2 for the launch)
    cudaDeviceGetAttribute(&plan->n_cta, cudaDevAttrMultiProcessorCount, plan->device);
    plan->cta_floats = (int)align_up((size_t)smem_floats, 64);
    rc = cuda_check(cudaMalloc((void**)&plan->gscratch,
                               (size_t)plan->n_cta * plan->cta_floats * sizeof(float)),
                    "cudaMalloc(plane scratch)");
    if (rc) {
      cudaFree(plan->dev_buf);
      delete plan;
      return rc;
    }
  }
  plan->dev_buf_bytes = bytes;
  char* base = (char*)plan->dev_buf;
  for (int i = 0; i < n_images; ++i) {
    DevImage& I = plan->img[i];
    auto put = [&](const std::vector<float>& v) -> const float* {
      if (v.empty()) return nullptr;
      const float* p = (const float*)base;
      cudaMemcpy((void*)p, v.data(), v.size() * 4, cudaMemcpyHostToDevice);
      base += align_up(v.size() * 4, 256);
      return p;
    };
    I.obs = put(hi[i].obs);
    I.grid = put(hi[i].grid);
    I.kern = put(hi[i].kern);
    I.err = put(hi[i].err);
  }
  rc = cuda_check(cudaGetLastError(), "plan upload");
  // the table of the interpolating shapelet profiles (Shapelets(interpolate=True))
  for (int i = 0; i < model->n_profiles && !rc; ++i)
    if (model->prof[i].type == GL_PROF_SHAPELETS && model->prof[i].interpolate && !plan->shp_tab)
      rc = shapelet_table(plan->device, &plan->shp_tab);
  plan->gen.shp_tab = plan->shp_tab;
  if (!rc && plan->fused_fits && (!lsq_model || plan->gen_ok)) rc = fused_kernel_prepare(plan->smem_bytes);
  if (!rc && lsq_model) {
    std::vector<std::vector<float>> errs(n_images);
    for (int i = 0; i < n_images; ++i) errs[i] = hi[i].err;
    rc = lsq_prepare(plan, errs);
  }
  if (rc) {
    cudaFree(plan->dev_buf);
    if (plan->gscratch) cudaFree(plan->gscratch);
    delete plan;
    return rc;
  }
  *out = plan;
  return GL_OK;
}

int gl_plan_set_prior(gl_plan* plan, const gl_prior_leaf* leaves, int n_leaves) {
  if (!plan || !leaves || n_leaves != plan->model.n_params) {
    set_error("gl_plan_set_prior: need one leaf per parameter (%d)", plan ? plan->model.n_params : -1);
    return GL_ERR_INVALID;
  }
  for (int i = 0; i < n_leaves; ++i) {
    const gl_prior_leaf& l = leaves[i];
    const bool ok = (l.dist == GL_DIST_NORMAL || l.dist == GL_DIST_LOGNORMAL) ? l.b > 0.f
                    : l.dist == GL_DIST_UNIFORM                            ? l.b > l.a
                    : l.dist == GL_DIST_TRUNCNORMAL                        ? (l.b > 0.f && l.d > l.c)
                                                                           : false;
    if (!ok) {
      set_error("prior leaf %d: bad distribution %d or parameters", i, l.dist);
      return GL_ERR_INVALID;
    }
    plan->prior[i] = make_leaf(l);
  }
  plan->has_prior = 1;
  return GL_OK;
}

int gl_plan_destroy(gl_plan* plan) {
  if (!plan) return GL_OK;
  lsq_destroy(plan);
  if (plan->dev_buf) cudaFree(plan->dev_buf);
  if (plan->gscratch) cudaFree(plan->gscratch);
  delete plan;
  return GL_OK;
}

int gl_lstsq_workspace(const gl_plan* plan, int bs, size_t* bytes, int* n_channels) {
  if (!plan || bs < 0 || !bytes) {
    set_error("gl_lstsq_workspace: bad arguments");
    return GL_ERR_INVALID;
  }
  if (!plan->lsq) {
    set_error("the plan has no linear-amplitude light profiles");
    return GL_ERR_INVALID;
  }
  *bytes = lsq_workspace_bytes((const LsqPlan*)plan->lsq, bs);
  if (n_channels) *n_channels = ((const LsqPlan*)plan->lsq)->D;
  return GL_OK;
}

int gl_lstsq(const gl_plan* plan, const float* x, const int* img_id, int bs, void* work,
             size_t work_bytes, float* coeffs, float* img_out, float* logL, float* chi2,
             void* stream) {
  GL_NVTX_RANGE("gl_lstsq");
  if (!plan || (bs > 0 && (!x || !work || !coeffs)) || bs < 0) {
    set_error("gl_lstsq: null plan, input, workspace or coeffs");
    return GL_ERR_INVALID;
  }
  if (!plan->lsq) {
    set_error("the plan has no linear-amplitude light profiles");
    return GL_ERR_INVALID;
  }
  int rc = check_device(plan);
  if (rc) return rc;
  if (logL || chi2)
    for (int i = 0; i < plan->n_images; ++i)
      if (!plan->img[i].obs) {
        set_error("image %d has no observed data", i);
        return GL_ERR_INVALID;
      }
  return lsq_run(plan, x, img_id, bs, (float*)work, work_bytes, coeffs, img_out, logL, chi2,
                 (cudaStream_t)stream);
}

int gl_plan_query(const gl_plan* plan, int* smem_bytes, int* threads_per_block, int* max_img_pix) {
  if (!plan) {
    set_error("gl_plan_query: null plan");
    return GL_ERR_INVALID;
  }
  if (smem_bytes) *smem_bytes = plan->smem_bytes;
  if (threads_per_block) *threads_per_block = kThreads;
  if (max_img_pix) *max_img_pix = plan->max_pix;
  return GL_OK;
}

static int grad_checks(const gl_plan* plan) {
  if (is_gen_family(plan->family) && plan->gen.explicit_shapelets > 1) {
    set_error("gradients with respect to the amplitudes of more than one explicit shapelet "
              "profile are not implemented; use Shapelets(use_lstsq=True)");
    return GL_ERR_UNSUPPORTED;
  }
  return GL_OK;
}

static int common_checks(const gl_plan* plan, const float* x, int bs) {
  if (!plan || (bs > 0 && !x) || bs < 0) {
    set_error("null plan / input or negative batch");
    return GL_ERR_INVALID;
  }
  if (plan->family < 0) {
    set_error("the plan's light profiles are solved linearly: use gl_lstsq");
    return GL_ERR_UNSUPPORTED;
  }
  return check_device(plan);
}

int gl_forward(const gl_plan* plan, const float* x, const int* img_id, int bs, float* logL,
               float* chi2, float* img_out, int* status, void* stream) {
  GL_NVTX_RANGE("gl_forward");
  int rc = common_checks(plan, x, bs);
  if (rc) return rc;
  if ((logL || chi2))
    for (int i = 0; i < plan->n_images; ++i)
      if (!plan->img[i].obs) {
        set_error("image %d has no observed data; pass logL = chi2 = NULL", i);
        return GL_ERR_INVALID;
      }
  FusedArgs a;
  fill_args(plan, a);
  a.bs = bs;
  a.x = x;
  a.img_id = img_id;
  a.logL = logL;
  a.chi2 = chi2;
  a.img_out = img_out;
  a.status = status;
  return launch_fused(a, plan->smem_bytes, (cudaStream_t)stream);
}

int gl_forward_grad(const gl_plan* plan, const float* x, const int* img_id, int bs, float* logL,
                    float* chi2, float* dlogL_dx, int* status, void* stream) {
  GL_NVTX_RANGE("gl_forward_grad");
  int rc = common_checks(plan, x, bs);
  if (!rc && dlogL_dx) rc = grad_checks(plan);
  if (rc) return rc;
  for (int i = 0; i < plan->n_images; ++i)
    if (!plan->img[i].obs) {
      set_error("image %d has no observed data", i);
      return GL_ERR_INVALID;
    }
  FusedArgs a;
  fill_args(plan, a);
  a.bs = bs;
  a.x = x;
  a.img_id = img_id;
  a.logL = logL;
  a.chi2 = chi2;
  a.grad = dlogL_dx;
  a.status = status;
  a.want_grad = dlogL_dx != nullptr;
  return launch_fused(a, plan->smem_bytes, (cudaStream_t)stream);
}

int gl_adjoint(const gl_plan* plan, const float* x, const int* img_id, int bs, const float* dlogL,
               float* dx, int* status, void* stream) {
  GL_NVTX_RANGE("gl_adjoint");
  int rc = common_checks(plan, x, bs);
  if (!rc) rc = grad_checks(plan);
  if (rc) return rc;
  if (!dx || !dlogL) {
    set_error("gl_adjoint: dlogL and dx are required");
    return GL_ERR_INVALID;
  }
  FusedArgs a;
  fill_args(plan, a);
  a.bs = bs;
  a.x = x;
  a.img_id = img_id;
  a.dlogL = dlogL;
  a.grad = dx;
  a.status = status;
  a.want_grad = 1;
  return launch_fused(a, plan->smem_bytes, (cudaStream_t)stream);
}

int gl_log_prob(const gl_plan* plan, const float* z, const int* img_id, int bs, float* logp,
                float* chi2, float* dlogp_dz, int* status, void* stream) {
  GL_NVTX_RANGE("gl_log_prob");
  int rc = common_checks(plan, z, bs);
  if (!rc && dlogp_dz) rc = grad_checks(plan);
  if (rc) return rc;
  if (!plan->has_prior) {
    set_error("gl_log_prob: the plan has no prior (gl_plan_set_prior)");
    return GL_ERR_INVALID;
  }
  FusedArgs a;
  fill_args(plan, a);
  a.bs = bs;
  a.x = z;
  a.img_id = img_id;
  a.logL = logp;
  a.chi2 = chi2;
  a.grad = dlogp_dz;
  a.status = status;
  a.zmode = 1;
  a.want_grad = dlogp_dz != nullptr;
  return launch_fused(a, plan->smem_bytes, (cudaStream_t)stream);
}

int gl_autotune(const gl_plan* plan, int bs, gl_tune_result* out) {
  if (!plan || !out || bs < 0) {
    set_error("gl_autotune: null plan or result, or negative batch");
    return GL_ERR_INVALID;
  }
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, plan->device);
  memset(out, 0, sizeof(*out));
  out->threads_per_block = kThreads;
  out->blocks = bs < sms ? bs : sms;
  out->samples_per_cta = out->blocks ? (bs + out->blocks - 1) / out->blocks : 0;
  out->global_planes = plan->gscratch != nullptr;
  out->smem_bytes = out->global_planes ? 0 : plan->smem_bytes;
  out->family = plan->family;
  for (int i = 0; i < plan->n_images; ++i)
    if (plan->img[i].KS > out->subkernel_side) out->subkernel_side = plan->img[i].KS;
  out->col_block = kFusedCB;
  return GL_OK;
}

int gl_lstsq_grad(const gl_plan* plan, const float* x, const int* img_id, int bs,
                  const float* coeffs, float* logL, float* chi2, float* grad, void* stream) {
  GL_NVTX_RANGE("gl_lstsq_grad");
  if (!plan || bs < 0 || (bs > 0 && (!x || !coeffs || !grad))) {
    set_error("gl_lstsq_grad: null plan, input, coefficients or gradient, or negative batch");
    return GL_ERR_INVALID;
  }
  if (!plan->lsq) {
    set_error("gl_lstsq_grad: the plan's light profiles are not solved linearly");
    return GL_ERR_INVALID;
  }
  if (!plan->gen_ok || plan->gen.n_amp != ((const LsqPlan*)plan->lsq)->D) {
    set_error("gl_lstsq_grad: the model is not supported by the fused kernel's general path");
    return GL_ERR_UNSUPPORTED;
  }
  int rc = check_device(plan);
  if (rc) return rc;
  for (int i = 0; i < plan->n_images; ++i)
    if (!plan->img[i].obs || !plan->img[i].err) {
      set_error("image %d has no observed data", i);
      return GL_ERR_INVALID;
    }
  FusedArgs a;
  fill_args(plan, a);
  a.family = plan->gen_family;
  a.gen.amps = coeffs;
  a.gen.noise_err = 1;
  a.gen.unit_cf = 1;
  a.bs = bs;
  a.x = x;
  a.img_id = img_id;
  a.logL = logL;
  a.chi2 = chi2;
  a.grad = grad;
  a.want_grad = 1;
  return launch_fused(a, plan->smem_bytes, (cudaStream_t)stream);
}

int gl_bijector_forward(const gl_plan* plan, const float* z, int bs, float* x, void* stream) {
  int rc = common_checks(plan, z, bs);
  if (rc) return rc;
  if (!plan->has_prior || !x) {
    set_error("gl_bijector_forward: plan has no prior or x is null");
    return GL_ERR_INVALID;
  }
  return launch_bijector_forward(plan->prior, plan->model.n_params, z, bs, x, (cudaStream_t)stream);
}

int gl_profile_eval(int type, const float* x, const float* y, int64_t n, const float* params,
                    const int* n_terms, float* out0, float* out1, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y || !params || !out0))) {
    set_error("gl_profile_eval: null pointer or negative size");
    return GL_ERR_INVALID;
  }
  const bool mass = type == GL_PROF_EPL || type == GL_PROF_SHEAR || type == GL_PROF_SIS ||
                    type == GL_PROF_SIE || type == GL_PROF_TNFW;
  if (mass && !out1) {
    set_error("gl_profile_eval: mass profiles need out1");
    return GL_ERR_INVALID;
  }
  if (type == GL_PROF_EPL && !n_terms) {
    set_error("gl_profile_eval: EPL needs the device term count");
    return GL_ERR_INVALID;
  }
  return launch_profile_eval(type, x, y, n, params, n_terms, out0, out1, (cudaStream_t)stream);
}

int gl_shapelets_eval(int n_max, int interpolate, const float* x, const float* y, int64_t n,
                      const float* params, const float* amps, float* out, void* stream) {
  if (n_max < 0 || n_max >= kShpTabRows || n < 0 || (n > 0 && (!x || !y || !params || !out))) {
    set_error("gl_shapelets_eval: bad arguments");
    return GL_ERR_INVALID;
  }
  const float* tab = nullptr;
  if (interpolate) {
    int dev = 0;
    cudaGetDevice(&dev);
    const int rc = shapelet_table(dev, &tab);
    if (rc) return rc;
  }
  return launch_shapelets_eval(n_max, tab, x, y, n, params, amps, out, (cudaStream_t)stream);
}

int gl_epl_term_count(const float* e1, const float* e2, int64_t n, int cap, int* k_out,
                      void* stream) {
  if (n < 1 || !e1 || !e2 || !k_out || cap < 0) {
    set_error("gl_epl_term_count: bad arguments");
    return GL_ERR_INVALID;
  }
  return launch_epl_term_count(e1, e2, n, cap, k_out, (cudaStream_t)stream);
}

}  // extern "C"
