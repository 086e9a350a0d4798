// Host dispatch of the fused forward + adjoint kernel over its families (the
// kernel itself is in gl_fused.cuh; each family is its own translation unit,
// gl_fused_fam*.cu).
#include <algorithm>

#include "gl_internal.cuh"
#include "gl_fused_ops.cuh"

namespace gl {

static int g_sm_count[kMaxDevices];   // per device, 0 until read
static int g_smem_set[kMaxDevices];   // dynamic smem attribute set per device (only ever raised)

// Largest static shared-memory footprint over the fused kernel's families.
int fused_static_smem_bytes() {
  return std::max({fam_static_smem<FAM_EPL_SHEAR_SE_SE>(), fam_static_smem<FAM_EPL_SHEAR_SE>(),
                   fam_static_smem<FAM_EPL_SE_SE>(), fam_static_smem<FAM_EPL_SE>(),
                   fam_static_smem<FAM_GENERIC>(), fam_static_smem<FAM_SIG_SIE_SHEAR_SE_SE>(),
                   fam_static_smem<FAM_SIG_SIS_SHEAR_SE_SE>(), fam_static_smem<FAM_SIG_EPL_SHEAR_SHP>()});
}

int fused_kernel_prepare(int smem_bytes) {
  const int dev = current_device_slot();
  if (smem_bytes <= g_smem_set[dev]) return GL_OK;
  cudaError_t e = fam_set_smem<FAM_EPL_SHEAR_SE_SE>(smem_bytes);
  if (e == cudaSuccess) e = fam_set_smem<FAM_EPL_SHEAR_SE>(smem_bytes);
  if (e == cudaSuccess) e = fam_set_smem<FAM_EPL_SE_SE>(smem_bytes);
  if (e == cudaSuccess) e = fam_set_smem<FAM_EPL_SE>(smem_bytes);
  if (e == cudaSuccess) e = fam_set_smem<FAM_EPL_SHEAR_SE_SE, false>(smem_bytes);
  if (e == cudaSuccess) e = fam_set_smem<FAM_SIG_SIE_SHEAR_SE_SE>(smem_bytes);
  if (e == cudaSuccess) e = fam_set_smem<FAM_SIG_SIS_SHEAR_SE_SE>(smem_bytes);
  if (e == cudaSuccess) e = fam_set_smem<FAM_SIG_EPL_SHEAR_SHP>(smem_bytes);
  if (e != cudaSuccess) {
    set_error("cudaFuncSetAttribute(max dynamic smem %d): %s", smem_bytes, cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  g_smem_set[dev] = smem_bytes;
  return GL_OK;
}

int launch_fused(const FusedArgs& a, int smem_bytes, cudaStream_t stream) {
  if (a.bs <= 0) return GL_OK;
  const int dev = current_device_slot();
  if (g_sm_count[dev] == 0) {
    int d = 0, n = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d);
    g_sm_count[dev] = n > 0 ? n : 1;
  }
  int grid = a.bs < g_sm_count[dev] ? a.bs : g_sm_count[dev];
  if (a.gscratch) {
    if (grid > a.n_cta) grid = a.n_cta;   // one plane slice per CTA
    // planes in global memory: the headline family and the general path
    // have such instantiations (plan creation routes the others to the latter)
    switch (a.family) {
      case FAM_EPL_SHEAR_SE_SE: fam_launch<FAM_EPL_SHEAR_SE_SE, true>(a, grid, 0, stream); break;
      case FAM_GENERIC: fam_launch<FAM_GENERIC, true>(a, grid, 0, stream); break;
      case FAM_SIG_SIE_SHEAR_SE_SE: fam_launch<FAM_SIG_SIE_SHEAR_SE_SE, true>(a, grid, 0, stream); break;
      case FAM_SIG_SIS_SHEAR_SE_SE: fam_launch<FAM_SIG_SIS_SHEAR_SE_SE, true>(a, grid, 0, stream); break;
      case FAM_SIG_EPL_SHEAR_SHP: fam_launch<FAM_SIG_EPL_SHEAR_SHP, true>(a, grid, 0, stream); break;
      default:
        set_error("model family %d has no global-memory plane kernel", a.family);
        return GL_ERR_INVALID;
    }
  } else {
    switch (a.family) {
      case FAM_EPL_SHEAR_SE_SE:
        if (a.corr_scalar)
          fam_launch<FAM_EPL_SHEAR_SE_SE, false, false>(a, grid, smem_bytes, stream);
        else
          fam_launch<FAM_EPL_SHEAR_SE_SE, false>(a, grid, smem_bytes, stream);
        break;
      case FAM_EPL_SHEAR_SE: fam_launch<FAM_EPL_SHEAR_SE, false>(a, grid, smem_bytes, stream); break;
      case FAM_EPL_SE_SE: fam_launch<FAM_EPL_SE_SE, false>(a, grid, smem_bytes, stream); break;
      case FAM_EPL_SE: fam_launch<FAM_EPL_SE, false>(a, grid, smem_bytes, stream); break;
      case FAM_SIG_SIE_SHEAR_SE_SE:
        fam_launch<FAM_SIG_SIE_SHEAR_SE_SE, false>(a, grid, smem_bytes, stream);
        break;
      case FAM_SIG_SIS_SHEAR_SE_SE:
        fam_launch<FAM_SIG_SIS_SHEAR_SE_SE, false>(a, grid, smem_bytes, stream);
        break;
      case FAM_SIG_EPL_SHEAR_SHP: fam_launch<FAM_SIG_EPL_SHEAR_SHP, false>(a, grid, smem_bytes, stream); break;
      case FAM_GENERIC:
        set_error("the general path needs the plan's global plane scratch");
        return GL_ERR_INVALID;
      default:
        set_error("unknown model family %d", a.family);
        return GL_ERR_INVALID;
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("fused kernel launch: %s", cudaGetErrorString(e));
    return GL_ERR_CUDA;
  }
  return GL_OK;
}

}  // namespace gl
