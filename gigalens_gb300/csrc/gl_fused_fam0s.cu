// Fused kernel, family FAM_EPL_SHEAR_SE_SE with scalar-FFMA PSF correlations
// (a tuning alternative to the packed-FFMA2 instantiation in gl_fused_fam0.cu).
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_EPL_SHEAR_SE_SE, false, false>(const FusedArgs&, int, int, cudaStream_t);
template cudaError_t fam_set_smem<FAM_EPL_SHEAR_SE_SE, false>(int);
}  // namespace gl
