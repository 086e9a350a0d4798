// Fused kernel, general path compiled for FAM_SIG_EPL_SHEAR_SHP (EPL + shear, shapelet source (the BackwardProbModel gradient)), with the image planes in shared memory.
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_SIG_EPL_SHEAR_SHP, false>(const FusedArgs&, int, int, cudaStream_t);
template cudaError_t fam_set_smem<FAM_SIG_EPL_SHEAR_SHP>(int);
template int fam_static_smem<FAM_SIG_EPL_SHEAR_SHP>();
}  // namespace gl
