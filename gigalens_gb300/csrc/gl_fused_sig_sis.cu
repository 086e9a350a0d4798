// Fused kernel, general path compiled for FAM_SIG_SIS_SHEAR_SE_SE (SIS + shear, SersicEllipse lens light and source), with the image planes in shared memory.
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_SIG_SIS_SHEAR_SE_SE, false>(const FusedArgs&, int, int, cudaStream_t);
template cudaError_t fam_set_smem<FAM_SIG_SIS_SHEAR_SE_SE>(int);
template int fam_static_smem<FAM_SIG_SIS_SHEAR_SE_SE>();
}  // namespace gl
