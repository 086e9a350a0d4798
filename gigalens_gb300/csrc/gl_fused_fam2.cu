// Fused kernel, family FAM_EPL_SE_SE (one translation unit per family).
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_EPL_SE_SE, false>(const FusedArgs&, int, int, cudaStream_t);
template cudaError_t fam_set_smem<FAM_EPL_SE_SE>(int);
template int fam_static_smem<FAM_EPL_SE_SE>();
}  // namespace gl
