// Fused kernel, family FAM_GENERIC (one translation unit per family).
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_GENERIC, false>(const FusedArgs&, int, int, cudaStream_t);
template cudaError_t fam_set_smem<FAM_GENERIC>(int);
template int fam_static_smem<FAM_GENERIC>();
}  // namespace gl
