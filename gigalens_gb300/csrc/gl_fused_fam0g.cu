// Fused kernel, family FAM_EPL_SHEAR_SE_SE (EPL + shear, Sersic lens light and source) with the image planes in a
// per-CTA slice of global memory (images whose planes exceed shared memory).
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_EPL_SHEAR_SE_SE, true>(const FusedArgs&, int, int, cudaStream_t);
}  // namespace gl
