// Fused kernel, general path compiled for FAM_SIG_EPL_SHEAR_SHP (EPL + shear, shapelet source (the BackwardProbModel gradient)), with the image planes in a per-CTA slice of global memory.
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_SIG_EPL_SHEAR_SHP, true>(const FusedArgs&, int, int, cudaStream_t);
}  // namespace gl
