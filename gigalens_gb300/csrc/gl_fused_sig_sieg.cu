// Fused kernel, general path compiled for FAM_SIG_SIE_SHEAR_SE_SE (SIE + shear, SersicEllipse lens light and source), with the image planes in a per-CTA slice of global memory.
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_SIG_SIE_SHEAR_SE_SE, true>(const FusedArgs&, int, int, cudaStream_t);
}  // namespace gl
