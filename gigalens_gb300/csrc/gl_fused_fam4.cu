// Fused kernel, family FAM_GENERIC (the general path), which keeps its image
// planes in a per-CTA slice of global memory at every image size.
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_GENERIC, true>(const FusedArgs&, int, int, cudaStream_t);
template int fam_static_smem<FAM_GENERIC>();
}  // namespace gl
