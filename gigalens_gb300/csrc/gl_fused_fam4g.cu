// Fused kernel, family FAM_GENERIC (the general path) with the image planes in a
// per-CTA slice of global memory (images whose planes exceed shared memory).
#include "gl_fused.cuh"

namespace gl {
template int fam_launch<FAM_GENERIC, true>(const FusedArgs&, int, int, cudaStream_t);
}  // namespace gl
