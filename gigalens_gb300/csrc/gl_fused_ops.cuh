// Per-family host entries of the fused kernel (defined in gl_fused.cuh,
// instantiated in gl_fused_fam*.cu).
#pragma once
#include "gl_internal.cuh"

namespace gl {
template <int FAM, bool GMEM, bool X2 = true>
int fam_launch(const FusedArgs& a, int grid, int smem_bytes, cudaStream_t stream);
template <int FAM, bool X2 = true>
cudaError_t fam_set_smem(int smem_bytes);
template <int FAM>
int fam_static_smem();
}  // namespace gl
