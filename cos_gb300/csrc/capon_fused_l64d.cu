// Fused element-space kernel, L = 64, any T, 8 warps, any M (its smaller tile
// fits larger M than the 12-warp one): the z/P, w and R modes (the blocked
// per-pixel path of capon_fused_wide.cuh).  The refinement modes of
// the same configuration are in capon_fused_l64d_refine.cu, so that the two
// compile in parallel; the candidate table is in capon_fused_l64.cu.
#include "capon_fused.cuh"

namespace cgb {
using CL64D = fused::Cfg<64, 32, 8, 2, 0, 0, false>;
int fused_l64d_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_basic<CL64D>(fp, mode, st, n, s);
}
size_t fused_l64d_smem(int K, int M) { return fused::smem_bytes<CL64D>(K, M); }
}  // namespace cgb
