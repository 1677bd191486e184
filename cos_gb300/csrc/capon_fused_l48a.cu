// Fused element-space kernel, L = 48, any T, 8 warps x 2 pixels, any M: the z/P, w and R modes (the
// blocked per-pixel path of capon_fused_wide.cuh).  The refinement modes of
// the same configuration are in capon_fused_l48a_refine.cu, so that the two
// compile in parallel; the candidate table is in capon_fused_l48.cu.
#include "capon_fused.cuh"

namespace cgb {
using CL48A = fused::Cfg<48, 16, 8, 1, 0, 0, true>;
int fused_l48a_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_basic<CL48A>(fp, mode, st, n, s);
}
size_t fused_l48a_smem(int K, int M) { return fused::smem_bytes<CL48A>(K, M); }
}  // namespace cgb
