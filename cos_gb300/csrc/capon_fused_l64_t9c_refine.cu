// Fused element-space kernel, L = 64, T = 9, 8 warps, any M: the refinement modes
// (every pixel, or the ill-conditioned ones), with the bytes of stash they need.
#include "capon_fused.cuh"

namespace cgb {
using CL64T9C = fused::Cfg<64, 32, 8, 2, 9, 0, false>;
int fused_l64_t9c_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_refining<CL64T9C>(fp, mode, st, n, s);
}
size_t fused_l64_t9c_stash(int num_sms) { return fused::stash_bytes<CL64T9C>(num_sms); }
}  // namespace cgb
