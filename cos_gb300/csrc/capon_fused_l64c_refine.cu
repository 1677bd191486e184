// Fused element-space kernel, L = 64, any T, 12 warps, any M: the refinement modes
// (every pixel, or the ill-conditioned ones), with the bytes of stash they need.
#include "capon_fused.cuh"

namespace cgb {
using CL64C = fused::Cfg<64, 32, 12, 1, 0, 0, false>;
int fused_l64c_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_refining<CL64C>(fp, mode, st, n, s);
}
size_t fused_l64c_stash(int num_sms) { return fused::stash_bytes<CL64C>(num_sms); }
}  // namespace cgb
