// Fused element-space kernel, L = 48, any T, 8 warps x 2 pixels, any M: the refinement modes
// (every pixel, or the ill-conditioned ones), with the bytes of stash they need.
#include "capon_fused.cuh"

namespace cgb {
using CL48A = fused::Cfg<48, 16, 8, 1, 0, 0, true>;
int fused_l48a_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_refining<CL48A>(fp, mode, st, n, s);
}
size_t fused_l48a_stash(int num_sms) { return fused::stash_bytes<CL48A>(num_sms); }
}  // namespace cgb
