// The refinement modes at L = 16 (every pixel, or the ill-conditioned ones):
// the blocked per-pixel path of capon_fused_wide.cuh at 8 lanes per pixel,
// four pixels per warp (two blocks of 8 rows), any temporal window and
// channel count.  The L = 16 candidate tables list it after their own
// configurations; it reports cudaErrorNotSupported for the z/P, w and R
// modes, which the L = 16 kernel serves.
#include "capon_fused.cuh"

namespace cgb {
using CL16R = fused::Cfg<16, 8, 8, 1, 0, 0, false, true>;
int fused_l16r_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_refine_only<CL16R>(fp, mode, st, n, s);
}
size_t fused_l16r_smem(int K, int M) { return fused::smem_bytes<CL16R>(K, M); }
size_t fused_l16r_stash(int num_sms) { return fused::stash_bytes<CL16R>(num_sms); }
}  // namespace cgb
