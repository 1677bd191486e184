// The refinement modes at L = 32 (every pixel, or the ill-conditioned ones):
// the blocked per-pixel path of capon_fused_wide.cuh at 16 lanes per pixel
// (two pixels per warp, two blocks of 16 rows), any temporal window and
// channel count.  The
// L = 32 candidate tables list it after their own configurations; it reports
// cudaErrorNotSupported for the z/P, w and R modes, which the L = 32 kernel
// serves.
#include "capon_fused.cuh"

namespace cgb {
using CL32R = fused::Cfg<32, 16, 12, 1, 0, 0, false, true>;
int fused_l32r_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_refine_only<CL32R>(fp, mode, st, n, s);
}
size_t fused_l32r_smem(int K, int M) { return fused::smem_bytes<CL32R>(K, M); }
size_t fused_l32r_stash(int num_sms) { return fused::stash_bytes<CL32R>(num_sms); }
}  // namespace cgb
