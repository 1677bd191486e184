// Fused element-space kernel for L = 64, temporal window T = 9, 8 warps, any M
// (one warp per pixel, the blocked per-pixel path of capon_fused_wide.cuh).
// One configuration per file so that the configurations compile in parallel;
// the candidate table is in capon_fused_l64_t9.cu.
#include "capon_fused.cuh"

namespace cgb {
using CL64T9c = fused::Cfg<64, 32, 8, 2, 9, 0, false>;
int fused_l64_t9c_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_any<CL64T9c>(fp, mode, st, n, s);
}
size_t fused_l64_t9c_smem(int K, int M) { return fused::smem_bytes<CL64T9c>(K, M); }
size_t fused_l64_t9c_stash(int num_sms) { return fused::stash_bytes<CL64T9c>(num_sms); }
}  // namespace cgb
