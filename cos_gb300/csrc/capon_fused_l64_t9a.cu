// Fused element-space kernel for L = 64, temporal window T = 9, 12 warps, M = 128
// (one warp per pixel, the blocked per-pixel path of capon_fused_wide.cuh).
// One configuration per file so that the configurations compile in parallel;
// the candidate table is in capon_fused_l64_t9.cu.
#include "capon_fused.cuh"

namespace cgb {
using CL64T9a = fused::Cfg<64, 32, 12, 1, 9, 128, false>;
int fused_l64_t9a_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_any<CL64T9a>(fp, mode, st, n, s);
}
size_t fused_l64_t9a_smem(int K, int M) { return fused::smem_bytes<CL64T9a>(K, M); }
size_t fused_l64_t9a_stash(int num_sms) { return fused::stash_bytes<CL64T9a>(num_sms); }
}  // namespace cgb
