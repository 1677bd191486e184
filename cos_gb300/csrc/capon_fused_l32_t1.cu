// Fused element-space kernel instantiations for L = 32, temporal window T = 1.
// The autotuner in capon_api.cu picks one per (L, K, M) shape; a candidate
// compiled for a fixed M reports cudaErrorNotSupported for other M.
#include "capon_fused.cuh"

namespace cgb {
int fused_l32r_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l32r_smem(int K, int M);
size_t fused_l32r_stash(int num_sms);

namespace {
int launch_0(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_any<fused::Cfg<32, 8, 8, 2, 1, 64, true>>(fp, mode, st, n, s);
}
int launch_1(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_any<fused::Cfg<32, 8, 8, 2, 1, 64, false>>(fp, mode, st, n, s);
}
int launch_2(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_any<fused::Cfg<32, 8, 8, 2, 1, 0, true>>(fp, mode, st, n, s);
}

const FusedCandidate kCand[] = {
    {"L32.G8.W8.N2.sync.M64.T1", 32, 1, 64, launch_0, fused::smem_bytes<fused::Cfg<32, 8, 8, 2, 1, 64, true>>},
    {"L32.G8.W8.N2.M64.T1", 32, 1, 64, launch_1, fused::smem_bytes<fused::Cfg<32, 8, 8, 2, 1, 64, false>>},
    {"L32.G8.W8.N2.sync.T1", 32, 1, 0, launch_2, fused::smem_bytes<fused::Cfg<32, 8, 8, 2, 1, 0, true>>},
    // the refinement modes (capon_fused_l32r.cu)
    {"L32.G16.W12.refine", 32, 0, 0, fused_l32r_launch, fused_l32r_smem, fused_l32r_stash, true},
};
}  // namespace

int fused_candidates_l32_t1(const FusedCandidate **out)
{
    *out = kCand;
    return (int)(sizeof(kCand) / sizeof(kCand[0]));
}

}  // namespace cgb
