// Fused element-space kernel instantiations for L = 16, temporal window T = 5.
// The autotuner in capon_api.cu picks one per (L, K, M) shape; a candidate
// compiled for a fixed M reports cudaErrorNotSupported for other M.
#include "capon_fused.cuh"

namespace cgb {
int fused_l16r_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l16r_smem(int K, int M);
size_t fused_l16r_stash(int num_sms);

namespace {
int launch_0(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_any<fused::Cfg<16, 4, 8, 1, 5, 32, true>>(fp, mode, st, n, s);
}
int launch_1(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_any<fused::Cfg<16, 4, 8, 1, 5, 32, false>>(fp, mode, st, n, s);
}
int launch_2(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_any<fused::Cfg<16, 4, 8, 1, 5, 0, true>>(fp, mode, st, n, s);
}

const FusedCandidate kCand[] = {
    {"L16.G4.W8.N1.sync.M32.T5", 16, 5, 32, launch_0, fused::smem_bytes<fused::Cfg<16, 4, 8, 1, 5, 32, true>>},
    {"L16.G4.W8.N1.M32.T5", 16, 5, 32, launch_1, fused::smem_bytes<fused::Cfg<16, 4, 8, 1, 5, 32, false>>},
    {"L16.G4.W8.N1.sync.T5", 16, 5, 0, launch_2, fused::smem_bytes<fused::Cfg<16, 4, 8, 1, 5, 0, true>>},
    // the refinement modes (capon_fused_l16r.cu)
    {"L16.G8.W8.refine", 16, 0, 0, fused_l16r_launch, fused_l16r_smem, fused_l16r_stash, true},
};
}  // namespace

int fused_candidates_l16_t5(const FusedCandidate **out)
{
    *out = kCand;
    return (int)(sizeof(kCand) / sizeof(kCand[0]));
}

}  // namespace cgb
