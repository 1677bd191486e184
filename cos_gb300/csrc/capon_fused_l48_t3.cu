// Fused element-space kernel instantiation for L = 48, temporal window T = 3:
// two pixels per warp (16 lanes each, three columns per lane), the blocked
// per-pixel path of capon_fused_wide.cuh; any channel count.
#include "capon_fused.cuh"

namespace cgb {
namespace {
using C0 = fused::Cfg<48, 16, 8, 1, 3, 0, true>;
int launch_0(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return fused::launch_any<C0>(fp, mode, st, n, s);
}

const FusedCandidate kCand[] = {
    {"L48.G16.W8.N1.sync.T3", 48, 3, 0, launch_0, fused::smem_bytes<C0>, fused::stash_bytes<C0>},
};
}  // namespace

int fused_candidates_l48_t3(const FusedCandidate **out)
{
    *out = kCand;
    return (int)(sizeof(kCand) / sizeof(kCand[0]));
}

}  // namespace cgb
