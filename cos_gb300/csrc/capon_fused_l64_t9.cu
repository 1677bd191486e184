// Candidate table of the fused element-space kernel for L = 64, temporal
// window T = 9 (the configurations are compiled in capon_fused_l64_t9[abc].cu).
// The autotuner in capon_api.cu picks one per (L, K, M) shape; a candidate
// compiled for a fixed M reports cudaErrorNotSupported for other M.
#include "capon_internal.h"

namespace cgb {
int fused_l64_t9a_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64_t9a_smem(int K, int M);
size_t fused_l64_t9a_stash(int num_sms);
int fused_l64_t9b_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64_t9b_smem(int K, int M);
size_t fused_l64_t9b_stash(int num_sms);
int fused_l64_t9c_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64_t9c_smem(int K, int M);
size_t fused_l64_t9c_stash(int num_sms);

namespace {
const FusedCandidate kCand[] = {
    {"L64.G32.W12.N1.M128.T9", 64, 9, 128, fused_l64_t9a_launch, fused_l64_t9a_smem, fused_l64_t9a_stash},
    {"L64.G32.W8.N2.M128.T9", 64, 9, 128, fused_l64_t9b_launch, fused_l64_t9b_smem, fused_l64_t9b_stash},
    {"L64.G32.W8.N2.T9", 64, 9, 0, fused_l64_t9c_launch, fused_l64_t9c_smem, fused_l64_t9c_stash},
};
}  // namespace

int fused_candidates_l64_t9(const FusedCandidate **out)
{
    *out = kCand;
    return (int)(sizeof(kCand) / sizeof(kCand[0]));
}

}  // namespace cgb
