// Candidate table of the fused element-space kernel for L = 48 (any temporal
// window: the L > 32 path takes it from the frame); the
// configurations are compiled in the capon_fused_l48?[_refine].cu files.
// The autotuner in capon_api.cu picks one per (L, K, M, mode) shape; a
// candidate compiled for a fixed M reports cudaErrorNotSupported for other M.
#include "capon_internal.h"

namespace cgb {
int fused_l48a_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
int fused_l48a_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l48a_smem(int K, int M);
size_t fused_l48a_stash(int num_sms);

namespace {
int launch_l48a(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return mode <= FUSED_R ? fused_l48a_launch(fp, mode, st, n, s) : fused_l48a_launch_refine(fp, mode, st, n, s);
}

const FusedCandidate kCand[] = {
    {"L48.G16.W8.N1.sync", 48, 0, 0, launch_l48a, fused_l48a_smem, fused_l48a_stash},
};
}  // namespace

int fused_candidates_l48(const FusedCandidate **out)
{
    *out = kCand;
    return (int)(sizeof(kCand) / sizeof(kCand[0]));
}

}  // namespace cgb
