// Candidate table of the fused element-space kernel for L = 64, temporal window T = 9; the
// configurations are compiled in the capon_fused_l64_t9?[_refine].cu files.
// The autotuner in capon_api.cu picks one per (L, K, M, mode) shape; a
// candidate compiled for a fixed M reports cudaErrorNotSupported for other M.
#include "capon_internal.h"

namespace cgb {
int fused_l64_t9a_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
int fused_l64_t9a_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64_t9a_smem(int K, int M);
size_t fused_l64_t9a_stash(int num_sms);
int fused_l64_t9b_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
int fused_l64_t9b_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64_t9b_smem(int K, int M);
size_t fused_l64_t9b_stash(int num_sms);
int fused_l64_t9c_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
int fused_l64_t9c_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64_t9c_smem(int K, int M);
size_t fused_l64_t9c_stash(int num_sms);

namespace {
int launch_l64_t9a(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return mode <= FUSED_R ? fused_l64_t9a_launch(fp, mode, st, n, s) : fused_l64_t9a_launch_refine(fp, mode, st, n, s);
}
int launch_l64_t9b(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return mode <= FUSED_R ? fused_l64_t9b_launch(fp, mode, st, n, s) : fused_l64_t9b_launch_refine(fp, mode, st, n, s);
}
int launch_l64_t9c(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return mode <= FUSED_R ? fused_l64_t9c_launch(fp, mode, st, n, s) : fused_l64_t9c_launch_refine(fp, mode, st, n, s);
}

const FusedCandidate kCand[] = {
    {"L64.G32.W12.N1.M128.T9", 64, 9, 128, launch_l64_t9a, fused_l64_t9a_smem, fused_l64_t9a_stash},
    {"L64.G32.W8.N2.M128.T9", 64, 9, 128, launch_l64_t9b, fused_l64_t9b_smem, fused_l64_t9b_stash},
    {"L64.G32.W8.N2.T9", 64, 9, 0, launch_l64_t9c, fused_l64_t9c_smem, fused_l64_t9c_stash},
};
}  // namespace

int fused_candidates_l64_t9(const FusedCandidate **out)
{
    *out = kCand;
    return (int)(sizeof(kCand) / sizeof(kCand[0]));
}

}  // namespace cgb
