// Candidate table of the fused element-space kernel for L = 64 (any temporal
// window: the L > 32 path takes it from the frame); the
// configurations are compiled in the capon_fused_l64?[_refine].cu files.
// The autotuner in capon_api.cu picks one per (L, K, M, mode) shape; a
// candidate compiled for a fixed M reports cudaErrorNotSupported for other M.
#include "capon_internal.h"

namespace cgb {
int fused_l64a_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
int fused_l64a_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64a_smem(int K, int M);
size_t fused_l64a_stash(int num_sms);
int fused_l64b_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
int fused_l64b_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64b_smem(int K, int M);
size_t fused_l64b_stash(int num_sms);
int fused_l64c_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
int fused_l64c_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64c_smem(int K, int M);
size_t fused_l64c_stash(int num_sms);

int fused_l64d_launch(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
int fused_l64d_launch_refine(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s);
size_t fused_l64d_smem(int K, int M);
size_t fused_l64d_stash(int num_sms);

namespace {
int launch_l64d(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return mode <= FUSED_R ? fused_l64d_launch(fp, mode, st, n, s) : fused_l64d_launch_refine(fp, mode, st, n, s);
}
int launch_l64a(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return mode <= FUSED_R ? fused_l64a_launch(fp, mode, st, n, s) : fused_l64a_launch_refine(fp, mode, st, n, s);
}
int launch_l64b(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return mode <= FUSED_R ? fused_l64b_launch(fp, mode, st, n, s) : fused_l64b_launch_refine(fp, mode, st, n, s);
}
int launch_l64c(const FramesParam &fp, int mode, unsigned *st, int n, cudaStream_t s)
{
    return mode <= FUSED_R ? fused_l64c_launch(fp, mode, st, n, s) : fused_l64c_launch_refine(fp, mode, st, n, s);
}

const FusedCandidate kCand[] = {
    {"L64.G32.W12.N1.M128", 64, 0, 128, launch_l64a, fused_l64a_smem, fused_l64a_stash},
    {"L64.G32.W8.N2.M128", 64, 0, 128, launch_l64b, fused_l64b_smem, fused_l64b_stash},
    {"L64.G32.W12.N1", 64, 0, 0, launch_l64c, fused_l64c_smem, fused_l64c_stash},
    {"L64.G32.W8.N2", 64, 0, 0, launch_l64d, fused_l64d_smem, fused_l64d_stash},
};
}  // namespace

int fused_candidates_l64(const FusedCandidate **out)
{
    *out = kCand;
    return (int)(sizeof(kCand) / sizeof(kCand[0]));
}

}  // namespace cgb
