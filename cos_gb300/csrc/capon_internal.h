// Internal interfaces between the host API (capon_api.cu) and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cgb {

// Device-side description of one frame.  Pixel p of beam bx sits at range
// row p + K; its snapshots are rows p .. p+2K.
struct FrameDev {
    const float2 *x;   // [Nx][Ny][M]
    float2 *z;         // [Nx][Npy]
    float *P;          // [Nx][Npy] or null
    float2 *w;         // [Nx][Npy][L] or null
    float2 *R;         // [Nx][Npy][L][L] or null
    float d;
    int L, K, M, Nx, Ny, Nb;
    int Npy;           // Ny - 2K pixels per beam
    int loading;       // COS_CAPON_LOAD_*
    int r_layout;      // COS_CAPON_R_*
    int refine;
    int fb;            // forward-backward averaged covariance
    const float2 *V;   // [Nb][L] beamspace subspace matrix, null = Butler
    int tile;          // pixels per range tile (kernel-specific)
    int tiles_per_beam;
    long long tile_begin;  // first global tile index of this frame
};

// Frame descriptors passed by value as a kernel parameter (graph-capturable).
static constexpr int kMaxFrames = 8;
struct FramesParam {
    FrameDev f[kMaxFrames];
    int n;
    // nonzero: every CTA waits on a barrier that nothing completes, so the
    // bounded wait runs out and the launch reports ERR_TIMEOUT (the test of
    // the timeout path; set from COS_CAPON_TEST_STALL, never by default)
    int stall_test;
    // FUSED_REFINE: per pixel group, the float-float covariance slots kept for
    // the residual (fused::WideStash); indexed by the launch's group number
    float4 *stash;
    size_t stash_bytes;
};

// Error bits written to the device status word.
enum : unsigned { ERR_TIMEOUT = 1u, ERR_NOT_PD = 2u };

// Bounded wait on a shared-memory mbarrier phase; returns false after
// `limit` polls (the caller records ERR_TIMEOUT and leaves).
static constexpr uint32_t kWaitLimit = 1u << 22;
// polls of the stall test's wait (a few milliseconds)
static constexpr uint32_t kStallTestLimit = 1u << 12;

// ---- launchers (return cudaError_t as int) ----------------------------------
// plain three-stage element-space pipeline; R_work must hold Nx*Npy*L*L complex
int launch_plain_build_r(const FrameDev &f, float2 *R_out, int r_ref_layout, cudaStream_t s);
int launch_plain_solve_hpd(const FrameDev &f, const float2 *R, float2 *Ria, unsigned *status,
                           cudaStream_t s);
int launch_plain_output(const FrameDev &f, const float2 *Ria, cudaStream_t s);
// precise element-space pipeline (float-float covariance, FP32 Cholesky,
// optional FP64-residual refinement); Rhi/Rlo hold Nx*Npy*L*L, dl Nx*Npy, Ria Nx*Npy*L
int launch_precise(const FrameDev &f, float2 *Rhi, float2 *Rlo, float *dl, float2 *Ria, unsigned *status,
                   bool refine, cudaStream_t s);
// FP32 Cholesky solve (optionally refined with an FP64 residual against
// Rhi + Rlo + dl; Rlo may be null) and the output stage
int launch_precise_solve(const FrameDev &f, const float2 *Rhi, const float2 *Rlo, const float *dl, float2 *Ria,
                         unsigned *status, bool refine, cudaStream_t s);
// forward-backward averaging in place, R = (R + J R^T J)/2, on per-pixel L x L
// matrices (either layout; Rlo, when given, the float-float low parts)
int launch_fb_average(const FrameDev &f, float2 *Rhi, float2 *Rlo, cudaStream_t s);
// beamspace frames up to this many beams run the range-tile kernel (which also
// carries forward-backward averaging)
static constexpr int kBeamspaceTileMaxNb = 5;
// Rhi (+ Rlo) plus the loading dl written in the frame's R layout
int launch_format_r(const FrameDev &f, const float2 *Rhi, const float2 *Rlo, const float *dl, float2 *out,
                    cudaStream_t s);
// tensor-core covariance (tcgen05, TMEM): Rw = R per pixel (column-major, not
// normalised, not loaded) and dl, for split = COS_CAPON_FORM_TC_*
bool tc_supported(const FrameDev &f, int split);
int launch_tc_covariance(const FrameDev &f, int split, float2 *Rw, float *dl, unsigned *status, int num_sms,
                         cudaStream_t s);
// sliding-window inverse form (Sherman-Morrison along range); f.tile carries
// the segment length (0 = default)
int launch_sliding_inverse(const FrameDev &f, unsigned *status, cudaStream_t s);
// general batched LU solve, column-major A
int launch_lu_solve(float2 *x, const float2 *A, const float2 *b, int N, int batch, cudaStream_t s);
// fused element-space path: candidate configurations per subarray length.
// A candidate's launch fills the tiling fields of the frames itself; all
// frames of one launch share L, K and M.
// What one fused launch writes.  The modes are separate instantiations so that
// the z/P kernel carries neither the back substitution nor the R stores, and
// the w kernel not the R stores: the unrolled code of each stays small enough
// for the instruction cache.
enum FusedMode : int {
    FUSED_ZP = 0,  // z and P
    FUSED_W = 1,   // z, P and w (back substitution)
    FUSED_R = 2,   // the loaded covariance R only (no factorisation)
    FUSED_REFINE = 3,  // z, P (and w) with one refinement step of R^-1 a (L > 32)
    // adaptive refinement (L > 32): the z/P (or w) mode on every pixel, then
    // the refinement pass on the pixels whose pivot spread exceeds kAdaptiveSpread
    FUSED_ADAPT_ZP = 4,
    FUSED_ADAPT_W = 5,
};
// Pivot spread max d_i / min d_i of the square-root-free Cholesky above which
// the adaptive mode refines a pixel.  On the precision stress data (L=64,
// K=4, two coherent scatterers at 40 dB, loading 1e-3) the pixels below it
// come within 1.6e-6 of FP64 without refinement (single-precision LAPACK on
// the oracle's R).
static constexpr float kAdaptiveSpread = 32.f;
struct FusedCandidate {
    const char *name;
    int L;
    int T;  // the temporal window 2K+1 the instantiation is compiled for, 0 = any
    int M;  // the channel count it is compiled for, 0 = any
    int (*launch)(const FramesParam &fp, int mode, unsigned *status, int num_sms, cudaStream_t s);
    size_t (*smem)(int K, int M);  // dynamic shared memory of a launch for (K, M)
    // the refinement modes: bytes of FramesParam::stash a launch needs (null:
    // the candidate has no refinement modes)
    size_t (*stash)(int num_sms);
    // serves the refinement modes only (the L <= 32 instantiation of the
    // blocked path); the others serve the z/P, w and R modes
    bool refine_only;
};
// shared memory one CTA may use; a candidate whose tile needs more for a
// frame's (K, M) is not used for it (the precise pipeline takes the frame)
static constexpr size_t kFusedSmemMax = 227 * 1024;
int fused_candidates_l16_t1(const FusedCandidate **out);
int fused_candidates_l16_t3(const FusedCandidate **out);
int fused_candidates_l16_t5(const FusedCandidate **out);
int fused_candidates_l32_t1(const FusedCandidate **out);
int fused_candidates_l32_t3(const FusedCandidate **out);
int fused_candidates_l32_t5(const FusedCandidate **out);
int fused_candidates_l48(const FusedCandidate **out);
int fused_candidates_l64(const FusedCandidate **out);
// tensor-core fused kernel (capon_tcf.cu): z and P only, compile-time (L, T, M)
int tc_fused_candidates(const FusedCandidate **out);
// adjoint of the output power
struct AdjDev {
    const float2 *x;   // [Nx][Ny][M]
    const float2 *w;   // [Nx][Npy][L]
    const float *gP;   // [Nx][Npy]
    float2 *gx;        // [Nx][Ny][M]   accumulated dloss/dconj(x)
    float *gd;         // [1]           accumulated dloss/dd, or null
    float *gth;        // [M]           accumulated dloss/dtheta, or null
    int L, K, M, Nx, Ny, Npy;
};

int launch_adjoint(const AdjDev &a, int num_sms, cudaStream_t s);
// time-domain steering (the step before the path)
struct TdibDev {
    const float2 *mf;      // [n_hydros][n_samples] matched-filtered channel data
    const double *x_r;     // [n_hydros] receiver along-track positions
    const double *D;       // [n_hydros] receiver depths
    const double *xarr;    // [n_x][n_y] pixel x
    const double *yarr;    // [n_x][n_y] pixel y
    double t0, dt, inv_c, fc;
    int n_hydros, n_samples, n_x, n_y;
    float2 *Xd;            // [n_x][n_y][n_hydros] or null
    float2 *image;         // [n_y][n_x] or null
};
int launch_tdib(const TdibDev &t, cudaStream_t s);
// LCA window selection
static constexpr int kLcaMaxFilter = 256;   // wrf entries
struct LcaDev {
    const float2 *Z;   // [Ny][Nx][Nw]
    const float *pw;   // [Nw][Ny][Nx] |Z|^2 (filled by launch_lca)
    float2 *img;       // [Ny][Nx]
    int *win;          // [Ny][Nx] or null
    int Ny, Nx, Nw, Yf, Xf, Ymid, Xmid, single;
    float wrf[kLcaMaxFilter];
};
int launch_lca(const LcaDev &a, float *pw, cudaStream_t s);
// beamspace path (Nb > 0)
int launch_beamspace(const FrameDev &f, float2 *R_out, cudaStream_t s);
int launch_butler(float2 *B, int Nb, int L, cudaStream_t s);

}  // namespace cgb
