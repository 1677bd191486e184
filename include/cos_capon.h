/*
 * cos_capon.h -- C ABI of the GB300-native Capon/MVDR per-pixel path.
 *
 * Plain pointers and sizes only.  Complex samples are interleaved float pairs
 * {re, im} (the reference's Complex<float>, framework/lib/Complex.h:12-166).
 * Every function returns an int status: 0 on success, otherwise one of the
 * COS_CAPON_* codes below, whose values are the CUDA runtime error numbers the
 * reference returns in the same situations.
 *
 * Array conventions (reference getCaponC.pyx:74-83, Capon.cpp:93-94):
 *   x  input cube      complex64 [Nx][Nz][M]        (beam, range, channel)
 *   z  amplitude       complex64 [Nx][Nz-2*Yavg]
 *   P  power           float32   [Nx][Nz-2*Yavg]   (1 / Re(a^H R_d^-1 a), R_d normalised)
 *   w  weights         complex64 [Nx][Nz-2*Yavg][L]
 *   R  covariance      complex64 [Nx][Nz-2*Yavg][L][L]
 * Range rows 0..Yavg-1 and Nz-Yavg..Nz-1 produce no pixel.
 */
#ifndef COS_CAPON_H
#define COS_CAPON_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define COS_CAPON_SUCCESS           0    /* cudaSuccess                                           */
#define COS_CAPON_ERR_INVALID_VALUE 1    /* cudaErrorInvalidValue: NULL context or buffer         */
#define COS_CAPON_ERR_OUT_OF_MEMORY 32   /* cudaErrorMemoryValueTooLarge (Capon.cpp:116-133)       */
#define COS_CAPON_ERR_LAUNCH        719  /* cudaErrorLaunchFailure: invalid sizes (Capon.cpp:98-107,
                                            BuildR.cpp:37-48, Solver.cpp:34-42)                    */
#define COS_CAPON_ERR_NOT_SUPPORTED 801  /* cudaErrorNotSupported: option outside what is built     */
#define COS_CAPON_ERR_TIMEOUT       909  /* cudaErrorTimeout: a bounded device-side wait expired   */
/* Every device-side wait is bounded; on expiry the kernel records the timeout,
   lets its own bulk copies land and returns, so the context stays usable and
   the call returns 909 (that call's outputs are undefined).  With the
   environment variable COS_CAPON_TEST_STALL=1 the fused kernel waits on a
   barrier that nothing completes, so the timeout path can be tested without a
   device fault. */

/* ---- options ------------------------------------------------------------ */
#define COS_CAPON_FORM_FUSED   0  /* one fused persistent kernel per launch (default)             */
#define COS_CAPON_FORM_PLAIN   1  /* plain FP32 three-stage pipeline: build R -> solve -> output   */
/* Tensor-core covariance (element space, M a multiple of 16 up to 128, L <= 64):
   the window Gram on tcgen05 in the named operand precision, smoothing in
   float-float, then the FP32 Cholesky (with refine=1 one FP64-residual step).
   No reference counterpart; precision forms for comparison against FP64.      */
#define COS_CAPON_FORM_TC_TF32   2  /* TF32 operands (rna), FP32 accumulation           */
#define COS_CAPON_FORM_TC_BF16X3 3  /* BF16 hi/lo split, three products, FP32 accum.    */
#define COS_CAPON_FORM_TC_TF32X3 4  /* TF32 hi/lo split, three products, FP32 accum.    */
/* R_d^-1 carried along range by Sherman-Morrison rank-1 changes instead of a
   factorisation per pixel (getCaponAllC.pyx:240-252 SOLVE_WOOD with the
   updates of woodburyc.pyx:15-107): element space, L <= 32, absolute loading
   (COS_CAPON_LOAD_ABSOLUTE, d > 0) only; no R output, no refinement, no fb.
   A fresh build-up starts every opts.segment pixels along range.              */
#define COS_CAPON_FORM_SLIDING_INVERSE 5
/* Tensor-core fused form: the per-range-row Hankel Gram of the covariance on
   tcgen05 (FP16 hi/lo split of row-scaled samples, three products, FP32
   accumulation in TMEM), the window sum and the register Cholesky on chip in
   one persistent kernel; R never reaches HBM.  Element space, z and P only
   (w or R requested returns 801), shapes (L, 2K+1, M) = (32, 5, 64),
   (32, 3, 64), (16, 3, 32).                                                  */
#define COS_CAPON_FORM_TC_FUSED 6

#define COS_CAPON_LOAD_ELEMENT   0  /* R_d = R + d*tr(R)/L*I before any beamspace transform
                                       (reference GPU default, buildR_kernel.cu:153-154)          */
#define COS_CAPON_LOAD_BEAMSPACE 1  /* load after the transform with tr(R_bs)/Nb
                                       (getCaponAllC.pyx:376-385; sliding route BuildR.cpp:82-86) */
#define COS_CAPON_LOAD_ABSOLUTE  2  /* R_d = R + d*I on the normalised R: an absolute (e.g.
                                       learnable) loading, the form the adjoint differentiates */

#define COS_CAPON_R_REFERENCE  0  /* R as the reference GPU writes it: per pixel column-major,
                                     loaded, not normalised (buildR_kernel.cu:84-86,153-157)       */
#define COS_CAPON_R_NORMALISED 1  /* R row-major, loaded, normalised by 1/((M-L+1)(2Yavg+1))
                                     (getCaponC.pyx:240-242)                                     */

#define COS_CAPON_REFINE_NONE     0  /* FP32 Cholesky                                              */
#define COS_CAPON_REFINE_ALL      1  /* one step of iterative refinement of R^-1 a with an FP64
                                        residual on every pixel                                   */
/* Element space on the fused path (L = 16, 32, 48, 64): every pixel in the
   FP32 form of the blocked per-pixel kernels, then the refinement step (with
   the accurate covariance) on the pixels whose square-root-free Cholesky has
   a pivot spread max d_i / min d_i above 32, the ill-conditioned ones.
   Elsewhere the same as COS_CAPON_REFINE_ALL.  (Both refinement values run
   inside the fused kernels for the shapes they serve; other shapes and forms
   refine in the precise pipeline.)                                           */
#define COS_CAPON_REFINE_ADAPTIVE 2

typedef struct cos_capon_opts {
    int form;       /* COS_CAPON_FORM_*                                       */
    int loading;    /* COS_CAPON_LOAD_*                                       */
    int r_layout;   /* COS_CAPON_R_*                                          */
    int refine;     /* COS_CAPON_REFINE_*                                     */
    int fb;         /* 1: forward-backward averaged covariance (R + J R^T J)/2
                       before loading and any beamspace transform
                       (getCaponAllC.pyx:346-347, getCaponPy_ref.py:103-104);
                       element space runs the float-float pipeline, beamspace
                       supports Nb <= 5                                        */
    int segment;    /* COS_CAPON_FORM_SLIDING_INVERSE: pixels along range per
                       fresh build-up of the inverse; 0 = 8                    */
} cos_capon_opts;

/* One frame (data cube + parameters) of a device-pointer call. */
typedef struct cos_capon_frame {
    const void *x;  /* device, complex64 [Nx][Ny][M]                          */
    void *z;        /* device, complex64 [Nx][Ny-2K]           (required)     */
    float *P;       /* device, float32   [Nx][Ny-2K]           or NULL        */
    void *w;        /* device, complex64 [Nx][Ny-2K][L]        or NULL        */
    void *R;        /* device, complex64 [Nx][Ny-2K][L][L]     or NULL        */
    float d;        /* diagonal loading coefficient (relative to trace)       */
    int L;          /* subarray length                                        */
    int K;          /* temporal half window: 2K+1 range samples               */
    int M;          /* channels                                               */
    int Nx;         /* beams                                                  */
    int Ny;         /* range samples                                          */
    int Nb;         /* beamspace dimension, 0 = element space                 */
    const void *V;  /* device, complex64 [Nb][L] subspace matrix (row-major)
                       for beamspace, or NULL for the Butler matrix of the
                       reference GPU path (capon_kernel.cu:47-77); a general V
                       follows getCaponAllC.pyx:226-231, 365-370:
                       a_bs = V 1, R_bs = V R V^H, g_bs = V g                 */
} cos_capon_frame;

typedef struct cos_capon_ctx cos_capon_ctx;

/* Create / destroy a context.  The context owns the device buffers of the
 * host-pointer calls (grown on demand, freed by destroy), its stream and its
 * device status word -- the role of the reference's Capon object
 * (Capon.h:13-125, Capon.cpp:50-71).  Uses the calling thread's current device.
 * Like that object, a context is not thread-safe: its work buffers (the
 * materialised-R pipelines, the LCA planes, the staging of host calls) serve
 * one call at a time, so calls that may overlap -- from several threads, or
 * device calls on different streams -- need a context each. */
int cos_capon_create(cos_capon_ctx **ctx);
int cos_capon_destroy(cos_capon_ctx *ctx);

/* Drop-in for ICapon<Complex<float>,float>::getCapon (ICapon.h:20-33) and its
 * implementation Capon::getCapon (Capon.cpp:73-152): host pointers, synchronous.
 * z and w are required; R may be NULL (the reference copies it back only under
 * COPY_R_DEVICE_HOST, Capon.cpp:9,253-259) and is written in the reference GPU
 * convention (COS_CAPON_R_REFERENCE).  d, L, Yavg, M, Nx, Nz, Nb mean what they
 * mean there; Nb > 0 selects beamspace with element-space loading. */
int cos_capon_get_capon(cos_capon_ctx *ctx, void *z, void *w, void *R, const void *x,
                        float d, int L, int Yavg, int M, int Nx, int Nz, int Nb);

/* Same call with the output power P (float32, may be NULL), optional w / R and
 * explicit options (NULL = defaults).  Host pointers, synchronous.  This is the
 * call behind the Python getCaponCUDAPy / getCaponCPy mirrors. */
int cos_capon_get_capon_ex(cos_capon_ctx *ctx, void *z, float *P, void *w, void *R,
                           const void *x, float d, int L, int Yavg, int M, int Nx, int Nz,
                           int Nb, const cos_capon_opts *opts);

/* Beamspace with a caller-given subspace matrix V (host, complex64 [Nb][L],
 * row-major): getCaponAllC.pyx:226-231, 365-370 semantics.  Element-space
 * loading becomes d tr(R)/L V V^H in beamspace (the reference loads R before
 * the transform).  w is the element-space weight V^H x_bs / (a_bs^H x_bs).
 * No reference GPU counterpart (its beamspace route always uses the Butler
 * matrix).  Host pointers, synchronous. */
int cos_capon_get_capon_subspace(cos_capon_ctx *ctx, void *z, float *P, void *w, const void *x, const void *V,
                                 float d, int L, int Yavg, int M, int Nx, int Nz, int Nb,
                                 const cos_capon_opts *opts);

/* Time-domain steering, the step that produces the Capon input cube
 * (framework/beamformer/delay/tdibC.pyx:9-67).
 * For beam nx, range pixel y and hydrophone n:
 *   Xd[nx][y][n] = interp_linear(mfdata[n], tau) * exp(j 2 pi fc tau)
 *   tau = (r_t + r_r) / c
 * r_t and r_r are measured from the origin (mean(x_r)/2, mean(D)/2) to
 * (xarr, yarr) and on to receiver n.  The time axis is uniform: t0 + k dt.
 * Samples outside it are NaN, as the reference's interp1d gives.
 * image[y][nx] = the mean of Xd over hydrophones (the reference returns
 * image.T).  mfdata is complex64 [n_hydros][n_samples]; x_r and D are float64
 * [n_hydros]; xarr and yarr are float64 [n_x][n_y].  Either Xd or image may be
 * NULL.  on_gpu = 1: every pointer is device memory and the call is
 * asynchronous on `stream`.  on_gpu = 0: host memory; synchronous. */
int cos_capon_tdib(cos_capon_ctx *ctx, const void *mfdata, int n_hydros, int n_samples, double t0, double dt,
                   const double *x_r, const double *D, double c, double fc, const double *xarr, const double *yarr,
                   int n_x, int n_y, void *Xd, void *image, int on_gpu, void *stream);

/* Low-complexity adaptive (LCA) window selection (framework/beamformer/lca/
 * lcac.py; lcacx.pyx:175-216).  Z: complex64 [Ny][Nx][Nw] beamformer outputs
 * for Nw windows; wrf: float64 [Yf][Xf] averaging filter (odd sizes, host
 * memory, Yf*Xf <= 256).  A 1 x 1 filter with a nonzero value selects per
 * pixel the window of least |Z|; otherwise interior pixels take the window of
 * least wrf-weighted sum of |Z|^2 over the neighbourhood (first minimum) and
 * border pixels get 0 / window 0.  img: complex64 [Ny][Nx]; win: int32
 * [Ny][Nx] or NULL.  on_gpu = 1: Z, img, win device memory, asynchronous on
 * `stream`; 0: host memory, synchronous. */
int cos_capon_lca(cos_capon_ctx *ctx, const void *Z, int Ny, int Nx, int Nw, const double *wrf, int Yf, int Xf,
                  void *img, int *win, int on_gpu, void *stream);

/* Device-pointer call: every pixel of `nframes` frames (each with its own M, L,
 * K, Nb) in one call on `stream` (fused frames of equal L, K, M share one
 * persistent launch) (a cudaStream_t; NULL = the default stream).  Asynchronous; no host synchronisation and no allocation once the
 * context has served a call of the same or larger shape, so it can be captured
 * into a CUDA graph after one warm-up call. */
int cos_capon_run(cos_capon_ctx *ctx, const cos_capon_frame *frames, int nframes,
                  const cos_capon_opts *opts, void *stream);

/* Drop-in for IBuildR::getR (IBuildR.h:85-98) / BuildR::getR (BuildR.cpp:21-106):
 * covariance with spatial smoothing, temporal averaging and diagonal loading,
 * written per pixel column-major and not normalised, as the reference does.
 * With Nb > 0, R is Nb x Nb in the Butler beamspace (element-space loading).
 * R_on_gpu / x_on_gpu: nonzero when that pointer is device memory. */
int cos_capon_build_r(cos_capon_ctx *ctx, void *R, const void *x, float d, int L, int Yavg,
                      int M, int Nx, int Nz, int Nb, int R_on_gpu, int x_on_gpu);

/* Drop-in for ISolver::solve (ISolver.h:119-128) / Solver::solve (Solver.cpp:23-116):
 * `batch` dense N x N complex systems A x = b, A column-major per system (the
 * layout the reference's BuildR produces and its solver reads), 1 <= N <= 72,
 * solved by LU with partial pivoting, so A need not be Hermitian. */
int cos_capon_solve(cos_capon_ctx *ctx, void *x, const void *A, const void *b, int N, int batch,
                    int x_on_gpu, int A_on_gpu, int b_on_gpu);

/* Butler (normalised DFT) beamspace matrix, Nb x L, row-major, host or device
 * pointer (B_on_gpu): B[b,l] = exp(-j*2*pi*bin(b)*l/L)/sqrt(L) with the beam
 * layout of capon_kernel.cu:47-77 (butler_matrix). */
int cos_capon_butler(cos_capon_ctx *ctx, void *B, int Nb, int L, int B_on_gpu);

/* Adjoint of the output power (no counterpart in the reference; the
 * differentiable path).  For a loss l(P) with per-pixel gradient gP = dl/dP of
 * a forward call with absolute loading R_d = R + d I (COS_CAPON_LOAD_ABSOLUTE),
 * accumulates
 *   gx[b][y][m]  += dl/dconj(x[b][y][m])                  (complex64)
 *   gd[0]        += dl/dd                                   (float32, or NULL)
 *   gtheta[m]    += dl/dtheta_m for inputs x_m exp(-j theta_m) (float32 [M], or NULL)
 * from the cube x and the weights w of that forward call (dP = w^H dR_d w, so
 * neither R nor its factor is stored or rebuilt).  Pixels with gP = 0 are
 * skipped.  The caller zeroes the accumulators.  Device pointers, asynchronous;
 * element space, L <= 64. */
typedef struct cos_capon_adjoint {
    const void *x;    /* device, complex64 [Nx][Ny][M]        */
    const void *w;    /* device, complex64 [Nx][Ny-2K][L]     */
    const float *gP;  /* device, float32   [Nx][Ny-2K]        */
    void *gx;         /* device, complex64 [Nx][Ny][M]        */
    float *gd;        /* device, float32   [1]  or NULL       */
    float *gtheta;    /* device, float32   [M]  or NULL       */
    int L, K, M, Nx, Ny;
} cos_capon_adjoint;

int cos_capon_backward(cos_capon_ctx *ctx, const cos_capon_adjoint *adj, void *stream);  /* NULL = default stream */

/* Status word of the last launch on this context (0, or COS_CAPON_ERR_TIMEOUT
 * when a bounded device-side wait gave up).  Synchronises the context stream.
 * A non-positive Cholesky pivot (e.g. no loading on a rank-deficient R) is not
 * an error, as in the reference, whose solver reports none: the affected
 * pixels' outputs are not finite. */
int cos_capon_device_status(cos_capon_ctx *ctx);

/* No counterpart in the reference.  Allocation-free variant of the plain FP32
 * three-stage pipeline for callers that cannot allocate device memory (code
 * running inside another framework's allocator, real-time loops that must not
 * call into the driver's allocator).  Its work buffers are a fixed file-scope
 * device array of 2^20 complex elements (8 MiB, held by every GPU that loads
 * the library until exit): frames with Nx*(Ny-2K)*(L*L+L) above that return
 * COS_CAPON_ERR_OUT_OF_MEMORY.  Element space only (Nb > 0 returns
 * COS_CAPON_ERR_NOT_SUPPORTED), device pointers, asynchronous on `stream` (a
 * cudaStream_t, NULL = default stream); no context, no cudaMalloc/cudaFree.
 * P, w and R may be NULL; R, when given, is written in the reference GPU
 * layout (COS_CAPON_R_REFERENCE).  Each call outside stream capture looks up
 * the array's device address on the current device (so a context re-created
 * after cudaDeviceReset is served correctly); a call during capture reuses the
 * address of the last call on that device, so make one call before capturing,
 * and recapture after a device reset.  All calls share the array, so calls
 * that overlap on the GPU (different streams, or threads) race and must be
 * serialised by the caller.  A non-positive Cholesky pivot is not reported (as
 * in the reference's solver): those pixels' outputs are not finite. */
int cos_capon_run_plain_noalloc(const cos_capon_frame *frame, void *stream);

/* Human-readable text for a status code. */
const char *cos_capon_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif /* COS_CAPON_H */
