// Plain FP32 three-stage Capon pipeline (the "plain FP32 GPU form").
//
// It keeps the reference GPU library's stage structure -- covariance to HBM,
// batched solve, output kernel (RealTimeCapon/Capon.cpp:236-410) -- written
// afresh for sm_103a: one warp per pixel, snapshots staged in shared memory,
// Hermitian Cholesky instead of pivoted LU.  It serves three roles:
//   * the denominator form the fused kernel is measured against,
//   * the covariance entry point cos_capon_build_r (IBuildR::getR),
//   * the general path for subarray lengths the fused kernel does not
//     instantiate.
// The general LU solver for cos_capon_solve (ISolver::solve) is here too.
#include <string.h>

#include <mutex>

#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {

static constexpr int kPlainWarps = 4;

// ---------------------------------------------------------------------------
// Stage 1: covariance.  Lane l walks the diagonals d = l, l+32 of R: the first
// entry R[0,d] = sum_t sum_s x_t[s] conj(x_t[s+d]) directly, then
//   R[k,k+d] = R[k-1,k-1+d] + sum_t (x_t[k-1+Ns] conj(x_t[k-1+d+Ns]) - x_t[k-1] conj(x_t[k-1+d]))
// (the sliding recurrence of buildR_kernel.cu:96-131), mirrored to the lower
// triangle by conjugation.  Lane 0's diagonal yields the trace; loading
// d*tr/L is then added to the real diagonal (buildR_kernel.cu:110-154).
// Output per pixel: column-major, unnormalised (ref layout) or row-major,
// normalised by 1/(Ns*T).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32 * kPlainWarps)
plain_build_r_kernel(FrameDev f, float2 *__restrict__ Rout, int ref_layout)
{
    extern __shared__ float2 smem[];
    const int M = f.M, L = f.L, K = f.K, T = 2 * K + 1, Ns = M - L + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long npix = (long long)f.Nx * f.Npy;
    const long long pix = (long long)blockIdx.x * kPlainWarps + warp;
    if (pix >= npix) return;  // whole warp leaves together
    const int bx = (int)(pix / f.Npy), p = (int)(pix % f.Npy);
    float2 *xs = smem + (size_t)warp * T * M;
    const float2 *xg = f.x + ((size_t)bx * f.Ny + p) * M;
    for (int i = lane; i < T * M; i += 32) xs[i] = xg[i];
    __syncwarp();

    float2 *Rp = Rout + (size_t)pix * L * L;
    const float norm = ref_layout ? 1.0f : 1.0f / ((float)Ns * (float)T);
    float trace = 0.f;
    for (int d = lane; d < L; d += 32) {
        float2 acc = make_float2(0.f, 0.f);
        for (int t = 0; t < T; ++t) {
            const float2 *xt = xs + t * M;
            for (int s = 0; s < Ns; ++s) acc = cadd(acc, cmulc(xt[s], xt[s + d]));
        }
        for (int k = 0; k + d < L; ++k) {
            if (k > 0) {
                for (int t = 0; t < T; ++t) {
                    const float2 *xt = xs + t * M;
                    acc = cadd(acc, csub(cmulc(xt[k - 1 + Ns], xt[k - 1 + d + Ns]),
                                         cmulc(xt[k - 1], xt[k - 1 + d])));
                }
            }
            // acc = R[k, k+d]
            const int a = k, b = k + d;
            const float2 v = cscale(acc, norm);
            if (ref_layout) {  // mem[a + b*L] = R[a,b]
                Rp[a + (size_t)b * L] = v;
                if (d) Rp[b + (size_t)a * L] = cconj(v);
            } else {           // mem[a*L + b] = R[a,b]
                Rp[(size_t)a * L + b] = v;
                if (d) Rp[(size_t)b * L + a] = cconj(v);
            }
            if (d == 0) trace += acc.x;
        }
    }
    trace = __shfl_sync(0xffffffffu, trace, 0);
    __syncwarp();
    const float dl = f.loading == COS_CAPON_LOAD_ABSOLUTE ? f.d * (float)(Ns * T) * norm
                                                          : f.d * trace * norm / (float)L;
    for (int k = lane; k < L; k += 32) Rp[(size_t)k * L + k].x += dl;
}

int launch_plain_build_r(const FrameDev &f, float2 *R_out, int r_ref_layout, cudaStream_t s)
{
    const long long npix = (long long)f.Nx * f.Npy;
    const size_t smem = (size_t)kPlainWarps * (2 * f.K + 1) * f.M * sizeof(float2);
    if (smem > 227 * 1024) return cudaErrorLaunchFailure;
    cudaError_t e = cudaFuncSetAttribute(plain_build_r_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long blocks = (npix + kPlainWarps - 1) / kPlainWarps;
    plain_build_r_kernel<<<(unsigned)blocks, 32 * kPlainWarps, smem, s>>>(f, R_out, r_ref_layout);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Stage 2: batched Hermitian positive definite solve R x = 1.  One warp per
// pixel; R (column-major) is copied into shared memory as a row-major upper
// factor U with U^H U = R (matrixDecompc.pyx:19-50 ordering), then
// U^H y = 1 and U x = y (linearSolvec.pyx:312-346).  A non-positive pivot sets
// ERR_NOT_PD in the status word (when one is given) and gives NaN, as the
// reference's complex square root of a negative pivot would not be a Cholesky
// factor either.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32 * kPlainWarps)
plain_solve_hpd_kernel(int L, long long batch, const float2 *__restrict__ Rin,
                       float2 *__restrict__ xout, unsigned *status)
{
    extern __shared__ float2 smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long sys = (long long)blockIdx.x * kPlainWarps + warp;
    if (sys >= batch) return;
    const int ld = L + 1;
    float2 *A = smem + (size_t)warp * (L * ld + 2 * L);
    float2 *y = A + (size_t)L * ld;
    const float2 *Rg = Rin + (size_t)sys * L * L;
    // column-major R: element (a,b) at a + b*L -> A[a][b]
    for (int i = lane; i < L * L; i += 32) {
        const int a = i % L, b = i / L;
        A[a * ld + b] = Rg[i];
    }
    __syncwarp();
    bool bad = false;
    for (int i = 0; i < L; ++i) {
        const float dv = A[i * ld + i].x;
        bad |= !(dv > 0.f);
        const float inv = rsqrtf(dv);
        __syncwarp();
        for (int j = i + 1 + lane; j < L; j += 32) A[i * ld + j] = cscale(A[i * ld + j], inv);
        if (lane == 0) A[i * ld + i] = make_float2(dv * inv, 0.f);
        __syncwarp();
        for (int j = i + 1 + lane; j < L; j += 32) {
            const float2 uij = A[i * ld + j];
            for (int k = i + 1; k <= j; ++k)
                A[k * ld + j] = csub(A[k * ld + j], cconjmul(A[i * ld + k], uij));
        }
        __syncwarp();
    }
    // forward U^H y = 1, column oriented: lane j keeps v_j (j = lane, lane+32);
    // at step i, y_i = v_i / U_ii and v_j -= conj(U_ij) y_i for j > i.
    float2 v0 = make_float2(1.f, 0.f), v1 = make_float2(1.f, 0.f);
    for (int i = 0; i < L; ++i) {
        const float2 vi = shfl2(i < 32 ? v0 : v1, i & 31, 32);
        const float2 yi = cscale(vi, 1.0f / A[i * ld + i].x);
        if (lane > i && lane < L) v0 = csub(v0, cconjmul(A[i * ld + lane], yi));
        if (lane + 32 > i && lane + 32 < L) v1 = csub(v1, cconjmul(A[i * ld + lane + 32], yi));
        if (lane == i) v0 = yi;
        if (lane + 32 == i) v1 = yi;
    }
    // back U x = y: x_i = v_i / U_ii, then v_k -= U_ki x_i for k < i.
    for (int i = L - 1; i >= 0; --i) {
        const float2 vi = shfl2(i < 32 ? v0 : v1, i & 31, 32);
        const float2 xi = cscale(vi, 1.0f / A[i * ld + i].x);
        if (lane < i) v0 = csub(v0, cmul(A[lane * ld + i], xi));
        if (lane + 32 < i) v1 = csub(v1, cmul(A[(lane + 32) * ld + i], xi));
        if (lane == i) v0 = xi;
        if (lane + 32 == i) v1 = xi;
    }
    (void)y;
    if (lane < L) xout[(size_t)sys * L + lane] = v0;
    if (lane + 32 < L) xout[(size_t)sys * L + lane + 32] = v1;
    if (bad && lane == 0 && status) atomicOr(status, ERR_NOT_PD);
}

int launch_plain_solve_hpd(const FrameDev &f, const float2 *R, float2 *Ria, unsigned *status,
                           cudaStream_t s)
{
    const long long batch = (long long)f.Nx * f.Npy;
    const int L = f.L;
    const size_t smem = (size_t)kPlainWarps * (L * (L + 1) + 2 * L) * sizeof(float2);
    if (smem > 227 * 1024) return cudaErrorLaunchFailure;
    cudaError_t e = cudaFuncSetAttribute(plain_solve_hpd_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long blocks = (batch + kPlainWarps - 1) / kPlainWarps;
    plain_solve_hpd_kernel<<<(unsigned)blocks, 32 * kPlainWarps, smem, s>>>(L, batch, R, Ria, status);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Stage 3: weights and outputs (amplitude_capon_kernel, capon_kernel.cu:338-427):
//   w = Ria / sum(Ria); g_l = (1/Ns) sum_{s<Ns} x_c[s+l]; z = sum_l conj(w_l) g_l;
//   P = 1 / ((Ns*T) * Re(sum(Ria)))  (Ria solves the unnormalised system).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32 * kPlainWarps)
plain_output_kernel(FrameDev f, const float2 *__restrict__ Ria)
{
    const int M = f.M, L = f.L, K = f.K, T = 2 * K + 1, Ns = M - L + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long npix = (long long)f.Nx * f.Npy;
    const long long pix = (long long)blockIdx.x * kPlainWarps + warp;
    if (pix >= npix) return;
    const int bx = (int)(pix / f.Npy), p = (int)(pix % f.Npy);
    const float2 *xc = f.x + ((size_t)bx * f.Ny + p + K) * M;
    const float2 *r = Ria + (size_t)pix * L;
    float2 sum = make_float2(0.f, 0.f);
    for (int l = lane; l < L; l += 32) sum = cadd(sum, r[l]);
    for (int o = 16; o; o >>= 1) sum = cadd(sum, shfl2_xor(sum, o, 32));
    const float den = cabs2(sum);
    const float2 isum = make_float2(sum.x / den, -sum.y / den);  // 1/sum
    float2 zacc = make_float2(0.f, 0.f);
    const float invNs = 1.0f / (float)Ns;
    for (int l = lane; l < L; l += 32) {
        const float2 wl = cmul(r[l], isum);
        if (f.w) f.w[(size_t)pix * L + l] = wl;
        float2 g = make_float2(0.f, 0.f);
        for (int s = 0; s < Ns; ++s) g = cadd(g, xc[s + l]);
        zacc = cadd(zacc, cconjmul(wl, cscale(g, invNs)));
    }
    for (int o = 16; o; o >>= 1) zacc = cadd(zacc, shfl2_xor(zacc, o, 32));
    if (lane == 0) {
        f.z[pix] = zacc;
        if (f.P) f.P[pix] = 1.0f / ((float)Ns * (float)T * sum.x);
    }
}

int launch_plain_output(const FrameDev &f, const float2 *Ria, cudaStream_t s)
{
    const long long npix = (long long)f.Nx * f.Npy;
    const long long blocks = (npix + kPlainWarps - 1) / kPlainWarps;
    plain_output_kernel<<<(unsigned)blocks, 32 * kPlainWarps, 0, s>>>(f, Ria);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// General batched solve A x = b (cos_capon_solve / ISolver::solve): one warp
// per system, [A | b] in shared memory, Gaussian elimination with partial
// pivoting by modulus, back substitution.  A column-major as in the
// reference's Solver (testRTC.pyx:227-229 solves A^T x = b on row-major input).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32 * kPlainWarps)
lu_solve_kernel(int N, long long batch, const float2 *__restrict__ Ag, const float2 *__restrict__ bg,
                float2 *__restrict__ xg)
{
    extern __shared__ float2 smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long sys = (long long)blockIdx.x * kPlainWarps + warp;
    if (sys >= batch) return;
    const int ld = N + 2;  // columns 0..N-1 = A, column N = b
    float2 *A = smem + (size_t)warp * N * ld;
    const float2 *As = Ag + (size_t)sys * N * N;
    for (int i = lane; i < N * N; i += 32) A[(i % N) * ld + i / N] = As[i];
    for (int i = lane; i < N; i += 32) A[i * ld + N] = bg[(size_t)sys * N + i];
    __syncwarp();
    for (int i = 0; i < N; ++i) {
        // pivot: row of max |A[r][i]| for r >= i
        float best = -1.f;
        int bi = i;
        for (int r = i + lane; r < N; r += 32) {
            const float v = cabs2(A[r * ld + i]);
            if (v > best) { best = v; bi = r; }
        }
        for (int o = 16; o; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (bi != i)
            for (int c = lane; c <= N; c += 32) {
                const float2 t = A[i * ld + c];
                A[i * ld + c] = A[bi * ld + c];
                A[bi * ld + c] = t;
            }
        __syncwarp();
        const float2 piv = A[i * ld + i];
        const float pd = cabs2(piv);
        const float2 ipiv = make_float2(piv.x / pd, -piv.y / pd);
        for (int r = i + 1; r < N; ++r) {
            const float2 fct = cmul(A[r * ld + i], ipiv);
            __syncwarp();
            for (int c = i + 1 + lane; c <= N; c += 32)
                A[r * ld + c] = csub(A[r * ld + c], cmul(fct, A[i * ld + c]));
            __syncwarp();
        }
    }
    if (lane == 0) {
        for (int i = N - 1; i >= 0; --i) {
            float2 v = A[i * ld + N];
            for (int k = i + 1; k < N; ++k) v = csub(v, cmul(A[i * ld + k], A[k * ld + N + 1]));
            const float2 piv = A[i * ld + i];
            const float pd = cabs2(piv);
            A[i * ld + N + 1] = cmul(v, make_float2(piv.x / pd, -piv.y / pd));
        }
    }
    __syncwarp();
    for (int i = lane; i < N; i += 32) xg[(size_t)sys * N + i] = A[i * ld + N + 1];
}

int launch_lu_solve(float2 *x, const float2 *A, const float2 *b, int N, int batch, cudaStream_t s)
{
    const size_t smem = (size_t)kPlainWarps * N * (N + 2) * sizeof(float2);
    if (smem > 227 * 1024) return cudaErrorLaunchFailure;
    cudaError_t e = cudaFuncSetAttribute(lu_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const long long blocks = ((long long)batch + kPlainWarps - 1) / kPlainWarps;
    lu_solve_kernel<<<(unsigned)blocks, 32 * kPlainWarps, smem, s>>>(N, batch, A, b, x);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free entry point (no counterpart in the reference).
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool or allocator callback, real-time loops that must
// not reach the driver's allocator, or processes whose device memory is
// reserved up front.  cos_capon_run_plain_noalloc runs the plain three-stage
// pipeline with its two work buffers (per-pixel covariance and R^-1 a) taken
// from a file-scope __device__ array of fixed size, so it allocates nothing.
// Every GPU that loads this library holds the array (8 MiB) until the process
// exits.  Like the reference's solver, it reports no non-positive pivot: the
// affected pixels' outputs are not finite.
// ---------------------------------------------------------------------------
#define COS_NOALLOC_SCRATCH_ELEMS (1u << 20)  // float2 elements: 8 MiB

static __device__ __align__(256) float2 g_noalloc_scratch[COS_NOALLOC_SCRATCH_ELEMS];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
float2 *g_scratch_ptr[kMaxDevices];

// Device address of the static array on the current device (the array's name
// is a host-side stand-in, not a device address).  Every call outside stream
// capture looks it up afresh, so that a context re-created after
// cudaDeviceReset gets the new address; a call during capture, when no lookup
// may touch the module, reuses the address of the last call on that device.
int noalloc_setup(cudaStream_t s, float2 **scratch)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (cs == cudaStreamCaptureStatusNone || !g_scratch_ptr[dev]) {
        if (cs != cudaStreamCaptureStatusNone) return cudaErrorStreamCaptureUnsupported;
        void *ps = nullptr;
        if ((e = cudaGetSymbolAddress(&ps, g_noalloc_scratch)) != cudaSuccess) return e;
        g_scratch_ptr[dev] = (float2 *)ps;
    }
    *scratch = g_scratch_ptr[dev];
    return cudaSuccess;
}
}  // namespace

}  // namespace cgb

extern "C" int cos_capon_run_plain_noalloc(const cos_capon_frame *fr, void *stream)
{
    using namespace cgb;
    if (!fr || !fr->x || !fr->z) return COS_CAPON_ERR_INVALID_VALUE;
    const int L = fr->L, K = fr->K, M = fr->M, Nx = fr->Nx, Ny = fr->Ny;
    if (Nx < 1 || Ny < 1 || L < 1 || M < 1 || K < 0 || fr->Nb < 0 || L > M || 2 * K >= Ny)
        return COS_CAPON_ERR_LAUNCH;
    if (fr->Nb > 0 || L > 64) return COS_CAPON_ERR_NOT_SUPPORTED;  // beamspace is not built here
    const size_t npix = (size_t)Nx * (Ny - 2 * K);
    const size_t need = npix * ((size_t)L * L + (size_t)L);
    if (need > COS_NOALLOC_SCRATCH_ELEMS) return COS_CAPON_ERR_OUT_OF_MEMORY;
    cudaStream_t s = (cudaStream_t)stream;
    float2 *scratch = nullptr;
    int e = noalloc_setup(s, &scratch);
    if (e) return e;
    FrameDev f;
    memset(&f, 0, sizeof(f));
    f.x = (const float2 *)fr->x;
    f.z = (float2 *)fr->z;
    f.P = fr->P;
    f.w = (float2 *)fr->w;
    f.d = fr->d;
    f.L = L;
    f.K = K;
    f.M = M;
    f.Nx = Nx;
    f.Ny = Ny;
    f.Npy = Ny - 2 * K;
    float2 *Rw = scratch, *Ria = scratch + npix * (size_t)L * L;
    // every element the solve reads is written by the covariance pass first,
    // so the previous call's contents never reach the outputs
    if ((e = launch_plain_build_r(f, Rw, 1, s))) return e;
    if ((e = launch_plain_solve_hpd(f, Rw, Ria, nullptr, s))) return e;
    if ((e = launch_plain_output(f, Ria, s))) return e;
    // R is the caller's memory: the reference layout (per pixel column-major,
    // loaded, not normalised), written by a second covariance pass
    if (fr->R && (e = launch_plain_build_r(f, (float2 *)fr->R, 1, s))) return e;
    return 0;
}
