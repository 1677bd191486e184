// Fused element-space Capon/MVDR kernel for sm_103a.
//
// One persistent launch walks work units (frame, beam, range tile).  Per unit:
//   1. TMA (cp.async.bulk) stages the tile's TILE+2K range rows of the beam
//      (one contiguous run of Xd[bx][p0..][0..M)) into shared memory,
//      double-buffered so the next unit's rows arrive during this unit's math;
//   2. the rows are expanded to (re, im, im, -re) quads, and two per-row
//      quantities shared by all pixels of the tile are formed:
//        c_y[j] = sum_{s<Ns} x_y[s] conj(x_y[s+j])   (first covariance row)
//        g_y[l] = sum_{s<Ns} x_y[s+l] / Ns          (subarray sums, getCaponC.pyx:246-255)
//   3. each pixel is owned by a group of G lanes; lane r holds columns
//      j = m*G + r (m < L/G) of the upper triangle of its covariance in
//      registers.  Row 0 is the window sum of c; rows k >= 1 follow the
//      diagonal recurrence of the reference buildR kernel (buildR_kernel.cu:96-131)
//        R[k,j] = R[k-1,j-1] + sum_t (x_t[k-1+Ns] conj(x_t[j-1+Ns]) - x_t[k-1] conj(x_t[j-1]))
//      with R[k-1,j-1] taken from the neighbouring lane by a shuffle;
//   4. diagonal loading d*tr(R)/L (getCaponC.pyx:257-262);
//   5. right-looking Cholesky U^H U = R in the same registers, the pivot row
//      broadcast through shared memory, with the two right-hand sides a = 1 and
//      g carried along, so y1 = U^-H a and y2 = U^-H g come out of the
//      factorisation (matrixDecompc.pyx:19-50, linearSolvec.pyx:312-327);
//   6. outputs: a^H R^-1 a = |y1|^2, z = w^H g = y1^H y2 / |y1|^2
//      (getCaponC.pyx:276-283), P = 1/((Ns*T) |y1|^2) for the normalised R,
//      and, when asked, w = U^-1 y1 / |y1|^2 by back substitution
//      (linearSolvec.pyx:330-346).
// Arithmetic is FP32 with packed fma.rn.f32x2.
#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {

// ---- mbarrier / bulk-copy primitives ---------------------------------------
COS_DEV uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

COS_DEV void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}
COS_DEV void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
COS_DEV bool mbar_try_wait(uint64_t *bar, uint32_t phase)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
// bounded wait; false when the limit was reached
COS_DEV bool mbar_wait_bounded(uint64_t *bar, uint32_t phase)
{
    for (uint32_t it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}
COS_DEV void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
COS_DEV void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
COS_DEV void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// ---- compile-time configuration --------------------------------------------
template <int L_, int G_, int WARPS_, int NITER_, int TMAX_>
struct Cfg {
    static constexpr int L = L_, G = G_, WARPS = WARPS_, NITER = NITER_, TMAX = TMAX_;
    static constexpr int NM = L / G;       // column slots per lane
    static constexpr int PPW = 32 / G;     // pixels per warp
    static constexpr int TILE = WARPS * PPW * NITER;
    static_assert(L % G == 0 && 32 % G == 0, "G must divide L and 32");
};

// shared-memory carve-up (bytes), host and device agree
struct Smem {
    int rows, XS;  // tile rows (TILE+2K), expanded row stride (quads)
    size_t off_raw0, off_raw1, off_xe, off_c, off_g, off_rb, off_bar, total;
    __host__ __device__ Smem(int TILE, int K, int M, int L, int WARPS, int PPW)
    {
        rows = TILE + 2 * K;
        XS = M + 2;
        const size_t raw = ((size_t)rows * M * sizeof(float2) + 127) & ~(size_t)127;
        off_raw0 = 0;
        off_raw1 = off_raw0 + raw;
        off_xe = off_raw1 + raw;
        off_c = off_xe + (((size_t)rows * XS * sizeof(float4) + 127) & ~(size_t)127);
        off_g = off_c + (((size_t)rows * L * sizeof(float2) + 127) & ~(size_t)127);
        off_rb = off_g + (((size_t)TILE * L * sizeof(float2) + 127) & ~(size_t)127);
        off_bar = off_rb + (((size_t)WARPS * PPW * (L + 1) * sizeof(float4) + 127) & ~(size_t)127);
        total = off_bar + 64;
    }
};

// unit u of the launch -> (frame, beam, first pixel)
COS_DEV int unit_frame(const FramesParam &fp, long long u)
{
    int f = 0;
    while (f + 1 < fp.n && u >= fp.f[f + 1].tile_begin) ++f;
    return f;
}

template <class C>
__global__ void __launch_bounds__(C::WARPS * 32, 1)
fused_kernel(const __grid_constant__ FramesParam fp, long long total_units, unsigned *status)
{
    constexpr int L = C::L, G = C::G, NM = C::NM, PPW = C::PPW, TILE = C::TILE, TMAX = C::TMAX;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int gi = lane / G, r = lane % G;
    const int nthreads = C::WARPS * 32;

    // all frames of one launch share K and M bounds through the first frame's
    // carve-up; the host groups frames so that K and M are equal within a launch
    const FrameDev &f0 = fp.f[0];
    const Smem S(TILE, f0.K, f0.M, L, C::WARPS, PPW);
    float2 *raw[2] = {(float2 *)(smem + S.off_raw0), (float2 *)(smem + S.off_raw1)};
    float4 *xe = (float4 *)(smem + S.off_xe);
    float2 *cs = (float2 *)(smem + S.off_c);
    float2 *gs = (float2 *)(smem + S.off_g);
    float4 *rb = (float4 *)(smem + S.off_rb) + (size_t)(warp * PPW + gi) * (L + 1);
    uint64_t *bar = (uint64_t *)(smem + S.off_bar);

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();

    // issue the loads of unit u into buffer b (thread 0 only)
    auto issue = [&](long long u, int b) {
        const FrameDev &f = fp.f[unit_frame(fp, u)];
        const long long lu = u - f.tile_begin;
        const int bx = (int)(lu / f.tiles_per_beam);
        const int p0 = (int)(lu % f.tiles_per_beam) * TILE;
        const int rows = min(TILE + 2 * f.K, f.Ny - p0);
        const float2 *src = f.x + ((size_t)bx * f.Ny + p0) * f.M;
        const uint32_t bytes = (uint32_t)((size_t)rows * f.M * sizeof(float2));
        fence_proxy_async();
        if ((bytes & 15u) == 0 && (((uintptr_t)src) & 15u) == 0) {
            mbar_expect_tx(&bar[b], bytes);
            bulk_g2s(raw[b], src, bytes, &bar[b]);
        } else {
            // unaligned cube (odd M): the consumer copies with plain loads
            mbar_expect_tx(&bar[b], 0);
        }
    };

    long long u = blockIdx.x;
    uint32_t ph0 = 0u, ph1 = 0u;
    if (tid == 0 && u < total_units) issue(u, 0);
    int b = 0;
    for (; u < total_units; u += gridDim.x, b ^= 1) {
        const long long un = u + gridDim.x;
        if (tid == 0 && un < total_units) issue(un, b ^ 1);

        const FrameDev &f = fp.f[unit_frame(fp, u)];
        const int M = f.M, K = f.K, T = 2 * K + 1, Ns = M - L + 1;
        const long long lu = u - f.tile_begin;
        const int bx = (int)(lu / f.tiles_per_beam);
        const int p0 = (int)(lu % f.tiles_per_beam) * TILE;
        const int rows = min(TILE + 2 * K, f.Ny - p0);
        const int XS = M + 2;

        const bool ok = mbar_wait_bounded(&bar[b], b ? ph1 : ph0);
        if (b) ph1 ^= 1u; else ph0 ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(status, ERR_TIMEOUT);
            return;
        }
        const float2 *src = f.x + ((size_t)bx * f.Ny + p0) * M;
        const bool direct = ((((size_t)rows * M * sizeof(float2)) & 15u) != 0) || ((((uintptr_t)src) & 15u) != 0);

        // ---- expand rows to quads; per-row first covariance row c and subarray sums g
        for (int i = tid; i < rows * M; i += nthreads) {
            const float2 v = direct ? src[i] : raw[b][i];
            const int rr = i / M, cc = i % M;
            xe[rr * XS + cc] = make_float4(v.x, v.y, v.y, -v.x);
        }
        __syncthreads();
        for (int i = tid; i < rows * L; i += nthreads) {
            const int rr = i / L, j = i % L;
            const float4 *xr = xe + rr * XS;
            float2 acc = make_float2(0.f, 0.f);
            for (int s = 0; s < Ns; ++s) {
                const float4 a = xr[s], c = xr[s + j];
                // a * conj(c)
                acc.x += a.x * c.x + a.y * c.y;
                acc.y += a.y * c.x - a.x * c.y;
            }
            cs[i] = acc;
        }
        const float invNs = 1.0f / (float)Ns;
        for (int i = tid; i < TILE * L; i += nthreads) {
            const int q = i / L, l = i % L;
            float2 acc = make_float2(0.f, 0.f);
            if (q + K < rows) {
                const float4 *xr = xe + (q + K) * XS;
                for (int s = 0; s < Ns; ++s) {
                    acc.x += xr[s + l].x;
                    acc.y += xr[s + l].y;
                }
            }
            gs[i] = make_float2(acc.x * invNs, acc.y * invNs);
        }
        __syncthreads();

        // ---- per-pixel math, G lanes per pixel
#pragma unroll 1
        for (int it = 0; it < C::NITER; ++it) {
            const int lp = (it * C::WARPS + warp) * PPW + gi;  // local pixel
            const int p = p0 + lp;
            const bool active = (p < f.Npy);
            const int lpc = lp;  // rows lp..lp+2K lie inside the TILE+2K row buffers; past `rows` they are stale
            const float4 *xw = xe + (size_t)lpc * XS;

            float2 A[L][NM];
            // row 0: window sum of c
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                const int j = m * G + r;
                float2 acc = make_float2(0.f, 0.f);
                for (int t = 0; t < T; ++t) acc = fadd2(acc, cs[(lpc + t) * L + j]);
                A[0][m] = acc;
            }
            // rows k >= 1: diagonal recurrence, column slot m outer
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                const int j = m * G + r;
                const int jm = j > 0 ? j - 1 : 0;
                // column operands (raw complex): x_t[j-1+Ns] and -x_t[j-1]
                float2 yn[TMAX], yc[TMAX];
#pragma unroll
                for (int t = 0; t < TMAX; ++t) {
                    if (t < T) {
                        const float4 a = xw[t * XS + jm + Ns], c = xw[t * XS + jm];
                        yn[t] = make_float2(a.x, a.y);
                        yc[t] = make_float2(-c.x, -c.y);
                    }
                }
#pragma unroll
                for (int k = 1; k < m * G + G; ++k) {
                    float2 snd;
                    if (m > 0 && k - 1 < m * G)
                        snd = (r == G - 1) ? A[k - 1][m - 1] : A[k - 1][m];
                    else
                        snd = A[k - 1][m];
                    const float2 prev = shfl2(snd, (r + G - 1) % G, G);
                    // x * conj(y) = (xr*yr + xi*yi) + i (xi*yr - xr*yi): with the row
                    // quad (xr, xi, xi, -xr), accumulate P += (xr,xi).(yr,yi) and
                    // Q += (xi,-xr).(yr,yi); then re = P.x + P.y, im = Q.x + Q.y.
                    float2 accP = make_float2(prev.x, 0.f), accQ = make_float2(prev.y, 0.f);
#pragma unroll
                    for (int t = 0; t < TMAX; ++t) {
                        if (t < T) {
                            const float4 xn = xw[t * XS + k - 1 + Ns];
                            const float4 xc = xw[t * XS + k - 1];
                            accP = ffma2(make_float2(xn.x, xn.y), yn[t], accP);
                            accQ = ffma2(make_float2(xn.z, xn.w), yn[t], accQ);
                            accP = ffma2(make_float2(xc.x, xc.y), yc[t], accP);
                            accQ = ffma2(make_float2(xc.z, xc.w), yc[t], accQ);
                        }
                    }
                    A[k][m] = make_float2(accP.x + accP.y, accQ.x + accQ.y);
                }
            }

            // ---- diagonal loading: trace over the lane's diagonal entries
            float tr = 0.f;
#pragma unroll
            for (int m = 0; m < NM; ++m)
#pragma unroll
                for (int q = 0; q < G; ++q)
                    if (q == r) tr += A[m * G + q][m].x;
#pragma unroll
            for (int o = G / 2; o; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o, G);
            const float dl = f.d * tr / (float)L;
#pragma unroll
            for (int m = 0; m < NM; ++m)
#pragma unroll
                for (int q = 0; q < G; ++q)
                    if (q == r) A[m * G + q][m].x += dl;

            // ---- optional R output (loaded covariance)
            if (f.R && active) {
                const size_t pix = (size_t)bx * f.Npy + p;
                float2 *Rp = f.R + pix * L * L;
                const float norm = f.r_layout == COS_CAPON_R_REFERENCE ? 1.0f : 1.0f / ((float)Ns * (float)T);
#pragma unroll
                for (int m = 0; m < NM; ++m) {
                    const int j = m * G + r;
#pragma unroll
                    for (int k = 0; k < m * G + G; ++k) {
                        if (k <= j) {
                            const float2 v = cscale(A[k][m], norm);
                            if (f.r_layout == COS_CAPON_R_REFERENCE) {
                                Rp[k + (size_t)j * L] = v;
                                if (k < j) Rp[j + (size_t)k * L] = cconj(v);
                            } else {
                                Rp[(size_t)k * L + j] = v;
                                if (k < j) Rp[(size_t)j * L + k] = cconj(v);
                            }
                        }
                    }
                }
            }

            // ---- right-hand sides: b1 = a = 1, b2 = g (rows m*G + r)
            float2 b1[NM], b2[NM];
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                b1[m] = make_float2(1.f, 0.f);
                b2[m] = gs[lpc * L + m * G + r];
            }

            // ---- Cholesky with the right-hand sides carried along
            bool bad = false;
#pragma unroll
            for (int i = 0; i < L; ++i) {
                const int oi = i % G, mi = i / G;
                const float dv = __shfl_sync(0xffffffffu, A[i][mi].x, oi, G);
                bad |= !(dv > 0.f);
                const float inv = rsqrtf(dv);
                // scale row i of the lane's columns; the owner of column i sets U_ii
#pragma unroll
                for (int m = mi; m < NM; ++m) A[i][m] = make_float2(A[i][m].x * inv, A[i][m].y * inv);
                if (r == oi) {
                    A[i][mi] = make_float2(dv * inv, 0.f);
                    b1[mi] = make_float2(b1[mi].x * inv, b1[mi].y * inv);
                    b2[mi] = make_float2(b2[mi].x * inv, b2[mi].y * inv);
                }
                const float2 y1 = shfl2(b1[mi], oi, G);
                const float2 y2 = shfl2(b2[mi], oi, G);
                // publish row i: (-Re, -Re, -Im, +Im) of U[i, j]
                __syncwarp();
#pragma unroll
                for (int m = mi; m < NM; ++m) {
                    const float2 v = A[i][m];
                    rb[m * G + r] = make_float4(-v.x, -v.x, -v.y, v.y);
                }
                __syncwarp();
                // right-hand sides, rows m*G + r > i:  b -= conj(U[i,row]) * y
#pragma unroll
                for (int m = mi; m < NM; ++m) {
                    const float2 u = A[i][m];
                    const float2 nu1 = make_float2(-u.x, -u.x), nu2 = make_float2(-u.y, u.y);
                    const bool below = (m * G + r > i);
                    const float2 t1 = cnmac_conj(b1[m], nu1, nu2, y1);
                    const float2 t2 = cnmac_conj(b2[m], nu1, nu2, y2);
                    if (below) {
                        b1[m] = t1;
                        b2[m] = t2;
                    }
                }
                // trailing update A[k][j] -= conj(U[i,k]) U[i,j], i < k; slot (k,m) exists for m >= k/G
                float2 vs[NM];
#pragma unroll
                for (int m = mi; m < NM; ++m) vs[m] = A[i][m];
#pragma unroll
                for (int k = i + 1; k < L; ++k) {
                    const float4 u4 = rb[k];
#pragma unroll
                    for (int m = (k / G > mi ? k / G : mi); m < NM; ++m)
                        A[k][m] = cnmac_conj(A[k][m], make_float2(u4.x, u4.y), make_float2(u4.z, u4.w), vs[m]);
                }
            }

            // ---- outputs
            float s11 = 0.f;
            float2 s12 = make_float2(0.f, 0.f);
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                s11 += cabs2(b1[m]);
                s12 = cadd(s12, cconjmul(b1[m], b2[m]));
            }
#pragma unroll
            for (int o = G / 2; o; o >>= 1) {
                s11 += __shfl_xor_sync(0xffffffffu, s11, o, G);
                s12 = cadd(s12, shfl2_xor(s12, o, G));
            }
            const size_t pix = (size_t)bx * f.Npy + p;
            if (active && r == 0) {
                const float is11 = 1.0f / s11;
                f.z[pix] = make_float2(s12.x * is11, s12.y * is11);
                if (f.P) f.P[pix] = is11 / ((float)Ns * (float)T);
            }
            if (bad && active && r == 0) atomicOr(status, ERR_NOT_PD);

            if (f.w) {
                // back substitution U x = y1, rows L-1 .. 0
                float2 xv[NM];
#pragma unroll
                for (int m = 0; m < NM; ++m) xv[m] = make_float2(0.f, 0.f);
#pragma unroll
                for (int i = L - 1; i >= 0; --i) {
                    const int oi = i % G, mi = i / G;
                    float2 part = make_float2(0.f, 0.f);
#pragma unroll
                    for (int m = mi; m < NM; ++m)
                        if (m * G + r > i) part = cadd(part, cmul(A[i][m], xv[m]));
#pragma unroll
                    for (int o = G / 2; o; o >>= 1) part = cadd(part, shfl2_xor(part, o, G));
                    if (r == oi) {
                        const float2 num = csub(b1[mi], part);
                        xv[mi] = cscale(num, 1.0f / A[i][mi].x);
                    }
                }
                if (active) {
                    const float is11 = 1.0f / s11;
#pragma unroll
                    for (int m = 0; m < NM; ++m) f.w[pix * L + m * G + r] = cscale(xv[m], is11);
                }
            }
        }
        __syncthreads();
    }
}

// ---- instantiations and launcher --------------------------------------------
using Cfg16 = Cfg<16, 4, 4, 2, 5>;
using Cfg32 = Cfg<32, 8, 4, 2, 5>;

bool fused_supported(int L) { return L == 16 || L == 32; }

template <class C>
static int launch_cfg(const FramesParam &fp, unsigned *status, int num_sms, cudaStream_t s)
{
    const FrameDev &f0 = fp.f[0];
    if (2 * f0.K + 1 > C::TMAX) return cudaErrorNotSupported;
    Smem S(C::TILE, f0.K, f0.M, C::L, C::WARPS, C::PPW);
    if (S.total > 227 * 1024) return cudaErrorNotSupported;
    cudaError_t e = cudaFuncSetAttribute(fused_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S.total);
    if (e != cudaSuccess) return e;
    const FrameDev &fl = fp.f[fp.n - 1];
    const long long total = fl.tile_begin + (long long)fl.Nx * fl.tiles_per_beam;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_kernel<C>, C::WARPS * 32, S.total);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorNotSupported;
    long long grid = (long long)num_sms * per_sm;
    if (grid > total) grid = total;
    fused_kernel<C><<<(unsigned)grid, C::WARPS * 32, S.total, s>>>(fp, total, status);
    return cudaGetLastError();
}

int fused_tile(int L)
{
    if (L == 16) return Cfg16::TILE;
    if (L == 32) return Cfg32::TILE;
    return 0;
}

int fused_tmax(int L)
{
    if (L == 16) return Cfg16::TMAX;
    if (L == 32) return Cfg32::TMAX;
    return 0;
}

int launch_fused_frames(const FramesParam &fp, unsigned *status, int num_sms, cudaStream_t s)
{
    const int L = fp.f[0].L;
    if (L == 16) return launch_cfg<Cfg16>(fp, status, num_sms, s);
    if (L == 32) return launch_cfg<Cfg32>(fp, status, num_sms, s);
    return cudaErrorNotSupported;
}

}  // namespace cgb
