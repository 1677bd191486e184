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
//   5. right-looking Cholesky in its square-root-free form R = L D L^H
//      (U = D^-1/2 (D L^H) is the reference's factor, matrixDecompc.pyx:19-50)
//      in the same registers, the pivot row broadcast through shared memory
//      (in the z/P mode one step ahead of its use), with the two right-hand
//      sides a = 1 and g carried along, so b1 = L^-1 a and b2 = L^-1 g come out
//      of the factorisation (the forward solve of linearSolvec.pyx:312-327,
//      with y = D^-1/2 b);
//   6. outputs: a^H R^-1 a = |y1|^2, z = w^H g = y1^H y2 / |y1|^2
//      (getCaponC.pyx:276-283), P = 1/((Ns*T) |y1|^2) for the normalised R,
//      and, when asked, w = R^-1 a / |y1|^2 by back substitution with D L^H
//      (linearSolvec.pyx:330-346).
// Arithmetic is FP32 with packed fma.rn.f32x2.
#pragma once
// the R-only mode leaves the factorisation after its R stores: in that
// instantiation the rest of the per-pixel code is unreachable by design
#pragma nv_diag_suppress 128
#include "capon_common.cuh"
#include "capon_fused_wide.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {
namespace fused {

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
COS_DEV bool mbar_wait_bounded(uint64_t *bar, uint32_t phase, uint32_t limit = kWaitLimit)
{
    for (uint32_t it = 0; it < limit; ++it)
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
// timeout exit of thread 0: record it, then wait (bounded) for the bulk copies
// still in flight into this CTA's shared memory -- buffer b (whose phase bit
// was already flipped) and, when a next unit was issued, buffer b^1 -- so
// that none lands after the CTA has left.  Kept out of line, away from the
// register allocation of the unit loop.
static __device__ __noinline__ void timeout_exit(unsigned *status, uint64_t *bar, int b, uint32_t ph0, uint32_t ph1,
                                          bool next_issued)
{
    atomicOr(status, ERR_TIMEOUT);
    mbar_wait_bounded(&bar[b], (b ? ph1 : ph0) ^ 1u);
    if (next_issued) mbar_wait_bounded(&bar[b ^ 1], b ? ph0 : ph1);
}
// test of the timeout path (thread 0): a bounded wait on barrier 2, which
// nothing completes, runs out; record it, let the first unit's copy land, leave
static __device__ __noinline__ void stall_test_exit(unsigned *status, uint64_t *bar, bool first_issued)
{
    if (!mbar_wait_bounded(&bar[2], 0u, kStallTestLimit)) atomicOr(status, ERR_TIMEOUT);
    if (first_issued) mbar_wait_bounded(&bar[0], 0u);
}
COS_DEV void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
COS_DEV void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// ---- compile-time configuration --------------------------------------------
// L: subarray length; G: lanes per pixel (lane r owns columns j = m*G + r);
// WARPS x NITER x (32/G) pixels per tile; T: the temporal window 2K+1 (exact,
// so the window loops carry no runtime bound; 0 = taken from the frame, for
// the L > 32 path only, whose window loops are rolled); M: channel count, 0 = taken at
// run time (a compile-time M turns every shared-memory offset of the unrolled
// code into an immediate); SYNC: barrier points that keep the CTA's warps in
// step, so that the long unrolled instruction stream is fetched once for all
// of them.
template <int L_, int G_, int WARPS_, int NITER_, int T_, int M_, bool SYNC_, bool WIDE_ = (L_ > 32)>
struct Cfg {
    static constexpr int L = L_, G = G_, WARPS = WARPS_, NITER = NITER_, M = M_;
    // RT_T: T from the frame; T then sizes only the unused L <= 32 code
    static constexpr bool RT_T = T_ == 0;
    static constexpr int T = RT_T ? 1 : T_;
    static constexpr bool SYNC = SYNC_;
    static constexpr int NM = L / G;       // column slots per lane
    static constexpr int PPW = 32 / G;     // pixels per warp
    static constexpr int TILE = WARPS * PPW * NITER;
    // the blocked per-pixel path of capon_fused_wide.cuh: always for L > 32;
    // at L <= 32 an instantiation of it serves the refinement modes
    static constexpr bool WIDE = WIDE_;
    // float4 slots of a pixel group's shared area, the largest of: the
    // pivot-row buffers (and, wide, the first covariance row and the 1/d of
    // factored rows); the G x (G+1) exchange area of the back substitution;
    // and, wide, the refinement's x0 (L complex) and its 8 x G partial sums
    static constexpr int AREA = WIDE ? WideArea<L, G>::Q : 2 * (L + 1);
    static constexpr int XCH = (G * (G + 1) + 1) / 2;
    static constexpr int RES = WIDE ? (L + 1) / 2 + 8 * G : 0;
    static constexpr int RBQ = AREA > XCH ? (AREA > RES ? AREA : RES) : (XCH > RES ? XCH : RES);
    static_assert(L % G == 0 && 32 % G == 0, "G must divide L and 32");
    static_assert(WIDE || !RT_T, "a run-time window needs the L > 32 path");
};

// shared-memory carve-up (bytes), host and device agree
struct Smem {
    int rows, XS;  // tile rows (TILE+2K), expanded row stride (quads)
    size_t off_raw0, off_raw1, off_xe, off_c, off_g, off_rb, off_bar, total;
    __host__ __device__ Smem(int TILE, int K, int M, int L, int WARPS, int PPW, int RBQ)
    {
        rows = TILE + 2 * K;
        XS = M + 2;
        const size_t raw = ((size_t)rows * M * sizeof(float2) + 127) & ~(size_t)127;
        off_raw0 = 0;
        off_raw1 = off_raw0 + raw;
        off_xe = off_raw1 + raw;
        off_c = off_xe + (((size_t)rows * XS * sizeof(float4) + 127) & ~(size_t)127);
        off_g = off_c + (((size_t)2 * rows * L * sizeof(float2) + 127) & ~(size_t)127);
        off_rb = off_g + (((size_t)TILE * L * sizeof(float2) + 127) & ~(size_t)127);
        off_bar = off_rb + (((size_t)WARPS * PPW * RBQ * sizeof(float4) + 127) & ~(size_t)127);
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

// MODE (FusedMode): z/P, z/P and w, or R alone; each mode carries only its
// own output code, so its unrolled instruction stream stays small.
template <class C, int MODE>
__global__ void __launch_bounds__(C::WARPS * 32, 1)
fused_kernel(const __grid_constant__ FramesParam fp, long long total_units, unsigned *status)
{
    constexpr int L = C::L, G = C::G, NM = C::NM, PPW = C::PPW, TILE = C::TILE, T = C::T;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int gi = lane / G, r = lane % G;
    const int nthreads = C::WARPS * 32;

    // all frames of one launch share K and M bounds through the first frame's
    // carve-up; the host groups frames so that K and M are equal within a launch
    const FrameDev &f0 = fp.f[0];
    const int K = C::RT_T ? f0.K : (C::T - 1) / 2;
    const Smem S(TILE, K, C::M ? C::M : f0.M, L, C::WARPS, PPW, C::RBQ);
    float2 *raw[2] = {(float2 *)(smem + S.off_raw0), (float2 *)(smem + S.off_raw1)};
    float4 *xe = (float4 *)(smem + S.off_xe);
    float2 *cs = (float2 *)(smem + S.off_c);
    float2 *cl = cs + (size_t)S.rows * L;
    float2 *gs = (float2 *)(smem + S.off_g);
    // each pixel group's shared area (Cfg::RBQ float4): the two pivot-row
    // buffers, alternating by Cholesky step, and what else its phases keep
    float4 *rb = (float4 *)(smem + S.off_rb) + (size_t)(warp * PPW + gi) * C::RBQ;
    uint64_t *bar = (uint64_t *)(smem + S.off_bar);

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);  // never arrived on: the stall test waits here
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
    if (fp.stall_test) {
        if (tid == 0) stall_test_exit(status, bar, u < total_units);
        return;
    }
    int b = 0;
    for (; u < total_units; u += gridDim.x, b ^= 1) {
        const long long un = u + gridDim.x;
        if (tid == 0 && un < total_units) issue(un, b ^ 1);

        const FrameDev &f = fp.f[unit_frame(fp, u)];
        const int M = C::M ? C::M : f.M, Ns = M - L + 1;
        const long long lu = u - f.tile_begin;
        const int bx = (int)(lu / f.tiles_per_beam);
        const int p0 = (int)(lu % f.tiles_per_beam) * TILE;
        const int rows = min(TILE + 2 * K, f.Ny - p0);
        const int XS = M + 2;

        const bool ok = mbar_wait_bounded(&bar[b], b ? ph1 : ph0);
        if (b) ph1 ^= 1u; else ph0 ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) timeout_exit(status, bar, b, ph0, ph1, u + gridDim.x < total_units);
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
        // c_y[j] for 4 consecutive j per thread (the window x[s+j..s+j+3] slides
        // through registers, one new load per term): packed FP32 products summed
        // in chunks of 4 terms, chunk sums accumulated in float-float (TwoSum),
        // so the first covariance row -- which every diagonal of R starts from --
        // carries one rounding only
        static_assert(L % 4 == 0, "L must be a multiple of 4");
        for (int i = tid; i < rows * (L / 4); i += nthreads) {
            const int rr = i / (L / 4), j0 = 4 * (i % (L / 4));
            const float4 *xr = xe + rr * XS;
            float2 hi[4], lo[4];
            float4 w0 = xr[j0], w1 = xr[j0 + 1], w2 = xr[j0 + 2];
#pragma unroll
            for (int q = 0; q < 4; ++q) hi[q] = lo[q] = make_float2(0.f, 0.f);
            if constexpr (MODE == FUSED_REFINE) {
                // the refinement mode: exact products (TwoProd by fma) and
                // float-float sums.  The recurrence carries this row into every
                // diagonal of R, so its rounding would be the same along a whole
                // diagonal, an error the refinement's residual would keep.
#pragma unroll 2
                for (int s = 0; s < Ns; ++s) {
                    const float4 a = xr[s], w3 = xr[s + j0 + 3];
                    const float4 c[4] = {w0, w1, w2, w3};
                    const float2 an = make_float2(a.x, a.y), az = make_float2(a.z, a.w);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        // a conj(c) = c.re (ar, ai) + c.im (ai, -ar)
                        const float2 sr = make_float2(c[q].x, c[q].x), si = make_float2(c[q].y, c[q].y);
                        const float2 p1 = fmul2(sr, an), p2 = fmul2(si, az);
                        const float2 e = fadd2(ffma2(sr, an, make_float2(-p1.x, -p1.y)),
                                               ffma2(si, az, make_float2(-p2.x, -p2.y)));
                        two_sum_acc(hi[q], lo[q], p1);
                        two_sum_acc(hi[q], lo[q], p2);
                        lo[q] = fadd2(lo[q], e);
                    }
                    w0 = w1;
                    w1 = w2;
                    w2 = w3;
                }
            } else {
                // three chunks per iteration: enough independent work to cover the
                // load and TwoSum latencies, without the code growth of a full
                // unroll (which slows the unrolled per-pixel phases that follow
                // through the instruction cache)
#pragma unroll 3
                for (int s0 = 0; s0 < Ns; s0 += 4) {
                    float2 P[4], Q[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) P[q] = Q[q] = make_float2(0.f, 0.f);
#pragma unroll
                    for (int ss = 0; ss < 4; ++ss) {
                        const int s = s0 + ss;
                        if (s < Ns) {
                            const float4 a = xr[s], w3 = xr[s + j0 + 3];
                            const float4 c[4] = {w0, w1, w2, w3};
#pragma unroll
                            for (int q = 0; q < 4; ++q) {
                                // a * conj(c): P += (ar, ai).(cr, ci), Q += (ai, -ar).(cr, ci)
                                P[q] = ffma2(make_float2(a.x, a.y), make_float2(c[q].x, c[q].y), P[q]);
                                Q[q] = ffma2(make_float2(a.z, a.w), make_float2(c[q].x, c[q].y), Q[q]);
                            }
                            w0 = w1;
                            w1 = w2;
                            w2 = w3;
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) two_sum_acc(hi[q], lo[q], make_float2(P[q].x + P[q].y, Q[q].x + Q[q].y));
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                cs[rr * L + j0 + q] = hi[q];
                cl[rr * L + j0 + q] = lo[q];
            }
        }
        // subarray sums of the centre rows, g[l] = (1/Ns) sum_{s<Ns} x[s+l]
        // (getCaponC.pyx:246-255), on all threads: item (row, 8 consecutive l)
        // sums the first window directly and slides g[l+1] = g[l] + x[l+Ns] - x[l]
        // over the rest
        static_assert(L % 8 == 0 || L < 8, "subarray-sum items take 8 consecutive l");
        {
            constexpr int LW = L >= 8 ? 8 : L;
            const float invNs = 1.0f / (float)Ns;
            for (int it2 = tid; it2 < TILE * (L / LW); it2 += nthreads) {
                const int q = it2 / (L / LW), l0 = LW * (it2 % (L / LW));
                if (q + K < rows) {
                    const float4 *xr = xe + (q + K) * XS;
                    float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
                    int s = 0;
                    for (; s + 1 < Ns; s += 2) {
                        a0 = fadd2(a0, make_float2(xr[l0 + s].x, xr[l0 + s].y));
                        a1 = fadd2(a1, make_float2(xr[l0 + s + 1].x, xr[l0 + s + 1].y));
                    }
                    if (s < Ns) a0 = fadd2(a0, make_float2(xr[l0 + s].x, xr[l0 + s].y));
                    float2 acc = fadd2(a0, a1);
#pragma unroll
                    for (int l = l0; l < l0 + LW; ++l) {
                        gs[q * L + l] = make_float2(acc.x * invNs, acc.y * invNs);
                        if (l + 1 < l0 + LW)
                            acc = fadd2(acc, make_float2(xr[l + Ns].x - xr[l].x, xr[l + Ns].y - xr[l].y));
                    }
                }
            }
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

            if constexpr (C::WIDE) {
                constexpr bool ADAPT = MODE == FUSED_ADAPT_ZP || MODE == FUSED_ADAPT_W;
                float4 *const stash =
                    (MODE == FUSED_REFINE || ADAPT)
                        ? fp.stash + ((size_t)blockIdx.x * C::WARPS * PPW + warp * PPW + gi) * WideStash<L, G>::Q
                        : nullptr;
                const float2 *crow = cs + (size_t)lpc * L, *clrow = cl + (size_t)lpc * L, *grow = gs + (size_t)lpc * L;
                const size_t pix = (size_t)bx * f.Npy + p;
                if constexpr (ADAPT) {
                    // every pixel in the z/P (w) mode; the ill-conditioned ones
                    // again through the refinement pass, which overwrites their
                    // outputs (decided per warp: both pixel groups of a warp at
                    // G = 16 take the pass when either needs it)
                    float spread = 0.f;
                    wide_pixel<C, MODE == FUSED_ADAPT_W ? FUSED_W : FUSED_ZP>(f, xw, XS, Ns, crow, clrow, grow, rb,
                                                                               nullptr, r, active, pix, status, &spread);
                    if (__any_sync(0xffffffffu, spread > kAdaptiveSpread)) {
                        __syncwarp();
                        wide_pixel<C, FUSED_REFINE, true>(f, xw, XS, Ns, crow, clrow, grow, rb, stash, r, active, pix,
                                                          status);
                    }
                } else {
                    wide_pixel<C, MODE>(f, xw, XS, Ns, crow, clrow, grow, rb, stash, r, active, pix, status);
                }
                continue;
            }
            float2 A[L][NM];
            // First covariance row R0[d] = sum_t c_{y+t}[d] (float-float, rounded once),
            // shared by the group through shared memory.
            // (the pivot-row buffer is free until the Cholesky; r0 starts G entries in,
            // so slots below the diagonal, d = j - k > -G, read in-bounds garbage)
            float2 *r0 = (float2 *)rb + G;
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                const int j = m * G + r;
                float2 h = make_float2(0.f, 0.f), l = make_float2(0.f, 0.f);
                for (int t = 0; t < T; ++t) {
                    two_sum_acc(h, l, cs[(lpc + t) * L + j]);
                    l = fadd2(l, cl[(lpc + t) * L + j]);
                }
                r0[j] = fadd2(h, l);
            }
            __syncwarp();
            // Along each diagonal, R[k,k+d] = R0[d] + S[k,k+d] with the increment sums
            //   S[k,j] = S[k-1,j-1] + D[k,j],
            //   D[k,j] = sum_t x_t[k-1+Ns] conj(x_t[j-1+Ns]) - x_t[k-1] conj(x_t[j-1]).
            // D telescopes (S[k,k+d] = sum over the last k subarray rows minus the
            // first k), so S stays small next to R and its FP32 running sum adds
            // little rounding; R itself is rounded once, when R0 is added.
            float2 S[NM];  // current row of S per column slot
            float tr = 0.f;  // trace over the lane's diagonal entries
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                S[m] = make_float2(0.f, 0.f);
                A[0][m] = r0[m * G + r];
            }
            if (r == 0) tr += A[0][0].x;
            // column operands (raw complex): x_t[j-1+Ns] and -x_t[j-1], j = m*G + r
            float2 yn[NM][T], yc[NM][T];
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                const int j = m * G + r;
                const int jm = j > 0 ? j - 1 : 0;
#pragma unroll
                for (int t = 0; t < T; ++t) {
                    const float4 a = xw[t * XS + jm + Ns], c = xw[t * XS + jm];
                    yn[m][t] = make_float2(a.x, a.y);
                    yc[m][t] = make_float2(-c.x, -c.y);
                }
            }
            // rows k >= 1, row outer; the previous row of S comes from lane r-1
            // (lane 0: slot m-1 of lane G-1)
#pragma unroll
            for (int k = 1; k < L; ++k) {
                const int m0 = k / G;  // slots (k, m) exist for m >= k/G
                float2 prv[NM];
#pragma unroll
                for (int m = 0; m < NM; ++m) {
                    if (m < m0) continue;
                    float2 sh;
                    if (m > 0 && k - 1 < m * G)
                        sh = (r == G - 1) ? S[m - 1] : S[m];
                    else
                        sh = S[m];
                    prv[m] = shfl2(sh, (r + G - 1) % G, G);
                }
                // with the row quads (xr, xi, xi, -xr): P += (xr,xi).(yr,yi),
                // Q += (xi,-xr).(yr,yi), then re = P.x + P.y, im = Q.x + Q.y
                float2 accP[NM], accQ[NM];
#pragma unroll
                for (int m = 0; m < NM; ++m) {
                    accP[m] = make_float2(0.f, 0.f);
                    accQ[m] = make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int t = 0; t < T; ++t) {
                    const float4 xn = xw[t * XS + k - 1 + Ns];
                    const float4 xc = xw[t * XS + k - 1];
#pragma unroll
                    for (int m = 0; m < NM; ++m) {
                        if (m < m0) continue;
                        accP[m] = ffma2(make_float2(xn.x, xn.y), yn[m][t], accP[m]);
                        accQ[m] = ffma2(make_float2(xn.z, xn.w), yn[m][t], accQ[m]);
                        accP[m] = ffma2(make_float2(xc.x, xc.y), yc[m][t], accP[m]);
                        accQ[m] = ffma2(make_float2(xc.z, xc.w), yc[m][t], accQ[m]);
                    }
                }
#pragma unroll
                for (int m = 0; m < NM; ++m) {
                    if (m < m0) continue;
                    const float2 dv = make_float2(accP[m].x + accP[m].y, accQ[m].x + accQ[m].y);
                    S[m] = fadd2(prv[m], dv);
                    const int d = m * G + r - k;  // diagonal of slot (k, m); < 0 below the diagonal
                    A[k][m] = fadd2(r0[d], S[m]);
                    if (k - m * G >= 0 && k - m * G < G && k - m * G == r) tr += A[k][m].x;
                }
            }
            __syncwarp();  // r0 aliases the pivot-row buffer

            if (C::SYNC) __syncthreads();
            // ---- diagonal loading d*tr(R)/L
#pragma unroll
            for (int o = G / 2; o; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o, G);
            // relative loading d*tr(R)/L, or an absolute d on the normalised R
            const float dl = f.loading == COS_CAPON_LOAD_ABSOLUTE ? f.d * (float)(Ns * T) : f.d * tr / (float)L;
#pragma unroll
            for (int m = 0; m < NM; ++m)
#pragma unroll
                for (int q = 0; q < G; ++q)
                    if (q == r) A[m * G + q][m].x += dl;

            // ---- optional R output (loaded covariance)
            if (MODE == FUSED_R) {
                if (f.R && active) {
                    const size_t pix = (size_t)bx * f.Npy + p;
                    float2 *Rp = f.R + pix * L * L;
                    const float norm = f.r_layout == COS_CAPON_R_REFERENCE ? 1.0f : 1.0f / ((float)Ns * (float)T);
#pragma unroll
                    for (int m = 0; m < NM; ++m) {
                        const int j = m * G + r;
#pragma unroll
                        for (int k = 0; k < L; ++k) {
                            if (k < m * G + G && k <= j) {
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
                continue;  // this mode writes R only
            }

            // ---- right-hand sides: b1 = a = 1, b2 = g (rows m*G + r); the w mode
            // carries b1 only and forms z from the back substitution's x
            float2 b1[NM], b2[NM];
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                b1[m] = make_float2(1.f, 0.f);
                b2[m] = gs[lpc * L + m * G + r];
            }

            // ---- square-root-free Cholesky (R = L D L^H, rows of D L^H kept in A)
            // with the right-hand sides carried along.  Step i leaves row i of
            // A as row i of D L^H (unscaled: A[i][i] = d_i) and eliminates it
            // from the rows below:
            //   A[k][j] -= conj(A[i][k]) A[i][j] / d_i,   b_k -= conj(A[i][k]) b_i / d_i,
            // so that b ends as L^-1 a, L^-1 g and, with y = D^-1/2 b,
            //   a^H R^-1 a = sum_i |b1_i|^2 / d_i,   a^H R^-1 g = sum_i conj(b1_i) b2_i / d_i,
            // the sums every lane accumulates from the published pivots.  Two
            // loops follow: the z/P mode's with look-ahead, and the w mode's in
            // the plain order.
            bool bad = false;
            float s11 = 0.f;
            float2 s12 = make_float2(0.f, 0.f);
            float dinv[NM];  // FUSED_W: 1/d_i of the lane's own rows, for the back substitution
#pragma unroll
            for (int m = 0; m < NM; ++m) dinv[m] = 0.f;
            if constexpr (MODE == FUSED_ZP) {
                // publish row `row` as (-Re, +Im, -Im, -Re) of A[row, j] into `buf`: with
                // the consumer's splats (vr, vr), (vi, vi) of its own A[i, j'] / d_i two
                // packed fmas give A[k][j'] -= conj(A[i,k]) A[i,j'] / d_i.  Slot `row`
                // holds d_row in its first word; slot L carries (b1_row, b2_row).
                auto publish = [&](const int row, float4 *buf) {
                    const int orow = row % G, mrow = row / G;
#pragma unroll
                    for (int m = 0; m < NM; ++m)
                        if (m >= mrow) buf[m * G + r] = make_float4(-A[row][m].x, A[row][m].y, -A[row][m].y, -A[row][m].x);
                    if (r == orow) buf[L] = make_float4(b1[mrow].x, b1[mrow].y, b2[mrow].x, b2[mrow].y);
                };
                // z/P mode looks ahead: step i updates and publishes row i+1 before its
                // bulk trailing update, so the store, the barrier and the next pivot's
                // load are off the serial chain (2.03 -> 1.99 ms per config-1 frame,
                // bit-identical).  The w mode keeps the plain order: with its factor
                // kept live it ran slower with the look-ahead (2.79 -> 2.94 ms).
                publish(0, rb);
#pragma unroll
                for (int i = 0; i < L; ++i) {
                    const int oi = i % G, mi = i / G;
                    // step i reads buffer i&1.  It was written at step i-1 and last read
                    // at step i-2, before the barrier that ended step i-1: one barrier
                    // per step suffices.
                    float4 *const rbi = rb + (i & 1) * (L + 1);
                    __syncwarp();
                    const float dv = -rbi[i].x;
                    const float4 yy = rbi[L];
                    bad |= !(dv > 0.f);
                    const float rdv = __fdividef(1.f, dv);
                    const float2 y1 = make_float2(yy.x * rdv, yy.y * rdv), y2 = make_float2(yy.z * rdv, yy.w * rdv);
                    s11 = fmaf(yy.x, y1.x, fmaf(yy.y, y1.y, s11));
                    s12 = cadd(s12, cconjmul(make_float2(yy.x, yy.y), y2));
                    // right-hand sides, rows m*G + r > i:  b -= conj(A[i,row]) * b_i / d_i
                    // (for m > mi every row of the slot is below i; for m = mi only r > i%G)
                    {
                        const float2 y1s = make_float2(y1.y, y1.x), y2s = make_float2(y2.y, y2.x);
#pragma unroll
                        for (int m = 0; m < NM; ++m) {
                            if (m < mi) continue;
                            const float2 n1 = make_float2(-A[i][m].x, -A[i][m].x), n2 = make_float2(-A[i][m].y, A[i][m].y);
                            const float2 t1 = ffma2(n2, y1s, ffma2(n1, y1, b1[m]));
                            const float2 t2 = ffma2(n2, y2s, ffma2(n1, y2, b2[m]));
                            if (m > mi || r > oi) {
                                b1[m] = t1;
                                b2[m] = t2;
                            }
                        }
                    }
                    // trailing update A[k][j] -= conj(A[i,k]) A[i,j] / d_i, i < k; slot (k,m) exists for m >= k/G
                    float2 vrr[NM], vii[NM];
#pragma unroll
                    for (int m = 0; m < NM; ++m) {
                        const float2 v = (m >= mi) ? A[i][m] : make_float2(0.f, 0.f);
                        const float vr = v.x * rdv, vi = v.y * rdv;
                        vrr[m] = make_float2(vr, vr);
                        vii[m] = make_float2(vi, vi);
                    }
                    auto update_row = [&](const int k) {
                        const float4 u4 = rbi[k];
#pragma unroll
                        for (int m = 0; m < NM; ++m)
                            if (m >= k / G && m >= mi)
                                A[k][m] = ffma2(vii[m], make_float2(u4.z, u4.w), ffma2(vrr[m], make_float2(u4.x, u4.y), A[k][m]));
                    };
                    if (i + 1 < L) {
                        update_row(i + 1);
                        publish(i + 1, rb + ((i + 1) & 1) * (L + 1));
                    }
                    // constant trip counts with compile-time conditions: loops whose
                    // bounds depend on i are otherwise not fully unrolled and the
                    // register matrix would fall back to local memory
#pragma unroll
                    for (int k = 1; k < L; ++k)
                        if (k > i + 1) update_row(k);
                    if (C::SYNC && (i % G) == G - 1) __syncthreads();
                }
            } else {
#pragma unroll
                for (int i = 0; i < L; ++i) {
                    const int oi = i % G, mi = i / G;
                    // publish row i as (-Re, +Im, -Im, -Re) of A[i, j]: with the consumer's
                    // splats (vr, vr), (vi, vi) of its own A[i, j'] / d_i two packed fmas
                    // give A[k][j'] -= conj(A[i,k]) A[i,j'] / d_i.  Slot i holds d_i in
                    // its first word; slot L carries b1_i.  The w mode carries no
                    // second right-hand side: z = x^H g / (a^H R^-1 a) follows from
                    // the back substitution's x = R^-1 a.
                    // Step i writes buffer i&1, last read at step i-2, before the
                    // barrier that ended step i-1: one barrier per step suffices.
                    float4 *const rbi = rb + (i & 1) * (L + 1);
                    float4 nq[NM];
#pragma unroll
                    for (int m = 0; m < NM; ++m) {
                        const float2 v = m >= mi ? A[i][m] : make_float2(0.f, 0.f);
                        nq[m] = make_float4(-v.x, v.y, -v.y, -v.x);
                    }
#pragma unroll
                    for (int m = 0; m < NM; ++m)
                        if (m >= mi) rbi[m * G + r] = nq[m];
                    if (r == oi) rbi[L] = make_float4(b1[mi].x, b1[mi].y, 0.f, 0.f);
                    __syncwarp();
                    const float dv = -rbi[i].x;
                    const float4 yy = rbi[L];
                    bad |= !(dv > 0.f);
                    const float rdv = __fdividef(1.f, dv);
                    if (MODE == FUSED_W) dinv[mi] = (r == oi) ? rdv : dinv[mi];
                    const float2 y1 = make_float2(yy.x * rdv, yy.y * rdv);
                    s11 = fmaf(yy.x, y1.x, fmaf(yy.y, y1.y, s11));
                    // right-hand sides, rows m*G + r > i:  b -= conj(A[i,row]) * b_i / d_i
                    // (for m > mi every row of the slot is below i; for m = mi only r > i%G)
                    {
                        const float2 y1s = make_float2(y1.y, y1.x);
#pragma unroll
                        for (int m = 0; m < NM; ++m) {
                            if (m < mi) continue;
                            const float2 n1 = make_float2(-A[i][m].x, -A[i][m].x), n2 = make_float2(-A[i][m].y, A[i][m].y);
                            const float2 t1 = ffma2(n2, y1s, ffma2(n1, y1, b1[m]));
                            if (m > mi || r > oi) b1[m] = t1;
                        }
                    }
                    // trailing update A[k][j] -= conj(A[i,k]) A[i,j] / d_i, i < k; slot (k,m) exists for m >= k/G
                    float2 vrr[NM], vii[NM];
#pragma unroll
                    for (int m = 0; m < NM; ++m) {
                        const float2 v = (m >= mi) ? A[i][m] : make_float2(0.f, 0.f);
                        const float vr = v.x * rdv, vi = v.y * rdv;
                        vrr[m] = make_float2(vr, vr);
                        vii[m] = make_float2(vi, vi);
                    }
                    // constant trip counts with compile-time conditions: loops whose
                    // bounds depend on i are otherwise not fully unrolled and the
                    // register matrix would fall back to local memory
#pragma unroll
                    for (int k = 1; k < L; ++k) {
                        if (k > i) {
                            const float4 u4 = rbi[k];
#pragma unroll
                            for (int m = 0; m < NM; ++m)
                                if (m >= k / G && m >= mi)
                                    A[k][m] = ffma2(vii[m], make_float2(u4.z, u4.w), ffma2(vrr[m], make_float2(u4.x, u4.y), A[k][m]));
                        }
                    }
                    if (C::SYNC && (i % G) == G - 1) __syncthreads();
                }
            }

            // ---- outputs (s11, and in the z/P mode s12, are complete on every lane)
            const size_t pix = (size_t)bx * f.Npy + p;
            if (active && r == 0) {
                const float is11 = 1.0f / s11;
                if (MODE == FUSED_ZP) f.z[pix] = make_float2(s12.x * is11, s12.y * is11);
                if (f.P) f.P[pix] = is11 / ((float)Ns * (float)T);
            }
            if (bad && active && r == 0) atomicOr(status, ERR_NOT_PD);

            if (MODE == FUSED_W) {
                // back substitution (D L^H) x = b1, x = R^-1 a, by blocks of G rows
                // (block m: rows m*G + q, q < G), last block first.  The code of
                // this stage runs between the factorisations of consecutive pixel
                // groups and must stay small, or it pushes their unrolled code out
                // of the instruction cache; so per block, through the (now idle)
                // pivot-row buffer, rows padded to G+1 entries (no bank conflicts):
                //   1. each lane sums its columns right of the block into the
                //      block's G rows; the partial sums are exchanged, and lane r
                //      adds up row m*G + r in a rolled loop;
                //   2. the G x G diagonal block is transposed, so lane r holds
                //      row m*G + r of it;
                //   3. a rolled loop solves the block: lane q forms x_q, a shuffle
                //      broadcasts it, lanes r < q take its term off their row.
                // Slots left of the diagonal hold unused, possibly non-finite
                // values: results are selected, never masked by a zero factor.
                float2 xv[NM];
#pragma unroll
                for (int m = 0; m < NM; ++m) xv[m] = make_float2(0.f, 0.f);
                float2 *const X = (float2 *)rb;  // G x (G+1) exchange / transpose area
#pragma unroll
                for (int m = NM - 1; m >= 0; --m) {
#pragma unroll
                    for (int q = 0; q < G; ++q) {
                        float2 e = make_float2(0.f, 0.f);
#pragma unroll
                        for (int mm = m + 1; mm < NM; ++mm) e = cadd(e, cmul(A[m * G + q][mm], xv[mm]));
                        X[q * (G + 1) + r] = e;
                    }
                    __syncwarp();
                    float2 acc = b1[m];
#pragma unroll 1
                    for (int l = 0; l < G; ++l) acc = csub(acc, X[r * (G + 1) + l]);
                    __syncwarp();
#pragma unroll
                    for (int q = 0; q < G; ++q) X[q * (G + 1) + r] = A[m * G + q][m];
                    __syncwarp();
                    float2 xm = xv[m];
#pragma unroll 1
                    for (int q = G - 1; q >= 0; --q) {
                        const float2 xq = shfl2(cscale(acc, dinv[m]), q, G);
                        if (r == q) xm = xq;
                        const float2 t = csub(acc, cmul(X[r * (G + 1) + q], xq));
                        acc = make_float2(r < q ? t.x : acc.x, r < q ? t.y : acc.y);
                    }
                    xv[m] = xm;
                    __syncwarp();  // the area is rewritten by the next block (and r0 by the next pixel)
                }
                // z = w^H g = x^H g / (a^H R^-1 a), g the subarray sums of the pixel
                float2 zp = make_float2(0.f, 0.f);
#pragma unroll
                for (int m = 0; m < NM; ++m) zp = cadd(zp, cconjmul(xv[m], gs[lpc * L + m * G + r]));
#pragma unroll
                for (int o = G / 2; o; o >>= 1) zp = cadd(zp, shfl2_xor(zp, o, G));
                const float is11 = 1.0f / s11;
                if (active && r == 0) f.z[pix] = cscale(zp, is11);
                if (active && f.w) {
#pragma unroll
                    for (int m = 0; m < NM; ++m) f.w[pix * L + m * G + r] = cscale(xv[m], is11);
                }
            }
        }
        __syncthreads();
    }
}

// ---- launch helper ---------------------------------------------------------
template <class C>
size_t smem_bytes(int K, int M)
{
    return Smem(C::TILE, K, C::M ? C::M : M, C::L, C::WARPS, C::PPW, C::RBQ).total;
}

// bytes of FramesParam::stash the refinement mode needs on num_sms SMs
template <class C>
size_t stash_bytes(int num_sms)
{
    if constexpr (!C::WIDE) {
        return 0;
    } else {
        int per_sm = 0, q = 0;
        for (auto k : {fused_kernel<C, FUSED_REFINE>, fused_kernel<C, FUSED_ADAPT_ZP>, fused_kernel<C, FUSED_ADAPT_W>}) {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, k, C::WARPS * 32, 0) != cudaSuccess) {
                cudaGetLastError();
                return 0;
            }
            per_sm = q > per_sm ? q : per_sm;
        }
        return (size_t)num_sms * per_sm * C::WARPS * C::PPW * WideStash<C::L, C::G>::Q * sizeof(float4);
    }
}

template <class C, int MODE>
int launch_cfg(FramesParam fp, unsigned *status, int num_sms, cudaStream_t s)
{
    const FrameDev &f0 = fp.f[0];
    if (!C::RT_T && 2 * f0.K + 1 != C::T) return cudaErrorNotSupported;
    for (int i = 0; i < fp.n; ++i)
        if (C::M && fp.f[i].M != C::M) return cudaErrorNotSupported;
    long long begin = 0;
    for (int i = 0; i < fp.n; ++i) {
        FrameDev &g = fp.f[i];
        g.tile = C::TILE;
        g.tiles_per_beam = (g.Npy + C::TILE - 1) / C::TILE;
        g.tile_begin = begin;
        begin += (long long)g.Nx * g.tiles_per_beam;
    }
    Smem S(C::TILE, f0.K, C::M ? C::M : f0.M, C::L, C::WARPS, C::PPW, C::RBQ);
    if (S.total > kFusedSmemMax) return cudaErrorNotSupported;
    cudaError_t e = cudaFuncSetAttribute(fused_kernel<C, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S.total);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_kernel<C, MODE>, C::WARPS * 32, S.total);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorNotSupported;
    long long grid = (long long)num_sms * per_sm;
    if (grid > begin) grid = begin;
    if ((MODE == FUSED_REFINE || MODE == FUSED_ADAPT_ZP || MODE == FUSED_ADAPT_W) &&
        (!fp.stash || fp.stash_bytes < (size_t)grid * C::WARPS * C::PPW * WideStash<C::L, C::G>::Q * sizeof(float4)))
        return cudaErrorNotSupported;
    fused_kernel<C, MODE><<<(unsigned)grid, C::WARPS * 32, S.total, s>>>(fp, begin, status);
    return cudaGetLastError();
}

// z/P, w and R modes
template <class C>
int launch_basic(const FramesParam &fp, int mode, unsigned *status, int num_sms, cudaStream_t s)
{
    switch (mode) {
    case FUSED_ZP: return launch_cfg<C, FUSED_ZP>(fp, status, num_sms, s);
    case FUSED_W: return launch_cfg<C, FUSED_W>(fp, status, num_sms, s);
    case FUSED_R: return launch_cfg<C, FUSED_R>(fp, status, num_sms, s);
    default: return cudaErrorNotSupported;
    }
}

// the refinement modes (L > 32; the wide instantiation files compile them in
// a translation unit of their own, in parallel with the others)
template <class C>
int launch_refining(const FramesParam &fp, int mode, unsigned *status, int num_sms, cudaStream_t s)
{
    if constexpr (!C::WIDE) {
        return cudaErrorNotSupported;
    } else {
        switch (mode) {
        case FUSED_REFINE: return launch_cfg<C, FUSED_REFINE>(fp, status, num_sms, s);
        case FUSED_ADAPT_ZP: return launch_cfg<C, FUSED_ADAPT_ZP>(fp, status, num_sms, s);
        case FUSED_ADAPT_W: return launch_cfg<C, FUSED_ADAPT_W>(fp, status, num_sms, s);
        default: return cudaErrorNotSupported;
        }
    }
}

// the refinement modes alone (an L <= 32 instantiation of the blocked path,
// which serves refinement next to the L <= 32 kernel's own modes)
template <class C>
int launch_refine_only(const FramesParam &fp, int mode, unsigned *status, int num_sms, cudaStream_t s)
{
    return mode <= FUSED_R ? (int)cudaErrorNotSupported : launch_refining<C>(fp, mode, status, num_sms, s);
}

template <class C>
int launch_any(const FramesParam &fp, int mode, unsigned *status, int num_sms, cudaStream_t s)
{
    return mode <= FUSED_R ? launch_basic<C>(fp, mode, status, num_sms, s)
                           : launch_refining<C>(fp, mode, status, num_sms, s);
}

}  // namespace fused
}  // namespace cgb
