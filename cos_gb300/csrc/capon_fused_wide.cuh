// Per-pixel part of the fused element-space kernel for L > 32 (sm_103a).
//
// G lanes own one pixel and lane r the columns j = m*G + r (m < L/G) of the
// upper triangle, as in the L <= 32 kernel: at L = 64 one warp per pixel
// (G = 32, columns r and 32 + r), at L = 48 two pixels per warp (G = 16, three
// columns per lane).  Covariance, loading and factorisation run block by
// block, block b being the rows b*G .. b*G + G - 1:
//   1. the block's rows of R by the diagonal recurrence of the reference
//      buildR kernel (buildR_kernel.cu:96-131),
//        R[k,k+d] = R0[d] + S[k,k+d],  S[k,j] = S[k-1,j-1] + D[k,j],
//        D[k,j]   = sum_t x_t[k-1+Ns] conj(x_t[j-1+Ns]) - x_t[k-1] conj(x_t[j-1]),
//      R0 (the first row) and S in float-float, R rounded once;
//   2. the loading d tr(R)/L on the block's diagonal (getCaponC.pyx:257-262);
//   3. the Schur update by the rows of D L^H factored in earlier blocks,
//        A[k][j] -= conj(A[p][k]) A[p][j] / d_p,  p < b*G;
//   4. the block's own steps of the square-root-free right-looking Cholesky
//      R = L D L^H (matrixDecompc.pyx:19-50; U = D^-1/2 (D L^H)), the trailing
//      update confined to the block, the right-hand sides a = 1 and g carried
//      along (the forward solve of linearSolvec.pyx:312-327).
// This is the right-looking order with each block's updates deferred until
// its rows exist: the same arithmetic, but at most (b+1) G (L/G - b) column
// slots are live at a time (64 of the 96 a lane's columns span at L = 64), so
// the factor stays in registers (255 a thread at 8 warps, 168 at 12, with a
// few spills).
//
// Why float-float S: with Ns = M - L + 1 subarrays no longer many times L,
// S[k, .] is not small next to R (at L = 64, M = 128 row 63 spans 63 of the
// 65 subarray rows), and an FP32 running sum would round values as large as
// R 63 times.  In the z/P, w and R modes each increment D (2T products of a
// few hundredths of R at most) is summed in FP32, t outer, straight into the
// slot that later holds R.  The refinement mode adds each range row's
// increment to S by TwoSum instead, and forms the first row with exact
// products: its residual is only as good as this matrix.
//
// Refinement (FUSED_REFINE): the float-float R goes to a per-warp stash, and
// after the factorisation x0 = R~^-1 a is corrected once by the FP64-assembled
// residual a - (R + dl I) x0.  The adaptive modes (FUSED_ADAPT_*) run the z/P
// or w mode on every pixel and the refinement pass on the pixels whose pivot
// spread exceeds kAdaptiveSpread.
//
// The trace for the loading is needed before block 0 is factored, when most
// rows do not exist yet; it is summed directly,
//   tr(R) = L R0[0] + sum_{k=1}^{L-1} (L - k) D[k,k].
//
// The temporal window T = 2K+1 may be a run-time value (Cfg T = 0): every
// window loop of this path is rolled.
#pragma once
#include <type_traits>

#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {
namespace fused {

// f(std::integral_constant<int, I>) for I = B .. E-1 in order: loops whose index
// must be a compile-time constant (it indexes the register matrix) however
// large the body, where a pragma unroll would stop at the compiler's size
// threshold and leave the matrix in local memory.  The bodies are lambdas
// marked always_inline: one left out of line would take the register matrix
// by reference, i.e. in local memory.
template <int B, int E, class F>
COS_DEV void static_for(F &&f)
{
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

// shared area of one pixel group for the wide path (float4 units; Cfg::RBQ
// also covers the back substitution's exchange and the refinement's residual):
//   [0, L+G)                   first covariance row, hi at float2 G + d, lo at L + 2G + d (-G < d < L)
//   [L+G, L+G + 2(L+1))        two pivot-row buffers (the Schur steps use their first G slots)
//   then L floats              1/d_p of the factored rows
// The w mode's back substitution reuses the area from 0 as its G x (G+1) exchange.
template <int L, int G>
struct WideArea {
    static constexpr int R0Q = L + G;
    static constexpr int PBQ = R0Q;
    static constexpr int DINVQ = PBQ + 2 * (L + 1);
    static constexpr int Q = DINVQ + (L + 3) / 4;
};

// float-float covariance slots kept for the refinement's residual, one region
// per pixel group: slot (k, m) of lane r (row k of column m*G + r, k < m*G + G)
// at float4 index slot(k, m) * G + r, as (hi.re, hi.im, lo.re, lo.im)
template <int L, int G>
struct WideStash {
    static constexpr int NM = L / G;
    static constexpr int SLOTS = G * NM * (NM + 1) / 2;
    static constexpr size_t Q = (size_t)SLOTS * G;  // float4 per group
    COS_DEV static int slot(int k, int m) { return G * m * (m + 1) / 2 + k; }
};

COS_DEV float2 fmul2(float2 a, float2 b)
{
    uint64_t ra = *reinterpret_cast<uint64_t *>(&a);
    uint64_t rb = *reinterpret_cast<uint64_t *>(&b);
    uint64_t rd;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    return *reinterpret_cast<float2 *>(&rd);
}
// (h, l) += (bh, bl), float-float complex
COS_DEV void ff_add(float2 &h, float2 &l, float2 bh, float2 bl)
{
    two_sum_acc(h, l, bh);
    l = fadd2(l, bl);
}
// (h, l) += (a + alo) x with the product of the high part exact (TwoProd by
// fma) and the low part's in FP32.  With xa = (x.re, x.im) and
// xb = (-x.im, x.re) this is a x; with xb = (x.im, -x.re) it is conj(a) x.
COS_DEV void ff_cmac(float2 &h, float2 &l, float4 a, float2 xa, float2 xb)
{
    const float2 sx = make_float2(a.x, a.x), sy = make_float2(a.y, a.y);
    const float2 p1 = fmul2(sx, xa), p2 = fmul2(sy, xb);
    const float2 e1 = ffma2(sx, xa, make_float2(-p1.x, -p1.y)), e2 = ffma2(sy, xb, make_float2(-p2.x, -p2.y));
    two_sum_acc(h, l, p1);
    two_sum_acc(h, l, p2);
    l = fadd2(l, fadd2(e1, e2));
    l = ffma2(make_float2(a.z, a.z), xa, l);
    l = ffma2(make_float2(a.w, a.w), xb, l);
}

// MODE: FUSED_ZP, FUSED_W, FUSED_R or FUSED_REFINE.  OWN_R0: the first
// covariance row is formed here, with exact products, from the pixel's own
// range rows (the refinement pass of the adaptive mode, whose tile carries
// the ordinary rows).  spread (z/P and w modes): the factorisation's pivot
// spread max d_i / min d_i, which the adaptive mode tests.
template <class C, int MODE, bool OWN_R0 = false>
COS_DEV void wide_pixel(const FrameDev &f, const float4 *xw, const int XS, const int Ns, const float2 *crow,
                        const float2 *clrow, const float2 *grow, float4 *area, float4 *stash, const int r,
                        const bool active, const size_t pix, unsigned *status, float *spread = nullptr)
{
    constexpr int L = C::L, G = C::G, NM = C::NM;
    const int T = C::RT_T ? 2 * f.K + 1 : C::T;
    // the w and the refinement modes carry the right-hand side a only and keep
    // the factor for the back substitution
    constexpr bool WMODE = MODE == FUSED_W || MODE == FUSED_REFINE;
    using WA = WideArea<L, G>;
    using WS = WideStash<L, G>;
    static_assert(WA::Q <= C::RBQ && (G * (G + 1) + 1) / 2 <= C::RBQ && (L + 1) / 2 + 8 * G <= C::RBQ,
                  "the pixel group's shared area holds every phase's layout");
    float2 *const r0h = (float2 *)area + G;
    float2 *const r0l = r0h + L + G;
    float4 *const pb = area + WA::PBQ;
    float *const dinv_s = (float *)(area + WA::DINVQ);

    // ---- first row R0[d] = sum_t c_{y+t}[d] in float-float: hi = fl(R0), lo the rest
#pragma unroll
    for (int m = 0; m < NM; ++m) {
        const int j = m * G + r;
        float2 h = make_float2(0.f, 0.f), l = make_float2(0.f, 0.f);
        if constexpr (OWN_R0) {
            // sum_t sum_s x_t[s] conj(x_t[s+j]), exact products (TwoProd by fma)
            for (int t = 0; t < T; ++t) {
                const float4 *xr = xw + t * XS;
#pragma unroll 4
                for (int s = 0; s < Ns; ++s) {
                    const float4 a = xr[s], c = xr[s + j];
                    const float2 an = make_float2(a.x, a.y), az = make_float2(a.z, a.w);
                    const float2 sr = make_float2(c.x, c.x), si = make_float2(c.y, c.y);
                    const float2 p1 = fmul2(sr, an), p2 = fmul2(si, az);
                    const float2 e = fadd2(ffma2(sr, an, make_float2(-p1.x, -p1.y)),
                                           ffma2(si, az, make_float2(-p2.x, -p2.y)));
                    two_sum_acc(h, l, p1);
                    two_sum_acc(h, l, p2);
                    l = fadd2(l, e);
                }
            }
        } else {
            for (int t = 0; t < T; ++t) {
                two_sum_acc(h, l, crow[t * L + j]);
                l = fadd2(l, clrow[t * L + j]);
            }
        }
        const float2 s = fadd2(h, l);
        r0h[j] = s;
        r0l[j] = fsub2(l, fsub2(s, h));
    }
    // ---- trace: L R0[0] + sum_k (L - k) D[k,k], D[k,k] = sum_t |x_t[k-1+Ns]|^2 - |x_t[k-1]|^2
    float trp = 0.f;
#pragma unroll
    for (int m = 0; m < NM; ++m) {
        const int k = m * G + r;
        if (k >= 1) {
            float dd = 0.f;
            for (int t = 0; t < T; ++t) {
                const float4 a = xw[t * XS + k - 1 + Ns], c = xw[t * XS + k - 1];
                dd = fmaf(a.x, a.x, fmaf(a.y, a.y, dd));
                dd = fmaf(-c.x, c.x, fmaf(-c.y, c.y, dd));
            }
            trp = fmaf((float)(L - k), dd, trp);
        }
    }
#pragma unroll
    for (int o = G / 2; o; o >>= 1) trp += __shfl_xor_sync(0xffffffffu, trp, o, G);
    __syncwarp();  // r0h / r0l complete
    const float tr = fmaf((float)L, r0h[0].x + r0l[0].x, trp);
    // relative loading d*tr(R)/L, or an absolute d on the normalised R
    const float dl = f.loading == COS_CAPON_LOAD_ABSOLUTE ? f.d * (float)(Ns * T) : f.d * tr / (float)L;

    float2 A[L][NM];
    float2 Sh[NM], Sl[NM];  // running S of the lane's columns, float-float
    float2 b1[NM], b2[NM];  // right-hand sides a = 1 and g, rows m*G + r
    float dinv[NM];         // w and refinement modes: 1/d of the lane's own rows
    bool bad = false;
    float dmin = 3.0e38f, dmax = 0.f;  // pivot range
    float s11 = 0.f;
    float2 s12 = make_float2(0.f, 0.f);
#pragma unroll
    for (int m = 0; m < NM; ++m) {
        Sh[m] = Sl[m] = make_float2(0.f, 0.f);
        A[0][m] = r0h[m * G + r];
        if constexpr (MODE == FUSED_REFINE) {
            const float2 lo = r0l[m * G + r];
            __stcg(stash + WS::slot(0, m) * G + r, make_float4(A[0][m].x, A[0][m].y, lo.x, lo.y));
        }
        b1[m] = make_float2(1.f, 0.f);
        b2[m] = MODE == FUSED_ZP ? grow[m * G + r] : make_float2(0.f, 0.f);
        dinv[m] = 0.f;
    }

    static_for<0, NM>([&](auto bc) __attribute__((always_inline)) {
        constexpr int b = decltype(bc)::value;
        constexpr int k0 = b * G > 0 ? b * G : 1, k1 = b * G + G;

        // R0 + S for slot (k, m), rounded once into the register matrix; the
        // refinement mode also keeps the float-float value
        auto finish = [&](const int k, const int m, const float2 h, const float2 l) __attribute__((always_inline)) {
            const int d = m * G + r - k;  // diagonal of slot (k, m); < 0 below the diagonal
            float2 rh = r0h[d], rl = fadd2(r0l[d], l);
            two_sum_acc(rh, rl, h);  // R0 + S
            const float2 v = fadd2(rh, rl);
            A[k][m] = v;
            if constexpr (MODE == FUSED_REFINE) {
                if (k <= m * G + r) {  // the rest of R, exactly: lo = (rh + rl) - v
                    const float2 lo = fsub2(rl, fsub2(v, rh));
                    __stcg(stash + WS::slot(k, m) * G + r, make_float4(v.x, v.y, lo.x, lo.y));
                }
            }
        };
        if constexpr (MODE == FUSED_REFINE) {
            // ---- 1. rows [k0, k1), row outer: each range row's increment
            // D_t[k,j] (four fmas from zero, so rounded at the size of its own
            // products) enters the float-float S by TwoSum.  Summed over t in
            // FP32 first, as the other modes do, the running sum grows to T
            // increments and its rounding to about an ulp of R; the
            // refinement's residual is only as good as this matrix.
#pragma unroll
            for (int k = k0; k < k1; ++k) {
                float2 h[NM], l[NM];
#pragma unroll
                for (int m = b; m < NM; ++m) {
                    const bool wrap = m > 0 && k - 1 < m * G && r == G - 1;
                    const int mp = m > 0 ? m - 1 : 0;
                    h[m] = shfl2(wrap ? Sh[mp] : Sh[m], (r + G - 1) % G, G);
                    l[m] = shfl2(wrap ? Sl[mp] : Sl[m], (r + G - 1) % G, G);
                }
#pragma unroll 1
                for (int t = 0; t < T; ++t) {
                    const float4 *xr = xw + t * XS;
                    const float4 xn = xr[k - 1 + Ns], xc = xr[k - 1];
#pragma unroll
                    for (int m = b; m < NM; ++m) {
                        const int j = m * G + r, jm = j > 0 ? j - 1 : 0;
                        const float4 a = xr[jm + Ns], c = xr[jm];
                        float2 dv = fmul2(make_float2(xn.x, xn.y), make_float2(a.x, a.x));
                        dv = ffma2(make_float2(xn.z, xn.w), make_float2(a.y, a.y), dv);
                        dv = ffma2(make_float2(xc.x, xc.y), make_float2(-c.x, -c.x), dv);
                        dv = ffma2(make_float2(xc.z, xc.w), make_float2(-c.y, -c.y), dv);
                        two_sum_acc(h[m], l[m], dv);
                    }
                }
#pragma unroll
                for (int m = b; m < NM; ++m) {
                    Sh[m] = h[m];
                    Sl[m] = l[m];
                    finish(k, m, h[m], l[m]);
                }
            }
        } else {
            // ---- 1. rows [k0, k1): increments D, t outer, into the slots
#pragma unroll
            for (int k = k0; k < k1; ++k)
#pragma unroll
                for (int m = b; m < NM; ++m) A[k][m] = make_float2(0.f, 0.f);
#pragma unroll 1
            for (int t = 0; t < T; ++t) {
                const float4 *xr = xw + t * XS;
                // splats of the lane's column operands x_t[j-1+Ns] and -x_t[j-1]
                float2 nr[NM], ni[NM], cr[NM], ci[NM];
#pragma unroll
                for (int m = b; m < NM; ++m) {
                    const int j = m * G + r, jm = j > 0 ? j - 1 : 0;
                    const float4 a = xr[jm + Ns], c = xr[jm];
                    nr[m] = make_float2(a.x, a.x);
                    ni[m] = make_float2(a.y, a.y);
                    cr[m] = make_float2(-c.x, -c.x);
                    ci[m] = make_float2(-c.y, -c.y);
                }
                // with the row quads (xr, xi, xi, -xr), x conj(y) is two packed fmas
#pragma unroll
                for (int k = k0; k < k1; ++k) {
                    const float4 xn = xr[k - 1 + Ns], xc = xr[k - 1];
#pragma unroll
                    for (int m = b; m < NM; ++m) {
                        float2 acc = A[k][m];
                        acc = ffma2(make_float2(xn.x, xn.y), nr[m], acc);
                        acc = ffma2(make_float2(xn.z, xn.w), ni[m], acc);
                        acc = ffma2(make_float2(xc.x, xc.y), cr[m], acc);
                        acc = ffma2(make_float2(xc.z, xc.w), ci[m], acc);
                        A[k][m] = acc;
                    }
                }
            }
            // recurrence: S[k-1, j-1] from lane r-1 (lane 0: slot m-1 of lane G-1)
#pragma unroll
            for (int k = k0; k < k1; ++k) {
                float2 ph[NM], pl[NM];
#pragma unroll
                for (int m = b; m < NM; ++m) {
                    const bool wrap = m > 0 && k - 1 < m * G && r == G - 1;
                    const int mp = m > 0 ? m - 1 : 0;
                    ph[m] = shfl2(wrap ? Sh[mp] : Sh[m], (r + G - 1) % G, G);
                    pl[m] = shfl2(wrap ? Sl[mp] : Sl[m], (r + G - 1) % G, G);
                }
#pragma unroll
                for (int m = b; m < NM; ++m) {
                    float2 h = ph[m], l = pl[m];
                    two_sum_acc(h, l, A[k][m]);  // S = S_prev + D
                    Sh[m] = h;
                    Sl[m] = l;
                    finish(k, m, h, l);
                }
            }
        }

        // SYNC: barriers at fixed points of the unrolled code keep the CTA's
        // warps in step, so that each stretch of it is fetched once for all
        if (C::SYNC) __syncthreads();
        // ---- 2. loading on the block's diagonal (row b*G + r, slot b)
#pragma unroll
        for (int q = 0; q < G; ++q)
            if (q == r) A[b * G + q][b].x += dl;

        if constexpr (MODE == FUSED_R) {
            // the loaded covariance, rows of this block
            if (f.R && active) {
                float2 *Rp = f.R + pix * L * L;
                const float norm = f.r_layout == COS_CAPON_R_REFERENCE ? 1.0f : 1.0f / ((float)Ns * (float)T);
#pragma unroll
                for (int m = b; m < NM; ++m) {
                    const int j = m * G + r;
#pragma unroll
                    for (int k = b * G; k < k1; ++k) {
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
        } else {
            // ---- 3. Schur update by the rows p < b*G of D L^H: step p publishes
            // A[p][b*G + q] (lane q, slot b) as (-Re, +Im, -Im, -Re) quads; the
            // buffers alternate by p, one barrier per step (the buffer written
            // at step p was last read at step p-2)
            static_for<0, b * G>([&](auto pc) __attribute__((always_inline)) {
                constexpr int p = decltype(pc)::value;
                float4 *const buf = pb + (p & 1) * (L + 1);
                {
                    const float2 u = A[p][b];
                    buf[r] = make_float4(-u.x, u.y, -u.y, -u.x);
                }
                __syncwarp();
                const float dp = dinv_s[p];
                float2 vrr[NM], vii[NM];
#pragma unroll
                for (int m = b; m < NM; ++m) {
                    const float vr = A[p][m].x * dp, vi = A[p][m].y * dp;
                    vrr[m] = make_float2(vr, vr);
                    vii[m] = make_float2(vi, vi);
                }
#pragma unroll
                for (int q = 0; q < G; ++q) {
                    const float4 u4 = buf[q];
#pragma unroll
                    for (int m = b; m < NM; ++m)
                        A[b * G + q][m] = ffma2(vii[m], make_float2(u4.z, u4.w),
                                                ffma2(vrr[m], make_float2(u4.x, u4.y), A[b * G + q][m]));
                }
                if (C::SYNC && p % 8 == 7) __syncthreads();
            });

            // ---- 4. the block's factorisation steps
            static_for<b * G, k1>([&](auto ic) __attribute__((always_inline)) {
                constexpr int i = decltype(ic)::value;
                constexpr int oi = i % G;
                float4 *const buf = pb + (i & 1) * (L + 1);
                // publish row i: slot i holds d_i in its first word, slot L the
                // right-hand sides of row i
#pragma unroll
                for (int m = b; m < NM; ++m)
                    buf[m * G + r] = make_float4(-A[i][m].x, A[i][m].y, -A[i][m].y, -A[i][m].x);
                if (r == oi)
                    buf[L] = MODE == FUSED_ZP ? make_float4(b1[b].x, b1[b].y, b2[b].x, b2[b].y)
                                              : make_float4(b1[b].x, b1[b].y, 0.f, 0.f);
                __syncwarp();
                const float dv = -buf[i].x;
                const float4 yy = buf[L];
                bad |= !(dv > 0.f);
                dmin = fminf(dmin, dv);
                dmax = fmaxf(dmax, dv);
                const float rdv = __frcp_rn(dv);
                if (b + 1 < NM && r == 0) dinv_s[i] = rdv;
                if (WMODE && r == oi) dinv[b] = rdv;
                const float2 y1 = make_float2(yy.x * rdv, yy.y * rdv), y2 = make_float2(yy.z * rdv, yy.w * rdv);
                s11 = fmaf(yy.x, y1.x, fmaf(yy.y, y1.y, s11));
                if (MODE == FUSED_ZP) s12 = cadd(s12, cconjmul(make_float2(yy.x, yy.y), y2));
                // right-hand sides, rows m*G + r > i:  b -= conj(A[i,row]) * b_i / d_i
                {
                    const float2 y1s = make_float2(y1.y, y1.x), y2s = make_float2(y2.y, y2.x);
#pragma unroll
                    for (int m = b; m < NM; ++m) {
                        const float2 n1 = make_float2(-A[i][m].x, -A[i][m].x), n2 = make_float2(-A[i][m].y, A[i][m].y);
                        const float2 t1 = ffma2(n2, y1s, ffma2(n1, y1, b1[m]));
                        const float2 t2 = ffma2(n2, y2s, ffma2(n1, y2, b2[m]));
                        if (m > b || r > oi) {
                            b1[m] = t1;
                            if (MODE == FUSED_ZP) b2[m] = t2;
                        }
                    }
                }
                // trailing update inside the block, rows i < k < k1
                float2 vrr[NM], vii[NM];
#pragma unroll
                for (int m = b; m < NM; ++m) {
                    const float vr = A[i][m].x * rdv, vi = A[i][m].y * rdv;
                    vrr[m] = make_float2(vr, vr);
                    vii[m] = make_float2(vi, vi);
                }
#pragma unroll
                for (int k = i + 1; k < k1; ++k) {
                    const float4 u4 = buf[k];
#pragma unroll
                    for (int m = b; m < NM; ++m)
                        A[k][m] = ffma2(vii[m], make_float2(u4.z, u4.w), ffma2(vrr[m], make_float2(u4.x, u4.y), A[k][m]));
                }
                if (C::SYNC && i % 8 == 7) __syncthreads();
            });
        }
    });
    if constexpr (MODE == FUSED_R) return;
    if (spread) *spread = bad ? 3.0e38f : dmax / dmin;

    // ---- outputs (s11, and in the z/P mode s12, are complete on every lane)
    if (MODE != FUSED_REFINE && active && r == 0) {
        const float is11 = 1.0f / s11;
        if (MODE == FUSED_ZP) f.z[pix] = make_float2(s12.x * is11, s12.y * is11);
        if (f.P) f.P[pix] = is11 / ((float)Ns * (float)T);
    }
    if (bad && active && r == 0) atomicOr(status, ERR_NOT_PD);

    if constexpr (WMODE) {
        // back substitution (D L^H) x = y by blocks of G rows, last block
        // first, through the G x (G+1) exchange area (see the L <= 32
        // kernel): partial sums of the columns right of the block, the
        // block's diagonal part transposed, then a rolled solve
        float2 *const X = (float2 *)area;
        auto back_subst = [&](const float2 (&y)[NM], float2 (&xv)[NM]) __attribute__((always_inline)) {
            __syncwarp();  // the area's earlier contents are no longer read
#pragma unroll
            for (int m = 0; m < NM; ++m) xv[m] = make_float2(0.f, 0.f);
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
                float2 acc = y[m];
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
                __syncwarp();
            }
        };
        float2 xv[NM];  // x = R^-1 a (unscaled), rows m*G + r
        back_subst(b1, xv);
        float s = s11;  // a^H R^-1 a
        if constexpr (MODE == FUSED_REFINE) {
            // ---- one refinement step: r = a - (R + dl I) x0 with R the
            // float-float covariance (its slots from the stash), x1 = x0 + R~^-1 r
            // with the FP32 factor R~ = L D L^H.  Each stored entry R[k][j]
            // (k <= j, lane j % G) gives R[k][j] x0_j to row k (summed across
            // lanes through shared memory, 8 rows at a time) and, k < j,
            // conj(R[k][j]) x0_k to row j (the lane's own).  Products of the
            // high parts are exact, sums float-float; the residual itself is
            // assembled in FP64.
            float2 *const xs = (float2 *)area;         // x0, L entries
            float4 *const red = area + (L + 1) / 2;    // 8 rows x G partial sums (within Cfg::RBQ)
            __syncwarp();
#pragma unroll
            for (int m = 0; m < NM; ++m) xs[m * G + r] = xv[m];
            __syncwarp();
            float2 lh[NM], ll[NM], th[NM], tl[NM], xa[NM], xb[NM];
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                lh[m] = ll[m] = th[m] = tl[m] = make_float2(0.f, 0.f);
                xa[m] = xv[m];
                xb[m] = make_float2(-xv[m].y, xv[m].x);
            }
#pragma unroll 1
            for (int c = 0; c < L / 8; ++c) {
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) {
                    const int k = c * 8 + kk;
                    const float2 xk = xs[k], xkb = make_float2(xk.y, -xk.x);
                    float2 ph = make_float2(0.f, 0.f), pl = make_float2(0.f, 0.f);
#pragma unroll
                    for (int m = 0; m < NM; ++m) {
                        const int j = m * G + r;
                        if (k <= j) {
                            const float4 e = __ldcg(stash + WS::slot(k, m) * G + r);
                            ff_cmac(ph, pl, e, xa[m], xb[m]);
                            if (k < j) ff_cmac(lh[m], ll[m], e, xk, xkb);
                        }
                    }
                    red[kk * G + r] = make_float4(ph.x, ph.y, pl.x, pl.y);
                }
                __syncwarp();
                // lane r adds up entries (r & ~7) .. +8 of row r & 7, then the
                // lanes of equal r & 7 combine; the owner of the row keeps it
                {
                    const int kk = r & 7, e0 = r & ~7;
                    float2 sh = make_float2(0.f, 0.f), sl = make_float2(0.f, 0.f);
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const float4 v = red[kk * G + e0 + e];
                        ff_add(sh, sl, make_float2(v.x, v.y), make_float2(v.z, v.w));
                    }
#pragma unroll
                    for (int o = 8; o < G; o <<= 1) ff_add(sh, sl, shfl2_xor(sh, o, G), shfl2_xor(sl, o, G));
                    if (e0 == (c * 8) % G) {
                        const int mk = (c * 8) / G;
#pragma unroll
                        for (int m = 0; m < NM; ++m)
                            if (m == mk) ff_add(th[m], tl[m], sh, sl);
                    }
                }
                __syncwarp();
            }
            float2 y[NM];
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                ff_add(lh[m], ll[m], th[m], tl[m]);
                const double rre = (1.0 - (double)dl * (double)xv[m].x) - (double)lh[m].x - (double)ll[m].x;
                const double rim = (0.0 - (double)dl * (double)xv[m].y) - (double)lh[m].y - (double)ll[m].y;
                y[m] = make_float2((float)rre, (float)rim);
            }
            // forward solve L y = r (the right-hand-side update of the
            // factorisation steps, replayed: L[k][i] = conj(A[i][k]) / d_i)
            static_for<0, L>([&](auto ic) __attribute__((always_inline)) {
                constexpr int i = decltype(ic)::value, oi = i % G, mi = i / G;
                const float2 yd = shfl2(cscale(y[mi], dinv[mi]), oi, G);
#pragma unroll
                for (int m = mi; m < NM; ++m) {
                    const float2 t = cnmac_conj(y[m], make_float2(-A[i][m].x, -A[i][m].x),
                                                make_float2(-A[i][m].y, A[i][m].y), yd);
                    if (m > mi || r > oi) y[m] = t;
                }
            });
            float2 dx[NM];
            back_subst(y, dx);
#pragma unroll
            for (int m = 0; m < NM; ++m) xv[m] = cadd(xv[m], dx[m]);
            // a^H x1 in float-float (its terms may cancel)
            float2 sh = make_float2(0.f, 0.f), sl = make_float2(0.f, 0.f);
#pragma unroll
            for (int m = 0; m < NM; ++m) two_sum_acc(sh, sl, xv[m]);
#pragma unroll
            for (int o = G / 2; o; o >>= 1) ff_add(sh, sl, shfl2_xor(sh, o, G), shfl2_xor(sl, o, G));
            s = sh.x + sl.x;
            if (active && r == 0 && f.P) f.P[pix] = 1.0f / (s * ((float)Ns * (float)T));
        }
        // z = w^H g = x^H g / (a^H R^-1 a)
        float2 zp = make_float2(0.f, 0.f);
#pragma unroll
        for (int m = 0; m < NM; ++m) zp = cadd(zp, cconjmul(xv[m], grow[m * G + r]));
#pragma unroll
        for (int o = G / 2; o; o >>= 1) zp = cadd(zp, shfl2_xor(zp, o, G));
        const float is = 1.0f / s;
        if (active && r == 0) f.z[pix] = cscale(zp, is);
        if (active && f.w) {
#pragma unroll
            for (int m = 0; m < NM; ++m) f.w[pix * L + m * G + r] = cscale(xv[m], is);
        }
    }
}

}  // namespace fused
}  // namespace cgb
