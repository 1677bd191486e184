// Register Cholesky of one pixel's loaded covariance with the two Capon
// right-hand sides carried along (sm_103a, FP32, packed fma.rn.f32x2).
//
// G lanes own one pixel; lane r holds the columns j = m*G + r (m < L/G) of the
// upper triangle, A[k][m] = R[k][m*G + r] for k <= m*G + r (slots with k > j
// hold unused values).  The factorisation is the square-root-free form
// R = L D L^H of the reference's Cholesky (matrixDecompc.pyx:19-50; its factor
// is U = D^-1/2 (D L^H)): step i leaves row i of A as row i of D L^H
// (A[i][i] = d_i) and eliminates it from the rows below,
//   A[k][j] -= conj(A[i][k]) A[i][j] / d_i,   b_k -= conj(A[i][k]) b_i / d_i,
// so that b ends as L^-1 a (a = 1) and L^-1 g, and, with y = D^-1/2 b (the
// forward solve of linearSolvec.pyx:312-327),
//   s11 = a^H R^-1 a = sum_i |b1_i|^2 / d_i,   s12 = a^H R^-1 g = sum_i conj(b1_i) b2_i / d_i,
// the sums every lane accumulates from the published pivots.
//
// Each step publishes the pivot row to shared memory as (-Re, +Im, -Im, -Re)
// quads, so the trailing update of a slot is two packed fmas with the
// consumer's splats of its own A[i][j] / d_i; the row's right-hand-side
// entries travel in one extra slot.  The step looks ahead: row i+1 is updated
// and published before the bulk trailing update of step i, which takes the
// store, the barrier and the next pivot's load off the serial chain.  Two
// pivot-row buffers per pixel alternate by step: the buffer written at step i
// was last read at step i-2, before the barrier that ended step i-1, so one
// warp barrier per step suffices.
#pragma once
#include "capon_common.cuh"

namespace cgb {

// rb: this pixel group's two pivot-row buffers of L+1 quads each.
// SYNC: a CTA barrier every G steps (keeps the CTA's warps in step so that
// the unrolled instruction stream is fetched once for all of them).
template <int L, int G, bool SYNC>
COS_DEV void factor_zp(float2 (&A)[L][L / G], float2 (&b2)[L / G], float4 *rb, const int r, float &s11,
                       float2 &s12, bool &bad)
{
    constexpr int NM = L / G;
    float2 b1[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) b1[m] = make_float2(1.f, 0.f);
    // publish row `row` as (-Re, +Im, -Im, -Re) of A[row, j] into `buf`; slot
    // `row` holds d_row in its first word; slot L carries (b1_row, b2_row)
    auto publish = [&](const int row, float4 *buf) {
        const int orow = row % G, mrow = row / G;
#pragma unroll
        for (int m = 0; m < NM; ++m)
            if (m >= mrow) buf[m * G + r] = make_float4(-A[row][m].x, A[row][m].y, -A[row][m].y, -A[row][m].x);
        if (r == orow) buf[L] = make_float4(b1[mrow].x, b1[mrow].y, b2[mrow].x, b2[mrow].y);
    };
    publish(0, rb);
#pragma unroll
    for (int i = 0; i < L; ++i) {
        const int oi = i % G, mi = i / G;
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
        if (SYNC && (i % G) == G - 1) __syncthreads();
    }
}

}  // namespace cgb
