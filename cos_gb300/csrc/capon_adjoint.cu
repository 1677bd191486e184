// Adjoint of the Capon output power for sm_103a.
//
// With the normalised, loaded covariance R_d = R + d I,
// R = 1/(Ns T) sum_{t,s} x_ts x_ts^H (x_ts the L-sample subarray s of range
// snapshot t), and the MVDR weights w = R_d^-1 a / (a^H R_d^-1 a), the power
// P = 1/(a^H R_d^-1 a) = w^H R_d w is stationary in w, so
//     dP = w^H dR_d w.
// Hence, per pixel, with e_ts = w^H x_ts:
//     dP/d conj(x_t[a]) = 1/(Ns T) sum_s e_ts w_{a-s}        (0 <= a-s < L)
//     dP/dd             = |w|^2
// and, for a per-channel phase x'_m = x_m exp(-j theta_m),
//     dP/dtheta_m       = 2 sum_t Im(conj(dP/dconj(x'_t[m])) x'_t[m]).
// Only the saved weights are needed: the covariance's adjoint is applied in
// factored form through e_ts, so R is neither stored nor rebuilt.
//
// Work units are range tiles of one beam (as in the forward kernel).  The CTA
// stages the tile's TILE+2K rows, each warp takes pixels of the tile, and the
// gradient rows are accumulated in shared memory; rows only this tile touches
// are added to the output directly, the 2K rows at each end (shared with the
// neighbouring tiles) with atomics.  Tiles without incoming gradient are
// skipped.
#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {

static constexpr int kAdjWarps = 8;
static constexpr int kAdjTile = 32;

__global__ void __launch_bounds__(32 * kAdjWarps) adjoint_kernel(AdjDev a)
{
    extern __shared__ float2 smem[];
    const int M = a.M, L = a.L, K = a.K, T = 2 * K + 1, Ns = M - L + 1;
    const int rows = kAdjTile + 2 * K;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float2 *xs = smem;                          // rows x M
    float2 *gs = xs + (size_t)rows * M;         // rows x M gradient accumulator
    float *ths = (float *)(gs + (size_t)rows * M);   // M channel sums
    float2 *wbuf = (float2 *)(ths + ((M + 1) & ~1)) + (size_t)warp * (L + T * Ns);
    float2 *ws = wbuf, *es = wbuf + L;
    const float scale = 1.0f / ((float)Ns * (float)T);
    const int tiles_per_beam = (a.Npy + kAdjTile - 1) / kAdjTile;
    const long long units = (long long)a.Nx * tiles_per_beam;
    float dacc = 0.f;

    for (int i = tid; i < M; i += blockDim.x) ths[i] = 0.f;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        const int bx = (int)(u / tiles_per_beam);
        const int p0 = (int)(u % tiles_per_beam) * kAdjTile;
        const int np = min(kAdjTile, a.Npy - p0);
        const int nr = np + 2 * K;
        // skip tiles with no incoming gradient
        bool any = false;
        for (int q = lane; q < np; q += 32) any |= (a.gP[(size_t)bx * a.Npy + p0 + q] != 0.f);
        if (!__syncthreads_or(any)) continue;
        const float2 *xg = a.x + ((size_t)bx * a.Ny + p0) * M;
        for (int i = tid; i < nr * M; i += blockDim.x) {
            xs[i] = xg[i];
            gs[i] = make_float2(0.f, 0.f);
        }
        __syncthreads();
        for (int q = warp; q < np; q += kAdjWarps) {
            const long long pix = (long long)bx * a.Npy + p0 + q;
            const float g = a.gP[pix];
            if (g == 0.f) continue;  // warp-uniform
            float wn = 0.f;
            for (int l = lane; l < L; l += 32) {
                const float2 wl = a.w[(size_t)pix * L + l];
                ws[l] = wl;
                wn += cabs2(wl);
            }
            for (int o = 16; o; o >>= 1) wn += __shfl_xor_sync(0xffffffffu, wn, o);
            if (lane == 0) dacc += g * wn;
            __syncwarp();
            // e_ts = w^H x_ts for the pixel's rows q .. q+2K
            for (int r = lane; r < T * Ns; r += 32) {
                const int t = r / Ns, s = r % Ns;
                const float2 *xt = xs + (size_t)(q + t) * M + s;
                float2 e = make_float2(0.f, 0.f);
                for (int l = 0; l < L; ++l) e = cadd(e, cconjmul(ws[l], xt[l]));
                es[r] = e;
            }
            __syncwarp();
            // dP/dconj(x_t[c]) into the shared accumulator (rows q+t are shared
            // by up to 2K+1 pixels of this tile: shared-memory atomics)
            for (int c = lane; c < M; c += 32) {
                const int s0 = max(0, c - L + 1), s1 = min(Ns - 1, c);
                for (int t = 0; t < T; ++t) {
                    float2 G = make_float2(0.f, 0.f);
                    for (int s = s0; s <= s1; ++s) G = cadd(G, cmul(es[t * Ns + s], ws[c - s]));
                    G = cscale(G, g * scale);
                    float2 *dst = gs + (size_t)(q + t) * M + c;
                    atomicAdd(&dst->x, G.x);
                    atomicAdd(&dst->y, G.y);
                }
            }
            __syncwarp();
        }
        __syncthreads();
        // write the tile's gradient rows; the channel-phase sums use them
        float2 *gout = a.gx + ((size_t)bx * a.Ny + p0) * M;
        for (int i = tid; i < nr * M; i += blockDim.x) {
            const int r = i / M, c = i % M;
            const float2 G = gs[i];
            if (G.x == 0.f && G.y == 0.f) continue;
            const float2 xv = xs[i];
            atomicAdd(&ths[c], 2.f * (G.x * xv.y - G.y * xv.x));
            // rows 0..2K-1 and the last 2K are shared with the neighbouring tiles
            if (r < 2 * K || r >= np) {
                atomicAdd(&gout[i].x, G.x);
                atomicAdd(&gout[i].y, G.y);
            } else {
                const float2 o = gout[i];
                gout[i] = make_float2(o.x + G.x, o.y + G.y);
            }
        }
        __syncthreads();
    }
    if (a.gth)
        for (int i = tid; i < M; i += blockDim.x)
            if (ths[i] != 0.f) atomicAdd(&a.gth[i], ths[i]);
    if (a.gd && lane == 0 && dacc != 0.f) atomicAdd(a.gd, dacc);
}

// Blocks of the register-blocked kernel and its shared-memory row padding:
// odd block lengths and an odd row pad spread the lanes of one load over the
// banks (at M=64, L=32, K=2 at most 2-3 lanes share a bank pair).
static constexpr int kAdjSB = 7, kAdjCB = 11, kAdjPad = 3;

// The same adjoint with the weights held in registers (L a template
// parameter) and both products register-blocked, for L = 8, 16, 32:
//   e_ts for SB consecutive s of one row t per lane: each sample x_t[s0+i]
//        is loaded once and meets w_l for every (s, l) with s - s0 + l = i;
//   G_t[c] = sum_s e_ts w_{c-s} for CB consecutive channels per lane: each
//        e_ts is loaded once and meets w_l for every (c, l) with c - l = s.
// Loads per complex multiply-add fall from two (the kernel above, bound by
// shared-memory bandwidth) to (SB + L - 1) / (SB L) and (CB + L - 1) / (CB L).
template <int LT>
__global__ void __launch_bounds__(32 * kAdjWarps) adjoint_blocked_kernel(AdjDev a)
{
    constexpr int SB = kAdjSB, CB = kAdjCB;
    extern __shared__ float2 smem[];
    const int M = a.M, K = a.K, T = 2 * K + 1, Ns = M - LT + 1, XS = M + kAdjPad;
    const int rows = kAdjTile + 2 * K;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float2 *xs = smem;                          // rows x XS
    float2 *gs = xs + (size_t)rows * XS;        // rows x XS gradient accumulator
    float *ths = (float *)(gs + (size_t)rows * XS);  // M channel sums
    float2 *wbuf = (float2 *)(ths + ((M + 1) & ~1)) + (size_t)warp * (LT + T * Ns);
    float2 *ws = wbuf, *es = wbuf + LT;
    const float scale = 1.0f / ((float)Ns * (float)T);
    const int tiles_per_beam = (a.Npy + kAdjTile - 1) / kAdjTile;
    const long long units = (long long)a.Nx * tiles_per_beam;
    const int nsb = (Ns + SB - 1) / SB, ncb = (M + CB - 1) / CB;
    float dacc = 0.f;

    for (int i = tid; i < M; i += blockDim.x) ths[i] = 0.f;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        const int bx = (int)(u / tiles_per_beam);
        const int p0 = (int)(u % tiles_per_beam) * kAdjTile;
        const int np = min(kAdjTile, a.Npy - p0);
        const int nr = np + 2 * K;
        bool any = false;
        for (int q = lane; q < np; q += 32) any |= (a.gP[(size_t)bx * a.Npy + p0 + q] != 0.f);
        if (!__syncthreads_or(any)) continue;
        const float2 *xg = a.x + ((size_t)bx * a.Ny + p0) * M;
        for (int i = tid; i < nr * M; i += blockDim.x) {
            const int r = i / M, c = i % M;
            xs[r * XS + c] = xg[i];
            gs[r * XS + c] = make_float2(0.f, 0.f);
        }
        __syncthreads();
        for (int q = warp; q < np; q += kAdjWarps) {
            const long long pix = (long long)bx * a.Npy + p0 + q;
            const float g = a.gP[pix];
            if (g == 0.f) continue;  // warp-uniform
            for (int l = lane; l < LT; l += 32) ws[l] = a.w[(size_t)pix * LT + l];
            __syncwarp();
            float2 wr[LT];
            float wn = 0.f;
#pragma unroll
            for (int l = 0; l < LT; ++l) {
                wr[l] = ws[l];
                wn += cabs2(wr[l]);
            }
            if (lane == 0) dacc += g * wn;
            // e_ts = w^H x_ts
            for (int it = lane; it < T * nsb; it += 32) {
                const int t = it / nsb, s0 = (it % nsb) * SB;
                const float2 *xt = xs + (size_t)(q + t) * XS;
                float2 acc[SB];
#pragma unroll
                for (int j = 0; j < SB; ++j) acc[j] = make_float2(0.f, 0.f);
#pragma unroll
                for (int i = 0; i < SB + LT - 1; ++i) {
                    const float2 v = xt[min(s0 + i, M - 1)];  // past the row only for s >= Ns (not stored)
#pragma unroll
                    for (int j = 0; j < SB; ++j) {
                        const int l = i - j;
                        if (l >= 0 && l < LT) acc[j] = cmac4_conj(acc[j], wr[l], v);
                    }
                }
#pragma unroll
                for (int j = 0; j < SB; ++j)
                    if (s0 + j < Ns) es[t * Ns + s0 + j] = acc[j];
            }
            __syncwarp();
            // dP/dconj(x_t[c]) = scale g sum_s e_ts w_{c-s} into the shared accumulator
            const float gsc = g * scale;
            for (int it = lane; it < T * ncb; it += 32) {
                const int t = it / ncb, c0 = (it % ncb) * CB;
                const float2 *et = es + t * Ns;
                float2 G[CB];
#pragma unroll
                for (int b = 0; b < CB; ++b) G[b] = make_float2(0.f, 0.f);
#pragma unroll
                for (int i = 0; i < LT + CB - 1; ++i) {
                    const int sidx = c0 - (LT - 1) + i;
                    const bool in = sidx >= 0 && sidx < Ns;
                    const float2 ev = et[min(max(sidx, 0), Ns - 1)];
                    const float2 e = make_float2(in ? ev.x : 0.f, in ? ev.y : 0.f);
#pragma unroll
                    for (int b = 0; b < CB; ++b) {
                        const int l = b + LT - 1 - i;
                        if (l >= 0 && l < LT) G[b] = cmac4(G[b], e, wr[l]);
                    }
                }
                float2 *dst = gs + (size_t)(q + t) * XS + c0;
#pragma unroll
                for (int b = 0; b < CB; ++b) {
                    if (c0 + b < M) {
                        atomicAdd(&dst[b].x, G[b].x * gsc);
                        atomicAdd(&dst[b].y, G[b].y * gsc);
                    }
                }
            }
            __syncwarp();
        }
        __syncthreads();
        // write the tile's gradient rows; the channel-phase sums use them
        float2 *gout = a.gx + ((size_t)bx * a.Ny + p0) * M;
        for (int i = tid; i < nr * M; i += blockDim.x) {
            const int r = i / M, c = i % M;
            const float2 G = gs[r * XS + c];
            if (G.x == 0.f && G.y == 0.f) continue;
            const float2 xv = xs[r * XS + c];
            atomicAdd(&ths[c], 2.f * (G.x * xv.y - G.y * xv.x));
            if (r < 2 * K || r >= np) {
                atomicAdd(&gout[i].x, G.x);
                atomicAdd(&gout[i].y, G.y);
            } else {
                const float2 o = gout[i];
                gout[i] = make_float2(o.x + G.x, o.y + G.y);
            }
        }
        __syncthreads();
    }
    if (a.gth)
        for (int i = tid; i < M; i += blockDim.x)
            if (ths[i] != 0.f) atomicAdd(&a.gth[i], ths[i]);
    if (a.gd && lane == 0 && dacc != 0.f) atomicAdd(a.gd, dacc);
}

template <class Kern>
static int launch_adjoint_with(Kern kern, const AdjDev &a, size_t smem, int num_sms, cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kAdjWarps, smem);
    if (e != cudaSuccess) return e;
    const long long units = (long long)a.Nx * ((a.Npy + kAdjTile - 1) / kAdjTile);
    long long grid = (long long)num_sms * (per_sm > 0 ? per_sm : 1);
    if (grid > units) grid = units;
    kern<<<(unsigned)grid, 32 * kAdjWarps, smem, s>>>(a);
    return cudaGetLastError();
}

int launch_adjoint(const AdjDev &a, int num_sms, cudaStream_t s)
{
    const int T = 2 * a.K + 1, Ns = a.M - a.L + 1, rows = kAdjTile + 2 * a.K;
    const size_t smem = (size_t)2 * rows * a.M * sizeof(float2) + (size_t)((a.M + 1) & ~1) * sizeof(float) +
                        (size_t)kAdjWarps * (a.L + T * Ns) * sizeof(float2);
    if (smem > 227 * 1024 || a.L > 64) return cudaErrorNotSupported;
    const size_t smem_b = smem + (size_t)2 * rows * kAdjPad * sizeof(float2);  // padded rows
    if (smem_b <= 227 * 1024) {
        switch (a.L) {
        case 8: return launch_adjoint_with(adjoint_blocked_kernel<8>, a, smem_b, num_sms, s);
        case 16: return launch_adjoint_with(adjoint_blocked_kernel<16>, a, smem_b, num_sms, s);
        case 32: return launch_adjoint_with(adjoint_blocked_kernel<32>, a, smem_b, num_sms, s);
        default: break;
        }
    }
    return launch_adjoint_with(adjoint_kernel, a, smem, num_sms, s);
}

}  // namespace cgb
