// Precise element-space pipeline for sm_103a: the path for subarray lengths
// without a fused instantiation (L = 48, 64, ...) and for the refinement option.
//
//   1. covariance per pixel in float-float: along each diagonal d,
//        R[k,k+d] = R0[d] + S[k,k+d],  S[k,k+d] = S[k-1,k-1+d] + D[k,k+d],
//        D[k,j]   = sum_t x_t[k-1+Ns] conj(x_t[j-1+Ns]) - x_t[k-1] conj(x_t[j-1])
//      (the diagonal recurrence of the reference buildR_kernel.cu:96-131, run on
//      telescoped increments), with R0 and S accumulated by TwoSum, written as
//      R_hi + R_lo (column-major per pixel, not normalised) plus the loading
//      dl = d tr(R)/L (getCaponC.pyx:257-262);
//   2. FP32 Cholesky of R_hi + dl I in shared memory, U^H y = a, U x0 = y
//      (matrixDecompc.pyx:19-50, linearSolvec.pyx:312-346); with refinement,
//      r = a - (R_hi + R_lo + dl I) x0 is formed in FP64 and x1 = x0 + R^-1 r is
//      solved with the same FP32 factor;
//   3. weights and outputs: the plain output stage (capon_plain.cu).
#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {

static constexpr int kPrecWarps = 4;

// (h, l) += x*y exactly up to the rounding of l: the product's error term comes
// from an fma (TwoProd), the sum's from TwoSum
COS_DEV void ff_add_prod(float &h, float &l, float x, float y)
{
    const float p = x * y;
    const float pe = fmaf(x, y, -p);
    const float s = h + p;
    const float bb = s - h;
    l += ((h - (s - bb)) + (p - bb)) + pe;
    h = s;
}
// (h, l) += sign * a * conj(b), complex, every product exact
COS_DEV void ff_add_cmulc(float2 &h, float2 &l, float2 a, float2 b, float sign)
{
    const float ax = sign * a.x, ay = sign * a.y;
    ff_add_prod(h.x, l.x, ax, b.x);
    ff_add_prod(h.x, l.x, ay, b.y);
    ff_add_prod(h.y, l.y, ay, b.x);
    ff_add_prod(h.y, l.y, -ax, b.y);
}

// EXACT: every product enters the float-float sums exactly (the FP64 residual of
// the refinement is only as good as this matrix); otherwise products are summed
// in FP32 chunks and only the chunk sums are compensated.
template <bool EXACT>
__global__ void __launch_bounds__(32 * kPrecWarps)
precise_build_r_kernel(FrameDev f, float2 *__restrict__ Rhi, float2 *__restrict__ Rlo, float *__restrict__ dlo)
{
    extern __shared__ float2 smem[];
    const int M = f.M, L = f.L, K = f.K, T = 2 * K + 1, Ns = M - L + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long npix = (long long)f.Nx * f.Npy;
    const long long pix = (long long)blockIdx.x * kPrecWarps + warp;
    if (pix >= npix) return;
    const int bx = (int)(pix / f.Npy), p = (int)(pix % f.Npy);
    float2 *xs = smem + (size_t)warp * T * M;
    const float2 *xg = f.x + ((size_t)bx * f.Ny + p) * M;
    for (int i = lane; i < T * M; i += 32) xs[i] = xg[i];
    __syncwarp();

    float2 *Rh = Rhi + (size_t)pix * L * L, *Rl = Rlo + (size_t)pix * L * L;
    float trh = 0.f, trl = 0.f;
    for (int d = lane; d < L; d += 32) {
        // R0[d]: T*Ns products, chunks of 4 summed in FP32, chunk sums by TwoSum
        float2 rh = make_float2(0.f, 0.f), rl = make_float2(0.f, 0.f);
        for (int t = 0; t < T; ++t) {
            const float2 *xt = xs + t * M;
            if (EXACT) {
                for (int s = 0; s < Ns; ++s) ff_add_cmulc(rh, rl, xt[s], xt[s + d], 1.f);
            } else {
                for (int s0 = 0; s0 < Ns; s0 += 4) {
                    float2 acc = make_float2(0.f, 0.f);
                    const int s1 = min(Ns, s0 + 4);
                    for (int s = s0; s < s1; ++s) acc = cadd(acc, cmulc(xt[s], xt[s + d]));
                    two_sum_acc(rh, rl, acc);
                }
            }
        }
        float2 sh = make_float2(0.f, 0.f), sl = make_float2(0.f, 0.f);
        for (int k = 0; k + d < L; ++k) {
            if (k > 0) {
                if (EXACT) {
                    for (int t = 0; t < T; ++t) {
                        const float2 *xt = xs + t * M;
                        ff_add_cmulc(sh, sl, xt[k - 1 + Ns], xt[k - 1 + d + Ns], 1.f);
                        ff_add_cmulc(sh, sl, xt[k - 1], xt[k - 1 + d], -1.f);
                    }
                } else {
                    float2 dv = make_float2(0.f, 0.f);
                    for (int t = 0; t < T; ++t) {
                        const float2 *xt = xs + t * M;
                        dv = cadd(dv, csub(cmulc(xt[k - 1 + Ns], xt[k - 1 + d + Ns]), cmulc(xt[k - 1], xt[k - 1 + d])));
                    }
                    two_sum_acc(sh, sl, dv);
                }
            }
            // R[k, k+d] = (rh, rl) + (sh, sl)
            float2 h = rh, l = fadd2(rl, sl);
            two_sum_acc(h, l, sh);
            const float2 vh = fadd2(h, l);
            const float2 vl = fsub2(l, fsub2(vh, h));
            const int a = k, b = k + d;   // column-major: element (a, b) at a + b*L
            Rh[a + (size_t)b * L] = vh;
            Rl[a + (size_t)b * L] = vl;
            if (d) {
                Rh[b + (size_t)a * L] = cconj(vh);
                Rl[b + (size_t)a * L] = cconj(vl);
            } else {
                float t2 = trh + vh.x;
                trl += (trh - (t2 - (t2 - trh))) + (vh.x - (t2 - trh)) + vl.x;
                trh = t2;
            }
        }
    }
    const float tr = __shfl_sync(0xffffffffu, trh + trl, 0);
    if (lane == 0) dlo[pix] = f.loading == COS_CAPON_LOAD_ABSOLUTE ? f.d * (float)(Ns * T) : f.d * tr / (float)L;
}

// One warp per pixel: FP32 Cholesky of R_hi + dl I in shared memory, x0 =
// R^-1 a; with REFINE one FP64-residual correction step.
//
// The upper triangle is stored packed by rows (row k at k*L - k(k-1)/2, L(L+1)/2
// entries: 16.6 KB at L = 64, so several warps share an SM).  Step i of the
// right-looking factorisation updates the pairs (k, j), i < k <= j < L; a
// CTA-wide table lists all pairs by decreasing k, so the trailing set of step i
// is the table's prefix of length n(n+1)/2, n = L-1-i, and the 32 lanes take
// equal, independent shares of it.
COS_DEV int prow(int k, int L) { return k * L - (k * (k - 1)) / 2; }

template <bool REFINE>
__global__ void __launch_bounds__(32 * kPrecWarps)
precise_solve_kernel(int L, long long batch, const float2 *__restrict__ Rhi, const float2 *__restrict__ Rlo,
                     const float *__restrict__ dlv, float2 *__restrict__ xout, unsigned *status)
{
    extern __shared__ float2 smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NP = L * (L + 1) / 2;
    uint16_t *pairs = (uint16_t *)(smem + (size_t)kPrecWarps * (NP + L));   // (k << 8) | j
    // the pair table, shared by the CTA's warps
    for (int e = threadIdx.x; e < NP; e += blockDim.x) {
        // e-th pair by decreasing k: row k = L - n holds n pairs, at
        // e in [n(n-1)/2, n(n+1)/2)
        int n = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
        while (n * (n + 1) / 2 <= e) ++n;
        while (n > 1 && (n - 1) * n / 2 > e) --n;
        const int k = L - n, j = k + (e - (n - 1) * n / 2);
        pairs[e] = (uint16_t)((k << 8) | j);
    }
    __syncthreads();
    const long long sys = (long long)blockIdx.x * kPrecWarps + warp;
    if (sys >= batch) return;
    float2 *A = smem + (size_t)warp * (NP + L);
    float2 *xb = A + NP;   // x0 broadcast buffer
    const float2 *Rh = Rhi + (size_t)sys * L * L, *Rl = Rlo ? Rlo + (size_t)sys * L * L : nullptr;
    const float dl = dlv[sys];
    for (int i = lane; i < L * L; i += 32) {
        const int a = i % L, b = i / L;   // column-major source element (a, b)
        if (a <= b) {
            float2 v = Rh[i];
            if (a == b) v = make_float2(v.x + dl, 0.f);
            A[prow(a, L) + (b - a)] = v;
        }
    }
    __syncwarp();
    bool bad = false;
    for (int i = 0; i < L; ++i) {
        float2 *Ai = A + prow(i, L);   // row i: Ai[j - i]
        const float dv = Ai[0].x;
        bad |= !(dv > 0.f);
        const float inv = rsqrtf(dv);
        __syncwarp();
        for (int j = i + 1 + lane; j < L; j += 32) Ai[j - i] = cscale(Ai[j - i], inv);
        if (lane == 0) Ai[0] = make_float2(dv * inv, 0.f);
        __syncwarp();
        const int n = L - 1 - i, cnt = n * (n + 1) / 2;
        for (int e = lane; e < cnt; e += 32) {
            const int kj = pairs[e], k = kj >> 8, j = kj & 255;
            float2 &dst = A[prow(k, L) + (j - k)];
            dst = csub(dst, cconjmul(Ai[k - i], Ai[j - i]));
        }
        __syncwarp();
    }
    auto U = [&](int r, int c) { return A[prow(r, L) + (c - r)]; };   // r <= c
    // solve U^H U x = b for the lane-distributed right-hand side v (rows lane, lane+32)
    auto solve = [&](float2 &v0, float2 &v1) {
        for (int i = 0; i < L; ++i) {
            const float2 vi = shfl2(i < 32 ? v0 : v1, i & 31, 32);
            const float2 yi = cscale(vi, 1.0f / U(i, i).x);
            if (lane > i && lane < L) v0 = csub(v0, cconjmul(U(i, lane), yi));
            if (lane + 32 > i && lane + 32 < L) v1 = csub(v1, cconjmul(U(i, lane + 32), yi));
            if (lane == i) v0 = yi;
            if (lane + 32 == i) v1 = yi;
        }
        for (int i = L - 1; i >= 0; --i) {
            const float2 vi = shfl2(i < 32 ? v0 : v1, i & 31, 32);
            const float2 xi = cscale(vi, 1.0f / U(i, i).x);
            if (lane < i) v0 = csub(v0, cmul(U(lane, i), xi));
            if (lane + 32 < i) v1 = csub(v1, cmul(U(lane + 32, i), xi));
            if (lane == i) v0 = xi;
            if (lane + 32 == i) v1 = xi;
        }
    };
    float2 x0 = make_float2(1.f, 0.f), x1 = make_float2(1.f, 0.f);
    solve(x0, x1);
    if (REFINE) {
        if (lane < L) xb[lane] = x0;
        if (lane + 32 < L) xb[lane + 32] = x1;
        __syncwarp();
        // r_i = 1 - sum_j (R_hi + R_lo + dl I)_ij x0_j in FP64, rows lane, lane+32
        float2 r[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int i = lane + 32 * q;
            double rr = 1.0, ri = 0.0;
            if (i < L) {
                for (int j = 0; j < L; ++j) {
                    const float2 h = Rh[i + (size_t)j * L], xj = xb[j];
                    const float2 l = Rlo ? Rl[i + (size_t)j * L] : make_float2(0.f, 0.f);
                    const double ar = (double)h.x + (double)l.x + (i == j ? (double)dl : 0.0);
                    const double ai = (double)h.y + (double)l.y;
                    rr -= ar * (double)xj.x - ai * (double)xj.y;
                    ri -= ar * (double)xj.y + ai * (double)xj.x;
                }
            }
            r[q] = make_float2((float)rr, (float)ri);
        }
        solve(r[0], r[1]);
        x0 = cadd(x0, r[0]);
        x1 = cadd(x1, r[1]);
    }
    if (lane < L) xout[(size_t)sys * L + lane] = x0;
    if (lane + 32 < L) xout[(size_t)sys * L + lane + 32] = x1;
    if (bad && lane == 0) atomicOr(status, ERR_NOT_PD);
}

// R of the pipeline (R_hi + R_lo, column-major, not normalised) plus the
// loading, in the caller's layout: the reference's (column-major, loaded, not
// normalised) or row-major, loaded and normalised by 1/(Ns T)
__global__ void format_r_kernel(long long n, int L, float scale, int ref_layout, const float2 *__restrict__ Rhi,
                                const float2 *__restrict__ Rlo, const float *__restrict__ dlv, float2 *__restrict__ out)
{
    const long long L2 = (long long)L * L;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n * L2;
         i += (long long)gridDim.x * blockDim.x) {
        const long long pix = i / L2;
        const int e = (int)(i % L2), a = e % L, b = e / L;   // source element (a, b), column-major
        float2 v = Rhi[i];
        if (Rlo) v = fadd2(v, Rlo[i]);
        if (a == b) v.x += dlv[pix];
        v = cscale(v, scale);
        out[pix * L2 + (ref_layout ? e : a * L + b)] = v;
    }
}

int launch_format_r(const FrameDev &f, const float2 *Rhi, const float2 *Rlo, const float *dl, float2 *out,
                    cudaStream_t s)
{
    const long long npix = (long long)f.Nx * f.Npy;
    const int ref = f.r_layout == COS_CAPON_R_REFERENCE;
    const float scale = ref ? 1.f : 1.f / ((float)(f.M - f.L + 1) * (float)(2 * f.K + 1));
    long long blocks = (npix * f.L * f.L + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    format_r_kernel<<<(unsigned)blocks, 256, 0, s>>>(npix, f.L, scale, ref, Rhi, Rlo, dl, out);
    return cudaGetLastError();
}

// Forward-backward averaging in place: (R + J R^T J)/2 maps element (a, b) to
// the mean of R[a,b] and conj(R[L-1-a, L-1-b]), i.e. flat index i and its
// mirror L^2-1-i in either storage order; one thread per mirror pair, the
// pair's two new values being conjugates.  With Rlo the pair is averaged in
// float-float (TwoSum, exact halving) and renormalised to hi + lo.
__global__ void fb_average_kernel(long long npix, int L, float2 *__restrict__ Rhi, float2 *__restrict__ Rlo)
{
    const long long L2 = (long long)L * L, half = (L2 + 1) / 2;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < npix * half;
         t += (long long)gridDim.x * blockDim.x) {
        const long long pix = t / half, i = t % half, j = L2 - 1 - i;
        float2 *h = Rhi + pix * L2;
        float2 *l = Rlo ? Rlo + pix * L2 : nullptr;
        const float2 a = h[i], b = cconj(h[j]);
        float2 s = fadd2(a, b);
        const float2 bb = fsub2(s, a);
        float2 e = fadd2(fsub2(a, fsub2(s, bb)), fsub2(b, bb));
        if (l) e = fadd2(e, fadd2(l[i], cconj(l[j])));
        s = cscale(s, 0.5f);
        e = cscale(e, 0.5f);
        const float2 v = fadd2(s, e);
        const float2 vl = fsub2(e, fsub2(v, s));
        if (i == j) {
            h[i] = make_float2(v.x, 0.f);
            if (l) l[i] = make_float2(vl.x, 0.f);
        } else {
            h[i] = v;
            h[j] = cconj(v);
            if (l) {
                l[i] = vl;
                l[j] = cconj(vl);
            }
        }
    }
}

int launch_fb_average(const FrameDev &f, float2 *Rhi, float2 *Rlo, cudaStream_t s)
{
    const long long npix = (long long)f.Nx * f.Npy;
    const long long n = npix * (((long long)f.L * f.L + 1) / 2);
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    fb_average_kernel<<<(unsigned)blocks, 256, 0, s>>>(npix, f.L, Rhi, Rlo);
    return cudaGetLastError();
}

int launch_precise_solve(const FrameDev &f, const float2 *Rhi, const float2 *Rlo, const float *dl, float2 *Ria,
                         unsigned *status, bool refine, cudaStream_t s)
{
    const long long npix = (long long)f.Nx * f.Npy;
    const size_t sm2 = (size_t)kPrecWarps * (f.L * (f.L + 1) / 2 + f.L) * sizeof(float2) +
                       (size_t)f.L * (f.L + 1) / 2 * sizeof(uint16_t);
    if (sm2 > 227 * 1024 || f.L > 64) return cudaErrorNotSupported;
    const long long blocks = (npix + kPrecWarps - 1) / kPrecWarps;
    cudaError_t e;
    if (refine) {
        e = cudaFuncSetAttribute(precise_solve_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
        if (e != cudaSuccess) return e;
        precise_solve_kernel<true><<<(unsigned)blocks, 32 * kPrecWarps, sm2, s>>>(f.L, npix, Rhi, Rlo, dl, Ria, status);
    } else {
        e = cudaFuncSetAttribute(precise_solve_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
        if (e != cudaSuccess) return e;
        precise_solve_kernel<false><<<(unsigned)blocks, 32 * kPrecWarps, sm2, s>>>(f.L, npix, Rhi, Rlo, dl, Ria, status);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return launch_plain_output(f, Ria, s);
}

int launch_precise(const FrameDev &f, float2 *Rhi, float2 *Rlo, float *dl, float2 *Ria, unsigned *status,
                   bool refine, cudaStream_t s)
{
    const long long npix = (long long)f.Nx * f.Npy;
    const size_t sm1 = (size_t)kPrecWarps * (2 * f.K + 1) * f.M * sizeof(float2);
    if (sm1 > 227 * 1024 || f.L > 64) return cudaErrorNotSupported;
    cudaError_t e;
    const long long blocks = (npix + kPrecWarps - 1) / kPrecWarps;
    // exact products always: this pipeline serves the stress cases (L = 48, 64,
    // light loading) and the refinement option, where the covariance's own
    // rounding is what limits the power accuracy
    e = cudaFuncSetAttribute(precise_build_r_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
    if (e != cudaSuccess) return e;
    precise_build_r_kernel<true><<<(unsigned)blocks, 32 * kPrecWarps, sm1, s>>>(f, Rhi, Rlo, dl);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (f.fb && (e = (cudaError_t)launch_fb_average(f, Rhi, Rlo, s)) != cudaSuccess) return e;
    return launch_precise_solve(f, Rhi, Rlo, dl, Ria, status, refine, s);
}

}  // namespace cgb
