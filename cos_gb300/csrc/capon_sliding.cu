// Sliding-window inverse form (COS_CAPON_FORM_SLIDING_INVERSE) for sm_103a.
//
// Instead of a covariance and a factorisation per pixel, R_d^-1 is carried
// along range by rank-1 changes (Sherman-Morrison): the SOLVE_WOOD branch of
// framework/beamformer/capon/getCaponAllC.pyx:240-252 with the update of
// framework/linalg/woodburyc.pyx:73-100,
//     A <- A + s x x^H,   B = A^-1 <- B - s (B x)(B x)^H / (1 + s x^H B x),
// one change per subarray x of a range row (woodburyc.pyx:15-42).  With
// absolute loading on the normalised covariance, R_d = sum x x^H / (Ns T) + d I,
// the unnormalised matrix is A = sum x x^H + Ns T d I and R_d^-1 = Ns T A^-1;
// a build-up from
// B = I / (Ns T d) over the 2K+1 rows of a window (woodburyc.pyx:46-70) starts
// every segment of `segment` pixels, and between two pixels row p+2K enters
// and row p-1 leaves.  Relative loading d tr(R)/L changes the whole diagonal
// from one pixel to the next, which no low-rank change expresses, so the form
// takes absolute loading only.
//
// Layout: a group of LP lanes (LP = 16 or 32, L <= LP) owns one (beam,
// segment) unit; lane i holds row i of B in registers (rows and columns
// L..LP-1 stay exactly zero).  The rows of the window sit in a shared-memory
// ring of 2K+2 slots, each complex stored twice as {re, re, im, im} so that a
// broadcast 16-byte load feeds two packed FMAs (B x) without a shuffle, and
// B x is passed between lanes through the same layout.
#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {

static constexpr int kSlideThreads = 128;
static constexpr int kSlideDefaultSegment = 8;

template <int LP>
struct SlideGroup {
    float4 *ring;    // (T+1) slots x stride float4
    float4 *ub;      // LP float4: B x of the current change
    int stride;      // M + LP: a row and a zero tail of LP entries
    unsigned mask;   // the group's lanes
};

// B <- B - s (Bv)(Bv)^H / (1 + s v^H B v) for the subarray v = row[0..L-1]
// (row points into a ring slot at the subarray's first element).
template <int LP>
__device__ __forceinline__ void sm_change(float2 (&b)[LP], const SlideGroup<LP> &g, const float4 *row, int i,
                                          float sign, bool &bad)
{
    float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < LP; ++j) {
        const float4 v = row[j];
        a0 = ffma2(b[j], make_float2(v.x, v.y), a0);   // (B.re v.re, B.im v.re)
        a1 = ffma2(b[j], make_float2(v.z, v.w), a1);   // (B.re v.im, B.im v.im)
    }
    const float2 u = make_float2(a0.x - a1.y, a0.y + a1.x);   // (B v)_i
    const float4 vi = row[i];
    float r = vi.x * u.x + vi.z * u.y;                           // Re(conj(v_i) u_i)
#pragma unroll
    for (int o = LP / 2; o; o >>= 1) r += __shfl_xor_sync(g.mask, r, o, LP);
    const float beta = 1.f + sign * r;
    bad |= !(beta > 0.f);
    const float c = sign / beta;
    __syncwarp(g.mask);                    // the previous change's readers of ub are done
    g.ub[i] = make_float4(u.x, u.x, u.y, u.y);
    __syncwarp(g.mask);
    // B_ij -= c u_i conj(u_j)
    const float2 n1 = make_float2(-c * u.x, -c * u.y), n2 = make_float2(-c * u.y, c * u.x);
#pragma unroll
    for (int j = 0; j < LP; ++j) {
        const float4 w = g.ub[j];
        b[j] = ffma2(n1, make_float2(w.x, w.y), b[j]);
        b[j] = ffma2(n2, make_float2(w.z, w.w), b[j]);
    }
}

template <int LP>
__global__ void __launch_bounds__(kSlideThreads)
sliding_inverse_kernel(FrameDev f, int segment, long long units, unsigned *status)
{
    extern __shared__ float4 slide_smem[];
    constexpr int kGroups = kSlideThreads / LP;
    const int lane = threadIdx.x & 31;
    const int gi = threadIdx.x / LP, i = threadIdx.x & (LP - 1);
    const int M = f.M, L = f.L, T = 2 * f.K + 1, Ns = M - L + 1;
    SlideGroup<LP> g;
    g.stride = M + LP;
    g.ring = slide_smem + (size_t)gi * ((size_t)(T + 1) * g.stride + LP);
    g.ub = g.ring + (size_t)(T + 1) * g.stride;
    g.mask = LP == 32 ? 0xffffffffu : (0xffffu << (lane & 16));
    const float nt = (float)Ns * (float)T;
    const float binit = 1.f / (nt * f.d);
    const int segs = (f.Npy + segment - 1) / segment;
    // zero tails: subarray offsets and the rows i >= L read up to M-L+LP-1
    for (int k = i; k < (T + 1) * LP; k += LP) g.ring[(k / LP) * g.stride + M + (k % LP)] = make_float4(0.f, 0.f, 0.f, 0.f);
    bool bad = false;

    for (long long unit = (long long)blockIdx.x * kGroups + gi; unit < units; unit += (long long)gridDim.x * kGroups) {
        const int bx = (int)(unit / segs), p0 = (int)(unit % segs) * segment;
        const int p1 = min(p0 + segment, f.Npy);
        const float2 *xb = f.x + (size_t)bx * f.Ny * M;
        auto stage = [&](int t) {
            float4 *dst = g.ring + (t % (T + 1)) * g.stride;
            const float2 *src = xb + (size_t)t * M;
            __syncwarp(g.mask);            // earlier readers of this slot are done
            for (int m = i; m < M; m += LP) {
                const float2 v = __ldg(src + m);
                dst[m] = make_float4(v.x, v.x, v.y, v.y);
            }
            __syncwarp(g.mask);
        };
        float2 b[LP];
#pragma unroll
        for (int j = 0; j < LP; ++j) b[j] = make_float2((j == i && i < L) ? binit : 0.f, 0.f);
        // build-up of the window of pixel p0: rows p0 .. p0+2K
        for (int t = p0; t < p0 + T; ++t) {
            stage(t);
            const float4 *r = g.ring + (t % (T + 1)) * g.stride;
            for (int s = 0; s < Ns; ++s) sm_change<LP>(b, g, r + s, i, 1.f, bad);
        }
        for (int p = p0; p < p1; ++p) {
            if (p > p0) {
                const int tin = p + T - 1, tout = p - 1;
                stage(tin);
                const float4 *r = g.ring + (tin % (T + 1)) * g.stride;
                for (int s = 0; s < Ns; ++s) sm_change<LP>(b, g, r + s, i, 1.f, bad);
                r = g.ring + (tout % (T + 1)) * g.stride;
                for (int s = 0; s < Ns; ++s) sm_change<LP>(b, g, r + s, i, -1.f, bad);
            }
            // R_d^-1 a = Ns T B 1, its sum, w, and the amplitude with the
            // subarray sums of the centre row (getCaponC.pyx:246-283)
            float2 rs = make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < LP; ++j) rs = fadd2(rs, b[j]);
            const float2 ria = cscale(rs, nt);
            float2 ar = ria;
#pragma unroll
            for (int o = LP / 2; o; o >>= 1) {
                ar.x += __shfl_xor_sync(g.mask, ar.x, o, LP);
                ar.y += __shfl_xor_sync(g.mask, ar.y, o, LP);
            }
            const float inv = 1.f / (ar.x * ar.x + ar.y * ar.y);
            const float2 wi = cscale(cmulc(ria, ar), inv);
            const float4 *xc = g.ring + ((p + f.K) % (T + 1)) * g.stride;
            float2 gs = make_float2(0.f, 0.f);
            for (int s = 0; s < Ns; ++s) {
                const float4 v = xc[i + s];
                gs.x += v.x;
                gs.y += v.z;
            }
            float2 zz = cconjmul(wi, cscale(gs, 1.f / (float)Ns));
#pragma unroll
            for (int o = LP / 2; o; o >>= 1) {
                zz.x += __shfl_xor_sync(g.mask, zz.x, o, LP);
                zz.y += __shfl_xor_sync(g.mask, zz.y, o, LP);
            }
            const size_t pix = (size_t)bx * f.Npy + p;
            if (i == 0) {
                f.z[pix] = zz;
                if (f.P) f.P[pix] = 1.f / ar.x;
            }
            if (f.w && i < L) f.w[pix * L + i] = wi;
        }
    }
    if (bad) atomicOr(status, ERR_NOT_PD);
}

int launch_sliding_inverse(const FrameDev &f, unsigned *status, cudaStream_t s)
{
    if (f.Nb != 0 || f.fb || f.R || f.refine || f.loading != COS_CAPON_LOAD_ABSOLUTE || f.L > 32)
        return COS_CAPON_ERR_NOT_SUPPORTED;
    if (!(f.d > 0.f) || f.tile < 0) return COS_CAPON_ERR_LAUNCH;
    const int segment = f.tile > 0 ? f.tile : kSlideDefaultSegment;
    const int LP = f.L <= 16 ? 16 : 32;
    const int T = 2 * f.K + 1;
    const size_t groups = kSlideThreads / LP;
    const size_t smem = groups * ((size_t)(T + 1) * (f.M + LP) + LP) * sizeof(float4);
    if (smem > 227 * 1024) return COS_CAPON_ERR_NOT_SUPPORTED;
    const long long units = (long long)f.Nx * ((f.Npy + segment - 1) / segment);
    const long long blocks = (units + (long long)groups - 1) / (long long)groups;
    const unsigned grid = (unsigned)(blocks < 0x7fffffffLL ? blocks : 0x7fffffffLL);
    cudaError_t e;
    if (LP == 16) {
        if ((e = cudaFuncSetAttribute(sliding_inverse_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem)) != cudaSuccess)
            return e;
        sliding_inverse_kernel<16><<<grid, kSlideThreads, smem, s>>>(f, segment, units, status);
    } else {
        if ((e = cudaFuncSetAttribute(sliding_inverse_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem)) != cudaSuccess)
            return e;
        sliding_inverse_kernel<32><<<grid, kSlideThreads, smem, s>>>(f, segment, units, status);
    }
    return cudaGetLastError();
}

}  // namespace cgb
