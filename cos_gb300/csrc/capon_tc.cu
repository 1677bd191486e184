// Tensor-core covariance forms for sm_103a: tcgen05.mma with TMEM accumulators.
//
// The per-pixel covariance R[a,b] = sum_{t,s} x_t[s+a] conj(x_t[s+b])
// (getCaponC.pyx:207-242: full-array band products, then the subarray sum)
// is split into
//   1. the window Gram  G[m,n] = sum_{t<T} x_t[m] conj(x_t[n])   (M x M, rank T)
//      as a real GEMM on the tensor cores, and
//   2. the spatial smoothing R[a,b] = sum_{s<Ns} G[s+a, s+b] on the CUDA cores,
//      one sliding float-float sum per diagonal b-a.
//
// Step 1 packs 128/M pixels into the 128 accumulator lanes of one
// tcgen05.mma (M=128, cta_group::1).  With rows (p, m) (pixel p, channel m) and
// the K index (p', t, c) (pixel, window row, real/imaginary part):
//   A[(p,m), (p',t,c)] = [p == p'] * {Re, Im} x_{p,t}[m]
//   B[(p',t,c), n]     = {Re, Im} x_{p',t}[n]            columns n < M
//   B[(p',t,c), M+n]   = {-Im, Re} x_{p',t}[n]           columns M <= M+n < 2M
// so that D[(p,m), n] = Re G_p[m,n] and D[(p,m), M+n] = Im G_p[m,n]; the
// block-diagonal A keeps the pixels apart inside one MMA.  Operands are staged
// in shared memory in the no-swizzle K-major core-matrix layout (8 rows x 16
// bytes per core matrix; LBO = next core matrix along K, SBO = next 8-row
// group), one elected thread issues the MMAs, tcgen05.commit arrives on an
// mbarrier, and the accumulators come back with tcgen05.ld.
//
// Operand precisions (the rank-T product is the only reduced-precision step;
// the smoothing, Cholesky and outputs are FP32, the refinement residual FP64):
//   TF32    A_hi B_hi                      (kind::tf32, inputs rounded rna)
//   TF32x3  A_hi B_lo + A_lo B_hi + A_hi B_hi, hi/lo a TF32 split
//   BF16x3  the same three products with a BF16 split (kind::f16, BF16 inputs)
// all accumulated in FP32 in TMEM.
#include <cuda_bf16.h>

#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {
namespace tc {

static constexpr int kThreads = 256;   // eight warps, two per 32-lane TMEM quadrant
static constexpr int kMaxTracePartials = 256;  // P * nseg <= kThreads
static constexpr int kTmemCols = 256;  // half the SM's TMEM: two CTAs share an SM
// shared-memory floor so that no third CTA lands on an SM (it would wait in
// tcgen05.alloc for a CTA to finish), and the ceiling under which two fit
static constexpr int kMinSmem = 77 * 1024;
static constexpr int kTwoCtaSmem = 113 * 1024;

struct Geom {
    int P;          // pixels per slot (128 / M)
    int N;          // MMA N: 2M rounded up to 16
    int Ktot;       // K extent of one slot, a multiple of the MMA K
    int S;          // slots per pass (TMEM holds S accumulators of N columns)
    int E;          // elements per 16-byte core-matrix row: 4 (tf32) or 8 (bf16)
    int esize;      // bytes per element
    int kstep;      // K of one MMA: 8 (tf32) or 16 (bf16)
    int copies;     // 1 (hi) or 2 (hi, lo)
    int aBytes;     // one copy of A of one slot
    int bBytes;     // one copy of B of one slot
    int slotBytes;  // all copies of A and B of one slot
    int opBytes;    // S slots (the band and the staged R reuse this area after the MMAs)
    int xsOff;      // staged windows: S*P pixels x T rows x M samples
    int bandOff;    // offset of the band (inside the operand area)
    int rstOff;     // offset of the staged R (inside the operand area)
    int bs;         // band row stride in floats (even, L+2)
    int nseg;       // segments per diagonal in the smoothing (P*L*nseg <= threads)
    int smem;
    uint32_t idesc;
};

struct Params {
    FrameDev f;
    Geom g;
    int split;        // COS_CAPON_FORM_TC_*
    float2 *Rw;       // [npix][L][L] column-major, not normalised, not loaded
    float *dl;        // [npix] loading in the same (unnormalised) units
    unsigned *status;
};

COS_DEV uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- mbarrier ----------------------------------------------------------------
COS_DEV void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
COS_DEV bool mbar_wait_bounded(uint64_t *bar, uint32_t phase)
{
    for (uint32_t it = 0; it < kWaitLimit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(phase)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// ---- tcgen05 -------------------------------------------------------------------
COS_DEV void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
COS_DEV void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
COS_DEV void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
COS_DEV void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: no swizzle, K-major core matrices
COS_DEV uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

template <bool BF16>
COS_DEV void mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    if (BF16)
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
            "l"(a), "l"(b), "r"(idesc), "r"(acc)
            : "memory");
    else
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
            "l"(a), "l"(b), "r"(idesc), "r"(acc)
            : "memory");
}
COS_DEV void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}
// 32 consecutive 32-bit columns of this warp's 32 TMEM lanes
COS_DEV void tmem_ld32(uint32_t taddr, uint32_t (&v)[32])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---- operand splits --------------------------------------------------------------
COS_DEV uint32_t tf32_rna(float v)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return r;
}
COS_DEV uint32_t bf16_bits(float v) { return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v)); }
COS_DEV float bf16_val(uint32_t b) { return __bfloat162float(__ushort_as_bfloat16((unsigned short)b)); }

// split(v) -> (hi, lo) bit patterns of the operand type
template <int SPLIT>
COS_DEV void split(float v, uint32_t &hi, uint32_t &lo)
{
    if (SPLIT == COS_CAPON_FORM_TC_BF16X3) {
        hi = bf16_bits(v);
        lo = bf16_bits(v - bf16_val(hi));
    } else {
        hi = tf32_rna(v);
        lo = (SPLIT == COS_CAPON_FORM_TC_TF32X3) ? tf32_rna(v - __uint_as_float(hi)) : 0u;
    }
}

// byte offset of element (r, k) in a K-major no-swizzle operand
COS_DEV int core_off(int r, int kc, int sbo) { return (r >> 3) * sbo + kc * 128 + (r & 7) * 16; }

// ---- the kernel -------------------------------------------------------------------------
// Eight warps: warps w and w+4 share TMEM lane quadrant w%4 and split its
// columns on readout.
template <int SPLIT>
__global__ void __launch_bounds__(kThreads, 2) tc_cov_kernel(const __grid_constant__ Params prm)
{
    constexpr bool BF16 = SPLIT == COS_CAPON_FORM_TC_BF16X3;
    constexpr int NT = SPLIT == COS_CAPON_FORM_TC_TF32 ? 1 : 3;   // products per slot
    extern __shared__ __align__(1024) unsigned char smem[];
    const FrameDev &f = prm.f;
    const Geom &g = prm.g;
    const int M = f.M, L = f.L, T = 2 * f.K + 1, Ns = M - L + 1, twoT = 2 * T;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    unsigned char *ops = smem;                                       // S slots of operands
    float *bandRe = (float *)(smem + g.bandOff);                     // [128][bs], after the MMAs
    float *bandIm = bandRe + 128 * g.bs;                             // [128][bs]
    float2 *Rst = (float2 *)(smem + g.rstOff);                       // staged R of one slot
    float2 *xs = (float2 *)(smem + g.xsOff);                         // staged pixel windows
    float *trp = (float *)(smem + g.xsOff + (size_t)g.S * g.P * T * M * sizeof(float2));
    uint64_t *bar = (uint64_t *)(trp + kMaxTracePartials);
    uint32_t *tmem_slot = (uint32_t *)(bar + 1);
    int *flag = (int *)(tmem_slot + 1);

    const long long npix = (long long)f.Nx * f.Npy;
    const long long per_pass = (long long)g.S * g.P;
    const long long units = (npix + per_pass - 1) / per_pass;
    const int kchunks = g.Ktot / g.E;
    const int sbo = kchunks * 128;
    const int rows_ab = 128 + g.N;
    // this thread's operand rows (fixed for the kernel): A rows, then B rows
    // diagonal segments of the smoothing: P*L diagonals x nseg pieces
    const int nseg = g.nseg, seglen = (L + nseg - 1) / nseg;

    if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
    if (tid == 0) {
        mbar_init(bar, 1);
        *flag = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    uint32_t phase = 0;

    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        const long long pix0 = u * per_pass;
        // 0. stage the unit's pixel windows (T rows each) in shared memory
        {
            const int npx = g.S * g.P;
            const int per = T * M;
            for (int i = tid; i < npx * per; i += kThreads) {
                const int q = i / per, off = i % per;
                const long long pix = pix0 + q;
                float2 v = make_float2(0.f, 0.f);
                if (pix < npix) {
                    const int bx = (int)(pix / f.Npy), py = (int)(pix % f.Npy);
                    v = f.x[((size_t)bx * f.Ny + py) * M + off];
                }
                xs[i] = v;
            }
        }
        __syncthreads();
        // 1. operands: A and B of every slot, hi (and lo) copies.  For a fixed
        // (slot, K chunk) the (pixel, window row) of each element pair is the
        // same for every operand row, so it is resolved once per chunk.
        for (int sk = 0; sk < g.S * kchunks; ++sk) {
            const int s = sk / kchunks, kc = sk % kchunks;
            const float2 *rowp[4];
            int pkv[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                rowp[e] = nullptr;
                pkv[e] = -1;
                const int k = kc * g.E + 2 * e;   // even: the real part of (p', t)
                if (2 * e < g.E) {
                    const int pk = k / twoT, t = (k % twoT) >> 1;
                    const long long pix = pix0 + (long long)s * g.P + pk;
                    if (pk < g.P && pix < npix) {
                        rowp[e] = xs + ((size_t)(s * g.P + pk) * T + t) * M;
                        pkv[e] = pk;
                    }
                }
            }
            unsigned char *slot = ops + (size_t)s * g.slotBytes;
            for (int row = tid; row < rows_ab; row += kThreads) {
                const bool isA = row < 128;
                int p = 0, ch = 0, part = 0;   // part: 0 A, 1 B re columns, 2 B im columns, 3 zero
                if (isA) {
                    p = row / M;
                    ch = row - p * M;
                    part = p < g.P ? 0 : 3;
                } else {
                    const int n = row - 128;
                    part = n < M ? 1 : (n < 2 * M ? 2 : 3);
                    ch = n < M ? n : n - M;
                }
                uint32_t hi[8], lo[8];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    float2 v = make_float2(0.f, 0.f);
                    if (rowp[e] && part != 3 && (part != 0 || pkv[e] == p)) {
                        v = rowp[e][ch];
                        if (part == 2) v = make_float2(-v.y, v.x);
                    }
                    split<SPLIT>(v.x, hi[2 * e], lo[2 * e]);
                    split<SPLIT>(v.y, hi[2 * e + 1], lo[2 * e + 1]);
                }
                uint4 h4, l4;
                if (BF16) {
                    h4 = make_uint4(hi[0] | (hi[1] << 16), hi[2] | (hi[3] << 16), hi[4] | (hi[5] << 16),
                                    hi[6] | (hi[7] << 16));
                    l4 = make_uint4(lo[0] | (lo[1] << 16), lo[2] | (lo[3] << 16), lo[4] | (lo[5] << 16),
                                    lo[6] | (lo[7] << 16));
                } else {
                    h4 = make_uint4(hi[0], hi[1], hi[2], hi[3]);
                    l4 = make_uint4(lo[0], lo[1], lo[2], lo[3]);
                }
                const int off = isA ? core_off(row, kc, sbo) : g.aBytes + core_off(row - 128, kc, sbo);
                *(uint4 *)(slot + off) = h4;
                if (NT == 3) *(uint4 *)(slot + g.aBytes + g.bBytes + off) = l4;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();

        // 2. one thread issues the MMAs of all slots and commits them to the barrier
        if (tid == 0) {
            tc_fence_after();
            const int nk = g.Ktot / g.kstep;
            for (int s = 0; s < g.S; ++s) {
                const uint32_t base = smem_u32(ops + (size_t)s * g.slotBytes);
                const uint32_t aH = base, bH = base + g.aBytes;
                const uint32_t aL = base + g.aBytes + g.bBytes, bL = aL + g.aBytes;
                const uint32_t d = tmem + (uint32_t)(s * g.N);
                int first = 1;
                // small products first, then hi*hi
#pragma unroll
                for (int term = 0; term < NT; ++term) {
                    const uint32_t a = (NT == 3 && term == 1) ? aL : aH;
                    const uint32_t b = (NT == 3 && term == 0) ? bL : bH;
                    for (int ks = 0; ks < nk; ++ks) {
                        mma<BF16>(d, sdesc(a + ks * 256, 128, sbo), sdesc(b + ks * 256, 128, sbo), g.idesc,
                                  first ? 0u : 1u);
                        first = 0;
                    }
                }
            }
            mma_commit(bar);
            if (!mbar_wait_bounded(bar, phase)) {
                atomicOr(prm.status, ERR_TIMEOUT);
                mbar_wait_bounded(bar, phase);   // let what is in flight drain
                *flag = 1;
            }
        }
        phase ^= 1u;
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (*flag) break;

        // 3. per slot: TMEM -> diagonal band -> smoothed R -> HBM
        for (int s = 0; s < g.S; ++s) {
            const long long spix = pix0 + (long long)s * g.P;
            if (spix >= npix) break;
            const int q4 = warp & 3;                   // TMEM lane quadrant
            const int r = q4 * 32 + lane;              // this thread's TMEM lane: row (p, m)
            const int p = r / M, m = r % M;
            const bool rv = p < g.P;
            for (int c0 = 32 * (warp >> 2); c0 < 2 * M; c0 += 64) {
                uint32_t v[32];
                tmem_ld32(tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(s * g.N + c0), v);
#pragma unroll
                for (int q = 0; q < 32; ++q) {
                    const int col = c0 + q;
                    const bool im = col >= M;
                    const int dd = (im ? col - M : col) - m;
                    if (rv && dd >= 0 && dd < L) (im ? bandIm : bandRe)[r * g.bs + dd] = __uint_as_float(v[q]);
                }
            }
            __syncthreads();
            // one thread per (pixel, diagonal, segment of the diagonal): sliding
            // float-float window sums, each segment starting from a full sum
            const int np = (int)min((long long)g.P, npix - spix);
            if (tid < np * L * nseg) {
                const int sg = tid % nseg, dg = (tid / nseg) % L, pp = tid / (nseg * L);
                const int j0 = sg * seglen, j1 = min(j0 + seglen, L - dg);
                const float *gr = bandRe + (size_t)pp * M * g.bs + dg;
                const float *gi = bandIm + (size_t)pp * M * g.bs + dg;
                float2 *Rp = Rst + (size_t)pp * L * L;
                float tr = 0.f;
                if (j0 < j1) {
                    float2 h = make_float2(0.f, 0.f), l = make_float2(0.f, 0.f);
                    for (int i = j0; i < j0 + Ns; ++i) two_sum_acc(h, l, make_float2(gr[i * g.bs], gi[i * g.bs]));
                    for (int j = j0; j < j1; ++j) {
                        if (j > j0) {
                            two_sum_acc(h, l, make_float2(gr[(j + Ns - 1) * g.bs], gi[(j + Ns - 1) * g.bs]));
                            two_sum_acc(h, l, make_float2(-gr[(j - 1) * g.bs], -gi[(j - 1) * g.bs]));
                        }
                        const float2 vv = fadd2(h, l);
                        Rp[j + (j + dg) * L] = vv;
                        if (dg)
                            Rp[(j + dg) + j * L] = cconj(vv);
                        else
                            tr += vv.x;
                    }
                }
                if (dg == 0) trp[pp * nseg + sg] = tr;
            }
            __syncthreads();
            if (tid < np) {
                float tr = 0.f;
                for (int sg = 0; sg < nseg; ++sg) tr += trp[tid * nseg + sg];
                prm.dl[spix + tid] = f.loading == COS_CAPON_LOAD_ABSOLUTE ? f.d * (float)(Ns * T) : f.d * tr / (float)L;
            }
            // the slot's R block is contiguous in HBM
            const int n2 = np * L * L;
            float2 *dst = prm.Rw + (size_t)spix * L * L;
            for (int i = tid; i < n2; i += kThreads) dst[i] = Rst[i];
            __syncthreads();
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

}  // namespace tc

using namespace tc;

// geometry of a frame for one split; false when the shape is outside the forms
static bool tc_geometry(const FrameDev &f, int split, Geom &g)
{
    const int M = f.M, L = f.L, T = 2 * f.K + 1;
    if (M < 16 || M > 128 || (M % 16) || L > 64 || L > M) return false;
    const bool bf16 = split == COS_CAPON_FORM_TC_BF16X3;
    g.P = 128 / M;
    g.N = ((2 * M + 15) / 16) * 16;
    g.E = bf16 ? 8 : 4;
    g.esize = bf16 ? 2 : 4;
    g.kstep = bf16 ? 16 : 8;
    g.Ktot = ((g.P * 2 * T + g.kstep - 1) / g.kstep) * g.kstep;
    g.copies = split == COS_CAPON_FORM_TC_TF32 ? 1 : 2;
    g.aBytes = 128 * g.Ktot * g.esize;
    g.bBytes = g.N * g.Ktot * g.esize;
    g.slotBytes = g.copies * (g.aBytes + g.bBytes);
    g.bs = L + 2;   // odd float offset between rows' writes of one band column
    const int bandBytes = 2 * 128 * g.bs * (int)sizeof(float);
    const int tail = kMaxTracePartials * (int)sizeof(float) + 64;
    g.nseg = kThreads / (g.P * L);
    if (g.nseg > L) g.nseg = L;
    const int rstBytes = g.P * L * L * (int)sizeof(float2);
    const int winBytes = g.P * T * M * (int)sizeof(float2);   // per slot
    auto layout = [&](int S) {
        g.S = S;
        int area = S * g.slotBytes;
        const int after = ((bandBytes + 15) & ~15) + rstBytes;   // band, then staged R
        if (area < after) area = after;
        g.opBytes = (area + 1023) & ~1023;
        g.bandOff = 0;
        g.rstOff = (bandBytes + 15) & ~15;
        g.xsOff = g.opBytes;
        g.smem = g.opBytes + S * winBytes + tail;
    };
    int S = kTmemCols / g.N;
    if (S > 4) S = 4;
    layout(S);
    while (g.S > 1 && g.smem > kTwoCtaSmem) layout(g.S - 1);
    if (g.smem > 227 * 1024) return false;
    if (g.smem < kMinSmem) g.smem = kMinSmem;
    // instruction descriptor: FP32 accumulator, K-major A and B, N>>3, M>>4
    const uint32_t fmt = bf16 ? 1u : 2u;   // BF16 (kind::f16) / TF32 (kind::tf32)
    g.idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(g.N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    return true;
}

bool tc_supported(const FrameDev &f, int split)
{
    Geom g;
    return tc_geometry(f, split, g);
}

template <int SPLIT>
static int launch_split(const Params &p, int num_sms, cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(tc_cov_kernel<SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         p.g.smem);
    if (e != cudaSuccess) return e;
    const long long npix = (long long)p.f.Nx * p.f.Npy;
    const long long units = (npix + (long long)p.g.S * p.g.P - 1) / ((long long)p.g.S * p.g.P);
    const long long per_sm = p.g.smem <= kTwoCtaSmem ? 2 : 1;
    const long long cap = per_sm * num_sms;
    const int grid = (int)(units < cap ? units : cap);
    tc_cov_kernel<SPLIT><<<grid, kThreads, p.g.smem, s>>>(p);
    return cudaGetLastError();
}

int launch_tc_covariance(const FrameDev &f, int split, float2 *Rw, float *dl, unsigned *status, int num_sms,
                         cudaStream_t s)
{
    Params p;
    memset(&p, 0, sizeof(p));
    if (!tc_geometry(f, split, p.g)) return cudaErrorNotSupported;
    p.f = f;
    p.split = split;
    p.Rw = Rw;
    p.dl = dl;
    p.status = status;
    switch (split) {
    case COS_CAPON_FORM_TC_TF32: return launch_split<COS_CAPON_FORM_TC_TF32>(p, num_sms, s);
    case COS_CAPON_FORM_TC_TF32X3: return launch_split<COS_CAPON_FORM_TC_TF32X3>(p, num_sms, s);
    case COS_CAPON_FORM_TC_BF16X3: return launch_split<COS_CAPON_FORM_TC_BF16X3>(p, num_sms, s);
    default: return cudaErrorNotSupported;
    }
}

}  // namespace cgb
