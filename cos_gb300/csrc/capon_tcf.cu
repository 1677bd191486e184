// Tensor-core fused element-space Capon/MVDR kernel for sm_103a
// (COS_CAPON_FORM_TC_FUSED): the covariance on tcgen05, R kept on chip.
//
// The per-pixel covariance (getCaponC.pyx:207-242; buildR_kernel.cu:45-161)
//   R_p[a,b] = sum_{t<T} C_{p+t}[a,b],   C_y[a,b] = sum_{s<Ns} x_y[s+a] conj(x_y[s+b])
// is the window sum of per-range-row Hankel Grams C_y.  One persistent CTA per
// SM holds two independent groups of four warps; each group has its own half
// of the shared memory and of the TMEM and walks its own units (frame, beam,
// 16 range pixels = 16+2K rows).  A group alternates a covariance phase, whose
// heavy work runs on the tensor cores, and a register-Cholesky phase on the
// CUDA cores, so one group's factorisation overlaps the other's MMAs: group
// 1 starts once group 0 has finished its first covariance phase, which puts
// the two groups half a period apart.
// Per unit, inside a group:
//
//  1. the rows arrive by one bulk copy (cp.async.bulk, mbarrier); per row a
//     power-of-2 scale sigma_y (the row's largest component lands in
//     [2^14, 2^15)) and the subarray sums g of the 16 centre rows.
//  2. covariance phase:
//     * the producer warp builds each row's MMA operands in shared memory:
//       the Hankel rows x_y[a .. a+Ns) need no copy per a, because a plane
//       whose 16-byte chunk q holds x_y[q .. q+8) makes consecutive Hankel
//       rows consecutive chunks, and the next 8 subarrays the chunk 8 further
//       on -- exactly the no-swizzle K-major core-matrix layout with
//       LBO = 256 B, SBO = 128 B.  Values are split hi + lo in FP16 (22
//       significant bits after the per-row scaling);
//     * one thread, handed each plane set by an mbarrier, issues the three
//       products hi*lo, lo*hi, hi*hi of
//         D[(a,p), b] = sum_k A[(a,p),k] B[b,k],
//         A[(a,0)] = [Re x_a | Im x_a],  A[(a,1)] = [Im x_a | -Re x_a],  B[b] = [Re x_b | Im x_b]
//       so D[(a,0),b] = Re C[a,b], D[(a,1),b] = Im C[a,b] (M = 128 rows of
//       which 2L carry data, N = L, K = 2 Ns in steps of 16 plus one tail
//       step whose B chunk is zero past the last subarray), accumulated in
//       FP32 in a TMEM ring of rows (tcgen05.commit -> mbarrier per row);
//     * the consumer warps (one per TMEM sub-partition with data) walk the
//       unit's pixels in order and slide the window sum: pixel p adds the
//       entering row p+2K and subtracts the leaving row p-1 (each read back
//       with tcgen05.ld, its row scale undone), restarting from a direct sum
//       every kRestart pixels and wherever the row scales of the window and
//       the leaving row differ by more than a factor 4 (a large leaving row
//       would cancel the small ones); they write the upper triangle of R_p to
//       shared memory and release a row's TMEM slot once no later pixel reads
//       it.
//  3. the group's warps each load four pixels' R into registers (G = 8 lanes
//     per pixel) and run the register Cholesky with the right-hand sides
//     a = 1 and g carried along (capon_chol.cuh), then
//     z = a^H R^-1 g / a^H R^-1 a and P = 1/((Ns T) a^H R^-1 a)
//     (getCaponC.pyx:246-289).
//
// Measured on GB300: a tcgen05.mma costs at least ~52 clock cycles up to
// N = 64 whatever its size, and a 32x32b.x32 TMEM load about 100, so the
// covariance of one range row (15 MMAs) is an instruction-bound ~1.1k cycles.
// R never reaches HBM: the only DRAM traffic is the cube (with a 2K-row halo
// per unit) and z, P.  Every mbarrier wait is bounded; on expiry the CTA
// records COS_CAPON_ERR_TIMEOUT, drains its in-flight copies and MMAs, frees
// its TMEM and leaves.
#include <cuda_fp16.h>

#include "capon_chol.cuh"
#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {
namespace tcf {

static constexpr int kThreads = 256;
static constexpr int kGroups = 2;             // independent 4-warp groups per CTA
static constexpr int kGroupThreads = 128;
static constexpr int kTile = 16;              // pixels per unit: one Cholesky pass of a group (4 warps x 4 pixels)
static constexpr int kSlots = 3;              // operand plane sets in flight per group
static constexpr int kTmemCols = 512;         // the whole TMEM: one CTA per SM
static constexpr int kGroupCols = kTmemCols / kGroups;
static constexpr int kRestart = 8;            // pixels per direct window sum (the others slide)
static constexpr int kMinSmem = 120 * 1024;   // keeps a second CTA (and its TMEM allocation) off the SM

template <int L_, int T_, int M_>
struct Cfg {
    static constexpr int L = L_, T = T_, M = M_, K = (T_ - 1) / 2;
    static constexpr int NS = M - L + 1;          // subarrays
    static constexpr int NI = NS / 16;            // main MMA K-steps per part (16 subarrays each)
    static constexpr int REM = NS - 16 * NI;      // subarrays of the tail step
    static constexpr int ROWS = kTile + 2 * K;
    static constexpr int QB = (16 * NI + L) / 8;  // 8-chunk groups of a plane (chunk q < 16 NI + L)
    static constexpr int PB = QB * 256;           // bytes of one plane (QB groups x {Re, Im} x 8 chunks x 16 B)
    static constexpr int BTB = 2 * L * 16;        // bytes of the B tail chunks (Re, Im)
    static constexpr int SETB = 4 * PB + 2 * BTB; // one plane set: P1 hi, P2 hi, P1 lo, P2 lo, BT hi, BT lo
    static constexpr int NUP = L * (L + 1) / 2;   // packed upper triangle
    static constexpr int G = 8, NM = L / G, PPW = 32 / G;
    static constexpr int RING = kGroupCols / L < 16 ? kGroupCols / L : 16;  // TMEM row slots of a group
    static constexpr int CSUBS = 2 * L / 32;      // TMEM sub-partitions whose lanes carry data = consumer warps
    static_assert(L == 16 || L == 32, "register Cholesky instantiated for L = 16, 32");
    static_assert(NI >= 1 && REM <= 8, "subarray count outside the built MMA schedule");
    static_assert(kGroupThreads / 32 * PPW == kTile, "one Cholesky pass per unit");
    static_assert(RING >= T + 2, "TMEM ring shorter than the window");
};

// shared-memory carve-up of one group (bytes); group g starts at g * bytes
template <class C>
struct Smem {
    static constexpr size_t rnd(size_t v) { return (v + 127) & ~(size_t)127; }
    static constexpr size_t raw = 0;
    static constexpr size_t gs = raw + rnd((size_t)C::ROWS * C::M * 8);
    static constexpr size_t rst = gs + rnd((size_t)kTile * C::L * 8);
    static constexpr size_t pl = rst + rnd((size_t)kTile * C::NUP * 8);
    // the data-free MMA rows (2L..127) of a plane set read up to one plane
    // past it: slack after the last set keeps them in bounds
    static constexpr size_t slack = 1024;
    static constexpr size_t rs = pl + rnd((size_t)kSlots * C::SETB + slack);
    static constexpr size_t bar = rs + rnd((size_t)3 * C::ROWS * 4);
    static constexpr size_t bytes = rnd(bar + (1 + 2 * C::RING + kSlots) * 8 + 16);   // + gflag[2]
    static constexpr size_t total_raw = kGroups * bytes + 128;   // + TMEM address, abort and start flags
    static constexpr size_t total = total_raw < (size_t)kMinSmem ? (size_t)kMinSmem : total_raw;
};

COS_DEV uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- mbarrier ------------------------------------------------------------------
COS_DEV void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count));
}
COS_DEV bool mbar_try(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait; gives up after `limit` polls or when another thread of the
// CTA has raised the abort flag
COS_DEV bool mbar_wait(uint64_t *bar, uint32_t parity, const volatile int *abort_flag, uint32_t limit = kWaitLimit)
{
    for (uint32_t it = 0; it < limit; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 255u) == 255u && abort_flag && *abort_flag) return false;
    }
    return false;
}
COS_DEV void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}
COS_DEV void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(saddr(dst)),
        "l"(src), "r"(bytes), "r"(saddr(bar))
        : "memory");
}
COS_DEV void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// barrier of one 4-warp group (ids 1 and 2; 0 is __syncthreads)
COS_DEV void group_sync(int g) { asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(kGroupThreads) : "memory"); }

// ---- tcgen05 ---------------------------------------------------------------------
COS_DEV void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
COS_DEV void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// shared-memory matrix descriptor: no swizzle, K-major core matrices
// (LBO = next core matrix along K, SBO = next 8-row group)
COS_DEV constexpr uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
COS_DEV void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
COS_DEV void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}
template <int N>
COS_DEV void tmem_ld(uint32_t taddr, uint32_t (&v)[N]);
template <>
COS_DEV void tmem_ld<32>(uint32_t taddr, uint32_t (&v)[32])
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
}
template <>
COS_DEV void tmem_ld<16>(uint32_t taddr, uint32_t (&v)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
}
COS_DEV void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// offset of row k's first entry R[k][k] in the packed upper triangle
template <int L>
COS_DEV constexpr int up_off(int k)
{
    return k * L - k * (k - 1) / 2;
}

// unit u of the launch -> frame index
COS_DEV int unit_frame(const FramesParam &fp, long long u)
{
    int f = 0;
    while (f + 1 < fp.n && u >= fp.f[f + 1].tile_begin) ++f;
    return f;
}

struct UnitGeo {
    int fi, bx, p0, np, nr;
};
template <class C>
COS_DEV UnitGeo unit_geo(const FramesParam &fp, long long u)
{
    UnitGeo g;
    g.fi = unit_frame(fp, u);
    const FrameDev &f = fp.f[g.fi];
    const long long lu = u - f.tile_begin;
    g.bx = (int)(lu / f.tiles_per_beam);
    g.p0 = (int)(lu % f.tiles_per_beam) * kTile;
    g.np = min(kTile, f.Npy - g.p0);
    g.nr = g.np + 2 * C::K;
    return g;
}

template <class C>
COS_DEV void issue_copy(const FramesParam &fp, long long u, float2 *raw, uint64_t *bar)
{
    const UnitGeo g = unit_geo<C>(fp, u);
    const FrameDev &f = fp.f[g.fi];
    const float2 *src = f.x + ((size_t)g.bx * f.Ny + g.p0) * C::M;
    fence_proxy_async();
    bulk_g2s(raw, src, (uint32_t)((size_t)g.nr * C::M * sizeof(float2)), bar);
}

// one row's operand planes, built by the 32 lanes of the producer warp
template <class C>
COS_DEV void build_planes(const float2 *__restrict__ xrow, float sc, unsigned char *set, int lane)
{
    constexpr int NQ = 8 * C::QB;  // chunks per part
    uint4 *P1H = (uint4 *)(set), *P2H = (uint4 *)(set + C::PB), *P1L = (uint4 *)(set + 2 * C::PB),
          *P2L = (uint4 *)(set + 3 * C::PB), *BTH = (uint4 *)(set + 4 * C::PB),
          *BTL = (uint4 *)(set + 4 * C::PB + C::BTB);
    auto split = [&](const float (&v)[8], uint4 &h4, uint4 &l4) {
        uint32_t h[4], l[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const __half2 hh = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
            const float2 hf = __half22float2(hh);
            const __half2 ll = __floats2half2_rn(v[2 * i] - hf.x, v[2 * i + 1] - hf.y);
            h[i] = *(const uint32_t *)&hh;
            l[i] = *(const uint32_t *)&ll;
        }
        h4 = make_uint4(h[0], h[1], h[2], h[3]);
        l4 = make_uint4(l[0], l[1], l[2], l[3]);
    };
    constexpr uint32_t sgn = 0x80008000u;
    // task q: both components of x[q .. q+8): P1 groups 2(q/8) (Re), 2(q/8)+1
    // (Im) at row q%8; P2 groups 2(q/8) (Im) and 2(q/8)+1 (-Re)
    for (int q = lane; q < NQ; q += 32) {
        float vr[8], vi[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const float2 x = (q + e < C::M) ? xrow[q + e] : make_float2(0.f, 0.f);
            vr[e] = x.x * sc;
            vi[e] = x.y * sc;
        }
        uint4 rh, rl, ih, il;
        split(vr, rh, rl);
        split(vi, ih, il);
        const int c0 = 16 * (q >> 3) + (q & 7), c1 = c0 + 8;
        P1H[c0] = rh;
        P1L[c0] = rl;
        P1H[c1] = ih;
        P1L[c1] = il;
        P2H[c0] = ih;
        P2L[c0] = il;
        P2H[c1] = make_uint4(rh.x ^ sgn, rh.y ^ sgn, rh.z ^ sgn, rh.w ^ sgn);
        P2L[c1] = make_uint4(rl.x ^ sgn, rl.y ^ sgn, rl.z ^ sgn, rl.w ^ sgn);
    }
    if (C::REM > 0) {
        // B tail: chunk b = component of x[b + 16 NI .. + REM), zero after
        for (int b = lane; b < C::L; b += 32) {
            float vr[8], vi[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int idx = b + 16 * C::NI + e;
                const float2 x = (e < C::REM && idx < C::M) ? xrow[idx] : make_float2(0.f, 0.f);
                vr[e] = x.x * sc;
                vi[e] = x.y * sc;
            }
            uint4 rh, rl, ih, il;
            split(vr, rh, rl);
            split(vi, ih, il);
            BTH[b] = rh;
            BTL[b] = rl;
            BTH[C::L + b] = ih;
            BTL[C::L + b] = il;
        }
    }
}

// the three split products of one row into TMEM columns `d` (issuer thread).
// The descriptors are compile-time constants relative to the plane set; the
// set's shared-memory address (>> 4) is added to their address field.
template <class C>
COS_DEV void issue_mmas(uint32_t set, uint32_t d)
{
    // FP32 accumulator, F16 A and B, both K-major, N = L, M = 128
    constexpr uint32_t idesc = (1u << 4) | ((uint32_t)(C::L >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    constexpr uint32_t P1H = 0, P2H = C::PB, P1L = 2 * C::PB, P2L = 3 * C::PB, BTH = 4 * C::PB,
                       BTL = 4 * C::PB + C::BTB;
    const uint64_t sb = (uint64_t)(set >> 4);
    uint32_t acc = 0;
    // small products first: A_hi B_lo, A_lo B_hi, then A_hi B_hi
#pragma unroll
    for (int term = 0; term < 3; ++term) {
        const uint32_t a1 = term == 1 ? P1L : P1H, a2 = term == 1 ? P2L : P2H;
        const uint32_t b1 = term == 0 ? P1L : P1H, bt = term == 0 ? BTL : BTH;
#pragma unroll
        for (int j = 0; j < C::NI; ++j) {  // K part 0: A from P1, B = Re groups of P1
            mma_f16(d, sdesc(a1 + 512 * j, 256, 128) + sb, sdesc(b1 + 512 * j, 256, 256) + sb, idesc, acc);
            acc = 1;
        }
#pragma unroll
        for (int j = 0; j < C::NI; ++j)  // K part 1: A from P2, B = Im groups of P1
            mma_f16(d, sdesc(a2 + 512 * j, 256, 128) + sb, sdesc(b1 + 128 + 512 * j, 256, 256) + sb, idesc, 1);
        if (C::REM > 0)  // tail: (part 0, part 1) chunks at subarray 16 NI; B zero past the last subarray
            mma_f16(d, sdesc(a1 + 512 * C::NI, C::PB, 128) + sb, sdesc(bt, C::L * 16, 128) + sb, idesc, 1);
    }
}

template <class C>
__global__ void __launch_bounds__(kThreads, 1)
tcf_kernel(const __grid_constant__ FramesParam fp, long long total_units, unsigned *status)
{
    using S = Smem<C>;
    constexpr int L = C::L, G = C::G, NM = C::NM, T = C::T, K = C::K, RING = C::RING;
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = warp >> 2, wig = warp & 3;  // group, warp in group (= TMEM sub-partition)
    unsigned char *gsm = smem + (size_t)grp * S::bytes;
    float2 *raw = (float2 *)(gsm + S::raw);
    float2 *gs = (float2 *)(gsm + S::gs);
    float2 *rst = (float2 *)(gsm + S::rst);
    unsigned char *planes = gsm + S::pl;
    float *rs_scale = (float *)(gsm + S::rs);
    float *rs_inv2 = rs_scale + C::ROWS;
    int *rs_exp = (int *)(rs_inv2 + C::ROWS);  // sigma_y = 2^rs_exp[y]
    uint64_t *bar_copy = (uint64_t *)(gsm + S::bar);
    uint64_t *bar_mma = bar_copy + 1;
    uint64_t *bar_free = bar_mma + RING;
    uint64_t *bar_ready = bar_free + RING;
    // gflag[0]: a failed copy wait in this group; gflag[1]: the group's
    // decision to stop, written by one thread between two group barriers so
    // that all four warps take the same branch (the abort flag can change
    // between their reads)
    volatile int *gflag = (volatile int *)(bar_ready + kSlots);
    uint32_t *tmem_slot = (uint32_t *)(smem + kGroups * S::bytes);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    volatile int *start_flag = abort_flag + 1;  // group 0 has finished its first covariance phase

    const bool consumer = wig < C::CSUBS;
    const bool issuer = wig == 2 && lane == 0;
    const bool producer = wig == 3;

    if (tid == 0) {
        *abort_flag = 0;
        *start_flag = 0;
    }
    if (wig == 0 && lane == 0) {
        mbar_init(bar_copy, 1);
        for (int i = 0; i < RING; ++i) {
            mbar_init(&bar_mma[i], 1);
            mbar_init(&bar_free[i], C::CSUBS);
        }
        for (int i = 0; i < kSlots; ++i) mbar_init(&bar_ready[i], 1);
        gflag[0] = 0;
        gflag[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = *tmem_slot + (uint32_t)(grp * kGroupCols);

    // the group's units: virtual CTA 2*blockIdx + grp of 2*gridDim
    const long long ustride = (long long)kGroups * gridDim.x;
    long long u = (long long)kGroups * blockIdx.x + grp;
    // issuer-thread state: a copy in flight, the last committed row
    bool copy_pending = false;
    long long last_commit = -1;
    if (issuer && u < total_units) {
        issue_copy<C>(fp, u, raw, bar_copy);
        copy_pending = true;
    }
    bool stalled = false;
    if (fp.stall_test) {
        // test of the timeout path: a bounded wait on a barrier that nothing
        // completes (bar_free[0], parity 0) runs out
        if (issuer && grp == 0 && !mbar_wait(&bar_free[0], 0u, nullptr, kStallTestLimit)) {
            atomicOr(status, ERR_TIMEOUT);
            *abort_flag = 1;
        }
        stalled = true;
    }
    uint32_t copy_parity = 0;
    long long gbase = 0;  // rows processed by this group before the current unit (TMEM ring index)
    if (grp == 1 && !stalled) {
        // half a period behind group 0 (bounded: group 0 may have no unit at all)
        if (wig == 0 && lane == 0)
            for (uint32_t it = 0; it < (1u << 20) && !*start_flag && !*abort_flag; ++it) __nanosleep(64);
        group_sync(grp);
    }

    for (; !stalled && u < total_units; u += ustride) {
        const UnitGeo geo = unit_geo<C>(fp, u);
        const FrameDev &f = fp.f[geo.fi];
        const int np = geo.np, nr = geo.nr;

        // ---- 1. rows, row scales, subarray sums (the group's four warps)
        {
            const bool okc = mbar_wait(bar_copy, copy_parity, abort_flag);
            if (!okc) gflag[0] = 1;
            group_sync(grp);
            if (wig == 0 && lane == 0) gflag[1] = (gflag[0] != 0 || *abort_flag) ? 1 : 0;
            group_sync(grp);
            const bool bad = gflag[1] != 0;
            if (bad) {
                if (issuer && !*abort_flag) {
                    atomicOr(status, ERR_TIMEOUT);
                    *abort_flag = 1;
                }
                break;
            }
        }
        copy_parity ^= 1u;
        if (issuer) copy_pending = false;
        for (int y = wig; y < nr; y += 4) {
            const float4 *xr = (const float4 *)(raw + (size_t)y * C::M);
            float mx = 0.f;
            for (int i = lane; i < C::M / 2; i += 32) {
                const float4 v = xr[i];
                mx = fmaxf(mx, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0) {
                // sigma = 2^(15 - e), mx in [2^(e-1), 2^e): the largest component lands in [2^14, 2^15)
                int e = 0;
                if (mx > 0.f && mx < 3.0e38f) frexpf(mx, &e);
                e = 15 - e;
                e = e < -60 ? -60 : (e > 60 ? 60 : e);
                rs_scale[y] = ldexpf(1.f, e);
                rs_inv2[y] = ldexpf(1.f, -2 * e);
                rs_exp[y] = e;
            }
        }
        {
            // g[l] = (1/Ns) sum_{s<Ns} x_{p+K}[s+l] (getCaponC.pyx:246-255): items of
            // 4 consecutive l, the first sum direct, then sliding
            constexpr int LW = 4;
            const float invNs = 1.0f / (float)C::NS;
            const int gt = tid & (kGroupThreads - 1);
            for (int it2 = gt; it2 < np * (L / LW); it2 += kGroupThreads) {
                const int q = it2 / (L / LW), l0 = LW * (it2 % (L / LW));
                const float2 *xr = raw + (size_t)(q + K) * C::M;
                float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
                int s = 0;
                for (; s + 1 < C::NS; s += 2) {
                    a0 = fadd2(a0, xr[l0 + s]);
                    a1 = fadd2(a1, xr[l0 + s + 1]);
                }
                if (s < C::NS) a0 = fadd2(a0, xr[l0 + s]);
                float2 acc = fadd2(a0, a1);
#pragma unroll
                for (int l = l0; l < l0 + LW; ++l) {
                    gs[q * L + l] = make_float2(acc.x * invNs, acc.y * invNs);
                    if (l + 1 < l0 + LW) acc = fadd2(acc, fsub2(xr[l + C::NS], xr[l]));
                }
            }
        }
        group_sync(grp);

        // ---- 2. covariance phase
        if (producer) {
            for (int y = 0; y < nr; ++y) {
                const long long Gr = gbase + y;
                bool ok = true;
                if (lane == 0 && Gr >= kSlots) {
                    const long long Gp = Gr - kSlots;  // the row whose MMAs last read this plane set
                    ok = mbar_wait(&bar_mma[Gp % RING], (uint32_t)((Gp / RING) & 1), abort_flag);
                    if (!ok && !*abort_flag) {
                        atomicOr(status, ERR_TIMEOUT);
                        *abort_flag = 1;
                    }
                }
                if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) break;
                unsigned char *set = planes + (size_t)(Gr % kSlots) * C::SETB;
                build_planes<C>(raw + (size_t)y * C::M, rs_scale[y], set, lane);
                fence_proxy_async();
                __syncwarp();
                if (lane == 0) mbar_arrive(&bar_ready[Gr % kSlots]);
            }
        } else if (issuer) {
            for (int y = 0; y < nr; ++y) {
                const long long Gr = gbase + y;
                bool ok = mbar_wait(&bar_ready[Gr % kSlots], (uint32_t)((Gr / kSlots) & 1), abort_flag);
                if (ok && Gr >= RING) {  // TMEM slot free: the consumers released row Gr - RING
                    const long long Gf = Gr - RING;
                    ok = mbar_wait(&bar_free[Gf % RING], (uint32_t)((Gf / RING) & 1), abort_flag);
                }
                if (!ok) {
                    if (!*abort_flag) {
                        atomicOr(status, ERR_TIMEOUT);
                        *abort_flag = 1;
                    }
                    break;
                }
                tc_after();
                issue_mmas<C>(saddr(planes + (size_t)(Gr % kSlots) * C::SETB), tmem + (uint32_t)((Gr % RING) * L));
                mma_commit(&bar_mma[Gr % RING]);
                last_commit = Gr;
            }
        } else if (consumer) {
            const int m = 32 * wig + lane;  // TMEM lane = MMA row (a, p)
            const int a = 8 * (m >> 4) + (m & 7), p = (m >> 3) & 1;
            const uint32_t tl = tmem + ((uint32_t)(32 * wig) << 16);
            float *dst0 = (float *)(rst + (up_off<L>(a) - a)) + p;  // entry (a, b) of pixel 0 at dst0[2b]
            float2 W[L / 2];  // the window sum of this lane's entries (b pairs)
            auto accumulate = [&](const uint32_t (&v)[L], float sc) {
                const float2 sc2 = make_float2(sc, sc);
#pragma unroll
                for (int j = 0; j < L / 2; ++j)
                    W[j] = ffma2(make_float2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1])), sc2, W[j]);
            };
            auto colof = [&](int y) { return tl + (uint32_t)(((gbase + y) % RING) * L); };
            bool ok = true;
            for (int px = 0; px < np && ok; ++px) {
                bool restart = (px % kRestart) == 0;
                if (!restart) {
                    int elo = rs_exp[px - 1], ehi = elo;
#pragma unroll
                    for (int t = 0; t < T; ++t) {
                        elo = min(elo, rs_exp[px + t]);
                        ehi = max(ehi, rs_exp[px + t]);
                    }
                    restart = ehi - elo > 2;
                }
                if (lane == 0) {
                    for (int t = restart ? 0 : T - 1; t < T && ok; ++t) {
                        const long long Gr = gbase + px + t;
                        ok = mbar_wait(&bar_mma[Gr % RING], (uint32_t)((Gr / RING) & 1), abort_flag);
                    }
                    if (!ok && !*abort_flag) {
                        atomicOr(status, ERR_TIMEOUT);
                        *abort_flag = 1;
                    }
                }
                ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
                if (!ok) break;
                tc_after();
                if (restart) {
                    uint32_t v[T][L];
#pragma unroll
                    for (int t = 0; t < T; ++t) tmem_ld<L>(colof(px + t), v[t]);
                    tmem_wait_ld();
#pragma unroll
                    for (int j = 0; j < L / 2; ++j) W[j] = make_float2(0.f, 0.f);
#pragma unroll
                    for (int t = 0; t < T; ++t) accumulate(v[t], rs_inv2[px + t]);
                } else {
                    uint32_t vn[L], vo[L];
                    tmem_ld<L>(colof(px + T - 1), vn);
                    tmem_ld<L>(colof(px - 1), vo);
                    tmem_wait_ld();
                    accumulate(vn, rs_inv2[px + T - 1]);
                    accumulate(vo, -rs_inv2[px - 1]);
                }
                // component p of row a, entries b >= a of the packed upper triangle
                float *dst = dst0 + (size_t)px * 2 * C::NUP;
#pragma unroll
                for (int j = 0; j < L / 2; ++j) {
                    if (2 * j >= a) dst[2 * (2 * j)] = W[j].x;
                    if (2 * j + 1 >= a) dst[2 * (2 * j + 1)] = W[j].y;
                }
                // row px-1 is read by no later pixel (the next one subtracts row px)
                tc_before();
                __syncwarp();
                if (lane == 0) {
                    if (px >= 1) mbar_arrive(&bar_free[(gbase + px - 1) % RING]);
                    if (px == np - 1)
                        for (int y = px; y < nr; ++y) mbar_arrive(&bar_free[(gbase + y) % RING]);
                }
            }
        }
        group_sync(grp);
        if (wig == 0 && lane == 0) gflag[1] = *abort_flag ? 1 : 0;
        group_sync(grp);
        if (gflag[1]) break;
        if (grp == 0 && wig == 0 && lane == 0) *start_flag = 1;
        // the rows are consumed: the next unit's copy lands during the factorisation
        if (issuer && u + ustride < total_units) {
            issue_copy<C>(fp, u + ustride, raw, bar_copy);
            copy_pending = true;
        }

        // ---- 3. factorisation: G lanes per pixel, 4 pixels per warp
        {
            const int gi = lane / G, r = lane % G;
            const int px = wig * C::PPW + gi;
            const bool active = px < np;
            const float2 *Rp = rst + (size_t)px * C::NUP;
            float2 A[L][NM];
#pragma unroll
            for (int k = 0; k < L; ++k)
#pragma unroll
                for (int mm = 0; mm < NM; ++mm)
                    if (mm >= k / G) A[k][mm] = Rp[up_off<L>(k) - k + mm * G + r];
            float tr = 0.f;
#pragma unroll
            for (int mm = 0; mm < NM; ++mm)
#pragma unroll
                for (int q = 0; q < G; ++q)
                    if (q == r) tr += A[mm * G + q][mm].x;
            __syncwarp();  // the pivot-row buffers below reuse this warp's R staging
            float4 *rb = (float4 *)(rst + (size_t)wig * C::PPW * C::NUP) + gi * 2 * (L + 1);
#pragma unroll
            for (int o = G / 2; o; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o, G);
            const float dl = f.loading == COS_CAPON_LOAD_ABSOLUTE ? f.d * (float)(C::NS * T) : f.d * tr / (float)L;
#pragma unroll
            for (int mm = 0; mm < NM; ++mm)
#pragma unroll
                for (int q = 0; q < G; ++q)
                    if (q == r) A[mm * G + q][mm].x += dl;
            float2 b2[NM];
#pragma unroll
            for (int mm = 0; mm < NM; ++mm) b2[mm] = gs[px * L + mm * G + r];
            float s11 = 0.f;
            float2 s12 = make_float2(0.f, 0.f);
            bool bad = false;
            factor_zp<L, G, false>(A, b2, rb, r, s11, s12, bad);
            const size_t pix = (size_t)geo.bx * f.Npy + geo.p0 + px;
            if (active && r == 0) {
                const float is11 = 1.0f / s11;
                f.z[pix] = make_float2(s12.x * is11, s12.y * is11);
                if (f.P) f.P[pix] = is11 / ((float)C::NS * (float)T);
                if (bad) atomicOr(status, ERR_NOT_PD);
            }
        }
        gbase += nr;
        group_sync(grp);  // the staging, g and the row scales are rewritten by the next unit
    }

    if (grp == 0 && wig == 0 && lane == 0) *start_flag = 1;   // also when group 0 had no unit
    // ---- drain: MMAs and the bulk copy still in flight, then free the TMEM
    if (issuer) {
        if (last_commit >= 0) mbar_wait(&bar_mma[last_commit % RING], (uint32_t)((last_commit / RING) & 1), nullptr);
        if (copy_pending) mbar_wait(bar_copy, copy_parity, nullptr);
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tmem_slot), "r"(kTmemCols)
                     : "memory");
}

template <class C>
int launch(const FramesParam &fp_in, int mode, unsigned *status, int num_sms, cudaStream_t s)
{
    if (mode != FUSED_ZP) return cudaErrorNotSupported;
    FramesParam fp = fp_in;
    long long begin = 0;
    for (int i = 0; i < fp.n; ++i) {
        FrameDev &g = fp.f[i];
        if (g.M != C::M || g.L != C::L || 2 * g.K + 1 != C::T || g.Nb != 0) return cudaErrorNotSupported;
        // the bulk copy wants a 16-byte aligned cube
        if (((uintptr_t)g.x) & 15u) return cudaErrorNotSupported;
        g.tile = kTile;
        g.tiles_per_beam = (g.Npy + kTile - 1) / kTile;
        g.tile_begin = begin;
        begin += (long long)g.Nx * g.tiles_per_beam;
    }
    const size_t smem = Smem<C>::total;
    if (smem > kFusedSmemMax) return cudaErrorNotSupported;
    cudaError_t e = cudaFuncSetAttribute(tcf_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    // one CTA per SM (the whole TMEM); fewer CTAs when the launch has fewer units
    long long grid = num_sms;
    const long long need = (begin + kGroups - 1) / kGroups;
    if (grid > need) grid = need;
    tcf_kernel<C><<<(unsigned)grid, kThreads, smem, s>>>(fp, begin, status);
    return cudaGetLastError();
}

template <class C>
size_t smem_bytes(int, int)
{
    return Smem<C>::total;
}

using C32T5 = Cfg<32, 5, 64>;
using C32T3 = Cfg<32, 3, 64>;
using C16T3 = Cfg<16, 3, 32>;

const FusedCandidate kCand[] = {
    {"TC.f16x3.L32.M64.T5", 32, 5, 64, launch<C32T5>, smem_bytes<C32T5>},
    {"TC.f16x3.L32.M64.T3", 32, 3, 64, launch<C32T3>, smem_bytes<C32T3>},
    {"TC.f16x3.L16.M32.T3", 16, 3, 32, launch<C16T3>, smem_bytes<C16T3>},
};

}  // namespace tcf

int tc_fused_candidates(const FusedCandidate **out)
{
    *out = tcf::kCand;
    return (int)(sizeof(tcf::kCand) / sizeof(tcf::kCand[0]));
}

}  // namespace cgb
