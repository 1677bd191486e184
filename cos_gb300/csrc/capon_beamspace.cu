// Beamspace Capon (Nb > 0) for sm_103a.
//
// Replaces the reference GPU beamspace routes (RealTimeCapon/Capon.cpp:285-417):
// instead of building the L x L element-space R and transforming it with three
// batched GEMMs (cublasCgemmBatched, Capon.cpp:599-650), every subarray
// snapshot is reduced to Nb Butler beams by a sliding DFT
// (sliding_beamspace_kernel.cu:26-82 recurrence)
//     Y_{s+1}[b] = e^{+j 2 pi bin_b / L} * (Y_s[b] + (x[s+L] - x[s]) / sqrt(L)),
// so that R_bs = B R B^H is formed directly as an Nb x Nb rank-(Ns*T) sum.
// With element-space loading the loaded matrix is
//     B (R + d tr(R)/L I) B^H = B R B^H + d tr(R)/L I      (B B^H = I),
// and tr(R) comes from the snapshot energies; the beamspace-trace convention
// loads with tr(R_bs)/Nb instead (getCaponAllC.pyx:376-385).  Then
//     a_bs = B 1,  x_bs = R_bs^-1 a_bs,  Ria = B^H x_bs,
//     w = Ria / sum(Ria),  z = sum conj(w) g  (capon_kernel.cu:338-427),
//     P = 1 / Re(a_bs^H R_bs,normalised^-1 a_bs).
// One warp per pixel.
#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {

int launch_beamspace_warp(const FrameDev &f, float2 *R_out, cudaStream_t s);

static constexpr int kBsWarps = 4;

struct BsSmem {
    size_t per_warp, table, total;
    int ld;  // Cm leading dimension
    __host__ __device__ BsSmem(int M, int L, int K, int Nb)
    {
        const int T = 2 * K + 1, Ns = M - L + 1;
        ld = Nb + 1;
        per_warp = (size_t)T * M + (size_t)T * Ns * Nb + 3 * (size_t)Nb * ld + 2 * (size_t)Nb + 2;
        table = (size_t)Nb * L + 2 * (size_t)Nb;
        total = (table + kBsWarps * per_warp) * sizeof(float2);
    }
};

__global__ void __launch_bounds__(32 * kBsWarps)
beamspace_kernel(FrameDev f, float2 *__restrict__ Rbs)
{
    extern __shared__ float2 sm[];
    const int M = f.M, L = f.L, K = f.K, T = 2 * K + 1, Ns = M - L + 1, Nb = f.Nb;
    const BsSmem S(M, L, K, Nb);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *Bt = sm;                        // Nb x L Butler matrix
    float2 *rot = Bt + (size_t)Nb * L;      // Nb sliding factors
    float2 *ab = rot + Nb;                  // a_bs = B 1
    float2 *ws = sm + S.table + (size_t)warp * S.per_warp;
    float2 *xs = ws;                              // T x M
    float2 *Y = xs + (size_t)T * M;               // T x Ns x Nb
    float2 *Cm = Y + (size_t)T * Ns * Nb;         // Nb x ld
    float2 *Ch = Cm + (size_t)Nb * S.ld;          // Nb x ld: R_bs high part (float-float)
    float2 *Cl = Ch + (size_t)Nb * S.ld;          // Nb x ld: R_bs low part
    float2 *xb = Cl + (size_t)Nb * S.ld;          // Nb
    const float isl = 1.0f / sqrtf((float)L);

    for (int i = threadIdx.x; i < Nb * L; i += blockDim.x) {
        const int bb = i / L, l = i % L;
        const int bin = butler_bin(bb, Nb, L);
        float sn, cs;
        sincospif(2.0f * (float)((bin * l) % L) / (float)L, &sn, &cs);
        Bt[i] = make_float2(cs * isl, -sn * isl);
    }
    for (int bb = threadIdx.x; bb < Nb; bb += blockDim.x) {
        float sn, cs;
        sincospif(2.0f * (float)butler_bin(bb, Nb, L) / (float)L, &sn, &cs);
        rot[bb] = make_float2(cs, sn);
    }
    __syncthreads();
    for (int bb = warp; bb < Nb; bb += kBsWarps) {
        float2 acc = make_float2(0.f, 0.f);
        for (int l = lane; l < L; l += 32) acc = cadd(acc, Bt[bb * L + l]);
        for (int o = 16; o; o >>= 1) acc = cadd(acc, shfl2_xor(acc, o, 32));
        if (lane == 0) ab[bb] = acc;
    }
    __syncthreads();

    const long long npix = (long long)f.Nx * f.Npy;
    const long long pix = (long long)blockIdx.x * kBsWarps + warp;
    if (pix >= npix) return;
    const int bx = (int)(pix / f.Npy), p = (int)(pix % f.Npy);
    const float2 *xg = f.x + ((size_t)bx * f.Ny + p) * M;
    for (int i = lane; i < T * M; i += 32) xs[i] = xg[i];
    __syncwarp();

    // sliding DFT over a contiguous chunk of subarrays per lane
    const int chunk = (Ns + 31) / 32;
    const int s0 = lane * chunk, s1 = min(Ns, s0 + chunk);
    float energy = 0.f;  // sum over the lane's subarrays of |x_t[s:s+L]|^2
    for (int t = 0; t < T && s0 < s1; ++t) {
        const float2 *xt = xs + t * M;
        float e = 0.f;
        for (int l = 0; l < L; ++l) e += cabs2(xt[s0 + l]);
        energy += e;
        for (int s = s0 + 1; s < s1; ++s) {
            e += cabs2(xt[s - 1 + L]) - cabs2(xt[s - 1]);
            energy += e;
        }
        for (int bb = 0; bb < Nb; ++bb) {
            float2 acc = make_float2(0.f, 0.f);
            for (int l = 0; l < L; ++l) acc = cadd(acc, cmul(Bt[bb * L + l], xt[s0 + l]));
            Y[((size_t)t * Ns + s0) * Nb + bb] = acc;
            const float2 rb = rot[bb];
            for (int s = s0 + 1; s < s1; ++s) {
                acc = cmul(rb, cadd(acc, cscale(csub(xt[s - 1 + L], xt[s - 1]), isl)));
                Y[((size_t)t * Ns + s) * Nb + bb] = acc;
            }
        }
    }
    for (int o = 16; o; o >>= 1) energy += __shfl_xor_sync(0xffffffffu, energy, o);
    __syncwarp();

    // Nb x Nb covariance, upper triangle by lanes, mirrored
    const int ne = Nb * (Nb + 1) / 2;
    for (int e = lane; e < ne; e += 32) {
        int bb = 0, rem = e;
        while (rem >= Nb - bb) { rem -= Nb - bb; ++bb; }
        const int cc = bb + rem;
        // chunks of 4 products summed in FP32, chunk sums accumulated in
        // float-float (TwoSum): one rounding for the whole T*Ns-term sum
        float2 hi = make_float2(0.f, 0.f), lo = make_float2(0.f, 0.f);
        for (int q0 = 0; q0 < T * Ns; q0 += 4) {
            float2 acc = make_float2(0.f, 0.f);
            const int q1 = min(T * Ns, q0 + 4);
            for (int q = q0; q < q1; ++q) acc = cadd(acc, cmulc(Y[(size_t)q * Nb + bb], Y[(size_t)q * Nb + cc]));
            two_sum_acc(hi, lo, acc);
        }
        const float2 v = fadd2(hi, lo);
        const float2 vl = fsub2(lo, fsub2(v, hi));  // v + vl == hi + lo
        Cm[bb * S.ld + cc] = v;
        Cm[cc * S.ld + bb] = cconj(v);
        Ch[bb * S.ld + cc] = v;
        Ch[cc * S.ld + bb] = cconj(v);
        Cl[bb * S.ld + cc] = vl;
        Cl[cc * S.ld + bb] = cconj(vl);
    }
    __syncwarp();
    float dl = 0.f;
    if (lane == 0) {
        if (f.loading == COS_CAPON_LOAD_ABSOLUTE) {
            dl = f.d * (float)(Ns * T);
        } else if (f.loading == COS_CAPON_LOAD_BEAMSPACE) {
            float tb = 0.f;
            for (int i = 0; i < Nb; ++i) tb += Cm[i * S.ld + i].x;
            dl = f.d * tb / (float)Nb;
        } else {
            dl = f.d * energy / (float)L;
        }
        for (int i = 0; i < Nb; ++i) Cm[i * S.ld + i] = make_float2(Cm[i * S.ld + i].x + dl, 0.f);
    }
    __syncwarp();
    if (Rbs) {  // loaded, unnormalised, column-major (as the reference BuildR writes R)
        float2 *Rp = Rbs + (size_t)pix * Nb * Nb;
        for (int i = lane; i < Nb * Nb; i += 32) Rp[i] = Cm[(i % Nb) * S.ld + i / Nb];
    }
    __syncwarp();
    // FP32 Cholesky (upper, row-major in Cm) and the two triangular solves for
    // a_bs, then one step of iterative refinement: the residual
    // r = a_bs - (R_hi + R_lo + dl I) x0 is formed in FP64 from the float-float
    // matrix -- the Butler transform gathers a scatterer into one beam, so a
    // single FP32 rounding of R_bs already perturbs the small eigenvalues by
    // ~1e-4 -- and the correction is solved with the same FP32 factor.
    if (lane == 0) {
        for (int i = 0; i < Nb; ++i) {
            float dv = Cm[i * S.ld + i].x;
            for (int k = 0; k < i; ++k) dv -= cabs2(Cm[k * S.ld + i]);
            const float u = sqrtf(dv), iu = 1.0f / u;
            Cm[i * S.ld + i] = make_float2(u, 0.f);
            for (int j = i + 1; j < Nb; ++j) {
                float2 v = Cm[i * S.ld + j];
                for (int k = 0; k < i; ++k) v = csub(v, cconjmul(Cm[k * S.ld + i], Cm[k * S.ld + j]));
                Cm[i * S.ld + j] = cscale(v, iu);
            }
        }
        for (int pass = 0; pass < 2; ++pass) {
            // right-hand side: a_bs (pass 0) or the FP64 residual (pass 1); the
            // solution is built in Cm's padding column (index Nb)
            for (int i = 0; i < Nb; ++i) {
                float2 v;
                if (pass == 0) {
                    v = ab[i];
                } else {
                    double rr = (double)ab[i].x, ri = (double)ab[i].y;
                    for (int j = 0; j < Nb; ++j) {
                        const double ar = (double)Ch[i * S.ld + j].x + (double)Cl[i * S.ld + j].x +
                                          (i == j ? (double)dl : 0.0);
                        const double ai = (double)Ch[i * S.ld + j].y + (double)Cl[i * S.ld + j].y;
                        const double xr = (double)xb[j].x, xi = (double)xb[j].y;
                        rr -= ar * xr - ai * xi;
                        ri -= ar * xi + ai * xr;
                    }
                    v = make_float2((float)rr, (float)ri);
                }
                // forward U^H y = v
                for (int k = 0; k < i; ++k) v = csub(v, cconjmul(Cm[k * S.ld + i], Cm[k * S.ld + Nb]));
                Cm[i * S.ld + Nb] = cscale(v, 1.0f / Cm[i * S.ld + i].x);
            }
            for (int i = Nb - 1; i >= 0; --i) {
                float2 v = Cm[i * S.ld + Nb];
                for (int k = i + 1; k < Nb; ++k) v = csub(v, cmul(Cm[i * S.ld + k], Cm[k * S.ld + Nb]));
                Cm[i * S.ld + Nb] = cscale(v, 1.0f / Cm[i * S.ld + i].x);
            }
            for (int i = 0; i < Nb; ++i) xb[i] = pass == 0 ? Cm[i * S.ld + Nb] : cadd(xb[i], Cm[i * S.ld + Nb]);
        }
    }
    __syncwarp();
    // Ria = B^H x_bs, w = Ria / sum(Ria), z = sum conj(w) g
    float2 ria[2], sum = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int l = lane + 32 * q;
        ria[q] = make_float2(0.f, 0.f);
        if (l < L) {
            for (int bb = 0; bb < Nb; ++bb) ria[q] = cadd(ria[q], cconjmul(Bt[bb * L + l], xb[bb]));
            sum = cadd(sum, ria[q]);
        }
    }
    for (int o = 16; o; o >>= 1) sum = cadd(sum, shfl2_xor(sum, o, 32));
    const float den = cabs2(sum);
    const float2 isum = make_float2(sum.x / den, -sum.y / den);
    const float2 *xc = xs + (size_t)K * M;
    const float invNs = 1.0f / (float)Ns;
    float2 zacc = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int l = lane + 32 * q;
        if (l < L) {
            const float2 wl = cmul(ria[q], isum);
            if (f.w) f.w[(size_t)pix * L + l] = wl;
            float2 g = make_float2(0.f, 0.f);
            for (int s = 0; s < Ns; ++s) g = cadd(g, xc[s + l]);
            zacc = cadd(zacc, cconjmul(wl, cscale(g, invNs)));
        }
    }
    for (int o = 16; o; o >>= 1) zacc = cadd(zacc, shfl2_xor(zacc, o, 32));
    if (lane == 0) {
        if (f.z) f.z[pix] = zacc;
        if (f.P) {
            float2 aRa = make_float2(0.f, 0.f);
            for (int bb = 0; bb < Nb; ++bb) aRa = cadd(aRa, cconjmul(ab[bb], xb[bb]));
            f.P[pix] = 1.0f / ((float)Ns * (float)T * aRa.x);
        }
    }
}

// ---------------------------------------------------------------------------
// Range-tile kernel for small beam counts (Nb <= 5).  A range row's subarray
// DFTs are shared by the 2K+1 pixels whose window contains the row, so they
// are computed once per row:
//   phase A  one half-warp per row: lane q slides the DFT over subarrays
//            [q c, q c + c) (a direct DFT at the chunk start, then the
//            recurrence), sums its Y Y^H products in FP32 and reduces across
//            the half-warp in float-float -> Q_row (Nb x Nb upper, hi + lo),
//            the row's snapshot energy and beam sums sum_s Y_s;
//   phase B  one thread per pixel: R_bs = sum of the window's Q rows
//            (float-float), loading, FP32 Cholesky, one FP64-residual
//            refinement step, P and z (g_bs = B g = the centre row's beam sums / Ns);
//   phase C  (w requested) w = B^H x_bs / a_bs^H x_bs, one thread per output.
static constexpr int kTileThreads = 256;
// lanes sharing one range row in the per-row phase.  Each starts its share
// of the subarrays with a direct DFT (fewer lanes: fewer of those per row)
// and sums the Y Y^H products in two FP32 accumulators, alternate subarrays,
// merged exactly before the float-float reduction across the lanes.  One
// accumulator per lane at 8 lanes (sums twice as long) raised the worst power
// error against FP64 4-5x at M=128, L=64, Nb=5; the pair keeps each FP32 sum
// as short as with 16 lanes.  A tile is sized so that its pixels plus their
// 2K halo rows make kTileRows rows, whole passes of 256 / kRowLanes rows.
static constexpr int kRowLanes = 8;
static constexpr int kTileRows = 64;

template <int NB>
struct BsTile {
    static constexpr int NQ = NB * (NB + 1) / 2;
};

struct BsTileSmem {
    int rows, tile;
    size_t off_x, off_q, off_e, off_g, off_b, off_xs, off_vv, total;
    __host__ __device__ BsTileSmem(int tile_, int K, int M, int L, int NB)
    {
        tile = tile_;
        rows = tile + 2 * K;
        const int NQ = NB * (NB + 1) / 2;
        off_x = 0;                                                          // rows x M
        off_q = off_x + (((size_t)rows * M * sizeof(float2) + 15) & ~(size_t)15);   // rows x 2NQ (hi, lo)
        off_e = off_q + (size_t)rows * 2 * NQ * sizeof(float2);             // rows: energy
        off_g = off_e + (((size_t)rows * sizeof(float) + 15) & ~(size_t)15); // rows x NB: beam sums
        off_b = off_g + (size_t)rows * NB * sizeof(float2);                 // Butler NB x L, rot NB, a_bs NB
        off_xs = off_b + (size_t)(NB * L + 2 * NB) * sizeof(float2);        // tile x (NB + 1): x_bs, 1/sum
        off_vv = off_xs + (size_t)tile * (NB + 1) * sizeof(float2);          // NQ: V V^H (packed upper)
        total = off_vv + (size_t)NQ * sizeof(float2);
    }
};

template <int NB>
__global__ void __launch_bounds__(kTileThreads, 2)
beamspace_tile_kernel(FrameDev f, float2 *__restrict__ Rbs, int tile)
{
    constexpr int NQ = BsTile<NB>::NQ;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int M = f.M, L = f.L, K = f.K, T = 2 * K + 1, Ns = M - L + 1;
    const BsTileSmem S(tile, K, M, L, NB);
    float2 *xs = (float2 *)(smraw + S.off_x);
    float2 *Qs = (float2 *)(smraw + S.off_q);
    float *Es = (float *)(smraw + S.off_e);
    float2 *Gs = (float2 *)(smraw + S.off_g);
    float2 *Bt = (float2 *)(smraw + S.off_b);
    float2 *rot = Bt + NB * L;
    float2 *ab = rot + NB;
    float2 *Xb = (float2 *)(smraw + S.off_xs);
    float2 *VV = (float2 *)(smraw + S.off_vv);
    const int tid = threadIdx.x;
    const float isl = 1.0f / sqrtf((float)L);
    // a caller-given subspace V: direct products per subarray (no sliding
    // recurrence) and element-space loadings enter as dl V V^H
    const bool direct = f.V != nullptr;
    const bool loadVV = direct && f.loading != COS_CAPON_LOAD_BEAMSPACE;

    const int tiles_per_beam = (f.Npy + tile - 1) / tile;
    const int bx = blockIdx.x / tiles_per_beam;
    const int p0 = (blockIdx.x % tiles_per_beam) * tile;
    const int np = min(tile, f.Npy - p0);
    const int rows = np + 2 * K;

    // Butler table (or the caller's V) and the a_bs = B 1 of this launch
    for (int i = tid; i < NB * L; i += kTileThreads) {
        if (direct) {
            Bt[i] = f.V[i];
        } else {
            const int bb = i / L, l = i % L;
            float sn, cs;
            sincospif(2.0f * (float)((butler_bin(bb, NB, L) * l) % L) / (float)L, &sn, &cs);
            Bt[i] = make_float2(cs * isl, -sn * isl);
        }
    }
    if (tid < NB) {
        float sn, cs;
        sincospif(2.0f * (float)butler_bin(tid, NB, L) / (float)L, &sn, &cs);
        rot[tid] = make_float2(cs, sn);
    }
    // stage the tile's rows (one contiguous run of the beam)
    const float2 *src = f.x + ((size_t)bx * f.Ny + p0) * M;
    for (int i = tid; i < rows * M; i += kTileThreads) xs[i] = src[i];
    __syncthreads();
    if (tid < NB) {
        float2 acc = make_float2(0.f, 0.f);
        for (int l = 0; l < L; ++l) acc = cadd(acc, Bt[tid * L + l]);
        ab[tid] = acc;
    }
    if (loadVV && tid < BsTile<NB>::NQ) {
        int i = 0, rem = tid;
        while (rem >= NB - i) {
            rem -= NB - i;
            ++i;
        }
        const int j = i + rem;
        float2 acc = make_float2(0.f, 0.f);
        for (int l = 0; l < L; ++l) acc = cadd(acc, cmulc(Bt[i * L + l], Bt[j * L + l]));
        VV[tid] = acc;
    }

    // ---- phase A: per-row terms, kRowLanes lanes per row (each starts its
    // share of the subarrays with a direct DFT, then slides)
    {
        constexpr int RL = kRowLanes, RPW = 32 / kRowLanes;
        const int sub = (tid & 31) / RL, q = tid % RL, warp = tid >> 5;
        const int c = (Ns + RL - 1) / RL;
        const int s0 = q * c, s1 = min(Ns, s0 + c);
        for (int base = RPW * warp; base < rows; base += kTileThreads / RL) {
            const int r = base + sub;
            // two FP32 accumulators, alternate subarrays: each sums at most
            // ceil(ceil(Ns / RL) / 2) products before the exact TwoSum merge
            float2 P[NQ], P2[NQ], Yg[NB];
            float en = 0.f;
#pragma unroll
            for (int e = 0; e < NQ; ++e) P[e] = P2[e] = make_float2(0.f, 0.f);
#pragma unroll
            for (int b = 0; b < NB; ++b) Yg[b] = make_float2(0.f, 0.f);
            // forward-backward averaging: the same products over the flipped,
            // conjugated row x~[m] = conj(x[M-1-m]) (its covariance is
            // J R^T J), halved at the end; energy and beam sums from x only
            const int passes = f.fb ? 2 : 1;
            for (int pass = 0; pass < passes && r < rows && s0 < s1; ++pass) {
                const float2 *xr = xs + (size_t)r * M;
                auto X = [&](int i) { return pass ? cconj(xr[M - 1 - i]) : xr[i]; };
                float2 Y[NB];
#pragma unroll
                for (int b = 0; b < NB; ++b) Y[b] = make_float2(0.f, 0.f);
                float e = 0.f;
                for (int l = 0; l < L; ++l) {
                    const float2 v = X(s0 + l);
                    e += cabs2(v);
#pragma unroll
                    for (int b = 0; b < NB; ++b) Y[b] = cadd(Y[b], cmul(Bt[b * L + l], v));
                }
                for (int s = s0; s < s1; ++s) {
                    if (s > s0) {
                        e += cabs2(X(s - 1 + L)) - cabs2(X(s - 1));
                        if (direct) {
#pragma unroll
                            for (int b = 0; b < NB; ++b) Y[b] = make_float2(0.f, 0.f);
                            for (int l = 0; l < L; ++l) {
                                const float2 v = X(s + l);
#pragma unroll
                                for (int b = 0; b < NB; ++b) Y[b] = cadd(Y[b], cmul(Bt[b * L + l], v));
                            }
                        } else {
                            const float2 dx = cscale(csub(X(s - 1 + L), X(s - 1)), isl);
#pragma unroll
                            for (int b = 0; b < NB; ++b) Y[b] = cmul(rot[b], cadd(Y[b], dx));
                        }
                    }
                    if (pass == 0) en += e;
                    const bool odd = ((s - s0) & 1) != 0;
#pragma unroll
                    for (int i = 0; i < NB; ++i) {
                        if (pass == 0) Yg[i] = cadd(Yg[i], Y[i]);
#pragma unroll
                        for (int j = i; j < NB; ++j) {
                            const int k = i * NB - i * (i - 1) / 2 + (j - i);
                            const float2 pr = cmulc(Y[i], Y[j]);
                            if (odd) P2[k] = cadd(P2[k], pr);
                            else P[k] = cadd(P[k], pr);
                        }
                    }
                }
            }
            // merge the two accumulators exactly, then the float-float
            // reduction over the row's lanes
            float2 lo[NQ];
#pragma unroll
            for (int e = 0; e < NQ; ++e) {
                lo[e] = make_float2(0.f, 0.f);
                two_sum_acc(P[e], lo[e], P2[e]);
            }
            if (f.fb) {
#pragma unroll
                for (int e = 0; e < NQ; ++e) {
                    P[e] = cscale(P[e], 0.5f);
                    lo[e] = cscale(lo[e], 0.5f);
                }
            }
#pragma unroll
            for (int o = RL / 2; o; o >>= 1) {
#pragma unroll
                for (int e = 0; e < NQ; ++e) {
                    const float2 oh = shfl2_xor(P[e], o, RL), ol = shfl2_xor(lo[e], o, RL);
                    two_sum_acc(P[e], lo[e], oh);
                    lo[e] = fadd2(lo[e], ol);
                }
#pragma unroll
                for (int b = 0; b < NB; ++b) Yg[b] = cadd(Yg[b], shfl2_xor(Yg[b], o, RL));
                en += __shfl_xor_sync(0xffffffffu, en, o, RL);
            }
            if (r < rows && q == 0) {
#pragma unroll
                for (int e = 0; e < NQ; ++e) {
                    Qs[(size_t)r * 2 * NQ + e] = P[e];
                    Qs[(size_t)r * 2 * NQ + NQ + e] = lo[e];
                }
                Es[r] = en;
#pragma unroll
                for (int b = 0; b < NB; ++b) Gs[(size_t)r * NB + b] = Yg[b];
            }
        }
    }
    __syncthreads();

    // ---- phase B: one thread per pixel
    for (int lp = tid; lp < np; lp += kTileThreads) {
        float2 Rh[NQ], Rl[NQ];
        float tr = 0.f;
#pragma unroll
        for (int e = 0; e < NQ; ++e) {
            Rh[e] = make_float2(0.f, 0.f);
            Rl[e] = make_float2(0.f, 0.f);
        }
        for (int t = 0; t < T; ++t) {
            const float2 *qr = Qs + (size_t)(lp + t) * 2 * NQ;
#pragma unroll
            for (int e = 0; e < NQ; ++e) {
                two_sum_acc(Rh[e], Rl[e], qr[e]);
                Rl[e] = fadd2(Rl[e], qr[NQ + e]);
            }
            tr += Es[lp + t];
        }
        // renormalise: (Rh, Rl) -> rounded value + remainder
#pragma unroll
        for (int e = 0; e < NQ; ++e) {
            const float2 v = fadd2(Rh[e], Rl[e]);
            Rl[e] = fsub2(Rl[e], fsub2(v, Rh[e]));
            Rh[e] = v;
        }
        float dl;
        if (f.loading == COS_CAPON_LOAD_ABSOLUTE) {
            dl = f.d * (float)(Ns * T);
        } else if (f.loading == COS_CAPON_LOAD_BEAMSPACE) {
            float tb = 0.f;
            int k = 0;
#pragma unroll
            for (int i = 0; i < NB; ++i) {
                tb += Rh[k].x;
                k += NB - i;
            }
            dl = f.d * tb / (float)NB;
        } else {
            dl = f.d * tr / (float)L;
        }
        const long long pix = (long long)bx * f.Npy + p0 + lp;
        if (Rbs) {  // loaded, unnormalised, column-major
            float2 *Rp = Rbs + (size_t)pix * NB * NB;
            int k = 0;
#pragma unroll
            for (int i = 0; i < NB; ++i)
#pragma unroll
                for (int j = i; j < NB; ++j, ++k) {
                    const float2 v = loadVV ? cadd(Rh[k], cscale(VV[k], dl))
                                            : ((i == j) ? make_float2(Rh[k].x + dl, 0.f) : Rh[k]);
                    Rp[i + j * NB] = v;
                    if (i != j) Rp[j + i * NB] = cconj(v);
                }
        }
        // FP32 Cholesky of Rh + dl I (upper, packed rows)
        float2 U[NQ];
        {
            int k = 0;
#pragma unroll
            for (int i = 0; i < NB; ++i)
#pragma unroll
                for (int j = i; j < NB; ++j, ++k)
                    U[k] = loadVV ? cadd(Rh[k], cscale(VV[k], dl)) : ((i == j) ? make_float2(Rh[k].x + dl, 0.f) : Rh[k]);
        }
        auto idx = [](int i, int j) { return i * NB - i * (i - 1) / 2 + (j - i); };   // i <= j
#pragma unroll
        for (int i = 0; i < NB; ++i) {
            float dv = U[idx(i, i)].x;
#pragma unroll
            for (int k = 0; k < i; ++k) dv -= cabs2(U[idx(k, i)]);
            const float u = sqrtf(dv), iu = 1.0f / u;
            U[idx(i, i)] = make_float2(u, 0.f);
#pragma unroll
            for (int j = i + 1; j < NB; ++j) {
                float2 v = U[idx(i, j)];
#pragma unroll
                for (int k = 0; k < i; ++k) v = csub(v, cconjmul(U[idx(k, i)], U[idx(k, j)]));
                U[idx(i, j)] = cscale(v, iu);
            }
        }
        auto solve = [&](float2 (&v)[NB]) {
#pragma unroll
            for (int i = 0; i < NB; ++i) {
#pragma unroll
                for (int k = 0; k < i; ++k) v[i] = csub(v[i], cconjmul(U[idx(k, i)], v[k]));
                v[i] = cscale(v[i], 1.0f / U[idx(i, i)].x);
            }
#pragma unroll
            for (int i = NB - 1; i >= 0; --i) {
#pragma unroll
                for (int k = i + 1; k < NB; ++k) v[i] = csub(v[i], cmul(U[idx(i, k)], v[k]));
                v[i] = cscale(v[i], 1.0f / U[idx(i, i)].x);
            }
        };
        float2 xb[NB], r[NB];
#pragma unroll
        for (int i = 0; i < NB; ++i) xb[i] = ab[i];
        solve(xb);
        // FP64 residual against the float-float matrix, one correction
#pragma unroll
        for (int i = 0; i < NB; ++i) {
            double rr = (double)ab[i].x, ri = (double)ab[i].y;
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                double ar, ai;
                if (i <= j) {
                    const int k = idx(i, j);
                    ar = (double)Rh[k].x + (double)Rl[k].x;
                    ai = (double)Rh[k].y + (double)Rl[k].y;
                    if (loadVV) {
                        ar += (double)dl * (double)VV[k].x;
                        ai += (double)dl * (double)VV[k].y;
                    } else if (i == j) {
                        ar += (double)dl;
                    }
                    if (i == j) ai = 0.0;
                } else {
                    const int k = idx(j, i);
                    ar = (double)Rh[k].x + (double)Rl[k].x;
                    ai = -((double)Rh[k].y + (double)Rl[k].y);
                    if (loadVV) {
                        ar += (double)dl * (double)VV[k].x;
                        ai -= (double)dl * (double)VV[k].y;
                    }
                }
                rr -= ar * (double)xb[j].x - ai * (double)xb[j].y;
                ri -= ar * (double)xb[j].y + ai * (double)xb[j].x;
            }
            r[i] = make_float2((float)rr, (float)ri);
        }
        solve(r);
        float2 aRa = make_float2(0.f, 0.f), zn = make_float2(0.f, 0.f);
        const float2 *gc = Gs + (size_t)(lp + K) * NB;
#pragma unroll
        for (int i = 0; i < NB; ++i) {
            xb[i] = cadd(xb[i], r[i]);
            aRa = cadd(aRa, cconjmul(ab[i], xb[i]));
            zn = cadd(zn, cconjmul(xb[i], gc[i]));
        }
        // sum(Ria) = a_bs^H x_bs; z = conj(x_bs)^T g_bs / conj(sum), g_bs = beam sums / Ns
        const float den = cabs2(aRa);
        const float2 isum = make_float2(aRa.x / den, -aRa.y / den);      // 1 / sum
        const float2 zz = cscale(cmul(zn, cconj(isum)), 1.0f / (float)Ns);
        if (f.z) f.z[pix] = zz;
        if (f.P) f.P[pix] = 1.0f / ((float)Ns * (float)T * aRa.x);
#pragma unroll
        for (int i = 0; i < NB; ++i) Xb[(size_t)lp * (NB + 1) + i] = xb[i];
        Xb[(size_t)lp * (NB + 1) + NB] = isum;
    }
    if (f.w) {
        __syncthreads();
        // ---- phase C: w = B^H x_bs / sum, one thread per (pixel, element)
        for (int i = tid; i < np * L; i += kTileThreads) {
            const int lp = i / L, l = i % L;
            const float2 *xv = Xb + (size_t)lp * (NB + 1);
            float2 ria = make_float2(0.f, 0.f);
#pragma unroll
            for (int b = 0; b < NB; ++b) ria = cadd(ria, cconjmul(Bt[b * L + l], xv[b]));
            f.w[((size_t)bx * f.Npy + p0) * L + i] = cmul(ria, xv[NB]);
        }
    }
}

template <int NB>
static int launch_tile(const FrameDev &f, float2 *R_out, cudaStream_t s)
{
    // tile + 2K rows = whole passes of the per-row phase when K is small
    int tile = kTileRows - 2 * f.K >= 16 ? kTileRows - 2 * f.K : 64;
    while (tile > 8 && BsTileSmem(tile, f.K, f.M, f.L, NB).total > 227 * 1024) tile /= 2;
    const BsTileSmem S(tile, f.K, f.M, f.L, NB);
    if (S.total > 227 * 1024) return cudaErrorNotSupported;
    cudaError_t e = cudaFuncSetAttribute(beamspace_tile_kernel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S.total);
    if (e != cudaSuccess) return e;
    const long long blocks = (long long)f.Nx * ((f.Npy + tile - 1) / tile);
    beamspace_tile_kernel<NB><<<(unsigned)blocks, kTileThreads, S.total, s>>>(f, R_out, tile);
    return cudaGetLastError();
}

int launch_beamspace(const FrameDev &f, float2 *R_out, cudaStream_t s)
{
    static_assert(kBeamspaceTileMaxNb == 5, "the tile kernel is instantiated for Nb = 1..5");
    if (f.V && f.Nb > kBeamspaceTileMaxNb) return cudaErrorNotSupported;
    switch (f.Nb) {
    case 1: return launch_tile<1>(f, R_out, s);
    case 2: return launch_tile<2>(f, R_out, s);
    case 3: return launch_tile<3>(f, R_out, s);
    case 4: return launch_tile<4>(f, R_out, s);
    case 5: return launch_tile<5>(f, R_out, s);
    default: break;
    }
    return launch_beamspace_warp(f, R_out, s);
}

// one warp per pixel: any Nb <= L
int launch_beamspace_warp(const FrameDev &f, float2 *R_out, cudaStream_t s)
{
    if (f.L > 64) return cudaErrorNotSupported;
    const BsSmem S(f.M, f.L, f.K, f.Nb);
    if (S.total > 227 * 1024) return cudaErrorNotSupported;
    cudaError_t e = cudaFuncSetAttribute(beamspace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S.total);
    if (e != cudaSuccess) return e;
    const long long npix = (long long)f.Nx * f.Npy;
    const long long blocks = (npix + kBsWarps - 1) / kBsWarps;
    beamspace_kernel<<<(unsigned)blocks, 32 * kBsWarps, S.total, s>>>(f, R_out);
    return cudaGetLastError();
}

__global__ void butler_kernel(float2 *B, int Nb, int L)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nb * L) return;
    const int bb = i / L, l = i % L;
    const int bin = butler_bin(bb, Nb, L);
    float sn, cs;
    sincospif(2.0f * (float)((bin * l) % L) / (float)L, &sn, &cs);
    const float isl = 1.0f / sqrtf((float)L);
    B[i] = make_float2(cs * isl, -sn * isl);
}

int launch_butler(float2 *B, int Nb, int L, cudaStream_t s)
{
    const int n = Nb * L;
    butler_kernel<<<(n + 127) / 128, 128, 0, s>>>(B, Nb, L);
    return cudaGetLastError();
}

}  // namespace cgb
