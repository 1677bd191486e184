// Time-domain steering (TDIB) for sm_103a: the step before the Capon path.
//
// Follows framework/beamformer/delay/tdibC.pyx:9-67: for beam nx, range pixel
// y and hydrophone n, with the transmitter/receiver origin at
// (xx, zz) = (mean(x_r)/2, mean(D)/2),
//     r_t   = sqrt((xx + X)^2 + Y^2 + zz^2)
//     r_r   = sqrt((xx + X - x_r[n])^2 + Y^2 + (zz - D[n])^2)
//     tau   = (r_t + r_r) / c
//     Xd    = interp_linear(mfdata[n], tau) * exp(j 2 pi fc tau)
// (NaN outside the time axis, as scipy's interp1d with bounds_error=False),
// and the delay-and-sum image is the mean of Xd over hydrophones.  The
// steered cube Xd[nx][y][n] is the Capon path's input layout.
//
// The carrier needs the delay to ~1e-9 relative, beyond FP32; GB300's FP64
// rate is a small fraction of its FP32 rate.  So FP64 is spent once per pixel
// (the base delay and phase) and the per-hydrophone terms are FP32 corrections
// of a few samples / cycles (see tdib_kernel).  Measured against the FP64
// restatement: ~2e-6 of the cube's scale.
#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {

static constexpr int kTdibMaxChunks = 8;   // hydrophones per lane: n_hydros <= 256

// A warp takes 32 consecutive range pixels of one beam.  Lane l evaluates the
// FP64 part of pixel y0+l once: r_t, the base delay 2 r_t / c split into an
// integer sample index and a fraction, and the base carrier phase fc 2 r_t / c
// reduced to a fraction of a cycle.  Per hydrophone only the small difference
// d = r_r - r_t is needed; it is formed in FP32 without cancellation,
//     e = r_r^2 - r_t^2 = c_n - 2 ax x_n,   c_n = x_n^2 + D_n^2 - 2 zz D_n
//     d = e / (r_t + sqrt(r_t^2 + e)),
// and enters the sample index as d/(c dt) and the phase as fc d/c (a few
// samples / cycles, so FP32 keeps ~1e-6 of a cycle).
__global__ void __launch_bounds__(256, 4) tdib_kernel(TdibDev t)
{
    const int lane = threadIdx.x & 31;
    const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int runs = (t.n_y + 31) / 32;
    if (wid >= (long long)t.n_x * runs) return;
    const int nx = (int)(wid / runs), y0 = (int)(wid % runs) * 32;
    // origin: half the mean receiver position and depth (the same
    // lane-strided sums and butterfly in every warp)
    double sx = 0.0, sz = 0.0;
    for (int n = lane; n < t.n_hydros; n += 32) {
        sx += t.x_r[n];
        sz += t.D[n];
    }
    for (int o = 16; o; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    const double xx = 0.5 * sx / (double)t.n_hydros, zz = 0.5 * sz / (double)t.n_hydros;
    // per-lane receiver constants
    float xn[kTdibMaxChunks], cn[kTdibMaxChunks];
#pragma unroll
    for (int k = 0; k < kTdibMaxChunks; ++k) {
        const int n = lane + 32 * k;
        xn[k] = cn[k] = 0.f;
        if (n < t.n_hydros) {
            const double x = t.x_r[n], dd = t.D[n];
            xn[k] = (float)x;
            cn[k] = (float)(x * x + dd * (dd - 2.0 * zz));
        }
    }
    // this lane's pixel: FP64 base terms
    const int yl = y0 + lane;
    float ax_f = 0.f, rt_f = 0.f, rt2_f = 0.f, bfrac = 0.f, bcyc = 0.f;
    int bi = 0;
    if (yl < t.n_y) {
        const double X = t.xarr[(size_t)nx * t.n_y + yl], Y = t.yarr[(size_t)nx * t.n_y + yl];
        const double ax = xx + X, rt2 = ax * ax + Y * Y + zz * zz, rt = sqrt(rt2);
        const double tau0 = 2.0 * rt * t.inv_c;
        const double u0 = (tau0 - t.t0) / t.dt;
        const double fu = floor(u0);
        const double cyc = t.fc * tau0;
        bi = (int)fu;
        bfrac = (float)(u0 - fu);
        bcyc = (float)(cyc - floor(cyc));
        ax_f = (float)ax;
        rt_f = (float)rt;
        rt2_f = (float)rt2;
    }
    const float ku = (float)(t.inv_c / t.dt), kc = (float)(t.fc * t.inv_c);
    const float qnan = __int_as_float(0x7fc00000);
    const int np = min(32, t.n_y - y0);
    // four pixels per iteration: more channel-data gathers in flight
#pragma unroll 4
    for (int p = 0; p < np; ++p) {
        const float a = __shfl_sync(0xffffffffu, ax_f, p), r = __shfl_sync(0xffffffffu, rt_f, p);
        const float r2 = __shfl_sync(0xffffffffu, rt2_f, p), fr = __shfl_sync(0xffffffffu, bfrac, p);
        const float bc = __shfl_sync(0xffffffffu, bcyc, p);
        const int b = __shfl_sync(0xffffffffu, bi, p);
        float2 acc = make_float2(0.f, 0.f);
        float2 *out = t.Xd ? t.Xd + ((size_t)nx * t.n_y + (y0 + p)) * t.n_hydros : nullptr;
#pragma unroll
        for (int k = 0; k < kTdibMaxChunks; ++k) {
            const int n = lane + 32 * k;
            if (n >= t.n_hydros) break;
            const float e = cn[k] - 2.f * a * xn[k];
            const float d = e / (r + sqrtf(r2 + e));
            const float uf = fr + d * ku;
            const float fl = floorf(uf);
            const long long il = (long long)b + (long long)fl;   // b saturates for far-away delays
            float2 v;
            if (il < 0 || il > t.n_samples - 1 || (il == t.n_samples - 1 && uf > fl)) {
                v = make_float2(qnan, qnan);   // outside the time axis
            } else {
                const int i = (int)il;
                const float wgt = uf - fl;
                const float2 *row = t.mf + (size_t)n * t.n_samples;
                const float2 lo = row[i], hi = row[i < t.n_samples - 1 ? i + 1 : i];
                const float2 sm = make_float2(lo.x + wgt * (hi.x - lo.x), lo.y + wgt * (hi.y - lo.y));
                float c = bc + d * kc;
                c -= floorf(c);
                float sn, cs;
                sincospif(2.0f * c, &sn, &cs);
                v = cmul(sm, make_float2(cs, sn));
            }
            if (out) out[n] = v;
            acc = cadd(acc, v);
        }
        if (t.image) {
            for (int o = 16; o; o >>= 1) acc = cadd(acc, shfl2_xor(acc, o, 32));
            if (lane == 0) t.image[(size_t)(y0 + p) * t.n_x + nx] = cscale(acc, 1.0f / (float)t.n_hydros);
        }
    }
}

int launch_tdib(const TdibDev &t, cudaStream_t s)
{
    if (t.n_hydros > 32 * kTdibMaxChunks) return cudaErrorNotSupported;
    const long long warps = (long long)t.n_x * ((t.n_y + 31) / 32);
    const long long blocks = (warps * 32 + 255) / 256;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    tdib_kernel<<<(unsigned)blocks, 256, 0, s>>>(t);
    return cudaGetLastError();
}

}  // namespace cgb
