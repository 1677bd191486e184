// Low-complexity adaptive (LCA) window selection for sm_103a.
//
// Follows framework/beamformer/lca/lcac.py (Z[Ny][Nx][Nw], the layout whose
// indexing is consistent; lcacx.pyx:175-216 is the same algorithm):
//   * wrf of size 1 x 1 with a nonzero value: per pixel the window of least
//     |Z| (argmin over w), for every pixel;
//   * otherwise, for interior pixels y in [Ymid, Ny-Ymid), x in [Xmid, Nx-Xmid):
//       s_w = sum_{yy,xx} |Z[y+yy-Ymid][x+xx-Xmid][w]|^2 wrf[yy][xx],
//     the first w of least s_w is selected; img = Z[y][x][w*], win = w*;
//     border pixels keep img = 0, win = 0.
// Two passes: |Z|^2 into planes [Nw][Ny][Nx] (coalesced along x), then one
// thread per pixel forms the Nw weighted sums (FP32) and the argmin.
#include "capon_common.cuh"
#include "capon_internal.h"
#include "../../include/cos_capon.h"

namespace cgb {

__global__ void lca_power_kernel(const float2 *__restrict__ Z, int Ny, int Nx, int Nw, float *__restrict__ pw)
{
    const long long n = (long long)Ny * Nx * Nw;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int w = (int)(i % Nw);
        const long long pix = i / Nw;   // y * Nx + x
        pw[(long long)w * Ny * Nx + pix] = cabs2(Z[i]);
    }
}

__global__ void lca_select_kernel(LcaDev a)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= a.Nx || y >= a.Ny) return;
    const long long pix = (long long)y * a.Nx + x;
    const long long plane = (long long)a.Ny * a.Nx;
    int best = 0;
    if (a.single) {
        float bv = 0.f;
        for (int w = 0; w < a.Nw; ++w) {
            const float v = a.pw[w * plane + pix];
            if (w == 0 || v < bv) {
                bv = v;
                best = w;
            }
        }
    } else {
        if (y < a.Ymid || y >= a.Ny - a.Ymid || x < a.Xmid || x >= a.Nx - a.Xmid) {
            a.img[pix] = make_float2(0.f, 0.f);
            if (a.win) a.win[pix] = 0;
            return;
        }
        float bv = 0.f;
        for (int w = 0; w < a.Nw; ++w) {
            const float *p = a.pw + w * plane;
            float s = 0.f;
            for (int yy = 0; yy < a.Yf; ++yy) {
                const float *row = p + (long long)(y + yy - a.Ymid) * a.Nx + (x - a.Xmid);
                for (int xx = 0; xx < a.Xf; ++xx) s = fmaf(row[xx], a.wrf[yy * a.Xf + xx], s);
            }
            if (w == 0 || s < bv) {
                bv = s;
                best = w;
            }
        }
    }
    a.img[pix] = a.Z[pix * a.Nw + best];
    if (a.win) a.win[pix] = best;
}

int launch_lca(const LcaDev &a, float *pw, cudaStream_t s)
{
    const long long n = (long long)a.Ny * a.Nx * a.Nw;
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    lca_power_kernel<<<(unsigned)blocks, 256, 0, s>>>(a.Z, a.Ny, a.Nx, a.Nw, pw);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    LcaDev b = a;
    b.pw = pw;
    dim3 grid((unsigned)((a.Nx + 127) / 128), (unsigned)a.Ny);
    lca_select_kernel<<<grid, 128, 0, s>>>(b);
    return cudaGetLastError();
}

}  // namespace cgb
