// Device helpers shared by the Capon/MVDR kernels (sm_103a).
//
// Complex numbers are interleaved float2 {re, im}, the layout of the
// reference's Complex<float> / cuComplex (framework/lib/Complex.h:12-166).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define COS_DEV __device__ __forceinline__

namespace cgb {

// ---- scalar complex ------------------------------------------------------
COS_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
COS_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
COS_DEV float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
COS_DEV float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
COS_DEV float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// a * conj(b)
COS_DEV float2 cmulc(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
// conj(a) * b
COS_DEV float2 cconjmul(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }
COS_DEV float cabs2(float2 a) { return a.x * a.x + a.y * a.y; }
// acc + a b and acc + conj(a) b as four fmas each (cadd of a cmul costs six:
// the compiler may not fuse the add into the products)
COS_DEV float2 cmac4(float2 acc, float2 a, float2 b)
{
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(-a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(a.y, b.x, acc.y);
    return acc;
}
COS_DEV float2 cmac4_conj(float2 acc, float2 a, float2 b)
{
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(-a.y, b.x, acc.y);
    return acc;
}

// ---- packed FP32x2 (Blackwell `fma.rn.f32x2`): two IEEE fmas per instruction
COS_DEV float2 ffma2(float2 a, float2 b, float2 c)
{
    uint64_t ra = *reinterpret_cast<uint64_t*>(&a);
    uint64_t rb = *reinterpret_cast<uint64_t*>(&b);
    uint64_t rc = *reinterpret_cast<uint64_t*>(&c);
    uint64_t rd;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
    return *reinterpret_cast<float2*>(&rd);
}
COS_DEV float2 fadd2(float2 a, float2 b)
{
    uint64_t ra = *reinterpret_cast<uint64_t*>(&a);
    uint64_t rb = *reinterpret_cast<uint64_t*>(&b);
    uint64_t rd;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    return *reinterpret_cast<float2*>(&rd);
}
COS_DEV float2 fsub2(float2 a, float2 b)
{
    uint64_t ra = *reinterpret_cast<uint64_t*>(&a);
    uint64_t rb = *reinterpret_cast<uint64_t*>(&b);
    uint64_t rd;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    return *reinterpret_cast<float2*>(&rd);
}

// acc += x * conj(y), with the y-dependent operands prepared once:
//   yrr = (y.re, y.re), yii = (y.im, y.im)
//   acc.re += x.re*y.re + x.im*y.im ; acc.im += x.im*y.re - x.re*y.im
COS_DEV float2 cmac_xyc(float2 acc, float2 x, float2 yrr, float2 yii)
{
    acc = ffma2(x, yrr, acc);
    return ffma2(make_float2(x.y, -x.x), yii, acc);
}

// acc -= conj(u) * v, with the u-dependent operands prepared once:
//   nu1 = (-u.re, -u.re), nu2 = (-u.im, u.im)
//   acc.re -= u.re*v.re + u.im*v.im ; acc.im -= u.re*v.im - u.im*v.re
COS_DEV float2 cnmac_conj(float2 acc, float2 nu1, float2 nu2, float2 v)
{
    acc = ffma2(nu1, v, acc);
    return ffma2(nu2, make_float2(v.y, v.x), acc);
}

// float-float accumulation of complex values: (hi, lo) += v exactly up to the
// rounding of lo (Knuth's TwoSum on both components, packed).
COS_DEV void two_sum_acc(float2 &hi, float2 &lo, float2 v)
{
    const float2 s = fadd2(hi, v);
    const float2 bb = fsub2(s, hi);
    const float2 e = fadd2(fsub2(hi, fsub2(s, bb)), fsub2(v, bb));
    hi = s;
    lo = fadd2(lo, e);
}

// ---- warp helpers ---------------------------------------------------------
COS_DEV float2 shfl2(float2 v, int src, int width)
{
    return make_float2(__shfl_sync(0xffffffffu, v.x, src, width),
                       __shfl_sync(0xffffffffu, v.y, src, width));
}
COS_DEV float2 shfl2_xor(float2 v, int mask, int width)
{
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, mask, width),
                       __shfl_xor_sync(0xffffffffu, v.y, mask, width));
}

// DFT bin of Butler beam b for subarray length L: beams b <= Nb/2 take bin b,
// the others the negative bins b + L - 2*(Nb/2) - 1
// (reference RealTimeCapon/capon_kernel.cu:53-59).
COS_DEV int butler_bin(int b, int Nb, int L) { return (b > Nb / 2) ? b + (L - 2 * (Nb / 2) - 1) : b; }

}  // namespace cgb
