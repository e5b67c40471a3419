// tb_f32x2.cuh -- FP32 arithmetic shared by the FP32 Chebyshev step kernels
// (staged, persistent, pipelined and batched): TwoSum pairs for the column dot
// products, and the 4x4-block product on a lane's two columns with the packed
// FP32x2 instructions of sm_100 and later (fma.rn.f32x2 / add.rn.f32x2).
// Each packed component is rounded exactly as the scalar fmaf / fadd, and the
// chains run in the scalar kernels' order, so packing changes no result bit.
#pragma once

#include <cuda_runtime.h>

namespace tb {

// (s, c) += x with the rounding error of s + x kept exactly in c (Knuth's
// TwoSum): column dot products accumulate as unevaluated FP32 pairs (hi, lo),
// since GB300 issues FP64 at only about 2 operations per clock per SM.
__device__ __forceinline__ void pair_add(float &s, float &c, float x)
{
    const float t = s + x;
    const float bp = t - s;
    const float e = (s - (t - bp)) + (x - bp);
    s = t;
    c += e;
}

// pair_add on both components of packed pairs; fma(-1, a, b) is b - a with
// the same single rounding
__device__ __forceinline__ void pair_add2(float2 &s, float2 &c, float2 x)
{
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 t = __fadd2_rn(s, x);
    const float2 bp = __ffma2_rn(m1, s, t);
    const float2 e = __fadd2_rn(__ffma2_rn(m1, __ffma2_rn(m1, bp, t), s), __ffma2_rn(m1, bp, x));
    s = t;
    c = __fadd2_rn(c, e);
}

// acc[q] += sum_m X[q][m] v[m] for one row-major 4x4 block (four float4 rows
// at xb) and rows m = 0..3 of a lane's two columns, v[m] = (T[m][c], T[m][c+1]):
// one fma.f32x2 per (q, m), chained in m order.
__device__ __forceinline__ void block_fma2(float2 (&acc)[4], const float4 *xb, const float2 (&v)[4])
{
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float4 xr = xb[q];
        acc[q] = __ffma2_rn(make_float2(xr.x, xr.x), v[0], acc[q]);
        acc[q] = __ffma2_rn(make_float2(xr.y, xr.y), v[1], acc[q]);
        acc[q] = __ffma2_rn(make_float2(xr.z, xr.z), v[2], acc[q]);
        acc[q] = __ffma2_rn(make_float2(xr.w, xr.w), v[3], acc[q]);
    }
}

// T_{k+1} = 2 acc - T_{k-1} on two columns: the doubling is exact, then
// fma(-1, p, 2 acc) rounds once
__device__ __forceinline__ float2 cheb_next2(float2 acc, float2 p)
{
    return __ffma2_rn(make_float2(-1.f, -1.f), p, __fadd2_rn(acc, acc));
}

}  // namespace tb
