// Float-float ("pair") arithmetic for the FP32 pipes.
//
// A value is the unevaluated sum h + l of two FP32 numbers (about 48 significant bits). On GB300
// the FP64 pipe issues about 1.7 operations per SM and clock against 128 for FP32, so a kernel
// whose FP64 form is bound by the FP64 issue rate can run its arithmetic on pairs instead.
//
// Building blocks (published error-free transformations):
//  * two_sum: Knuth's TwoSum (The Art of Computer Programming vol. 2, 4.2.2), s + e = a + b
//    exactly, any a, b;
//  * the exact product error of an FMA, e = fma(a, b, -ab) (a * b = p + e exactly);
//  * quick_two_sum: Dekker's Fast2Sum (1971), exact when |a| >= |b| or a = 0.
// The pair add and multiply are the "sloppy" double-float forms of Dekker (1971) and of
// Hida, Li and Bailey's QD library (2001): the high parts are added (multiplied) exactly and the
// low parts folded into the error term. They return the pair UNNORMALISED (|l| may exceed half
// an ulp of h); ff_norm restores the canonical form with Fast2Sum. Errors are bounded by a few
// units of 2^-48 of the operands' magnitudes, like an FP64 sum's 2^-53.
// Every operation uses the _rn intrinsics, so the compiler neither contracts nor reassociates.
#pragma once

#include <cuda_runtime.h>

namespace gfgpu {

struct ffv {
    float h, l;
};

__device__ __forceinline__ ffv ff_make(float h, float l)
{
    ffv r;
    r.h = h;
    r.l = l;
    return r;
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ ffv ff_add(ffv x, ffv y)
{
    float s, e;
    two_sum(x.h, y.h, s, e);
    return ff_make(s, __fadd_rn(e, __fadd_rn(x.l, y.l)));
}

__device__ __forceinline__ ffv ff_neg(ffv x)
{
    return ff_make(-x.h, -x.l);
}

__device__ __forceinline__ ffv ff_sub(ffv x, ffv y)
{
    return ff_add(x, ff_neg(y));
}

__device__ __forceinline__ ffv ff_mul(ffv x, ffv y)
{
    const float p = __fmul_rn(x.h, y.h);
    float e = __fmaf_rn(x.h, y.h, -p);
    e = __fmaf_rn(x.h, y.l, e);
    e = __fmaf_rn(x.l, y.h, e);
    return ff_make(p, e);
}

// 2 x (exact)
__device__ __forceinline__ ffv ff_twice(ffv x)
{
    return ff_make(__fmul_rn(2.0f, x.h), __fmul_rn(2.0f, x.l));
}

// canonical pair (|l| <= ulp(h) / 2) by Fast2Sum
__device__ __forceinline__ ffv ff_norm(ffv x)
{
    const float s = __fadd_rn(x.h, x.l);
    return ff_make(s, __fsub_rn(x.l, __fsub_rn(s, x.h)));
}

// double -> pair: h = rn(x), l = rn(x - h) (x - h is exact in FP64); |x| within FP32 range
__device__ __forceinline__ ffv ff_from_double(double x)
{
    const float h = __double2float_rn(x);
    return ff_make(h, __double2float_rn(x - static_cast<double>(h)));
}

__device__ __forceinline__ double ff_to_double(ffv x)
{
    return static_cast<double>(x.h) + static_cast<double>(x.l);
}

} // namespace gfgpu
