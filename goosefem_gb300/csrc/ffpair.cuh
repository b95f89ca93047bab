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

// float -> double on the integer pipe: exact (as a conversion is) for normal floats and zeros;
// subnormals, infinities and NaN take the conversion instruction
__device__ __forceinline__ double ff_f32_to_f64(float f)
{
    const uint32_t u = __float_as_uint(f), ef = (u >> 23) & 0xffu;
    if (ef - 1u >= 254u) {
        if ((u & 0x7fffffffu) == 0u) return __hiloint2double(static_cast<int>(u & 0x80000000u), 0);
        return static_cast<double>(f);
    }
    const uint32_t hi = (u & 0x80000000u) | ((ef + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    return __hiloint2double(static_cast<int>(hi), static_cast<int>((u & 7u) << 29));
}

// double -> pair: h = rn(x), l = rn(x - h) (x - h is exact in FP64), with the bits of
// __double2float_rn. On GB300 the F64 <-> F32 conversions issue at the FP64 rate, so for
// 2^-74 <= |x| < 2^127 the split runs on the integer pipe: h is x's significand rounded to 24 bits
// (nearest, ties to even; a carry into the exponent is the correct rounding), and x - h is the
// signed integer (remainder - carry 2^29) times 2^(e - 1075), which one I2F rounds to 24 bits and
// a power-of-two scale places exactly (a normal float for e >= 949). Other x (0, tiny, huge,
// non-finite) take the conversion instructions. |x| within FP32 range.
__device__ __forceinline__ ffv ff_from_double(double x)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const uint32_t hi = static_cast<uint32_t>(b >> 32), e = (hi >> 20) & 0x7ffu;
    if (e - 949u > 200u) {
        const float h = __double2float_rn(x);
        return ff_make(h, __double2float_rn(x - static_cast<double>(h)));
    }
    const uint32_t top = static_cast<uint32_t>(b >> 29) & 0x7fffffu;
    const uint32_t r = static_cast<uint32_t>(b) & 0x1fffffffu;
    const uint32_t up = (r > 0x10000000u || (r == 0x10000000u && (top & 1u))) ? 1u : 0u;
    const uint32_t sign = hi & 0x80000000u;
    const float h = __uint_as_float(sign | (((e - 896u) << 23) + top + up));
    const int d = static_cast<int>(r) - static_cast<int>(up << 29);
    // the sign on the integer, so that x == h gives l = +0 as the FP64 subtraction does
    const float l = __fmul_rn(__int2float_rn(sign ? -d : d), __uint_as_float((e - 948u) << 23));
    return ff_make(h, l);
}

// pair -> double: rn(h + l), one FP64 addition of the two exactly converted parts
__device__ __forceinline__ double ff_to_double(ffv x)
{
    return ff_f32_to_f64(x.h) + ff_f32_to_f64(x.l);
}

} // namespace gfgpu
