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

// Conversions between FP64 and pairs on the integer pipe, branch-free. On GB300 the F64 <-> F32
// conversion instructions issue at the FP64 rate, and a fallback to them for rare operands is no
// cure: inlined behind a per-lane condition it is if-converted into predicated FP64 instructions
// that issue for every operand (measured: the pipe 82 % busy in a kernel with 8 FP64 additions per
// element), as a call it stops the loads of later grid-stride iterations from being scheduled
// ahead, and behind a warp vote it costs a vote per conversion. So the rare operands are handled by
// selects, with the domain stated below.

// float -> double: exact (as the conversion is) for normal floats, zeros and infinities; NaN stays
// NaN; subnormal floats (|f| < 2^-126) give +-0
__device__ __forceinline__ double ff_f32_to_f64(float f)
{
    const uint32_t u = __float_as_uint(f), ef = (u >> 23) & 0xffu;
    const uint32_t eh = ef == 0u ? 0u : (ef == 255u ? 0x7ffu : ef + 896u);
    const uint32_t m = ef == 0u ? 0u : (u & 0x7fffffu);
    const uint32_t hi = (u & 0x80000000u) | (eh << 20) | (m >> 3);
    return __hiloint2double(static_cast<int>(hi), static_cast<int>((m & 7u) << 29));
}

// double -> pair: h = rn(x), l = rn(x - h) (x - h is exact in FP64), the bits of
// __double2float_rn, for zeros and 2^-74 <= |x| < 2^128 (where h does not round up to infinity):
// h is x's significand rounded to 24 bits (nearest, ties to even; a carry into the exponent is the
// correct rounding), and x - h is the signed integer (remainder - carry 2^29) times 2^(e - 1075),
// which one I2F rounds to 24 bits and a power-of-two scale places exactly (a normal float for
// e >= 949). +-0 gives (+-0, +0). Below 2^-74, h = rn(x) and l = 0 (below 2^-126, h = +-0): a
// relative error of 2^-24 there, far below 2^-48 of any value of 2^-26 or more in the same vector.
// |x| >= 2^128 gives (+-inf, 0), NaN gives (NaN, 0).
__device__ __forceinline__ ffv ff_from_double(double x)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const uint32_t hi = static_cast<uint32_t>(b >> 32), e = (hi >> 20) & 0x7ffu;
    const uint32_t sign = hi & 0x80000000u;
    const uint32_t top = static_cast<uint32_t>(b >> 29) & 0x7fffffu;
    const uint32_t r = static_cast<uint32_t>(b) & 0x1fffffffu;
    const uint32_t up = (r > 0x10000000u || (r == 0x10000000u && (top & 1u))) ? 1u : 0u;
    const int d = static_cast<int>(r) - static_cast<int>(up << 29);
    uint32_t hb = sign | (((e - 896u) << 23) + top + up);
    // the sign on the integer, so that x == h gives l = +0 as the FP64 subtraction does
    float l = __fmul_rn(__int2float_rn(sign ? -d : d), __uint_as_float(((e - 948u) & 0xffu) << 23));
    if (e < 949u) l = 0.0f;
    if (e < 897u) hb = sign;
    if (e > 1150u) {
        hb = (e == 0x7ffu && (b << 12) != 0ull) ? 0x7fffffffu : (sign | 0x7f800000u);
        l = 0.0f;
    }
    return ff_make(__uint_as_float(hb), l);
}

// pair -> double: rn(h + l), one FP64 addition of the two exactly converted parts
__device__ __forceinline__ double ff_to_double(ffv x)
{
    return ff_f32_to_f64(x.h) + ff_f32_to_f64(x.l);
}

} // namespace gfgpu
