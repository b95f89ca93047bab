// Float-float pairs of two lanes at once, on the packed FP32x2 instructions of sm_100+
// (add/sub/fma.rn.f32x2: one instruction, two independent FP32 results).
//
// An ff2 holds two pair values (lane 0 and lane 1, e.g. the x and y components of a node):
// h = {h0, h1} and l = {l0, l1}, each a 64-bit register of two FP32 numbers. The operations are
// those of ffpair.cuh (Knuth's TwoSum and Dekker's TwoDiff for sums, the FMA product error for
// products, Fast2Sum for renormalisation) applied lane-wise, so each lane's bits equal what the
// scalar functions of ffpair.cuh give for that lane. There is no f32x2 negation: the product error
// fma(a, b, -ab) takes -ab from a subtraction from zero (exact).
//
// The products take their high part from an FMA with an addend of -0 that the kernel reads at run
// time (a kernel parameter), p = fma(a, b, -0) = rn(a b), not from mul.rn.f32x2. With the
// multiply, ptxas rewrites the sequence mul / fma(a, b, -p) / TwoSum of p (measured on sm_103a:
// every packed result then differs from the scalar one at the 2^-24 level, whatever -fmad,
// volatile asm or the optimisation level); with an FMA whose addend it cannot fold, the packed
// results equal the scalar ones bit for bit. The addend is -0 rather than +0 so that a product
// of -0 keeps its sign, as rn(a b) does.
#pragma once

#include <cuda_runtime.h>

#include "ffpair.cuh"

namespace gfgpu {

typedef unsigned long long f2; // two FP32 lanes: lane 0 in the low 32 bits

__device__ __forceinline__ f2 f2_make(float a, float b)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}

__device__ __forceinline__ float f2_lo(f2 v)
{
    float a;
    asm("{\n .reg .b32 lo, hi;\n mov.b64 {lo, hi}, %1;\n mov.b32 %0, lo;\n}" : "=f"(a) : "l"(v));
    return a;
}

__device__ __forceinline__ float f2_hi(f2 v)
{
    float b;
    asm("{\n .reg .b32 lo, hi;\n mov.b64 {lo, hi}, %1;\n mov.b32 %0, hi;\n}" : "=f"(b) : "l"(v));
    return b;
}

__device__ __forceinline__ f2 f2_add(f2 a, f2 b)
{
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ f2 f2_sub(f2 a, f2 b)
{
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c)
{
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

struct ff2 {
    f2 h, l;
};

__device__ __forceinline__ ff2 ff2_make(f2 h, f2 l)
{
    ff2 r;
    r.h = h;
    r.l = l;
    return r;
}

// the pair lanes (x, y) -> ff2 and back
__device__ __forceinline__ ff2 ff2_from(ffv x, ffv y)
{
    return ff2_make(f2_make(x.h, y.h), f2_make(x.l, y.l));
}

__device__ __forceinline__ ffv ff2_lane0(ff2 v)
{
    return ff_make(f2_lo(v.h), f2_lo(v.l));
}

__device__ __forceinline__ ffv ff2_lane1(ff2 v)
{
    return ff_make(f2_hi(v.h), f2_hi(v.l));
}

// the same scalar pair in both lanes
__device__ __forceinline__ ff2 ff2_bcast(ffv x)
{
    return ff2_make(f2_make(x.h, x.h), f2_make(x.l, x.l));
}

// x + y: TwoSum on the high parts, the low parts folded in (unnormalised; 8 instructions)
__device__ __forceinline__ ff2 ff2_add(ff2 x, ff2 y)
{
    const f2 s = f2_add(x.h, y.h);
    const f2 bb = f2_sub(s, x.h);
    const f2 e = f2_add(f2_sub(x.h, f2_sub(s, bb)), f2_sub(y.h, bb));
    return ff2_make(s, f2_add(e, f2_add(x.l, y.l)));
}

// x - y: TwoDiff on the high parts (unnormalised; 8 instructions)
__device__ __forceinline__ ff2 ff2_sub(ff2 x, ff2 y)
{
    const f2 s = f2_sub(x.h, y.h);
    const f2 bb = f2_sub(s, x.h);
    const f2 e = f2_sub(f2_sub(x.h, f2_sub(s, bb)), f2_add(y.h, bb));
    return ff2_make(s, f2_add(e, f2_sub(x.l, y.l)));
}

// -0 in both lanes, the addend of ff2_mul's high product; pass it in from a kernel parameter
constexpr unsigned long long kF2NegZero = 0x8000000080000000ull;

// x * y: exact product of the high parts plus the cross terms (unnormalised; 5 instructions).
// nz: kF2NegZero, read at run time (see the note at the top)
__device__ __forceinline__ ff2 ff2_mul(ff2 x, ff2 y, f2 nz)
{
    const f2 p = f2_fma(x.h, y.h, nz);
    f2 e = f2_fma(x.h, y.h, f2_sub(0ull, p));
    e = f2_fma(x.h, y.l, e);
    e = f2_fma(x.l, y.h, e);
    return ff2_make(p, e);
}

// Fast2Sum renormalisation (3 instructions)
__device__ __forceinline__ ff2 ff2_norm(ff2 x)
{
    const f2 s = f2_add(x.h, x.l);
    return ff2_make(s, f2_sub(x.l, f2_sub(s, x.h)));
}

// -x (exact)
__device__ __forceinline__ ff2 ff2_neg(ff2 x)
{
    return ff2_make(f2_sub(0ull, x.h), f2_sub(0ull, x.l));
}

} // namespace gfgpu
