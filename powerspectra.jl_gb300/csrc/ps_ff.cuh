// ps_ff.cuh -- two-word FP32 ("float-float") arithmetic for the chosen kernel.
//
// A value is the unevaluated sum h + l of two floats with |l| <= ulp(h)/2 after
// normalisation, which carries ~48 significant bits on the FP32 pipe.  The
// error-free building blocks are the classical ones:
//   two_prod (Dekker 1971, with an FMA):   a*b = p + e exactly
//   fast_two_sum (Dekker 1971):            a+b = s + e exactly when |a| >= |b|
//   two_sum (Knuth, TAOCP vol. 2):         a+b = s + e exactly
// Every primitive uses the __f*_rn intrinsics, which the compiler never
// contracts or reassociates, so the error terms stay exact.
#pragma once

namespace ps {

struct ff {
    float h, l;
};

__device__ __forceinline__ ff ff_make(float h) { return ff{h, 0.0f}; }

__device__ __forceinline__ ff fast_two_sum(float a, float b)
{
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return ff{s, e};
}

// a + b = s + e exactly, for any a and b (Knuth)
__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ ff two_prod(float a, float b)
{
    float p = __fmul_rn(a, b);
    return ff{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ ff ff_neg(ff x) { return ff{-x.h, -x.l}; }

// x * y, normalised (~2^-46 relative)
__device__ __forceinline__ ff ff_mul(ff x, ff y)
{
    float p = __fmul_rn(x.h, y.h);
    float e = __fmaf_rn(x.h, y.h, -p);
    e = __fmaf_rn(x.h, y.l, e);
    e = __fmaf_rn(x.l, y.h, e);
    return fast_two_sum(p, e);
}

// x * y with a float y
__device__ __forceinline__ ff ff_mulf(ff x, float y)
{
    float p = __fmul_rn(x.h, y);
    float e = __fmaf_rn(x.h, y, -p);
    e = __fmaf_rn(x.l, y, e);
    return fast_two_sum(p, e);
}

// x + y (Knuth two_sum on the high words, low words added to the error)
__device__ __forceinline__ ff ff_add(ff x, ff y)
{
    float s = __fadd_rn(x.h, y.h);
    float bb = __fsub_rn(s, x.h);
    float e = __fadd_rn(__fsub_rn(x.h, __fsub_rn(s, bb)), __fsub_rn(y.h, bb));
    e = __fadd_rn(e, __fadd_rn(x.l, y.l));
    return fast_two_sum(s, e);
}

// Product of two exactly representable float-float integers, left unnormalised
// (the low word may reach a few ulp of the high word); used only as the input
// of ff_rsqrt and ff_mul.
__device__ __forceinline__ ff ff_mul_raw(ff x, ff y)
{
    float p = __fmul_rn(x.h, y.h);
    float e = __fmaf_rn(x.h, y.h, -p);
    e = __fmaf_rn(x.h, y.l, e);
    e = __fmaf_rn(x.l, y.h, e);
    return ff{p, e};
}

// x * y for a float y, left unnormalised
__device__ __forceinline__ ff ff_mulf_raw(ff x, float y)
{
    float p = __fmul_rn(x.h, y);
    return ff{p, __fmaf_rn(x.l, y, __fmaf_rn(x.h, y, -p))};
}

// x + y left unnormalised: the Knuth two_sum of the high words with the low
// words added to its error term (the renormalising fast_two_sum is skipped).
// Products and this sum accept unnormalised inputs; after a cancelling sum the
// low word may exceed ulp(h), so a consumer that needs the value as one float
// must round h + l rather than take h.
__device__ __forceinline__ ff ff_add_raw(ff x, ff y)
{
    float s = __fadd_rn(x.h, y.h);
    float bb = __fsub_rn(s, x.h);
    float e = __fadd_rn(__fsub_rn(x.h, __fsub_rn(s, bb)), __fsub_rn(y.h, bb));
    return ff{s, __fadd_rn(e, __fadd_rn(x.l, y.l))};
}

// 1/sqrt(P): hardware FP32 estimate, then one Newton-Raphson step
// y' = y + y (1 - P y^2) / 2 whose residual 1 - P y^2 is formed with FMAs
// from the exact square of y, which doubles the ~22 correct bits.
__device__ __forceinline__ ff ff_rsqrt(ff P)
{
    float y = rsqrtf(P.h);
    ff q = two_prod(y, y);
    float r = __fmaf_rn(-P.h, q.h, 1.0f);
    r = __fmaf_rn(-P.h, q.l, r);
    r = __fmaf_rn(-P.l, q.h, r);
    float c = __fmul_rn(__fmul_rn(0.5f, y), r);
    return fast_two_sum(y, c);
}

__device__ __forceinline__ double ff_to_double(ff x) { return (double)x.h + (double)x.l; }

}  // namespace ps
