// dfloat.cuh -- double-float (unevaluated sum of two FP32 values) arithmetic.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the FP64
// residual of the refinement loop is evaluated with FP32 error-free
// transformations instead: Knuth's TwoSum, Dekker's FastTwoSum and the FMA
// form of TwoProd.  A df value carries about 48 significand bits, which keeps
// ||b - A phi|| accurate far below the 1e-8 * ||b|| refinement target.
#pragma once
#include <cuda_runtime.h>

namespace cmsl {

struct df {
    float h, l;
};

__host__ __device__ __forceinline__ df df_make(float h, float l = 0.f) { return df{h, l}; }

// |a| >= |b| not required (Knuth TwoSum)
__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return df{s, e};
}

// requires |a| >= |b| or a == 0 (Dekker FastTwoSum)
__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    const float s = a + b;
    return df{s, b - (s - a)};
}

__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = a * b;
    return df{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ df df_add(df a, df b)
{
    df s = two_sum(a.h, b.h);
    s.l += a.l + b.l;
    return fast_two_sum(s.h, s.l);
}

// Accurate double-float sum (both halves through TwoSum; the "IEEE" add of
// Hida, Li and Bailey's QD library), for sums whose terms may cancel.
__device__ __forceinline__ df df_add_acc(df a, df b)
{
    df s = two_sum(a.h, b.h);
    const df t = two_sum(a.l, b.l);
    s.l += t.h;
    s = fast_two_sum(s.h, s.l);
    s.l += t.l;
    return fast_two_sum(s.h, s.l);
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.h, -a.l}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df df_add_f(df a, float b)
{
    df s = two_sum(a.h, b);
    s.l += a.l;
    return fast_two_sum(s.h, s.l);
}

__device__ __forceinline__ df df_mul_f(df a, float b)
{
    df p = two_prod(a.h, b);
    p.l = fmaf(a.l, b, p.l);
    return fast_two_sum(p.h, p.l);
}

__device__ __forceinline__ df df_mul(df a, df b)
{
    df p = two_prod(a.h, b.h);
    p.l = fmaf(a.h, b.l, fmaf(a.l, b.h, p.l));
    return fast_two_sum(p.h, p.l);
}

// Host split of a double into a df pair.
__host__ __forceinline__ df df_from_double(double x)
{
    const float h = (float)x;
    return df{h, (float)(x - (double)h)};
}

}  // namespace cmsl
