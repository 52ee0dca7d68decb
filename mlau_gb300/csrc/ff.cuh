// Float-float arithmetic for the FP32-split kernels: a value is hi + lo with
// two FP32 numbers, |lo| at most about one ulp of hi, i.e. some 48
// significand bits.  Built from error-free transformations - Knuth's two-sum,
// Dekker's fast-two-sum and the FMA two-product (Dekker 1971; Shewchuk 1997;
// the "double-double" algorithms of Hida, Li and Bailey 2001 with FP32
// parts) - so it runs on the FP32 pipe, which on this part issues 64 times
// the FP64 rate.  Relative error per operation is a few times 2^-48.
//
// The translation unit must not reassociate FP32 additions (no fast-math);
// FMA contraction is harmless here (the products that matter are explicit
// fmaf calls).
#pragma once

#include <cuda_runtime.h>

#include "split_conv.cuh"

namespace mlau {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b)
{
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ ff ff_two_prod(float a, float b)
{
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ ff ff_add(ff x, ff y)
{
    ff s = ff_two_sum(x.hi, y.hi);
    const ff t = ff_two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = ff_fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return ff_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_neg(ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }

__device__ __forceinline__ ff ff_add_f(ff x, float b)
{
    ff s = ff_two_sum(x.hi, b);
    s.lo += x.lo;
    return ff_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_mul(ff x, ff y)
{
    ff p = ff_two_prod(x.hi, y.hi);
    p.lo = fmaf(x.hi, y.lo, p.lo);
    p.lo = fmaf(x.lo, y.hi, p.lo);
    return ff_fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ ff ff_mul_f(ff x, float b)
{
    ff p = ff_two_prod(x.hi, b);
    p.lo = fmaf(x.lo, b, p.lo);
    return ff_fast_two_sum(p.hi, p.lo);
}

// times a power of two: exact
__device__ __forceinline__ ff ff_scale(ff x, float p2) { return {x.hi * p2, x.lo * p2}; }

__device__ __forceinline__ ff ff_sqr(ff x)
{
    ff p = ff_two_prod(x.hi, x.hi);
    p.lo = fmaf(2.0f * x.hi, x.lo, p.lo);
    return ff_fast_two_sum(p.hi, p.lo);
}

// FP64 <-> float-float: split2 (integer field operations) and one FP64 add
// (exact for the usual exponent spread of hi and lo).
__device__ __forceinline__ ff ff_from(double x)
{
    const float2 p = split2(x);
    return {p.x, p.y};
}
__device__ __forceinline__ double ff_to_double(ff x) { return to_f64(x.hi) + to_f64(x.lo); }
__device__ __forceinline__ float2 ff_pair(ff x) { return make_float2(x.hi, x.lo); }

}  // namespace mlau
