// FP64 <-> FP32 conversions for the FP32-split kernels (split3d.cu,
// batch2d_split.cu).
#pragma once

#include <cuda_runtime.h>

namespace mlau {

// FP64 <-> FP32 conversions run on the FP64 pipe, which on this part is the
// step's bottleneck; the helpers below do the common cases with integer bit
// operations (exact IEEE field arithmetic) and fall back to the native
// conversion for zero, tiny, huge and non-finite values.
// The native conversions run on the FP64 pipe; kept out of line so that the
// common integer paths below do not execute them predicated.
static __device__ __noinline__ float2 split2_native(double x)
{
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}
static __device__ __noinline__ float to_f32_native(double x) { return (float)x; }
static __device__ __noinline__ double to_f64_native(float f) { return (double)f; }

// x = hi + lo with hi the top 24 significand bits of x (truncated) and lo the
// remaining 29 bits rounded to FP32: |x - (hi + lo)| <= 2^-47 |x|.
__device__ __forceinline__ float2 split2(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 949 || e > 1150) {
        if ((b << 1) == 0) return make_float2(__uint_as_float((unsigned)(b >> 32)), 0.f);  // +-0
        return split2_native(x);
    }
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    const float hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | (unsigned)(m >> 29));
    // the low 29 bits carry weight 2^(e - 1075); that power of two is a normal float here
    const float lo = (float)(unsigned)(m & 0x1FFFFFFFu) * __uint_as_float((unsigned)(e - 948) << 23);
    return make_float2(hi, __uint_as_float(__float_as_uint(lo) | sign));
}

// FP64 -> FP32, truncating the significand (error below one FP32 ulp).
__device__ __forceinline__ float to_f32(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 897 || e > 1150) {
        if ((b << 1) == 0) return __uint_as_float((unsigned)(b >> 32));  // +-0
        return to_f32_native(x);
    }
    return __uint_as_float(((unsigned)(b >> 63) << 31) | ((unsigned)(e - 896) << 23) |
                           (unsigned)((b & 0xFFFFFFFFFFFFFull) >> 29));
}

// FP32 -> FP64, exact.
__device__ __forceinline__ double to_f64(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned ef = (u >> 23) & 0xff;
    if (ef == 0 || ef == 0xff) {
        if ((u << 1) == 0) return __longlong_as_double((long long)((unsigned long long)u << 32));  // +-0
        return to_f64_native(f);
    }
    const unsigned long long b = ((unsigned long long)(u >> 31) << 63) |
                                 ((unsigned long long)(ef + 896) << 52) |
                                 ((unsigned long long)(u & 0x7fffff) << 29);
    return __longlong_as_double((long long)b);
}

}  // namespace mlau
