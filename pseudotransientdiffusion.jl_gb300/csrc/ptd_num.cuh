// ptd_num.cuh -- the two FP64-accuracy number types of the PT kernels.
//
// F64   native IEEE double: every operation on the FP64 pipe.
// DF64  double-float (float2 {hi, lo}, value hi + lo, |lo| <= ulp(hi)/2):
//       ~48-bit significand carried entirely on the FP32 pipe with
//       error-free transformations (Knuth two-sum, FMA two-product).
//
// GB300 executes FP64 at ~1/72 of its FP32 rate (measured: 0.50 T DFMA/s
// against 36.5 T FFMA/s), so a PT iteration done in native FP64 is bound by
// the FP64 pipe long before HBM.  A DF64 value occupies the same 8 bytes as a
// double, so the DF64 kernels move exactly the bytes of the FP64 kernels while
// running their arithmetic on the FP32 pipe.  The converged H agrees with the
// FP64 solution to ~1e-13 relative (parity bar 1e-10).
//
// Every DF64 primitive uses the explicitly rounded intrinsics (__fadd_rn,
// __fmul_rn, __fmaf_rn) so that the compiler cannot contract or reassociate
// the error-free transformations.
#pragma once

#include <cuda_runtime.h>

#include "ptd_device.cuh"

namespace ptd {

struct F64 {
    using T = double;      // register and storage type
    static constexpr bool native = true;
    __device__ static __forceinline__ T add(T a, T b) { return a + b; }
    __device__ static __forceinline__ T sub(T a, T b) { return a - b; }
    __device__ static __forceinline__ T mul(T a, T b) { return a * b; }
    __device__ static __forceinline__ T mad(T a, T b, T c) { return fma(a, b, c); }        // a*b + c
    __device__ static __forceinline__ T nmad(T a, T b, T c) { return fma(-a, b, c); }      // c - a*b
    // (the hardware f64<->f32 conversions issue on the FP64 pipe: use the
    // integer-pipe bit conversions of ptd_device.cuh instead)
    __device__ static __forceinline__ float lo_f(T a) { return d2f_bits(a); }
    __device__ static __forceinline__ double to_d(T a) { return a; }
    __device__ static __forceinline__ T zero() { return 0.0; }
    __device__ static __forceinline__ T shfl_down(T v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }
    __device__ static __forceinline__ T shfl_up(T v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
};

struct DF64 {
    using T = float2;      // {hi, lo}
    static constexpr bool native = false;

    __device__ static __forceinline__ T two_sum(float a, float b)
    {
        const float s = __fadd_rn(a, b);
        const float bb = __fsub_rn(s, a);
        const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
        return make_float2(s, e);
    }
    __device__ static __forceinline__ T fast_two_sum(float a, float b)
    {
        const float s = __fadd_rn(a, b);
        return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
    }
    __device__ static __forceinline__ T add(T a, T b)
    {
        const T s = two_sum(a.x, b.x);
        return fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
    }
    __device__ static __forceinline__ T neg(T a) { return make_float2(-a.x, -a.y); }
    __device__ static __forceinline__ T sub(T a, T b) { return add(a, neg(b)); }
    __device__ static __forceinline__ T mul(T a, T b)
    {
        const float p = __fmul_rn(a.x, b.x);
        float e = __fmaf_rn(a.x, b.x, -p);
        e = __fmaf_rn(a.x, b.y, e);
        e = __fmaf_rn(a.y, b.x, e);
        return fast_two_sum(p, e);
    }
    __device__ static __forceinline__ T mulf(T a, float c)
    {
        const float p = __fmul_rn(a.x, c);
        const float e = __fmaf_rn(a.y, c, __fmaf_rn(a.x, c, -p));
        return fast_two_sum(p, e);
    }
    __device__ static __forceinline__ T mad(T a, T b, T c) { return add(mul(a, b), c); }
    __device__ static __forceinline__ T nmad(T a, T b, T c) { return sub(c, mul(a, b)); }
    __device__ static __forceinline__ float lo_f(T a) { return a.x; }
    __device__ static __forceinline__ double to_d(T a) { return (double)a.x + (double)a.y; }
    __device__ static __forceinline__ T zero() { return make_float2(0.0f, 0.0f); }
    __device__ static __forceinline__ T shfl_down(T v, int d)
    {
        return make_float2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
    }
    __device__ static __forceinline__ T shfl_up(T v, int d)
    {
        return make_float2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
    }
};

// Split a double into a double-float (host or device).
__host__ __device__ __forceinline__ float2 split_df(double x)
{
    const float hi = (float)x;
    const float lo = (float)(x - (double)hi);
    return make_float2(hi, lo);
}

}  // namespace ptd
