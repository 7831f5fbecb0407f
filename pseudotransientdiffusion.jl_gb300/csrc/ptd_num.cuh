// ptd_num.cuh -- the FP64-accuracy number types of the PT kernels.
//
// F64   native IEEE double: every operation on the FP64 pipe.
// DF64  double-float (float2 {hi, lo}, value hi + lo, |lo| <= ulp(hi)/2):
//       ~48-bit significand carried entirely on the FP32 pipe with
//       error-free transformations (Knuth two-sum, FMA two-product).
// DFH   DF64 arithmetic on an FP64 state: H and Hold are IEEE doubles, the
//       fluxes and D double-floats.  Only the operations that need H's full
//       53 bits run on the FP64 pipe (below).
//
// GB300 executes FP64 at ~1/58 of its FP32 rate (measured: 0.627 T DFMA/s
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
    // the H interface (see DFH): H values are plain T here
    using HV = T;
    using HS = T;
    __device__ static __forceinline__ HV ldh(const void* p, long long i) { return static_cast<const T*>(p)[i]; }
    __device__ static __forceinline__ HS ldo(const void* p, long long i) { return static_cast<const T*>(p)[i]; }
    __device__ static __forceinline__ void sth(void* p, long long i, HS v) { static_cast<T*>(p)[i] = v; }
    __device__ static __forceinline__ float hf(HV h) { return d2f_bits(h); }
    __device__ static __forceinline__ HV shfl_down_h(HV v, int d) { return shfl_down(v, d); }
    __device__ static __forceinline__ T hdiff(HV r, HV l) { return r - l; }
    __device__ static __forceinline__ T hsum(HV l, HV r) { return l + r; }
    __device__ static __forceinline__ T hdo(HV h, HS o) { return h - o; }
    __device__ static __forceinline__ T hdn(HS h, HS o) { return h - o; }
    __device__ static __forceinline__ HS hstep(HV h, T rp, float e) { return fma(-f2d_bits(e), rp, h); }
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
    // a*b + c: the exact-product pair (p, e) of a.x*b.x, plus the cross
    // terms, summed into c with one normalisation (15 FP32 operations instead
    // of 18 for add(mul(a, b), c); same error bound)
    __device__ static __forceinline__ T mad(T a, T b, T c)
    {
        const float p = __fmul_rn(a.x, b.x);
        float e = __fmaf_rn(a.x, b.x, -p);
        e = __fmaf_rn(a.x, b.y, e);
        e = __fmaf_rn(a.y, b.x, e);
        const T s = two_sum(p, c.x);
        return fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(e, c.y)));
    }
    __device__ static __forceinline__ T nmad(T a, T b, T c) { return sub(c, mul(a, b)); }
    // w - c*t with a float c, one normalisation (14 operations instead of 19)
    __device__ static __forceinline__ T nmadf(T t, float c, T w)
    {
        const float p = __fmul_rn(t.x, c);
        const float e = __fmaf_rn(t.y, c, __fmaf_rn(t.x, c, -p));
        const T s = two_sum(w.x, -p);
        return fast_two_sum(s.x, __fadd_rn(s.y, __fsub_rn(w.y, e)));
    }
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
    using HV = T;
    using HS = T;
    __device__ static __forceinline__ HV ldh(const void* p, long long i) { return static_cast<const T*>(p)[i]; }
    __device__ static __forceinline__ HS ldo(const void* p, long long i) { return static_cast<const T*>(p)[i]; }
    __device__ static __forceinline__ void sth(void* p, long long i, HS v) { static_cast<T*>(p)[i] = v; }
    __device__ static __forceinline__ float hf(HV h) { return h.x; }
    __device__ static __forceinline__ HV shfl_down_h(HV v, int d) { return shfl_down(v, d); }
    __device__ static __forceinline__ T hdiff(HV r, HV l) { return sub(r, l); }
    __device__ static __forceinline__ T hsum(HV l, HV r) { return add(l, r); }
    __device__ static __forceinline__ T hdo(HV h, HS o) { return sub(h, o); }
    __device__ static __forceinline__ T hdn(HS h, HS o) { return sub(h, o); }
    __device__ static __forceinline__ HS hstep(HV h, T rp, float e) { return nmadf(rp, e, h); }
};

// A double as a double-float, with integer operations only (the hardware
// f64 -> f32 conversion issues on the FP64 pipe): hi = x truncated to 24
// significant bits, lo = the remainder truncated to 24 bits, so
// |x - (hi + lo)| < 2^-47 |x| and |lo| < ulp(hi).  For 2^-126 <= |x| < 2^-74
// the remainder is dropped (absolute error < 2^-97), below 2^-126 the result
// is 0.  |x| >= 2^128, Inf and NaN give hi = Inf: every double-float operation
// on it (two-sum, two-product) then yields NaN, so a NaN state still shows up
// as a NaN residual.
__device__ __forceinline__ float2 split_bits(double x)
{
    const unsigned hi32 = (unsigned)__double2hiint(x);
    const unsigned lo32 = (unsigned)__double2loint(x);
    const unsigned sign = hi32 & 0x80000000u;
    const int E = (int)((hi32 >> 20) & 0x7ffu);
    const int ef = E - 896;   // biased float exponent of x
    unsigned h = sign | ((unsigned)ef << 23) | ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
    h = ef <= 0 ? sign : h;
    h = ef >= 255 ? (sign | 0x7f800000u) : h;
    // remainder: the low 29 significand bits, worth m29 * 2^(E - 1075); a
    // scale exponent <= 0 (x < 2^-74) gives the scale 0 and so lo = 0
    const int es = E - 948;   // biased float exponent of 2^(E - 1075)
    const float m29 = __uint2float_rz(lo32 & 0x1fffffffu);
    const float l = __fmul_rn(m29, __uint_as_float((unsigned)max(es, 0) << 23));
    return make_float2(__uint_as_float(h), __uint_as_float(__float_as_uint(l) | sign));
}

struct DFH : DF64 {
    // H in registers: the double and its double-float split (taken once per load)
    struct HV {
        double d;
        float2 f;
    };
    using HS = double;   // H as stored
    __device__ static __forceinline__ HV ldh(const void* p, long long i)
    {
        const double d = static_cast<const double*>(p)[i];
        return HV{d, split_bits(d)};
    }
    __device__ static __forceinline__ HS ldo(const void* p, long long i) { return static_cast<const double*>(p)[i]; }
    __device__ static __forceinline__ void sth(void* p, long long i, HS v) { static_cast<double*>(p)[i] = v; }
    __device__ static __forceinline__ float hf(const HV& h) { return h.f.x; }
    __device__ static __forceinline__ HV shfl_down_h(const HV& v, int d)
    {
        return HV{__shfl_down_sync(0xffffffffu, v.d, d), shfl_down(v.f, d)};
    }
    // Differences of H values are taken in FP64 -- exact for close values --
    // and then split: an error of 2^-48 |H| in a face gradient is multiplied
    // by K*sigma in the residual and stalls it above tol on fine grids (the
    // DF64 form's limit).
    __device__ static __forceinline__ T hdiff(const HV& r, const HV& l) { return split_bits(r.d - l.d); }
    __device__ static __forceinline__ T hsum(const HV& l, const HV& r) { return add(l.f, r.f); }
    __device__ static __forceinline__ T hdo(const HV& h, HS o) { return split_bits(h.d - o); }
    __device__ static __forceinline__ T hdn(HS h, HS o) { return split_bits(h - o); }
    // H - e*Rp in FP64 with Rp's full double-float accuracy: e*hi and e*lo
    // are exact in FP64 (24 x 24 bits), so two FMAs give the increment to
    // ~2^-48.  (With the increment rounded to FP32 the 2D 8192^2 grid takes
    // a different PT iteration count than FP64.)
    __device__ static __forceinline__ HS hstep(const HV& h, T rp, float e)
    {
        const double ed = f2d_bits(e);
        return fma(-ed, f2d_bits(rp.y), fma(-ed, f2d_bits(rp.x), h.d));
    }
};

// ---------------------------------------------------------------------------
// Two double-floats at once (the values of two faces): component .x of hi and
// lo is the first value, .y the second.  Every operation is the DF64 one above
// done with FP32x2 instructions (__fadd2_rn, __fmul2_rn, __ffma2_rn: one
// instruction for both components, each rounded exactly like the scalar
// operation), so each component is bit for bit what the scalar DF64 code
// gives; the double-float arithmetic of two faces issues as many
// instructions as that of one.
struct DF2 {
    float2 hi, lo;
};

__device__ __forceinline__ DF2 df2_pack(float2 a, float2 b) { return DF2{make_float2(a.x, b.x), make_float2(a.y, b.y)}; }
__device__ __forceinline__ float2 df2_first(const DF2& v) { return make_float2(v.hi.x, v.lo.x); }
__device__ __forceinline__ float2 df2_second(const DF2& v) { return make_float2(v.hi.y, v.lo.y); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ void df2_two_sum(float2 a, float2 b, float2& s, float2& e)
{
    s = add2(a, b);
    const float2 bb = sub2(s, a);
    e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}
__device__ __forceinline__ DF2 df2_fast_two_sum(float2 a, float2 b)
{
    const float2 s = add2(a, b);
    return DF2{s, sub2(b, sub2(s, a))};
}
__device__ __forceinline__ DF2 df2_add(const DF2& a, const DF2& b)
{
    float2 s, e;
    df2_two_sum(a.hi, b.hi, s, e);
    return df2_fast_two_sum(s, add2(e, add2(a.lo, b.lo)));
}
__device__ __forceinline__ DF2 df2_sub(const DF2& a, const DF2& b)
{
    return df2_add(a, DF2{neg2(b.hi), neg2(b.lo)});
}
__device__ __forceinline__ DF2 df2_mul(const DF2& a, const DF2& b)
{
    const float2 p = mul2(a.hi, b.hi);
    float2 e = fma2(a.hi, b.hi, neg2(p));
    e = fma2(a.hi, b.lo, e);
    e = fma2(a.lo, b.hi, e);
    return df2_fast_two_sum(p, e);
}
// a*b + c (DF64::mad)
__device__ __forceinline__ DF2 df2_mad(const DF2& a, const DF2& b, const DF2& c)
{
    const float2 p = mul2(a.hi, b.hi);
    float2 e = fma2(a.hi, b.hi, neg2(p));
    e = fma2(a.hi, b.lo, e);
    e = fma2(a.lo, b.hi, e);
    float2 s, t;
    df2_two_sum(p, c.hi, s, t);
    return df2_fast_two_sum(s, add2(t, add2(e, c.lo)));
}
// w - c*t with float coefficients c (DF64::nmadf)
__device__ __forceinline__ DF2 df2_nmadf(const DF2& t, float2 c, const DF2& w)
{
    const float2 p = mul2(t.hi, c);
    const float2 e = fma2(t.lo, c, fma2(t.hi, c, neg2(p)));
    float2 s, u;
    df2_two_sum(w.hi, neg2(p), s, u);
    return df2_fast_two_sum(s, add2(u, sub2(w.lo, e)));
}

// Split a double into a double-float (host or device).
__host__ __device__ __forceinline__ float2 split_df(double x)
{
    const float hi = (float)x;
    const float lo = (float)(x - (double)hi);
    return make_float2(hi, lo);
}

}  // namespace ptd
