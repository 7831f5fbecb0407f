// ptd_device.cuh -- device-side building blocks of the fused PT kernels.
//
// The reference evaluates the damped flux and the H update as
//   q_new = (q*theta - D_f*dH/dx) / (1 + theta)                 (compute_flux!)
//   H_new = (H + dtau*(Hold/dt - div q)) / (1 + dtau/dt)          (compute_update!)
// (scripts/diff_2D_nonlin.jl:28-39).  Both are rewritten here in the
// algebraically identical fixed-point-preserving form
//   w_new = w - c * (w + K_f * g)          c = 1/(1+theta),  g = H_R - H_L
//   H_new = H - e * ((H - Hold)/dt + sum_d (w_R - w_L) * sigma_d)
//                                          e = dtau/(1 + dtau/dt)
// where w is the flux scaled by dx/kappa (q = w * kappa / dx) and K_f the
// face conductance without its constant factor kappa:
//   LIN      K_f = 1,             kappa = D
//   LINSTEP  K_f = D_L + D_R,     kappa = 1/2   (@av_xi(D) = (D_L+D_R)*0.5)
//   NONLIN   K_f = (H_L + H_R)^3, kappa = 1/8   ((@av_xi(H))^3)
// and sigma_d = kappa / dx_d^2.  At a fixed point w = -K_f g and
// (H-Hold)/dt + div q = 0 whatever c and e are, so the iteration parameters
// (Re, theta, dtau -- pure convergence accelerators) are evaluated in FP32
// while everything that defines the solution (K_f, g, w, H, the divergence
// and the residual) stays in FP64.  This removes every FP64 division and
// square root from the hot loop; GB300's FP64 rate is a small fraction of its
// FP32 rate, so the FP64 instruction count is what bounds the FP64 kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ptd {

enum { LIN = 0, LINSTEP = 1, NONLIN = 2, NONLIN_EXPM = 3 };

constexpr unsigned FULL = 0xffffffffu;

// FP32 constants of the iteration-parameter formulas.
struct FParams {
    float fA;           // L^2/dt
    float fpi, fpi2;    // pi, pi^2
    float fk1;          // NONLIN cell: 1/(Vpdtau*L*Resc)
    float fk2;          // NONLIN face: L*Resc/Vpdtau
    float fk3;          // LINSTEP cell: Re/(Vpdtau*L)
    float frdt;         // 1/dt
};

// Everything a PT-iteration kernel needs, passed by value.  Field pointers
// are untyped: the kernels read them as double (F64) or float2 (DF64).
struct PTArgs {
    int nx, ny, nz;
    long long sy;       // elements between consecutive y rows (row pitch)
    long long sz;       // elements between consecutive z planes
    double rdt;         // 1/dt
    double sig[3];      // kappa / dx_d^2
    float2 rdt_df;      // the same constants as double-floats
    float2 sig_df[3];
    float fc_lin;       // LIN, LINSTEP: 1/(1+theta)
    float fe_lin;       // LIN: dtau/(1+dtau/dt)
    FParams f;
    const void* Hin;
    void* Hout;
    const void* Hold;
    const void* win[3];
    void* wout[3];
    const void* D;      // LINSTEP cell diffusivity
    const int* done;    // nonzero: the step has stopped, skip the iteration
    double* acc;        // residual accumulator: sum R^2 (RMS) or max |R| bits (MAX)
    // Per-block (1D, 3D) / per-warp (2D) partials of the check residual, one
    // slot each, that the judge sums in a fixed order: the same residual norm
    // on every run.  NULL: the partials go into acc by atomics instead.
    double* parts;
    int norm_max;
    // equal sigma_d in every dimension (square cells): the update is formed
    // as (H - Hold) rdt/sigma + sum_d (w_R - w_L) with e*sigma, one
    // multiplication fewer per cell
    int sq;
    double rdt_sig;     // rdt / sigma
    float2 rdt_sig_df;
    float fsig;         // sigma (FP32, scales e)
};

// ---------------------------------------------------------------------------
// Exact FP32 -> FP64 and truncating FP64 -> FP32 conversions done with integer
// operations: the hardware conversion instructions share the scarce FP64 pipe
// (measured: the FP64 3D kernel is 28 % slower with F2F conversions).  Only
// used for the iteration parameters, where any deterministic approximation is
// acceptable.
__device__ __forceinline__ double f2d_bits(float f)
{
    unsigned b = __float_as_uint(f);
    unsigned e = (b >> 23) & 0xffu;
    unsigned hi = (b & 0x80000000u) | ((b & 0x7fffffffu) >> 3);
    hi += (e == 0u) ? 0u : ((e == 255u) ? 0x70000000u : 0x38000000u);
    unsigned lo = (e == 0u) ? 0u : (b << 29);
    if (e == 0u) hi &= 0x80000000u;   // zero / denormal -> signed zero
    return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ float d2f_bits(double x)
{
    int hi = __double2hiint(x);
    unsigned lo = (unsigned)__double2loint(x);
    unsigned sign = (unsigned)hi & 0x80000000u;
    int ef = ((hi >> 20) & 0x7ff) - 896;   // 1023 - 127
    unsigned m = (((unsigned)hi & 0xfffffu) << 3) | (lo >> 29);
    unsigned r = sign | ((unsigned)ef << 23) | m;
    r = (ef <= 0) ? sign : r;
    r = (ef >= 255) ? (sign | 0x7f800000u) : r;
    return __uint_as_float(r);
}

__device__ __forceinline__ float frcp(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float fsqrt(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// NONLIN face: c = 1/(1+theta), theta = L*Resc/(Vpdtau*Re_f),
// Re_f = pi + sqrt(pi^2 + L^2/(D_f dt)), D_f = ((h_L+h_R)/2)^3
// (scripts/diff_2D_nonlin.jl:19-25).  D_f -> 0 gives Re_f -> inf, c -> 1.
__device__ __forceinline__ float nonlin_face_c3(const FParams& a, float df)
{
    float re = a.fpi + fsqrt(a.fpi2 + a.fA * frcp(df));
    float th = a.fk2 * frcp(re);
    return frcp(1.0f + th);
}

__device__ __forceinline__ float nonlin_face_c(const FParams& a, float hsum, float efac = 1.0f)
{
    float m = 0.5f * hsum;
    return nonlin_face_c3(a, efac * m * m * m);
}
// (With s^3 = (s*s)*s already formed, 0.125f * s^3 is bit for bit the
// D_f = m*m*m of m = s/2: scaling by powers of two commutes with rounding.)

// NONLIN cell: e = 1/(1/dtau + 1/dt) with
// 1/dtau = H^3 Re / (Vpdtau L Resc) = (pi H^3 + sqrt(pi^2 H^6 + L^2 H^3/dt)) * k1
// (scripts/diff_2D_nonlin.jl:23,26); finite for H^3 -> 0 (e -> dt).
__device__ __forceinline__ float nonlin_cell_e(const FParams& a, float h, float efac = 1.0f)
{
    float h3 = efac * h * h * h;
    float inv = (a.fpi * h3 + fsqrt(a.fpi2 * h3 * h3 + a.fA * h3)) * a.fk1;
    return frcp(inv + a.frdt);
}

// (NONLIN_EXPM: D = exp(m) H^3 -- efac = exp(m) at the cell, the arithmetic
// mean of exp(m) at a face.)

// The face parameter c with every operation explicit (no contraction left to
// the compiler), for the FP32 kernels whose scalar and packed two-lane forms
// must round identically (ptd_rb_body.cuh, ptd_dc_body.cuh):
// c = 1/(1 + fk2/Re_f) = Re_f/(Re_f + fk2), Re_f = pi + sqrt(pi^2 + fA/D_f),
// in three MUFU operations (the reciprocal of Re_f saved).  D_f -> 0 gives
// Re_f -> inf and c -> 1, taken explicitly where Re_f + fk2 overflows.
__device__ __forceinline__ float face_c_rn(const FParams& f, float df)
{
    const float q = __fmaf_rn(f.fA, frcp(df), f.fpi2);
    const float re = __fadd_rn(f.fpi, fsqrt(q));
    const float den = __fadd_rn(re, f.fk2);
    return den < INFINITY ? __fmul_rn(re, frcp(den)) : 1.0f;
}

// Two lanes at once (FP32x2 instructions, sm_100 and later: two faces per
// instruction, each component rounded exactly like the scalar operation).
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 f2(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.0f), a); }   // a - b
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// LINSTEP cell: 1/dtau = maxloc(D) * Re / (Vpdtau L) (compute_iter_params!,
// scripts/diff_2D_linstep.jl:18-21).
__device__ __forceinline__ float linstep_cell_e(const FParams& a, float dmax)
{
    return frcp(dmax * a.fk3 + a.frdt);
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(FULL, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// Block-wide residual reduction into acc (sum of squares, or max |R| as the
// ordered bit pattern of a non-negative double; NaN orders above +inf), or,
// with parts, into the block's own slot parts[slot] (same encoding).  The
// reduction inside the block has a fixed order either way.
__device__ __forceinline__ void block_reduce_residual(double* acc, int norm_max, double part_sum,
                                                      unsigned long long part_max, double* parts = nullptr,
                                                      long long slot = 0)
{
    __shared__ double s_sum[32];
    __shared__ unsigned long long s_max[32];
    const int nthr = blockDim.x * blockDim.y * blockDim.z;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int wid = tid >> 5, ln = tid & 31;
    const int nw = (nthr + 31) >> 5;
    if (norm_max) {
        part_max = warp_max_u64(part_max);
        if (ln == 0) s_max[wid] = part_max;
    } else {
        part_sum = warp_sum(part_sum);
        if (ln == 0) s_sum[wid] = part_sum;
    }
    __syncthreads();
    if (wid == 0) {
        if (norm_max) {
            unsigned long long v = ln < nw ? s_max[ln] : 0ull;
            v = warp_max_u64(v);
            if (ln == 0 && parts) parts[slot] = __longlong_as_double((long long)v);
            else if (ln == 0 && v) atomicMax(reinterpret_cast<unsigned long long*>(acc), v);
        } else {
            double v = ln < nw ? s_sum[ln] : 0.0;
            v = warp_sum(v);
            if (ln == 0 && parts) parts[slot] = v;
            else if (ln == 0) atomicAdd(acc, v);
        }
    }
}

__device__ __forceinline__ void block_reduce_residual(const PTArgs& a, double part_sum,
                                                      unsigned long long part_max, long long slot)
{
    block_reduce_residual(a.acc, a.norm_max, part_sum, part_max, a.parts, slot);
}

__device__ __forceinline__ void accumulate_residual(double r, double& sum, unsigned long long& mx)
{
    sum = fma(r, r, sum);
    unsigned long long b = (unsigned long long)__double_as_longlong(r) & 0x7fffffffffffffffull;
    mx = b > mx ? b : mx;
}

// FP32 form for the FP32 inner iterations of the defect correction: their
// residual is an FP32 value, so one thread's sum of squares and max |r| over
// its cells (one march of at most a few hundred) stay in FP32 and are widened
// once per thread (widen_max32) for the FP64 block reduction.  A per-cell
// f32->f64 conversion and DFMA run on the FP64 pipe, 1/64 of the FP32 rate
// on this GPU: measured on the 256-instance batch, a check launch of the
// two-iteration kernel took 532 us with them and 483 us without (a plain
// launch 213 us; the rest of the gap is the check variant's register count).
__device__ __forceinline__ void accumulate_residual32(float r, float& sum, unsigned& mx)
{
    sum = fmaf(r, r, sum);
    const unsigned b = __float_as_uint(r) & 0x7fffffffu;
    mx = b > mx ? b : mx;
}

// An FP32 max |r| (bit pattern) as the FP64 bit pattern block_reduce_residual
// compares; NaN stays NaN, so it still wins the max.
__device__ __forceinline__ unsigned long long widen_max32(unsigned mx)
{
    return (unsigned long long)__double_as_longlong((double)__uint_as_float(mx));
}

// Warp-level flush of the FP32 partials into acc (the encoding of
// block_reduce_residual: sum of squares, or the max |r| bit pattern), one
// atomic per warp.  The 2D inner kernels call it from inside the last step
// of their y march, with all 32 lanes converged: a reduction after the march
// made ptxas give their check variants 52-98 registers (32-40 this way),
// halving the resident warps of a latency-bound kernel.
// With parts, the warp's result goes into its own slot parts[slot] instead.
__device__ __forceinline__ void warp_flush_residual32(double* acc, int norm_max, float part_sum, unsigned part_max,
                                                      int lane, double* parts = nullptr, long long slot = 0)
{
    if (norm_max) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned w = __shfl_xor_sync(FULL, part_max, o);
            part_max = w > part_max ? w : part_max;
        }
        if (lane == 0 && parts) parts[slot] = __longlong_as_double((long long)widen_max32(part_max));
        else if (lane == 0 && part_max) atomicMax(reinterpret_cast<unsigned long long*>(acc), widen_max32(part_max));
    } else {
        const double v = warp_sum((double)part_sum);
        if (lane == 0 && parts) parts[slot] = v;
        else if (lane == 0) atomicAdd(acc, v);
    }
}

// Slot of this warp (2D kernels: warps numbered x fastest) / block (1D, 3D)
// in a residual-slot array.
__device__ __forceinline__ long long warp_slot()
{
    return ((long long)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.y + threadIdx.y;
}
__device__ __forceinline__ long long block_slot()
{
    return ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
}

// Fixed-order sum (or max, for the max-norm bit patterns) of nparts slots by a
// block of 256 threads: thread t takes slots t, t + 256, ... in order, then a
// fixed tree over the threads.  Every thread returns the result.
__device__ __forceinline__ double sum_slots(const double* parts, long long nparts, int norm_max)
{
    __shared__ double s_sum[256];
    __shared__ unsigned long long s_max[256];
    const int t = threadIdx.x;
    double sum = 0.0;
    unsigned long long mx = 0ull;
    for (long long i = t; i < nparts; i += 256) {
        const double v = parts[i];
        const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
        mx = bits > mx ? bits : mx;
        sum += v;
    }
    s_sum[t] = sum;
    s_max[t] = mx;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) {
            s_sum[t] += s_sum[t + o];
            s_max[t] = s_max[t + o] > s_max[t] ? s_max[t + o] : s_max[t];
        }
        __syncthreads();
    }
    const double r = norm_max ? __longlong_as_double((long long)s_max[0]) : s_sum[0];
    __syncthreads();
    return r;
}

// FP64 form of warp_flush_residual32 for the 2D kernels whose check partials
// are doubles (FP64, DF64, DFH, and the rebased FP32 form, whose check
// residual carries the FP64 base residual): same encoding, one atomic per
// warp, called from inside the last step of the y march with all 32 lanes
// converged (after the march, the check variants held 61-97 registers).
// With parts, the warp's result goes into its own slot parts[slot] instead.
__device__ __forceinline__ void warp_flush_residual(double* acc, int norm_max, double part_sum,
                                                    unsigned long long part_max, int lane, double* parts = nullptr,
                                                    long long slot = 0)
{
    if (norm_max) {
        part_max = warp_max_u64(part_max);
        if (lane == 0 && parts) parts[slot] = __longlong_as_double((long long)part_max);
        else if (lane == 0 && part_max) atomicMax(reinterpret_cast<unsigned long long*>(acc), part_max);
    } else {
        part_sum = warp_sum(part_sum);
        if (lane == 0 && parts) parts[slot] = part_sum;
        else if (lane == 0) atomicAdd(acc, part_sum);
    }
}

__device__ __forceinline__ bool step_done(const int* done)
{
    return __ldcg(done) != 0;
}

}  // namespace ptd
