// ptd_batch.cu -- many independent 2D solves of uneven grid sizes, each with
// its own initial condition and D field, advanced together.
//
// No reference counterpart (the reference solves one grid per process); the
// per-instance algorithm is the reference's (scripts/diff_2D_linstep.jl and
// siblings) or the FP32 + FP64 defect correction of ptd_dc.cu.
//
// Layout: every field of every instance lives in one concatenated device
// buffer (instance i at element offset off_i, row pitch a multiple of 32).
// One kernel launch per PT iteration covers the whole batch: a work table
// maps each CTA to (instance, x tile block, y chunk), the CTA loads its
// instance's arguments from a device table and runs the same kernel body as
// the one-grid solver.  Each instance has its own control block (check
// accumulator, done flag, iteration counter); CTAs of a finished instance
// return at entry, so a CUDA graph holding nchk iterations + the batched judge
// is replayed until every instance has stopped, with no host round trip per
// check and no instance waiting for another.
//
// FP32_DC: the inexact-Newton state machine of ptd_dc.cu runs per instance on
// the device (forcing term, FP32-floor-aware inner target, backtracking), so
// instances that need different numbers of outer corrections also proceed
// independently; the host only replays graphs until all have finished.
//
// FP32_RB: the rebased FP32 form of ptd_rb.cu (ptd_rb_body.cuh) per instance.
// A physical step of the whole batch is one CUDA graph launch: a WHILE node
// whose body is one phase of every instance -- check blocks of two-iteration
// launches over all instances, each followed by the per-instance FP32 judge,
// then the FP64 rebase of every running instance (fold, base quantities,
// per-instance FP64 judge) -- and which the FP64 judge ends once every
// instance has stopped.  An instance whose phase or step is over skips the
// iteration launches (its CTAs return at entry) and waits for the next
// rebase; no host round trip per check or per phase.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "ptd_dc_body.cuh"
#include "ptd_internal.h"
#include "ptd_pt_body.cuh"
#include "ptd_rb_body.cuh"

namespace ptd {

enum { PH_START = 0, PH_INNER = 1, PH_BACKTRACK = 2, PH_CONVERGED = 3, PH_CAPPED = 4, PH_NAN = 5 };

// Per-instance control block of the batched defect correction.
struct BDev {
    int done;        // inner solve finished (or not running)
    int nchecks;
    int iter;        // inner iterations of the current inner solve
    int best_at;
    double acc;      // inner residual accumulator
    double err;
    double best;
    double target;
    double outer_acc;            // FP64 residual accumulator
    unsigned long long hmax_bits;
    double err_ref;  // residual norm of the last accepted state
    double a_last;   // factor of the last correction applied
    double a_next;   // factor the next apply uses
    int phase;
    int nhalf;
    int outer;
    int total_inner;
    // constants
    double norm_den;
    double cond_scale;   // dt * sum_d 4/dx_d^2
    double dconst;       // Dmax of the linear models
};

// The sum (or max) of slots first .. first+count-1 by one warp, in a fixed
// order: lane l takes slots first+l, first+l+32, ... in order, then a fixed
// shuffle tree.  Every lane returns the result.
__device__ __forceinline__ double warp_sum_range(const double* parts, long long first, long long count, int norm_max)
{
    const int lane = threadIdx.x & 31;
    double sum = 0.0;
    unsigned long long mx = 0ull;
    for (long long k = first + lane; k < first + count; k += 32) {
        const double v = parts[k];
        const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
        mx = bits > mx ? bits : mx;
        sum += v;
    }
    return norm_max ? __longlong_as_double((long long)warp_max_u64(mx)) : warp_sum(sum);
}

// ---------------------------------------------------------------------------
template <class N, int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) pt2d_batch_kernel(const PTArgs* __restrict__ tab,
                                                         const int4* __restrict__ work, int chunk)
{
    const int4 w = work[blockIdx.x];
    const PTArgs a = tab[w.x];
    if (step_done(a.done)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    // the body flushes its check partials into its warp's slot (work item k,
    // warp w -> k * W + w; last step of its march)
    pt2d_body<N, MODEL, CHECK>(a, w.y * blockDim.y + threadIdx.y, w.z, chunk, part, pmax,
                               (long long)blockIdx.x * blockDim.y + threadIdx.y);
}

// The check of every running instance (one warp each), its residual summed
// from its warps' slots (work items wfirst .. wfirst+wcount-1, W warps each)
// in a fixed order.
__global__ void judge_batch_kernel(DevState* st, int ninst, int nchk, int itmax, double tol,
                                   const double* norm_den, int norm_max, const double* parts, const int* wfirst,
                                   const int* wcount, int W)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= ninst || st[i].done) return;   // uniform over the warp; no iteration ran
    const double acc = warp_sum_range(parts, (long long)wfirst[i] * W, (long long)wcount[i] * W, norm_max);
    if ((threadIdx.x & 31) != 0) return;
    DevState& s = st[i];
    s.acc = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(norm_den[i]);
    s.nchecks += 1;
    s.iter += nchk;
    s.err = err;
    if (!(err > tol)) s.done = (err != err) ? DONE_NAN : DONE_CONVERGED;
    else if (s.iter + nchk > itmax) s.done = DONE_CAP;
}

// Last node of a pass of a batch solve graph's loop (one block): ends the loop
// once no instance is running; every pass adds a check block to each running
// instance and an instance with no room for another before itmax stops, so
// the loop ends within itmax/nchk + 1 passes (max_passes: a bound kept all
// the same).
template <class S>
__global__ void __launch_bounds__(256) batch_loop_judge_kernel(const S* st, int ninst, int* passes, int max_passes,
                                                               cudaGraphConditionalHandle loop)
{
    int running = 0;
    for (int i = threadIdx.x; i < ninst; i += blockDim.x) running |= st[i].done == 0;
    const int any = __syncthreads_or(running);
    if (threadIdx.x == 0) {
        *passes += 1;
        if (!any || *passes >= max_passes) cudaGraphSetConditional(loop, 0);
    }
}

__global__ void reset_batch_kernel(DevState* st, int ninst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    st[i].done = DONE_RUNNING;
    st[i].nchecks = 0;
    st[i].iter = 0;
    st[i].acc = 0.0;
    st[i].err = 0.0;
}

// ---------------------------------------------------------------------------
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) dc2d_batch_kernel(const DcArgs* __restrict__ tab,
                                                         const int4* __restrict__ work, int chunk)
{
    const int4 w = work[blockIdx.x];
    const DcArgs a = tab[w.x];
    if (dc_done(a.done)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    // the body flushes its check partials into its warp's slot (last step of its march)
    dc2d_body<MODEL, CHECK>(a, w.y * blockDim.y + threadIdx.y, w.z, chunk, part, pmax,
                            (long long)blockIdx.x * blockDim.y + threadIdx.y);
}

// two inner iterations per launch (temporal blocking, ptd_dc_body.cuh)
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) dc2d_tb2_batch_kernel(const DcArgs* __restrict__ tab,
                                                             const int4* __restrict__ work, int chunk)
{
    const int4 w = work[blockIdx.x];
    const DcArgs a = tab[w.x];
    if (dc_done(a.done)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    // the body flushes its check partials into its warp's slot (last step of its march)
    dc2d_tb2_body<MODEL, CHECK>(a, w.y * blockDim.y + threadIdx.y, w.z, chunk, part, pmax,
                                (long long)blockIdx.x * blockDim.y + threadIdx.y);
}

// The inner check of every instance still in its inner solve (one warp each),
// its residual summed from its warps' slots in a fixed order.
__global__ void inner_judge_batch_kernel(BDev* st, int ninst, int nchk, int itmax, int norm_max, int stall,
                                         const double* parts, const int* wfirst, const int* wcount, int W)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= ninst || st[i].done) return;   // uniform over the warp; no iteration ran
    const double acc = warp_sum_range(parts, (long long)wfirst[i] * W, (long long)wcount[i] * W, norm_max);
    if ((threadIdx.x & 31) != 0) return;
    BDev& s = st[i];
    s.acc = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(s.norm_den);
    s.err = err;
    s.nchecks += 1;
    s.iter += nchk;
    if (err < 0.95 * s.best) {
        s.best = err;
        s.best_at = s.nchecks;
    }
    if (!(err > s.target)) s.done = 1;
    else if (s.iter + nchk > itmax) s.done = 1;
    else if (s.nchecks - s.best_at >= stall) s.done = 1;   // FP32 floor reached
}

// FP64 residual of each unfinished instance over one chunk of its inner
// cells (cwork: {instance, first inner cell, count}); writes r as FP32.
template <int MODEL>
__global__ void __launch_bounds__(256) resid64_batch_kernel(const PTArgs* __restrict__ tab, BDev* st,
                                                            float* const* rf, const int4* __restrict__ cwork,
                                                            double* parts64)
{
    const int4 w = cwork[blockIdx.x];
    const int inst = w.x;
    if (st[inst].phase >= PH_CONVERGED) return;
    const PTArgs a = tab[inst];
    const double* Hp = static_cast<const double*>(a.Hin);
    const double* Hold = a.Hold ? static_cast<const double*>(a.Hold) : Hp;
    const double* Dp = static_cast<const double*>(a.D);
    float* r_out = rf[inst];
    const long long nix = a.nx - 2;
    double part = 0.0;
    unsigned long long pmax = 0ull, hm = 0ull;
    for (int t = threadIdx.x; t < w.z; t += blockDim.x) {
        const long long cell = (long long)w.y + t;
        const long long ix = 1 + cell % nix, iy = 1 + cell / nix;
        const long long c = iy * a.sy + ix;
        const long long stp[2] = {1, a.sy};
        const double H = Hp[c];
        double div = 0.0;
        for (int d = 0; d < 2; ++d) {
            const double HR = Hp[c + stp[d]], HL = Hp[c - stp[d]];
            double uR, uL;
            if (MODEL == LIN) {
                uR = HR - H;
                uL = H - HL;
            } else if (MODEL == LINSTEP) {
                uR = (Dp[c] + Dp[c + stp[d]]) * (HR - H);
                uL = (Dp[c - stp[d]] + Dp[c]) * (H - HL);
            } else {
                const double sR = H + HR, sL = HL + H;
                uR = sR * sR * sR * (HR - H);
                uL = sL * sL * sL * (H - HL);
            }
            div = fma(uR - uL, a.sig[d], div);
        }
        const double r = fma(-(H - Hold[c]), a.rdt, div);
        r_out[c] = (float)r;
        accumulate_residual(r, part, pmax);
        const unsigned long long hb = (unsigned long long)__double_as_longlong(H) & 0x7fffffffffffffffull;
        hm = hb > hm ? hb : hm;
    }
    hm = warp_max_u64(hm);
    if ((threadIdx.x & 31) == 0 && hm) atomicMax(&st[inst].hmax_bits, hm);
    block_reduce_residual(nullptr, a.norm_max, part, pmax, parts64, blockIdx.x);   // the chunk's slot
}

// Per-instance inexact-Newton state machine (see ptd_dc.cu).
// One warp per instance: the FP64 residual from the instance's chunk slots
// (ffirst .. ffirst+fcount-1) in a fixed order, then its Newton state.
__global__ void outer_judge_batch_kernel(BDev* st, int ninst, int norm_max, double tol, double rtol,
                                         int max_outer, int itmax, int nonlin, const double* parts64,
                                         const int* ffirst, const int* fcount)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= ninst || st[i].phase >= PH_CONVERGED) return;   // uniform over the warp
    const double acc = warp_sum_range(parts64, ffirst[i], fcount[i], norm_max);
    if ((threadIdx.x & 31) != 0) return;
    BDev& s = st[i];
    s.outer_acc = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(s.norm_den);
    const double hmax = __longlong_as_double((long long)s.hmax_bits);
    s.hmax_bits = 0ull;
    double eta = 0.1;
    if (s.phase == PH_START) {
        s.outer = 0;
        s.total_inner = 0;
        s.nhalf = 0;
    } else {
        if (s.phase == PH_INNER) s.total_inner += s.iter;
        if (!(err < s.err_ref) && s.nhalf < 4) {   // also catches NaN
            s.phase = PH_BACKTRACK;
            s.a_next = -0.5 * s.a_last;
            s.a_last *= 0.5;
            s.nhalf += 1;
            s.done = 1;
            return;
        }
        s.outer += 1;
        const double q = err / s.err_ref;
        eta = fmin(0.5, fmax(rtol, 0.9 * q * q));
    }
    s.err_ref = err;
    s.nhalf = 0;
    s.done = 1;
    if (!(err > tol)) {
        s.phase = (err != err) ? PH_NAN : PH_CONVERGED;
        return;
    }
    if (s.outer >= max_outer || s.total_inner >= itmax) {
        s.phase = PH_CAPPED;
        return;
    }
    const double dmax = nonlin ? hmax * hmax * hmax : s.dconst;
    const double floor = fmin(0.5, 0.5 * 5.96e-8 * (1.0 + s.cond_scale * dmax));
    s.target = fmax(fmax(eta, floor) * err, 0.25 * tol);
    s.phase = PH_INNER;
    s.a_last = 1.0;
    s.a_next = 1.0;
    s.done = 0;
    s.nchecks = 0;
    s.iter = 0;
    s.best = err;
    s.best_at = 0;
    s.acc = 0.0;
}

__global__ void start_batch_kernel(BDev* st, int ninst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    st[i].phase = PH_START;
    st[i].done = 1;
    st[i].outer_acc = 0.0;
    st[i].hmax_bits = 0ull;
    st[i].acc = 0.0;
}

// H += a * delta (a from the instance's phase), refresh Hf; zero the
// correction state for the next inner solve.
__global__ void __launch_bounds__(256) apply_batch_kernel(const DcArgs* __restrict__ tab0, const BDev* st,
                                                          const int4* __restrict__ fwork, double* const* Hs,
                                                          const int* cur_parity)
{
    const int4 w = fwork[blockIdx.x];
    const int inst = w.x;
    const BDev& s = st[inst];
    double a;
    if (s.phase == PH_INNER) a = 1.0;
    else if (s.phase == PH_BACKTRACK) a = s.a_next;
    else return;
    const DcArgs& t = tab0[inst];
    const float* delta = cur_parity[inst] ? t.dout : t.din;
    double* H = Hs[inst];
    float* Hf = const_cast<float*>(t.Hf);
    for (int k = threadIdx.x; k < w.z; k += blockDim.x) {
        const long long e = (long long)w.y + k;
        const double h = fma(a, (double)delta[e], H[e]);
        H[e] = h;
        Hf[e] = __double2float_rn(h);
    }
}

// Zero the correction state (delta and its fluxes, both parities) of the
// instances about to start an inner solve.
__global__ void __launch_bounds__(256) zero_batch_kernel(const DcArgs* __restrict__ tab0, const BDev* st,
                                                         const int4* __restrict__ fwork, int ndim)
{
    const int4 w = fwork[blockIdx.x];
    const int inst = w.x;
    if (st[inst].phase != PH_INNER || st[inst].iter != 0) return;
    const DcArgs& t = tab0[inst];
    float* ptrs[2 + 2 * 3];
    int np = 0;
    ptrs[np++] = const_cast<float*>(t.din);
    ptrs[np++] = t.dout;
    for (int d = 0; d < ndim; ++d) {
        ptrs[np++] = const_cast<float*>(t.win[d]);
        ptrs[np++] = t.wout[d];
    }
    for (int k = threadIdx.x; k < w.z; k += blockDim.x) {
        const long long e = (long long)w.y + k;
        for (int q = 0; q < np; ++q) ptrs[q][e] = 0.0f;
    }
}

__global__ void set_done_batch_kernel(BDev* st, int ninst, int v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ninst) st[i].done = v;
}

// buffer of each instance's current correction: one swap per launch, `tb`
// inner iterations per launch
__global__ void parity_batch_kernel(const BDev* st, int* cur_parity, int ninst, int tb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    if (st[i].phase == PH_INNER) cur_parity[i] = (st[i].iter / tb) & 1;
}

__global__ void tofloat_batch_kernel(const double* src, float* dst, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        dst[t] = __double2float_rn(src[t]);
}

// ---------------------------------------------------------------------------
// FP32_RB: one (TB = 1) or two (TB = 2) rebased FP32 iterations over every
// instance whose phase is running.  CTA b takes the b-th work item of the
// running instances (`active`, rebuilt after every judge by
// compact_active_kernel, in instance order); CTAs past their number return at
// entry after one load, so once most instances have stopped a launch costs
// their remaining work rather than a table walk per work item of the whole
// batch.  (A persistent grid walking the list held 74-98 registers against
// the march's 40-64.)
template <int MODEL, bool CHECK, int TB>
__global__ void __launch_bounds__(256) rb2d_batch_kernel(const RbArgs* __restrict__ tab,
                                                         const int4* __restrict__ work,
                                                         const int* __restrict__ active, const int* nactive,
                                                         int chunk)
{
    if ((int)blockIdx.x >= __ldcg(nactive)) return;
    const int4 w = work[active[blockIdx.x]];
    const RbArgs a = tab[w.x];
    if (rb_skip(a.skip)) return;   // its phase ended since the list was built
    float part = 0.0f;
    unsigned pmax = 0u;
    // the bodies flush their check partials into the warp's slot: work item k, warp w -> k * W + w
    const long long slot = (long long)active[blockIdx.x] * blockDim.y + threadIdx.y;
    if (TB == 2) rb2d_tb2_body<MODEL, CHECK>(a, w.y * blockDim.y + threadIdx.y, w.z, chunk, part, pmax, slot);
    else rb2d_body<MODEL, CHECK>(a, w.y * blockDim.y + threadIdx.y, w.z, chunk, part, pmax, slot);
}

// The work items of the running instances, in instance order (one block):
// instance i owns items wfirst[i] .. wfirst[i] + wcount[i] - 1.
__global__ void __launch_bounds__(256) compact_active_kernel(const RbDev* st, const int* wfirst, const int* wcount,
                                                             int ninst, int* active, int* nactive)
{
    __shared__ int s_off[256];
    __shared__ int s_base;
    const int t = threadIdx.x;
    if (t == 0) s_base = 0;
    __syncthreads();
    for (int i0 = 0; i0 < ninst; i0 += 256) {
        const int i = i0 + t;
        const int c = (i < ninst && !st[i].skip && !st[i].step_done) ? wcount[i] : 0;
        // inclusive scan of the counts over the block
        s_off[t] = c;
        __syncthreads();
        for (int o = 1; o < 256; o <<= 1) {
            const int v = t >= o ? s_off[t - o] : 0;
            __syncthreads();
            s_off[t] += v;
            __syncthreads();
        }
        const int start = s_base + s_off[t] - c;
        for (int q = 0; q < c; ++q) active[start + q] = wfirst[i] + q;
        __syncthreads();
        if (t == 255) s_base += s_off[255];
        __syncthreads();
    }
    if (t == 0) *nactive = s_base;
}

__global__ void rb_reset_batch_kernel(RbDev* st, int ninst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ninst) rb_reset(&st[i]);
}

// The FP32 check of every instance (one warp each), its residual summed from
// its warps' slots (work items wfirst .. wfirst+wcount-1, W warps each).
__global__ void rb_check_judge_batch_kernel(RbDev* st, int ninst, int nchk, int itmax, double tol,
                                            const double* norm_den, int norm_max, const double* parts,
                                            const int* wfirst, const int* wcount, int W)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= ninst || st[i].skip || st[i].step_done) return;   // uniform over the warp; no iteration ran
    const double acc = warp_sum_range(parts, (long long)wfirst[i] * W, (long long)wcount[i] * W, norm_max);
    if ((threadIdx.x & 31) == 0) {
        st[i].acc = acc;
        rb_check_judge(&st[i], nullptr, 0, nchk, itmax, tol, norm_den[i], norm_max);
    }
}

// The FP64 judge of every instance (one block); in the step graph's WHILE
// node (in_loop) it ends the loop once no instance is running.  Every pass of
// the body adds at least one check block to each running instance, and an
// instance with no room for another block before itmax stops (capped), so the
// loop ends within itmax/nchk passes.
__global__ void __launch_bounds__(256) rb_base_judge_batch_kernel(RbDev* st, int ninst, double tol,
                                                                  const double* norm_den, int norm_max,
                                                                  cudaGraphConditionalHandle loop, int in_loop,
                                                                  int* passes, const double* parts64,
                                                                  const int* ffirst, const int* fcount)
{
    int running = 0;
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i = threadIdx.x >> 5; i < ninst; i += nw) {   // one warp per instance
        // the FP64 residual from the instance's base-kernel slots (its field
        // chunks ffirst .. ffirst+fcount-1), in a fixed order
        if (!st[i].step_done) {
            const double acc = warp_sum_range(parts64, ffirst[i], fcount[i], norm_max);
            if (lane == 0) st[i].acc64 = acc;
        }
        if (lane == 0 && !rb_base_judge(&st[i], tol, norm_den[i], norm_max)) running = 1;
        __syncwarp();
    }
    const int any = __syncthreads_or(running);
    if (in_loop && threadIdx.x == 0) {
        *passes += 1;
        if (!any) cudaGraphSetConditional(loop, 0);
    }
}

// Fold the changes of every running instance into its base (one chunk of an
// instance's padded fields per CTA, fwork: {instance, first element, count}).
__global__ void __launch_bounds__(256) rb_fold_batch_kernel(const RbFoldArgs* __restrict__ ftab, const RbDev* st,
                                                            const int4* __restrict__ fwork, int tb)
{
    const int4 w = fwork[blockIdx.x];
    if (st[w.x].step_done) return;
    const int parity = (st[w.x].phase_iter / tb) & 1;   // one buffer swap per launch of tb iterations
    const RbFoldArgs f = ftab[w.x];
    for (int k = threadIdx.x; k < w.z; k += blockDim.x) rb_fold_elem(f, parity, (long long)w.y + k);
}

// Base quantities of every running instance (of all instances at a step
// start: use_st = 0), one chunk of an instance's padded field per CTA.
__global__ void __launch_bounds__(256) rb_base_batch_kernel(const RbBaseArgs* __restrict__ btab, const RbDev* st,
                                                            const int4* __restrict__ fwork, int use_st)
{
    const int4 w = fwork[blockIdx.x];
    if (use_st && st[w.x].step_done) return;   // uniform over the block
    const RbBaseArgs b = btab[w.x];
    double part = 0.0;
    unsigned long long pmax = 0ull;
    for (int k = threadIdx.x; k < w.z; k += blockDim.x) {
        const long long e = (long long)w.y + k;
        const int ix = (int)(e % b.sy), iy = (int)(e / b.sy);
        if (ix < b.nx) rb_base_cell(b, ix, iy, 0, part, pmax);   // padding columns hold no cell
    }
    block_reduce_residual(b.acc64, b.norm_max, part, pmax, b.parts, blockIdx.x);   // the chunk's slot
}

// ---------------------------------------------------------------------------
// Host <-> device transfers go through a contiguous packed copy of all
// instances' fields (one plain copy per instance at the link's rate instead
// of a pitched copy of nx-element rows); these kernels convert between the
// packed layout and the padded one.  pwork: {instance, first packed element,
// count}.
struct PackInst {
    long long poff;   // offset of the instance in the packed buffer
    long long off;    // offset of the instance in the padded fields
    long long sy;     // its row pitch
    int nx, pad;
};

__global__ void __launch_bounds__(256) unpack_batch_kernel(const double* __restrict__ packed, double* __restrict__ dst,
                                                           const PackInst* __restrict__ pi,
                                                           const int4* __restrict__ pwork)
{
    const int4 w = pwork[blockIdx.x];
    const PackInst I = pi[w.x];
    for (int k = threadIdx.x; k < w.z; k += blockDim.x) {
        const long long e = (long long)w.y + k;
        const long long r = e / I.nx;
        dst[I.off + r * I.sy + (e - r * I.nx)] = packed[I.poff + e];
    }
}

__global__ void __launch_bounds__(256) pack_batch_kernel(const double* __restrict__ src, double* __restrict__ packed,
                                                         const PackInst* __restrict__ pi,
                                                         const int4* __restrict__ pwork)
{
    const int4 w = pwork[blockIdx.x];
    const PackInst I = pi[w.x];
    for (int k = threadIdx.x; k < w.z; k += blockDim.x) {
        const long long e = (long long)w.y + k;
        const long long r = e / I.nx;
        packed[I.poff + e] = src[I.off + r * I.sy + (e - r * I.nx)];
    }
}

// ---------------------------------------------------------------------------
#define BCK(call)                                                 \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);       \
    } while (0)

struct Inst {
    int nx, ny;
    long long sy, nfield, off;
    Derived dv;
    ptd_params p;   // one-grid view of the instance
};

}  // namespace ptd

using namespace ptd;

struct ptd_batch {
    ptd_batch_params bp;
    int ninst = 0;
    int model = 0;
    bool df64 = false, dc = false;
    std::vector<Inst> inst;
    long long total = 0;       // elements of one concatenated field
    cudaStream_t s = nullptr;
    // host <-> device copies of the instances, spread over four copy
    // streams (joined to s by events), so that the set-up of the many small
    // copies overlaps
    cudaStream_t cs[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[4] = {nullptr, nullptr, nullptr, nullptr};
    LaunchCfg cfg;
    // plain PT (FP64 / DF64)
    void* H[2] = {nullptr, nullptr};
    void* Hold = nullptr;
    void* W[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    void* D = nullptr;
    double* stage = nullptr;
    DevState* st = nullptr;
    DevState* h_st = nullptr;
    double* norm_den = nullptr;
    PTArgs* tab[2] = {nullptr, nullptr};
    // FP32 DC
    double* H64 = nullptr;
    double* Hold64 = nullptr;
    double* D64 = nullptr;
    float* Hf = nullptr;
    float* Df = nullptr;
    float* rf = nullptr;
    float* d[2] = {nullptr, nullptr};
    float* w32[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    BDev* bst = nullptr;
    BDev* h_bst = nullptr;
    DcArgs* dtab[2] = {nullptr, nullptr};
    PTArgs* rtab = nullptr;
    float** rf_ptrs = nullptr;
    double** H_ptrs = nullptr;
    int* cur_parity = nullptr;
    int4* cwork = nullptr;
    int ncwork = 0;
    int4* fwork = nullptr;
    int nfwork = 0;
    // FP32_RB (H64, Hold64, D64, Hf, Df, d, w32 as above): FP64 base fluxes,
    // FP32 base defects, the base check residual (FP32), per-instance control blocks
    bool rb = false;
    double* wb64[2] = {nullptr, nullptr};
    float* tb32[2] = {nullptr, nullptr};
    float* Rb32 = nullptr;
    float* Cb32 = nullptr;
    RbDev* rdev = nullptr;
    RbDev* h_rdev = nullptr;
    RbArgs* rbtab[2] = {nullptr, nullptr};
    RbFoldArgs* ftab = nullptr;
    RbBaseArgs* btab = nullptr;
    int* passes = nullptr;
    int* h_passes = nullptr;
    int* wfirst = nullptr;     // per instance: its first work item and its count
    int* wcount = nullptr;
    int* active = nullptr;     // work items of the running instances, and their count
    int* nactive = nullptr;
    // deterministic residuals of the rebased batch: per-warp check slots (work
    // item k, warp w -> k * W + w; sized for the smallest work items the tuner
    // can choose) and per-chunk FP64 slots, with each instance's chunk range
    double* parts = nullptr;
    long long nparts = 0;
    double* parts64 = nullptr;
    int* ffirst = nullptr;
    int* fcount = nullptr;
    // packed host <-> device transfers
    double* packed = nullptr;
    PackInst* pinst = nullptr;
    int4* pwork = nullptr;
    int npwork = 0;
    cudaGraphExec_t gstep = nullptr;
    int blocks_per_phase = 1;
    // common
    int4* work = nullptr;
    int nwork = 0;
    int nchk = 10;
    int tb = 1;        // FP32_DC, FP32_RB: FP32 iterations per launch (2: temporal blocking)
    int stall = 10;
    cudaGraphExec_t g = nullptr;   // FP64 / DF64: one step; FP32_DC: one round of inner solves
    int kernels_per_graph = 0;
    long long launches = 0, iterations = 0;
};

namespace {

int bfail(int status, const char* msg) { return set_error(status, msg); }

template <class T>
int balloc(T** p, size_t bytes)
{
    cudaError_t e = cudaMalloc((void**)p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(e == cudaErrorMemoryAllocation ? PTD_ENOMEM : PTD_ECUDA, "batch: cudaMalloc failed");
    }
    return PTD_OK;
}

cudaError_t launch_pt_batch(ptd_batch* b, int par, bool check)
{
    const dim3 blk(32, b->cfg.warps2d);
    const bool c = check;
    const PTArgs* t = b->tab[par];
#define PTB(NT, M)                                                                                           \
    (c ? pt2d_batch_kernel<NT, M, true><<<b->nwork, blk, 0, b->s>>>(t, b->work, b->cfg.chunk2d)                \
       : pt2d_batch_kernel<NT, M, false><<<b->nwork, blk, 0, b->s>>>(t, b->work, b->cfg.chunk2d))
    if (b->df64) {
        if (b->model == LIN) PTB(DF64, LIN);
        else if (b->model == LINSTEP) PTB(DF64, LINSTEP);
        else PTB(DF64, NONLIN);
    } else {
        if (b->model == LIN) PTB(F64, LIN);
        else if (b->model == LINSTEP) PTB(F64, LINSTEP);
        else PTB(F64, NONLIN);
    }
#undef PTB
    return cudaGetLastError();
}

cudaError_t launch_dc_batch(ptd_batch* b, int par, bool check)
{
    const dim3 blk(32, b->cfg.warps2d);
    const DcArgs* t = b->dtab[par];
#define DCB(M)                                                                                                 \
    (b->tb == 2 ? (check ? dc2d_tb2_batch_kernel<M, true><<<b->nwork, blk, 0, b->s>>>(t, b->work, b->cfg.chunk2d) \
                         : dc2d_tb2_batch_kernel<M, false><<<b->nwork, blk, 0, b->s>>>(t, b->work, b->cfg.chunk2d)) \
                : (check ? dc2d_batch_kernel<M, true><<<b->nwork, blk, 0, b->s>>>(t, b->work, b->cfg.chunk2d)    \
                         : dc2d_batch_kernel<M, false><<<b->nwork, blk, 0, b->s>>>(t, b->work, b->cfg.chunk2d)))
    if (b->model == LIN) DCB(LIN);
    else if (b->model == LINSTEP) DCB(LINSTEP);
    else DCB(NONLIN);
#undef DCB
    return cudaGetLastError();
}

cudaError_t launch_rb_batch(ptd_batch* b, int par, bool check)
{
    const dim3 blk(32, b->cfg.warps2d);
    const RbArgs* t = b->rbtab[par];
#define RBK(M, C, T) rb2d_batch_kernel<M, C, T><<<b->nwork, blk, 0, b->s>>>(t, b->work, b->active, b->nactive, b->cfg.chunk2d)
#define RBB(M) (b->tb == 2 ? (check ? RBK(M, true, 2) : RBK(M, false, 2)) : (check ? RBK(M, true, 1) : RBK(M, false, 1)))
    if (b->model == LIN) RBB(LIN);
    else if (b->model == LINSTEP) RBB(LINSTEP);
    else RBB(NONLIN);
#undef RBB
#undef RBK
    return cudaGetLastError();
}

// The list of the running instances' work items (after every judge).
cudaError_t compact_rb(ptd_batch* b)
{
    compact_active_kernel<<<1, 256, 0, b->s>>>(b->rdev, b->wfirst, b->wcount, b->ninst, b->active, b->nactive);
    return cudaGetLastError();
}

void build_work(ptd_batch* b, std::vector<int4>& work)
{
    work.clear();
    const int W = b->cfg.warps2d, ch = b->cfg.chunk2d;
    for (int i = 0; i < b->ninst; ++i) {
        // x tiles of 31 updated columns, or 28 for the temporally blocked kernel
        const int tiles = ((b->dc || b->rb) && b->tb == 2) ? (b->inst[i].nx - 2 + 27) / 28
                                                            : (b->inst[i].nx - 2 + 30) / 31;
        const int bx = (tiles + W - 1) / W;
        const int by = (b->inst[i].ny - 2 + ch - 1) / ch;
        for (int y = 0; y < by; ++y)
            for (int x = 0; x < bx; ++x) work.push_back(make_int4(i, x, y, 0));
    }
}

int upload_work(ptd_batch* b)
{
    std::vector<int4> work;
    build_work(b, work);
    if (b->work) cudaFree(b->work);
    b->work = nullptr;
    int rc = balloc(&b->work, work.size() * sizeof(int4));
    if (rc) return rc;
    BCK(cudaMemcpy(b->work, work.data(), work.size() * sizeof(int4), cudaMemcpyHostToDevice));
    b->nwork = (int)work.size();
    // each instance's work items (contiguous): its check slots
    std::vector<int> first(b->ninst, 0), count(b->ninst, 0);
    for (int k = (int)work.size() - 1; k >= 0; --k) {
        first[work[k].x] = k;
        count[work[k].x] += 1;
    }
    if (!b->wfirst) rc = balloc(&b->wfirst, b->ninst * sizeof(int));
    if (!rc && !b->wcount) rc = balloc(&b->wcount, b->ninst * sizeof(int));
    if (rc) return rc;
    BCK(cudaMemcpy(b->wfirst, first.data(), b->ninst * sizeof(int), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->wcount, count.data(), b->ninst * sizeof(int), cudaMemcpyHostToDevice));
    if (b->rb) {
        if (b->active) cudaFree(b->active);
        b->active = nullptr;
        rc = balloc(&b->active, work.size() * sizeof(int));
        if (!rc && !b->nactive) rc = balloc(&b->nactive, sizeof(int));
        if (rc) return rc;
        BCK(cudaMemset(b->nactive, 0, sizeof(int)));
    }
    return PTD_OK;
}

// FP32_RB: one physical step of the batch as one graph (the header comment).
int capture_rb(ptd_batch* b)
{
    if (b->gstep) cudaGraphExecDestroy(b->gstep);
    b->gstep = nullptr;
    cudaGraph_t g = nullptr;
    BCK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle loop;
    cudaError_t err = cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = loop;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (err == cudaSuccess) err = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    if (err != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err, "batch: conditional graph node");
    }
    cudaGraph_t body = np.conditional.phGraph_out[0];
    err = cudaStreamBeginCaptureToGraph(b->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (err != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err, "cudaStreamBeginCaptureToGraph");
    }
    const int n = b->ninst, nb = (n + 3) / 4;   // the check judge: one warp per instance, 4 per block
    const int nl = b->nchk / b->tb;   // launches per check block (tb divides nchk)
    int par = 0, nk = 0;
    for (int blk = 0; blk < b->blocks_per_phase && err == cudaSuccess; ++blk) {
        for (int it = 0; it < nl && err == cudaSuccess; ++it) {
            err = launch_rb_batch(b, par, it == nl - 1);
            par ^= 1;
            ++nk;
        }
        if (err == cudaSuccess) {
            rb_check_judge_batch_kernel<<<nb, 128, 0, b->s>>>(b->rdev, n, b->nchk, b->bp.itmax, b->bp.tol,
                                                              b->norm_den, b->bp.norm == PTD_NORM_MAX, b->parts,
                                                              b->wfirst, b->wcount, b->cfg.warps2d);
            err = cudaGetLastError();
            ++nk;
        }
        if (err == cudaSuccess) {
            err = compact_rb(b);
            ++nk;
        }
    }
    if (err == cudaSuccess) {
        rb_fold_batch_kernel<<<b->nfwork, 256, 0, b->s>>>(b->ftab, b->rdev, b->fwork, b->tb);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) {
        rb_base_batch_kernel<<<b->nfwork, 256, 0, b->s>>>(b->btab, b->rdev, b->fwork, 1);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) {
        rb_base_judge_batch_kernel<<<1, 256, 0, b->s>>>(b->rdev, n, b->bp.tol, b->norm_den,
                                                        b->bp.norm == PTD_NORM_MAX, loop, 1, b->passes,
                                                        b->parts64, b->ffirst, b->fcount);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = compact_rb(b);
    nk += 4;
    cudaError_t e2 = cudaStreamEndCapture(b->s, &body);
    if (err != cudaSuccess || e2 != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err != cudaSuccess ? err : e2, "batch: capture the rebased phase");
    }
    cudaError_t e3 = cudaGraphInstantiate(&b->gstep, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return cuda_fail(e3, "cudaGraphInstantiate");
    b->kernels_per_graph = nk;
    return PTD_OK;
}

int capture(ptd_batch* b)
{
    if (b->rb) return capture_rb(b);
    // FP64 / DF64: the whole step; FP32_DC: one inner solve of every instance
    // in its inner phase.  One graph: a WHILE node whose body is one check
    // block of every running instance (nchk/tb launches and the per-instance
    // judge; two blocks when the launch count is odd, so that every pass starts
    // on buffer parity 0) and the loop judge, which ends the loop once no
    // instance is running.
    if (b->g) cudaGraphExecDestroy(b->g);
    b->g = nullptr;
    cudaGraph_t g = nullptr;
    BCK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle loop;
    cudaError_t err = cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = loop;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (err == cudaSuccess) err = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    cudaGraph_t body = err == cudaSuccess ? np.conditional.phGraph_out[0] : nullptr;
    if (err == cudaSuccess)
        err = cudaStreamBeginCaptureToGraph(b->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (err != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err, "batch capture");
    }
    const int n = b->ninst, nbw = (n + 3) / 4;   // judges: one warp per instance, 4 per block
    const int nl = b->dc ? b->nchk / b->tb : b->nchk;   // launches per check block
    const int nblk = (nl & 1) ? 2 : 1;
    const int W = b->cfg.warps2d, norm_max = b->bp.norm == PTD_NORM_MAX;
    int par = 0, nk = 0;
    for (int blk = 0; blk < nblk && err == cudaSuccess; ++blk) {
        for (int it = 0; it < nl && err == cudaSuccess; ++it) {
            const bool check = it == nl - 1;
            err = b->dc ? launch_dc_batch(b, par, check) : launch_pt_batch(b, par, check);
            par ^= 1;
            ++nk;
        }
        if (err == cudaSuccess) {
            if (b->dc)
                inner_judge_batch_kernel<<<nbw, 128, 0, b->s>>>(b->bst, n, b->nchk, b->bp.itmax, norm_max, b->stall,
                                                                b->parts, b->wfirst, b->wcount, W);
            else
                judge_batch_kernel<<<nbw, 128, 0, b->s>>>(b->st, n, b->nchk, b->bp.itmax, b->bp.tol, b->norm_den,
                                                          norm_max, b->parts, b->wfirst, b->wcount, W);
            err = cudaGetLastError();
            ++nk;
        }
    }
    if (err == cudaSuccess) {
        const int max_passes = b->bp.itmax / b->nchk + 2;
        if (b->dc) batch_loop_judge_kernel<BDev><<<1, 256, 0, b->s>>>(b->bst, n, b->passes, max_passes, loop);
        else batch_loop_judge_kernel<DevState><<<1, 256, 0, b->s>>>(b->st, n, b->passes, max_passes, loop);
        err = cudaGetLastError();
        ++nk;
    }
    cudaError_t e2 = cudaStreamEndCapture(b->s, &body);
    if (err != cudaSuccess || e2 != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err != cudaSuccess ? err : e2, "batch capture");
    }
    cudaError_t e3 = cudaGraphInstantiate(&b->g, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return cuda_fail(e3, "cudaGraphInstantiate");
    b->kernels_per_graph = nk;   // per pass
    return PTD_OK;
}

void one_grid_params(const ptd_batch_params& bp, int nx, int ny, ptd_params& p)
{
    std::memset(&p, 0, sizeof(p));
    p.ndim = 2;
    p.model = bp.model;
    p.nx = nx;
    p.ny = ny;
    p.nz = 1;
    p.lx = bp.lx;
    p.ly = bp.ly;
    p.lz = 1.0;
    p.dt = bp.dt;
    p.nt = bp.nt;
    p.itmax = bp.itmax;
    p.nchk = bp.nchk;
    p.precision = bp.precision;
    p.tol = bp.tol;
    p.cfl = bp.cfl;
    p.resc = bp.resc;
    p.D = bp.D;
    p.norm = bp.norm;
}

// Field work: chunks of every instance's padded fields ({instance, first
// element, count}), and (with cells) of its inner cells.
int build_chunks(ptd_batch* b, bool cells)
{
    std::vector<int4> cw, fw;
    const int CH = 2048;
    for (int i = 0; i < b->ninst; ++i) {
        const Inst& I = b->inst[i];
        const long long nc = (long long)(I.nx - 2) * (I.ny - 2);
        for (long long s0 = 0; cells && s0 < nc; s0 += CH)
            cw.push_back(make_int4(i, (int)s0, (int)std::min<long long>(CH, nc - s0), 0));
        for (long long s0 = 0; s0 < I.nfield; s0 += CH)
            fw.push_back(make_int4(i, (int)s0, (int)std::min<long long>(CH, I.nfield - s0), 0));
    }
    int rc = cells ? balloc(&b->cwork, cw.size() * sizeof(int4)) : PTD_OK;
    if (!rc) rc = balloc(&b->fwork, fw.size() * sizeof(int4));
    if (rc) return rc;
    if (cells) BCK(cudaMemcpy(b->cwork, cw.data(), cw.size() * sizeof(int4), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->fwork, fw.data(), fw.size() * sizeof(int4), cudaMemcpyHostToDevice));
    b->ncwork = (int)cw.size();
    b->nfwork = (int)fw.size();
    return PTD_OK;
}

// FP32_RB: the per-instance argument blocks of the iteration (per buffer
// parity), the fold and the base kernels.
// Residual slots of every form: per-warp check slots, the most warps any
// launch shape gives (28-column tiles at most, up to 8 warps per CTA, rows per
// chunk >= 8: ptd_batch_set_config's bounds), and one FP64 slot per chunk of
// build_chunks -- cell chunks (the FP32_DC residual) or field chunks (the
// FP32_RB base) -- with each instance's chunk range.
int alloc_slots(ptd_batch* b, bool cells)
{
    const int n = b->ninst;
    long long np = 0, nf = 0;
    std::vector<int> ff(n), fc(n);
    for (int i = 0; i < n; ++i) {
        const Inst& I = b->inst[i];
        np += (long long)((I.nx - 2 + 27) / 28 + 7) * ((I.ny - 2 + 7) / 8);
        ff[i] = (int)nf;
        const long long m = cells ? (long long)(I.nx - 2) * (I.ny - 2) : I.nfield;
        fc[i] = (int)((m + 2047) / 2048);   // the chunks of build_chunks
        nf += fc[i];
    }
    int rc = balloc(&b->parts, (size_t)np * sizeof(double));
    if (!rc) rc = balloc(&b->parts64, (size_t)nf * sizeof(double));
    if (!rc) rc = balloc(&b->ffirst, n * sizeof(int));
    if (!rc) rc = balloc(&b->fcount, n * sizeof(int));
    if (rc) return rc;
    b->nparts = np;
    BCK(cudaMemcpy(b->ffirst, ff.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->fcount, fc.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    return PTD_OK;
}

int fill_tables_rb(ptd_batch* b)
{
    const int n = b->ninst;
    {
        const int rc = alloc_slots(b, false);
        if (rc) return rc;
    }
    std::vector<RbArgs> t[2] = {std::vector<RbArgs>(n), std::vector<RbArgs>(n)};
    std::vector<RbFoldArgs> ft(n);
    std::vector<RbBaseArgs> bt(n);
    std::vector<double> nd(n);
    for (int i = 0; i < n; ++i) {
        const Inst& I = b->inst[i];
        const long long o = I.off;
        nd[i] = I.dv.norm_den;
        for (int q = 0; q < 2; ++q) {
            RbArgs& a = t[q][i];
            std::memset(&a, 0, sizeof(a));
            a.nx = I.nx;
            a.ny = I.ny;
            a.nz = 1;
            a.sy = I.sy;
            a.sz = I.nfield;
            a.rdt = (float)I.dv.rdt;
            for (int d = 0; d < 3; ++d) a.sig[d] = (float)I.dv.sig[d];
            a.c_lin = (float)I.dv.c_lin;
            a.e_lin = (float)I.dv.e_lin;
            a.f = fparams(I.dv);
            a.din = b->d[q] + o;
            a.dout = b->d[q ^ 1] + o;
            for (int d = 0; d < 3; ++d) {
                const int dd = d < 2 ? d : 0;
                a.win[d] = b->w32[dd][q] + o;
                a.wout[d] = b->w32[dd][q ^ 1] + o;
                a.tb[d] = b->tb32[dd] + o;
            }
            a.Rb = b->Rb32 + o;
            a.Cb = b->Cb32 + o;
            a.Hf = b->Hf + o;
            a.Df = b->Df ? b->Df + o : nullptr;
            a.skip = &b->rdev[i].skip;
            a.acc = &b->rdev[i].acc;
            a.parts = b->parts;
            a.norm_max = b->bp.norm == PTD_NORM_MAX;
        }
        RbFoldArgs& f = ft[i];
        std::memset(&f, 0, sizeof(f));
        f.n = I.nfield;
        f.H = b->H64 + o;
        f.ndim = 2;
        f.d[0] = b->d[0] + o;
        f.d[1] = b->d[1] + o;
        for (int d = 0; d < 2; ++d) {
            f.wb[d] = b->wb64[d] + o;
            f.w[d][0] = b->w32[d][0] + o;
            f.w[d][1] = b->w32[d][1] + o;
        }
        RbBaseArgs& g = bt[i];
        std::memset(&g, 0, sizeof(g));
        g.nx = I.nx;
        g.ny = I.ny;
        g.nz = 1;
        g.ndim = 2;
        g.model = b->model;
        g.sy = I.sy;
        g.sz = I.nfield;
        g.rdt = I.dv.rdt;
        for (int d = 0; d < 3; ++d) g.sig[d] = I.dv.sig[d];
        g.H = b->H64 + o;
        g.Hold = b->Hold64 + o;
        for (int d = 0; d < 2; ++d) {
            g.wb[d] = b->wb64[d] + o;
            g.tb[d] = b->tb32[d] + o;
        }
        g.D = b->D64 ? b->D64 + o : nullptr;
        g.Rb = b->Rb32 + o;
        g.Cb = b->Cb32 + o;
        g.Hf = b->Hf + o;
        g.acc64 = &b->rdev[i].acc64;
        g.parts = b->parts64;
        g.norm_max = b->bp.norm == PTD_NORM_MAX;
    }
    for (int q = 0; q < 2; ++q)
        BCK(cudaMemcpy(b->rbtab[q], t[q].data(), n * sizeof(RbArgs), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->ftab, ft.data(), n * sizeof(RbFoldArgs), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->btab, bt.data(), n * sizeof(RbBaseArgs), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->norm_den, nd.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    return build_chunks(b, false);
}

int fill_tables(ptd_batch* b)
{
    if (b->rb) return fill_tables_rb(b);
    const int n = b->ninst;
    {
        const int rc = alloc_slots(b, b->dc);
        if (rc) return rc;
    }
    if (!b->dc) {
        std::vector<PTArgs> t[2] = {std::vector<PTArgs>(n), std::vector<PTArgs>(n)};
        std::vector<double> nd(n);
        const size_t es = sizeof(double);   // bytes per element (double or float2)
        for (int i = 0; i < n; ++i) {
            const Inst& I = b->inst[i];
            nd[i] = I.dv.norm_den;
            for (int q = 0; q < 2; ++q) {
                PTArgs& a = t[q][i];
                fill_args(I.p, I.dv, a);
                a.sy = I.sy;
                a.sz = I.nfield;
                auto at = [&](void* base) -> char* { return (char*)base + (size_t)I.off * es; };
                a.Hin = at(b->H[q]);
                a.Hout = at(b->H[q ^ 1]);
                a.Hold = at(b->Hold);
                for (int d = 0; d < 3; ++d) {
                    a.win[d] = at(b->W[d < 2 ? d : 0][q]);
                    a.wout[d] = at(b->W[d < 2 ? d : 0][q ^ 1]);
                }
                a.D = b->D ? at(b->D) : nullptr;
                a.done = &b->st[i].done;
                a.acc = &b->st[i].acc;
                a.parts = b->parts;
            }
        }
        for (int q = 0; q < 2; ++q)
            BCK(cudaMemcpy(b->tab[q], t[q].data(), n * sizeof(PTArgs), cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(b->norm_den, nd.data(), n * sizeof(double), cudaMemcpyHostToDevice));
        return PTD_OK;
    }
    std::vector<DcArgs> t[2] = {std::vector<DcArgs>(n), std::vector<DcArgs>(n)};
    std::vector<PTArgs> r(n);
    std::vector<float*> rp(n);
    std::vector<double*> hp(n);
    std::vector<BDev> bd(n);
    for (int i = 0; i < n; ++i) {
        const Inst& I = b->inst[i];
        for (int q = 0; q < 2; ++q) {
            DcArgs& a = t[q][i];
            std::memset(&a, 0, sizeof(a));
            a.nx = I.nx;
            a.ny = I.ny;
            a.nz = 1;
            a.sy = I.sy;
            a.sz = I.nfield;
            a.rdt = (float)I.dv.rdt;
            for (int d = 0; d < 3; ++d) a.sig[d] = (float)I.dv.sig[d];
            a.c_lin = (float)I.dv.c_lin;
            a.e_lin = (float)I.dv.e_lin;
            a.f = fparams(I.dv);
            a.din = b->d[q] + I.off;
            a.dout = b->d[q ^ 1] + I.off;
            for (int d = 0; d < 3; ++d) {
                a.win[d] = b->w32[d < 2 ? d : 0][q] + I.off;
                a.wout[d] = b->w32[d < 2 ? d : 0][q ^ 1] + I.off;
            }
            a.Hf = b->Hf + I.off;
            a.Df = b->Df ? b->Df + I.off : nullptr;
            a.r = b->rf + I.off;
            a.done = &b->bst[i].done;
            a.acc = &b->bst[i].acc;
            a.parts = b->parts;
            a.norm_max = b->bp.norm == PTD_NORM_MAX;
        }
        PTArgs& a = r[i];
        fill_args(I.p, I.dv, a);
        a.sy = I.sy;
        a.sz = I.nfield;
        a.Hin = b->H64 + I.off;
        a.Hold = b->Hold64 + I.off;
        a.D = b->D64 ? b->D64 + I.off : nullptr;
        rp[i] = b->rf + I.off;
        hp[i] = b->H64 + I.off;
        std::memset(&bd[i], 0, sizeof(BDev));
        bd[i].norm_den = I.dv.norm_den;
        double cs = 0.0;
        for (int d = 0; d < 2; ++d) cs += 4.0 / (I.dv.h[d] * I.dv.h[d]);
        bd[i].cond_scale = cs * b->bp.dt;
        bd[i].dconst = b->bp.D;
        bd[i].done = 1;
        bd[i].phase = PH_CONVERGED;
    }
    for (int q = 0; q < 2; ++q)
        BCK(cudaMemcpy(b->dtab[q], t[q].data(), n * sizeof(DcArgs), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->rtab, r.data(), n * sizeof(PTArgs), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->rf_ptrs, rp.data(), n * sizeof(float*), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->H_ptrs, hp.data(), n * sizeof(double*), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->bst, bd.data(), n * sizeof(BDev), cudaMemcpyHostToDevice));
    // cell work (inner cells, residual) and field work (whole fields, apply)
    return build_chunks(b, true);
}

void free_batch(ptd_batch* b)
{
    if (!b) return;
    if (b->s) cudaStreamSynchronize(b->s);
    if (b->g) cudaGraphExecDestroy(b->g);
    if (b->gstep) cudaGraphExecDestroy(b->gstep);
    void* rbp[] = {b->wb64[0], b->wb64[1], b->tb32[0], b->tb32[1], b->Rb32, b->Cb32, b->rdev,
                   b->rbtab[0], b->rbtab[1], b->ftab, b->btab, b->passes, b->wfirst, b->wcount,
                   b->active, b->nactive, b->packed, b->pinst, b->pwork, b->parts, b->parts64,
                   b->ffirst, b->fcount};
    for (void* p : rbp) cudaFree(p);
    if (b->h_rdev) cudaFreeHost(b->h_rdev);
    if (b->h_passes) cudaFreeHost(b->h_passes);
    void* ptrs[] = {b->H[0], b->H[1], b->Hold, b->W[0][0], b->W[0][1], b->W[1][0], b->W[1][1], b->D,
                    b->stage, b->st, b->norm_den, b->tab[0], b->tab[1], b->H64, b->Hold64, b->D64, b->Hf,
                    b->Df, b->rf, b->d[0], b->d[1], b->w32[0][0], b->w32[0][1], b->w32[1][0], b->w32[1][1],
                    b->bst, b->dtab[0], b->dtab[1], b->rtab, b->rf_ptrs, b->H_ptrs, b->cur_parity,
                    b->cwork, b->fwork, b->work};
    for (void* p : ptrs) cudaFree(p);
    if (b->h_st) cudaFreeHost(b->h_st);
    if (b->h_bst) cudaFreeHost(b->h_bst);
    for (int k = 0; k < 4; ++k) {
        if (b->ev_join[k]) cudaEventDestroy(b->ev_join[k]);
        if (b->cs[k]) cudaStreamDestroy(b->cs[k]);
    }
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->s) cudaStreamDestroy(b->s);
    delete b;
}

// The packed layout: instance i's nx*ny values at poff_i (x fastest, no
// padding), and its conversion table.
int setup_packing(ptd_batch* b)
{
    std::vector<PackInst> pi(b->ninst);
    std::vector<int4> pw;
    long long poff = 0;
    const int CH = 4096;
    for (int i = 0; i < b->ninst; ++i) {
        const Inst& I = b->inst[i];
        pi[i] = PackInst{poff, I.off, I.sy, I.nx, 0};
        const long long n = (long long)I.nx * I.ny;
        for (long long s0 = 0; s0 < n; s0 += CH)
            pw.push_back(make_int4(i, (int)s0, (int)std::min<long long>(CH, n - s0), 0));
        poff += n;
    }
    int rc = balloc(&b->packed, (size_t)poff * sizeof(double));
    if (!rc) rc = balloc(&b->pinst, pi.size() * sizeof(PackInst));
    if (!rc) rc = balloc(&b->pwork, pw.size() * sizeof(int4));
    if (rc) return rc;
    BCK(cudaMemcpy(b->pinst, pi.data(), pi.size() * sizeof(PackInst), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->pwork, pw.data(), pw.size() * sizeof(int4), cudaMemcpyHostToDevice));
    b->npwork = (int)pw.size();
    return PTD_OK;
}

// The instances' copies between the caller's arrays and the packed buffer,
// instance i on copy stream i % 4, after the work queued so far on the
// solver's stream and before the work queued on it next.
int copy_instances(ptd_batch* b, double* const* dst, const double* const* src, bool to_packed)
{
    BCK(cudaEventRecord(b->ev_fork, b->s));
    for (int k = 0; k < 4; ++k) BCK(cudaStreamWaitEvent(b->cs[k], b->ev_fork, 0));
    long long poff = 0;
    for (int i = 0; i < b->ninst; ++i) {
        const Inst& I = b->inst[i];
        const size_t n = (size_t)I.nx * I.ny;
        if (to_packed)
            BCK(cudaMemcpyAsync(b->packed + poff, src[i], n * sizeof(double), cudaMemcpyDefault, b->cs[i % 4]));
        else
            BCK(cudaMemcpyAsync(dst[i], b->packed + poff, n * sizeof(double), cudaMemcpyDefault, b->cs[i % 4]));
        poff += (long long)n;
    }
    for (int k = 0; k < 4; ++k) {
        BCK(cudaEventRecord(b->ev_join[k], b->cs[k]));
        BCK(cudaStreamWaitEvent(b->s, b->ev_join[k], 0));
    }
    return PTD_OK;
}

// Upload instance fields: src[i] (nx_i*ny_i doubles, host or device) into
// the concatenated padded field dst (FP64): one contiguous copy per instance
// into the packed buffer, then one conversion kernel.
int upload(ptd_batch* b, double* dst, const double* const* src)
{
    const int rc = copy_instances(b, nullptr, src, true);
    if (rc) return rc;
    unpack_batch_kernel<<<b->npwork, 256, 0, b->s>>>(b->packed, dst, b->pinst, b->pwork);
    BCK(cudaGetLastError());
    return PTD_OK;
}

int download(ptd_batch* b, double* const* dst, const double* src)
{
    pack_batch_kernel<<<b->npwork, 256, 0, b->s>>>(src, b->packed, b->pinst, b->pwork);
    BCK(cudaGetLastError());
    return copy_instances(b, dst, nullptr, false);
}

}  // namespace

extern "C" int ptd_batch_params_init(ptd_batch_params* p, int32_t ninst, int32_t model)
{
    if (!p) return bfail(PTD_EINVAL, "ptd_batch_params_init: p is NULL");
    if (ninst < 1) return bfail(PTD_EINVAL, "ninst must be >= 1");
    ptd_params q;
    int rc = ptd_params_init(&q, 2, model);
    if (rc) return rc;
    std::memset(p, 0, sizeof(*p));
    p->ninst = ninst;
    p->model = model;
    p->lx = q.lx;
    p->ly = q.ly;
    p->dt = q.dt;
    p->nt = q.nt;
    p->itmax = q.itmax;
    p->nchk = q.nchk;
    p->precision = PTD_PREC_FP64;
    p->tol = q.tol;
    p->cfl = q.cfl;
    p->resc = q.resc;
    p->D = q.D;
    p->norm = PTD_NORM_RMS;
    return PTD_OK;
}

extern "C" int ptd_batch_create(ptd_batch** out, const ptd_batch_params* p, const int32_t* nx, const int32_t* ny)
{
    if (!out) return bfail(PTD_EINVAL, "ptd_batch_create: out is NULL");
    *out = nullptr;
    if (!p || !nx || !ny) return bfail(PTD_EINVAL, "ptd_batch_create: NULL argument");
    if (p->ninst < 1) return bfail(PTD_EINVAL, "ninst must be >= 1");
    if (p->nchk < 1 || p->itmax < p->nchk || p->itmax % p->nchk)
        return bfail(PTD_EINVAL, "batch: itmax must be a positive multiple of nchk");
    for (int k = 0; k < 8; ++k)
        if (p->reserved[k]) return bfail(PTD_EINVAL, "reserved fields must be zero");
    if (p->precision == PTD_PREC_DFH) return bfail(PTD_EINVAL, "batch: precision FP64, DF64, FP32_DC or FP32_RB");
    ptd_batch* b = new (std::nothrow) ptd_batch();
    if (!b) return bfail(PTD_ENOMEM, "batch: host allocation failed");
    b->bp = *p;
    b->ninst = p->ninst;
    b->model = p->model;
    b->df64 = p->precision == PTD_PREC_DF64;
    b->dc = p->precision == PTD_PREC_FP32_DC;
    b->rb = p->precision == PTD_PREC_FP32_RB;
    b->inst.resize(b->ninst);
    long long off = 0;
    int rc = PTD_OK;
    for (int i = 0; i < b->ninst && !rc; ++i) {
        Inst& I = b->inst[i];
        one_grid_params(*p, nx[i], ny[i], I.p);
        rc = validate(&I.p);
        if (rc) break;
        derive(I.p, I.dv);
        I.nx = nx[i];
        I.ny = ny[i];
        I.sy = ((nx[i] + 31) / 32) * 32;
        I.nfield = I.sy * ny[i];
        I.off = off;
        off += ((I.nfield + 63) / 64) * 64;
        if (off > kMaxCells) rc = bfail(PTD_EINVAL, "batch: the instances hold more than 2^40 cells in all");
    }
    if (rc) {
        delete b;
        return rc;
    }
    b->total = off;
    {
        ptd_params q = b->inst[0].p;
        int nmax = 0;
        for (auto& I : b->inst) nmax = std::max(nmax, std::max(I.nx, I.ny));
        q.nx = q.ny = nmax;
        b->cfg = tuned_config(q);
        b->cfg.chunk2d = 32;
        b->stall = std::max(10, (2 * nmax + 49) / 50);
    }
    b->nchk = b->dc ? std::max(1, std::min(p->nchk, 50)) : p->nchk;
    if (b->dc && p->itmax % b->nchk) b->nchk = p->nchk;
    b->tb = ((b->dc || b->rb) && b->nchk % 2 == 0 && !(p->flags & PTD_FLAG_DC_NO_TBLOCK)) ? 2 : 1;
    // FP32_RB: a phase is the check blocks of ~200 iterations between two rebases
    b->blocks_per_phase = std::max(1, (200 + b->nchk - 1) / b->nchk);
    cudaError_t e = cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking);
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
        e = cudaStreamCreateWithFlags(&b->cs[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        free_batch(b);
        return cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    const size_t db = (size_t)b->total * sizeof(double), fb = (size_t)b->total * sizeof(float);
    const int n = b->ninst;
    if (b->rb) {
        const bool ls = p->model == PTD_MODEL_LINSTEP;
        rc = balloc(&b->H64, db);
        if (!rc) rc = balloc(&b->Hold64, db);
        if (!rc && ls) rc = balloc(&b->D64, db);
        if (!rc) rc = balloc(&b->Hf, fb);
        if (!rc && ls) rc = balloc(&b->Df, fb);
        for (int q = 0; q < 2 && !rc; ++q) rc = balloc(&b->d[q], fb);
        for (int d = 0; d < 2 && !rc; ++d) {
            for (int q = 0; q < 2 && !rc; ++q) rc = balloc(&b->w32[d][q], fb);
            if (!rc) rc = balloc(&b->wb64[d], db);
            if (!rc) rc = balloc(&b->tb32[d], fb);
        }
        if (!rc) rc = balloc(&b->Rb32, fb);
        if (!rc) rc = balloc(&b->Cb32, fb);
        if (!rc) rc = balloc(&b->rdev, n * sizeof(RbDev));
        for (int q = 0; q < 2 && !rc; ++q) rc = balloc(&b->rbtab[q], n * sizeof(RbArgs));
        if (!rc) rc = balloc(&b->ftab, n * sizeof(RbFoldArgs));
        if (!rc) rc = balloc(&b->btab, n * sizeof(RbBaseArgs));
        if (!rc) rc = balloc(&b->norm_den, n * sizeof(double));
        if (!rc && cudaMallocHost((void**)&b->h_rdev, n * sizeof(RbDev)) != cudaSuccess)
            rc = bfail(PTD_ENOMEM, "batch: cudaMallocHost failed");
        if (!rc) {
            double* zd[] = {b->wb64[0], b->wb64[1]};
            for (double* z : zd)
                if (cudaMemset(z, 0, db) != cudaSuccess) rc = bfail(PTD_ECUDA, "batch: cudaMemset failed");
            // faces past the last one of each direction are read (never used) by the halo lanes
            float* zf[] = {b->tb32[0], b->tb32[1], b->Rb32, b->Cb32};
            for (float* z : zf)
                if (cudaMemset(z, 0, fb) != cudaSuccess) rc = bfail(PTD_ECUDA, "batch: cudaMemset failed");
            if (cudaMemset(b->rdev, 0, n * sizeof(RbDev)) != cudaSuccess)
                rc = bfail(PTD_ECUDA, "batch: cudaMemset failed");
        }
    } else if (!b->dc) {
        for (int q = 0; q < 2 && !rc; ++q) rc = balloc(&b->H[q], db);
        if (!rc) rc = balloc(&b->Hold, db);
        for (int d = 0; d < 2 && !rc; ++d)
            for (int q = 0; q < 2 && !rc; ++q) rc = balloc(&b->W[d][q], db);
        if (!rc && p->model == PTD_MODEL_LINSTEP) rc = balloc(&b->D, db);
        if (!rc && b->df64) rc = balloc(&b->stage, db);
        if (!rc) rc = balloc(&b->st, n * sizeof(DevState));
        if (!rc) rc = balloc(&b->norm_den, n * sizeof(double));
        for (int q = 0; q < 2 && !rc; ++q) rc = balloc(&b->tab[q], n * sizeof(PTArgs));
        if (!rc && cudaMallocHost((void**)&b->h_st, n * sizeof(DevState)) != cudaSuccess)
            rc = bfail(PTD_ENOMEM, "batch: cudaMallocHost failed");
        if (!rc) {
            e = cudaMemset(b->st, 0, n * sizeof(DevState));
            if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemset");
        }
    } else {
        if (!rc) rc = balloc(&b->H64, db);
        if (!rc) rc = balloc(&b->Hold64, db);
        if (!rc && p->model == PTD_MODEL_LINSTEP) rc = balloc(&b->D64, db);
        if (!rc) rc = balloc(&b->Hf, fb);
        if (!rc && p->model == PTD_MODEL_LINSTEP) rc = balloc(&b->Df, fb);
        if (!rc) rc = balloc(&b->rf, fb);
        for (int q = 0; q < 2 && !rc; ++q) rc = balloc(&b->d[q], fb);
        for (int d = 0; d < 2 && !rc; ++d)
            for (int q = 0; q < 2 && !rc; ++q) rc = balloc(&b->w32[d][q], fb);
        if (!rc) rc = balloc(&b->bst, n * sizeof(BDev));
        for (int q = 0; q < 2 && !rc; ++q) rc = balloc(&b->dtab[q], n * sizeof(DcArgs));
        if (!rc) rc = balloc(&b->rtab, n * sizeof(PTArgs));
        if (!rc) rc = balloc(&b->rf_ptrs, n * sizeof(float*));
        if (!rc) rc = balloc(&b->H_ptrs, n * sizeof(double*));
        if (!rc) rc = balloc(&b->cur_parity, n * sizeof(int));
        if (!rc && cudaMallocHost((void**)&b->h_bst, n * sizeof(BDev)) != cudaSuccess)
            rc = bfail(PTD_ENOMEM, "batch: cudaMallocHost failed");
    }
    if (!rc) rc = balloc(&b->passes, sizeof(int));   // passes of a solve graph's loop
    if (!rc && cudaMallocHost((void**)&b->h_passes, sizeof(int)) != cudaSuccess)
        rc = bfail(PTD_ENOMEM, "batch: cudaMallocHost failed");
    if (!rc) {
        void* zs[] = {b->H[0], b->H[1], b->Hold, b->W[0][0], b->W[0][1], b->W[1][0], b->W[1][1], b->D,
                      b->H64, b->Hold64, b->D64};
        for (void* z : zs)
            if (z && cudaMemset(z, 0, db) != cudaSuccess) rc = bfail(PTD_ECUDA, "batch: cudaMemset failed");
        float* zf[] = {b->Hf, b->Df, b->rf, b->d[0], b->d[1], b->w32[0][0], b->w32[0][1], b->w32[1][0],
                       b->w32[1][1]};
        for (float* z : zf)
            if (z && cudaMemset(z, 0, fb) != cudaSuccess) rc = bfail(PTD_ECUDA, "batch: cudaMemset failed");
    }
    if (!rc) rc = fill_tables(b);
    if (!rc) rc = setup_packing(b);
    if (!rc) rc = upload_work(b);
    if (!rc) rc = capture(b);
    if (rc) {
        free_batch(b);
        return rc;
    }
    *out = b;
    return PTD_OK;
}

extern "C" void ptd_batch_destroy(ptd_batch* b) { free_batch(b); }

extern "C" int ptd_batch_counters(ptd_batch* b, int64_t* launches, int64_t* iterations)
{
    if (!b) return bfail(PTD_EINVAL, "batch is NULL");
    if (launches) *launches = b->launches;
    if (iterations) *iterations = b->iterations;
    return PTD_OK;
}

static int batch_read_states(ptd_batch* b)
{
    if (b->rb) BCK(cudaMemcpyAsync(b->h_rdev, b->rdev, b->ninst * sizeof(RbDev), cudaMemcpyDeviceToHost, b->s));
    else if (b->dc) BCK(cudaMemcpyAsync(b->h_bst, b->bst, b->ninst * sizeof(BDev), cudaMemcpyDeviceToHost, b->s));
    else BCK(cudaMemcpyAsync(b->h_st, b->st, b->ninst * sizeof(DevState), cudaMemcpyDeviceToHost, b->s));
    BCK(cudaStreamSynchronize(b->s));
    return PTD_OK;
}

// Plain PT: one physical step of every instance.
static int batch_pt_step(ptd_batch* b, int32_t* iters, double* err_last, int* nan_any)
{
    const int n = b->ninst, tb = 128, nb = (n + tb - 1) / tb;
    reset_batch_kernel<<<nb, tb, 0, b->s>>>(b->st, n);
    BCK(cudaGetLastError());
    b->launches += 1;
    // the whole step: one graph launch, ended on the device
    BCK(cudaMemsetAsync(b->passes, 0, sizeof(int), b->s));
    if (b->nchk <= b->bp.itmax) BCK(cudaGraphLaunch(b->g, b->s));
    BCK(cudaMemcpyAsync(b->h_passes, b->passes, sizeof(int), cudaMemcpyDeviceToHost, b->s));
    {
        const int rc = batch_read_states(b);
        if (rc) return rc;
    }
    b->launches += (long long)(*b->h_passes) * b->kernels_per_graph;
    // bring every instance back to parity 0, then Hold <- H
    const size_t es = sizeof(double);
    for (int i = 0; i < n; ++i) {
        const DevState& s = b->h_st[i];
        iters[i] = s.iter;
        b->iterations += s.iter;
        if (err_last) err_last[i] = s.err;
        if (s.done == DONE_NAN) *nan_any = 1;
        if (s.iter & 1) {
            const Inst& I = b->inst[i];
            const size_t bytes = (size_t)I.nfield * es, o = (size_t)I.off * es;
            BCK(cudaMemcpyAsync((char*)b->H[0] + o, (char*)b->H[1] + o, bytes, cudaMemcpyDeviceToDevice, b->s));
            for (int d = 0; d < 2; ++d)
                BCK(cudaMemcpyAsync((char*)b->W[d][0] + o, (char*)b->W[d][1] + o, bytes, cudaMemcpyDeviceToDevice,
                                    b->s));
        }
    }
    BCK(cudaMemcpyAsync(b->Hold, b->H[0], (size_t)b->total * es, cudaMemcpyDeviceToDevice, b->s));
    return PTD_OK;
}

static int batch_residual(ptd_batch* b)
{
    if (b->model == LIN)
        resid64_batch_kernel<LIN><<<b->ncwork, 256, 0, b->s>>>(b->rtab, b->bst, b->rf_ptrs, b->cwork, b->parts64);
    else if (b->model == LINSTEP)
        resid64_batch_kernel<LINSTEP><<<b->ncwork, 256, 0, b->s>>>(b->rtab, b->bst, b->rf_ptrs, b->cwork, b->parts64);
    else resid64_batch_kernel<NONLIN><<<b->ncwork, 256, 0, b->s>>>(b->rtab, b->bst, b->rf_ptrs, b->cwork, b->parts64);
    BCK(cudaGetLastError());
    const int n = b->ninst, nbw = (n + 3) / 4;   // one warp per instance, 4 per block
    const double rtol = b->bp.dc_inner_rtol > 0.0 ? b->bp.dc_inner_rtol : 1e-3;
    const int max_outer = b->bp.dc_max_outer > 0 ? b->bp.dc_max_outer : 30;
    outer_judge_batch_kernel<<<nbw, 128, 0, b->s>>>(b->bst, n, b->bp.norm == PTD_NORM_MAX, b->bp.tol, rtol,
                                                    max_outer, b->bp.itmax, b->model == NONLIN, b->parts64, b->ffirst,
                                                    b->fcount);
    BCK(cudaGetLastError());
    b->launches += 2;
    return PTD_OK;
}

// FP32 defect correction: one physical step of every instance.
static int batch_dc_step(ptd_batch* b, int32_t* iters, double* err_last, int* nan_any, int* capped_any)
{
    const int n = b->ninst, tb = 128, nb = (n + tb - 1) / tb;
    start_batch_kernel<<<nb, tb, 0, b->s>>>(b->bst, n);
    BCK(cudaGetLastError());
    int rc = batch_residual(b);
    if (rc) return rc;
    for (int round = 0; round < 4 * 64; ++round) {
        rc = batch_read_states(b);
        if (rc) return rc;
        bool all_fin = true, any_inner = false;
        for (int i = 0; i < n; ++i) {
            all_fin = all_fin && b->h_bst[i].phase >= PH_CONVERGED;
            any_inner = any_inner || b->h_bst[i].phase == PH_INNER;
        }
        if (all_fin) break;
        if (any_inner) {
            zero_batch_kernel<<<b->nfwork, 256, 0, b->s>>>(b->dtab[0], b->bst, b->fwork, 2);
            BCK(cudaGetLastError());
            b->launches += 1;
            // the inner solves: one graph launch, ended on the device
            BCK(cudaMemsetAsync(b->passes, 0, sizeof(int), b->s));
            BCK(cudaGraphLaunch(b->g, b->s));
            BCK(cudaMemcpyAsync(b->h_passes, b->passes, sizeof(int), cudaMemcpyDeviceToHost, b->s));
            rc = batch_read_states(b);
            if (rc) return rc;
            b->launches += (long long)(*b->h_passes) * b->kernels_per_graph;
            for (int i = 0; i < n; ++i)
                if (b->h_bst[i].phase == PH_INNER) b->iterations += b->h_bst[i].iter;
            parity_batch_kernel<<<nb, tb, 0, b->s>>>(b->bst, b->cur_parity, n, b->tb);
            BCK(cudaGetLastError());
        }
        apply_batch_kernel<<<b->nfwork, 256, 0, b->s>>>(b->dtab[0], b->bst, b->fwork, b->H_ptrs, b->cur_parity);
        BCK(cudaGetLastError());
        b->launches += 2;
        rc = batch_residual(b);
        if (rc) return rc;
    }
    for (int i = 0; i < n; ++i) {
        const BDev& s = b->h_bst[i];
        iters[i] = s.total_inner;
        if (err_last) err_last[i] = s.err_ref;
        if (s.phase == PH_NAN) *nan_any = 1;
        if (s.phase == PH_CAPPED || s.phase < PH_CONVERGED) *capped_any = 1;
    }
    BCK(cudaMemcpyAsync(b->Hold64, b->H64, (size_t)b->total * sizeof(double), cudaMemcpyDeviceToDevice, b->s));
    return PTD_OK;
}

// FP32_RB: one physical step of every instance -- the base quantities of the
// step's start state, then the step graph (phases until every instance has
// stopped).  An instance that reaches itmax stops at its last full check
// block.
static int batch_rb_step(ptd_batch* b, int32_t* iters, double* err_last, int* nan_any, int* capped_any)
{
    const int n = b->ninst, nb = (n + 127) / 128;
    rb_reset_batch_kernel<<<nb, 128, 0, b->s>>>(b->rdev, n);
    BCK(cudaGetLastError());
    rb_base_batch_kernel<<<b->nfwork, 256, 0, b->s>>>(b->btab, b->rdev, b->fwork, 0);
    BCK(cudaGetLastError());
    rb_base_judge_batch_kernel<<<1, 256, 0, b->s>>>(b->rdev, n, b->bp.tol, b->norm_den, b->bp.norm == PTD_NORM_MAX,
                                                    cudaGraphConditionalHandle{}, 0, b->passes, b->parts64,
                                                    b->ffirst, b->fcount);
    BCK(cudaGetLastError());
    BCK(compact_rb(b));
    BCK(cudaMemsetAsync(b->passes, 0, sizeof(int), b->s));
    b->launches += 4;
    if (b->nchk <= b->bp.itmax) BCK(cudaGraphLaunch(b->gstep, b->s));
    BCK(cudaMemcpyAsync(b->h_passes, b->passes, sizeof(int), cudaMemcpyDeviceToHost, b->s));
    int rc = batch_read_states(b);
    if (rc) return rc;
    b->launches += (long long)(*b->h_passes) * b->kernels_per_graph;
    for (int i = 0; i < n; ++i) {
        const RbDev& st = b->h_rdev[i];
        iters[i] = st.iter;
        b->iterations += st.iter;
        if (err_last) err_last[i] = st.err64;
        if (st.step_done == DONE_NAN) *nan_any = 1;
        if (st.step_done == DONE_CAP || st.step_done == DONE_RUNNING) *capped_any = 1;
    }
    BCK(cudaMemcpyAsync(b->Hold64, b->H64, (size_t)b->total * sizeof(double), cudaMemcpyDeviceToDevice, b->s));
    return PTD_OK;
}

extern "C" int ptd_batch_solve(ptd_batch* b, double* const* H, const double* const* D, int32_t* iters,
                               double* err_last, int32_t* n_done)
{
    if (!b) return bfail(PTD_EINVAL, "batch is NULL");
    if (!H || !iters) return bfail(PTD_EINVAL, "ptd_batch_solve: H and iters are required");
    if (b->model == PTD_MODEL_LINSTEP && !D) return bfail(PTD_EINVAL, "the step model needs D");
    for (int i = 0; i < b->ninst; ++i)
        if (!H[i] || (b->model == PTD_MODEL_LINSTEP && !D[i])) return bfail(PTD_EINVAL, "NULL instance field");
    const size_t db = (size_t)b->total * sizeof(double);
    int rc;
    const int n = b->ninst;
    if (b->rb) {
        const size_t fb = (size_t)b->total * sizeof(float);
        BCK(cudaMemsetAsync(b->H64, 0, db, b->s));
        if ((rc = upload(b, b->H64, H))) return rc;
        BCK(cudaMemcpyAsync(b->Hold64, b->H64, db, cudaMemcpyDeviceToDevice, b->s));
        for (int d = 0; d < 2; ++d) {
            BCK(cudaMemsetAsync(b->wb64[d], 0, db, b->s));
            for (int q = 0; q < 2; ++q) BCK(cudaMemsetAsync(b->w32[d][q], 0, fb, b->s));
        }
        for (int q = 0; q < 2; ++q) BCK(cudaMemsetAsync(b->d[q], 0, fb, b->s));
        if (b->D64) {
            BCK(cudaMemsetAsync(b->D64, 0, db, b->s));
            if ((rc = upload(b, b->D64, D))) return rc;
            tofloat_batch_kernel<<<fill_blocks(), 256, 0, b->s>>>(b->D64, b->Df, b->total);
            BCK(cudaGetLastError());
        }
    } else if (!b->dc) {
        double* h0 = b->df64 ? b->stage : (double*)b->H[0];
        BCK(cudaMemsetAsync(h0, 0, db, b->s));
        if ((rc = upload(b, h0, H))) return rc;
        if (b->df64) BCK(launch_to_df64(h0, b->H[0], b->total, b->s));
        BCK(cudaMemcpyAsync(b->H[1], b->H[0], db, cudaMemcpyDeviceToDevice, b->s));
        BCK(cudaMemcpyAsync(b->Hold, b->H[0], db, cudaMemcpyDeviceToDevice, b->s));
        for (int d = 0; d < 2; ++d)
            for (int q = 0; q < 2; ++q) BCK(cudaMemsetAsync(b->W[d][q], 0, db, b->s));
        if (b->D) {
            double* d0 = b->df64 ? b->stage : (double*)b->D;
            BCK(cudaMemsetAsync(d0, 0, db, b->s));
            if ((rc = upload(b, d0, D))) return rc;
            if (b->df64) BCK(launch_to_df64(d0, b->D, b->total, b->s));
        }
    } else {
        BCK(cudaMemsetAsync(b->H64, 0, db, b->s));
        if ((rc = upload(b, b->H64, H))) return rc;
        BCK(cudaMemcpyAsync(b->Hold64, b->H64, db, cudaMemcpyDeviceToDevice, b->s));
        tofloat_batch_kernel<<<fill_blocks(), 256, 0, b->s>>>(b->H64, b->Hf, b->total);
        BCK(cudaGetLastError());
        if (b->D64) {
            BCK(cudaMemsetAsync(b->D64, 0, db, b->s));
            if ((rc = upload(b, b->D64, D))) return rc;
            tofloat_batch_kernel<<<fill_blocks(), 256, 0, b->s>>>(b->D64, b->Df, b->total);
            BCK(cudaGetLastError());
        }
        BCK(cudaMemsetAsync(b->rf, 0, (size_t)b->total * sizeof(float), b->s));
        BCK(cudaMemsetAsync(b->cur_parity, 0, n * sizeof(int), b->s));
    }
    std::vector<int32_t> it(n);
    int nan_any = 0, capped_any = 0;
    for (int step = 0; step < b->bp.nt; ++step) {
        rc = b->rb   ? batch_rb_step(b, it.data(), err_last, &nan_any, &capped_any)
             : b->dc ? batch_dc_step(b, it.data(), err_last, &nan_any, &capped_any)
                     : batch_pt_step(b, it.data(), err_last, &nan_any);
        if (rc) return rc;
        for (int i = 0; i < n; ++i) iters[(size_t)i * b->bp.nt + step] = it[i];
        if (nan_any) break;
    }
    if (!b->dc && b->df64) {
        BCK(launch_from_df64(b->H[0], b->stage, b->total, b->s));
        rc = download(b, H, b->stage);
    } else {
        rc = download(b, H, (b->dc || b->rb) ? b->H64 : (double*)b->H[0]);
    }
    if (rc) return rc;
    BCK(cudaStreamSynchronize(b->s));
    if (n_done) *n_done = n;
    if (nan_any) return bfail(PTD_ENAN, "an instance's residual is NaN");
    if ((b->bp.flags & PTD_FLAG_STRICT) && capped_any) return bfail(PTD_ENOTCONV, "an instance did not converge");
    return PTD_OK;
}

// Autotuner: time each (warps per block, rows per y chunk[, iterations per
// launch]) candidate on the current state with a few plain launches, keep the
// fastest per inner iteration, re-capture.  FP32_DC with an even check cadence
// also tries the temporally blocked kernel (two iterations per launch).
extern "C" int ptd_batch_tune(ptd_batch* b, int32_t* warps_out, int32_t* chunk_out, float* us_out)
{
    if (!b) return bfail(PTD_EINVAL, "batch is NULL");
    const int Ws[] = {2, 4, 8};
    const int Cs[] = {16, 32, 64, 128};
    const bool fp32 = b->dc || b->rb;
    const bool try_tb = fp32 && b->nchk % 2 == 0 && !(b->bp.flags & PTD_FLAG_DC_NO_TBLOCK);
    float best = 1e30f;   // ms per inner iteration
    LaunchCfg bestc = b->cfg;
    int best_tb = b->tb;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    // plain iterations on the current fields with every instance's flag cleared
    // (the fields are zero after ptd_batch_create; ptd_batch_solve uploads its
    // own state afterwards)
    if (b->rb) {
        BCK(cudaMemsetAsync(b->rdev, 0, b->ninst * sizeof(RbDev), b->s));
    } else if (b->dc) {
        set_done_batch_kernel<<<(b->ninst + 127) / 128, 128, 0, b->s>>>(b->bst, b->ninst, 0);
        BCK(cudaGetLastError());
    } else {
        BCK(cudaMemsetAsync(b->st, 0, b->ninst * sizeof(DevState), b->s));
    }
    for (int tbc = 1; tbc <= (try_tb ? 2 : 1); ++tbc)
        for (int W : Ws)
            for (int C : Cs) {
                b->tb = fp32 ? tbc : 1;
                b->cfg.warps2d = W;
                b->cfg.chunk2d = C;
                int rc = upload_work(b);
                if (rc) return rc;
                if (b->rb) BCK(compact_rb(b));   // every instance running
                const int nl = 12 / tbc;   // 12 inner iterations either way
                for (int rep = 0; rep < 2; ++rep) {
                    BCK(cudaEventRecord(e0, b->s));
                    for (int it = 0; it < nl; ++it)
                        BCK(b->rb   ? launch_rb_batch(b, it & 1, false)
                            : b->dc ? launch_dc_batch(b, it & 1, false)
                                    : launch_pt_batch(b, it & 1, false));
                    BCK(cudaEventRecord(e1, b->s));
                    BCK(cudaEventSynchronize(e1));
                }
                float ms = 0.0f;
                BCK(cudaEventElapsedTime(&ms, e0, e1));
                ms /= 12.0f;
                b->launches += 2 * nl;
                if (ms < best) {
                    best = ms;
                    bestc = b->cfg;
                    best_tb = b->tb;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (b->dc) {
        set_done_batch_kernel<<<(b->ninst + 127) / 128, 128, 0, b->s>>>(b->bst, b->ninst, 1);
        BCK(cudaGetLastError());
    }
    b->cfg = bestc;
    b->tb = best_tb;
    int rc = upload_work(b);
    if (!rc) rc = capture(b);
    if (rc) return rc;
    if (warps_out) *warps_out = bestc.warps2d;
    if (chunk_out) *chunk_out = bestc.chunk2d;
    if (us_out) *us_out = best * 1000.0f;
    return PTD_OK;
}

extern "C" int ptd_batch_config(ptd_batch* b, int32_t* warps, int32_t* chunk, int32_t* iters_per_launch)
{
    if (!b) return bfail(PTD_EINVAL, "batch is NULL");
    if (warps) *warps = b->cfg.warps2d;
    if (chunk) *chunk = b->cfg.chunk2d;
    if (iters_per_launch) *iters_per_launch = (b->dc || b->rb) ? b->tb : 1;
    return PTD_OK;
}

extern "C" int ptd_batch_set_config(ptd_batch* b, int32_t warps, int32_t chunk, int32_t iters_per_launch)
{
    if (!b) return bfail(PTD_EINVAL, "batch is NULL");
    if (warps != 1 && warps != 2 && warps != 4 && warps != 8) return bfail(PTD_EINVAL, "warps must be 1, 2, 4 or 8");
    if (chunk < 8 || chunk > 4096) return bfail(PTD_EINVAL, "rows per y chunk must be in [8, 4096]");
    const bool fp32 = b->dc || b->rb;
    if (iters_per_launch != 1 && !(iters_per_launch == 2 && fp32 && b->nchk % 2 == 0))
        return bfail(PTD_EINVAL, "iterations per launch: 1, or 2 for FP32_DC / FP32_RB with an even nchk");
    BCK(cudaStreamSynchronize(b->s));
    b->cfg.warps2d = warps;
    b->cfg.chunk2d = chunk;
    b->tb = iters_per_launch;
    int rc = upload_work(b);
    if (!rc) rc = capture(b);
    return rc;
}
