// ptd_pt.cu -- fused PT-iteration kernels (one launch per iteration), generic
// over the number type: F64 (native FP64), DF64 (double-float on the FP32
// pipe, same 8 bytes per value) and DFH (DF64 arithmetic on an FP64 H), see
// ptd_num.cuh.
//
// One launch computes, for every face, the damped flux of iteration k+1 from
// H^k and the flux of iteration k, and for every inner cell H^{k+1} from those
// new fluxes: the reference's compute_flux! + compute_update! pair
// (scripts/diff_2D_nonlin.jl:28-39, diff_3D/diff_3D_nonlin_multixpu.jl:37-50,
// diff_1D_nonlin.jl:24-33 and the lin/linstep siblings) in a single pass over
// memory.  H and the fluxes are double-buffered (read k, write k+1), which
// keeps the reference's Jacobi semantics across tile boundaries.  On a check
// iteration (template CHECK) the same pass also forms the reference's mixed
// residual (check_res!, scripts/diff_2D_nonlin.jl:41-44): undamped flux from
// H^k, time term from H^{k+1}, reduced to sum R^2 / max|R| in the same launch.
//
// Tiling (2D and 3D): a warp owns 32 consecutive x cells of which lanes 1..31
// are updated and lane 0 is the left neighbour, so each lane computes exactly
// one x face (its right face) and gets its left face from lane-1 by a shuffle:
// no face is evaluated twice inside a warp and no lane runs a divergent extra
// face.  Tiles therefore advance by 31 cells in x.  2D marches each warp up a
// chunk of y rows carrying the face below in a register; 3D stacks R warps
// as y rows of an x-y tile (rows 1..R-1 updated, row 0 the neighbour, y faces
// exchanged through shared memory, one barrier per plane) and marches the
// tile along z carrying the z face below in a register.
#include "ptd_pair_body.cuh"

namespace ptd {

// ---------------------------------------------------------------------------
// One-grid kernels: the block index is the tile index.
template <class N, int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) pt1d_kernel(PTArgs a)
{
    if (step_done(a.done)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    pt1d_body<N, MODEL, CHECK>(a, blockIdx.x, part, pmax);
    if (CHECK) block_reduce_residual(a, part, pmax, blockIdx.x);
}

template <class N, int MODEL, bool CHECK>
__global__ void __launch_bounds__(256, CHECK ? 5 : 6) pt2d_kernel(PTArgs a, int chunk)
{
    if (step_done(a.done)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    // the body flushes its check partials (last step of its march) into the
    // warp's slot, warps numbered x fastest
    const long long slot = ((long long)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.y + threadIdx.y;
    pt2d_body<N, MODEL, CHECK>(a, blockIdx.x * blockDim.y + threadIdx.y, blockIdx.y, chunk, part, pmax, slot);
}

// Resident CTAs per SM the register allocation must allow: 48 warps (3 CTAs
// of 16 warps) for the plain iterations of the LIN and NONLIN models, which
// fit in 40 registers (DFH NONLIN with a 24-byte spill), 32 warps for the
// check iterations and the models with a per-cell field (more live values).
template <class N, int MODEL, bool CHECK, int R>
__global__ void __launch_bounds__(32 * R, (CHECK || MODEL == LINSTEP || MODEL == NONLIN_EXPM) ? 32 / R : 48 / R)
    pt3d_kernel(PTArgs a, int chunk)
{
    if (step_done(a.done)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    pt3d_body<N, MODEL, CHECK, R>(a, blockIdx.x, blockIdx.y, blockIdx.z, chunk, part, pmax);
    if (CHECK)
        block_reduce_residual(a, part, pmax, ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
}

// 2D, the double-float forms (DF64, DFH): two x-adjacent cells per lane
// (ptd_pair_body.cuh), 62-cell tiles.  (The same pairing in 3D was slower than
// the one-cell kernel at 512^3 -- DF64 2244 against 2045 us: its 60-96
// registers leave 16-32 resident warps per SM for a march with a barrier per
// plane.)
template <class N, int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) pt2d_pair_kernel(PTArgs a, int chunk)
{
    if (step_done(a.done)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    const long long slot = ((long long)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.y + threadIdx.y;
    pt2d_pair_body<N, MODEL, CHECK>(a, blockIdx.x * blockDim.y + threadIdx.y, blockIdx.y, chunk, part, pmax, slot);
}

// ---------------------------------------------------------------------------
// Consistent residual (both flux terms from the updated H): one thread per
// inner cell, generic over ndim (unused dimensions have extent 1).
template <class N, int MODEL>
__global__ void __launch_bounds__(256) resid_consistent_kernel(PTArgs a, int ndim)
{
    using T = typename N::T;
    using HV = typename N::HV;
    if (step_done(a.done)) return;
    const long long ninner_x = a.nx - 2;
    const long long ninner_y = ndim > 1 ? a.ny - 2 : 1;
    const long long ninner_z = ndim > 2 ? a.nz - 2 : 1;
    const long long total = ninner_x * ninner_y * ninner_z;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long ix = 1 + t % ninner_x;
        const long long rest = t / ninner_x;
        const long long iy = ndim > 1 ? 1 + rest % ninner_y : 0;
        const long long iz = ndim > 2 ? 1 + rest / ninner_y : 0;
        const long long c = iz * a.sz + iy * a.sy + ix;
        const long long stp[3] = {1, a.sy, a.sz};
        const HV H = N::ldh(a.Hout, c);
        T div = N::zero();
        for (int d = 0; d < ndim; ++d) {
            const HV HR = N::ldh(a.Hout, c + stp[d]), HL = N::ldh(a.Hout, c - stp[d]);
            T uR, uL;
            if (MODEL == LIN) {
                uR = N::hdiff(HR, H);
                uL = N::hdiff(H, HL);
            } else if (MODEL == LINSTEP) {
                const T Dc = ld<N>(a.D, c);
                uR = N::mul(N::add(Dc, ld<N>(a.D, c + stp[d])), N::hdiff(HR, H));
                uL = N::mul(N::add(ld<N>(a.D, c - stp[d]), Dc), N::hdiff(H, HL));
            } else {
                const T sR = N::hsum(H, HR), sL = N::hsum(HL, H);
                uR = N::mul(N::mul(N::mul(sR, sR), sR), N::hdiff(HR, H));
                uL = N::mul(N::mul(N::mul(sL, sL), sL), N::hdiff(H, HL));
                if (MODEL == NONLIN_EXPM) {
                    const T Ec = ld<N>(a.D, c);
                    uR = N::mul(uR, N::add(Ec, ld<N>(a.D, c + stp[d])));
                    uL = N::mul(uL, N::add(ld<N>(a.D, c - stp[d]), Ec));
                }
            }
            div = N::mad(N::sub(uR, uL), cst<N>(a, d), div);
        }
        const T r = N::sub(div, N::mul(N::hdo(H, N::ldo(a.Hold, c)), cst<N>(a, 3)));
        accumulate_residual(N::to_d(r), part, pmax);
    }
    block_reduce_residual(a, part, pmax, blockIdx.x);
}

// The check of one block: err from the accumulated residual, appended to the
// error history; the step stops at err <= tol, NaN, or when no full check
// block fits before itmax.  Returns the new done state.
__device__ __forceinline__ int judge_step(DevState* st, double* errhist, int errcap, int nchk, int itmax, double tol,
                                          double norm_den, int norm_max)
{
    const double acc = st->acc;
    st->acc = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(norm_den);
    const int n = st->nchecks;
    if (n < errcap) errhist[n] = err;
    st->nchecks = n + 1;
    st->iter += nchk;
    st->err = err;
    int done = DONE_RUNNING;
    if (!(err > tol)) done = (err != err) ? DONE_NAN : DONE_CONVERGED;
    else if (st->iter + nchk > itmax) done = DONE_CAP;
    st->done = done;
    return done;
}

__global__ void judge_kernel(DevState* st, double* errhist, int errcap, int nchk, int itmax,
                             double tol, double norm_den, int norm_max)
{
    if (st->done) return;
    judge_step(st, errhist, errcap, nchk, itmax, tol, norm_den, norm_max);
}

// The judge of the one-grid solver, at the end of the body of the WHILE
// graph node of a physical step: it sums (or maxes) the check partials of the
// block's PT kernels from their slots in a fixed order -- thread t takes the
// slots t, t + 256, ... in order, then a fixed tree over the threads -- so the
// residual norm, and with it the stopping iteration, is the same on every run;
// when the step stops it also ends the loop (the node's condition set to 0),
// so the graph runs exactly the check blocks of the step.
__global__ void __launch_bounds__(256) judge_parts_kernel(DevState* st, const double* parts, long long nparts,
                                                          double* errhist, int errcap, int nchk, int itmax, double tol,
                                                          double norm_den, int norm_max, cudaGraphConditionalHandle loop)
{
    __shared__ double s_sum[256];
    __shared__ unsigned long long s_max[256];
    const int t = threadIdx.x;
    // a step already stopped (a second block in the body after the stop)
    // leaves the loop too; every thread reads done before thread 0 writes it
    if (st->done) {
        if (t == 0) cudaGraphSetConditional(loop, 0);
        return;
    }
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
    if (t == 0) {
        st->acc = norm_max ? __longlong_as_double((long long)s_max[0]) : s_sum[0];
        if (judge_step(st, errhist, errcap, nchk, itmax, tol, norm_den, norm_max) != DONE_RUNNING)
            cudaGraphSetConditional(loop, 0);
    }
}

__global__ void reset_state_kernel(DevState* st)
{
    st->done = DONE_RUNNING;
    st->nchecks = 0;
    st->iter = 0;
    st->acc = 0.0;
    st->err = 0.0;
}

// E = exp(m) of the NONLIN_EXPM model, as F64 or DF64.
__global__ void expm_kernel(const double* m, void* E, long long n, int df64)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const double e = exp(m[t]);
        if (df64) reinterpret_cast<float2*>(E)[t] = split_df(e);
        else reinterpret_cast<double*>(E)[t] = e;
    }
}

cudaError_t launch_expm(const double* m, void* E, long long n, bool df64, cudaStream_t s)
{
    expm_kernel<<<fill_blocks(), 256, 0, s>>>(m, E, n, df64 ? 1 : 0);
    return cudaGetLastError();
}

// FP64 <-> DF64 conversion of whole fields (host boundary only).
__global__ void to_df64_kernel(const double* src, float2* dst, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        dst[t] = split_df(src[t]);
}

__global__ void from_df64_kernel(const float2* src, double* dst, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        dst[t] = (double)src[t].x + (double)src[t].y;
}

// ---------------------------------------------------------------------------
template <class N, int MODEL, bool CHECK>
static cudaError_t launch_model(const PTArgs& a, int ndim, const LaunchCfg& cfg, cudaStream_t s)
{
    if (ndim == 1) {
        const int bs = 256;
        pt1d_kernel<N, MODEL, CHECK><<<(a.nx + bs - 1) / bs, bs, 0, s>>>(a);
        return cudaGetLastError();
    }
    if constexpr (!N::native) {
        if (ndim == 2) {
            const int W = cfg.warps2d;
            const int tiles = (a.nx - 2 + 61) / 62;
            dim3 grid((tiles + W - 1) / W, (a.ny - 2 + cfg.chunk2d - 1) / cfg.chunk2d);
            pt2d_pair_kernel<N, MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, cfg.chunk2d);
            return cudaGetLastError();
        }
    }
    if (ndim == 2) {
        const int W = cfg.warps2d;
        const int tiles = (a.nx - 2 + 30) / 31;
        dim3 grid((tiles + W - 1) / W, (a.ny - 2 + cfg.chunk2d - 1) / cfg.chunk2d);
        pt2d_kernel<N, MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, cfg.chunk2d);
    } else {
        const int tx = (a.nx - 2 + 30) / 31;
        const int nzc = (a.nz - 2 + cfg.chunk3d - 1) / cfg.chunk3d;
        if (cfg.rows3d == 8) {
            dim3 grid(tx, (a.ny - 2 + 6) / 7, nzc);
            pt3d_kernel<N, MODEL, CHECK, 8><<<grid, dim3(32, 8), 0, s>>>(a, cfg.chunk3d);
        } else {
            dim3 grid(tx, (a.ny - 2 + 14) / 15, nzc);
            pt3d_kernel<N, MODEL, CHECK, 16><<<grid, dim3(32, 16), 0, s>>>(a, cfg.chunk3d);
        }
    }
    return cudaGetLastError();
}

template <class N>
static cudaError_t launch_type(const PTArgs& a, int ndim, int model, bool check, const LaunchCfg& cfg,
                               cudaStream_t s)
{
    switch (model * 2 + (check ? 1 : 0)) {
    case 0: return launch_model<N, LIN, false>(a, ndim, cfg, s);
    case 1: return launch_model<N, LIN, true>(a, ndim, cfg, s);
    case 2: return launch_model<N, LINSTEP, false>(a, ndim, cfg, s);
    case 3: return launch_model<N, LINSTEP, true>(a, ndim, cfg, s);
    case 4: return launch_model<N, NONLIN, false>(a, ndim, cfg, s);
    case 5: return launch_model<N, NONLIN, true>(a, ndim, cfg, s);
    case 6: return launch_model<N, NONLIN_EXPM, false>(a, ndim, cfg, s);
    case 7: return launch_model<N, NONLIN_EXPM, true>(a, ndim, cfg, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_pt(const PTArgs& a, int ndim, int model, bool check, int num, const LaunchCfg& cfg,
                      cudaStream_t s)
{
    if (num == NUM_DF64) return launch_type<DF64>(a, ndim, model, check, cfg, s);
    if (num == NUM_DFH) return launch_type<DFH>(a, ndim, model, check, cfg, s);
    return launch_type<F64>(a, ndim, model, check, cfg, s);
}

template <class N>
static void resid_consistent_type(const PTArgs& a, int ndim, int model, cudaStream_t s)
{
    const int bs = 256, nb = fill_blocks();
    if (model == LIN) resid_consistent_kernel<N, LIN><<<nb, bs, 0, s>>>(a, ndim);
    else if (model == LINSTEP) resid_consistent_kernel<N, LINSTEP><<<nb, bs, 0, s>>>(a, ndim);
    else if (model == NONLIN) resid_consistent_kernel<N, NONLIN><<<nb, bs, 0, s>>>(a, ndim);
    else resid_consistent_kernel<N, NONLIN_EXPM><<<nb, bs, 0, s>>>(a, ndim);
}

cudaError_t launch_resid_consistent(const PTArgs& a, int ndim, int model, int num, cudaStream_t s)
{
    if (num == NUM_DF64) resid_consistent_type<DF64>(a, ndim, model, s);
    else if (num == NUM_DFH) resid_consistent_type<DFH>(a, ndim, model, s);
    else resid_consistent_type<F64>(a, ndim, model, s);
    return cudaGetLastError();
}

// Load every kernel the FP64 2D solve launches (the six model x check
// variants of the fused kernel, the judge and the state reset) on the current
// device.  The runtime loads device code lazily, on a kernel's first launch;
// a caller that must not see device memory change during later solves calls
// this once up front.
cudaError_t preload_pt2d_f64()
{
    cudaFuncAttributes fa;
    const void* fns[] = {
        (const void*)pt2d_kernel<F64, LIN, false>,     (const void*)pt2d_kernel<F64, LIN, true>,
        (const void*)pt2d_kernel<F64, LINSTEP, false>, (const void*)pt2d_kernel<F64, LINSTEP, true>,
        (const void*)pt2d_kernel<F64, NONLIN, false>,  (const void*)pt2d_kernel<F64, NONLIN, true>,
        (const void*)judge_kernel,                     (const void*)reset_state_kernel};
    for (const void* f : fns) {
        const cudaError_t e = cudaFuncGetAttributes(&fa, f);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_judge(DevState* st, double* errhist, int errcap, int nchk, int itmax, double tol,
                         double norm_den, int norm_max, cudaStream_t s)
{
    judge_kernel<<<1, 1, 0, s>>>(st, errhist, errcap, nchk, itmax, tol, norm_den, norm_max);
    return cudaGetLastError();
}

cudaError_t launch_judge_parts(DevState* st, const double* parts, long long nparts, double* errhist, int errcap,
                               int nchk, int itmax, double tol, double norm_den, int norm_max,
                               cudaGraphConditionalHandle loop, cudaStream_t s)
{
    judge_parts_kernel<<<1, 256, 0, s>>>(st, parts, nparts, errhist, errcap, nchk, itmax, tol, norm_den, norm_max,
                                         loop);
    return cudaGetLastError();
}

// The number of check-residual slots the fused kernel of a check iteration
// writes with this launch shape (the grids of launch_model below: blocks in
// 1D and 3D, warps in 2D), or the consistent-residual kernel's blocks.
long long pt_check_slots(int ndim, int nx, int ny, int nz, const LaunchCfg& cfg, bool consistent, int num)
{
    if (consistent) return fill_blocks();
    if (ndim == 1) return (nx + 255) / 256;
    if (ndim == 2) {
        const int tw = num != NUM_F64 ? 62 : 31;   // the double-float forms: two cells per lane
        const int W = cfg.warps2d;
        const long long tiles = (nx - 2 + tw - 1) / tw;
        return ((tiles + W - 1) / W) * W * (long long)((ny - 2 + cfg.chunk2d - 1) / cfg.chunk2d);
    }
    const long long tx = (nx - 2 + 30) / 31;
    const long long nzc = (nz - 2 + cfg.chunk3d - 1) / cfg.chunk3d;
    const int rows = cfg.rows3d;
    const long long ty = (ny - 2 + rows - 2) / (rows - 1);
    return tx * ty * nzc;
}

cudaError_t launch_reset_state(DevState* st, cudaStream_t s)
{
    reset_state_kernel<<<1, 1, 0, s>>>(st);
    return cudaGetLastError();
}

cudaError_t launch_to_df64(const double* src, void* dst, long long n, cudaStream_t s)
{
    to_df64_kernel<<<fill_blocks(), 256, 0, s>>>(src, reinterpret_cast<float2*>(dst), n);
    return cudaGetLastError();
}

__global__ void add_fields_kernel(double* dst, const double* src, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        dst[t] += src[t];
}

cudaError_t add_fields(double* dst, const double* src, long long n, cudaStream_t s)
{
    add_fields_kernel<<<fill_blocks(), 256, 0, s>>>(dst, src, n);
    return cudaGetLastError();
}

cudaError_t launch_from_df64(const void* src, double* dst, long long n, cudaStream_t s)
{
    from_df64_kernel<<<fill_blocks(), 256, 0, s>>>(reinterpret_cast<const float2*>(src), dst, n);
    return cudaGetLastError();
}

}  // namespace ptd
