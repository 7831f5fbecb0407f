// ptd_rb.cu -- the one-grid solver of the rebased FP32 form (PTD_PREC_FP32_RB):
// kernels, the FP64 rebase (fold, base quantities) and the step driver.  The
// form and its iteration bodies are described in ptd_rb_body.cuh.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "ptd_internal.h"
#include "ptd_rb_body.cuh"

namespace ptd {

template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) rb1d_kernel(RbArgs a)
{
    if (rb_skip(a.skip)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    rb1d_body<MODEL, CHECK>(a, blockIdx.x, part, pmax);
    if (CHECK) block_reduce_residual(a.acc, a.norm_max, (double)part, widen_max32(pmax), a.parts, blockIdx.x);
}

template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) rb2d_kernel(RbArgs a, int chunk)
{
    if (rb_skip(a.skip)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    // the body flushes its check partials into its warp's slot (last step of its march)
    rb2d_body<MODEL, CHECK>(a, blockIdx.x * blockDim.y + threadIdx.y, blockIdx.y, chunk, part, pmax, warp_slot());
}

// Two iterations per launch, two columns per lane (LIN, NONLIN).
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) rb2d_tb2_pair_kernel(RbArgs a, int chunk)
{
    if (rb_skip(a.skip)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    if constexpr (MODEL == LIN || MODEL == NONLIN)
        rb2d_tb2_pair_body<MODEL, CHECK>(a, blockIdx.x * blockDim.y + threadIdx.y, blockIdx.y, chunk, part, pmax,
                                         warp_slot());
}

// The plain NONLIN variant is capped at 32 registers (8 CTAs of 256 threads
// per SM; ptxas spills 16 bytes): at its natural 40 the march, bound by
// memory latency, ran at most 48 of 64 warps per SM.  Measured at 4096^2:
// 77.9 -> 76.8 us per iteration.  A minimum of 0 blocks leaves the other
// variants' register allocation as without the bound.
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256, (MODEL == NONLIN && !CHECK) ? 8 : 0) rb2d_tb2_kernel(RbArgs a, int chunk)
{
    if (rb_skip(a.skip)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    // the body flushes its check partials into its warp's slot (last step of its march)
    rb2d_tb2_body<MODEL, CHECK>(a, blockIdx.x * blockDim.y + threadIdx.y, blockIdx.y, chunk, part, pmax, warp_slot());
}

// Two iterations per launch in 3D (LIN, NONLIN): 16-warp CTAs, 2 resident per SM.
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(512, 2) rb3d_tb2_kernel(RbArgs a, int chunk)
{
    if (rb_skip(a.skip)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    if constexpr (MODEL == LIN || MODEL == NONLIN)
        rb3d_tb2_body<MODEL, CHECK, 16>(a, blockIdx.x, blockIdx.y, blockIdx.z, chunk, part, pmax);
    if (CHECK) block_reduce_residual(a.acc, a.norm_max, part, pmax, a.parts, block_slot());
}

// 16-warp CTAs of 31 x 15 updated cells.  (32-row tiles, 1024-thread CTAs
// of 31 x 31 cells, gave the same iterates bit for bit but took 1.31 against
// 1.24 ms per iteration at 512^3: the per-plane barrier of twice the warps.)
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(512) rb3d_kernel(RbArgs a, int chunk)
{
    if (rb_skip(a.skip)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    rb3d_body<MODEL, CHECK, 16>(a, blockIdx.x, blockIdx.y, blockIdx.z, chunk, part, pmax);
    if (CHECK) block_reduce_residual(a.acc, a.norm_max, part, pmax, a.parts, block_slot());
}

__global__ void rb_fold_kernel(RbFoldArgs f, int parity)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < f.n;
         t += (long long)gridDim.x * blockDim.x)
        rb_fold_elem(f, parity, t);
}

__global__ void __launch_bounds__(256) rb_base_kernel(RbBaseArgs b, const RbDev* st)
{
    if (st && st->step_done) return;
    const long long total = (long long)b.nx * b.ny * b.nz;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(t % b.nx);
        const long long rest = t / b.nx;
        rb_base_cell(b, ix, (int)(rest % b.ny), (int)(rest / b.ny), part, pmax);
    }
    block_reduce_residual(b.acc64, b.norm_max, part, pmax, b.parts, blockIdx.x);
}

// 2D / 3D: rb_base_cell's quantities with each face evaluated once.  A warp
// takes 32 consecutive x cells of one row and marches over a chunk of rows
// (2D) or planes (3D, one y row per warp): the face to a cell's left is the
// next lane down's right face (a shuffle), the face below it in the march the
// previous step's face above; only the tile's first lane and the march's
// first step evaluate theirs, and in 3D both y faces are evaluated per cell.
// Every face is the same rb_u64 evaluation, so the quantities are
// rb_base_cell's bit for bit; the residual goes into the block's slot.
constexpr int kBaseChunk = 32;   // rows (2D) / planes (3D) per warp
template <int NDIM>
__global__ void __launch_bounds__(256) rb_base_march_kernel(RbBaseArgs b, const RbDev* st)
{
    if (st && st->step_done) return;   // uniform over the grid
    const int lane = threadIdx.x;
    const int ix = 32 * blockIdx.x + lane;
    const int ixc = min(ix, b.nx - 1);   // lanes past the row compute on its last cell, store nothing
    const bool own = ix < b.nx;
    int iy, k0, k1, nm;
    long long sm;   // the march: y in 2D, z in 3D
    if (NDIM == 2) {
        iy = 0;
        k0 = (blockIdx.y * blockDim.y + threadIdx.y) * kBaseChunk;
        nm = b.ny;
        sm = b.sy;
    } else {
        iy = blockIdx.y * blockDim.y + threadIdx.y;
        k0 = blockIdx.z * kBaseChunk;
        nm = b.nz;
        sm = b.sz;
    }
    k1 = min(k0 + kBaseChunk, nm);
    double part = 0.0;
    unsigned long long pmax = 0ull;
    if (k0 < k1 && iy < b.ny) {   // uniform over the warp
        const bool xin = ixc >= 1 && ixc <= b.nx - 2;
        const bool yin = NDIM == 2 || (iy >= 1 && iy <= b.ny - 2);
        double udn = 0.0;   // the face below the cell in the march
        for (int k = k0; k < k1; ++k) {
            const long long c = NDIM == 2 ? (long long)k * b.sy + ixc : (long long)k * b.sz + (long long)iy * b.sy + ixc;
            const bool min_ = k >= 1 && k <= nm - 2;
            const bool inner = xin && yin && min_;
            // x faces: right by every lane, left from the lane below
            const double ur = ixc <= b.nx - 2 ? rb_u64(b, c, c + 1) : 0.0;
            double ul = __shfl_up_sync(FULL, ur, 1);
            if (lane == 0 && inner) ul = rb_u64(b, c - 1, c);
            // march faces: above now, below from the previous step
            const double uup = k <= nm - 2 ? rb_u64(b, c, c + sm) : 0.0;
            if (k == k0 && inner) udn = rb_u64(b, c - sm, c);
            if (own) {
                b.Hf[c] = __double2float_rn(b.H[c]);
                const int dm = NDIM - 1;   // the march direction's index
                if (ixc <= b.nx - 2) b.tb[0][c] = (float)(b.wb[0][c] + ur);
                if (k <= nm - 2) b.tb[dm][c] = (float)(b.wb[dm][c] + uup);
                double uyr = 0.0;
                if (NDIM == 3 && iy <= b.ny - 2) {
                    uyr = rb_u64(b, c, c + b.sy);
                    b.tb[1][c] = (float)(b.wb[1][c] + uyr);
                }
                if (inner) {
                    // the order of rb_base_cell: x, y, z
                    double divw = 0.0, divu = 0.0;
                    divw = fma(b.wb[0][c] - b.wb[0][c - 1], b.sig[0], divw);
                    divu = fma(ur - ul, b.sig[0], divu);
                    if (NDIM == 3) {
                        const double uyl = rb_u64(b, c - b.sy, c);
                        divw = fma(b.wb[1][c] - b.wb[1][c - b.sy], b.sig[1], divw);
                        divu = fma(uyr - uyl, b.sig[1], divu);
                    }
                    divw = fma(b.wb[dm][c] - b.wb[dm][c - sm], b.sig[dm], divw);
                    divu = fma(uup - udn, b.sig[dm], divu);
                    const double dh = (b.H[c] - b.Hold[c]) * b.rdt;
                    b.Rb[c] = (float)(dh + divw);
                    const double cb = divu - dh;
                    if (NDIM == 3) b.Cb64[c] = cb;
                    else b.Cb[c] = (float)cb;
                    accumulate_residual(cb, part, pmax);
                }
            }
            udn = uup;
        }
    }
    block_reduce_residual(b.acc64, b.norm_max, part, pmax, b.parts,
                          ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
}

__global__ void rb_reset_kernel(RbDev* st) { rb_reset(st); }

// After each block of nchk iterations: the FP32 check err (rb_check_judge),
// and whether the FP64 rebase that follows the block in the step graph runs
// (the condition of its IF node: the phase is over).
__global__ void __launch_bounds__(256) rb_check_judge_kernel(RbDev* st, const double* parts, long long nparts,
                                                             double* errhist, int errcap, int nchk, int itmax,
                                                             double tol, double norm_den, int norm_max,
                                                             int phase_cap, cudaGraphConditionalHandle rebase)
{
    // every thread reads the flags before thread 0 can change them
    const bool idle = st->skip || st->step_done;
    __syncthreads();
    if (idle) {   // no PT kernel ran: the slots are stale
        if (threadIdx.x == 0) {
            st->blocks += 1;
            cudaGraphSetConditional(rebase, 0);
        }
        return;
    }
    const double acc = sum_slots(parts, nparts, norm_max);
    if (threadIdx.x == 0) {
        st->blocks += 1;
        st->acc = acc;
        rb_check_judge(st, errhist, errcap, nchk, itmax, tol, norm_den, norm_max, phase_cap);
        cudaGraphSetConditional(rebase, st->skip ? 1 : 0);
    }
}

// After each rebase: the FP64 err of the base (rb_base_judge); inside the
// step graph (in_loop) it also counts the phase.  Every phase adds at least
// one check block of nchk iterations (its first judge runs with skip clear)
// and a phase that leaves no room for another block before itmax ends the
// step (capped), so the step graph's loop ends within itmax/nchk passes.
__global__ void __launch_bounds__(256) rb_base_judge_kernel(RbDev* st, const double* parts, long long nparts,
                                                            double tol, double norm_den, int norm_max, int in_loop)
{
    // every thread reads step_done before thread 0 can change it
    const bool stopped = st->step_done != 0;
    __syncthreads();
    if (stopped) {   // the base kernel did not run: the slots are stale
        if (threadIdx.x == 0 && in_loop) st->phases += 1;
        return;
    }
    const double acc = sum_slots(parts, nparts, norm_max);
    if (threadIdx.x == 0) {
        if (in_loop) st->phases += 1;
        st->acc64 = acc;
        rb_base_judge(st, tol, norm_den, norm_max);
    }
}

// Last node of the step graph's loop body (at the body's own level, where the
// loop's condition is set): ends the loop once the step has stopped.  Every
// pass of a running step adds a check block, so a step still running after
// max_passes passes (itmax/nchk + 2) has lost its stop: it ends as capped.
__global__ void rb_loop_judge_kernel(RbDev* st, int max_passes, cudaGraphConditionalHandle loop)
{
    st->passes += 1;
    if (!st->step_done && st->passes > max_passes) {
        st->step_done = DONE_CAP;
        st->skip = 1;
    }
    if (st->step_done) cudaGraphSetConditional(loop, 0);
}

__global__ void rb_tofloat_kernel(const double* src, float* dst, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        dst[t] = __double2float_rn(src[t]);
}

// ---------------------------------------------------------------------------
struct RbState {
    ptd_params p;
    Derived dv;
    LaunchCfg cfg;
    ptd_ctx_base g;
    cudaStream_t s = nullptr;
    float* d[2] = {nullptr, nullptr};
    float* w[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    float* tb[3] = {nullptr, nullptr, nullptr};
    float* Rb = nullptr;
    float* Cb = nullptr;                          // base check residual (1D, 2D: FP32)
    double* Cb64 = nullptr;                       // base check residual (3D: FP64)
    float* Hf = nullptr;
    float* Df = nullptr;
    double* H = nullptr;                          // owned by the context: the base H_b
    double* Hold = nullptr;                       // owned by the context
    double* wb[3] = {nullptr, nullptr, nullptr};  // owned by the context: the base fluxes
    const double* D = nullptr;                    // owned by the context (LINSTEP)
    RbDev* dev = nullptr;
    RbDev* h_dev = nullptr;
    int* zero_flag = nullptr;
    double* errhist = nullptr;
    int errcap = 0;
    double* parts = nullptr;                      // check-residual slots of the check launches
    long long nparts = 0;
    double* parts64 = nullptr;                    // FP64 residual slots of the base kernel
    long long nparts64 = 0;
    int phase_iters = 200;                        // PT iterations of a phase at most
    int tblk = 1;                                 // iterations per launch (2: temporal blocking, 2D)
    cudaGraphExec_t gphase = nullptr;
    int kernels_per_block = 0;                    // PT launches and check judge of one check block
    int blocks_per_pass = 1;                      // check blocks per pass of the step graph's loop
    DcCounters k;
};

namespace {

#define RCK(call)                                                 \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);       \
    } while (0)

void rb_args(const RbState* rb, int parity, const int* skip, RbArgs& a)
{
    std::memset(&a, 0, sizeof(a));
    a.nx = rb->g.nx;
    a.ny = rb->g.ny;
    a.nz = rb->g.nz;
    a.sy = rb->g.sy;
    a.sz = rb->g.sz;
    a.rdt = (float)rb->dv.rdt;
    for (int d = 0; d < 3; ++d) a.sig[d] = (float)rb->dv.sig[d];
    a.c_lin = (float)rb->dv.c_lin;
    a.e_lin = (float)rb->dv.e_lin;
    a.f = fparams(rb->dv);
    a.din = rb->d[parity];
    a.dout = rb->d[parity ^ 1];
    for (int d = 0; d < 3; ++d) {
        const int dd = rb->w[d][0] ? d : 0;
        a.win[d] = rb->w[dd][parity];
        a.wout[d] = rb->w[dd][parity ^ 1];
        a.tb[d] = rb->tb[rb->tb[d] ? d : 0];
    }
    a.Rb = rb->Rb;
    a.Cb = rb->Cb;
    a.Cb64 = rb->Cb64;
    a.Hf = rb->Hf;
    a.Df = rb->Df;
    a.skip = skip;
    a.acc = &rb->dev->acc;
    a.parts = rb->parts;
    a.norm_max = rb->p.norm == PTD_NORM_MAX;
}

template <int MODEL, bool CHECK>
cudaError_t rb_launch_model(const RbArgs& a, int ndim, const LaunchCfg& cfg, cudaStream_t s, int tb)
{
    if (ndim == 1) {
        rb1d_kernel<MODEL, CHECK><<<(a.nx + 255) / 256, 256, 0, s>>>(a);
    } else if (ndim == 2 && tb == 2) {
        // twice the configured rows per y march: the march starts with two
        // extra level-1 rows (4096^2 nonlinear, 2 warps: 87.2 us per
        // iteration at 16 rows, 85.9 at 32, 86.0 at 64)
        const int W = cfg.warps2d, chunk = 2 * cfg.chunk2d;
        if (MODEL == LIN || MODEL == NONLIN) {   // two columns per lane, 60 per warp
            const int tiles = (a.nx - 1 + 59) / 60;
            dim3 grid((tiles + W - 1) / W, (a.ny - 2 + chunk - 1) / chunk);
            rb2d_tb2_pair_kernel<MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, chunk);
        } else {
            const int tiles = (a.nx - 2 + 27) / 28;
            dim3 grid((tiles + W - 1) / W, (a.ny - 2 + chunk - 1) / chunk);
            rb2d_tb2_kernel<MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, chunk);
        }
    } else if (ndim == 2) {
        const int W = cfg.warps2d;
        const int tiles = (a.nx - 2 + 30) / 31;
        dim3 grid((tiles + W - 1) / W, (a.ny - 2 + cfg.chunk2d - 1) / cfg.chunk2d);
        rb2d_kernel<MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, cfg.chunk2d);
    } else if (tb == 2) {
        // 28 x 12 level-2 cells per 16-warp CTA; the z march runs two planes
        // more than its chunk (the level-1 start)
        const int chunk = cfg.chunk3d;
        dim3 grid((a.nx - 2 + 27) / 28, (a.ny - 2 + 11) / 12, (a.nz - 2 + chunk - 1) / chunk);
        rb3d_tb2_kernel<MODEL, CHECK><<<grid, dim3(32, 16), 0, s>>>(a, chunk);
    } else {
        const int tx = (a.nx - 2 + 30) / 31;
        dim3 grid(tx, (a.ny - 2 + 14) / 15, (a.nz - 2 + cfg.chunk3d - 1) / cfg.chunk3d);
        rb3d_kernel<MODEL, CHECK><<<grid, dim3(32, 16), 0, s>>>(a, cfg.chunk3d);
    }
    return cudaGetLastError();
}

// One launch of tb PT iterations (tb = 2: 2D; 3D LIN and NONLIN).
cudaError_t rb_launch(const RbArgs& a, int ndim, int model, bool check, const LaunchCfg& cfg, cudaStream_t s,
                      int tb = 1)
{
    switch (model * 2 + (check ? 1 : 0)) {
    case 0: return rb_launch_model<LIN, false>(a, ndim, cfg, s, tb);
    case 1: return rb_launch_model<LIN, true>(a, ndim, cfg, s, tb);
    case 2: return rb_launch_model<LINSTEP, false>(a, ndim, cfg, s, tb);
    case 3: return rb_launch_model<LINSTEP, true>(a, ndim, cfg, s, tb);
    case 4: return rb_launch_model<NONLIN, false>(a, ndim, cfg, s, tb);
    case 5: return rb_launch_model<NONLIN, true>(a, ndim, cfg, s, tb);
    case 6: return rb_launch_model<NONLIN_EXPM, false>(a, ndim, cfg, s, tb);
    case 7: return rb_launch_model<NONLIN_EXPM, true>(a, ndim, cfg, s, tb);
    }
    return cudaErrorInvalidValue;
}

// niter PT iterations without checks from buffer parity 0 (pairs per launch
// when temporal blocking is on); returns the parity of the result.
cudaError_t rb_run_plain(const RbState* rb, int32_t niter, const int* skip, int& par, long long& launches)
{
    par = 0;
    for (int32_t it = 0; it < niter;) {
        const int tb = (rb->tblk == 2 && niter - it >= 2) ? 2 : 1;
        RbArgs a;
        rb_args(rb, par, skip, a);
        cudaError_t e = rb_launch(a, rb->p.ndim, rb->p.model, false, rb->cfg, rb->s, tb);
        if (e != cudaSuccess) return e;
        par ^= 1;
        ++launches;
        it += tb;
    }
    return cudaSuccess;
}

// The check-residual slots of the check launch (the grids of
// rb_launch_model): warps in 2D, blocks in 1D and 3D.
long long rb_check_slots(const RbState* rb)
{
    const ptd_params& p = rb->p;
    const LaunchCfg& c = rb->cfg;
    if (p.ndim == 1) return (p.nx + 255) / 256;
    if (p.ndim == 2) {
        const bool pair = rb->tblk == 2 && (p.model == PTD_MODEL_LIN || p.model == PTD_MODEL_NONLIN);
        const long long tiles = pair ? (p.nx - 1 + 59) / 60 : (rb->tblk == 2 ? (p.nx - 2 + 27) / 28 : (p.nx - 2 + 30) / 31);
        const int chunk = rb->tblk == 2 ? 2 * c.chunk2d : c.chunk2d;
        const int W = c.warps2d;
        return (tiles + W - 1) / W * W * (long long)((p.ny - 2 + chunk - 1) / chunk);
    }
    const long long nzc = (p.nz - 2 + c.chunk3d - 1) / c.chunk3d;
    if (rb->tblk == 2) return (long long)((p.nx - 2 + 27) / 28) * ((p.ny - 2 + 11) / 12) * nzc;
    return (long long)((p.nx - 2 + 30) / 31) * ((p.ny - 2 + 14) / 15) * nzc;
}

// The grid of rb_base_march_kernel (8 warps per CTA); its CTA count is the
// number of FP64 residual slots of a rebase.
dim3 base_grid(const RbState* rb)
{
    const ptd_params& p = rb->p;
    const unsigned gx = (p.nx + 31) / 32;
    if (p.ndim == 2) return dim3(gx, ((p.ny + kBaseChunk - 1) / kBaseChunk + 7) / 8, 1);
    return dim3(gx, (p.ny + 7) / 8, (p.nz + kBaseChunk - 1) / kBaseChunk);
}

// One rebase's base kernel: 1D grid-stride, 2D / 3D the march kernel.
cudaError_t launch_base(const RbState* rb, const RbBaseArgs& b, const RbDev* st)
{
    if (rb->p.ndim == 1) rb_base_kernel<<<fill_blocks(), 256, 0, rb->s>>>(b, st);
    else if (rb->p.ndim == 2) rb_base_march_kernel<2><<<base_grid(rb), dim3(32, 8), 0, rb->s>>>(b, st);
    else rb_base_march_kernel<3><<<base_grid(rb), dim3(32, 8), 0, rb->s>>>(b, st);
    return cudaGetLastError();
}

// (Re)allocate the residual slots for the current launch configuration.
int rb_alloc_parts(RbState* rb)
{
    const long long n = rb_check_slots(rb);
    if (n > rb->nparts) {
        cudaFree(rb->parts);
        rb->parts = nullptr;
        rb->nparts = 0;
        if (cudaMalloc((void**)&rb->parts, (size_t)n * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(PTD_ENOMEM, "rb: cudaMalloc failed");
        }
    }
    rb->nparts = n;
    if (!rb->parts64) {
        const dim3 bg = base_grid(rb);
        rb->nparts64 = rb->p.ndim == 1 ? fill_blocks() : (long long)bg.x * bg.y * bg.z;
        if (cudaMalloc((void**)&rb->parts64, (size_t)rb->nparts64 * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(PTD_ENOMEM, "rb: cudaMalloc failed");
        }
    }
    return PTD_OK;
}

RbFoldArgs fold_args(const RbState* rb)
{
    RbFoldArgs f;
    std::memset(&f, 0, sizeof(f));
    f.n = rb->g.nfield;
    f.H = rb->H;
    f.ndim = rb->p.ndim;
    f.d[0] = rb->d[0];
    f.d[1] = rb->d[1];
    for (int d = 0; d < rb->p.ndim; ++d) {
        f.wb[d] = rb->wb[d];
        f.w[d][0] = rb->w[d][0];
        f.w[d][1] = rb->w[d][1];
    }
    return f;
}

RbBaseArgs base_args(const RbState* rb)
{
    RbBaseArgs b;
    std::memset(&b, 0, sizeof(b));
    b.nx = rb->g.nx;
    b.ny = rb->g.ny;
    b.nz = rb->g.nz;
    b.ndim = rb->p.ndim;
    b.model = rb->p.model;
    b.sy = rb->g.sy;
    b.sz = rb->g.sz;
    b.rdt = rb->dv.rdt;
    for (int d = 0; d < 3; ++d) b.sig[d] = rb->dv.sig[d];
    b.H = rb->H;
    b.Hold = rb->Hold;
    for (int d = 0; d < rb->p.ndim; ++d) {
        b.wb[d] = rb->wb[d];
        b.tb[d] = rb->tb[d];
    }
    b.D = rb->D;
    b.Rb = rb->Rb;
    b.Cb = rb->Cb;
    b.Cb64 = rb->Cb64;
    b.Hf = rb->Hf;
    b.acc64 = &rb->dev->acc64;
    b.parts = rb->parts64;
    b.norm_max = rb->p.norm == PTD_NORM_MAX;
    return b;
}

// The rebased PT iteration of one physical step as one CUDA graph: a WHILE
// node whose body is one check block of nchk iterations with its FP32 judge,
// followed by the rebase (fold, base quantities, FP64 judge) in an IF node
// that the judge opens when the phase is over, and the loop judge, which ends
// the loop when the step stops (the body's layout is below).
int rb_capture(RbState* rb)
{
    cudaGraph_t g = nullptr;
    RCK(cudaGraphCreate(&g, 0));
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
        return cuda_fail(err, "conditional graph node");
    }
    cudaGraph_t body = np.conditional.phGraph_out[0];
    // The loop body: one check block (nchk/tb launches and the check judge)
    // followed by an IF node holding the FP64 rebase (fold, base quantities,
    // base judge), which runs when the judge has ended the phase; two such
    // blocks when the launch count is odd, so that every pass starts on
    // buffer parity 0; last, the loop judge.  No launch is issued past the
    // end of a phase.
    const int nchk = rb->p.nchk;
    const int nl = nchk / rb->tblk;   // launches per check block (tb divides nchk)
    const int nblk = (nl & 1) ? 2 : 1;
    int par = 0;
    cudaGraphNode_t prev = nullptr;   // the previous block's IF node
    for (int b = 0; b < nblk && err == cudaSuccess; ++b) {
        cudaGraphConditionalHandle rebase;
        err = cudaGraphConditionalHandleCreate(&rebase, body, 0, cudaGraphCondAssignDefault);
        if (err == cudaSuccess)
            err = cudaStreamBeginCaptureToGraph(rb->s, body, prev ? &prev : nullptr, nullptr, prev ? 1 : 0,
                                                cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) break;
        for (int it = 0; it < nl && err == cudaSuccess; ++it) {
            RbArgs a;
            rb_args(rb, par, &rb->dev->skip, a);
            err = rb_launch(a, rb->p.ndim, rb->p.model, it == nl - 1, rb->cfg, rb->s, rb->tblk);
            par ^= 1;
        }
        if (err == cudaSuccess) {
            rb_check_judge_kernel<<<1, 256, 0, rb->s>>>(rb->dev, rb->parts, rb->nparts, rb->errhist, rb->errcap, nchk,
                                                        rb->p.itmax, rb->p.tol, rb->dv.norm_den,
                                                        rb->p.norm == PTD_NORM_MAX, rb->phase_iters, rebase);
            err = cudaGetLastError();
        }
        // the judge is the capture's last node: the IF node follows it
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaError_t e1 = cudaStreamGetCaptureInfo(rb->s, &cs, nullptr, nullptr, &deps, nullptr, &nd);
        cudaGraphNode_t leaf = (e1 == cudaSuccess && nd == 1) ? deps[0] : nullptr;
        cudaGraph_t captured = body;
        cudaError_t e2 = cudaStreamEndCapture(rb->s, &captured);
        if (err == cudaSuccess) err = e1 != cudaSuccess ? e1 : e2;
        if (err == cudaSuccess && !leaf) err = cudaErrorStreamCaptureInvalidated;
        cudaGraphNodeParams ip = {cudaGraphNodeTypeConditional};
        ip.conditional.handle = rebase;
        ip.conditional.type = cudaGraphCondTypeIf;
        ip.conditional.size = 1;
        cudaGraphNode_t ifn = nullptr;
        if (err == cudaSuccess) err = cudaGraphAddNode(&ifn, body, &leaf, nullptr, 1, &ip);
        if (err == cudaSuccess)
            err = cudaStreamBeginCaptureToGraph(rb->s, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) break;
        rb_fold_kernel<<<fill_blocks(), 256, 0, rb->s>>>(fold_args(rb), par);
        err = cudaGetLastError();
        if (err == cudaSuccess) err = launch_base(rb, base_args(rb), rb->dev);
        if (err == cudaSuccess) {
            rb_base_judge_kernel<<<1, 256, 0, rb->s>>>(rb->dev, rb->parts64, rb->nparts64, rb->p.tol,
                                                       rb->dv.norm_den, rb->p.norm == PTD_NORM_MAX, 1);
            err = cudaGetLastError();
        }
        cudaGraph_t ifbody = ip.conditional.phGraph_out[0];
        e2 = cudaStreamEndCapture(rb->s, &ifbody);
        if (err == cudaSuccess) err = e2;
        prev = ifn;
    }
    // the loop's condition, set at the body's level after the last rebase node
    if (err == cudaSuccess)
        err = cudaStreamBeginCaptureToGraph(rb->s, body, &prev, nullptr, 1, cudaStreamCaptureModeThreadLocal);
    if (err == cudaSuccess) {
        rb_loop_judge_kernel<<<1, 1, 0, rb->s>>>(rb->dev, rb->p.itmax / nchk + 2, loop);
        err = cudaGetLastError();
        cudaGraph_t captured = body;
        const cudaError_t e4 = cudaStreamEndCapture(rb->s, &captured);
        if (err == cudaSuccess) err = e4;
    }
    if (err != cudaSuccess) {
        cudaStreamCaptureStatus cs;
        if (cudaStreamIsCapturing(rb->s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
            cudaGraph_t dropped = nullptr;
            cudaStreamEndCapture(rb->s, &dropped);
        }
        cudaGetLastError();
        cudaGraphDestroy(g);
        return cuda_fail(err, "capture rebased step");
    }
    cudaError_t e3 = cudaGraphInstantiate(&rb->gphase, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return cuda_fail(e3, "cudaGraphInstantiate");
    rb->kernels_per_block = nl + 1;
    rb->blocks_per_pass = nblk;
    return PTD_OK;
}

}  // namespace

int rb_create(const ptd_ctx_base& g, const ptd_params& p, const Derived& dv, cudaStream_t s, RbState** out)
{
    *out = nullptr;
    RbState* rb = new (std::nothrow) RbState();
    if (!rb) return set_error(PTD_ENOMEM, "rb_create: host allocation failed");
    rb->p = p;
    rb->dv = dv;
    rb->g = g;
    rb->s = s;
    rb->cfg = tuned_config(p);
    // a phase: the check blocks between two FP64 rebases, ~200 PT iterations
    // at most.  Longer phases cost iterations: with 1000 the 2D 4096^2 steps
    // took 6900 / 6100 / 5800 / 5700 / 5500 PT iterations against FP64's 6500
    // / 5800 / 5600 / 5500 / 5300, the 3D 512^3 steps 1450 / 1370 / 1330
    // against 790 / 700 / 680; without the cap the 2D steps did not converge.
    rb->phase_iters = std::max(p.nchk, 200);
    // two iterations per launch with an even check cadence: 2D (every model),
    // and 3D (LIN, NONLIN) when asked for (PTD_FLAG_RB_TBLOCK_3D: at 512^3
    // 1233 against 1243 us per iteration, issue-bound at half the bytes)
    const bool tb3 = p.ndim == 3 && (p.model == PTD_MODEL_LIN || p.model == PTD_MODEL_NONLIN) &&
                     (p.flags & PTD_FLAG_RB_TBLOCK_3D);
    rb->tblk = ((p.ndim == 2 || tb3) && p.nchk % 2 == 0 && !(p.flags & PTD_FLAG_DC_NO_TBLOCK)) ? 2 : 1;
    if (rb->tblk == 2 && p.ndim == 3)   // 28 x 12 level-2 cells per CTA, 2 CTAs per SM
        rb->cfg.chunk3d = z_chunk((long long)((p.nx - 2 + 27) / 28) * ((p.ny - 2 + 11) / 12), p.nz, 2LL * sm_count());
    rb->errcap = (p.nchk <= p.itmax ? p.itmax / p.nchk : 0) + 2;
    const size_t fb = (size_t)g.nfield * sizeof(float);
    auto alloc = [&](void** ptr, size_t n) -> int {
        cudaError_t e = cudaMalloc(ptr, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(e == cudaErrorMemoryAllocation ? PTD_ENOMEM : PTD_ECUDA, "rb: cudaMalloc failed");
        }
        return PTD_OK;
    };
    int rc = alloc((void**)&rb->d[0], fb);
    if (!rc) rc = alloc((void**)&rb->d[1], fb);
    for (int d = 0; d < p.ndim && !rc; ++d) {
        for (int q = 0; q < 2 && !rc; ++q) rc = alloc((void**)&rb->w[d][q], fb);
        if (!rc) rc = alloc((void**)&rb->tb[d], fb);
    }
    if (!rc) rc = alloc((void**)&rb->Rb, fb);
    if (!rc && p.ndim < 3) rc = alloc((void**)&rb->Cb, (size_t)g.nfield * sizeof(float));
    if (!rc && p.ndim == 3) rc = alloc((void**)&rb->Cb64, (size_t)g.nfield * sizeof(double));
    if (!rc) rc = alloc((void**)&rb->Hf, fb);
    if (!rc && (p.model == PTD_MODEL_LINSTEP || p.model == PTD_MODEL_NONLIN_EXPM)) rc = alloc((void**)&rb->Df, fb);
    if (!rc) rc = alloc((void**)&rb->dev, sizeof(RbDev));
    if (!rc) rc = alloc((void**)&rb->zero_flag, sizeof(int));
    if (!rc) rc = alloc((void**)&rb->errhist, (size_t)rb->errcap * sizeof(double));
    if (!rc) rc = rb_alloc_parts(rb);
    if (!rc && cudaMallocHost((void**)&rb->h_dev, sizeof(RbDev)) != cudaSuccess) {
        cudaGetLastError();
        rc = set_error(PTD_ENOMEM, "rb: cudaMallocHost failed");
    }
    if (!rc) {
        cudaError_t e = cudaMemsetAsync(rb->dev, 0, sizeof(RbDev), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(rb->zero_flag, 0, sizeof(int), s);
        for (int q = 0; q < 2 && e == cudaSuccess; ++q) e = cudaMemsetAsync(rb->d[q], 0, fb, s);
        for (int d = 0; d < p.ndim && e == cudaSuccess; ++d) {
            for (int q = 0; q < 2 && e == cudaSuccess; ++q) e = cudaMemsetAsync(rb->w[d][q], 0, fb, s);
            // faces past the last one of each direction are read (never used) by the halo lanes
            if (e == cudaSuccess) e = cudaMemsetAsync(rb->tb[d], 0, fb, s);
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(rb->Rb, 0, fb, s);
        if (e != cudaSuccess) rc = cuda_fail(e, "rb: cudaMemsetAsync");
    }
    if (rc) {
        rb_destroy(rb);
        return rc;
    }
    *out = rb;
    return PTD_OK;
}

void rb_destroy(RbState* rb)
{
    if (!rb) return;
    if (rb->s) cudaStreamSynchronize(rb->s);
    if (rb->gphase) cudaGraphExecDestroy(rb->gphase);
    cudaFree(rb->d[0]);
    cudaFree(rb->d[1]);
    for (int d = 0; d < 3; ++d) {
        cudaFree(rb->w[d][0]);
        cudaFree(rb->w[d][1]);
        cudaFree(rb->tb[d]);
    }
    cudaFree(rb->Rb);
    cudaFree(rb->Cb);
    cudaFree(rb->Cb64);
    cudaFree(rb->Hf);
    cudaFree(rb->Df);
    cudaFree(rb->dev);
    cudaFree(rb->zero_flag);
    cudaFree(rb->errhist);
    cudaFree(rb->parts);
    cudaFree(rb->parts64);
    if (rb->h_dev) cudaFreeHost(rb->h_dev);
    delete rb;
}

// The context's FP64 fields become the base: H_b = H, w_b = W (zeroed by the
// caller), Hold; the FP32 changes start at zero.
int rb_set_state(RbState* rb, double* H, double* Hold, double* const* wb, const double* D, cudaStream_t s)
{
    rb->H = H;
    rb->Hold = Hold;
    for (int d = 0; d < rb->p.ndim; ++d) rb->wb[d] = wb[d];
    rb->D = D;
    const size_t fb = (size_t)rb->g.nfield * sizeof(float);
    for (int q = 0; q < 2; ++q) RCK(cudaMemsetAsync(rb->d[q], 0, fb, s));
    for (int d = 0; d < rb->p.ndim; ++d)
        for (int q = 0; q < 2; ++q) RCK(cudaMemsetAsync(rb->w[d][q], 0, fb, s));
    if (rb->Df) {
        rb_tofloat_kernel<<<fill_blocks(), 256, 0, s>>>(D, rb->Df, rb->g.nfield);
        RCK(cudaGetLastError());
    }
    if (!rb->gphase) {
        int rc = rb_capture(rb);
        if (rc) return rc;
    }
    return PTD_OK;
}

int rb_step(RbState* rb, int32_t* iters, double* err_hist, int32_t err_cap, int32_t* n_err, int* nan_flag,
            int* capped)
{
    rb_reset_kernel<<<1, 1, 0, rb->s>>>(rb->dev);
    RCK(cudaGetLastError());
    RCK(launch_base(rb, base_args(rb), rb->dev));
    rb_base_judge_kernel<<<1, 256, 0, rb->s>>>(rb->dev, rb->parts64, rb->nparts64, rb->p.tol, rb->dv.norm_den,
                                               rb->p.norm == PTD_NORM_MAX, 0);
    RCK(cudaGetLastError());
    rb->k.launches += 3;
    rb->h_dev->step_done = DONE_RUNNING;
    rb->h_dev->iter = 0;
    rb->h_dev->nchecks = 0;
    if (rb->p.nchk <= rb->p.itmax) {
        // the whole step: phases until the FP64 judge stops it
        RCK(cudaGraphLaunch(rb->gphase, rb->s));
        RCK(cudaMemcpyAsync(rb->h_dev, rb->dev, sizeof(RbDev), cudaMemcpyDeviceToHost, rb->s));
        RCK(cudaStreamSynchronize(rb->s));
        rb->k.launches += (long long)rb->h_dev->blocks * rb->kernels_per_block +
                          rb->h_dev->blocks / rb->blocks_per_pass + 3LL * rb->h_dev->phases;
    }
    const RbDev& st = *rb->h_dev;
    int32_t iter = st.iter;
    *nan_flag = st.step_done == DONE_NAN;
    *capped = st.step_done == DONE_CAP || st.step_done == DONE_RUNNING;
    if (*capped && iter < rb->p.itmax) {
        // no further check block fits (or nchk > itmax: the perf scripts'
        // fixed iterations): the remaining PT iterations up to itmax without
        // checks, from the folded base, then fold them in
        const int32_t tail = rb->p.itmax - iter;
        int par = 0;
        long long nl = 0;
        RCK(rb_run_plain(rb, tail, rb->zero_flag, par, nl));
        rb_fold_kernel<<<fill_blocks(), 256, 0, rb->s>>>(fold_args(rb), par);
        RCK(cudaGetLastError());
        rb->k.launches += nl + 1;
        iter = rb->p.itmax;
    }
    *iters = iter;
    rb->k.iterations += iter;
    if (err_hist && st.nchecks > 0 && *n_err < err_cap) {
        const int k = std::min(st.nchecks, std::min(err_cap - *n_err, rb->errcap));
        RCK(cudaMemcpyAsync(err_hist + *n_err, rb->errhist, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost,
                            rb->s));
        *n_err += k;
    } else if (st.nchecks > 0 && *n_err < err_cap) {
        *n_err += std::min(st.nchecks, err_cap - *n_err);
    }
    RCK(cudaMemcpyAsync(rb->Hold, rb->H, (size_t)rb->g.nfield * sizeof(double), cudaMemcpyDeviceToDevice,
                        rb->s));
    RCK(cudaStreamSynchronize(rb->s));
    return PTD_OK;
}

// Fixed FP32 iterations without checks (perf protocol), then one rebase.
int rb_iterate(RbState* rb, int32_t niter)
{
    RCK(launch_base(rb, base_args(rb), nullptr));
    int par = 0;
    long long nl = 0;
    RCK(rb_run_plain(rb, niter, rb->zero_flag, par, nl));
    rb_fold_kernel<<<fill_blocks(), 256, 0, rb->s>>>(fold_args(rb), par);
    RCK(cudaGetLastError());
    rb->k.launches += nl + 2;
    rb->k.iterations += niter;
    return PTD_OK;
}

int rb_set_config(RbState* rb, const LaunchCfg& cfg)
{
    rb->cfg = cfg;
    const int rc = rb_alloc_parts(rb);
    if (rc) return rc;
    if (rb->gphase) {   // captured once the base fields are known (rb_set_state)
        cudaGraphExecDestroy(rb->gphase);
        rb->gphase = nullptr;
        return rb_capture(rb);
    }
    return PTD_OK;
}

DcCounters rb_counters(const RbState* rb) { return rb ? rb->k : DcCounters{}; }

}  // namespace ptd
