// ptd_dc.cu -- FP32 PT iterations inside an FP64 defect-correction loop.
//
// Per physical step the FP64 problem is F(H) = (H - Hold)/dt + div q(H) = 0
// with q the reference's face flux (K_f times the H difference, K_f = D,
// (D_L+D_R)/2 or ((H_L+H_R)/2)^3).  The outer loop is an inexact Newton
// iteration carried out in FP64 on the GPU:
//   r = -F(H)                       FP64 residual (both flux terms from H)
//   err = ||r|| (RMS or max);  stop when err <= tol
//   solve J delta = r  approximately with the accelerated PT iteration in
//                      FP32 (the same damped-wave scheme as the FP64 kernels,
//                      applied to the linearised operator J; K_f and the
//                      iteration parameters from an FP32 copy of H)
//   H += delta                      FP64
// J = I/dt + div(-K_f grad . - dK_f/dH grad H .) : for D = H^3 the Newton term
// 3 s^2 (H_R - H_L) (delta_L + delta_R) (s = H_L + H_R, scaled by 1/8) is
// included, so the outer iteration converges quadratically; the linear models
// have none.  H, the residual, its norm and the update stay FP64, which is
// what convergence to tol = 1e-8 needs; the FP32 inner iterations move half
// the bytes of the FP64 ones and run on the FP32 pipe.
//
// The inner iterations use the fused-kernel layout of ptd_pt.cu (31-cell x
// tiles per warp, y march in 2D, z march with shared-memory y exchange in 3D)
// and the same device-side check/judge/done protocol, so a CUDA graph of
// nchk inner iterations is replayed without a host round trip per check.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "ptd_internal.h"
#include "ptd_dc_body.cuh"

namespace ptd {

// The outer loop stops at an FP64 residual of kDcStop * tol.  The FP64 PT
// solve it stands in for stops at tol, so its H lies up to ~dt*tol (RMS) from
// the converged implicit step; stopping ten times lower puts this form's H
// well inside that band, so that what separates it from the FP64 solution is
// the FP64 solution's own stopping error.  Newton's fast final convergence
// makes the tighter stop cheap (at most one more outer correction).
constexpr double kDcStop = 0.1;

template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) dc1d_kernel(DcArgs a)
{
    if (dc_done(a.done)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    dc1d_body<MODEL, CHECK>(a, blockIdx.x, part, pmax);
    if (CHECK) block_reduce_residual(a.acc, a.norm_max, (double)part, widen_max32(pmax), a.parts, block_slot());
}

template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) dc2d_kernel(DcArgs a, int chunk)
{
    if (dc_done(a.done)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    // the body flushes its check partials into its warp's slot (last step of its march)
    dc2d_body<MODEL, CHECK>(a, blockIdx.x * blockDim.y + threadIdx.y, blockIdx.y, chunk, part, pmax, warp_slot());
}

// two inner iterations per launch (temporal blocking), see dc2d_tb2_body
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) dc2d_tb2_kernel(DcArgs a, int chunk)
{
    if (dc_done(a.done)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    // the body flushes its check partials into its warp's slot (last step of its march)
    dc2d_tb2_body<MODEL, CHECK>(a, blockIdx.x * blockDim.y + threadIdx.y, blockIdx.y, chunk, part, pmax,
                                warp_slot());
}

template <int MODEL, bool CHECK, int R>
__global__ void __launch_bounds__(32 * R) dc3d_kernel(DcArgs a, int chunk)
{
    if (dc_done(a.done)) return;
    float part = 0.0f;
    unsigned pmax = 0u;
    dc3d_body<MODEL, CHECK, R>(a, blockIdx.x, blockIdx.y, blockIdx.z, chunk, part, pmax);
    if (CHECK) block_reduce_residual(a.acc, a.norm_max, (double)part, widen_max32(pmax), a.parts, block_slot());
}

// ---------------------------------------------------------------------------
// FP64 residual r = -F(H) with both flux terms from H (consistent form of
// check_res!, scripts/diff_2D_nonlin.jl:41-44), written as FP32 for the
// inner solve and reduced (sum r^2 or max |r|) in FP64 into the block's slot
// of parts (summed in a fixed order by the outer judge).
template <int MODEL>
__global__ void __launch_bounds__(256) dc_resid64_kernel(PTArgs a, int ndim, float* rf, double* parts,
                                                         unsigned long long* hmax)
{
    unsigned long long hm = 0ull;
    const long long nix = a.nx - 2;
    const long long niy = ndim > 1 ? a.ny - 2 : 1;
    const long long niz = ndim > 2 ? a.nz - 2 : 1;
    const long long total = nix * niy * niz;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long ix = 1 + t % nix;
        const long long rest = t / nix;
        const long long iy = ndim > 1 ? 1 + rest % niy : 0;
        const long long iz = ndim > 2 ? 1 + rest / niy : 0;
        const long long c = iz * a.sz + iy * a.sy + ix;
        const long long st[3] = {1, a.sy, a.sz};
        const double* Hp = static_cast<const double*>(a.Hin);
        const double* Dp = static_cast<const double*>(a.D);
        const double H = Hp[c];
        double div = 0.0;
        for (int d = 0; d < ndim; ++d) {
            const double HR = Hp[c + st[d]], HL = Hp[c - st[d]];
            double uR, uL;
            if (MODEL == LIN) {
                uR = HR - H;
                uL = H - HL;
            } else if (MODEL == LINSTEP) {
                uR = (Dp[c] + Dp[c + st[d]]) * (HR - H);
                uL = (Dp[c - st[d]] + Dp[c]) * (H - HL);
            } else {
                const double sR = H + HR, sL = HL + H;
                uR = sR * sR * sR * (HR - H);
                uL = sL * sL * sL * (H - HL);
            }
            div = fma(uR - uL, a.sig[d], div);
        }
        const double r = fma(-(H - static_cast<const double*>(a.Hold)[c]), a.rdt, div);
        rf[c] = (float)r;
        accumulate_residual(r, part, pmax);
        const unsigned long long hb = (unsigned long long)__double_as_longlong(H) & 0x7fffffffffffffffull;
        hm = hb > hm ? hb : hm;
    }
    hm = warp_max_u64(hm);
    if ((threadIdx.x & 31) == 0 && hm) atomicMax(hmax, hm);
    block_reduce_residual(nullptr, a.norm_max, part, pmax, parts, blockIdx.x);
}

// H += a * delta on every cell (delta is zero on the boundary); refresh the FP32 copy.
__global__ void dc_apply_kernel(double* H, float* Hf, const float* delta, double a, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const double h = fma(a, (double)delta[t], H[t]);
        H[t] = h;
        Hf[t] = __double2float_rn(h);
    }
}

__global__ void dc_tofloat_kernel(const double* src, float* dst, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        dst[t] = __double2float_rn(src[t]);
}

// Outer judge: err of the FP64 residual; sets the inner target and resets
// the inner control block.  The target is max(eta, floor) * err with floor
// the attainable relative accuracy of an FP32 solve, ~ eps_32 * cond(J),
// cond(J) ~ 1 + dt * Dmax * sum_d 4/dx_d^2 (Dmax = H_max^3 for D = H^3).
__global__ void __launch_bounds__(256) dc_outer_judge_kernel(DcDev* st, const double* parts, long long nparts,
                                                             double norm_den, int norm_max, double rtol,
                                                             double tol, double cond_scale, double dconst,
                                                             int nonlin)
{
    const double acc = sum_slots(parts, nparts, norm_max);
    if (threadIdx.x != 0) return;
    st->outer_acc = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(norm_den);
    st->outer_err = err;
    const double hmax = __longlong_as_double((long long)st->hmax_bits);
    st->hmax_bits = 0ull;
    const double dmax = nonlin ? hmax * hmax * hmax : dconst;
    const double floor = fmin(0.5, 0.5 * 5.96e-8 * (1.0 + cond_scale * dmax));
    st->target = fmax(fmax(rtol, floor) * err, 0.25 * tol);
    st->done = 0;
    st->nchecks = 0;
    st->iter = 0;
    st->best_at = 0;
    st->acc = 0.0;
    st->err = 0.0;
    st->best = err;
}

// The inner judge, at the end of the body of the inner solve graph's WHILE
// node: it ends the loop when the inner solve stops.  Every pass adds nchk
// iterations until no further block fits in the solve's budget (cap), so the
// loop ends within cap/nchk passes.
__global__ void __launch_bounds__(256) dc_inner_judge_kernel(DcDev* st, const double* parts, long long nparts,
                                                             int nchk, double norm_den, int norm_max, int stall,
                                                             cudaGraphConditionalHandle loop)
{
    // every thread reads the flag before thread 0 can change it
    const bool done = st->done != 0;
    __syncthreads();
    if (done) {   // no inner kernel ran: the slots are stale
        if (threadIdx.x == 0) cudaGraphSetConditional(loop, 0);
        return;
    }
    const double acc = sum_slots(parts, nparts, norm_max);
    if (threadIdx.x != 0) return;
    st->acc = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(norm_den);
    st->err = err;
    st->nchecks += 1;
    st->iter += nchk;
    if (err < 0.95 * st->best) {
        st->best = err;
        st->best_at = st->nchecks;
    }
    if (!(err > st->target)) st->done = (err != err) ? DONE_NAN : DONE_CONVERGED;
    else if (st->iter + nchk > st->cap) st->done = DONE_CAP;
    // FP32 attainable accuracy reached (about eps_32 * cond(J)): the inner
    // residual has stopped decreasing (no 5% gain over the last `stall`
    // checks, a window that grows with the grid so that the PT transient of
    // a large grid is not mistaken for stagnation); the FP64 outer
    // correction takes over from here.
    else if (st->nchecks - st->best_at >= stall) st->done = DONE_CONVERGED;
    if (st->done) cudaGraphSetConditional(loop, 0);
}

// The iteration budget and the pass counter of the next inner solve.
__global__ void dc_inner_start_kernel(DcDev* st, int cap)
{
    st->cap = cap;
    st->passes = 0;
}

__global__ void dc_count_pass_kernel(DcDev* st) { st->passes += 1; }

// ---------------------------------------------------------------------------
struct DcState {
    ptd_params p;
    Derived dv;
    LaunchCfg cfg;
    cudaStream_t s = nullptr;
    int ndim = 0, model = 0;
    long long nfield = 0;
    float* d[2] = {nullptr, nullptr};
    float* w[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    float* Hf = nullptr;
    float* Df = nullptr;
    float* rf = nullptr;
    double* H = nullptr;       // owned by the context: current FP64 H
    double* Hold = nullptr;    // owned by the context
    const double* D = nullptr; // owned by the context (LINSTEP)
    DcDev* dev = nullptr;
    DcDev* h_dev = nullptr;
    int* zero_flag = nullptr;
    cudaGraphExec_t gblock[2] = {nullptr, nullptr};
    int kernels_per_block = 0;
    int nchk = 0;
    int tb = 1;                // inner iterations per launch (2: temporal blocking, 2D)
    int cur = 0;
    double rtol = 1e-3;
    int max_outer = 30;
    int stall = 6;             // inner stagnation window, in checks
    double* parts = nullptr;   // check-residual slots of the inner check launches
    long long nparts = 0;
    double* parts64 = nullptr; // FP64 residual slots of dc_resid64_kernel (one per block)
    long long nparts64 = 0;
    DcCounters k;
    ptd_ctx_base g;
};

template <int MODEL, bool CHECK>
static cudaError_t dc_launch_model(const DcArgs& a, int ndim, const LaunchCfg& cfg, cudaStream_t s, int tb)
{
    if (ndim == 1) {
        dc1d_kernel<MODEL, CHECK><<<(a.nx + 255) / 256, 256, 0, s>>>(a);
    } else if (ndim == 2 && tb == 2) {
        const int W = cfg.warps2d;
        const int tiles = (a.nx - 2 + 27) / 28;
        dim3 grid((tiles + W - 1) / W, (a.ny - 2 + cfg.chunk2d - 1) / cfg.chunk2d);
        dc2d_tb2_kernel<MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, cfg.chunk2d);
    } else if (ndim == 2) {
        const int W = cfg.warps2d;
        const int tiles = (a.nx - 2 + 30) / 31;
        dim3 grid((tiles + W - 1) / W, (a.ny - 2 + cfg.chunk2d - 1) / cfg.chunk2d);
        dc2d_kernel<MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, cfg.chunk2d);
    } else {
        const int tx = (a.nx - 2 + 30) / 31;
        dim3 grid(tx, (a.ny - 2 + 14) / 15, (a.nz - 2 + cfg.chunk3d - 1) / cfg.chunk3d);
        dc3d_kernel<MODEL, CHECK, 16><<<grid, dim3(32, 16), 0, s>>>(a, cfg.chunk3d);
    }
    return cudaGetLastError();
}

static cudaError_t dc_launch(const DcArgs& a, int ndim, int model, bool check, const LaunchCfg& cfg,
                             cudaStream_t s, int tb = 1)
{
    switch (model * 2 + (check ? 1 : 0)) {
    case 0: return dc_launch_model<LIN, false>(a, ndim, cfg, s, tb);
    case 1: return dc_launch_model<LIN, true>(a, ndim, cfg, s, tb);
    case 2: return dc_launch_model<LINSTEP, false>(a, ndim, cfg, s, tb);
    case 3: return dc_launch_model<LINSTEP, true>(a, ndim, cfg, s, tb);
    case 4: return dc_launch_model<NONLIN, false>(a, ndim, cfg, s, tb);
    case 5: return dc_launch_model<NONLIN, true>(a, ndim, cfg, s, tb);
    }
    return cudaErrorInvalidValue;
}

static void dc_args(const DcState* dc, int parity, const int* done, DcArgs& a)
{
    std::memset(&a, 0, sizeof(a));
    a.nx = dc->g.nx;
    a.ny = dc->g.ny;
    a.nz = dc->g.nz;
    a.sy = dc->g.sy;
    a.sz = dc->g.sz;
    a.rdt = (float)dc->dv.rdt;
    for (int d = 0; d < 3; ++d) a.sig[d] = (float)dc->dv.sig[d];
    a.c_lin = (float)dc->dv.c_lin;
    a.e_lin = (float)dc->dv.e_lin;
    a.f = fparams(dc->dv);
    a.din = dc->d[parity];
    a.dout = dc->d[parity ^ 1];
    for (int d = 0; d < 3; ++d) {
        a.win[d] = dc->w[d][parity] ? dc->w[d][parity] : dc->w[0][parity];
        a.wout[d] = dc->w[d][parity ^ 1] ? dc->w[d][parity ^ 1] : dc->w[0][parity ^ 1];
    }
    a.Hf = dc->Hf;
    a.Df = dc->Df;
    a.r = dc->rf;
    a.done = done;
    a.acc = &dc->dev->acc;
    a.parts = dc->parts;
    a.norm_max = dc->p.norm == PTD_NORM_MAX;
}

// Residual slots of an inner check launch with the current launch shape.
static long long dc_check_slots(const DcState* dc)
{
    const LaunchCfg& c = dc->cfg;
    if (dc->ndim == 1) return (dc->g.nx + 255) / 256;
    if (dc->ndim == 2) {
        const long long tiles = dc->tb == 2 ? (dc->g.nx - 2 + 27) / 28 : (dc->g.nx - 2 + 30) / 31;
        const int W = c.warps2d;
        return (tiles + W - 1) / W * W * (long long)((dc->g.ny - 2 + c.chunk2d - 1) / c.chunk2d);
    }
    return (long long)((dc->g.nx - 2 + 30) / 31) * ((dc->g.ny - 2 + 14) / 15) *
           ((dc->g.nz - 2 + c.chunk3d - 1) / c.chunk3d);
}

// (Re)allocate the residual slots for the current launch shape.
static int dc_alloc_parts(DcState* dc)
{
    const long long n = dc_check_slots(dc);
    if (n > dc->nparts) {
        cudaFree(dc->parts);
        dc->parts = nullptr;
        dc->nparts = 0;
        if (cudaMalloc((void**)&dc->parts, (size_t)n * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(PTD_ENOMEM, "dc: cudaMalloc failed");
        }
    }
    dc->nparts = n;
    if (!dc->parts64) {
        dc->nparts64 = fill_blocks();
        if (cudaMalloc((void**)&dc->parts64, (size_t)dc->nparts64 * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(PTD_ENOMEM, "dc: cudaMalloc failed");
        }
    }
    return PTD_OK;
}

#define DCK(call)                                                 \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);       \
    } while (0)

// One inner solve as one CUDA graph: a WHILE node whose body is one check
// block (nchk/tb inner launches and the inner judge; two blocks when that
// launch count is odd, so that every pass starts on the same buffer parity),
// ended by the judge.
static int dc_capture(DcState* dc, int parity)
{
    cudaGraph_t g = nullptr;
    DCK(cudaGraphCreate(&g, 0));
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
    err = cudaStreamBeginCaptureToGraph(dc->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (err != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err, "cudaStreamBeginCaptureToGraph");
    }
    int par = parity, nk = 0;
    const int nl = dc->nchk / dc->tb;   // launches per check block
    const int nblk = (nl & 1) ? 2 : 1;
    for (int b = 0; b < nblk && err == cudaSuccess; ++b) {
        for (int it = 0; it < nl && err == cudaSuccess; ++it) {
            DcArgs a;
            dc_args(dc, par, &dc->dev->done, a);
            err = dc_launch(a, dc->ndim, dc->model, it == nl - 1, dc->cfg, dc->s, dc->tb);
            ++nk;
            par ^= 1;
        }
        if (err == cudaSuccess && b == 0) {
            dc_count_pass_kernel<<<1, 1, 0, dc->s>>>(dc->dev);
            err = cudaGetLastError();
            ++nk;
        }
        if (err == cudaSuccess) {
            dc_inner_judge_kernel<<<1, 256, 0, dc->s>>>(dc->dev, dc->parts, dc->nparts, dc->nchk, dc->dv.norm_den,
                                                         dc->p.norm == PTD_NORM_MAX, dc->stall, loop);
            err = cudaGetLastError();
            ++nk;
        }
    }
    cudaError_t e2 = cudaStreamEndCapture(dc->s, &body);
    if (err != cudaSuccess || e2 != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err != cudaSuccess ? err : e2, "capture inner block");
    }
    cudaError_t e3 = cudaGraphInstantiate(&dc->gblock[parity], g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return cuda_fail(e3, "cudaGraphInstantiate");
    dc->kernels_per_block = nk;   // per pass
    return PTD_OK;
}

int dc_create(const ptd_ctx_base& g, const ptd_params& p, const Derived& dv, cudaStream_t s, DcState** out)
{
    *out = nullptr;
    DcState* dc = new (std::nothrow) DcState();
    if (!dc) return set_error(PTD_ENOMEM, "dc_create: host allocation failed");
    dc->p = p;
    dc->dv = dv;
    dc->g = g;
    dc->s = s;
    dc->ndim = p.ndim;
    dc->model = p.model;
    dc->nfield = g.nfield;
    dc->cfg = tuned_config(p);
    dc->nchk = std::max(1, std::min(p.nchk, 50));
    // 2D: two inner iterations per launch when a check block has an even count
    dc->tb = (p.ndim == 2 && dc->nchk % 2 == 0 && !(p.flags & PTD_FLAG_DC_NO_TBLOCK)) ? 2 : 1;
    dc->rtol = p.dc_inner_rtol > 0.0 ? p.dc_inner_rtol : 1e-3;
    dc->max_outer = p.dc_max_outer > 0 ? p.dc_max_outer : 30;
    {
        const int nmax = std::max(p.nx, std::max(p.ny, p.nz));
        dc->stall = std::max(10, (2 * nmax + dc->nchk - 1) / dc->nchk);
    }
    const size_t fb = (size_t)g.nfield * sizeof(float);
    auto alloc = [&](void** ptr, size_t n) -> int {
        cudaError_t e = cudaMalloc(ptr, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(e == cudaErrorMemoryAllocation ? PTD_ENOMEM : PTD_ECUDA, "dc: cudaMalloc failed");
        }
        return PTD_OK;
    };
    int rc = alloc((void**)&dc->d[0], fb);
    if (!rc) rc = alloc((void**)&dc->d[1], fb);
    for (int d = 0; d < p.ndim && !rc; ++d)
        for (int q = 0; q < 2 && !rc; ++q) rc = alloc((void**)&dc->w[d][q], fb);
    if (!rc) rc = alloc((void**)&dc->Hf, fb);
    if (!rc) rc = alloc((void**)&dc->rf, fb);
    if (!rc && p.model == PTD_MODEL_LINSTEP) rc = alloc((void**)&dc->Df, fb);
    if (!rc) rc = alloc((void**)&dc->dev, sizeof(DcDev));
    if (!rc) rc = alloc((void**)&dc->zero_flag, sizeof(int));
    if (!rc && cudaMallocHost((void**)&dc->h_dev, sizeof(DcDev)) != cudaSuccess) {
        cudaGetLastError();
        rc = set_error(PTD_ENOMEM, "dc: cudaMallocHost failed");
    }
    if (!rc) {
        cudaError_t e = cudaMemsetAsync(dc->dev, 0, sizeof(DcDev), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(dc->zero_flag, 0, sizeof(int), s);
        if (e != cudaSuccess) rc = cuda_fail(e, "dc: cudaMemsetAsync");
    }
    if (!rc) rc = dc_alloc_parts(dc);
    for (int q = 0; q < 2 && !rc; ++q) rc = dc_capture(dc, q);
    if (rc) {
        dc_destroy(dc);
        return rc;
    }
    *out = dc;
    return PTD_OK;
}

void dc_destroy(DcState* dc)
{
    if (!dc) return;
    if (dc->s) cudaStreamSynchronize(dc->s);
    for (int q = 0; q < 2; ++q)
        if (dc->gblock[q]) cudaGraphExecDestroy(dc->gblock[q]);
    cudaFree(dc->d[0]);
    cudaFree(dc->d[1]);
    for (int d = 0; d < 3; ++d)
        for (int q = 0; q < 2; ++q) cudaFree(dc->w[d][q]);
    cudaFree(dc->Hf);
    cudaFree(dc->rf);
    cudaFree(dc->Df);
    cudaFree(dc->dev);
    cudaFree(dc->zero_flag);
    cudaFree(dc->parts);
    cudaFree(dc->parts64);
    if (dc->h_dev) cudaFreeHost(dc->h_dev);
    delete dc;
}

int dc_set_state(DcState* dc, const ptd_ctx_base&, double* H, double* Hold, const double* D, cudaStream_t s)
{
    dc->H = H;
    dc->Hold = Hold;
    dc->D = D;
    const size_t fb = (size_t)dc->nfield * sizeof(float);
    DCK(cudaMemsetAsync(dc->d[0], 0, fb, s));
    DCK(cudaMemsetAsync(dc->d[1], 0, fb, s));
    for (int d = 0; d < 3; ++d)
        for (int q = 0; q < 2; ++q)
            if (dc->w[d][q]) DCK(cudaMemsetAsync(dc->w[d][q], 0, fb, s));
    DCK(cudaMemsetAsync(dc->rf, 0, fb, s));
    const int nb = fill_blocks();
    dc_tofloat_kernel<<<nb, 256, 0, s>>>(H, dc->Hf, dc->nfield);
    DCK(cudaGetLastError());
    if (dc->Df) {
        dc_tofloat_kernel<<<nb, 256, 0, s>>>(D, dc->Df, dc->nfield);
        DCK(cudaGetLastError());
    }
    dc->cur = 0;
    return PTD_OK;
}

static int dc_residual(DcState* dc, double eta, double* err)
{
    PTArgs a;
    fill_args(dc->p, dc->dv, a);
    a.sy = dc->g.sy;
    a.sz = dc->g.sz;
    a.Hin = dc->H;
    a.Hold = dc->Hold;
    a.D = dc->D;
    const int nb = (int)dc->nparts64;   // one slot per block
    unsigned long long* hm = &dc->dev->hmax_bits;
    if (dc->model == LIN) dc_resid64_kernel<LIN><<<nb, 256, 0, dc->s>>>(a, dc->ndim, dc->rf, dc->parts64, hm);
    else if (dc->model == LINSTEP)
        dc_resid64_kernel<LINSTEP><<<nb, 256, 0, dc->s>>>(a, dc->ndim, dc->rf, dc->parts64, hm);
    else dc_resid64_kernel<NONLIN><<<nb, 256, 0, dc->s>>>(a, dc->ndim, dc->rf, dc->parts64, hm);
    DCK(cudaGetLastError());
    double cond_scale = 0.0;
    for (int d = 0; d < dc->ndim; ++d) cond_scale += 4.0 / (dc->dv.h[d] * dc->dv.h[d]);
    cond_scale *= dc->p.dt;
    dc_outer_judge_kernel<<<1, 256, 0, dc->s>>>(dc->dev, dc->parts64, dc->nparts64, dc->dv.norm_den,
                                                dc->p.norm == PTD_NORM_MAX, eta, kDcStop * dc->p.tol, cond_scale,
                                                dc->p.D, dc->model == NONLIN);
    DCK(cudaGetLastError());
    dc->k.launches += 2;
    DCK(cudaMemcpyAsync(dc->h_dev, dc->dev, sizeof(DcDev), cudaMemcpyDeviceToHost, dc->s));
    DCK(cudaStreamSynchronize(dc->s));
    *err = dc->h_dev->outer_err;
    return PTD_OK;
}

// Inner FP32 solve of J delta = r from delta = 0; returns its iterations.
static int dc_inner(DcState* dc, long long budget, int* iters)
{
    const size_t fb = (size_t)dc->nfield * sizeof(float);
    DCK(cudaMemsetAsync(dc->d[0], 0, fb, dc->s));
    DCK(cudaMemsetAsync(dc->d[1], 0, fb, dc->s));
    for (int d = 0; d < dc->ndim; ++d) {
        DCK(cudaMemsetAsync(dc->w[d][0], 0, fb, dc->s));
        DCK(cudaMemsetAsync(dc->w[d][1], 0, fb, dc->s));
    }
    dc->cur = 0;
    // at least one block even when the step's budget is spent (as before)
    const long long cap = std::max<long long>(dc->nchk, std::min<long long>(budget, 1LL << 30));
    dc_inner_start_kernel<<<1, 1, 0, dc->s>>>(dc->dev, (int)cap);
    DCK(cudaGetLastError());
    DCK(cudaGraphLaunch(dc->gblock[0], dc->s));
    DCK(cudaMemcpyAsync(dc->h_dev, dc->dev, sizeof(DcDev), cudaMemcpyDeviceToHost, dc->s));
    DCK(cudaStreamSynchronize(dc->s));
    const int iter = dc->h_dev->iter;
    dc->k.launches += 1 + (long long)dc->h_dev->passes * dc->kernels_per_block;
    dc->cur = (iter / dc->tb) & 1;   // one buffer swap per launch
    dc->k.iterations += iter;
    *iters = iter;
    return PTD_OK;
}

static int dc_apply(DcState* dc, double a)
{
    dc_apply_kernel<<<fill_blocks(), 256, 0, dc->s>>>(dc->H, dc->Hf, dc->d[dc->cur], a, dc->nfield);
    DCK(cudaGetLastError());
    dc->k.launches += 1;
    return PTD_OK;
}

// One physical step: inexact Newton in FP64 around FP32 PT inner solves.
// Forcing term (inner relative tolerance) eta: 0.1 on the first correction,
// then Eisenstat-Walker 0.9*(err_k/err_{k-1})^2 clamped to [dc_inner_rtol, 0.5];
// a correction that does not lower the FP64 residual is halved (at most 4 times).
int dc_step(DcState* dc, const ptd_ctx_base& g, int32_t* iters, double* err_hist, int32_t err_cap,
            int32_t* n_err, int* nan_flag, int* capped)
{
    (void)g;
    long long total = 0;
    int converged = 0;
    double err_prev = -1.0, eta = 0.1;
    int outer = 0;
    double err = 0.0;
    int rc = dc_residual(dc, eta, &err);
    if (rc) return rc;
    while (true) {
        if (err_hist && *n_err < err_cap) err_hist[*n_err] = err;
        *n_err += 1;
        if (err <= kDcStop * dc->p.tol) {
            converged = 1;
            break;
        }
        if (outer >= dc->max_outer || total >= dc->p.itmax || err != err) break;
        if (err_prev > 0.0) eta = std::min(0.5, std::max(dc->rtol, 0.9 * (err / err_prev) * (err / err_prev)));
        // dc_residual left r and the inner target for this eta in place
        if (err_prev > 0.0) {
            rc = dc_residual(dc, eta, &err);
            if (rc) return rc;
        }
        int it = 0;
        rc = dc_inner(dc, (long long)dc->p.itmax - total, &it);
        if (rc) return rc;
        total += it;
        rc = dc_apply(dc, 1.0);
        if (rc) return rc;
        double err_new = 0.0;
        rc = dc_residual(dc, eta, &err_new);
        if (rc) return rc;
        double a = 1.0;
        for (int h = 0; h < 4 && !(err_new < err); ++h) {   // also catches NaN
            rc = dc_apply(dc, -0.5 * a);
            if (rc) return rc;
            a *= 0.5;
            rc = dc_residual(dc, eta, &err_new);
            if (rc) return rc;
        }
        err_prev = err;
        err = err_new;
        ++outer;
    }
    if (err != err) *nan_flag = 1;
    *iters = (int32_t)total;
    if (!converged && !*nan_flag) *capped = 1;
    const size_t bytes = (size_t)dc->nfield * sizeof(double);
    DCK(cudaMemcpyAsync(dc->Hold, dc->H, bytes, cudaMemcpyDeviceToDevice, dc->s));
    DCK(cudaStreamSynchronize(dc->s));
    return PTD_OK;
}

int dc_set_config(DcState* dc, const LaunchCfg& cfg)
{
    DCK(cudaStreamSynchronize(dc->s));   // the slots may be reallocated
    dc->cfg = cfg;
    const int rc = dc_alloc_parts(dc);
    if (rc) return rc;
    for (int q = 0; q < 2; ++q) {
        if (dc->gblock[q]) cudaGraphExecDestroy(dc->gblock[q]);
        dc->gblock[q] = nullptr;
        int rc = dc_capture(dc, q);
        if (rc) return rc;
    }
    return PTD_OK;
}

int dc_iterate(DcState* dc, const ptd_ctx_base&, int32_t niter)
{
    // fixed inner iterations (perf protocol): two per launch where the
    // temporally blocked kernel is in use, a single one for an odd remainder
    int32_t it = 0;
    while (it < niter) {
        const int tb = (dc->tb == 2 && niter - it >= 2) ? 2 : 1;
        DcArgs a;
        dc_args(dc, dc->cur, dc->zero_flag, a);
        DCK(dc_launch(a, dc->ndim, dc->model, false, dc->cfg, dc->s, tb));
        dc->cur ^= 1;
        dc->k.launches += 1;
        dc->k.iterations += tb;
        it += tb;
    }
    return PTD_OK;
}

const double* dc_current(const DcState* dc) { return dc->H; }
DcCounters dc_counters(const DcState* dc) { return dc ? dc->k : DcCounters{}; }

}  // namespace ptd
