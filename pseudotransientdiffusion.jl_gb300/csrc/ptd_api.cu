// ptd_api.cu -- the C ABI (include/ptd.h): contexts, the physical-time and
// PT-iteration driver, host <-> device transfers.
//
// The driver restates the loop of the reference's diffusion_{1,2,3}D_()
// (scripts/diff_2D_nonlin.jl:76-91, the same in every solver script):
//   for each physical step: iter = 0, err = 2 tol;
//     while err > tol and iter < itmax: one PT iteration; iter += 1;
//       if iter % nout == 0: err = norm(ResH)/sqrt(length(ResH))
//     Hold = H; NaN check
// with the iterations, the checks and the stopping decision all on the GPU:
// one check block (nchk fused PT kernels, the last one also forming the
// residual, then a one-thread judge kernel that computes err and sets a done
// flag) is the body of a WHILE node of a CUDA graph, which the judge ends, so one graph launch runs a whole physical step and the host reads the
// small device state once per step.  The iteration count is exactly the
// reference's (the first multiple of nchk at which err <= tol).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/ptd.h"
#include "ptd_internal.h"
#include "ptd_num.cuh"

using namespace ptd;

namespace {

thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

}  // namespace

int ptd::set_error(int status, const char* msg)
{
    g_last_error = msg ? msg : "";
    return status;
}

int ptd::cuda_fail(cudaError_t e, const char* where)
{
    return fail(PTD_ECUDA, "%s: %s", where, cudaGetErrorString(e));
}

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return ptd::cuda_fail(_e, #call);   \
    } while (0)

// ---------------------------------------------------------------------------
extern "C" int ptd_abi_version(void) { return PTD_ABI_VERSION; }

extern "C" const char* ptd_strerror(int status)
{
    switch (status) {
    case PTD_OK: return "ok";
    case PTD_EINVAL: return "invalid argument";
    case PTD_ENAN: return "residual is NaN";
    case PTD_ENOTCONV: return "not converged within itmax";
    case PTD_ECUDA: return "CUDA error";
    case PTD_ENOMEM: return "out of memory";
    case PTD_ESTATE: return "call out of order";
    case PTD_ETIMEOUT: return "device wait timed out";
    }
    return "unknown status";
}

extern "C" const char* ptd_last_error(void) { return g_last_error.c_str(); }

extern "C" int ptd_params_init(ptd_params* p, int32_t ndim, int32_t model)
{
    if (!p) return fail(PTD_EINVAL, "ptd_params_init: p is NULL");
    if (ndim < 1 || ndim > 3) return fail(PTD_EINVAL, "ptd_params_init: ndim must be 1, 2 or 3");
    if (model < PTD_MODEL_LIN || model > PTD_MODEL_NONLIN_EXPM)
        return fail(PTD_EINVAL, "ptd_params_init: unknown model %d", model);
    std::memset(p, 0, sizeof(*p));
    p->ndim = ndim;
    p->model = model;
    const int n = ndim == 3 ? 64 : 512;
    p->nx = n;
    p->ny = ndim > 1 ? n : 1;
    p->nz = ndim > 2 ? n : 1;
    p->lx = p->ly = p->lz = 10.0;
    p->dt = 0.2;
    p->nt = 5;
    p->itmax = 100000;
    p->nchk = 10;
    p->precision = PTD_PREC_FP64;
    p->tol = 1e-8;
    if (ndim == 1) p->cfl = model == PTD_MODEL_NONLIN ? 1.0 : 0.99;
    else p->cfl = 1.0 / std::sqrt((double)ndim);
    p->resc = (model >= PTD_MODEL_NONLIN && ndim > 1) ? 1.0 / 1.2 : 1.0;
    p->D = 1.0;
    p->resid_mode = PTD_RESID_MIXED;
    p->norm = PTD_NORM_RMS;
    return PTD_OK;
}

int ptd::validate(const ptd_params* p)
{
    if (!p) return fail(PTD_EINVAL, "params is NULL");
    if (p->ndim < 1 || p->ndim > 3) return fail(PTD_EINVAL, "ndim must be 1, 2 or 3 (got %d)", p->ndim);
    if (p->model < PTD_MODEL_LIN || p->model > PTD_MODEL_NONLIN_EXPM)
        return fail(PTD_EINVAL, "unknown model %d", p->model);
    if (p->model == PTD_MODEL_NONLIN_EXPM && p->precision == PTD_PREC_FP32_DC)
        return fail(PTD_EINVAL, "the exp(m) H^3 model runs in FP64 or DF64");
    const int n[3] = {p->nx, p->ny, p->nz};
    for (int d = 0; d < 3; ++d) {
        if (d < p->ndim && n[d] < 3)
            return fail(PTD_EINVAL, "n[%d] = %d: each dimension needs >= 3 cells", d, n[d]);
        if (d >= p->ndim && n[d] != 1)
            return fail(PTD_EINVAL, "n[%d] = %d must be 1 for a %dD grid", d, n[d], p->ndim);
        if (n[d] > (1 << 30)) return fail(PTD_EINVAL, "n[%d] too large", d);
    }
    // padded cells, formed in floating point so that the test cannot overflow
    const double nxp = p->ndim == 1 ? (double)p->nx : std::ceil(p->nx / 32.0) * 32.0;
    if (nxp * (double)p->ny * (double)p->nz > (double)kMaxCells)
        return fail(PTD_EINVAL, "grid of %d x %d x %d cells too large (limit 2^40 cells)", p->nx, p->ny, p->nz);
    const double l[3] = {p->lx, p->ly, p->lz};
    for (int d = 0; d < p->ndim; ++d)
        if (!(l[d] > 0.0) || !std::isfinite(l[d])) return fail(PTD_EINVAL, "domain length %d must be > 0", d);
    if (!(p->dt > 0.0) || !std::isfinite(p->dt)) return fail(PTD_EINVAL, "dt must be > 0");
    if (p->nt < 0) return fail(PTD_EINVAL, "nt must be >= 0");
    if (p->itmax < 0) return fail(PTD_EINVAL, "itmax must be >= 0");
    if (p->nchk < 1) return fail(PTD_EINVAL, "nchk must be >= 1");
    if (!(p->tol >= 0.0)) return fail(PTD_EINVAL, "tol must be >= 0");
    if (!(p->cfl > 0.0) || !std::isfinite(p->cfl)) return fail(PTD_EINVAL, "cfl must be > 0");
    if (!(p->resc > 0.0) || !std::isfinite(p->resc)) return fail(PTD_EINVAL, "resc must be > 0");
    if (p->model < PTD_MODEL_NONLIN && (!(p->D > 0.0) || !std::isfinite(p->D)))
        return fail(PTD_EINVAL, "D must be > 0");
    if (p->precision != PTD_PREC_FP64 && p->precision != PTD_PREC_FP32_DC && p->precision != PTD_PREC_DF64 &&
        p->precision != PTD_PREC_DFH && p->precision != PTD_PREC_FP32_RB)
        return fail(PTD_EINVAL, "unknown precision %d", p->precision);
    if (p->precision == PTD_PREC_FP32_RB) {
        if (p->resid_mode != PTD_RESID_MIXED) return fail(PTD_EINVAL, "FP32_RB: mixed residual only");
    }
    if (p->resid_mode != PTD_RESID_MIXED && p->resid_mode != PTD_RESID_CONSISTENT)
        return fail(PTD_EINVAL, "unknown resid_mode %d", p->resid_mode);
    if (p->norm != PTD_NORM_RMS && p->norm != PTD_NORM_MAX) return fail(PTD_EINVAL, "unknown norm %d", p->norm);
    if (p->flags & ~(PTD_FLAG_STRICT | PTD_FLAG_AUTOTUNE | PTD_FLAG_DC_NO_TBLOCK | PTD_FLAG_RB_TBLOCK_3D))
        return fail(PTD_EINVAL, "unknown flags 0x%x", p->flags);
    for (int k = 0; k < 8; ++k)
        if (p->reserved[k]) return fail(PTD_EINVAL, "reserved fields must be zero");
    return PTD_OK;
}

// Scalar iteration parameters, restating the reference's a1 block
// (scripts/diff_2D_lin.jl:49-53, diff_2D_linstep.jl:67-71, diff_2D_nonlin.jl:59-62):
// dx = lx/nx, Vpdtau = CFL*min(dx..), L = max(lx..), Re = pi + sqrt(pi^2 + L^2/D/dt),
// theta = L/Vpdtau/Re, dtau = Vpdtau*L/D/Re.
void ptd::derive(const ptd_params& p, Derived& dv)
{
    const double pi = 3.141592653589793;
    const double l[3] = {p.lx, p.ly, p.lz};
    const int n[3] = {p.nx, p.ny, p.nz};
    double hmin = 0.0, L = 0.0;
    for (int d = 0; d < p.ndim; ++d) {
        dv.h[d] = l[d] / (double)n[d];
        hmin = d == 0 ? dv.h[d] : std::min(hmin, dv.h[d]);
        L = d == 0 ? l[d] : std::max(L, l[d]);
    }
    dv.vpdt = p.cfl * hmin;
    dv.L = L;
    dv.rdt = 1.0 / p.dt;
    double kappa = 1.0;
    dv.c_lin = dv.e_lin = 0.0;
    dv.k1 = dv.k2 = dv.k3 = 0.0;
    if (p.model == PTD_MODEL_LIN) {
        const double re = pi + std::sqrt(pi * pi + ((L * L / p.D) / p.dt));
        const double theta = (L / dv.vpdt) / re;
        const double dtau = ((dv.vpdt * L) / p.D) / re;
        dv.c_lin = 1.0 / (1.0 + theta);
        dv.e_lin = dtau / (1.0 + dtau / p.dt);
        kappa = p.D;
    } else if (p.model == PTD_MODEL_LINSTEP) {
        const double re = pi + std::sqrt(pi * pi + ((L * L / p.D) / p.dt));
        const double theta = (L / dv.vpdt) / re;
        dv.c_lin = 1.0 / (1.0 + theta);
        dv.k3 = re / (dv.vpdt * L);
        kappa = 0.5;
    } else {
        dv.k1 = 1.0 / (dv.vpdt * L * p.resc);
        dv.k2 = L * p.resc / dv.vpdt;
        kappa = p.model == PTD_MODEL_NONLIN_EXPM ? 0.0625 : 0.125;
    }
    for (int d = 0; d < 3; ++d) dv.sig[d] = d < p.ndim ? kappa / (dv.h[d] * dv.h[d]) : 0.0;
    dv.A = L * L / p.dt;
    long long inner = 1;
    for (int d = 0; d < p.ndim; ++d) inner *= (long long)(n[d] - 2);
    dv.norm_den = p.norm_len > 0.0 ? p.norm_len : (double)inner;
}

FParams ptd::fparams(const Derived& dv)
{
    FParams f;
    f.fA = (float)dv.A;
    f.fpi = 3.14159265358979f;
    f.fpi2 = (float)(3.141592653589793 * 3.141592653589793);
    f.fk1 = (float)dv.k1;
    f.fk2 = (float)dv.k2;
    f.fk3 = (float)dv.k3;
    f.frdt = (float)dv.rdt;
    return f;
}

void ptd::fill_args(const ptd_params& p, const Derived& dv, PTArgs& a)
{
    std::memset(&a, 0, sizeof(a));
    a.nx = p.nx;
    a.ny = p.ny;
    a.nz = p.nz;
    a.rdt = dv.rdt;
    for (int d = 0; d < 3; ++d) a.sig[d] = dv.sig[d];
    a.rdt_df = split_df(dv.rdt);
    for (int d = 0; d < 3; ++d) a.sig_df[d] = split_df(dv.sig[d]);
    a.fc_lin = (float)dv.c_lin;
    a.fe_lin = (float)dv.e_lin;
    a.f = fparams(dv);
    a.norm_max = p.norm == PTD_NORM_MAX;
    a.sq = 1;
    for (int d = 1; d < p.ndim; ++d) a.sq = a.sq && dv.sig[d] == dv.sig[0];
    a.rdt_sig = dv.rdt / dv.sig[0];
    a.rdt_sig_df = split_df(a.rdt_sig);
    a.fsig = (float)dv.sig[0];
}

// ---------------------------------------------------------------------------
int ptd::copy_field_in(const ptd_ctx_base& g, double* dst, const double* src, cudaStream_t s)
{
    const size_t w = (size_t)g.nx * sizeof(double);
    const size_t rows = (size_t)g.ny * g.nz;
    CK(cudaMemcpy2DAsync(dst, (size_t)g.sy * sizeof(double), src, w, w, rows, cudaMemcpyDefault, s));
    return PTD_OK;
}

int ptd::copy_field_out(const ptd_ctx_base& g, double* dst, const double* src, cudaStream_t s)
{
    const size_t w = (size_t)g.nx * sizeof(double);
    const size_t rows = (size_t)g.ny * g.nz;
    CK(cudaMemcpy2DAsync(dst, w, src, (size_t)g.sy * sizeof(double), w, rows, cudaMemcpyDefault, s));
    return PTD_OK;
}

// ---------------------------------------------------------------------------
struct ptd_ctx : ptd_ctx_base {
    ptd_params p;
    Derived dv;
    LaunchCfg cfg;
    cudaStream_t stream = nullptr;
    double* H[2] = {nullptr, nullptr};
    double* Hold = nullptr;
    double* W[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    double* D = nullptr;
    DevState* st = nullptr;
    double* parts = nullptr;      // check-residual partials, one slot per block / warp (fixed-order sum)
    long long parts_cap = 0;
    int* zero_flag = nullptr;
    double* errhist = nullptr;
    int errcap = 0;
    DevState* h_st = nullptr;     // pinned mirror of *st
    cudaGraphExec_t gstep[2] = {nullptr, nullptr};   // one physical step's check loop, per start parity
    cudaGraphExec_t gplain[2] = {nullptr, nullptr};
    int blocks_per_pass = 1;      // check blocks in the body of the step graph's loop
    int plain_len = 32;
    int cur = 0;                  // buffer holding the current H
    bool have_state = false;
    long long launches = 0, iterations = 0;
    int kernels_per_block = 0;
    DcState* dc = nullptr;        // FP32 defect-correction resources
    RbState* rb = nullptr;        // FP32 rebased-form resources
    bool df64 = false;            // H and Hold hold double-floats (PTD_PREC_DF64)
    bool ddf = false;             // D and the fluxes hold double-floats (PTD_PREC_DF64, PTD_PREC_DFH)
    int num = NUM_F64;            // number type of the PT kernels
    double* stage = nullptr;      // DF64: FP64 staging field for the host boundary
};

static void args_for(const ptd_ctx* c, int parity, const int* done, PTArgs& a)
{
    fill_args(c->p, c->dv, a);
    a.sy = c->sy;
    a.sz = c->sz;
    a.Hin = c->H[parity];
    a.Hout = c->H[parity ^ 1];
    a.Hold = c->Hold;
    for (int d = 0; d < 3; ++d) {
        a.win[d] = c->W[d][parity] ? c->W[d][parity] : c->W[0][parity];
        a.wout[d] = c->W[d][parity ^ 1] ? c->W[d][parity ^ 1] : c->W[0][parity ^ 1];
    }
    a.D = c->D;
    a.done = done;
    a.acc = &c->st->acc;
    a.parts = c->parts;
}

// The slot array of the check partials, large enough for the launch shape in use.
static int ensure_parts(ptd_ctx* c)
{
    const long long n = pt_check_slots(c->p.ndim, c->nx, c->ny, c->nz, c->cfg, c->p.resid_mode == PTD_RESID_CONSISTENT, c->num);
    if (n <= c->parts_cap) return PTD_OK;
    if (c->parts) {
        CK(cudaStreamSynchronize(c->stream));
        cudaFree(c->parts);
        c->parts = nullptr;
        c->parts_cap = 0;
    }
    const cudaError_t e = cudaMalloc((void**)&c->parts, (size_t)n * sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? PTD_ENOMEM : PTD_ECUDA, "cudaMalloc(check partials): %s",
                    cudaGetErrorString(e));
    }
    c->parts_cap = n;
    return PTD_OK;
}

// The PT iteration of one physical step as one CUDA graph: a WHILE node whose
// body is one check block (nchk fused PT kernels, the last one also forming
// the residual, then the judge), two blocks when nchk is odd so that every
// pass of the body starts on the same buffer parity.  The judge ends the loop
// when the step stops (err <= tol, NaN, or no full block left before itmax),
// so the graph runs exactly the reference's check blocks, and the host waits
// once per step.  Every pass of the body raises the iteration count by nchk
// until the judge stops the loop, so the loop ends within itmax/nchk passes.
static int capture_step(ptd_ctx* c, int parity, cudaGraphExec_t* out)
{
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
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
    err = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (err != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err, "cudaStreamBeginCaptureToGraph");
    }
    const int nchk = c->p.nchk;
    const int nblk = (nchk & 1) ? 2 : 1;
    const long long nparts =
        pt_check_slots(c->p.ndim, c->nx, c->ny, c->nz, c->cfg, c->p.resid_mode == PTD_RESID_CONSISTENT, c->num);
    int par = parity;
    int nk = 0;
    for (int b = 0; b < nblk && err == cudaSuccess; ++b) {
        for (int it = 0; it < nchk && err == cudaSuccess; ++it) {
            PTArgs a;
            args_for(c, par, &c->st->done, a);
            const bool check = it == nchk - 1;
            if (check && c->p.resid_mode == PTD_RESID_CONSISTENT) {
                err = launch_pt(a, c->p.ndim, c->p.model, false, c->num, c->cfg, c->stream);
                if (err == cudaSuccess) err = launch_resid_consistent(a, c->p.ndim, c->p.model, c->num, c->stream);
                nk += 2;
            } else {
                err = launch_pt(a, c->p.ndim, c->p.model, check, c->num, c->cfg, c->stream);
                nk += 1;
            }
            par ^= 1;
        }
        if (err == cudaSuccess)
            err = launch_judge_parts(c->st, c->parts, nparts, c->errhist, c->errcap, nchk, c->p.itmax, c->p.tol,
                                     c->dv.norm_den, c->p.norm == PTD_NORM_MAX, loop, c->stream);
        nk += 1;
    }
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &body);
    if (err != cudaSuccess || e2 != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err != cudaSuccess ? err : e2, "capture the check block of the step graph");
    }
    cudaError_t e3 = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return cuda_fail(e3, "cudaGraphInstantiate");
    c->kernels_per_block = nk / nblk;
    c->blocks_per_pass = nblk;
    return PTD_OK;
}

static int capture_plain(ptd_ctx* c, int parity, cudaGraphExec_t* out)
{
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int par = parity;
    cudaError_t err = cudaSuccess;
    for (int it = 0; it < c->plain_len && err == cudaSuccess; ++it) {
        PTArgs a;
        args_for(c, par, c->zero_flag, a);
        err = launch_pt(a, c->p.ndim, c->p.model, false, c->num, c->cfg, c->stream);
        par ^= 1;
    }
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (err != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(err, "capture plain block");
    }
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
    cudaError_t e3 = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return cuda_fail(e3, "cudaGraphInstantiate");
    return PTD_OK;
}

__global__ void fill_one_kernel(double* a, long long n, int df64)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        if (df64) reinterpret_cast<float2*>(a)[t] = make_float2(1.0f, 0.0f);
        else a[t] = 1.0;
    }
}

// Autotuner: on a synthetic state (H = 1, zero fluxes) time every launch
// shape of the fused kernel -- 2D: warps per CTA x rows per y march; 3D: z
// march length x warps per CTA -- and keep the fastest.
static int autotune(ptd_ctx* c)
{
    const bool d3 = c->p.ndim == 3;
    std::vector<LaunchCfg> cands;
    if (d3) {
        for (int rows : {8, 16})
            for (int ch : {16, 32, 64, 128, 256}) {
                LaunchCfg k = c->cfg;
                k.rows3d = rows;
                k.chunk3d = ch;
                cands.push_back(k);
            }
    } else {
        for (int w : {2, 4, 8})
            for (int ch : {16, 32, 64, 128}) {
                LaunchCfg k = c->cfg;
                k.warps2d = w;
                k.chunk2d = ch;
                cands.push_back(k);
            }
    }
    for (double* f : {c->H[0], c->H[1], c->Hold}) {
        fill_one_kernel<<<fill_blocks(), 256, 0, c->stream>>>(f, c->nfield, c->df64 ? 1 : 0);
        CK(cudaGetLastError());
    }
    if (c->D) {
        fill_one_kernel<<<fill_blocks(), 256, 0, c->stream>>>(c->D, c->nfield, c->ddf ? 1 : 0);
        CK(cudaGetLastError());
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    LaunchCfg bestc = c->cfg;
    for (const LaunchCfg& k : cands) {
        c->cfg = k;
        int par = 0;
        for (int rep = 0; rep < 2; ++rep) {
            CK(cudaEventRecord(e0, c->stream));
            for (int it = 0; it < 4; ++it) {
                PTArgs a;
                args_for(c, par, c->zero_flag, a);
                CK(launch_pt(a, c->p.ndim, c->p.model, false, c->num, c->cfg, c->stream));
                par ^= 1;
            }
            CK(cudaEventRecord(e1, c->stream));
            CK(cudaEventSynchronize(e1));
        }
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        c->launches += 8;
        if (ms < best) {
            best = ms;
            bestc = k;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->cfg = bestc;
    return PTD_OK;
}

static void free_ctx(ptd_ctx* c)
{
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (int q = 0; q < 2; ++q) {
        if (c->gstep[q]) cudaGraphExecDestroy(c->gstep[q]);
        if (c->gplain[q]) cudaGraphExecDestroy(c->gplain[q]);
    }
    if (c->dc) dc_destroy(c->dc);
    if (c->rb) rb_destroy(c->rb);
    cudaFree(c->H[0]);
    cudaFree(c->H[1]);
    cudaFree(c->Hold);
    for (int d = 0; d < 3; ++d)
        for (int q = 0; q < 2; ++q) cudaFree(c->W[d][q]);
    cudaFree(c->D);
    cudaFree(c->st);
    cudaFree(c->parts);
    cudaFree(c->zero_flag);
    cudaFree(c->errhist);
    cudaFree(c->stage);
    if (c->h_st) cudaFreeHost(c->h_st);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" int ptd_create(ptd_ctx** out, const ptd_params* p)
{
    if (!out) return fail(PTD_EINVAL, "ptd_create: ctx is NULL");
    *out = nullptr;
    int rc = validate(p);
    if (rc) return rc;
    ptd_ctx* c = new (std::nothrow) ptd_ctx();
    if (!c) return fail(PTD_ENOMEM, "ptd_create: host allocation failed");
    c->p = *p;
    derive(c->p, c->dv);
    c->nx = p->nx;
    c->ny = p->ny;
    c->nz = p->nz;
    c->sy = p->ndim == 1 ? p->nx : ((p->nx + 31) / 32) * 32;
    c->sz = c->sy * p->ny;
    c->nfield = c->sz * p->nz;
    c->cfg = tuned_config(*p);
    c->df64 = p->precision == PTD_PREC_DF64;
    c->ddf = c->df64 || p->precision == PTD_PREC_DFH;
    c->num = c->df64 ? NUM_DF64 : (p->precision == PTD_PREC_DFH ? NUM_DFH : NUM_F64);
    const size_t bytes = (size_t)c->nfield * sizeof(double);
    auto alloc = [&](void** ptr, size_t n) -> int {
        cudaError_t e = cudaMalloc(ptr, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(e == cudaErrorMemoryAllocation ? PTD_ENOMEM : PTD_ECUDA, "cudaMalloc(%zu): %s", n,
                        cudaGetErrorString(e));
        }
        return PTD_OK;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_ctx(c);
        return cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    rc = alloc((void**)&c->H[0], bytes);
    if (!rc) rc = alloc((void**)&c->H[1], bytes);
    if (!rc) rc = alloc((void**)&c->Hold, bytes);
    for (int d = 0; d < p->ndim && !rc; ++d)
        for (int q = 0; q < 2 && !rc; ++q) rc = alloc((void**)&c->W[d][q], bytes);
    if (!rc && (p->model == PTD_MODEL_LINSTEP || p->model == PTD_MODEL_NONLIN_EXPM))
        rc = alloc((void**)&c->D, bytes);
    if (!rc && (c->ddf || p->model == PTD_MODEL_NONLIN_EXPM)) rc = alloc((void**)&c->stage, bytes);
    if (!rc) rc = alloc((void**)&c->st, sizeof(DevState));
    if (!rc) rc = alloc((void**)&c->zero_flag, sizeof(int));
    c->errcap = (p->nchk <= p->itmax ? p->itmax / p->nchk : 0) + 2;
    if (!rc) rc = alloc((void**)&c->errhist, (size_t)c->errcap * sizeof(double));
    if (!rc && cudaMallocHost((void**)&c->h_st, sizeof(DevState)) != cudaSuccess) {
        cudaGetLastError();
        rc = fail(PTD_ENOMEM, "cudaMallocHost failed");
    }
    if (rc) {
        free_ctx(c);
        return rc;
    }
    e = cudaMemsetAsync(c->zero_flag, 0, sizeof(int), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->st, 0, sizeof(DevState), c->stream);
    if (e != cudaSuccess) {
        free_ctx(c);
        return cuda_fail(e, "cudaMemsetAsync");
    }
    if (p->precision == PTD_PREC_FP32_DC) {
        rc = dc_create(*c, c->p, c->dv, c->stream, &c->dc);
        if (rc) {
            free_ctx(c);
            return rc;
        }
    } else if (p->precision == PTD_PREC_FP32_RB) {
        rc = rb_create(*c, c->p, c->dv, c->stream, &c->rb);
        if (rc) {
            free_ctx(c);
            return rc;
        }
    } else {
        if ((p->flags & PTD_FLAG_AUTOTUNE) && p->ndim > 1) rc = autotune(c);
        if (!rc) rc = ensure_parts(c);
        for (int q = 0; q < 2 && !rc; ++q) {
            if (p->nchk <= p->itmax) rc = capture_step(c, q, &c->gstep[q]);
            if (!rc) rc = capture_plain(c, q, &c->gplain[q]);
        }
        if (rc) {
            free_ctx(c);
            return rc;
        }
    }
    *out = c;
    return PTD_OK;
}

extern "C" void ptd_destroy(ptd_ctx* c) { free_ctx(c); }

extern "C" void* ptd_stream(ptd_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" int ptd_launch_config(ptd_ctx* c, int32_t cfg[4])
{
    if (!c || !cfg) return fail(PTD_EINVAL, "ptd_launch_config: NULL argument");
    cfg[0] = c->cfg.warps2d;
    cfg[1] = c->cfg.chunk2d;
    cfg[2] = c->cfg.rows3d;
    cfg[3] = c->cfg.chunk3d;
    return PTD_OK;
}

extern "C" int ptd_set_launch_config(ptd_ctx* c, const int32_t cfg[4])
{
    if (!c || !cfg) return fail(PTD_EINVAL, "ptd_set_launch_config: NULL argument");
    if (cfg[0] != 1 && cfg[0] != 2 && cfg[0] != 4 && cfg[0] != 8)
        return fail(PTD_EINVAL, "warps per 2D CTA must be 1, 2, 4 or 8 (got %d)", cfg[0]);
    if (cfg[1] < 1 || cfg[1] > 4096) return fail(PTD_EINVAL, "rows per 2D march must be in [1, 4096]");
    if (cfg[2] != 8 && cfg[2] != 16) return fail(PTD_EINVAL, "warps per 3D CTA must be 8 or 16 (got %d)", cfg[2]);
    if (cfg[3] < 1 || cfg[3] > 4096) return fail(PTD_EINVAL, "planes per 3D march must be in [1, 4096]");
    LaunchCfg k = c->cfg;
    k.warps2d = cfg[0];
    k.chunk2d = cfg[1];
    k.rows3d = cfg[2];
    k.chunk3d = cfg[3];
    CK(cudaStreamSynchronize(c->stream));
    c->cfg = k;
    int rc = PTD_OK;
    if (c->dc) {
        rc = dc_set_config(c->dc, k);
    } else if (c->rb) {
        rc = rb_set_config(c->rb, k);
    } else {
        rc = ensure_parts(c);
        for (int q = 0; q < 2 && !rc; ++q) {
            if (c->gstep[q]) cudaGraphExecDestroy(c->gstep[q]);
            if (c->gplain[q]) cudaGraphExecDestroy(c->gplain[q]);
            c->gstep[q] = nullptr;
            c->gplain[q] = nullptr;
            if (c->p.nchk <= c->p.itmax) rc = capture_step(c, q, &c->gstep[q]);
            if (!rc) rc = capture_plain(c, q, &c->gplain[q]);
        }
    }
    return rc;
}

extern "C" int ptd_sync(ptd_ctx* c)
{
    if (!c) return fail(PTD_EINVAL, "ctx is NULL");
    CK(cudaStreamSynchronize(c->stream));
    return PTD_OK;
}

extern "C" int ptd_counters(ptd_ctx* c, int64_t* launches, int64_t* iters)
{
    if (!c) return fail(PTD_EINVAL, "ctx is NULL");
    long long l = c->launches, it = c->iterations;
    if (c->dc || c->rb) {
        const DcCounters k = c->dc ? dc_counters(c->dc) : rb_counters(c->rb);
        l += k.launches;
        it += k.iterations;
    }
    if (launches) *launches = l;
    if (iters) *iters = it;
    return PTD_OK;
}

extern "C" int ptd_set_state(ptd_ctx* c, const double* H, const double* D)
{
    return ptd_set_state2(c, H, nullptr, D);
}

extern "C" int ptd_set_state2(ptd_ctx* c, const double* H, const double* Hold, const double* D)
{
    if (!c) return fail(PTD_EINVAL, "ctx is NULL");
    if (!H) return fail(PTD_EINVAL, "H is NULL");
    if (c->p.model == PTD_MODEL_LINSTEP && !D) return fail(PTD_EINVAL, "the step model needs D");
    if (c->p.model == PTD_MODEL_NONLIN_EXPM && !D) return fail(PTD_EINVAL, "the exp(m) H^3 model needs m (in D)");
    const size_t bytes = (size_t)c->nfield * sizeof(double);
    // padding stays zero: clear whole buffers first
    double* Hdst = c->df64 ? c->stage : c->H[0];
    CK(cudaMemsetAsync(Hdst, 0, bytes, c->stream));
    int rc = copy_field_in(*c, Hdst, H, c->stream);
    if (rc) return rc;
    if (c->df64) {
        CK(launch_to_df64(c->stage, c->H[0], c->nfield, c->stream));
        c->launches += 1;
    }
    CK(cudaMemcpyAsync(c->H[1], c->H[0], bytes, cudaMemcpyDeviceToDevice, c->stream));
    if (Hold) {
        // a separate previous state (e.g. the reaction form: H from 0, Hold = Heq)
        double* Odst = c->df64 ? c->stage : c->Hold;
        CK(cudaMemsetAsync(Odst, 0, bytes, c->stream));
        rc = copy_field_in(*c, Odst, Hold, c->stream);
        if (rc) return rc;
        if (c->df64) {
            CK(launch_to_df64(c->stage, c->Hold, c->nfield, c->stream));
            c->launches += 1;
        }
    } else {
        CK(cudaMemcpyAsync(c->Hold, c->H[0], bytes, cudaMemcpyDeviceToDevice, c->stream));
    }
    for (int d = 0; d < 3; ++d)
        for (int q = 0; q < 2; ++q)
            if (c->W[d][q]) CK(cudaMemsetAsync(c->W[d][q], 0, bytes, c->stream));
    if (c->p.model == PTD_MODEL_NONLIN_EXPM) {
        CK(cudaMemsetAsync(c->stage, 0, bytes, c->stream));
        rc = copy_field_in(*c, c->stage, D, c->stream);
        if (rc) return rc;
        CK(launch_expm(c->stage, c->D, c->nfield, c->ddf, c->stream));
        c->launches += 1;
    }
    if (c->p.model == PTD_MODEL_LINSTEP) {
        double* Ddst = c->ddf ? c->stage : c->D;
        CK(cudaMemsetAsync(Ddst, 0, bytes, c->stream));
        rc = copy_field_in(*c, Ddst, D, c->stream);
        if (rc) return rc;
        if (c->ddf) {
            CK(launch_to_df64(c->stage, c->D, c->nfield, c->stream));
            c->launches += 1;
        }
    }
    c->cur = 0;
    if (c->dc) {
        rc = dc_set_state(c->dc, *c, c->H[0], c->Hold, c->D, c->stream);
        if (rc) return rc;
    }
    if (c->rb) {
        double* wb[3] = {c->W[0][0], c->W[1][0], c->W[2][0]};
        rc = rb_set_state(c->rb, c->H[0], c->Hold, wb, c->D, c->stream);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(c->stream));
    c->have_state = true;
    return PTD_OK;
}

extern "C" int ptd_get_state(ptd_ctx* c, double* H)
{
    if (!c) return fail(PTD_EINVAL, "ctx is NULL");
    if (!H) return fail(PTD_EINVAL, "H is NULL");
    if (!c->have_state) return fail(PTD_ESTATE, "no state set");
    const double* src = c->dc ? dc_current(c->dc) : c->H[c->cur];
    if (c->df64) {
        CK(launch_from_df64(src, c->stage, c->nfield, c->stream));
        c->launches += 1;
        src = c->stage;
    }
    int rc = copy_field_out(*c, H, src, c->stream);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return PTD_OK;
}

// Run n PT iterations without checks starting from buffer c->cur.
static int run_plain(ptd_ctx* c, long long n)
{
    while (n >= c->plain_len) {
        CK(cudaGraphLaunch(c->gplain[c->cur], c->stream));
        c->launches += c->plain_len;
        c->iterations += c->plain_len;
        if (c->plain_len & 1) c->cur ^= 1;
        n -= c->plain_len;
    }
    for (; n > 0; --n) {
        PTArgs a;
        args_for(c, c->cur, c->zero_flag, a);
        CK(launch_pt(a, c->p.ndim, c->p.model, false, c->num, c->cfg, c->stream));
        c->launches += 1;
        c->iterations += 1;
        c->cur ^= 1;
    }
    return PTD_OK;
}

extern "C" int ptd_iterate(ptd_ctx* c, int32_t niter)
{
    if (!c) return fail(PTD_EINVAL, "ctx is NULL");
    if (niter < 0) return fail(PTD_EINVAL, "niter must be >= 0");
    if (!c->have_state) return fail(PTD_ESTATE, "no state set");
    if (c->dc) return dc_iterate(c->dc, *c, niter);
    if (c->rb) return rb_iterate(c->rb, niter);
    return run_plain(c, niter);
}

// One physical step of the FP64 solver.  Returns the PT iteration count in
// *iters and appends the step's errors to err_hist.
static int fp64_step(ptd_ctx* c, int32_t* iters, double* err_hist, int32_t err_cap, int32_t* n_err,
                     int* nan_flag, int* capped)
{
    const ptd_params& p = c->p;
    CK(launch_reset_state(c->st, c->stream));
    c->launches += 1;
    const long long blocks_max = p.nchk <= p.itmax ? p.itmax / p.nchk : 0;
    const int start = c->cur;
    int done = DONE_RUNNING, iter = 0, nchecks = 0;
    if (blocks_max > 0) {
        CK(cudaGraphLaunch(c->gstep[start], c->stream));
        CK(cudaMemcpyAsync(c->h_st, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        done = c->h_st->done;
        iter = c->h_st->iter;
        nchecks = c->h_st->nchecks;
        // every pass of the loop body launches blocks_per_pass check blocks
        const long long passes = (nchecks + c->blocks_per_pass - 1) / c->blocks_per_pass;
        c->launches += passes * c->blocks_per_pass * c->kernels_per_block;
    }
    c->iterations += iter;
    c->cur = (start + iter) & 1;
    if (done == DONE_RUNNING || done == DONE_CAP) {
        const long long tail = (long long)p.itmax - iter;
        int rc = run_plain(c, tail);
        if (rc) return rc;
        iter = p.itmax;
        *capped = 1;
    }
    *iters = iter;
    const size_t bytes = (size_t)c->nfield * sizeof(double);
    CK(cudaMemcpyAsync(c->Hold, c->H[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
    if (err_hist && nchecks > 0 && *n_err < err_cap) {
        const int k = std::min(nchecks, std::min(err_cap - *n_err, c->errcap));
        CK(cudaMemcpyAsync(err_hist + *n_err, c->errhist, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost,
                           c->stream));
    }
    *n_err += nchecks;
    CK(cudaStreamSynchronize(c->stream));
    *nan_flag = done == DONE_NAN;
    return PTD_OK;
}

extern "C" int ptd_step(ptd_ctx* c, int32_t nsteps, int32_t* iters_per_step, double* err_hist,
                        int32_t err_cap, int32_t* n_err)
{
    if (!c) return fail(PTD_EINVAL, "ctx is NULL");
    if (nsteps < 0) return fail(PTD_EINVAL, "nsteps must be >= 0");
    if (!c->have_state) return fail(PTD_ESTATE, "no state set");
    if (err_cap < 0) return fail(PTD_EINVAL, "err_cap must be >= 0");
    int32_t ne = 0;
    int any_capped = 0;
    for (int s = 0; s < nsteps; ++s) {
        int32_t it = 0;
        int nan_flag = 0, capped = 0;
        int rc = c->dc   ? dc_step(c->dc, *c, &it, err_hist, err_cap, &ne, &nan_flag, &capped)
                 : c->rb ? rb_step(c->rb, &it, err_hist, err_cap, &ne, &nan_flag, &capped)
                         : fp64_step(c, &it, err_hist, err_cap, &ne, &nan_flag, &capped);
        if (rc) return rc;
        if (iters_per_step) iters_per_step[s] = it;
        any_capped |= capped;
        if (nan_flag) {
            if (n_err) *n_err = ne;
            return fail(PTD_ENAN, "residual is NaN after physical step %d", s + 1);
        }
    }
    if (n_err) *n_err = ne;
    if ((c->p.flags & PTD_FLAG_STRICT) && any_capped)
        return fail(PTD_ENOTCONV, "a physical step reached itmax = %d without err <= tol", c->p.itmax);
    return PTD_OK;
}

extern "C" int ptd_solve(ptd_ctx* c, double* H, const double* D, int32_t* iters_per_step,
                         double* err_hist, int32_t err_cap, int32_t* n_err)
{
    if (!c) return fail(PTD_EINVAL, "ctx is NULL");
    int rc = ptd_set_state(c, H, D);
    if (rc) return rc;
    int rs = ptd_step(c, c->p.nt, iters_per_step, err_hist, err_cap, n_err);
    if (rs && rs != PTD_ENAN && rs != PTD_ENOTCONV) return rs;
    rc = ptd_get_state(c, H);
    if (rc) return rc;
    return rs;
}

int ptd::ctx_current_f64(ptd_ctx* c, double* dst)
{
    const double* src = c->dc ? dc_current(c->dc) : c->H[c->cur];
    if (c->df64) {
        CK(launch_from_df64(src, dst, c->nfield, c->stream));
        c->launches += 1;
    } else {
        CK(cudaMemcpyAsync(dst, src, (size_t)c->nfield * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    }
    return PTD_OK;
}
