// ptd_noalloc.cu -- a 2D FP64 solve that allocates nothing.
//
// Some callers cannot allocate GPU memory at the moment they need a solve:
// code that runs under a memory-pool or allocator policy that forbids new
// device allocations (a host framework that has already reserved the whole
// device for its own pool), callbacks invoked while such an allocator holds
// its lock, or embedded drivers that must not grow their footprint after
// start-up.  ptd_solve_2d_noalloc serves them: it runs the same fused FP64 PT
// kernel as ptd_solve on caller-owned device buffers, and takes every piece
// of scratch (the second H buffer, Hold, the double-buffered fluxes and the
// device control block) from one file-scope device array of fixed size
// instead of cudaMalloc.  It creates no stream, graph or pinned buffer
// either: it launches on the caller's stream and reads its few control words
// back into pageable host memory.
//
// The array belongs to this file's device module.  The CUDA runtime loads a
// module on a device lazily (the default module loading of CUDA 12.2 and
// later), so the array's 24 MiB are reserved on a device the first time this
// entry point runs there (its cudaGetSymbolAddress), and stay reserved until
// the process exits; the kernels a solve launches are loaded the same way.  A
// caller that cannot allocate later makes that first call at start-up, before
// its own allocator takes the device: a call with p->nt = 0 maps the array,
// loads the kernels and returns.
#include <cstring>
#include <mutex>

#include "../../include/ptd.h"
#include "ptd_internal.h"

namespace ptd {

// 6 FP64 fields of PTD_NOALLOC_MAX_CELLS cells (H1, Hold, 2 x-flux, 2 y-flux
// buffers) plus the control block: 24 MiB + 4 KiB.
constexpr long long kScratchDoubles = 6LL * PTD_NOALLOC_MAX_CELLS + 512;
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

namespace {

std::mutex g_mu;
double* g_addr[64] = {nullptr};   // device address of the array, per device

// Once per device, with that device current: the device address of the
// array (host code cannot use the symbol itself as a device pointer).
int scratch_address(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return set_error(PTD_EINVAL, "ptd_solve_2d_noalloc: device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return PTD_OK;
}

}  // namespace
}  // namespace ptd

using namespace ptd;

#define NCK(call)                                                 \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);       \
    } while (0)

extern "C" int ptd_solve_2d_noalloc(const ptd_params* p, double* H, const double* D, void* stream,
                                    int32_t* iters_per_step)
{
    int rc = validate(p);
    if (rc) return rc;
    // map the array on this device first, so that a call with nt = 0 (the
    // start-up call) reserves it and touches nothing else
    double* base = nullptr;
    rc = scratch_address(&base);
    if (rc) return rc;
    if (p->nt == 0) {
        // the start-up call: also load the kernels a solve launches, so that
        // later calls leave the device's memory reservation unchanged
        NCK(preload_pt2d_f64());
        return PTD_OK;
    }
    if (p->ndim != 2) return set_error(PTD_EINVAL, "ptd_solve_2d_noalloc: 2D grids only");
    if (p->precision != PTD_PREC_FP64) return set_error(PTD_EINVAL, "ptd_solve_2d_noalloc: FP64 only");
    if (p->model != PTD_MODEL_LIN && p->model != PTD_MODEL_LINSTEP && p->model != PTD_MODEL_NONLIN)
        return set_error(PTD_EINVAL, "ptd_solve_2d_noalloc: models LIN, LINSTEP, NONLIN only");
    if (p->resid_mode != PTD_RESID_MIXED) return set_error(PTD_EINVAL, "ptd_solve_2d_noalloc: mixed residual only");
    const long long N = (long long)p->nx * p->ny;
    if (N > PTD_NOALLOC_MAX_CELLS)
        return set_error(PTD_EINVAL, "ptd_solve_2d_noalloc: nx*ny exceeds PTD_NOALLOC_MAX_CELLS (524288)");
    if (!H) return set_error(PTD_EINVAL, "ptd_solve_2d_noalloc: H is NULL");
    if (p->model == PTD_MODEL_LINSTEP && !D) return set_error(PTD_EINVAL, "ptd_solve_2d_noalloc: the step model needs D");
    // H (and D) must be plain device memory of the current device, the device
    // whose copy of the array the kernels use (managed or host memory, or
    // memory of another GPU, would be read across the interconnect)
    int dev = 0;
    NCK(cudaGetDevice(&dev));
    const double* const ptrs[2] = {H, p->model == PTD_MODEL_LINSTEP ? D : nullptr};
    for (int k = 0; k < 2; ++k) {
        if (!ptrs[k]) continue;
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, ptrs[k]) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
            at.device != dev) {
            cudaGetLastError();
            return set_error(PTD_EINVAL, k == 0 ? "ptd_solve_2d_noalloc: H must be device memory of the current device"
                                                : "ptd_solve_2d_noalloc: D must be device memory of the current device");
        }
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // carve the array: H1 | Hold | wx0 | wx1 | wy0 | wy1 | control block
    double* Hb[2] = {H, base};
    double* Hold = base + N;
    double* W[2][2] = {{base + 2 * N, base + 3 * N}, {base + 4 * N, base + 5 * N}};
    DevState* st = reinterpret_cast<DevState*>(base + 6 * N);
    const size_t bytes = (size_t)N * sizeof(double);

    // the array keeps the previous call's contents: start from zero fluxes
    // and a zero control block
    NCK(cudaMemsetAsync(W[0][0], 0, 4 * bytes, s));
    NCK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
    NCK(cudaMemcpyAsync(Hb[1], H, bytes, cudaMemcpyDeviceToDevice, s));
    NCK(cudaMemcpyAsync(Hold, H, bytes, cudaMemcpyDeviceToDevice, s));

    Derived dv;
    derive(*p, dv);
    LaunchCfg cfg = tuned_config(*p);
    auto args = [&](int par, PTArgs& a) {
        fill_args(*p, dv, a);
        a.sy = p->nx;
        a.sz = N;
        a.Hin = Hb[par];
        a.Hout = Hb[par ^ 1];
        a.Hold = Hold;
        for (int d = 0; d < 3; ++d) {
            a.win[d] = W[d < 2 ? d : 0][par];
            a.wout[d] = W[d < 2 ? d : 0][par ^ 1];
        }
        a.D = D;
        a.done = &st->done;
        a.acc = &st->acc;
    };
    const long long blocks_max = p->nchk <= p->itmax ? p->itmax / p->nchk : 0;
    DevState hs;
    int any_capped = 0;
    for (int step = 0; step < p->nt; ++step) {
        NCK(launch_reset_state(st, s));
        int par = 0, done = DONE_RUNNING, iter = 0;
        for (long long blk = 0; blk < blocks_max; ++blk) {
            for (int it = 0; it < p->nchk; ++it) {
                PTArgs a;
                args(par, a);
                NCK(launch_pt(a, 2, p->model, it == p->nchk - 1, false, cfg, s));
                par ^= 1;
            }
            NCK(launch_judge(st, nullptr, 0, p->nchk, p->itmax, p->tol, dv.norm_den, p->norm == PTD_NORM_MAX, s));
            if ((blk & 7) == 7 || blk == blocks_max - 1) {
                NCK(cudaMemcpyAsync(&hs, st, sizeof(DevState), cudaMemcpyDeviceToHost, s));
                NCK(cudaStreamSynchronize(s));
                done = hs.done;
                iter = hs.iter;
                if (done != DONE_RUNNING) break;
            }
        }
        par = iter & 1;   // blocks after `done` returned at entry
        if (done == DONE_RUNNING || done == DONE_CAP) {
            for (long long t = iter; t < p->itmax; ++t) {
                PTArgs a;
                args(par, a);
                a.done = reinterpret_cast<const int*>(&st->pad);   // always zero: no skipping in the tail
                NCK(launch_pt(a, 2, p->model, false, false, cfg, s));
                par ^= 1;
            }
            iter = p->itmax;
            any_capped = 1;
        }
        if (iters_per_step) iters_per_step[step] = iter;
        if (par) {   // bring the state back to the caller's buffer
            NCK(cudaMemcpyAsync(H, Hb[1], bytes, cudaMemcpyDeviceToDevice, s));
            NCK(cudaMemcpyAsync(W[0][0], W[0][1], bytes, cudaMemcpyDeviceToDevice, s));
            NCK(cudaMemcpyAsync(W[1][0], W[1][1], bytes, cudaMemcpyDeviceToDevice, s));
        }
        NCK(cudaMemcpyAsync(Hold, H, bytes, cudaMemcpyDeviceToDevice, s));
        NCK(cudaMemcpyAsync(Hb[1], H, bytes, cudaMemcpyDeviceToDevice, s));
        NCK(cudaStreamSynchronize(s));
        if (done == DONE_NAN) return set_error(PTD_ENAN, "ptd_solve_2d_noalloc: residual is NaN");
    }
    if ((p->flags & PTD_FLAG_STRICT) && any_capped)
        return set_error(PTD_ENOTCONV, "ptd_solve_2d_noalloc: a step reached itmax without err <= tol");
    return PTD_OK;
}
