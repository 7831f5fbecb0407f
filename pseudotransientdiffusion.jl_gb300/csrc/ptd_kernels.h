// ptd_kernels.h -- host-side launch interface of the device kernels.
#pragma once

#include <cuda_runtime.h>

#include "ptd_device.cuh"

namespace ptd {

// Device-side control block of one physical step.  The check kernel adds
// into acc; the judge kernel turns acc into err, appends it to the error
// history, advances iter by one check block and raises done when the step
// stops (err <= tol, NaN, or no full check block left before itmax).  Every
// PT kernel returns at entry once done is set, so a CUDA graph holding many
// check blocks can be replayed without a host round trip per check.
struct DevState {
    int done;      // 0 running, 1 converged, 2 NaN residual, 3 iteration cap
    int nchecks;   // residual checks in this step
    int iter;      // PT iterations completed by check blocks in this step
    int pad;
    double acc;    // residual accumulator (sum R^2, or max |R| bits)
    double err;    // last err
};

enum { DONE_RUNNING = 0, DONE_CONVERGED = 1, DONE_NAN = 2, DONE_CAP = 3 };

struct LaunchCfg {
    int chunk2d = 64;   // rows per 2D y-march
    int warps2d = 4;    // 31-cell strips per 2D block
    int chunk3d = 128;  // planes per 3D z-march
    int rows3d = 16;    // warps (y rows) per 3D block (8 or 16)
};

// number types of the PT kernels (ptd_num.cuh)
enum { NUM_F64 = 0, NUM_DF64 = 1, NUM_DFH = 2 };

// Streaming multiprocessors of the current device (queried once per device,
// ptd_tune.cu), and the grid of the grid-stride helper kernels: 8 CTAs of 256
// threads per SM.
int sm_count();
inline int fill_blocks() { return 8 * sm_count(); }

cudaError_t launch_pt(const PTArgs& a, int ndim, int model, bool check, int num, const LaunchCfg& cfg,
                      cudaStream_t s);
cudaError_t launch_resid_consistent(const PTArgs& a, int ndim, int model, int num, cudaStream_t s);
cudaError_t launch_to_df64(const double* src, void* dst, long long n, cudaStream_t s);
cudaError_t launch_expm(const double* m, void* E, long long n, bool df64, cudaStream_t s);
cudaError_t launch_from_df64(const void* src, double* dst, long long n, cudaStream_t s);
cudaError_t launch_judge(DevState* st, double* errhist, int errcap, int nchk, int itmax, double tol,
                         double norm_den, int norm_max, cudaStream_t s);
cudaError_t launch_judge_parts(DevState* st, const double* parts, long long nparts, double* errhist, int errcap,
                               int nchk, int itmax, double tol, double norm_den, int norm_max,
                               cudaGraphConditionalHandle loop, cudaStream_t s);
// num: NUM_* of the kernels (the double-float forms tile differently)
long long pt_check_slots(int ndim, int nx, int ny, int nz, const LaunchCfg& cfg, bool consistent, int num);
cudaError_t launch_reset_state(DevState* st, cudaStream_t s);
cudaError_t preload_pt2d_f64();

}  // namespace ptd
