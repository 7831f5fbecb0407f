// ptd_internal.h -- declarations shared by the host-side translation units.
#pragma once

#include <cuda_runtime.h>

#include "../../include/ptd.h"
#include "ptd_kernels.h"

namespace ptd {

// Scalar iteration parameters derived from ptd_params (all FP64, host side).
struct Derived {
    double h[3] = {0, 0, 0};  // cell sizes
    double vpdt = 0;          // Vpdtau
    double L = 0;             // max(lx, ly, lz)
    double rdt = 0;           // 1/dt
    double sig[3] = {0, 0, 0};// kappa/dx_d^2
    double c_lin = 0, e_lin = 0;
    double k1 = 0, k2 = 0, k3 = 0;
    double A = 0;             // L^2/dt
    double norm_den = 1;      // RMS divisor
};

// Grid geometry shared by every context kind: padded row pitch sy (a
// multiple of 32 elements in 2D/3D), plane pitch sz, field size nfield.
struct ptd_ctx_base {
    int nx = 0, ny = 0, nz = 0;
    long long sy = 0, sz = 0, nfield = 0;
};

// Largest grid accepted, in cells including the padding of each row to 32
// elements: 2^40 (8.8 TB per FP64 field, far beyond any device), so that no
// byte count or offset derived from a grid's size overflows 64 bits.
constexpr long long kMaxCells = 1LL << 40;

int set_error(int status, const char* msg);
int cuda_fail(cudaError_t e, const char* where);
int validate(const ptd_params* p);
void derive(const ptd_params& p, Derived& dv);
void fill_args(const ptd_params& p, const Derived& dv, PTArgs& a);
FParams fparams(const Derived& dv);
LaunchCfg tuned_config(const ptd_params& p);
int z_chunk(long long bxy, int nz, long long slots);
int copy_field_in(const ptd_ctx_base& g, double* dst, const double* src, cudaStream_t s);
int copy_field_out(const ptd_ctx_base& g, double* dst, const double* src, cudaStream_t s);

// The current H of a one-grid context as an FP64 padded field (device to
// device; converts DF64).  ptd_api.cu.
int ctx_current_f64(ptd_ctx* c, double* dst);
// dst += src over n elements.  ptd_pt.cu.
cudaError_t add_fields(double* dst, const double* src, long long n, cudaStream_t s);

// FP32 + FP64 defect correction (ptd_dc.cu).
struct DcState;
int dc_create(const ptd_ctx_base& g, const ptd_params& p, const Derived& dv, cudaStream_t s, DcState** out);
void dc_destroy(DcState* dc);
int dc_set_state(DcState* dc, const ptd_ctx_base& g, double* H, double* Hold, const double* D, cudaStream_t s);
int dc_step(DcState* dc, const ptd_ctx_base& g, int32_t* iters, double* err_hist, int32_t err_cap,
            int32_t* n_err, int* nan_flag, int* capped);
int dc_iterate(DcState* dc, const ptd_ctx_base& g, int32_t niter);
int dc_set_config(DcState* dc, const LaunchCfg& cfg);
const double* dc_current(const DcState* dc);

struct DcCounters {
    long long launches = 0;
    long long iterations = 0;
};
DcCounters dc_counters(const DcState* dc);

// FP32 PT iterations on the change since an FP64 base, rebased (ptd_rb.cu).
struct RbState;
int rb_create(const ptd_ctx_base& g, const ptd_params& p, const Derived& dv, cudaStream_t s, RbState** out);
void rb_destroy(RbState* rb);
int rb_set_state(RbState* rb, double* H, double* Hold, double* const* wb, const double* D, cudaStream_t s);
int rb_step(RbState* rb, int32_t* iters, double* err_hist, int32_t err_cap, int32_t* n_err, int* nan_flag,
            int* capped);
int rb_iterate(RbState* rb, int32_t niter);
int rb_set_config(RbState* rb, const LaunchCfg& cfg);
DcCounters rb_counters(const RbState* rb);

}  // namespace ptd
