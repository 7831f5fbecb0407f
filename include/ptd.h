/*
 * ptd.h -- C ABI of the GB300 (sm_103a) accelerated pseudo-transient (PT)
 * diffusion library, libptd.so.
 *
 * Drop-in boundary.  The reference (PTsolvers/PseudoTransientDiffusion.jl) has
 * no FFI of its own: its boundary is the script-level solver driver
 * diffusion_{1,2,3}D_() (e.g. scripts/diff_2D_nonlin.jl:46-106), configured by
 * NX/NY/NZ (scripts/diff_2D_nonlin.jl:6-7) and hard-coded physics/numerics,
 * returning (xc[,yc,zc], H) (scripts/diff_2D_nonlin.jl:105,108-112) and
 * printing the total PT iteration count (scripts/diff_2D_nonlin.jl:92).  The
 * entry points below are what a host-language wrapper of that driver (a
 * Julia `ccall`, Python `ctypes`) binds: the driver keeps its names and
 * defaults, builds H0 (and D for the step model) exactly as the script does,
 * and hands the PT solve to this library.
 *
 * Conventions
 *  - Arrays are the reference's: Float64, nx*ny*nz cells including the frozen
 *    boundary cells, x fastest (Julia column-major).  Pointers may be host
 *    memory (pageable or pinned) or device memory of the current device; the
 *    library detects which.
 *  - Every function returns a ptd_status (0 = PTD_OK).  The library never
 *    aborts the process; ptd_last_error() gives a one-line detail.
 *  - Ownership: the caller owns H and D; a context owns its device buffers
 *    (allocated by ptd_create, freed by ptd_destroy) and its CUDA stream.
 *  - Threading: a context is used by one host thread at a time.
 */
#ifndef PTD_H
#define PTD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTD_ABI_VERSION 1

#if defined(__GNUC__)
#define PTD_API __attribute__((visibility("default")))
#else
#define PTD_API
#endif

/* Status codes.  PTD_ENAN mirrors the reference's `if isnan(err) error("NaN")`
 * after a physical step (scripts/diff_2D_nonlin.jl:90). */
typedef enum ptd_status {
    PTD_OK = 0,
    PTD_EINVAL = 1,    /* invalid argument or parameter combination */
    PTD_ENAN = 2,      /* the residual norm was NaN at the end of a physical step */
    PTD_ENOTCONV = 3,  /* itmax reached without err <= tol (only with PTD_FLAG_STRICT) */
    PTD_ECUDA = 4,     /* a CUDA runtime call failed */
    PTD_ENOMEM = 5,    /* device or host allocation failed */
    PTD_ESTATE = 6,    /* call out of order (e.g. stepping before a state was set) */
    PTD_ETIMEOUT = 7   /* a device-side wait gave up (never expected) */
} ptd_status;

/* Diffusion models of the reference's solver scripts:
 *  LIN      D = const                     scripts/diff_{1D,2D}_lin.jl, diff_3D_lin_multixpu.jl
 *  LINSTEP  D = per-cell field (step)     scripts/diff_{1D,2D}_linstep.jl, diff_3D_linstep_multixpu.jl
 *  NONLIN   D = H^3 (face: (avg H)^3)     scripts/diff_{1D,2D}_nonlin.jl, diff_3D_nonlin_multixpu.jl */
enum { PTD_MODEL_LIN = 0, PTD_MODEL_LINSTEP = 1, PTD_MODEL_NONLIN = 2, PTD_MODEL_NONLIN_EXPM = 3 };
/* PTD_MODEL_NONLIN_EXPM (no reference counterpart; the model of the adjoint
 * solver): D = exp(m) H^3 with a per-cell log-coefficient field m passed in
 * place of D; face value ((exp(m_L)+exp(m_R))/2) ((H_L+H_R)/2)^3.  FP64,
 * DF64, DFH and FP32_RB. */

/* Arithmetic of the PT iterations.
 *  FP64     every PT iteration in native FP64 (the reference's form).
 *  FP32_DC  FP32 PT iterations on a correction inside an FP64
 *           defect-correction loop (residual, norm and H update in FP64).
 *  DF64     the FP64 form with every value held as a double-float (two
 *           FP32 numbers, ~48-bit significand, 8 bytes like a double) and
 *           computed on the FP32 pipe; same iterations and iteration counts
 *           as FP64, H within ~1e-13 relative of it.  The 48-bit H limits
 *           the attainable residual on fine 1D/2D grids (1D nx >= 2048,
 *           2D >= 1024^2 at tol 1e-8).
 *  DFH      DF64 arithmetic on an FP64 state: H and Hold are doubles (the
 *           differences of H values and the H update in FP64: 5 FP64
 *           operations per cell in 2D, 6 in 3D), fluxes and D double-floats.
 *           Same iteration counts as FP64 and H within ~1e-14 of it on the
 *           2D/3D grids of the reference and of the benchmarks (up to 8192^2
 *           and 512^3).  The 48-bit flux arithmetic sets a residual floor
 *           ~32x FP64's, which stalls 1D lin/linstep grids of nx >= 8192.
 *           Single grids only (not the batch or the adjoint).
 *  FP32_RB  FP32 PT iterations on the change since an FP64 base state
 *           (H_b, fluxes w_b), rebased in FP64 every ~200 iterations: the
 *           FP32 iteration carries only changes and defects that shrink as
 *           the step converges, and keeps the PT iteration's momentum across
 *           rebases (no restarted inner solves).  A step stops when the
 *           reference's check residual (every nchk, formed in FP32 from the
 *           FP64 base residual) and the FP64 residual of the rebased state
 *           are both <= tol; H is the FP64 base.  Every model, mixed
 *           residual; single grids and the batch (ptd_batch_*). */
enum { PTD_PREC_FP64 = 0, PTD_PREC_FP32_DC = 1, PTD_PREC_DF64 = 2, PTD_PREC_DFH = 3, PTD_PREC_FP32_RB = 4 };

/* Residual used for the stopping test.  MIXED is the reference's: the
 * undamped flux from the H the fluxes of that iteration were computed on, the
 * time term from the updated H (scripts/diff_2D_nonlin.jl:31-32,41-44). */
enum { PTD_RESID_MIXED = 0, PTD_RESID_CONSISTENT = 1 };

/* Norm of the residual: RMS = norm(ResH)/sqrt(length(ResH)) (the reference,
 * scripts/diff_2D_nonlin.jl:85), or MAX = max|R|. */
enum { PTD_NORM_RMS = 0, PTD_NORM_MAX = 1 };

/* Flags */
#define PTD_FLAG_STRICT 0x1   /* return PTD_ENOTCONV when a step stops at itmax */
#define PTD_FLAG_AUTOTUNE 0x2 /* ptd_create times every launch shape of the fused kernel (2D: warps per CTA
                                 x rows per y march; 3D: z-march length x warps per CTA) and keeps the fastest */
#define PTD_FLAG_DC_NO_TBLOCK 0x4 /* FP32_DC and FP32_RB in 2D: one FP32 iteration per launch (default: two
                                     per launch, temporally blocked, when the check cadence is even) */
#define PTD_FLAG_RB_TBLOCK_3D 0x8 /* FP32_RB in 3D (LIN, NONLIN): two FP32 iterations per launch (z temporal
                                     blocking, even check cadence; same iterates).  Off by default: at 512^3 it
                                     moves half the bytes of the one-iteration kernel but is issue-bound at
                                     about the same time per iteration */

typedef struct ptd_params {
    int32_t ndim;        /* 1, 2, 3 */
    int32_t model;       /* PTD_MODEL_* */
    int32_t nx, ny, nz;  /* cells including boundary cells; unused dims = 1 */
    double lx, ly, lz;   /* domain lengths */
    double dt;           /* physical time step */
    int32_t nt;          /* physical time steps solved by ptd_solve */
    int32_t itmax;       /* PT iteration cap per physical step (itMax) */
    int32_t nchk;        /* residual check cadence (nout) */
    int32_t precision;   /* PTD_PREC_* */
    double tol;          /* stop when err <= tol */
    double cfl;          /* CFL: Vpdtau = cfl * min(dx,dy,dz) */
    double resc;         /* iteration-parameter scaling (Resc); 1 for the linear models */
    double D;            /* LIN: the diffusivity; LINSTEP: the D in Re (max(D1,D2)) */
    int32_t resid_mode;  /* PTD_RESID_* */
    int32_t norm;        /* PTD_NORM_* */
    double norm_len;     /* RMS divisor; <= 0 means the number of inner cells */
    int32_t flags;       /* PTD_FLAG_* */
    int32_t dc_max_outer;/* FP32_DC: outer FP64 corrections per step cap (0: default 30) */
    double dc_inner_rtol;/* FP32_DC: smallest inner relative tolerance (0: default 1e-3) */
    int32_t reserved[8]; /* zero */
} ptd_params;

typedef struct ptd_ctx ptd_ctx;

/* Fill p with the defaults of the reference script for (ndim, model):
 * lx=ly=lz=10, dt=0.2, nt=5 (ttot=1), tol=1e-8, itmax=1e5, nchk=10, D=1,
 * cfl = 0.99 (1D lin/linstep), 1.0 (1D nonlin), 1/sqrt(2) (2D), 1/sqrt(3) (3D),
 * resc = 1/1.2 for 2D/3D nonlinear, else 1; n = 512 (1D/2D) or 64 (3D).
 * Replaces: the parameter blocks of scripts/diff_1D_lin.jl:35-50,
 * diff_2D_nonlin.jl:48-62, diff_3D/diff_3D_nonlin_multixpu.jl:59-74 (and siblings). */
PTD_API int ptd_params_init(ptd_params* p, int32_t ndim, int32_t model);

/* Validate p and allocate the device buffers of one grid (PTD_EINVAL for a
 * grid above 2^40 cells, rows padded to 32 elements).
 * Replaces: the @zeros/@ones allocations of the driver (e.g.
 * scripts/diff_2D_nonlin.jl:65-73). */
PTD_API int ptd_create(ptd_ctx** ctx, const ptd_params* p);

/* Solve p->nt physical steps: H in = H0, H out = H after nt steps.
 * D: LINSTEP cell diffusivity (nx*ny*nz), else NULL.
 * iters_per_step (nullable): PT iterations of each step (nt entries).
 * err_hist (nullable): err of every residual check, in order, up to err_cap;
 * n_err (nullable): number of checks performed.
 * Replaces: the physical-time + PT loop of diffusion_2D_()
 * (scripts/diff_2D_nonlin.jl:76-91; same in every driver). */
PTD_API int ptd_solve(ptd_ctx* ctx, double* H, const double* D, int32_t* iters_per_step,
              double* err_hist, int32_t err_cap, int32_t* n_err);

/* Resident-state interface (the same loop split in pieces; used for timing
 * and by callers that keep H on the device between calls). */
PTD_API int ptd_set_state(ptd_ctx* ctx, const double* H, const double* D); /* H and Hold <- H, fluxes <- 0 */
/* H <- H, Hold <- Hold (NULL: H), fluxes <- 0.  With H = 0 and Hold = Heq, one
 * step of dt = theta_kin is the reference's steady reaction-diffusion solve
 * (scripts/diff_2D_react.jl:15-72: Heq/theta_kin in place of Hold/dt, Da in
 * place of Re, one PT loop). */
PTD_API int ptd_set_state2(ptd_ctx* ctx, const double* H, const double* Hold, const double* D);
PTD_API int ptd_step(ptd_ctx* ctx, int32_t nsteps, int32_t* iters_per_step, double* err_hist,
             int32_t err_cap, int32_t* n_err);                       /* nsteps physical steps */
PTD_API int ptd_iterate(ptd_ctx* ctx, int32_t niter);  /* niter PT iterations, no checks (perf protocol,
                                                  scripts/diff_3D/diff_3D_nonlin_perf.jl:97-105) */
PTD_API int ptd_get_state(ptd_ctx* ctx, double* H);    /* H out */

/* Launch shape in use: {warps per 2D CTA, rows per 2D y march, warps per 3D CTA, planes per 3D z march}. */
PTD_API int ptd_launch_config(ptd_ctx* ctx, int32_t cfg[4]);
/* Set it (e.g. a shape found by PTD_FLAG_AUTOTUNE on another context of the
 * same size): warps per 2D CTA in {1,2,4,8}, rows per 2D march in [1,4096],
 * warps per 3D CTA in {8,16} (the FP32 forms use 16), planes per 3D march in
 * [1,4096].  The state is kept. */
PTD_API int ptd_set_launch_config(ptd_ctx* ctx, const int32_t cfg[4]);

/* The context's CUDA stream (cudaStream_t) and a device synchronize of it. */
PTD_API void* ptd_stream(ptd_ctx* ctx);
PTD_API int ptd_sync(ptd_ctx* ctx);

/* Counters since ptd_create: kernels launched by the library (each kernel of
 * a replayed CUDA graph counts) and PT iterations executed. */
PTD_API int ptd_counters(ptd_ctx* ctx, int64_t* kernel_launches, int64_t* pt_iterations);

PTD_API void ptd_destroy(ptd_ctx* ctx);

/* ---------------------------------------------------------------------------
 * Batched 2D solves: many independent grids of uneven sizes, each with its own
 * H0 (and D for the step model), advanced together by one kernel launch per
 * PT iteration with per-instance convergence flags.  No reference
 * counterpart (the reference solves one grid per run); the per-instance
 * algorithm is that of ptd_solve (FP64, DF64) or its FP32_DC or FP32_RB form.
 * FP32_RB: one physical step of the whole batch is one CUDA graph launch
 * (phases of every instance until all have stopped); an instance that
 * reaches itmax stops at its last full check block.
 * Constraint: itmax is a multiple of nchk. */
typedef struct ptd_batch_params {
    int32_t ninst;       /* number of instances */
    int32_t model;       /* PTD_MODEL_* */
    double lx, ly;       /* domain lengths (shared) */
    double dt;
    int32_t nt, itmax, nchk, precision;
    double tol, cfl, resc, D;
    int32_t norm, flags;
    int32_t dc_max_outer, pad0;
    double dc_inner_rtol;
    int32_t reserved[8];
} ptd_batch_params;

typedef struct ptd_batch ptd_batch;

/* Defaults of the 2D script for `model` (lx = ly = 10, dt = 0.2, nt = 5, ...). */
PTD_API int ptd_batch_params_init(ptd_batch_params* p, int32_t ninst, int32_t model);
/* nx[i], ny[i]: cells of instance i (including boundary cells). */
PTD_API int ptd_batch_create(ptd_batch** b, const ptd_batch_params* p, const int32_t* nx, const int32_t* ny);
/* H[i] in: H0 of instance i, out: H after nt steps (nx[i]*ny[i], x fastest; host
 * or device).  D[i]: step-model diffusivity or NULL.  iters: ninst*nt PT
 * iterations (FP32_DC: inner FP32 iterations), instance-major.  err_last
 * (nullable, ninst): last residual norm of each instance (FP32_RB: the FP64
 * residual of its returned H).  n_done: ninst. */
PTD_API int ptd_batch_solve(ptd_batch* b, double* const* H, const double* const* D, int32_t* iters,
                            double* err_last, int32_t* n_done);
/* Autotuner: times every (warps per CTA, rows per y chunk) launch shape of the
 * batched kernel on the batch's own instances -- for FP32_DC and FP32_RB also
 * one or two (temporally blocked) FP32 iterations per launch -- and keeps the
 * fastest per iteration. */
PTD_API int ptd_batch_tune(ptd_batch* b, int32_t* warps, int32_t* chunk, float* us_per_iteration);
/* The launch shape in use: warps per CTA, rows per y chunk, FP32 iterations
 * per launch (2 = the temporally blocked FP32_DC or FP32_RB kernel). */
PTD_API int ptd_batch_config(ptd_batch* b, int32_t* warps, int32_t* chunk, int32_t* iters_per_launch);
/* Set the launch shape: warps per CTA (1, 2, 4, 8), rows per y chunk (8..4096)
 * and FP32 iterations per launch (1, or 2 for FP32_DC / FP32_RB with an even
 * check cadence). */
PTD_API int ptd_batch_set_config(ptd_batch* b, int32_t warps, int32_t chunk, int32_t iters_per_launch);
PTD_API int ptd_batch_counters(ptd_batch* b, int64_t* kernel_launches, int64_t* pt_iterations);
PTD_API void ptd_batch_destroy(ptd_batch* b);

/* ---------------------------------------------------------------------------
 * Discrete adjoint (3D, D = H^3 or D = exp(m) H^3).  No reference counterpart
 * (the reference has no adjoint).  ptd_adj_forward solves p->nt implicit steps
 * from H0 (m: the log-coefficient field, model PTD_MODEL_NONLIN_EXPM), keeps
 * one FP64 checkpoint of H per physical step and returns
 * L = 1/2 sum_inner (H^nt - Ht)^2 (and H^nt when HN != NULL);
 * ptd_adj_gradient then returns dL/dm and dL/dH0 (every cell, each nullable)
 * by solving the transposed linearised PT system of every step backwards. */
typedef struct ptd_adj ptd_adj;
PTD_API int ptd_adj_create(ptd_adj** a, const ptd_params* p);
PTD_API int ptd_adj_forward(ptd_adj* a, const double* H0, const double* m, const double* Ht, double* loss,
                            double* HN, int32_t* iters_per_step);
PTD_API int ptd_adj_gradient(ptd_adj* a, double* grad_m, double* grad_H0, int32_t* adj_iters_per_step);
/* Last ptd_adj_gradient: the final RMS residual of each step's adjoint solve
 * and its stopping target (1e-10 x the RMS of its right-hand side); nt
 * entries each, nullable.  A solve also stops when its residual has stalled
 * (no 1 % gain over ~2 max(nx,ny,nz) iterations) at an arithmetic floor below
 * 1e-7 x the RMS of its right-hand side.  With PTD_FLAG_STRICT,
 * ptd_adj_gradient returns PTD_ENOTCONV when a solve stopped at itmax. */
PTD_API int ptd_adj_residuals(ptd_adj* a, double* err, double* target);
PTD_API int ptd_adj_counters(ptd_adj* a, int64_t* kernel_launches, int64_t* pt_iterations);
PTD_API void ptd_adj_destroy(ptd_adj* a);

/* ---------------------------------------------------------------------------
 * ptd_solve_2d_noalloc: the 2D FP64 solve of ptd_solve for callers that cannot
 * allocate GPU memory when they need a solve (a host framework whose memory
 * pool already owns the device, code running while such an allocator holds
 * its lock, drivers that must not grow their footprint after start-up).  It
 * has no counterpart in the reference.  It runs the fused FP64 PT kernel on
 * the caller's device buffers and takes all scratch from one fixed device
 * array compiled into the library (24 MiB, held from the first call on a GPU
 * until the process exits); it calls no cudaMalloc/cudaFree, creates
 * no stream or graph and launches on `stream` (a cudaStream_t, NULL = legacy
 * default stream).
 *   p      2D, PTD_PREC_FP64, models LIN/LINSTEP/NONLIN, mixed residual;
 *          nx*ny <= PTD_NOALLOC_MAX_CELLS, else PTD_EINVAL.
 *   H      device memory of the current device (cudaMalloc'ed or from a
 *          pool; not managed, host or another GPU's memory, PTD_EINVAL), nx*ny
 *          doubles, x fastest: in H0, out H after p->nt steps.
 *   D      device memory of the current device (LINSTEP) or NULL.
 *   iters_per_step  host, p->nt entries (nullable).
 * The array is reserved on a device by the first call there (the CUDA
 * runtime loads the library's device code lazily; that call also looks up the
 * array's device address with cudaGetSymbolAddress).  A caller that cannot
 * allocate later therefore makes one call at start-up, before its own
 * allocator takes the device and before any stream capture: with p->nt = 0
 * the call only reserves the array, loads the kernels a solve launches and
 * returns (H may then be NULL).  Later calls change no device memory
 * reservation.
 * Every call uses the same array: calls that overlap on the GPU (from two
 * streams or two threads) race and must be serialised by the caller. */
#define PTD_NOALLOC_MAX_CELLS 524288
PTD_API int ptd_solve_2d_noalloc(const ptd_params* p, double* H, const double* D, void* stream,
                                 int32_t* iters_per_step);

/* Diagnostic, no reference counterpart: the FP64 FMA throughput of the
 * current GPU in operations per second (8 independent FMA chains per thread,
 * 8 CTAs of 256 threads per SM, CUDA-event timed; ~20 ms).  It is the roofline
 * of the native-FP64 PT kernels, which need 19 (2D) / 27 (3D) FP64
 * instructions per cell and so are bound by this rate rather than by HBM. */
PTD_API int ptd_measure_fp64_rate(double* ops_per_s);

PTD_API const char* ptd_strerror(int status);
PTD_API const char* ptd_last_error(void);   /* detail of the last failure on this thread */
PTD_API int ptd_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PTD_H */
