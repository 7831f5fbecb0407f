/*
 * ptd_oracle.h -- CPU FP64 restatement of the reference's accelerated
 * pseudo-transient (PT) diffusion solvers.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA library
 * (the tests, the smoke check and the CPU-baseline leg of the benchmark call
 * it); the product path never links or calls it.
 *
 * Parity pin: the restatement reproduces the reference's own golden arrays
 * (test/reftest-files/ BSON files, decoded into tests/golden/reftests.json) and the
 * published iteration counts (output/out_diff_*.txt, decoded into
 * tests/golden/iteration_counts.json); the tests in tests/test_oracle.py
 * check both.
 */
#ifndef PTD_ORACLE_H
#define PTD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_params {
    int32_t ndim;       /* 1, 2 or 3 */
    int32_t model;      /* 0 linear (scalar D), 1 step (D field), 2 nonlinear (D = H^3),
                           3 nonlinear with a log-coefficient field m: D = exp(m) H^3,
                           face value ((exp(m_L)+exp(m_R))/2) ((H_L+H_R)/2)^3 */
    int32_t nx, ny, nz; /* cells including the two frozen boundary cells per dimension */
    double lx, ly, lz;  /* domain lengths */
    double dt;          /* physical time step */
    int32_t nt;         /* physical time steps */
    int32_t itmax;      /* PT iteration cap per physical step */
    int32_t nout;       /* residual check cadence (every nout-th iteration) */
    double tol;         /* stop when err <= tol */
    double cfl;         /* CFL number of the pseudo-time step */
    double resc;        /* iteration-parameter scaling (nonlinear 2D/3D: 1/1.2; else 1) */
    double D;           /* model 0: D; model 1: the max(D1,D2) used in Re */
    int32_t recip;      /* 1: reciprocal arithmetic of the *_perf scripts, 0: division form */
    int32_t resid;      /* 0: mixed residual (reference), 1: consistent residual */
    int32_t norm;       /* 0: RMS norm (reference), 1: max |R| */
    int32_t nthreads;   /* OpenMP threads (<= 0: runtime default) */
    double norm_len;    /* RMS divisor (number of residual cells); <= 0: the inner-cell count.
                           The multi-rank 3D scripts divide by len_ResH_g
                           (diff_3D_nonlin_multixpu.jl:89), which differs from the
                           global inner-cell count when dims > 1. */
} ora_params;

/* Solve nt physical steps in place.
 *   H        in: H0 (nx*ny*nz, x fastest); out: H after nt steps.
 *   Dfield   model 1: cell diffusivity; model 3: the log-coefficient m (nx*ny*nz);
 *            else NULL.
 *   iters    out: PT iterations of each physical step (nt entries).
 *   errhist  out (nullable): err of every residual check, in order.
 *   errcap   capacity of errhist;  nerr out (nullable): checks performed.
 * Returns 0, or 2 when a step ended with a NaN residual (the reference raises
 * error("NaN") there), or 1 on invalid arguments. */
int ora_solve(const ora_params* p, double* H, const double* Dfield, int32_t* iters,
              double* errhist, int32_t errcap, int32_t* nerr);

/* As ora_solve with the first step's previous state Hold0 given separately
 * (NULL: H).  The reaction scripts (scripts/diff_{1D,2D}_react.jl) are one
 * step with dt = theta_kin, H = 0 and Hold0 = Heq. */
int ora_solve2(const ora_params* p, double* H, const double* Hold0, const double* Dfield, int32_t* iters,
               double* errhist, int32_t errcap, int32_t* nerr);

/* Run exactly `niter` PT iterations of one physical step (no residual checks),
 * starting from H with damped fluxes q (3 arrays of nx*ny*nz, face between
 * cell c and c+stride stored at c; zero on the first call).  Used as the timed
 * CPU baseline (the reference's fixed-iteration perf protocol). */
int ora_iterate(const ora_params* p, double* H, const double* Hold, const double* Dfield,
                double* qx, double* qy, double* qz, int32_t niter);

/* The residual R of the last iteration's state: given H (post-update), Hold and
 * H_pre (the state the fluxes were evaluated on), returns the norm (p->norm). */
double ora_residual_norm(const ora_params* p, const double* H, const double* Hold,
                         const double* Hpre, const double* Dfield);

/* Discrete adjoint (models 2 and 3) of nt implicit steps whose converged
 * states are Hs[0..nt] (Hs[0] = H0, each nx*ny*nz): gradient of
 * L = 1/2 sum_inner (H^nt - Ht)^2 with respect to m (model 3) and H0 (all
 * cells; the boundary cells stay frozen at H0 through every step).  Each
 * transposed step J^T lam = g is solved by BiCGSTAB to relative residual rtol.
 * Returns 0, 1 on bad arguments, 3 when a linear solve did not reach rtol. */
int ora_adjoint(const ora_params* p, const double* Hs, const double* m, const double* Ht,
                double* grad_m, double* grad_H0, double rtol);

#ifdef __cplusplus
}
#endif
#endif
