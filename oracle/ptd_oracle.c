/*
 * ptd_oracle.c -- CPU FP64 restatement of the reference's accelerated
 * pseudo-transient diffusion solvers (TEST INFRASTRUCTURE: the checker for
 * the CUDA library, never part of the product path).
 *
 * Followed line by line (file:line within the reference project):
 *   linear     scripts/diff_1D_lin.jl:17-31 (kernels), :46-50 (parameters),
 *              scripts/diff_2D_lin.jl:18-34, :150-154,
 *              scripts/diff_3D/diff_3D_lin_multixpu.jl:24-42, :205-209
 *   step       scripts/diff_1D_linstep.jl:17-30, :159-171,
 *              scripts/diff_2D_linstep.jl:18-39, :67-87,
 *              scripts/diff_3D/diff_3D_linstep_multixpu.jl:24-47, :82-108
 *   nonlinear  scripts/diff_1D_nonlin.jl:17-38, :52-53,
 *              scripts/diff_2D_nonlin.jl:18-44, :185-188,
 *              scripts/diff_3D/diff_3D_nonlin_multixpu.jl:24-55, :71-74
 *   reciprocal scripts/diff_2D_nonlin_perf.jl:19-49, :74 and
 *   ("perf")   scripts/diff_3D/diff_3D_nonlin_perf.jl:19-55, :78
 *   driver     scripts/diff_2D_nonlin.jl:76-91 (physical-time + PT loop,
 *              check every nout-th iteration, RMS norm, NaN check)
 *
 * Finite-difference macros of ParallelStencil.jl (third-party, not vendored,
 * unpinned: the reference's Project.toml has no [compat] and no Manifest) are
 * restated from their expanded forms in the perf scripts
 * (scripts/diff_2D_nonlin_perf.jl:19-21,30-31,36): @d_xi(A) = A[i+1,j+1]-A[i,j+1],
 * @av_xi(A) = (A[i,j+1]+A[i+1,j+1])*0.5, @d_xa(A) = A[i+1,j]-A[i,j],
 * @inn(A) = A[i+1,j+1]; @maxloc(A) is the star stencil (the cell and its face
 * neighbours), pinned by the step-model golden arrays.
 *
 * Storage: every array is nx*ny*nz with x fastest (Julia column-major).  The
 * flux across the face between cell c and c+stride[d] is stored at index c.
 * The expressions keep the reference's evaluation order so that rounding
 * matches its output to ~1e-15.
 */
#include "ptd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    const ora_params* p;
    int ndim;
    long n[3];
    long s[3];
    double h[3];    /* dx, dy, dz */
    double rh[3];   /* 1/dx, ...  (perf scripts: _dx = 1.0/dx) */
    double vpdt;    /* Vpdtau = CFL * min(dx, dy, dz) */
    double L, L2;   /* max(lx, ly, lz) and its square */
    double pi, pipi;
    double rdt;     /* _dt = 1.0/dt */
    double theta;   /* linear models: L / Vpdtau / Re */
    double dtau;    /* linear model:  Vpdtau * L / D / Re */
    double re;      /* linear models: Re */
    int nth;
} octx;

static int setup(octx* c, const ora_params* p)
{
    memset(c, 0, sizeof(*c));
    c->p = p;
    if (!p || p->ndim < 1 || p->ndim > 3 || p->model < 0 || p->model > 3) return 1;
    c->ndim = p->ndim;
    c->n[0] = p->nx;
    c->n[1] = p->ndim > 1 ? p->ny : 1;
    c->n[2] = p->ndim > 2 ? p->nz : 1;
    for (int d = 0; d < p->ndim; ++d)
        if (c->n[d] < 3) return 1;
    c->s[0] = 1;
    c->s[1] = c->n[0];
    c->s[2] = c->n[0] * c->n[1];
    double l[3] = {p->lx, p->ly, p->lz};
    double hmin = 0.0, L = 0.0;
    for (int d = 0; d < p->ndim; ++d) {
        c->h[d] = l[d] / (double)c->n[d];
        c->rh[d] = 1.0 / c->h[d];
        hmin = (d == 0) ? c->h[d] : fmin(hmin, c->h[d]);
        L = (d == 0) ? l[d] : fmax(L, l[d]);
    }
    c->vpdt = p->cfl * hmin;
    c->L = L;
    c->L2 = L * L;
    c->pi = 3.141592653589793;
    c->pipi = c->pi * c->pi;
    c->rdt = 1.0 / p->dt;
    if (p->model < 2) {
        /* Re = pi + sqrt(pi^2 + (L^2 / D / dt)) -- diff_2D_lin.jl:51, diff_2D_linstep.jl:70 */
        c->re = c->pi + sqrt(c->pipi + ((c->L2 / p->D) / p->dt));
        c->theta = (c->L / c->vpdt) / c->re;
        c->dtau = ((c->vpdt * c->L) / p->D) / c->re;
    }
    c->nth = p->nthreads;
#ifdef _OPENMP
    if (c->nth <= 0) c->nth = omp_get_max_threads();
#else
    c->nth = 1;
#endif
    return 0;
}

/* Index range of dimension e for the faces normal to d (or the inner cells when d < 0). */
static void face_range(const octx* c, int d, int e, long* lo, long* hi)
{
    if (e >= c->ndim) { *lo = 0; *hi = 1; return; }
    if (e == d) { *lo = 0; *hi = c->n[e] - 1; return; }
    *lo = 1; *hi = c->n[e] - 1;
}

/* Face diffusivity and damping ratio theta for the face (c, c+s).
 * nonlinear: diff_2D_nonlin.jl:19-25, perf form diff_2D_nonlin_perf.jl:20-26 */
static inline void face_coef(const octx* c, const double* H, const double* Df, long i, long ir,
                             double* Dface, double* th)
{
    const ora_params* p = c->p;
    if (p->model == 0) { *Dface = p->D; *th = c->theta; return; }
    if (p->model == 1) { *Dface = (Df[i] + Df[ir]) * 0.5; *th = c->theta; return; }
    double a = (H[i] + H[ir]) * 0.5;
    double d3 = a * a * a;
    if (p->model == 3) d3 = ((Df[i] + Df[ir]) * 0.5) * d3;   /* Df holds exp(m) */
    double re = p->recip ? c->pi + sqrt(c->pipi + (c->L2 / d3) * c->rdt)
                         : c->pi + sqrt(c->pipi + (c->L2 / d3) / p->dt);
    *Dface = d3;
    *th = ((c->L / c->vpdt) / re) * p->resc;
}

/* compute_flux!: damped flux q (and, when q2 != NULL, the undamped flux q2)
 * of every direction in one parallel pass, as the reference evaluates all of
 * its flux arrays in one kernel over the union of their index ranges, each
 * guarded by its own size (diff_2D_nonlin.jl:28-34, diff_2D_lin.jl:18-24,
 * diff_2D_linstep.jl:23-29, perf form diff_2D_nonlin_perf.jl:29-33).  Every
 * face is independent of the others, so the pass order does not change a
 * result bit. */
static void flux_all(const octx* c, double* const q[3], double* const q2[3], const double* H, const double* Df)
{
    const long n0 = c->n[0], n1 = c->n[1], n2 = c->n[2];
    const int ndim = c->ndim, recip = c->p->recip;
    /* k and j span the union of the face ranges: 0..n-2 along a face's own
     * dimension, 1..n-2 along the others */
    const long k1 = ndim > 2 ? n2 - 1 : 1;
    const long j1 = ndim > 1 ? n1 - 1 : 1;
#pragma omp parallel for collapse(2) schedule(static) num_threads(c->nth)
    for (long k = 0; k < k1; ++k)
        for (long j = 0; j < j1; ++j) {
            const int kin = ndim < 3 || k >= 1;   /* k inside 1..n2-2 */
            const int jin = ndim < 2 || j >= 1;
            for (int d = 0; d < ndim; ++d) {
                /* face range of direction d: its own index 0..n-2, the others 1..n-2 */
                if (d != 2 && !kin) continue;
                if (d != 1 && !jin) continue;
                const long i0 = d == 0 ? 0 : 1, i1 = n0 - 1;
                const long sd = c->s[d];
                const double hd = c->h[d], rhd = c->rh[d];
                double* qd = q[d];
                double* q2d = q2 ? q2[d] : NULL;
                for (long i = i0; i < i1; ++i) {
                    long ic = i + n0 * j + n0 * n1 * k;
                    long ir = ic + sd;
                    double Dface, th;
                    face_coef(c, H, Df, ic, ir, &Dface, &th);
                    double dH = H[ir] - H[ic];
                    if (recip) {
                        qd[ic] = (qd[ic] * th - Dface * rhd * dH) / (1.0 + th);
                        if (q2d) q2d[ic] = -Dface * rhd * dH;
                    } else {
                        qd[ic] = (qd[ic] * th - Dface * dH / hd) / (1.0 + th);
                        if (q2d) q2d[ic] = -Dface * dH / hd;
                    }
                }
            }
        }
}

/* Undamped flux only (consistent residual; compute_flux_res!, diff_2D_nonlin_perf.jl:40-44). */
static void flux2_dim(const octx* c, int d, double* q2, const double* H, const double* Df)
{
    long lo[3], hi[3];
    for (int e = 0; e < 3; ++e) face_range(c, d, e, &lo[e], &hi[e]);
    const long sd = c->s[d];
#pragma omp parallel for collapse(2) schedule(static) num_threads(c->nth)
    for (long k = lo[2]; k < hi[2]; ++k)
        for (long j = lo[1]; j < hi[1]; ++j)
            for (long i = lo[0]; i < hi[0]; ++i) {
                long ic = i + c->s[1] * j + c->s[2] * k;
                long ir = ic + sd;
                double Dface, th;
                face_coef(c, H, Df, ic, ir, &Dface, &th);
                double dH = H[ir] - H[ic];
                q2[ic] = c->p->recip ? -Dface * c->rh[d] * dH : -Dface * dH / c->h[d];
            }
}

static void inner_range(const octx* c, long lo[3], long hi[3])
{
    for (int e = 0; e < 3; ++e) face_range(c, -1, e, &lo[e], &hi[e]);
}

static int is_inner(const octx* c, long idx)
{
    long ii[3] = {idx % c->n[0], (idx / c->n[0]) % c->n[1], idx / (c->n[0] * c->n[1])};
    for (int d = 0; d < c->ndim; ++d)
        if (ii[d] < 1 || ii[d] > c->n[d] - 2) return 0;
    return 1;
}

/* Divergence of the three face arrays at inner cell i, in the reference's
 * order ((qx/dx + qy/dy) + qz/dz) -- diff_2D_nonlin.jl:37,42. */
static inline double divergence(const octx* c, double* const q[3], long i)
{
    double acc = 0.0;
    for (int d = 0; d < c->ndim; ++d) {
        double dq = q[d][i] - q[d][i - c->s[d]];
        double t = c->p->recip ? c->rh[d] * dq : dq / c->h[d];
        acc = (d == 0) ? t : acc + t;
    }
    return acc;
}

/* Pseudo-time step per cell: linear diff_2D_lin.jl:53, step (compute_iter_params!)
 * diff_2D_linstep.jl:18-21, nonlinear diff_2D_nonlin.jl:23,26 (perf :24,27). */
static inline double cell_dtau(const octx* c, const double* H, const double* dtau_arr, long i)
{
    const ora_params* p = c->p;
    if (p->model == 0) return c->dtau;
    if (p->model == 1) return dtau_arr[i];
    double h3 = H[i] * H[i] * H[i];
    if (p->model == 3) h3 = dtau_arr[i] * h3;   /* dtau_arr holds exp(m) for model 3 */
    double re = p->recip ? c->pi + sqrt(c->pipi + (c->L2 / h3) * c->rdt)
                         : c->pi + sqrt(c->pipi + (c->L2 / h3) / p->dt);
    return (((c->vpdt * c->L) / h3) / re) * p->resc;
}

/* compute_update!: diff_2D_nonlin.jl:36-39 (division form),
 * diff_2D_nonlin_perf.jl:35-38 (reciprocal form). */
static void update(const octx* c, double* H, const double* Hold, double* const q[3], const double* dtau_arr)
{
    long lo[3], hi[3];
    inner_range(c, lo, hi);
    const double dt = c->p->dt, rdt = c->rdt;
    const int recip = c->p->recip;
#pragma omp parallel for collapse(2) schedule(static) num_threads(c->nth)
    for (long k = lo[2]; k < hi[2]; ++k)
        for (long j = lo[1]; j < hi[1]; ++j)
            for (long i = lo[0]; i < hi[0]; ++i) {
                long ic = i + c->s[1] * j + c->s[2] * k;
                double div = divergence(c, q, ic);
                double dtau = cell_dtau(c, H, dtau_arr, ic);
                if (recip)
                    H[ic] = (H[ic] + dtau * (rdt * Hold[ic] - div)) / (1.0 + rdt * dtau);
                else
                    H[ic] = (H[ic] + dtau * (Hold[ic] / dt - div)) / (1.0 + dtau / dt);
            }
}

/* check_res! + norm: diff_2D_nonlin.jl:41-44,83-86; 3D norm_g
 * diff_3D_nonlin_multixpu.jl:20,113 (one rank: identical to norm/sqrt(length)). */
static double residual_norm(const octx* c, const double* H, const double* Hold, double* const q2[3])
{
    long lo[3], hi[3];
    inner_range(c, lo, hi);
    const double dt = c->p->dt, rdt = c->rdt;
    const int recip = c->p->recip, use_max = c->p->norm == 1;
    double sum = 0.0, mx = 0.0;
    int nan = 0;
    long len = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
#pragma omp parallel for collapse(2) schedule(static) num_threads(c->nth) reduction(+ : sum) reduction(max : mx) reduction(| : nan)
    for (long k = lo[2]; k < hi[2]; ++k)
        for (long j = lo[1]; j < hi[1]; ++j)
            for (long i = lo[0]; i < hi[0]; ++i) {
                long ic = i + c->s[1] * j + c->s[2] * k;
                double div2 = divergence(c, q2, ic);
                double r = recip ? -rdt * (H[ic] - Hold[ic]) - div2 : -(H[ic] - Hold[ic]) / dt - div2;
                sum += r * r;
                double a = fabs(r);
                if (a != a) nan = 1;
                else if (a > mx) mx = a;
            }
    if (use_max) return nan ? NAN : mx;
    double n = c->p->norm_len > 0.0 ? c->p->norm_len : (double)len;
    return sqrt(sum) / sqrt(n);
}

static void step_dtau(const octx* c, const double* Df, double* dtau_arr)
{
    /* compute_iter_params!: dtau_rho = Vpdtau * L / @maxloc(D) / Re (star stencil) */
    long lo[3], hi[3];
    inner_range(c, lo, hi);
    for (long k = lo[2]; k < hi[2]; ++k)
        for (long j = lo[1]; j < hi[1]; ++j)
            for (long i = lo[0]; i < hi[0]; ++i) {
                long ic = i + c->s[1] * j + c->s[2] * k;
                double m = Df[ic];
                for (int d = 0; d < c->ndim; ++d) {
                    m = fmax(m, Df[ic - c->s[d]]);
                    m = fmax(m, Df[ic + c->s[d]]);
                }
                dtau_arr[ic] = ((c->vpdt * c->L) / m) / c->re;
            }
}

int ora_solve(const ora_params* p, double* H, const double* Dfield, int32_t* iters,
              double* errhist, int32_t errcap, int32_t* nerr)
{
    return ora_solve2(p, H, NULL, Dfield, iters, errhist, errcap, nerr);
}

int ora_solve2(const ora_params* p, double* H, const double* Hold0, const double* Dfield, int32_t* iters,
               double* errhist, int32_t errcap, int32_t* nerr)
{
    octx c;
    if (setup(&c, p) || !H || !iters || p->nt < 0 || p->nout < 1) return 1;
    if ((p->model == 1 || p->model == 3) && !Dfield) return 1;
    long N = c.n[0] * c.n[1] * c.n[2];
    double* Hold = (double*)malloc(sizeof(double) * N);
    double* buf = (double*)calloc((size_t)6 * N, sizeof(double));
    double* dtau_arr = (p->model == 1 || p->model == 3) ? (double*)calloc(N, sizeof(double)) : NULL;
    double* expm = NULL;
    if (!Hold || !buf || ((p->model == 1 || p->model == 3) && !dtau_arr)) {
        free(Hold); free(buf); free(dtau_arr);
        return 1;
    }
    double* q[3] = {buf, buf + N, buf + 2 * N};
    double* q2[3] = {buf + 3 * N, buf + 4 * N, buf + 5 * N};
    memcpy(Hold, Hold0 ? Hold0 : H, sizeof(double) * N);
    if (p->model == 1) step_dtau(&c, Dfield, dtau_arr);
    if (p->model == 3) {
        for (long i = 0; i < N; ++i) dtau_arr[i] = exp(Dfield[i]);
        expm = dtau_arr;
    }
    const double* Dcoef = p->model == 3 ? expm : Dfield;
    int32_t ne = 0, status = 0;
    for (int it = 0; it < p->nt; ++it) {
        int32_t iter = 0;
        double err = 2.0 * p->tol;
        while (err > p->tol && iter < p->itmax) {
            int check = ((iter + 1) % p->nout) == 0;
            flux_all(&c, q, (check && p->resid == 0) ? q2 : NULL, H, Dcoef);
            update(&c, H, Hold, q, dtau_arr);
            iter += 1;
            if (check) {
                if (p->resid == 1)
                    for (int d = 0; d < c.ndim; ++d) flux2_dim(&c, d, q2[d], H, Dcoef);
                err = residual_norm(&c, H, Hold, q2);
                if (errhist && ne < errcap) errhist[ne] = err;
                ne += 1;
            }
        }
        iters[it] = iter;
        memcpy(Hold, H, sizeof(double) * N);
        if (err != err) { status = 2; break; }
    }
    if (nerr) *nerr = ne;
    free(Hold);
    free(buf);
    free(dtau_arr);
    return status;
}

int ora_iterate(const ora_params* p, double* H, const double* Hold, const double* Dfield,
                double* qx, double* qy, double* qz, int32_t niter)
{
    octx c;
    if (setup(&c, p) || !H || !Hold || !qx) return 1;
    if ((p->model == 1 || p->model == 3) && !Dfield) return 1;
    double* q[3] = {qx, qy ? qy : qx, qz ? qz : qx};
    double* dtau_arr = NULL;
    if (p->model == 1 || p->model == 3) {
        long N = c.n[0] * c.n[1] * c.n[2];
        dtau_arr = (double*)calloc(N, sizeof(double));
        if (!dtau_arr) return 1;
        if (p->model == 1) step_dtau(&c, Dfield, dtau_arr);
        else
            for (long i = 0; i < N; ++i) dtau_arr[i] = exp(Dfield[i]);
    }
    const double* Dcoef = p->model == 3 ? dtau_arr : Dfield;
    for (int32_t it = 0; it < niter; ++it) {
        flux_all(&c, q, NULL, H, Dcoef);
        update(&c, H, Hold, q, dtau_arr);
    }
    free(dtau_arr);
    return 0;
}

double ora_residual_norm(const ora_params* p, const double* H, const double* Hold,
                         const double* Hpre, const double* Dfield)
{
    octx c;
    if (setup(&c, p)) return NAN;
    long N = c.n[0] * c.n[1] * c.n[2];
    double* buf = (double*)calloc((size_t)4 * N, sizeof(double));
    if (!buf) return NAN;
    double* q2[3] = {buf, buf + N, buf + 2 * N};
    const double* Dcoef = Dfield;
    if (p->model == 3) {
        for (long i = 0; i < N; ++i) buf[3 * N + i] = exp(Dfield[i]);
        Dcoef = buf + 3 * N;
    }
    for (int d = 0; d < c.ndim; ++d) flux2_dim(&c, d, q2[d], Hpre ? Hpre : H, Dcoef);
    double r = residual_norm(&c, H, Hold, q2);
    free(buf);
    return r;
}

/* ------------------------------------------------------------------------ */
/* Discrete adjoint of nt implicit steps (models 2 and 3), FP64 reference.
 * Physical-unit restatement: q_f = -D_f (H_R - H_L)/h, D_f = E_f a^3,
 * a = (H_L+H_R)/2, E_f = (E_L+E_R)/2 (E = exp(m); E = 1 for model 2);
 * F_i = (H_i - Hold_i)/dt + sum_d (q_{i+1/2} - q_{i-1/2})/h_d = 0 per step.
 * L = 1/2 sum_inner (H^N - Ht)^2.  For n = N..1: J_n^T lam = g (BiCGSTAB,
 * matrix-free), dL/dm -= lam^T dF/dm, dL/dH0_boundary -= lam^T dF/dH_b,
 * g <- lam/dt; finally dL/dH0_inner = g.  This is new work (the reference has
 * no adjoint); it is the checker of the GPU adjoint. */
typedef struct {
    const octx* c;
    const double* H;   /* linearisation point H^n */
    const double* E;   /* exp(m) or NULL (model 2) */
} adj_ctx;

static inline double e_at(const adj_ctx* A, long i) { return A->E ? A->E[i] : 1.0; }

/* y = J^T x on inner cells (x zero on the boundary, y zero there). */
static void apply_JT(const adj_ctx* A, const double* x, double* y)
{
    const octx* c = A->c;
    long lo[3], hi[3];
    inner_range(c, lo, hi);
    const double rdt = 1.0 / c->p->dt;
#pragma omp parallel for collapse(2) schedule(static) num_threads(c->nth)
    for (long k = lo[2]; k < hi[2]; ++k)
        for (long j = lo[1]; j < hi[1]; ++j)
            for (long i = lo[0]; i < hi[0]; ++i) {
                long ic = i + c->s[1] * j + c->s[2] * k;
                double acc = x[ic] * rdt;
                for (int d = 0; d < c->ndim; ++d) {
                    const double h = c->h[d];
                    for (int side = 0; side < 2; ++side) {
                        long L = side ? ic : ic - c->s[d];
                        long R = L + c->s[d];
                        const double HL = A->H[L], HR = A->H[R];
                        const double a = (HL + HR) * 0.5;
                        const double Ef = (e_at(A, L) + e_at(A, R)) * 0.5;
                        const double Df = Ef * a * a * a, dD = Ef * 1.5 * a * a;
                        const double g = HR - HL;
                        /* dq/dH_L = (D - dD g)/h, dq/dH_R = (-D - dD g)/h */
                        const double dq = side ? (Df - dD * g) / h : (-Df - dD * g) / h;
                        acc += (x[L] - x[R]) / h * dq;
                    }
                }
                y[ic] = acc;
            }
}

static double dot_inner(const octx* c, const double* a, const double* b)
{
    long lo[3], hi[3];
    inner_range(c, lo, hi);
    double s = 0.0;
#pragma omp parallel for collapse(2) schedule(static) num_threads(c->nth) reduction(+ : s)
    for (long k = lo[2]; k < hi[2]; ++k)
        for (long j = lo[1]; j < hi[1]; ++j)
            for (long i = lo[0]; i < hi[0]; ++i) {
                long ic = i + c->s[1] * j + c->s[2] * k;
                s += a[ic] * b[ic];
            }
    return s;
}

/* BiCGSTAB for J^T x = b (inner cells), x0 = 0. */
static int bicgstab_JT(const adj_ctx* A, const double* b, double* x, double rtol, long N)
{
    double* r = (double*)calloc(N, sizeof(double));
    double* r0 = (double*)calloc(N, sizeof(double));
    double* pv = (double*)calloc(N, sizeof(double));
    double* v = (double*)calloc(N, sizeof(double));
    double* sv = (double*)calloc(N, sizeof(double));
    double* t = (double*)calloc(N, sizeof(double));
    if (!r || !r0 || !pv || !v || !sv || !t) {
        free(r); free(r0); free(pv); free(v); free(sv); free(t);
        return 1;
    }
    memset(x, 0, sizeof(double) * N);
    memcpy(r, b, sizeof(double) * N);
    memcpy(r0, b, sizeof(double) * N);
    double bn = sqrt(dot_inner(A->c, b, b));
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    int ok = 1;
    for (int it = 0; it < 20000 && bn > 0.0; ++it) {
        double rho1 = dot_inner(A->c, r0, r);
        double beta = (rho1 / rho) * (alpha / omega);
        for (long i = 0; i < N; ++i) pv[i] = r[i] + beta * (pv[i] - omega * v[i]);
        apply_JT(A, pv, v);
        alpha = rho1 / dot_inner(A->c, r0, v);
        for (long i = 0; i < N; ++i) sv[i] = r[i] - alpha * v[i];
        apply_JT(A, sv, t);
        omega = dot_inner(A->c, t, sv) / dot_inner(A->c, t, t);
        for (long i = 0; i < N; ++i) {
            x[i] += alpha * pv[i] + omega * sv[i];
            r[i] = sv[i] - omega * t[i];
        }
        rho = rho1;
        if (sqrt(dot_inner(A->c, r, r)) <= rtol * bn) { ok = 1; break; }
        ok = 0;
    }
    free(r); free(r0); free(pv); free(v); free(sv); free(t);
    return ok ? 0 : 3;
}

int ora_adjoint(const ora_params* p, const double* Hs, const double* m, const double* Ht,
                double* grad_m, double* grad_H0, double rtol)
{
    octx c;
    if (setup(&c, p) || (p->model != 2 && p->model != 3) || !Hs || !Ht || !grad_H0) return 1;
    if (p->model == 3 && (!m || !grad_m)) return 1;
    const long N = c.n[0] * c.n[1] * c.n[2];
    double* E = NULL;
    double* g = (double*)calloc(N, sizeof(double));
    double* lam = (double*)calloc(N, sizeof(double));
    if (p->model == 3) {
        E = (double*)malloc(sizeof(double) * N);
        for (long i = 0; i < N; ++i) E[i] = exp(m[i]);
        memset(grad_m, 0, sizeof(double) * N);
    }
    memset(grad_H0, 0, sizeof(double) * N);
    long lo[3], hi[3];
    inner_range(&c, lo, hi);
    const double* HN = Hs + (size_t)p->nt * N;
    for (long k = lo[2]; k < hi[2]; ++k)
        for (long j = lo[1]; j < hi[1]; ++j)
            for (long i = lo[0]; i < hi[0]; ++i) {
                long ic = i + c.s[1] * j + c.s[2] * k;
                g[ic] = HN[ic] - Ht[ic];
            }
    int status = 0;
    for (int n = p->nt; n >= 1; --n) {
        adj_ctx A = {&c, Hs + (size_t)n * N, E};
        if (bicgstab_JT(&A, g, lam, rtol, N)) status = 3;
        /* accumulate dL/dm and the boundary part of dL/dH0 face by face */
        for (int d = 0; d < c.ndim; ++d) {
            long flo[3], fhi[3];
            for (int e = 0; e < 3; ++e) face_range(&c, d, e, &flo[e], &fhi[e]);
            const double h = c.h[d];
            for (long k = flo[2]; k < fhi[2]; ++k)
                for (long j = flo[1]; j < fhi[1]; ++j)
                    for (long i = flo[0]; i < fhi[0]; ++i) {
                        long L = i + c.s[1] * j + c.s[2] * k, R = L + c.s[d];
                        const double HL = A.H[L], HR = A.H[R];
                        const double a = (HL + HR) * 0.5, gg = HR - HL;
                        const double EL = e_at(&A, L), ER = e_at(&A, R);
                        const double Ef = (EL + ER) * 0.5;
                        const double Df = Ef * a * a * a, dD = Ef * 1.5 * a * a;
                        const double w = (lam[L] - lam[R]) / h;   /* lam^T dF = w * dq */
                        if (E) {
                            /* dq/dm_L = -(0.5 E_L a^3) g / h */
                            grad_m[L] -= w * (-(0.5 * EL * a * a * a) * gg / h);
                            grad_m[R] -= w * (-(0.5 * ER * a * a * a) * gg / h);
                        }
                        /* boundary cells of H (frozen = H0 there) */
                        const int Lb = !is_inner(&c, L), Rb = !is_inner(&c, R);
                        if (Lb) grad_H0[L] -= w * ((Df - dD * gg) / h);
                        if (Rb) grad_H0[R] -= w * ((-Df - dD * gg) / h);
                    }
        }
        for (long i = 0; i < N; ++i) g[i] = lam[i] / p->dt;
    }
    for (long k = lo[2]; k < hi[2]; ++k)
        for (long j = lo[1]; j < hi[1]; ++j)
            for (long i = lo[0]; i < hi[0]; ++i) {
                long ic = i + c.s[1] * j + c.s[2] * k;
                grad_H0[ic] += g[ic];
            }
    free(E); free(g); free(lam);
    return status;
}
