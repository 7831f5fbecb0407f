// ptd_fp64.cu -- fused FP64 PT-iteration kernels (one launch per iteration).
//
// One launch computes, for every face, the damped flux of iteration k+1 from
// H^k and the flux of iteration k, and for every inner cell H^{k+1} from those
// new fluxes: the reference's compute_flux! + compute_update! pair
// (scripts/diff_2D_nonlin.jl:154-165, diff_3D/diff_3D_nonlin_multixpu.jl:37-50,
// diff_1D_nonlin.jl:24-33 and the lin/linstep siblings) in a single pass over
// memory.  H and the fluxes are double-buffered (read k, write k+1), which
// keeps the reference's Jacobi semantics across tile boundaries.  On a check
// iteration (template CHECK) the same pass also forms the reference's mixed
// residual (check_res!, scripts/diff_2D_nonlin.jl:167-170): undamped flux from
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
#include "ptd_device.cuh"
#include "ptd_kernels.h"

namespace ptd {

// ---------------------------------------------------------------------------
// 1D: one thread per cell; the left face is recomputed (1D grids are small).
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) pt1d_kernel(PTArgs a)
{
    if (step_done(a.done)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = a.nx;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    if (i < nx) {
        const double Hc = a.Hin[i];
        const float hc = MODEL == NONLIN ? d2f_bits(Hc) : 0.0f;
        const double Dc = MODEL == LINSTEP ? a.D[i] : 0.0;
        double wr = 0.0, ur = 0.0;
        double Dr = 0.0;
        if (i <= nx - 2) {
            const double Hr = a.Hin[i + 1];
            Dr = MODEL == LINSTEP ? a.D[i + 1] : 0.0;
            wr = face_update<MODEL, CHECK>(a, Hc, Hr, MODEL == NONLIN ? hc + d2f_bits(Hr) : 0.0f,
                                           Dc, Dr, a.win[0][i], ur);
            a.wout[0][i] = wr;
        }
        if (i >= 1 && i <= nx - 2) {
            const double Hl = a.Hin[i - 1];
            const double Dl = MODEL == LINSTEP ? a.D[i - 1] : 0.0;
            double ul = 0.0;
            const double wl = face_update<MODEL, CHECK>(
                a, Hl, Hc, MODEL == NONLIN ? d2f_bits(Hl) + hc : 0.0f, Dl, Dc, a.win[0][i - 1], ul);
            const double Ho = a.Hold[i];
            const double div = (wr - wl) * a.sig[0];
            double e;
            if (MODEL == LIN) {
                e = a.e_lin;
            } else if (MODEL == LINSTEP) {
                const float dmax = fmaxf(fmaxf(d2f_bits(Dl), d2f_bits(Dr)), d2f_bits(Dc));
                e = f2d_bits(linstep_cell_e(a.f, dmax));
            } else {
                e = f2d_bits(nonlin_cell_e(a.f, hc));
            }
            const double Hn = fma(-e, fma(Hc - Ho, a.rdt, div), Hc);
            a.Hout[i] = Hn;
            if (CHECK) {
                const double r = fma(-(Hn - Ho), a.rdt, (ur - ul) * a.sig[0]);
                accumulate_residual(r, part, pmax);
            }
        }
    }
    if (CHECK) block_reduce_residual(a, part, pmax);
}

// ---------------------------------------------------------------------------
// 2D: blockDim = (32, W); warp w of block b owns the x strip of tile
// t = b*W + w: cells i = 31t + lane (lane 0 = left neighbour), and marches
// rows j0 .. j1-1 of chunk blockIdx.y.
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) pt2d_kernel(PTArgs a, int chunk)
{
    if (step_done(a.done)) return;
    const int lane = threadIdx.x;
    const int tile = blockIdx.x * blockDim.y + threadIdx.y;
    const int i = 31 * tile + lane;
    const int nx = a.nx, ny = a.ny;
    const int j0 = 1 + blockIdx.y * chunk;
    const int j1 = min(j0 + chunk, ny - 1);
    double part = 0.0;
    unsigned long long pmax = 0ull;
    const bool warp_active = (31 * tile < nx - 1) && (j0 < j1);
    if (warp_active) {
        const int ic = min(i, nx - 1);
        const bool xface = i <= nx - 2;
        const bool inner_x = i >= 1 && i <= nx - 2;
        const bool upd = inner_x && lane >= 1;
        const bool own_x = xface && (lane >= 1 || tile == 0);
        const long long sy = a.sy;
        long long idx = (long long)j0 * sy + ic;

        double Hc = a.Hin[idx];
        float hc = MODEL == NONLIN ? d2f_bits(Hc) : 0.0f;
        double Dc = MODEL == LINSTEP ? a.D[idx] : 0.0;
        float dcf = MODEL == LINSTEP ? d2f_bits(Dc) : 0.0f;
        float dbf = 0.0f;
        double wyb = 0.0, uyb = 0.0;
        if (upd) {
            // face (j0 - 1/2), owned by the chunk below unless j0 == 1
            const double Hb = a.Hin[idx - sy];
            const double Db = MODEL == LINSTEP ? a.D[idx - sy] : 0.0;
            dbf = MODEL == LINSTEP ? d2f_bits(Db) : 0.0f;
            wyb = face_update<MODEL, CHECK>(a, Hb, Hc, MODEL == NONLIN ? d2f_bits(Hb) + hc : 0.0f, Db,
                                            Dc, a.win[1][idx - sy], uyb);
            if (j0 == 1) a.wout[1][idx - sy] = wyb;
        }
        for (int j = j0; j < j1; ++j, idx += sy) {
            const double Hn = a.Hin[idx + sy];
            const double wx = a.win[0][idx];
            const double wy = a.win[1][idx];
            const double Ho = a.Hold[idx];
            const double Dn = MODEL == LINSTEP ? a.D[idx + sy] : 0.0;
            double Hr = __shfl_down_sync(FULL, Hc, 1);
            float hr = MODEL == NONLIN ? __shfl_down_sync(FULL, hc, 1) : 0.0f;
            double Dr = MODEL == LINSTEP ? __shfl_down_sync(FULL, Dc, 1) : 0.0;
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                Hr = ok ? a.Hin[idx + 1] : Hc;
                if (MODEL == NONLIN) hr = d2f_bits(Hr);
                if (MODEL == LINSTEP) Dr = ok ? a.D[idx + 1] : Dc;
            }
            const float hn = MODEL == NONLIN ? d2f_bits(Hn) : 0.0f;
            double ux = 0.0, uy = 0.0, wxn = 0.0, wyn = 0.0;
            if (xface) wxn = face_update<MODEL, CHECK>(a, Hc, Hr, hc + hr, Dc, Dr, wx, ux);
            if (upd) wyn = face_update<MODEL, CHECK>(a, Hc, Hn, hc + hn, Dc, Dn, wy, uy);
            const double wxl = __shfl_up_sync(FULL, wxn, 1);
            const double uxl = CHECK ? __shfl_up_sync(FULL, ux, 1) : 0.0;
            const float dlf = MODEL == LINSTEP ? __shfl_up_sync(FULL, dcf, 1) : 0.0f;
            const float dnf = MODEL == LINSTEP ? d2f_bits(Dn) : 0.0f;
            if (own_x) a.wout[0][idx] = wxn;
            if (upd) {
                a.wout[1][idx] = wyn;
                double e;
                if (MODEL == LIN) {
                    e = a.e_lin;
                } else if (MODEL == LINSTEP) {
                    const float dmax =
                        fmaxf(fmaxf(fmaxf(dcf, dlf), fmaxf(d2f_bits(Dr), dbf)), dnf);
                    e = f2d_bits(linstep_cell_e(a.f, dmax));
                } else {
                    e = f2d_bits(nonlin_cell_e(a.f, hc));
                }
                const double div = fma(wyn - wyb, a.sig[1], (wxn - wxl) * a.sig[0]);
                const double Hnew = fma(-e, fma(Hc - Ho, a.rdt, div), Hc);
                a.Hout[idx] = Hnew;
                if (CHECK) {
                    const double r =
                        fma(-(Hnew - Ho), a.rdt, fma(uy - uyb, a.sig[1], (ux - uxl) * a.sig[0]));
                    accumulate_residual(r, part, pmax);
                }
            }
            Hc = Hn;
            hc = hn;
            wyb = wyn;
            uyb = uy;
            if (MODEL == LINSTEP) {
                dbf = dcf;
                Dc = Dn;
                dcf = dnf;
            }
        }
    }
    if (CHECK) block_reduce_residual(a, part, pmax);
}

// ---------------------------------------------------------------------------
// 3D: blockDim = (32, R).  Block (bx, by, bz) owns cells
// i = 31*bx + lane, j = (R-1)*by + r (lane 0 / row 0 are the neighbours) and
// marches planes k0 .. k1-1 of z chunk bz.
template <int MODEL, bool CHECK, int R>
__global__ void __launch_bounds__(32 * R) pt3d_kernel(PTArgs a, int chunk)
{
    if (step_done(a.done)) return;
    __shared__ double sH[2][R][32];
    __shared__ double sW[2][R][32];
    __shared__ double sU[CHECK ? 2 : 1][CHECK ? R : 1][32];
    __shared__ float sF[2][R][32];   // NONLIN: H as float; LINSTEP: D as float
    __shared__ double sD[MODEL == LINSTEP ? 2 : 1][MODEL == LINSTEP ? R : 1][32];

    const int lane = threadIdx.x, r = threadIdx.y;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int i = 31 * blockIdx.x + lane;
    const int j = (R - 1) * blockIdx.y + r;
    const int k0 = 1 + blockIdx.z * chunk;
    const int k1 = min(k0 + chunk, nz - 1);
    double part = 0.0;
    unsigned long long pmax = 0ull;
    if (k0 < k1) {   // uniform over the block
        const int ic = min(i, nx - 1), jc = min(j, ny - 1);
        const bool inner_x = i >= 1 && i <= nx - 2;
        const bool inner_y = j >= 1 && j <= ny - 2;
        const bool xface = i <= nx - 2 && inner_y;
        const bool yface = j <= ny - 2 && inner_x;
        const bool zface = inner_x && inner_y;
        const bool upd = zface && lane >= 1 && r >= 1;
        const bool own_x = xface && (lane >= 1 || blockIdx.x == 0) && r >= 1;
        const bool own_y = yface && lane >= 1 && (r >= 1 || blockIdx.y == 0);
        const bool top = r == R - 1;
        const bool up_ok = jc + 1 < ny;
        const long long sy = a.sy, sz = a.sz;
        long long idx = (long long)k0 * sz + (long long)jc * sy + ic;

        double Hc = a.Hin[idx];
        float hc = MODEL == NONLIN ? d2f_bits(Hc) : 0.0f;
        double Dc = MODEL == LINSTEP ? a.D[idx] : 0.0;
        float dcf = MODEL == LINSTEP ? d2f_bits(Dc) : 0.0f;
        float dbf = 0.0f;
        double wzb = 0.0, uzb = 0.0;
        if (upd) {
            const double Hb = a.Hin[idx - sz];
            const double Db = MODEL == LINSTEP ? a.D[idx - sz] : 0.0;
            dbf = MODEL == LINSTEP ? d2f_bits(Db) : 0.0f;
            wzb = face_update<MODEL, CHECK>(a, Hb, Hc, MODEL == NONLIN ? d2f_bits(Hb) + hc : 0.0f, Db,
                                            Dc, a.win[2][idx - sz], uzb);
            if (k0 == 1) a.wout[2][idx - sz] = wzb;
        }
        int p = 0;
        sH[0][r][lane] = Hc;
        if (MODEL == NONLIN) sF[0][r][lane] = hc;
        if (MODEL == LINSTEP) {
            sD[0][r][lane] = Dc;
            sF[0][r][lane] = dcf;
        }
        __syncthreads();
        for (int k = k0; k < k1; ++k, idx += sz) {
            const double Hn = a.Hin[idx + sz];
            const double wx = a.win[0][idx];
            const double wy = a.win[1][idx];
            const double wz = a.win[2][idx];
            const double Ho = a.Hold[idx];
            const double Dn = MODEL == LINSTEP ? a.D[idx + sz] : 0.0;
            // neighbours in y (row above: shared memory, top row: global)
            double Hu, Du = 0.0;
            float hu = 0.0f, duf = 0.0f;
            if (!top) {
                Hu = sH[p][r + 1][lane];
                if (MODEL == NONLIN) hu = sF[p][r + 1][lane];
                if (MODEL == LINSTEP) {
                    Du = sD[p][r + 1][lane];
                    duf = sF[p][r + 1][lane];
                }
            } else {
                Hu = up_ok ? a.Hin[idx + sy] : Hc;
                if (MODEL == NONLIN) hu = d2f_bits(Hu);
                if (MODEL == LINSTEP) {
                    Du = up_ok ? a.D[idx + sy] : Dc;
                    duf = d2f_bits(Du);
                }
            }
            // neighbour in x
            double Hr = __shfl_down_sync(FULL, Hc, 1);
            float hr = MODEL == NONLIN ? __shfl_down_sync(FULL, hc, 1) : 0.0f;
            double Dr = MODEL == LINSTEP ? __shfl_down_sync(FULL, Dc, 1) : 0.0;
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                Hr = ok ? a.Hin[idx + 1] : Hc;
                if (MODEL == NONLIN) hr = d2f_bits(Hr);
                if (MODEL == LINSTEP) Dr = ok ? a.D[idx + 1] : Dc;
            }
            const float hn = MODEL == NONLIN ? d2f_bits(Hn) : 0.0f;
            const float dnf = MODEL == LINSTEP ? d2f_bits(Dn) : 0.0f;
            double ux = 0.0, uy = 0.0, uz = 0.0, wxn = 0.0, wyn = 0.0, wzn = 0.0;
            if (xface && r >= 1) wxn = face_update<MODEL, CHECK>(a, Hc, Hr, hc + hr, Dc, Dr, wx, ux);
            if (yface) wyn = face_update<MODEL, CHECK>(a, Hc, Hu, hc + hu, Dc, Du, wy, uy);
            if (upd) wzn = face_update<MODEL, CHECK>(a, Hc, Hn, hc + hn, Dc, Dn, wz, uz);
            if (own_x) a.wout[0][idx] = wxn;
            if (own_y) a.wout[1][idx] = wyn;
            if (upd) a.wout[2][idx] = wzn;
            const double wxl = __shfl_up_sync(FULL, wxn, 1);
            const double uxl = CHECK ? __shfl_up_sync(FULL, ux, 1) : 0.0;
            const float dlf = MODEL == LINSTEP ? __shfl_up_sync(FULL, dcf, 1) : 0.0f;
            // publish this plane's y faces and the next plane's H, one barrier
            sW[p][r][lane] = wyn;
            if (CHECK) sU[p][r][lane] = uy;
            sH[p ^ 1][r][lane] = Hn;
            if (MODEL == NONLIN) sF[p ^ 1][r][lane] = hn;
            if (MODEL == LINSTEP) {
                sD[p ^ 1][r][lane] = Dn;
                sF[p ^ 1][r][lane] = dnf;
            }
            // the row below's D for maxloc (sF[p] is rewritten only after the barrier)
            const float ddf = (MODEL == LINSTEP && r >= 1) ? sF[p][r - 1][lane] : 0.0f;
            __syncthreads();
            if (upd) {
                const double wyb = sW[p][r - 1][lane];
                double e;
                if (MODEL == LIN) {
                    e = a.e_lin;
                } else if (MODEL == LINSTEP) {
                    const float dmax = fmaxf(fmaxf(fmaxf(dcf, dlf), fmaxf(d2f_bits(Dr), duf)),
                                             fmaxf(fmaxf(ddf, dbf), dnf));
                    e = f2d_bits(linstep_cell_e(a.f, dmax));
                } else {
                    e = f2d_bits(nonlin_cell_e(a.f, hc));
                }
                const double div =
                    fma(wzn - wzb, a.sig[2], fma(wyn - wyb, a.sig[1], (wxn - wxl) * a.sig[0]));
                const double Hnew = fma(-e, fma(Hc - Ho, a.rdt, div), Hc);
                a.Hout[idx] = Hnew;
                if (CHECK) {
                    const double uyb = sU[p][r - 1][lane];
                    const double r2 = fma(-(Hnew - Ho), a.rdt,
                                          fma(uz - uzb, a.sig[2],
                                              fma(uy - uyb, a.sig[1], (ux - uxl) * a.sig[0])));
                    accumulate_residual(r2, part, pmax);
                }
            }
            Hc = Hn;
            hc = hn;
            wzb = wzn;
            uzb = uz;
            if (MODEL == LINSTEP) {
                dbf = dcf;
                Dc = Dn;
                dcf = dnf;
            }
            p ^= 1;
        }
    }
    if (CHECK) block_reduce_residual(a, part, pmax);
}

// ---------------------------------------------------------------------------
// Consistent residual (both flux terms from the updated H): one thread per
// inner cell, generic over ndim (unused dimensions have extent 1).
template <int MODEL>
__global__ void __launch_bounds__(256) resid_consistent_kernel(PTArgs a, int ndim)
{
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
        const long long st[3] = {1, a.sy, a.sz};
        const double H = a.Hout[c];
        double div = 0.0;
        for (int d = 0; d < ndim; ++d) {
            double uR = 0.0, uL = 0.0;
            const double HR = a.Hout[c + st[d]], HL = a.Hout[c - st[d]];
            if (MODEL == LIN) {
                uR = HR - H;
                uL = H - HL;
            } else if (MODEL == LINSTEP) {
                uR = (a.D[c] + a.D[c + st[d]]) * (HR - H);
                uL = (a.D[c - st[d]] + a.D[c]) * (H - HL);
            } else {
                const double sR = H + HR, sL = HL + H;
                uR = sR * sR * sR * (HR - H);
                uL = sL * sL * sL * (H - HL);
            }
            div = fma(uR - uL, a.sig[d], div);
        }
        const double r = fma(-(H - a.Hold[c]), a.rdt, div);
        accumulate_residual(r, part, pmax);
    }
    block_reduce_residual(a, part, pmax);
}

__global__ void judge_kernel(DevState* st, double* errhist, int errcap, int nchk, int itmax,
                             double tol, double norm_den, int norm_max)
{
    if (st->done) return;
    const double acc = st->acc;
    st->acc = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(norm_den);
    const int n = st->nchecks;
    if (n < errcap) errhist[n] = err;
    st->nchecks = n + 1;
    st->iter += nchk;
    st->err = err;
    if (!(err > tol)) st->done = (err != err) ? DONE_NAN : DONE_CONVERGED;
    else if (st->iter + nchk > itmax) st->done = DONE_CAP;
}

__global__ void reset_state_kernel(DevState* st)
{
    st->done = DONE_RUNNING;
    st->nchecks = 0;
    st->iter = 0;
    st->acc = 0.0;
    st->err = 0.0;
}

// ---------------------------------------------------------------------------
template <int MODEL, bool CHECK>
static cudaError_t launch_model(const PTArgs& a, int ndim, const LaunchCfg& cfg, cudaStream_t s)
{
    if (ndim == 1) {
        const int bs = 256;
        pt1d_kernel<MODEL, CHECK><<<(a.nx + bs - 1) / bs, bs, 0, s>>>(a);
    } else if (ndim == 2) {
        const int W = cfg.warps2d;
        const int tiles = (a.nx - 2 + 30) / 31;
        dim3 grid((tiles + W - 1) / W, (a.ny - 2 + cfg.chunk2d - 1) / cfg.chunk2d);
        pt2d_kernel<MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, cfg.chunk2d);
    } else {
        const int tx = (a.nx - 2 + 30) / 31;
        const int nzc = (a.nz - 2 + cfg.chunk3d - 1) / cfg.chunk3d;
        if (cfg.rows3d == 8) {
            dim3 grid(tx, (a.ny - 2 + 6) / 7, nzc);
            pt3d_kernel<MODEL, CHECK, 8><<<grid, dim3(32, 8), 0, s>>>(a, cfg.chunk3d);
        } else {
            dim3 grid(tx, (a.ny - 2 + 14) / 15, nzc);
            pt3d_kernel<MODEL, CHECK, 16><<<grid, dim3(32, 16), 0, s>>>(a, cfg.chunk3d);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_pt_fp64(const PTArgs& a, int ndim, int model, bool check, const LaunchCfg& cfg,
                           cudaStream_t s)
{
    switch (model * 2 + (check ? 1 : 0)) {
    case 0: return launch_model<LIN, false>(a, ndim, cfg, s);
    case 1: return launch_model<LIN, true>(a, ndim, cfg, s);
    case 2: return launch_model<LINSTEP, false>(a, ndim, cfg, s);
    case 3: return launch_model<LINSTEP, true>(a, ndim, cfg, s);
    case 4: return launch_model<NONLIN, false>(a, ndim, cfg, s);
    case 5: return launch_model<NONLIN, true>(a, ndim, cfg, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_resid_consistent(const PTArgs& a, int ndim, int model, cudaStream_t s)
{
    const int bs = 256, nb = 152 * 8;
    if (model == LIN) resid_consistent_kernel<LIN><<<nb, bs, 0, s>>>(a, ndim);
    else if (model == LINSTEP) resid_consistent_kernel<LINSTEP><<<nb, bs, 0, s>>>(a, ndim);
    else resid_consistent_kernel<NONLIN><<<nb, bs, 0, s>>>(a, ndim);
    return cudaGetLastError();
}

cudaError_t launch_judge(DevState* st, double* errhist, int errcap, int nchk, int itmax, double tol,
                         double norm_den, int norm_max, cudaStream_t s)
{
    judge_kernel<<<1, 1, 0, s>>>(st, errhist, errcap, nchk, itmax, tol, norm_den, norm_max);
    return cudaGetLastError();
}

cudaError_t launch_reset_state(DevState* st, cudaStream_t s)
{
    reset_state_kernel<<<1, 1, 0, s>>>(st);
    return cudaGetLastError();
}

}  // namespace ptd
