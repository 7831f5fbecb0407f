// ptd_pt.cu -- fused PT-iteration kernels (one launch per iteration), generic
// over the number type: F64 (native FP64) and DF64 (double-float on the FP32
// pipe, same 8 bytes per value), see ptd_num.cuh.
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
#include "ptd_num.cuh"

namespace ptd {

// w - c*t with a float damping coefficient c.
__device__ __forceinline__ double nmadf(F64, float c, double t, double w) { return fma(-f2d_bits(c), t, w); }
__device__ __forceinline__ float2 nmadf(DF64, float c, float2 t, float2 w) { return DF64::sub(w, DF64::mulf(t, c)); }

template <class N>
__device__ __forceinline__ typename N::T ld(const void* p, long long i)
{
    return reinterpret_cast<const typename N::T*>(p)[i];
}
template <class N>
__device__ __forceinline__ void st(void* p, long long i, typename N::T v)
{
    reinterpret_cast<typename N::T*>(p)[i] = v;
}

// One face: new scaled flux, and u = K_f * g (undamped flux) when U.
template <class N, int MODEL, bool U>
__device__ __forceinline__ typename N::T face_t(const PTArgs& a, typename N::T HL, typename N::T HR, float hsum,
                                                typename N::T DL, typename N::T DR, typename N::T w,
                                                typename N::T& u)
{
    using T = typename N::T;
    const T g = N::sub(HR, HL);
    if (MODEL == LIN) {
        if (U) u = g;
        return nmadf(N(), a.fc_lin, N::add(g, w), w);
    }
    float c;
    T K;
    if (MODEL == LINSTEP) {
        K = N::add(DL, DR);
        c = a.fc_lin;
    } else {
        const T s = N::add(HL, HR);
        K = N::mul(N::mul(s, s), s);
        c = nonlin_face_c(a.f, hsum);
    }
    T t;
    if (U) {
        u = N::mul(K, g);
        t = N::native ? N::mad(K, g, w) : N::add(u, w);
    } else {
        t = N::mad(K, g, w);
    }
    return nmadf(N(), c, t, w);
}

template <class N>
__device__ __forceinline__ typename N::T cst(const PTArgs& a, int which);
template <>
__device__ __forceinline__ double cst<F64>(const PTArgs& a, int which)
{
    return which < 3 ? a.sig[which] : a.rdt;
}
template <>
__device__ __forceinline__ float2 cst<DF64>(const PTArgs& a, int which)
{
    return which < 3 ? a.sig_df[which] : a.rdt_df;
}

template <int MODEL>
__device__ __forceinline__ float cell_e(const PTArgs& a, float h, float dmax)
{
    if (MODEL == LIN) return a.fe_lin;
    if (MODEL == LINSTEP) return linstep_cell_e(a.f, dmax);
    return nonlin_cell_e(a.f, h);
}

// H_new = H - e*((H - Hold)/dt + div)
template <class N>
__device__ __forceinline__ typename N::T h_update(const PTArgs& a, typename N::T Hc, typename N::T Ho,
                                                  typename N::T div, float e)
{
    const typename N::T Rp = N::mad(N::sub(Hc, Ho), cst<N>(a, 3), div);
    return nmadf(N(), e, Rp, Hc);
}

// ---------------------------------------------------------------------------
// 1D: one thread per cell; the left face is recomputed (1D grids are small).
template <class N, int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) pt1d_kernel(PTArgs a)
{
    using T = typename N::T;
    if (step_done(a.done)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = a.nx;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    if (i < nx) {
        const T Hc = ld<N>(a.Hin, i);
        const float hc = N::lo_f(Hc);
        const T Dc = MODEL == LINSTEP ? ld<N>(a.D, i) : N::zero();
        T wr = N::zero(), ur = N::zero(), Dr = N::zero();
        if (i <= nx - 2) {
            const T Hr = ld<N>(a.Hin, i + 1);
            if (MODEL == LINSTEP) Dr = ld<N>(a.D, i + 1);
            wr = face_t<N, MODEL, CHECK>(a, Hc, Hr, hc + N::lo_f(Hr), Dc, Dr, ld<N>(a.win[0], i), ur);
            st<N>(a.wout[0], i, wr);
        }
        if (i >= 1 && i <= nx - 2) {
            const T Hl = ld<N>(a.Hin, i - 1);
            const T Dl = MODEL == LINSTEP ? ld<N>(a.D, i - 1) : N::zero();
            T ul = N::zero();
            const T wl = face_t<N, MODEL, CHECK>(a, Hl, Hc, N::lo_f(Hl) + hc, Dl, Dc, ld<N>(a.win[0], i - 1), ul);
            const T Ho = ld<N>(a.Hold, i);
            const T div = N::mul(N::sub(wr, wl), cst<N>(a, 0));
            const float e = cell_e<MODEL>(a, hc, fmaxf(fmaxf(N::lo_f(Dl), N::lo_f(Dr)), N::lo_f(Dc)));
            const T Hn = h_update<N>(a, Hc, Ho, div, e);
            st<N>(a.Hout, i, Hn);
            if (CHECK) {
                const T r = N::sub(N::mul(N::sub(ur, ul), cst<N>(a, 0)), N::mul(N::sub(Hn, Ho), cst<N>(a, 3)));
                accumulate_residual(N::to_d(r), part, pmax);
            }
        }
    }
    if (CHECK) block_reduce_residual(a, part, pmax);
}

// ---------------------------------------------------------------------------
// 2D: blockDim = (32, W); warp w of block b owns the x strip of tile
// t = b*W + w: cells i = 31t + lane (lane 0 = left neighbour), and marches
// rows j0 .. j1-1 of chunk blockIdx.y.
template <class N, int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) pt2d_kernel(PTArgs a, int chunk)
{
    using T = typename N::T;
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

        T Hc = ld<N>(a.Hin, idx);
        float hc = N::lo_f(Hc);
        T Dc = MODEL == LINSTEP ? ld<N>(a.D, idx) : N::zero();
        float dcf = MODEL == LINSTEP ? N::lo_f(Dc) : 0.0f;
        float dbf = 0.0f;
        T wyb = N::zero(), uyb = N::zero();
        if (upd) {
            // face (j0 - 1/2), owned by the chunk below unless j0 == 1
            const T Hb = ld<N>(a.Hin, idx - sy);
            const T Db = MODEL == LINSTEP ? ld<N>(a.D, idx - sy) : N::zero();
            dbf = MODEL == LINSTEP ? N::lo_f(Db) : 0.0f;
            wyb = face_t<N, MODEL, CHECK>(a, Hb, Hc, N::lo_f(Hb) + hc, Db, Dc, ld<N>(a.win[1], idx - sy), uyb);
            if (j0 == 1) st<N>(a.wout[1], idx - sy, wyb);
        }
        for (int j = j0; j < j1; ++j, idx += sy) {
            const T Hn = ld<N>(a.Hin, idx + sy);
            const T wx = ld<N>(a.win[0], idx);
            const T wy = ld<N>(a.win[1], idx);
            const T Ho = ld<N>(a.Hold, idx);
            const T Dn = MODEL == LINSTEP ? ld<N>(a.D, idx + sy) : N::zero();
            T Hr = N::shfl_down(Hc, 1);
            float hr = __shfl_down_sync(FULL, hc, 1);
            T Dr = MODEL == LINSTEP ? N::shfl_down(Dc, 1) : N::zero();
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                Hr = ok ? ld<N>(a.Hin, idx + 1) : Hc;
                hr = N::lo_f(Hr);
                if (MODEL == LINSTEP) Dr = ok ? ld<N>(a.D, idx + 1) : Dc;
            }
            const float hn = N::lo_f(Hn);
            T ux = N::zero(), uy = N::zero(), wxn = N::zero(), wyn = N::zero();
            if (xface) wxn = face_t<N, MODEL, CHECK>(a, Hc, Hr, hc + hr, Dc, Dr, wx, ux);
            if (upd) wyn = face_t<N, MODEL, CHECK>(a, Hc, Hn, hc + hn, Dc, Dn, wy, uy);
            const T wxl = N::shfl_up(wxn, 1);
            const T uxl = CHECK ? N::shfl_up(ux, 1) : N::zero();
            const float dlf = MODEL == LINSTEP ? __shfl_up_sync(FULL, dcf, 1) : 0.0f;
            const float dnf = MODEL == LINSTEP ? N::lo_f(Dn) : 0.0f;
            if (own_x) st<N>(a.wout[0], idx, wxn);
            if (upd) {
                st<N>(a.wout[1], idx, wyn);
                const float dmax =
                    MODEL == LINSTEP ? fmaxf(fmaxf(fmaxf(dcf, dlf), fmaxf(N::lo_f(Dr), dbf)), dnf) : 0.0f;
                const float e = cell_e<MODEL>(a, hc, dmax);
                const T div = N::mad(N::sub(wyn, wyb), cst<N>(a, 1), N::mul(N::sub(wxn, wxl), cst<N>(a, 0)));
                const T Hnew = h_update<N>(a, Hc, Ho, div, e);
                st<N>(a.Hout, idx, Hnew);
                if (CHECK) {
                    const T divu = N::mad(N::sub(uy, uyb), cst<N>(a, 1), N::mul(N::sub(ux, uxl), cst<N>(a, 0)));
                    const T r = N::sub(divu, N::mul(N::sub(Hnew, Ho), cst<N>(a, 3)));
                    accumulate_residual(N::to_d(r), part, pmax);
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
template <class N, int MODEL, bool CHECK, int R>
__global__ void __launch_bounds__(32 * R) pt3d_kernel(PTArgs a, int chunk)
{
    using T = typename N::T;
    if (step_done(a.done)) return;
    __shared__ T sH[2][R][32];
    __shared__ T sW[2][R][32];
    __shared__ T sU[CHECK ? 2 : 1][CHECK ? R : 1][32];
    __shared__ float sF[2][R][32];   // H as float (NONLIN) / D as float (LINSTEP)
    __shared__ T sD[MODEL == LINSTEP ? 2 : 1][MODEL == LINSTEP ? R : 1][32];

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
        const bool xface = i <= nx - 2 && inner_y && r >= 1;
        const bool yface = j <= ny - 2 && inner_x;
        const bool upd = inner_x && inner_y && lane >= 1 && r >= 1;
        const bool own_x = xface && (lane >= 1 || blockIdx.x == 0);
        const bool own_y = yface && lane >= 1 && (r >= 1 || blockIdx.y == 0);
        const bool top = r == R - 1;
        const bool up_ok = jc + 1 < ny;
        const long long sy = a.sy, sz = a.sz;
        long long idx = (long long)k0 * sz + (long long)jc * sy + ic;

        T Hc = ld<N>(a.Hin, idx);
        float hc = N::lo_f(Hc);
        T Dc = MODEL == LINSTEP ? ld<N>(a.D, idx) : N::zero();
        float dcf = MODEL == LINSTEP ? N::lo_f(Dc) : 0.0f;
        float dbf = 0.0f;
        T wzb = N::zero(), uzb = N::zero();
        if (upd) {
            const T Hb = ld<N>(a.Hin, idx - sz);
            const T Db = MODEL == LINSTEP ? ld<N>(a.D, idx - sz) : N::zero();
            dbf = MODEL == LINSTEP ? N::lo_f(Db) : 0.0f;
            wzb = face_t<N, MODEL, CHECK>(a, Hb, Hc, N::lo_f(Hb) + hc, Db, Dc, ld<N>(a.win[2], idx - sz), uzb);
            if (k0 == 1) st<N>(a.wout[2], idx - sz, wzb);
        }
        int p = 0;
        sH[0][r][lane] = Hc;
        sF[0][r][lane] = MODEL == LINSTEP ? dcf : hc;
        if (MODEL == LINSTEP) sD[0][r][lane] = Dc;
        __syncthreads();
        for (int k = k0; k < k1; ++k, idx += sz) {
            const T Hn = ld<N>(a.Hin, idx + sz);
            const T wx = ld<N>(a.win[0], idx);
            const T wy = ld<N>(a.win[1], idx);
            const T wz = ld<N>(a.win[2], idx);
            const T Ho = ld<N>(a.Hold, idx);
            const T Dn = MODEL == LINSTEP ? ld<N>(a.D, idx + sz) : N::zero();
            // neighbours in y (row above: shared memory, top row: global)
            T Hu, Du = N::zero();
            float hu = 0.0f, duf = 0.0f;
            if (!top) {
                Hu = sH[p][r + 1][lane];
                if (MODEL == LINSTEP) {
                    Du = sD[p][r + 1][lane];
                    duf = sF[p][r + 1][lane];
                } else {
                    hu = sF[p][r + 1][lane];
                }
            } else {
                Hu = up_ok ? ld<N>(a.Hin, idx + sy) : Hc;
                hu = N::lo_f(Hu);
                if (MODEL == LINSTEP) {
                    Du = up_ok ? ld<N>(a.D, idx + sy) : Dc;
                    duf = N::lo_f(Du);
                }
            }
            // the row below's D for maxloc (sF[p] is rewritten only after the barrier)
            const float ddf = (MODEL == LINSTEP && r >= 1) ? sF[p][r - 1][lane] : 0.0f;
            // neighbour in x
            T Hr = N::shfl_down(Hc, 1);
            float hr = __shfl_down_sync(FULL, hc, 1);
            T Dr = MODEL == LINSTEP ? N::shfl_down(Dc, 1) : N::zero();
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                Hr = ok ? ld<N>(a.Hin, idx + 1) : Hc;
                hr = N::lo_f(Hr);
                if (MODEL == LINSTEP) Dr = ok ? ld<N>(a.D, idx + 1) : Dc;
            }
            const float hn = N::lo_f(Hn);
            const float dnf = MODEL == LINSTEP ? N::lo_f(Dn) : 0.0f;
            T ux = N::zero(), uy = N::zero(), uz = N::zero(), wxn = N::zero(), wyn = N::zero(), wzn = N::zero();
            if (xface) wxn = face_t<N, MODEL, CHECK>(a, Hc, Hr, hc + hr, Dc, Dr, wx, ux);
            if (yface) wyn = face_t<N, MODEL, CHECK>(a, Hc, Hu, hc + hu, Dc, Du, wy, uy);
            if (upd) wzn = face_t<N, MODEL, CHECK>(a, Hc, Hn, hc + hn, Dc, Dn, wz, uz);
            if (own_x) st<N>(a.wout[0], idx, wxn);
            if (own_y) st<N>(a.wout[1], idx, wyn);
            if (upd) st<N>(a.wout[2], idx, wzn);
            const T wxl = N::shfl_up(wxn, 1);
            const T uxl = CHECK ? N::shfl_up(ux, 1) : N::zero();
            const float dlf = MODEL == LINSTEP ? __shfl_up_sync(FULL, dcf, 1) : 0.0f;
            // publish this plane's y faces and the next plane's H, one barrier
            sW[p][r][lane] = wyn;
            if (CHECK) sU[p][r][lane] = uy;
            sH[p ^ 1][r][lane] = Hn;
            sF[p ^ 1][r][lane] = MODEL == LINSTEP ? dnf : hn;
            if (MODEL == LINSTEP) sD[p ^ 1][r][lane] = Dn;
            __syncthreads();
            if (upd) {
                const T wyb = sW[p][r - 1][lane];
                const float dmax = MODEL == LINSTEP ? fmaxf(fmaxf(fmaxf(dcf, dlf), fmaxf(N::lo_f(Dr), duf)),
                                                            fmaxf(fmaxf(ddf, dbf), dnf))
                                                    : 0.0f;
                const float e = cell_e<MODEL>(a, hc, dmax);
                const T div = N::mad(N::sub(wzn, wzb), cst<N>(a, 2),
                                     N::mad(N::sub(wyn, wyb), cst<N>(a, 1), N::mul(N::sub(wxn, wxl), cst<N>(a, 0))));
                const T Hnew = h_update<N>(a, Hc, Ho, div, e);
                st<N>(a.Hout, idx, Hnew);
                if (CHECK) {
                    const T uyb = sU[p][r - 1][lane];
                    const T divu = N::mad(N::sub(uz, uzb), cst<N>(a, 2),
                                          N::mad(N::sub(uy, uyb), cst<N>(a, 1), N::mul(N::sub(ux, uxl), cst<N>(a, 0))));
                    const T r2 = N::sub(divu, N::mul(N::sub(Hnew, Ho), cst<N>(a, 3)));
                    accumulate_residual(N::to_d(r2), part, pmax);
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
template <class N, int MODEL>
__global__ void __launch_bounds__(256) resid_consistent_kernel(PTArgs a, int ndim)
{
    using T = typename N::T;
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
        const long long stp[3] = {1, a.sy, a.sz};
        const T H = ld<N>(a.Hout, c);
        T div = N::zero();
        for (int d = 0; d < ndim; ++d) {
            const T HR = ld<N>(a.Hout, c + stp[d]), HL = ld<N>(a.Hout, c - stp[d]);
            T uR, uL;
            if (MODEL == LIN) {
                uR = N::sub(HR, H);
                uL = N::sub(H, HL);
            } else if (MODEL == LINSTEP) {
                const T Dc = ld<N>(a.D, c);
                uR = N::mul(N::add(Dc, ld<N>(a.D, c + stp[d])), N::sub(HR, H));
                uL = N::mul(N::add(ld<N>(a.D, c - stp[d]), Dc), N::sub(H, HL));
            } else {
                const T sR = N::add(H, HR), sL = N::add(HL, H);
                uR = N::mul(N::mul(N::mul(sR, sR), sR), N::sub(HR, H));
                uL = N::mul(N::mul(N::mul(sL, sL), sL), N::sub(H, HL));
            }
            div = N::mad(N::sub(uR, uL), cst<N>(a, d), div);
        }
        const T r = N::sub(div, N::mul(N::sub(H, ld<N>(a.Hold, c)), cst<N>(a, 3)));
        accumulate_residual(N::to_d(r), part, pmax);
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

// FP64 <-> DF64 conversion of whole fields (host boundary only).
__global__ void to_df64_kernel(const double* src, float2* dst, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        dst[t] = split_df(src[t]);
}

__global__ void from_df64_kernel(const float2* src, double* dst, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        dst[t] = (double)src[t].x + (double)src[t].y;
}

// ---------------------------------------------------------------------------
template <class N, int MODEL, bool CHECK>
static cudaError_t launch_model(const PTArgs& a, int ndim, const LaunchCfg& cfg, cudaStream_t s)
{
    if (ndim == 1) {
        const int bs = 256;
        pt1d_kernel<N, MODEL, CHECK><<<(a.nx + bs - 1) / bs, bs, 0, s>>>(a);
    } else if (ndim == 2) {
        const int W = cfg.warps2d;
        const int tiles = (a.nx - 2 + 30) / 31;
        dim3 grid((tiles + W - 1) / W, (a.ny - 2 + cfg.chunk2d - 1) / cfg.chunk2d);
        pt2d_kernel<N, MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, cfg.chunk2d);
    } else {
        const int tx = (a.nx - 2 + 30) / 31;
        const int nzc = (a.nz - 2 + cfg.chunk3d - 1) / cfg.chunk3d;
        if (cfg.rows3d == 8) {
            dim3 grid(tx, (a.ny - 2 + 6) / 7, nzc);
            pt3d_kernel<N, MODEL, CHECK, 8><<<grid, dim3(32, 8), 0, s>>>(a, cfg.chunk3d);
        } else {
            dim3 grid(tx, (a.ny - 2 + 14) / 15, nzc);
            pt3d_kernel<N, MODEL, CHECK, 16><<<grid, dim3(32, 16), 0, s>>>(a, cfg.chunk3d);
        }
    }
    return cudaGetLastError();
}

template <class N>
static cudaError_t launch_type(const PTArgs& a, int ndim, int model, bool check, const LaunchCfg& cfg,
                               cudaStream_t s)
{
    switch (model * 2 + (check ? 1 : 0)) {
    case 0: return launch_model<N, LIN, false>(a, ndim, cfg, s);
    case 1: return launch_model<N, LIN, true>(a, ndim, cfg, s);
    case 2: return launch_model<N, LINSTEP, false>(a, ndim, cfg, s);
    case 3: return launch_model<N, LINSTEP, true>(a, ndim, cfg, s);
    case 4: return launch_model<N, NONLIN, false>(a, ndim, cfg, s);
    case 5: return launch_model<N, NONLIN, true>(a, ndim, cfg, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_pt(const PTArgs& a, int ndim, int model, bool check, bool df64, const LaunchCfg& cfg,
                      cudaStream_t s)
{
    return df64 ? launch_type<DF64>(a, ndim, model, check, cfg, s) : launch_type<F64>(a, ndim, model, check, cfg, s);
}

cudaError_t launch_resid_consistent(const PTArgs& a, int ndim, int model, bool df64, cudaStream_t s)
{
    const int bs = 256, nb = 152 * 8;
    if (df64) {
        if (model == LIN) resid_consistent_kernel<DF64, LIN><<<nb, bs, 0, s>>>(a, ndim);
        else if (model == LINSTEP) resid_consistent_kernel<DF64, LINSTEP><<<nb, bs, 0, s>>>(a, ndim);
        else resid_consistent_kernel<DF64, NONLIN><<<nb, bs, 0, s>>>(a, ndim);
    } else {
        if (model == LIN) resid_consistent_kernel<F64, LIN><<<nb, bs, 0, s>>>(a, ndim);
        else if (model == LINSTEP) resid_consistent_kernel<F64, LINSTEP><<<nb, bs, 0, s>>>(a, ndim);
        else resid_consistent_kernel<F64, NONLIN><<<nb, bs, 0, s>>>(a, ndim);
    }
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

cudaError_t launch_to_df64(const double* src, void* dst, long long n, cudaStream_t s)
{
    to_df64_kernel<<<152 * 8, 256, 0, s>>>(src, reinterpret_cast<float2*>(dst), n);
    return cudaGetLastError();
}

cudaError_t launch_from_df64(const void* src, double* dst, long long n, cudaStream_t s)
{
    from_df64_kernel<<<152 * 8, 256, 0, s>>>(reinterpret_cast<const float2*>(src), dst, n);
    return cudaGetLastError();
}

}  // namespace ptd
