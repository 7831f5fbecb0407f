// ptd_adjoint.cu -- discrete adjoint of the implicit PT solve (3D, D = exp(m) H^3
// or D = H^3): gradient of L = 1/2 sum_inner (H^nt - H_target)^2 with respect
// to the per-cell log-coefficient m and the initial state H0.
//
// No reference counterpart (the reference has no adjoint); this is new work
// checked against central finite differences and the CPU FP64 reference
// adjoint of oracle/ptd_oracle.c.
//
// Per physical step n = nt..1 the forward residual is (scaled as in
// ptd_device.cuh) F_i = (H_i - Hold_i)/dt - sum_d sigma_d (u_{i+1/2} - u_{i-1/2}),
// u_f = K_f (H_R - H_L), K_f = (E_L + E_R) s^3, s = H_L + H_R, E = exp(m).
// The adjoint state solves J^T lam = g with J = dF/dH at the converged H^n:
//   (J^T lam)_j = lam_j/dt + sum_d sigma_d [ (w_{j+1/2} - w_{j-1/2})      -- symmetric part,
//                                            + (n_{j+1/2} + n_{j-1/2}) ]   -- transposed Newton term
// with v_f = lam_R - lam_L, w_f -> -K_f v_f (damped exactly like the forward
// flux) and n_f = 3 (E_L+E_R) s^2 (H_R - H_L) v_f (the 3H^2 derivative of
// D = H^3, transposed).  The transposed stencil is iterated with the same
// accelerated PT scheme and parameters as the forward (one fused kernel per
// iteration, z-march, device-side checks), then
//   dL/dm_j  -= sum_{f ∋ j} sigma v_f E_j s^3 (H_R - H_L)
//   dL/dH0_b -= sum_{f ∋ b} sigma v_f du_f/dH_b      (boundary cells: frozen at H0)
//   g <- lam / dt                                    (dL/dH^{n-1})
// and after step 1 dL/dH0 (inner cells) = g.  The forward keeps one FP64
// checkpoint of H per physical step; the adjoint sweep needs no recomputation.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "ptd_internal.h"
#include "ptd_pt_body.cuh"

namespace ptd {

struct AdjArgs {
    int nx, ny, nz;
    long long sy, sz;
    double rdt;
    double sig[3];
    float2 rdt_df;
    float2 sig_df[3];
    FParams f;
    const void* lin;    // lam (iteration k)
    void* lout;         // lam (iteration k+1)
    const void* win[3];
    void* wout[3];
    const void* H;      // H^n (frozen, number type of the kernel)
    const void* E;      // exp(m) (number type of the kernel); NULL for D = H^3
    const void* g;      // right-hand side
    const int* done;
    double* acc;
};

// done: 1 converged (err <= target), 2 itmax, 3 stalled at an arithmetic
// floor below the acceptable level (err <= accept, no 1 % improvement over
// `stall` checks)
struct AdjState {
    int done, nchecks, iter, best_at;
    double acc, err, target, accept, best;
};

template <class N>
__device__ __forceinline__ typename N::T acst(const AdjArgs& a, int which);
template <>
__device__ __forceinline__ double acst<F64>(const AdjArgs& a, int which)
{
    return which < 3 ? a.sig[which] : a.rdt;
}
template <>
__device__ __forceinline__ float2 acst<DF64>(const AdjArgs& a, int which)
{
    return which < 3 ? a.sig_df[which] : a.rdt_df;
}

// One adjoint face: damped symmetric flux, and the Newton-transpose value n.
// kv = K v (undamped, for the check).
template <class N, bool EXPM, bool U>
__device__ __forceinline__ typename N::T adj_face(const AdjArgs& a, typename N::T HL, typename N::T HR, float hsum,
                                                  typename N::T EL, typename N::T ER, typename N::T lL,
                                                  typename N::T lR, typename N::T w, typename N::T& n,
                                                  typename N::T& kv)
{
    using T = typename N::T;
    const T v = N::sub(lR, lL);
    const T s = N::add(HL, HR);
    const T s2 = N::mul(s, s);
    T K = N::mul(s2, s);
    T Kp = N::add(N::add(s2, s2), s2);   // K' = 3 s^2 (times E_L + E_R)
    float efac = 1.0f;
    if (EXPM) {
        const T e2 = N::add(EL, ER);
        K = N::mul(K, e2);
        Kp = N::mul(Kp, e2);
        efac = 0.5f * N::lo_f(e2);
    } else {
        // D = H^3 is the EXPM form with E = 1: (E_L + E_R) = 2, kappa 1/16
        K = N::add(K, K);
        Kp = N::add(Kp, Kp);
    }
    n = N::mul(N::mul(Kp, N::sub(HR, HL)), v);
    const T kvv = N::mul(K, v);
    if (U) kv = kvv;
    const float c = nonlin_face_c(a.f, hsum, efac);
    return nmadf(N(), c, N::add(w, kvv), w);
}

template <class N, bool EXPM, bool CHECK, int R>
__global__ void __launch_bounds__(32 * R) adj3d_kernel(const AdjArgs* __restrict__ ap, int chunk)
{
    using T = typename N::T;
    const AdjArgs a = *ap;
    if (step_done(a.done)) return;
    __shared__ T sL[2][R][32];     // lam of the plane
    __shared__ T sH[2][R][32];     // H of the plane
    __shared__ T sE[EXPM ? 2 : 1][EXPM ? R : 1][32];
    __shared__ T sW[2][R][32];     // y faces: damped flux
    __shared__ T sN[2][R][32];     // y faces: Newton-transpose value
    __shared__ T sK[CHECK ? 2 : 1][CHECK ? R : 1][32];

    const int lane = threadIdx.x, r = threadIdx.y;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int i = 31 * blockIdx.x + lane;
    const int j = (R - 1) * blockIdx.y + r;
    const int k0 = 1 + blockIdx.z * chunk;
    const int k1 = min(k0 + chunk, nz - 1);
    double part = 0.0;
    unsigned long long pmax = 0ull;
    if (k0 < k1) {
        const int ic = min(i, nx - 1), jc = min(j, ny - 1);
        const bool inner_x = i >= 1 && i <= nx - 2, inner_y = j >= 1 && j <= ny - 2;
        const bool xface = i <= nx - 2 && inner_y && r >= 1;
        const bool yface = j <= ny - 2 && inner_x;
        const bool upd = inner_x && inner_y && lane >= 1 && r >= 1;
        const bool own_x = xface && (lane >= 1 || blockIdx.x == 0);
        const bool own_y = yface && lane >= 1 && (r >= 1 || blockIdx.y == 0);
        const bool top = r == R - 1, up_ok = jc + 1 < ny;
        const long long sy = a.sy, sz = a.sz;
        long long idx = (long long)k0 * sz + (long long)jc * sy + ic;
        T lc = ld<N>(a.lin, idx), Hc = ld<N>(a.H, idx);
        T Ec = EXPM ? ld<N>(a.E, idx) : N::zero();
        float hc = N::lo_f(Hc);
        T wzb = N::zero(), nzb = N::zero(), kzb = N::zero();
        if (upd) {
            const T lb = ld<N>(a.lin, idx - sz), Hb = ld<N>(a.H, idx - sz);
            const T Eb = EXPM ? ld<N>(a.E, idx - sz) : N::zero();
            wzb = adj_face<N, EXPM, CHECK>(a, Hb, Hc, N::lo_f(Hb) + hc, Eb, Ec, lb, lc, ld<N>(a.win[2], idx - sz),
                                           nzb, kzb);
            if (k0 == 1) st<N>(a.wout[2], idx - sz, wzb);
        }
        int p = 0;
        sL[0][r][lane] = lc;
        sH[0][r][lane] = Hc;
        if (EXPM) sE[0][r][lane] = Ec;
        __syncthreads();
        for (int k = k0; k < k1; ++k, idx += sz) {
            const T ln = ld<N>(a.lin, idx + sz), Hn = ld<N>(a.H, idx + sz);
            const T En = EXPM ? ld<N>(a.E, idx + sz) : N::zero();
            const T wx = ld<N>(a.win[0], idx), wy = ld<N>(a.win[1], idx), wz = ld<N>(a.win[2], idx);
            const T gg = ld<N>(a.g, idx);
            T lu, Hu, Eu = N::zero();
            if (!top) {
                lu = sL[p][r + 1][lane];
                Hu = sH[p][r + 1][lane];
                if (EXPM) Eu = sE[p][r + 1][lane];
            } else {
                lu = up_ok ? ld<N>(a.lin, idx + sy) : lc;
                Hu = up_ok ? ld<N>(a.H, idx + sy) : Hc;
                if (EXPM) Eu = up_ok ? ld<N>(a.E, idx + sy) : Ec;
            }
            T lr = N::shfl_down(lc, 1), Hr = N::shfl_down(Hc, 1);
            T Er = EXPM ? N::shfl_down(Ec, 1) : N::zero();
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                lr = ok ? ld<N>(a.lin, idx + 1) : lc;
                Hr = ok ? ld<N>(a.H, idx + 1) : Hc;
                if (EXPM) Er = ok ? ld<N>(a.E, idx + 1) : Ec;
            }
            T nx_ = N::zero(), ny_ = N::zero(), nz_ = N::zero();
            T kx = N::zero(), ky = N::zero(), kz = N::zero();
            T wxn = N::zero(), wyn = N::zero(), wzn = N::zero();
            if (xface) wxn = adj_face<N, EXPM, CHECK>(a, Hc, Hr, hc + N::lo_f(Hr), Ec, Er, lc, lr, wx, nx_, kx);
            if (yface) wyn = adj_face<N, EXPM, CHECK>(a, Hc, Hu, hc + N::lo_f(Hu), Ec, Eu, lc, lu, wy, ny_, ky);
            if (upd) wzn = adj_face<N, EXPM, CHECK>(a, Hc, Hn, hc + N::lo_f(Hn), Ec, En, lc, ln, wz, nz_, kz);
            if (own_x) st<N>(a.wout[0], idx, wxn);
            if (own_y) st<N>(a.wout[1], idx, wyn);
            if (upd) st<N>(a.wout[2], idx, wzn);
            const T wxl = N::shfl_up(wxn, 1), nxl = N::shfl_up(nx_, 1);
            const T kxl = CHECK ? N::shfl_up(kx, 1) : N::zero();
            sW[p][r][lane] = wyn;
            sN[p][r][lane] = ny_;
            if (CHECK) sK[p][r][lane] = ky;
            sL[p ^ 1][r][lane] = ln;
            sH[p ^ 1][r][lane] = Hn;
            if (EXPM) sE[p ^ 1][r][lane] = En;
            __syncthreads();
            if (upd) {
                const T wyb = sW[p][r - 1][lane], nyb = sN[p][r - 1][lane];
                const float e = nonlin_cell_e(a.f, hc, EXPM ? N::lo_f(Ec) : 1.0f);
                // sum_d sigma_d [(w_+ - w_-) + (n_+ + n_-)]
                T div = N::mul(N::add(N::sub(wxn, wxl), N::add(nx_, nxl)), acst<N>(a, 0));
                div = N::mad(N::add(N::sub(wyn, wyb), N::add(ny_, nyb)), acst<N>(a, 1), div);
                div = N::mad(N::add(N::sub(wzn, wzb), N::add(nz_, nzb)), acst<N>(a, 2), div);
                const T A = N::sub(N::mad(lc, acst<N>(a, 3), div), gg);
                const T lnew = nmadf(N(), e, A, lc);
                st<N>(a.lout, idx, lnew);
                if (CHECK) {
                    const T kyb = sK[p][r - 1][lane];
                    // R = g - lam rdt + sum sigma [(kv_+ - kv_-) - (n_+ + n_-)]
                    T q = N::mul(N::sub(N::sub(kx, kxl), N::add(nx_, nxl)), acst<N>(a, 0));
                    q = N::mad(N::sub(N::sub(ky, kyb), N::add(ny_, nyb)), acst<N>(a, 1), q);
                    q = N::mad(N::sub(N::sub(kz, kzb), N::add(nz_, nzb)), acst<N>(a, 2), q);
                    const T res = N::add(N::sub(gg, N::mul(lnew, acst<N>(a, 3))), q);
                    accumulate_residual(N::to_d(res), part, pmax);
                }
            }
            lc = ln;
            Hc = Hn;
            hc = N::lo_f(Hn);
            if (EXPM) Ec = En;
            wzb = wzn;
            nzb = nz_;
            kzb = kz;
            p ^= 1;
        }
    }
    if (CHECK) block_reduce_residual(a.acc, 0, part, pmax);
}

// Gradient accumulation of one step (FP64, one thread per cell of the whole
// grid) and the next right-hand side g = lam/dt.
template <class N, bool EXPM>
__global__ void __launch_bounds__(256) adj_grad_kernel(AdjArgs a, const double* Hn, const double* Ed, double* gm,
                                                       double* gh, void* g_next, long long total_cells)
{
    const long long stp[3] = {1, a.sy, a.sz};
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total_cells;
         t += (long long)gridDim.x * blockDim.x) {
        const long long ix = t % a.nx, iy = (t / a.nx) % a.ny, iz = t / ((long long)a.nx * a.ny);
        const long long c = iz * a.sz + iy * a.sy + ix;
        const long long id[3] = {ix, iy, iz};
        const int n[3] = {a.nx, a.ny, a.nz};
        auto inner = [&](long long cc, int dd, int side) -> bool {
            long long q[3] = {id[0], id[1], id[2]};
            q[dd] += side;
            for (int e = 0; e < 3; ++e)
                if (q[e] < 1 || q[e] > n[e] - 2) return false;
            (void)cc;
            return true;
        };
        const bool ci = inner(c, 0, 0);
        const double lamc = ci ? N::to_d(ld<N>(a.lin, c)) : 0.0;
        double dm = 0.0, dh = 0.0;
        const double Hc = Hn[c];
        const double Ec = EXPM ? Ed[c] : 1.0;
        for (int d = 0; d < 3; ++d) {
            for (int side = -1; side <= 1; side += 2) {
                const long long q[3] = {id[0] + (d == 0 ? side : 0), id[1] + (d == 1 ? side : 0),
                                        id[2] + (d == 2 ? side : 0)};
                if (q[d] < 0 || q[d] > n[d] - 1) continue;
                const long long o = c + side * stp[d];
                // a face exists in the reference only between cells whose
                // other coordinates are inner
                bool face_ok = true;
                for (int e = 0; e < 3; ++e)
                    if (e != d && (id[e] < 1 || id[e] > n[e] - 2)) face_ok = false;
                if (!face_ok) continue;
                const bool oi = inner(o, d, side);
                const double lamo = oi ? N::to_d(ld<N>(a.lin, o)) : 0.0;
                const double Ho = Hn[o];
                const double Eo = EXPM ? Ed[o] : 1.0;
                // orient the face: L = lower index
                const double HL = side > 0 ? Hc : Ho, HR = side > 0 ? Ho : Hc;
                const double lL = side > 0 ? lamc : lamo, lR = side > 0 ? lamo : lamc;
                const double e2 = side > 0 ? Ec + Eo : Eo + Ec;
                const double s = HL + HR, gH = HR - HL, v = lR - lL;
                const double sv = a.sig[d] * v;
                if (EXPM) dm -= sv * Ec * s * s * s * gH;
                if (!ci) {
                    const double K = e2 * s * s * s, Kp = 3.0 * e2 * s * s;
                    const double du = side > 0 ? (-K + Kp * gH) : (K + Kp * gH);   // this cell is L (side>0) or R
                    dh -= sv * du;
                }
            }
        }
        if (EXPM) gm[c] += dm;
        if (!ci) gh[c] += dh;
        // next right-hand side
        if (ci) {
            const double gn = lamc * a.rdt;
            if (N::native) reinterpret_cast<double*>(g_next)[c] = gn;
            else reinterpret_cast<float2*>(g_next)[c] = split_df(gn);
        }
    }
}

__global__ void adj_target_kernel(AdjState* st, double rtol, double accept_rtol, double norm_den,
                                  double floor_abs)
{
    const double gn = sqrt(st->acc) / sqrt(norm_den);
    st->acc = 0.0;
    st->target = fmax(rtol * gn, floor_abs);
    st->accept = fmax(accept_rtol * gn, floor_abs);
    st->done = gn == 0.0 ? 1 : 0;
    st->nchecks = 0;
    st->iter = 0;
    st->err = gn;
    st->best = gn;
    st->best_at = 0;
}

__global__ void adj_judge_kernel(AdjState* st, int nchk, int itmax, double norm_den, int stall)
{
    if (st->done) return;
    const double err = sqrt(st->acc) / sqrt(norm_den);
    st->acc = 0.0;
    st->err = err;
    st->nchecks += 1;
    st->iter += nchk;
    if (err < 0.99 * st->best) {
        st->best = err;
        st->best_at = st->nchecks;
    }
    if (!(err > st->target)) st->done = 1;
    else if (err != err) st->done = 2;
    else if (st->nchecks - st->best_at >= stall && err <= st->accept) st->done = 3;
    else if (st->iter + nchk > itmax) st->done = 2;
}

// sum over inner cells of v^2 (v as N::T) into acc; loss uses the FP64 variant.
template <class N>
__global__ void __launch_bounds__(256) adj_sumsq_kernel(const void* v, double* acc, int nx, int ny, int nz,
                                                        long long sy, long long sz)
{
    const long long nix = nx - 2, niy = ny - 2, niz = nz - 2, total = nix * niy * niz;
    double part = 0.0;
    unsigned long long pm = 0ull;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long ix = 1 + t % nix, iy = 1 + (t / nix) % niy, iz = 1 + t / (nix * niy);
        const double x = N::to_d(ld<N>(v, iz * sz + iy * sy + ix));
        part = fma(x, x, part);
    }
    block_reduce_residual(acc, 0, part, pm);
}

__global__ void __launch_bounds__(256) adj_misfit_kernel(const double* HN, const double* Ht, void* g, double* acc,
                                                         int nx, int ny, int nz, long long sy, long long sz, int df64)
{
    const long long nix = nx - 2, niy = ny - 2, niz = nz - 2, total = nix * niy * niz;
    double part = 0.0;
    unsigned long long pm = 0ull;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long ix = 1 + t % nix, iy = 1 + (t / nix) % niy, iz = 1 + t / (nix * niy);
        const long long c = iz * sz + iy * sy + ix;
        const double d = HN[c] - Ht[c];
        part = fma(d, d, part);
        if (g) {
            if (df64) reinterpret_cast<float2*>(g)[c] = split_df(d);
            else reinterpret_cast<double*>(g)[c] = d;
        }
    }
    block_reduce_residual(acc, 0, part, pm);
}

__global__ void expd_kernel(const double* m, double* E, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        E[t] = exp(m[t]);
}

}  // namespace ptd

using namespace ptd;

struct ptd_adj {
    ptd_params p;
    ptd_ctx* fwd = nullptr;
    ptd_ctx_base g;
    Derived dv;
    LaunchCfg cfg;
    cudaStream_t s = nullptr;
    bool df64 = false, expm = false;
    double* ck = nullptr;       // (nt+1) FP64 checkpoints
    double* Ht = nullptr;       // target (FP64, padded)
    double* Ed = nullptr;       // exp(m) FP64
    void* E = nullptr;          // exp(m) in the kernel number type
    void* Hk = nullptr;         // H^n in the kernel number type
    void* lam[2] = {nullptr, nullptr};
    void* w[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    void* gbuf = nullptr;       // right-hand side
    double* gm = nullptr;
    double* gh = nullptr;
    double* stage = nullptr;
    AdjState* st = nullptr;
    AdjState* h_st = nullptr;
    double* h_acc = nullptr;
    AdjArgs* d_args[2] = {nullptr, nullptr};
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int nchk = 20;
    double rtol = 1e-10;        // adjoint solve target, relative to its right-hand side
    double accept_rtol = 1e-7;  // a solve stalled at an arithmetic floor below this is accepted
    int stall = 10;             // checks without 1 % improvement that count as stalled
    bool have_fwd = false;
    long long launches = 0, iterations = 0;
    std::vector<double> step_err, step_target;   // last adjoint solve: final residual and target per step
    bool any_capped = false;
};

namespace {

#define ACK(call)                                                 \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);       \
    } while (0)

cudaError_t adj_launch(ptd_adj* A, int par, bool check)
{
    const dim3 blk(32, 16);
    const int tx = (A->g.nx - 2 + 30) / 31, ty = (A->g.ny - 2 + 14) / 15;
    const int ch = A->cfg.chunk3d;
    const dim3 grid(tx, ty, (A->g.nz - 2 + ch - 1) / ch);
    const AdjArgs* ap = A->d_args[par];
#define ADJ(NT, EX)                                                                          \
    (check ? adj3d_kernel<NT, EX, true, 16><<<grid, blk, 0, A->s>>>(ap, ch)                   \
           : adj3d_kernel<NT, EX, false, 16><<<grid, blk, 0, A->s>>>(ap, ch))
    if (A->df64) {
        if (A->expm) ADJ(DF64, true);
        else ADJ(DF64, false);
    } else {
        if (A->expm) ADJ(F64, true);
        else ADJ(F64, false);
    }
#undef ADJ
    return cudaGetLastError();
}

void adj_fill(ptd_adj* A, int par, AdjArgs& a)
{
    std::memset(&a, 0, sizeof(a));
    a.nx = A->g.nx;
    a.ny = A->g.ny;
    a.nz = A->g.nz;
    a.sy = A->g.sy;
    a.sz = A->g.sz;
    a.rdt = A->dv.rdt;
    a.rdt_df = split_df(A->dv.rdt);
    for (int d = 0; d < 3; ++d) {
        // the adjoint uses kappa = 1/16 for both models (D = H^3 as E = 1)
        a.sig[d] = 0.0625 / (A->dv.h[d] * A->dv.h[d]);
        a.sig_df[d] = split_df(a.sig[d]);
    }
    a.f = fparams(A->dv);
    a.lin = A->lam[par];
    a.lout = A->lam[par ^ 1];
    for (int d = 0; d < 3; ++d) {
        a.win[d] = A->w[d][par];
        a.wout[d] = A->w[d][par ^ 1];
    }
    a.H = A->Hk;
    a.E = A->expm ? A->E : nullptr;
    a.g = A->gbuf;
    a.done = &A->st->done;
    a.acc = &A->st->acc;
}

int adj_capture(ptd_adj* A)
{
    for (int q = 0; q < 2; ++q) {
        AdjArgs a;
        adj_fill(A, q, a);
        ACK(cudaMemcpy(A->d_args[q], &a, sizeof(a), cudaMemcpyHostToDevice));
    }
    for (int q = 0; q < 2; ++q) {
        cudaGraph_t gr = nullptr;
        ACK(cudaStreamBeginCapture(A->s, cudaStreamCaptureModeThreadLocal));
        cudaError_t err = cudaSuccess;
        int par = q;
        for (int it = 0; it < A->nchk && err == cudaSuccess; ++it) {
            err = adj_launch(A, par, it == A->nchk - 1);
            par ^= 1;
        }
        if (err == cudaSuccess) {
            adj_judge_kernel<<<1, 1, 0, A->s>>>(A->st, A->nchk, A->p.itmax, A->dv.norm_den, A->stall);
            err = cudaGetLastError();
        }
        cudaError_t e2 = cudaStreamEndCapture(A->s, &gr);
        if (err != cudaSuccess) {
            if (gr) cudaGraphDestroy(gr);
            return cuda_fail(err, "adjoint capture");
        }
        if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
        cudaError_t e3 = cudaGraphInstantiate(&A->graph[q], gr, 0);
        cudaGraphDestroy(gr);
        if (e3 != cudaSuccess) return cuda_fail(e3, "cudaGraphInstantiate");
    }
    return PTD_OK;
}

void adj_free(ptd_adj* A)
{
    if (!A) return;
    if (A->s) cudaStreamSynchronize(A->s);
    for (int q = 0; q < 2; ++q)
        if (A->graph[q]) cudaGraphExecDestroy(A->graph[q]);
    if (A->fwd) ptd_destroy(A->fwd);
    void* ptrs[] = {A->ck, A->Ht, A->Ed, A->E, A->Hk, A->lam[0], A->lam[1], A->gbuf, A->gm, A->gh, A->stage,
                    A->st, A->d_args[0], A->d_args[1]};
    for (void* q : ptrs) cudaFree(q);
    for (int d = 0; d < 3; ++d)
        for (int q = 0; q < 2; ++q) cudaFree(A->w[d][q]);
    if (A->h_st) cudaFreeHost(A->h_st);
    delete A;
}

}  // namespace

extern "C" int ptd_adj_create(ptd_adj** out, const ptd_params* p)
{
    if (!out) return set_error(PTD_EINVAL, "ptd_adj_create: out is NULL");
    *out = nullptr;
    int rc = validate(p);
    if (rc) return rc;
    if (p->ndim != 3) return set_error(PTD_EINVAL, "the adjoint solver is 3D");
    if (p->model != PTD_MODEL_NONLIN && p->model != PTD_MODEL_NONLIN_EXPM)
        return set_error(PTD_EINVAL, "the adjoint solver supports D = H^3 and D = exp(m) H^3");
    if (p->precision == PTD_PREC_FP32_DC || p->precision == PTD_PREC_DFH || p->precision == PTD_PREC_FP32_RB)
        return set_error(PTD_EINVAL, "the adjoint runs in FP64 or DF64");
    ptd_adj* A = new (std::nothrow) ptd_adj();
    if (!A) return set_error(PTD_ENOMEM, "adjoint: host allocation failed");
    A->p = *p;
    A->df64 = p->precision == PTD_PREC_DF64;
    A->expm = p->model == PTD_MODEL_NONLIN_EXPM;
    derive(A->p, A->dv);
    A->cfg = tuned_config(A->p);
    {   // stagnation window: ~2 n_max iterations, the PT iteration's own time scale
        const int nmax = std::max(p->nx, std::max(p->ny, p->nz));
        A->stall = std::max(10, (2 * nmax + A->nchk - 1) / A->nchk);
    }
    A->g.nx = p->nx;
    A->g.ny = p->ny;
    A->g.nz = p->nz;
    A->g.sy = ((p->nx + 31) / 32) * 32;
    A->g.sz = A->g.sy * p->ny;
    A->g.nfield = A->g.sz * p->nz;
    ptd_params pf = *p;
    pf.nt = 1;
    rc = ptd_create(&A->fwd, &pf);
    if (rc) {
        adj_free(A);
        return rc;
    }
    A->s = static_cast<cudaStream_t>(ptd_stream(A->fwd));
    const size_t b = (size_t)A->g.nfield * sizeof(double);
    auto al = [&](void** q, size_t n) -> int {
        if (cudaMalloc(q, n) != cudaSuccess) {
            cudaGetLastError();
            return set_error(PTD_ENOMEM, "adjoint: cudaMalloc failed");
        }
        return cudaMemset(*q, 0, n) == cudaSuccess ? PTD_OK : set_error(PTD_ECUDA, "adjoint: cudaMemset failed");
    };
    rc = al((void**)&A->ck, b * (size_t)(p->nt + 1));
    if (!rc) rc = al((void**)&A->Ht, b);
    if (!rc) rc = al((void**)&A->Ed, b);
    if (!rc) rc = al(&A->E, b);
    if (!rc) rc = al(&A->Hk, b);
    for (int q = 0; q < 2 && !rc; ++q) rc = al(&A->lam[q], b);
    for (int d = 0; d < 3 && !rc; ++d)
        for (int q = 0; q < 2 && !rc; ++q) rc = al(&A->w[d][q], b);
    if (!rc) rc = al(&A->gbuf, b);
    if (!rc) rc = al((void**)&A->gm, b);
    if (!rc) rc = al((void**)&A->gh, b);
    if (!rc) rc = al((void**)&A->stage, b);
    if (!rc) rc = al((void**)&A->st, sizeof(AdjState));
    for (int q = 0; q < 2 && !rc; ++q) rc = al((void**)&A->d_args[q], sizeof(AdjArgs));
    if (!rc && cudaMallocHost((void**)&A->h_st, sizeof(AdjState)) != cudaSuccess)
        rc = set_error(PTD_ENOMEM, "adjoint: cudaMallocHost failed");
    if (!rc) rc = adj_capture(A);
    if (rc) {
        adj_free(A);
        return rc;
    }
    *out = A;
    return PTD_OK;
}

extern "C" void ptd_adj_destroy(ptd_adj* A) { adj_free(A); }

static int adj_loss(ptd_adj* A, double* loss)
{
    const double* HN = A->ck + (size_t)A->p.nt * A->g.nfield;
    ACK(cudaMemsetAsync(&A->st->acc, 0, sizeof(double), A->s));
    adj_misfit_kernel<<<152 * 8, 256, 0, A->s>>>(HN, A->Ht, nullptr, &A->st->acc, A->g.nx, A->g.ny, A->g.nz, A->g.sy,
                                                  A->g.sz, 0);
    ACK(cudaGetLastError());
    ACK(cudaMemcpyAsync(A->h_st, A->st, sizeof(AdjState), cudaMemcpyDeviceToHost, A->s));
    ACK(cudaStreamSynchronize(A->s));
    if (loss) *loss = 0.5 * A->h_st->acc;
    return PTD_OK;
}

// Forward solve of nt steps from H0 with log-coefficient m (NULL for D = H^3),
// keeping one FP64 checkpoint per step; L = 1/2 sum_inner (H^nt - Ht)^2.
extern "C" int ptd_adj_forward(ptd_adj* A, const double* H0, const double* m, const double* Ht, double* loss,
                               double* HN, int32_t* iters_per_step)
{
    if (!A || !H0 || !Ht) return set_error(PTD_EINVAL, "ptd_adj_forward: NULL argument");
    if (A->expm && !m) return set_error(PTD_EINVAL, "ptd_adj_forward: m is required");
    int rc = ptd_set_state(A->fwd, H0, m);
    if (rc) return rc;
    const size_t b = (size_t)A->g.nfield * sizeof(double);
    rc = copy_field_in(A->g, A->Ht, Ht, A->s);
    if (rc) return rc;
    if (A->expm) {
        rc = copy_field_in(A->g, A->stage, m, A->s);
        if (rc) return rc;
        expd_kernel<<<152 * 8, 256, 0, A->s>>>(A->stage, A->Ed, A->g.nfield);
        ACK(cudaGetLastError());
        ACK(launch_expm(A->stage, A->E, A->g.nfield, A->df64, A->s));
    }
    ACK(cudaMemsetAsync(A->ck, 0, b, A->s));
    rc = copy_field_in(A->g, A->ck, H0, A->s);
    if (rc) return rc;
    for (int n = 1; n <= A->p.nt; ++n) {
        int32_t it = 0;
        rc = ptd_step(A->fwd, 1, &it, nullptr, 0, nullptr);
        if (rc && rc != PTD_ENOTCONV) return rc;
        if (iters_per_step) iters_per_step[n - 1] = it;
        rc = ctx_current_f64(A->fwd, A->ck + (size_t)n * A->g.nfield);
        if (rc) return rc;
    }
    A->have_fwd = true;
    rc = adj_loss(A, loss);
    if (rc) return rc;
    if (HN) {
        rc = copy_field_out(A->g, HN, A->ck + (size_t)A->p.nt * A->g.nfield, A->s);
        if (rc) return rc;
        ACK(cudaStreamSynchronize(A->s));
    }
    return PTD_OK;
}

// Adjoint sweep over the checkpoints of the last ptd_adj_forward: dL/dm (model
// exp(m) H^3) and dL/dH0 (all cells), each nullable.  adj_iters (nullable,
// nt entries): PT iterations of each adjoint solve, in step order.
extern "C" int ptd_adj_gradient(ptd_adj* A, double* grad_m, double* grad_H0, int32_t* adj_iters)
{
    if (!A) return set_error(PTD_EINVAL, "ptd_adj_gradient: NULL argument");
    if (!A->have_fwd) return set_error(PTD_ESTATE, "ptd_adj_gradient: run ptd_adj_forward first");
    const size_t b = (size_t)A->g.nfield * sizeof(double);
    A->step_err.assign(A->p.nt, 0.0);
    A->step_target.assign(A->p.nt, 0.0);
    A->any_capped = false;
    ACK(cudaMemsetAsync(A->gm, 0, b, A->s));
    ACK(cudaMemsetAsync(A->gh, 0, b, A->s));
    // g = H^nt - Ht on inner cells
    ACK(cudaMemsetAsync(A->gbuf, 0, b, A->s));
    const double* HN = A->ck + (size_t)A->p.nt * A->g.nfield;
    adj_misfit_kernel<<<152 * 8, 256, 0, A->s>>>(HN, A->Ht, A->gbuf, &A->st->acc, A->g.nx, A->g.ny, A->g.nz,
                                                  A->g.sy, A->g.sz, A->df64);
    ACK(cudaGetLastError());
    ACK(cudaMemsetAsync(&A->st->acc, 0, sizeof(double), A->s));
    const long long cells = (long long)A->g.nx * A->g.ny * A->g.nz;
    for (int n = A->p.nt; n >= 1; --n) {
        const double* Hn = A->ck + (size_t)n * A->g.nfield;
        if (A->df64) ACK(launch_to_df64(Hn, A->Hk, A->g.nfield, A->s));
        else ACK(cudaMemcpyAsync(A->Hk, Hn, b, cudaMemcpyDeviceToDevice, A->s));
        for (int q = 0; q < 2; ++q) {
            ACK(cudaMemsetAsync(A->lam[q], 0, b, A->s));
            for (int d = 0; d < 3; ++d) ACK(cudaMemsetAsync(A->w[d][q], 0, b, A->s));
        }
        // target: rtol * ||g||_rms
        if (A->df64)
            adj_sumsq_kernel<DF64><<<152 * 8, 256, 0, A->s>>>(A->gbuf, &A->st->acc, A->g.nx, A->g.ny, A->g.nz,
                                                              A->g.sy, A->g.sz);
        else
            adj_sumsq_kernel<F64><<<152 * 8, 256, 0, A->s>>>(A->gbuf, &A->st->acc, A->g.nx, A->g.ny, A->g.nz,
                                                             A->g.sy, A->g.sz);
        ACK(cudaGetLastError());
        adj_target_kernel<<<1, 1, 0, A->s>>>(A->st, A->rtol, A->accept_rtol, A->dv.norm_den, 1e-300);
        ACK(cudaGetLastError());
        A->launches += 3;
        long long launched = 0, batch = 1;
        const long long blocks_max = std::max(1, A->p.itmax / A->nchk);
        while (launched < blocks_max) {
            const long long k = std::min(batch, blocks_max - launched);
            for (long long j = 0; j < k; ++j) {
                ACK(cudaGraphLaunch(A->graph[(int)(((launched + j) * A->nchk) & 1)], A->s));
                A->launches += A->nchk + 1;
            }
            launched += k;
            ACK(cudaMemcpyAsync(A->h_st, A->st, sizeof(AdjState), cudaMemcpyDeviceToHost, A->s));
            ACK(cudaStreamSynchronize(A->s));
            if (A->h_st->done) break;
            batch = std::min<long long>(batch * 2, 64);
        }
        const int iters = A->h_st->iter;
        A->iterations += iters;
        if (adj_iters) adj_iters[n - 1] = iters;
        A->step_err[n - 1] = A->h_st->err;
        A->step_target[n - 1] = A->h_st->target;
        if (A->h_st->done == 2) A->any_capped = true;   // 3 (stalled below accept_rtol) is accepted
        AdjArgs a;
        adj_fill(A, iters & 1, a);
#define AGK(NT, EX) adj_grad_kernel<NT, EX><<<152 * 8, 256, 0, A->s>>>(a, Hn, A->Ed, A->gm, A->gh, A->gbuf, cells)
        if (A->df64) {
            if (A->expm) AGK(DF64, true);
            else AGK(DF64, false);
        } else {
            if (A->expm) AGK(F64, true);
            else AGK(F64, false);
        }
#undef AGK
        ACK(cudaGetLastError());
        A->launches += 1;
    }
    // dL/dH0 on inner cells = g (lam_1 / dt)
    if (grad_H0) {
        // gh += g on inner cells: fold through the staging field
        if (A->df64) ACK(launch_from_df64(A->gbuf, A->stage, A->g.nfield, A->s));
        else ACK(cudaMemcpyAsync(A->stage, A->gbuf, b, cudaMemcpyDeviceToDevice, A->s));
        ACK(add_fields(A->gh, A->stage, A->g.nfield, A->s));
        int rc = copy_field_out(A->g, grad_H0, A->gh, A->s);
        if (rc) return rc;
    }
    if (grad_m && A->expm) {
        int rc = copy_field_out(A->g, grad_m, A->gm, A->s);
        if (rc) return rc;
    }
    ACK(cudaStreamSynchronize(A->s));
    if ((A->p.flags & PTD_FLAG_STRICT) && A->any_capped)
        return set_error(PTD_ENOTCONV, "ptd_adj_gradient: an adjoint solve reached itmax");
    return PTD_OK;
}

extern "C" int ptd_adj_residuals(ptd_adj* A, double* err, double* target)
{
    if (!A) return set_error(PTD_EINVAL, "adjoint is NULL");
    for (int n = 0; n < A->p.nt; ++n) {
        if (err) err[n] = A->step_err[n];
        if (target) target[n] = A->step_target[n];
    }
    return PTD_OK;
}

extern "C" int ptd_adj_counters(ptd_adj* A, int64_t* launches, int64_t* iterations)
{
    if (!A) return set_error(PTD_EINVAL, "adjoint is NULL");
    int64_t fl = 0, fi = 0;
    ptd_counters(A->fwd, &fl, &fi);
    if (launches) *launches = A->launches + fl;
    if (iterations) *iterations = A->iterations + fi;
    return PTD_OK;
}
