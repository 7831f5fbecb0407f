// ptd_pt_body.cuh -- bodies of the fused PT-iteration kernels, generic over
// the number type (F64, DF64, DFH) and callable with explicit tile indices, so the
// same code serves one grid (ptd_pt.cu) and a batch of grids (ptd_batch.cu).
// See ptd_pt.cu for the algorithm and the tiling.
#pragma once

#include "ptd_device.cuh"
#include "ptd_kernels.h"
#include "ptd_num.cuh"

namespace ptd {

// w - c*t with a float damping coefficient c.
__device__ __forceinline__ double nmadf(F64, float c, double t, double w) { return fma(-f2d_bits(c), t, w); }
__device__ __forceinline__ float2 nmadf(DF64, float c, float2 t, float2 w) { return DF64::nmadf(t, c, w); }

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
__device__ __forceinline__ typename N::T face_t(const PTArgs& a, const typename N::HV& HL,
                                                const typename N::HV& HR, float hsum, typename N::T DL,
                                                typename N::T DR, typename N::T w, typename N::T& u)
{
    using T = typename N::T;
    const T g = N::hdiff(HR, HL);
    if (MODEL == LIN) {
        if (U) u = g;
        return nmadf(N(), a.fc_lin, N::add(g, w), w);
    }
    float c;
    T K;
    if (MODEL == LINSTEP) {
        K = N::add(DL, DR);
        c = a.fc_lin;
    } else if (MODEL == NONLIN) {
        const T s = N::hsum(HL, HR);
        K = N::mul(N::mul(s, s), s);
        c = nonlin_face_c(a.f, hsum);
    } else {   // NONLIN_EXPM: D holds exp(m); K = (E_L + E_R) s^3, kappa = 1/16
        const T s = N::hsum(HL, HR);
        const T e2 = N::add(DL, DR);
        K = N::mul(N::mul(N::mul(s, s), s), e2);
        c = nonlin_face_c(a.f, hsum, 0.5f * N::lo_f(e2));
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

// ---------------------------------------------------------------------------
// Two faces of one cell at once (the double-float forms): the same arithmetic
// as two face_t calls, packed into FP32x2 instructions (DF2, ptd_num.cuh), so
// every component is bit for bit the scalar result.  L is the cell, Ra / Rb
// its neighbours across the two faces.
__device__ __forceinline__ DF2 hdiff2(DF64, float2 L, float2 Ra, float2 Rb)
{
    return df2_sub(df2_pack(Ra, Rb), df2_pack(L, L));
}
__device__ __forceinline__ DF2 hdiff2(DFH, const DFH::HV& L, const DFH::HV& Ra, const DFH::HV& Rb)
{
    // FP64 differences, split with integer operations (DFH::hdiff)
    return df2_pack(split_bits(Ra.d - L.d), split_bits(Rb.d - L.d));
}
__device__ __forceinline__ DF2 hsum2(DF64, float2 L, float2 Ra, float2 Rb)
{
    return df2_add(df2_pack(L, L), df2_pack(Ra, Rb));
}
__device__ __forceinline__ DF2 hsum2(DFH, const DFH::HV& L, const DFH::HV& Ra, const DFH::HV& Rb)
{
    return df2_add(df2_pack(L.f, L.f), df2_pack(Ra.f, Rb.f));
}

template <class N, int MODEL, bool U>
__device__ __forceinline__ DF2 face2_t(const PTArgs& a, const typename N::HV& HL, const typename N::HV& HRa,
                                       const typename N::HV& HRb, float hsa, float hsb, float2 DL, float2 DRa,
                                       float2 DRb, const DF2& w, DF2& u)
{
    const DF2 g = hdiff2(N(), HL, HRa, HRb);
    if (MODEL == LIN) {
        if (U) u = g;
        return df2_nmadf(df2_add(g, w), f2(a.fc_lin), w);
    }
    float2 c;
    DF2 K;
    if (MODEL == LINSTEP) {
        K = df2_add(df2_pack(DL, DL), df2_pack(DRa, DRb));
        c = f2(a.fc_lin);
    } else if (MODEL == NONLIN) {
        const DF2 s = hsum2(N(), HL, HRa, HRb);
        K = df2_mul(df2_mul(s, s), s);
        c = f2(nonlin_face_c(a.f, hsa), nonlin_face_c(a.f, hsb));
    } else {   // NONLIN_EXPM
        const DF2 s = hsum2(N(), HL, HRa, HRb);
        const DF2 e2 = df2_add(df2_pack(DL, DL), df2_pack(DRa, DRb));
        K = df2_mul(df2_mul(df2_mul(s, s), s), e2);
        c = f2(nonlin_face_c(a.f, hsa, 0.5f * e2.hi.x), nonlin_face_c(a.f, hsb, 0.5f * e2.hi.y));
    }
    DF2 t;
    if (U) {
        u = df2_mul(K, g);
        t = df2_add(u, w);
    } else {
        t = df2_mad(K, g, w);
    }
    return df2_nmadf(t, c, w);
}

template <class N>
__device__ __forceinline__ typename N::T cst(const PTArgs& a, int which);
// which: 0..2 sigma_d, 3 rdt, 4 rdt/sigma (square cells)
template <>
__device__ __forceinline__ double cst<F64>(const PTArgs& a, int which)
{
    return which < 3 ? a.sig[which] : (which == 3 ? a.rdt : a.rdt_sig);
}
template <>
__device__ __forceinline__ float2 cst<DF64>(const PTArgs& a, int which)
{
    return which < 3 ? a.sig_df[which] : (which == 3 ? a.rdt_df : a.rdt_sig_df);
}
template <>
__device__ __forceinline__ float2 cst<DFH>(const PTArgs& a, int which)
{
    return which < 3 ? a.sig_df[which] : (which == 3 ? a.rdt_df : a.rdt_sig_df);
}

template <int MODEL>
struct ModelTraits {
    static constexpr bool hasd = MODEL == LINSTEP || MODEL == NONLIN_EXPM;   // a per-cell field in a.D
};

template <int MODEL>
__device__ __forceinline__ float cell_e(const PTArgs& a, float h, float dmax)
{
    if (MODEL == LIN) return a.fe_lin;
    if (MODEL == LINSTEP) return linstep_cell_e(a.f, dmax);
    if (MODEL == NONLIN_EXPM) return nonlin_cell_e(a.f, h, dmax);   // dmax carries exp(m) of the cell
    return nonlin_cell_e(a.f, h);
}

// H_new = H - e*((H - Hold)/dt + div)
template <class N>
__device__ __forceinline__ typename N::HS h_update(const PTArgs& a, const typename N::HV& Hc, typename N::HS Ho,
                                                   typename N::T div, float e)
{
    const typename N::T Rp = N::mad(N::hdo(Hc, Ho), cst<N>(a, 3), div);
    return N::hstep(Hc, Rp, e);
}

// The same for square cells from the undivided flux differences:
// H_new = H - (e sigma)*((H - Hold) rdt/sigma + sum_d (w_R - w_L)).
template <class N>
__device__ __forceinline__ typename N::HS h_update_sq(const PTArgs& a, const typename N::HV& Hc, typename N::HS Ho,
                                                      typename N::T dsum, float e)
{
    const typename N::T Rp = N::mad(N::hdo(Hc, Ho), cst<N>(a, 4), dsum);
    return N::hstep(Hc, Rp, e * a.fsig);
}

// ---------------------------------------------------------------------------
// 1D: one thread per cell; the left face is recomputed (1D grids are small).
template <class N, int MODEL, bool CHECK>
__device__ __forceinline__ void pt1d_body(const PTArgs& a, int bx, double& part, unsigned long long& pmax)
{
    using T = typename N::T;
    using HV = typename N::HV;
    using HS = typename N::HS;
    const int i = bx * blockDim.x + threadIdx.x;
    const int nx = a.nx;
    if (i < nx) {
        const HV Hc = N::ldh(a.Hin, i);
        const float hc = N::hf(Hc);
        constexpr bool HASD = ModelTraits<MODEL>::hasd;
        const T Dc = HASD ? ld<N>(a.D, i) : N::zero();
        T wr = N::zero(), ur = N::zero(), Dr = N::zero();
        if (i <= nx - 2) {
            const HV Hr = N::ldh(a.Hin, i + 1);
            if (HASD) Dr = ld<N>(a.D, i + 1);
            wr = face_t<N, MODEL, CHECK>(a, Hc, Hr, hc + N::hf(Hr), Dc, Dr, ld<N>(a.win[0], i), ur);
            st<N>(a.wout[0], i, wr);
        }
        if (i >= 1 && i <= nx - 2) {
            const HV Hl = N::ldh(a.Hin, i - 1);
            const T Dl = HASD ? ld<N>(a.D, i - 1) : N::zero();
            T ul = N::zero();
            const T wl = face_t<N, MODEL, CHECK>(a, Hl, Hc, N::hf(Hl) + hc, Dl, Dc, ld<N>(a.win[0], i - 1), ul);
            const HS Ho = N::ldo(a.Hold, i);
            const float e = cell_e<MODEL>(a, hc, MODEL == NONLIN_EXPM ? N::lo_f(Dc)
                                                 : fmaxf(fmaxf(N::lo_f(Dl), N::lo_f(Dr)), N::lo_f(Dc)));
            const HS Hn = h_update_sq<N>(a, Hc, Ho, N::sub(wr, wl), e);   // one dimension: sigma is the only one
            N::sth(a.Hout, i, Hn);
            if (CHECK) {
                const T r = N::sub(N::mul(N::sub(ur, ul), cst<N>(a, 0)), N::mul(N::hdn(Hn, Ho), cst<N>(a, 3)));
                accumulate_residual(N::to_d(r), part, pmax);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// 2D: blockDim = (32, W); warp w of block b owns the x strip of tile
// t = b*W + w: cells i = 31t + lane (lane 0 = left neighbour), and marches
// rows j0 .. j1-1 of y chunk cy.
// slot: the warp's slot in a.parts (when a.parts is set).
template <class N, int MODEL, bool CHECK>
__device__ __forceinline__ void pt2d_body(const PTArgs& a, int tile, int cy, int chunk, double& part,
                                          unsigned long long& pmax, long long slot = 0)
{
    using T = typename N::T;
    using HV = typename N::HV;
    using HS = typename N::HS;
    const int lane = threadIdx.x;
    const int i = 31 * tile + lane;
    const int nx = a.nx, ny = a.ny;
    const int j0 = 1 + cy * chunk;
    const int j1 = min(j0 + chunk, ny - 1);
    const bool warp_active = (31 * tile < nx - 1) && (j0 < j1);
    if (warp_active) {
        const int ic = min(i, nx - 1);
        const bool xface = i <= nx - 2;
        const bool inner_x = i >= 1 && i <= nx - 2;
        const bool upd = inner_x && lane >= 1;
        const bool own_x = xface && (lane >= 1 || tile == 0);
        const long long sy = a.sy;
        long long idx = (long long)j0 * sy + ic;

        constexpr bool HASD = ModelTraits<MODEL>::hasd;
        HV Hc = N::ldh(a.Hin, idx);
        float hc = N::hf(Hc);
        T Dc = HASD ? ld<N>(a.D, idx) : N::zero();
        float dcf = MODEL == LINSTEP ? N::lo_f(Dc) : 0.0f;
        float dbf = 0.0f;
        T wyb = N::zero(), uyb = N::zero();
        if (upd) {
            // face (j0 - 1/2), owned by the chunk below unless j0 == 1
            const HV Hb = N::ldh(a.Hin, idx - sy);
            const T Db = HASD ? ld<N>(a.D, idx - sy) : N::zero();
            dbf = MODEL == LINSTEP ? N::lo_f(Db) : 0.0f;
            wyb = face_t<N, MODEL, CHECK>(a, Hb, Hc, N::hf(Hb) + hc, Db, Dc, ld<N>(a.win[1], idx - sy), uyb);
            if (j0 == 1) st<N>(a.wout[1], idx - sy, wyb);
        }
        for (int j = j0; j < j1; ++j, idx += sy) {
            const HV Hn = N::ldh(a.Hin, idx + sy);
            const T wx = ld<N>(a.win[0], idx);
            const T wy = ld<N>(a.win[1], idx);
            const HS Ho = N::ldo(a.Hold, idx);
            const T Dn = HASD ? ld<N>(a.D, idx + sy) : N::zero();
            HV Hr = N::shfl_down_h(Hc, 1);
            float hr = __shfl_down_sync(FULL, hc, 1);
            T Dr = HASD ? N::shfl_down(Dc, 1) : N::zero();
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                Hr = ok ? N::ldh(a.Hin, idx + 1) : Hc;
                hr = N::hf(Hr);
                if (HASD) Dr = ok ? ld<N>(a.D, idx + 1) : Dc;
            }
            const float hn = N::hf(Hn);
            T ux = N::zero(), uy = N::zero(), wxn = N::zero(), wyn = N::zero(), dx, dy, dux, duy;
            if constexpr (N::native) {
                if (xface) wxn = face_t<N, MODEL, CHECK>(a, Hc, Hr, hc + hr, Dc, Dr, wx, ux);
                if (upd) wyn = face_t<N, MODEL, CHECK>(a, Hc, Hn, hc + hn, Dc, Dn, wy, uy);
            } else {
                // both faces in one packed evaluation (lanes that need only one
                // of them discard the other)
                DF2 u2;
                const DF2 w2 = face2_t<N, MODEL, CHECK>(a, Hc, Hr, Hn, hc + hr, hc + hn, Dc, Dr, Dn,
                                                        df2_pack(wx, wy), u2);
                wxn = df2_first(w2);
                wyn = df2_second(w2);
                if (CHECK) {
                    ux = df2_first(u2);
                    uy = df2_second(u2);
                }
            }
            const T wxl = N::shfl_up(wxn, 1);
            const T uxl = CHECK ? N::shfl_up(ux, 1) : N::zero();
            const float dlf = MODEL == LINSTEP ? __shfl_up_sync(FULL, dcf, 1) : 0.0f;
            const float dnf = MODEL == LINSTEP ? N::lo_f(Dn) : 0.0f;
            if (own_x) st<N>(a.wout[0], idx, wxn);
            if (upd) {
                st<N>(a.wout[1], idx, wyn);
                const float dmax = MODEL == LINSTEP ? fmaxf(fmaxf(fmaxf(dcf, dlf), fmaxf(N::lo_f(Dr), dbf)), dnf)
                                                    : (MODEL == NONLIN_EXPM ? N::lo_f(Dc) : 0.0f);
                const float e = cell_e<MODEL>(a, hc, dmax);
                // the flux differences (x, y), packed for the double-float forms
                if constexpr (N::native) {
                    dx = N::sub(wxn, wxl);
                    dy = N::sub(wyn, wyb);
                    if (CHECK) {
                        dux = N::sub(ux, uxl);
                        duy = N::sub(uy, uyb);
                    }
                } else {
                    const DF2 d2 = df2_sub(df2_pack(wxn, wyn), df2_pack(wxl, wyb));
                    dx = df2_first(d2);
                    dy = df2_second(d2);
                    if (CHECK) {
                        const DF2 du2 = df2_sub(df2_pack(ux, uy), df2_pack(uxl, uyb));
                        dux = df2_first(du2);
                        duy = df2_second(du2);
                    }
                }
                HS Hnew;
                if (a.sq) {
                    Hnew = h_update_sq<N>(a, Hc, Ho, N::add(dy, dx), e);
                } else {
                    const T div = N::mad(dy, cst<N>(a, 1), N::mul(dx, cst<N>(a, 0)));
                    Hnew = h_update<N>(a, Hc, Ho, div, e);
                }
                N::sth(a.Hout, idx, Hnew);
                if (CHECK) {
                    const T divu = N::mad(duy, cst<N>(a, 1), N::mul(dux, cst<N>(a, 0)));
                    const T r = N::sub(divu, N::mul(N::hdn(Hnew, Ho), cst<N>(a, 3)));
                    accumulate_residual(N::to_d(r), part, pmax);
                }
            }
            Hc = Hn;
            hc = hn;
            wyb = wyn;
            uyb = uy;
            if (HASD) {
                dbf = dcf;
                Dc = Dn;
                dcf = dnf;
            }
            if (CHECK && j == j1 - 1) warp_flush_residual(a.acc, a.norm_max, part, pmax, lane, a.parts, slot);
        }
    } else if (CHECK && a.parts && lane == 0) {
        a.parts[slot] = 0.0;   // a warp with no cells: its slot still holds this check's (empty) part
    }
}

// ---------------------------------------------------------------------------
// 3D: blockDim = (32, R).  Block (bx, by, bz) owns cells
// i = 31*bx + lane, j = (R-1)*by + r (lane 0 / row 0 are the neighbours) and
// marches planes k0 .. k1-1 of z chunk bz.  Every thread of the block must
// call it (it holds block barriers).
template <class N, int MODEL, bool CHECK, int R>
__device__ __forceinline__ void pt3d_body(const PTArgs& a, int bx, int by, int bz, int chunk, double& part,
                                          unsigned long long& pmax)
{
    using T = typename N::T;
    using HV = typename N::HV;
    using HS = typename N::HS;
    __shared__ HV sH[2][R][32];
    __shared__ T sW[2][R][32];
    __shared__ T sU[CHECK ? 2 : 1][CHECK ? R : 1][32];
    constexpr bool HASD = ModelTraits<MODEL>::hasd;
    __shared__ float sF[2][R][32];   // H as float (NONLIN*) / D as float (LINSTEP)
    __shared__ T sD[HASD ? 2 : 1][HASD ? R : 1][32];

    const int lane = threadIdx.x, r = threadIdx.y;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int i = 31 * bx + lane;
    const int j = (R - 1) * by + r;
    const int k0 = 1 + bz * chunk;
    const int k1 = min(k0 + chunk, nz - 1);
    if (k0 < k1) {   // uniform over the block
        const int ic = min(i, nx - 1), jc = min(j, ny - 1);
        const bool inner_x = i >= 1 && i <= nx - 2;
        const bool inner_y = j >= 1 && j <= ny - 2;
        const bool xface = i <= nx - 2 && inner_y && r >= 1;
        const bool yface = j <= ny - 2 && inner_x;
        const bool upd = inner_x && inner_y && lane >= 1 && r >= 1;
        const bool own_x = xface && (lane >= 1 || bx == 0);
        const bool own_y = yface && lane >= 1 && (r >= 1 || by == 0);
        const bool top = r == R - 1;
        const bool up_ok = jc + 1 < ny;
        const long long sy = a.sy, sz = a.sz;
        long long idx = (long long)k0 * sz + (long long)jc * sy + ic;

        HV Hc = N::ldh(a.Hin, idx);
        float hc = N::hf(Hc);
        T Dc = HASD ? ld<N>(a.D, idx) : N::zero();
        float dcf = MODEL == LINSTEP ? N::lo_f(Dc) : 0.0f;
        float dbf = 0.0f;
        T wzb = N::zero(), uzb = N::zero();
        if (upd) {
            const HV Hb = N::ldh(a.Hin, idx - sz);
            const T Db = HASD ? ld<N>(a.D, idx - sz) : N::zero();
            dbf = MODEL == LINSTEP ? N::lo_f(Db) : 0.0f;
            wzb = face_t<N, MODEL, CHECK>(a, Hb, Hc, N::hf(Hb) + hc, Db, Dc, ld<N>(a.win[2], idx - sz), uzb);
            if (k0 == 1) st<N>(a.wout[2], idx - sz, wzb);
        }
        int p = 0;
        sH[0][r][lane] = Hc;
        sF[0][r][lane] = MODEL == LINSTEP ? dcf : hc;
        if (HASD) sD[0][r][lane] = Dc;
        __syncthreads();
        for (int k = k0; k < k1; ++k, idx += sz) {
            const HV Hn = N::ldh(a.Hin, idx + sz);
            const T wx = ld<N>(a.win[0], idx);
            const T wy = ld<N>(a.win[1], idx);
            const T wz = ld<N>(a.win[2], idx);
            const HS Ho = N::ldo(a.Hold, idx);
            const T Dn = HASD ? ld<N>(a.D, idx + sz) : N::zero();
            // neighbours in y (row above: shared memory, top row: global)
            HV Hu;
            T Du = N::zero();
            float hu = 0.0f, duf = 0.0f;
            if (!top) {
                Hu = sH[p][r + 1][lane];
                if (HASD) Du = sD[p][r + 1][lane];
                if (MODEL == LINSTEP) duf = sF[p][r + 1][lane];
                else hu = sF[p][r + 1][lane];
            } else {
                Hu = up_ok ? N::ldh(a.Hin, idx + sy) : Hc;
                hu = N::hf(Hu);
                if (HASD) {
                    Du = up_ok ? ld<N>(a.D, idx + sy) : Dc;
                    duf = N::lo_f(Du);
                }
            }
            // the row below's D for maxloc (sF[p] is rewritten only after the barrier)
            const float ddf = (MODEL == LINSTEP && r >= 1) ? sF[p][r - 1][lane] : 0.0f;
            // neighbour in x
            HV Hr = N::shfl_down_h(Hc, 1);
            float hr = __shfl_down_sync(FULL, hc, 1);
            T Dr = HASD ? N::shfl_down(Dc, 1) : N::zero();
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                Hr = ok ? N::ldh(a.Hin, idx + 1) : Hc;
                hr = N::hf(Hr);
                if (HASD) Dr = ok ? ld<N>(a.D, idx + 1) : Dc;
            }
            const float hn = N::hf(Hn);
            const float dnf = MODEL == LINSTEP ? N::lo_f(Dn) : 0.0f;
            T ux = N::zero(), uy = N::zero(), uz = N::zero(), wxn = N::zero(), wyn = N::zero(), wzn = N::zero();
            if constexpr (N::native) {
                if (xface) wxn = face_t<N, MODEL, CHECK>(a, Hc, Hr, hc + hr, Dc, Dr, wx, ux);
                if (yface) wyn = face_t<N, MODEL, CHECK>(a, Hc, Hu, hc + hu, Dc, Du, wy, uy);
            } else {
                // the x and y faces in one packed evaluation
                DF2 u2;
                const DF2 w2 = face2_t<N, MODEL, CHECK>(a, Hc, Hr, Hu, hc + hr, hc + hu, Dc, Dr, Du,
                                                        df2_pack(wx, wy), u2);
                wxn = df2_first(w2);
                wyn = df2_second(w2);
                if (CHECK) {
                    ux = df2_first(u2);
                    uy = df2_second(u2);
                }
            }
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
            if (HASD) sD[p ^ 1][r][lane] = Dn;
            __syncthreads();
            if (upd) {
                const T wyb = sW[p][r - 1][lane];
                const float dmax = MODEL == LINSTEP ? fmaxf(fmaxf(fmaxf(dcf, dlf), fmaxf(N::lo_f(Dr), duf)),
                                                            fmaxf(fmaxf(ddf, dbf), dnf))
                                                    : (MODEL == NONLIN_EXPM ? N::lo_f(Dc) : 0.0f);
                const float e = cell_e<MODEL>(a, hc, dmax);
                // the flux differences (x, y packed for the double-float forms; z)
                T dx, dy, dux, duy;
                const T dz = N::sub(wzn, wzb);
                if constexpr (N::native) {
                    dx = N::sub(wxn, wxl);
                    dy = N::sub(wyn, wyb);
                    if (CHECK) {
                        const T uyb = sU[p][r - 1][lane];
                        dux = N::sub(ux, uxl);
                        duy = N::sub(uy, uyb);
                    }
                } else {
                    const DF2 d2 = df2_sub(df2_pack(wxn, wyn), df2_pack(wxl, wyb));
                    dx = df2_first(d2);
                    dy = df2_second(d2);
                    if (CHECK) {
                        const T uyb = sU[p][r - 1][lane];
                        const DF2 du2 = df2_sub(df2_pack(ux, uy), df2_pack(uxl, uyb));
                        dux = df2_first(du2);
                        duy = df2_second(du2);
                    }
                }
                HS Hnew;
                if (a.sq) {
                    Hnew = h_update_sq<N>(a, Hc, Ho, N::add(N::add(dz, dy), dx), e);
                } else {
                    const T div = N::mad(dz, cst<N>(a, 2), N::mad(dy, cst<N>(a, 1), N::mul(dx, cst<N>(a, 0))));
                    Hnew = h_update<N>(a, Hc, Ho, div, e);
                }
                N::sth(a.Hout, idx, Hnew);
                if (CHECK) {
                    const T divu = N::mad(N::sub(uz, uzb), cst<N>(a, 2), N::mad(duy, cst<N>(a, 1), N::mul(dux, cst<N>(a, 0))));
                    const T r2 = N::sub(divu, N::mul(N::hdn(Hnew, Ho), cst<N>(a, 3)));
                    accumulate_residual(N::to_d(r2), part, pmax);
                }
            }
            Hc = Hn;
            hc = hn;
            wzb = wzn;
            uzb = uz;
            if (HASD) {
                dbf = dcf;
                Dc = Dn;
                dcf = dnf;
            }
            p ^= 1;
        }
    }
}


}  // namespace ptd
