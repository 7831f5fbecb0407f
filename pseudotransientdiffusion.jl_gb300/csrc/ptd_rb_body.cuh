// ptd_rb_body.cuh -- device code of the FP32 PT iterations on the change since
// an FP64 base state (PTD_PREC_FP32_RB, "rebased" FP32 form): argument and
// control blocks, the iteration bodies, and the judges of one grid; shared by
// the one-grid solver (ptd_rb.cu) and the batched solver (ptd_batch.cu).
//
// The FP64 PT iteration (ptd_device.cuh)
//   w^{k+1} = w^k - c (w^k + u(H^k)),          u = K_f(H) g(H)
//   H^{k+1} = H^k - e ((H^k - Hold)/dt + sum_d sigma_d (w^{k+1}_R - w^{k+1}_L))
// is run in delta form around an FP64 base (H_b, w_b): H = H_b + delta,
// w = w_b + omega, with delta and omega in FP32:
//   omega^{k+1} = omega^k - c (t_b + omega^k + u_d(delta^k))
//   delta^{k+1} = delta^k - e (R_b + delta^k/dt + sum_d sigma_d (omega^{k+1}_R - omega^{k+1}_L))
// where t_b = w_b + u(H_b) (the base flux defect), R_b = (H_b - Hold)/dt +
// div w_b (the base update residual) and u_d = u(H_b + delta) - u(H_b) are
// formed so that no FP32 quantity carries H or w themselves, only changes
// since the base and defects of the base, all of which shrink as the step
// converges: FP32 rounding is relative to them and sets no floor.  For D = H^3
// (s = H_L + H_R, g = H_R - H_L, s_d, g_d the same of delta)
//   u_d = s_d (3 s (s + s_d) + s_d^2) g + (s + s_d)^3 g_d.
// Every `phase` (a few hundred iterations) the base is rebased in FP64:
// H_b += delta, w_b += omega, delta = omega = 0, and t_b, R_b and the FP64
// residual of the base are recomputed.  Unlike a defect-correction loop
// (ptd_dc.cu) that restarts an inner solve from zero for each correction,
// this keeps the PT iteration's momentum (the fluxes) across rebases, so a
// physical step takes about the FP64 iteration's count of FP32 iterations.
//
// The FP32 base quantities (t_b, R_b) carry rounding relative to the residual
// at the phase start, which bounds what one phase can attain: a phase also
// ends once its residual has dropped 1e4-fold, so the number of rebases per
// step grows only logarithmically with the residual reduction.
//
// Stopping: every nchk iterations the mixed residual of the reference's check
// (check_res!, scripts/diff_2D_nonlin.jl:41-44) is formed from the base's
// FP64 check residual C_b = div u(H_b) - (H_b - Hold)/dt and the FP32
// changes; when its norm is <= tol the phase ends early, the base is rebased
// and the step stops if the FP64 residual of the rebased state is <= tol too
// (else the iteration continues).  The returned H is the FP64 base.
#pragma once

#include "ptd_device.cuh"
#include "ptd_kernels.h"

namespace ptd {

struct RbArgs {
    int nx, ny, nz;
    long long sy, sz;
    float rdt;
    float sig[3];
    float c_lin, e_lin;
    FParams f;
    const float* din;     // delta (iteration k)
    float* dout;          // delta (iteration k+1)
    const float* win[3];  // omega
    float* wout[3];
    const float* tb[3];   // base flux defect w_b + u(H_b), per face
    const float* Rb;      // base update residual
    const float* Cb;      // base check residual, rounded to FP32 (1D, 2D; read on check iterations only)
    const double* Cb64;   // base check residual, FP64 (3D)
    const float* Hf;      // H_b as FP32 (iteration parameters, u_d)
    const float* Df;      // LINSTEP: D, NONLIN_EXPM: exp(m), as FP32
    const int* skip;
    double* acc;
    // Per-warp (2D) / per-block (1D, 3D) slots of the check residual that the
    // judge sums in a fixed order (the same residual norm on every run); NULL:
    // the partials go into acc by atomics instead (the batched solver).
    double* parts;
    int norm_max;
};

struct RbDev {
    int skip;         // PT kernels return at entry: the phase is over or the step done
    int step_done;    // DONE_* of the physical step
    int iter;         // PT iterations of this step
    int phase_iter;   // PT iterations of this phase (the buffer parity)
    int nchecks;
    int capped;
    int phases;       // phases run in this step (FP64 rebases inside the step graph)
    int blocks;       // check blocks run in this step (one-grid solver)
    int passes;       // passes of the step graph's loop (one-grid solver)
    int pad1;
    double acc;       // FP32 check residual accumulator (sum or max bits)
    double acc64;     // FP64 base residual accumulator
    double err;       // last FP32 check err
    double err64;     // last FP64 err
};

// Cell parameter of the rebased kernels, every operation explicit (the face
// parameter is face_c_rn, ptd_device.cuh), so that every kernel variant
// rounds identically: e = 1/((pi H^3 + sqrt(pi^2 H^6 + fA H^3)) k1 + 1/dt)
// (nonlin_cell_e, scripts/diff_2D_nonlin.jl:23,26).
__device__ __forceinline__ float rb_e(const FParams& f, float h3)
{
    const float q = __fmaf_rn(__fmul_rn(f.fpi2, h3), h3, __fmul_rn(f.fA, h3));
    const float p = __fmaf_rn(f.fpi, h3, fsqrt(q));
    return frcp(__fmaf_rn(p, f.fk1, f.frdt));
}

// One face: new omega, and u_d (the change of the undamped flux) when U.
template <int MODEL, bool U>
__device__ __forceinline__ float rb_face(const RbArgs& a, float dL, float dR, float hL, float hR, float DL,
                                         float DR, float w, float tb, float& u)
{
    const float gd = dR - dL;
    float ud, c;
    if (MODEL == LIN) {
        ud = gd;
        c = a.c_lin;
    } else if (MODEL == LINSTEP) {
        ud = __fmul_rn(DL + DR, gd);
        c = a.c_lin;
    } else {   // NONLIN, NONLIN_EXPM (D holds exp(m): K = (E_L + E_R) s^3, kappa 1/16)
        const float sb = hL + hR, sd = dL + dR, gb = hR - hL;
        const float st = sb + sd;
        const float st3 = __fmul_rn(__fmul_rn(st, st), st);
        ud = __fmaf_rn(__fmul_rn(sd, __fmaf_rn(__fmul_rn(3.0f, sb), st, __fmul_rn(sd, sd))), gb,
                       __fmul_rn(st3, gd));
        if (MODEL == NONLIN_EXPM) {
            const float e2 = DL + DR;
            ud = __fmul_rn(ud, e2);
            const float m = __fmul_rn(0.5f, st);
            c = face_c_rn(a.f, __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(0.5f, e2), m), m), m));
        } else {
            c = face_c_rn(a.f, __fmul_rn(0.125f, st3));   // D_f = (st/2)^3
        }
    }
    if (U) u = ud;
    return __fmaf_rn(-c, w + (tb + ud), w);
}

template <int MODEL>
__device__ __forceinline__ float rb_cell_e(const RbArgs& a, float h, float dmax)
{
    if (MODEL == LIN) return a.e_lin;
    if (MODEL == LINSTEP) return linstep_cell_e(a.f, dmax);
    float h3 = __fmul_rn(__fmul_rn(h, h), h);
    if (MODEL == NONLIN_EXPM) h3 = __fmul_rn(__fmul_rn(__fmul_rn(dmax, h), h), h);   // dmax carries exp(m)
    return rb_e(a.f, h3);
}

// Two faces: the flux arithmetic packed, the iteration parameters c (MUFU
// work with constant operands, which scalar instructions take for free)
// scalar.  3 sb is formed as (sb + sb) + sb: sb + sb is exact, so the sum
// rounds once, like the scalar 3.0f * sb.
template <int MODEL, bool U>
__device__ __forceinline__ float2 rb_face2(const RbArgs& a, float2 dL, float2 dR, float2 hL, float2 hR, float2 DL,
                                           float2 DR, float2 w, float2 tb, float2& u)
{
    const float2 gd = sub2(dR, dL);
    float2 ud;
    float cx, cy;
    if (MODEL == LIN) {
        ud = gd;
        cx = cy = a.c_lin;
    } else {   // NONLIN
        const float2 sb = add2(hL, hR), sd = add2(dL, dR), gb = sub2(hR, hL);
        const float2 st = add2(sb, sd);
        const float2 st3 = mul2(mul2(st, st), st);
        ud = fma2(mul2(sd, fma2(add2(add2(sb, sb), sb), st, mul2(sd, sd))), gb, mul2(st3, gd));
        cx = face_c_rn(a.f, __fmul_rn(0.125f, st3.x));
        cy = face_c_rn(a.f, __fmul_rn(0.125f, st3.y));
    }
    if (U) u = ud;
    return fma2(f2(-cx, -cy), add2(w, add2(tb, ud)), w);
}

__device__ __forceinline__ bool rb_skip(const int* skip) { return __ldcg(skip) != 0; }

// ---------------------------------------------------------------------------
// 1D: one thread per cell; the left face is recomputed (1D grids are small).
template <int MODEL, bool CHECK>
__device__ __forceinline__ void rb1d_body(const RbArgs& a, int bx, float& part, unsigned& pmax)
{
    constexpr bool LS = MODEL == LINSTEP;
    constexpr bool HASD = LS || MODEL == NONLIN_EXPM;   // a per-cell field in Df
    const int i = bx * blockDim.x + threadIdx.x;
    const int nx = a.nx;
    if (i >= nx) return;
    const float dc = a.din[i], hc = a.Hf[i];
    const float Dc = HASD ? a.Df[i] : 0.0f;
    float wr = 0.0f, ur = 0.0f, Dr = 0.0f;
    if (i <= nx - 2) {
        Dr = HASD ? a.Df[i + 1] : 0.0f;
        wr = rb_face<MODEL, CHECK>(a, dc, a.din[i + 1], hc, a.Hf[i + 1], Dc, Dr, a.win[0][i], a.tb[0][i], ur);
        a.wout[0][i] = wr;
    }
    if (i >= 1 && i <= nx - 2) {
        const float Dl = HASD ? a.Df[i - 1] : 0.0f;
        float ul = 0.0f;
        const float wl = rb_face<MODEL, CHECK>(a, a.din[i - 1], dc, a.Hf[i - 1], hc, Dl, Dc, a.win[0][i - 1],
                                               a.tb[0][i - 1], ul);
        const float e = rb_cell_e<MODEL>(a, hc + dc, LS ? fmaxf(fmaxf(Dl, Dr), Dc) : Dc);
        const float dnew = fmaf(-e, fmaf(dc, a.rdt, a.Rb[i] + (wr - wl) * a.sig[0]), dc);
        a.dout[i] = dnew;
        if (CHECK)
            accumulate_residual32(fmaf(-dnew, a.rdt, a.Cb[i] + (ur - ul) * a.sig[0]), part,
                                pmax);
    }
}

// ---------------------------------------------------------------------------
// 2D: the tiling of ptd_pt_body.cuh (31 updated columns per warp, y march).
template <int MODEL, bool CHECK>
__device__ __forceinline__ void rb2d_body(const RbArgs& a, int tile, int cy, int chunk, float& part,
                                          unsigned& pmax, long long slot = 0)
{
    constexpr bool LS = MODEL == LINSTEP;
    constexpr bool HASD = LS || MODEL == NONLIN_EXPM;   // a per-cell field in Df
    const int lane = threadIdx.x;
    const int i = 31 * tile + lane;
    const int nx = a.nx, ny = a.ny;
    const int j0 = 1 + cy * chunk;
    const int j1 = min(j0 + chunk, ny - 1);
    if ((31 * tile < nx - 1) && (j0 < j1)) {
        const int ic = min(i, nx - 1);
        const bool xface = i <= nx - 2;
        const bool upd = i >= 1 && i <= nx - 2 && lane >= 1;
        const bool own_x = xface && (lane >= 1 || tile == 0);
        const long long sy = a.sy;
        long long idx = (long long)j0 * sy + ic;
        float dc = a.din[idx], hc = a.Hf[idx];
        float Dc = HASD ? a.Df[idx] : 0.0f, Db = 0.0f;
        float wyb = 0.0f, uyb = 0.0f;
        if (upd) {
            Db = HASD ? a.Df[idx - sy] : 0.0f;
            wyb = rb_face<MODEL, CHECK>(a, a.din[idx - sy], dc, a.Hf[idx - sy], hc, Db, Dc, a.win[1][idx - sy],
                                        a.tb[1][idx - sy], uyb);
            if (j0 == 1) a.wout[1][idx - sy] = wyb;
        }
        for (int j = j0; j < j1; ++j, idx += sy) {
            const float dn = a.din[idx + sy], hn = a.Hf[idx + sy];
            const float wx = a.win[0][idx], wy = a.win[1][idx];
            const float tbx = a.tb[0][idx], tby = a.tb[1][idx], rb = a.Rb[idx];
            const float Dn = HASD ? a.Df[idx + sy] : 0.0f;
            float dr = __shfl_down_sync(FULL, dc, 1);
            float hr = __shfl_down_sync(FULL, hc, 1);
            float Dr = HASD ? __shfl_down_sync(FULL, Dc, 1) : 0.0f;
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                dr = ok ? a.din[idx + 1] : dc;
                hr = ok ? a.Hf[idx + 1] : hc;
                if (HASD) Dr = ok ? a.Df[idx + 1] : Dc;
            }
            float ux = 0.0f, uy = 0.0f, wxn = 0.0f, wyn = 0.0f;
            if (xface) wxn = rb_face<MODEL, CHECK>(a, dc, dr, hc, hr, Dc, Dr, wx, tbx, ux);
            if (upd) wyn = rb_face<MODEL, CHECK>(a, dc, dn, hc, hn, Dc, Dn, wy, tby, uy);
            const float wxl = __shfl_up_sync(FULL, wxn, 1);
            const float uxl = CHECK ? __shfl_up_sync(FULL, ux, 1) : 0.0f;
            const float Dl = HASD ? __shfl_up_sync(FULL, Dc, 1) : 0.0f;
            if (own_x) a.wout[0][idx] = wxn;
            if (upd) {
                a.wout[1][idx] = wyn;
                const float e = rb_cell_e<MODEL>(a, hc + dc, LS ? fmaxf(fmaxf(fmaxf(Dc, Dl), fmaxf(Dr, Db)), Dn) : Dc);
                const float div = fmaf(wyn - wyb, a.sig[1], (wxn - wxl) * a.sig[0]);
                const float dnew = fmaf(-e, fmaf(dc, a.rdt, rb + div), dc);
                a.dout[idx] = dnew;
                if (CHECK) {
                    const float divu = fmaf(uy - uyb, a.sig[1], (ux - uxl) * a.sig[0]);
                    accumulate_residual32(fmaf(-dnew, a.rdt, a.Cb[idx] + divu), part, pmax);
                }
            }
            dc = dn;
            hc = hn;
            wyb = wyn;
            uyb = uy;
            if (HASD) {
                Db = Dc;
                Dc = Dn;
            }
            if (CHECK && j == j1 - 1) warp_flush_residual32(a.acc, a.norm_max, part, pmax, lane, a.parts, slot);
        }
    } else if (CHECK && a.parts && lane == 0) {
        a.parts[slot] = 0.0;   // a warp with no cells: its slot still holds this check's (empty) part
    }
}

// ---------------------------------------------------------------------------
// 2D, two iterations per launch (temporal blocking).  The first iteration
// (level 1) runs one row ahead of the second (level 2) in the y march; the
// level-1 deltas and fluxes of the current and previous rows stay in
// registers, so a launch reads and writes each field once for two
// iterations.  A warp covers 32 columns, lane L <-> column 28 t + L - 1:
// level-1 x faces on lanes 0..30, level-1 updates on lanes 1..30, level-2
// x faces on lanes 1..29 and level-2 updates on lanes 2..29 (28 columns per
// warp), so every right neighbour comes from a shuffle.  Each iteration's
// arithmetic is rb2d_body's, operation for operation.
template <int MODEL>
__device__ __forceinline__ float rb_star(float Dc, float Db, float Dn)
{
    if (MODEL != LINSTEP) return Dc;   // NONLIN_EXPM: exp(m) of the cell; unused otherwise
    const float Dr = __shfl_down_sync(FULL, Dc, 1);
    const float Dl = __shfl_up_sync(FULL, Dc, 1);
    return fmaxf(fmaxf(fmaxf(Dc, Dl), fmaxf(Dr, Db)), Dn);
}

template <int MODEL, bool CHECK>
__device__ __forceinline__ void rb2d_tb2_body(const RbArgs& a, int tile, int cy, int chunk, float& part,
                                              unsigned& pmax, long long slot = 0)
{
    constexpr bool HASD = MODEL == LINSTEP || MODEL == NONLIN_EXPM;
    const int lane = threadIdx.x;
    const int nx = a.nx, ny = a.ny;
    const int j0 = 1 + cy * chunk;
    const int j1 = min(j0 + chunk, ny - 1);
    if (28 * tile >= nx - 2 || j0 >= j1) {   // uniform over the warp
        if (CHECK && a.parts && lane == 0) a.parts[slot] = 0.0;
        return;
    }
    const int i = 28 * tile + lane - 1;
    const int ic = min(max(i, 0), nx - 1);          // clamped column of this lane's loads
    const bool colin = i >= 1 && i <= nx - 2;
    const bool upd1 = colin && lane >= 1 && lane <= 30;
    const bool xf2 = i >= 0 && i <= nx - 2 && lane >= 1 && lane <= 29;
    const bool upd2 = colin && lane >= 2 && lane <= 29;
    const bool own_x = xf2 && (lane <= 28 || i == nx - 2);   // face i+1/2 of lane 29: the next tile's lane 1
    const long long sy = a.sy;
    const float s0 = a.sig[0], s1 = a.sig[1], rdt = a.rdt;
    float u;

    // level-1 x face of a row at offset o (flux omega of the input state);
    // hr, Dr: the right neighbour's H_b and D, reused by level 2
    auto x1 = [&](long long o, float d, float h, float D, float& tbx, float& hr, float& Dr) {
        const float dr = __shfl_down_sync(FULL, d, 1);
        hr = __shfl_down_sync(FULL, h, 1);
        Dr = HASD ? __shfl_down_sync(FULL, D, 1) : 0.0f;
        tbx = a.tb[0][o];
        return rb_face<MODEL, false>(a, d, dr, h, hr, D, Dr, a.win[0][o], tbx, u);
    };
    auto cell = [&](float d, float e, float r, float wx, float wxl, float wy, float wyb) {
        return fmaf(-e, fmaf(d, rdt, r + fmaf(wy - wyb, s1, (wx - wxl) * s0)), d);
    };

    // ---- prologue: level 1 of rows j0-1 (A) and j0 (B), level-2 face j0-1/2
    const long long oA = (long long)(j0 - 1) * sy + ic, oB = oA + sy, oC = oB + sy;
    const float dA = a.din[oA], hA = a.Hf[oA];
    const float DA = HASD ? a.Df[oA] : 0.0f;
    const float dB = a.din[oB], hB = a.Hf[oB];
    const float DB = HASD ? a.Df[oB] : 0.0f;
    float d1 = a.din[oC], h1 = a.Hf[oC];    // row j0+1 <= ny-1
    float D1 = HASD ? a.Df[oC] : 0.0f;
    const float tbyA = a.tb[1][oA];
    const float wyAB = rb_face<MODEL, false>(a, dA, dB, hA, hB, DA, DB, a.win[1][oA], tbyA, u);  // omega'_y(j0-1/2)
    float pA = dA;                          // delta'(j0-1)
    if (j0 >= 2) {                          // row j0-1 is interior: level 1 there
        const long long oZ = oA - sy;
        const float dZ = a.din[oZ], hZ = a.Hf[oZ];
        const float DZ = HASD ? a.Df[oZ] : 0.0f;
        const float wyZA = rb_face<MODEL, false>(a, dZ, dA, hZ, hA, DZ, DA, a.win[1][oZ], a.tb[1][oZ], u);
        float tbxA, hAr, DAr;
        const float wxA = x1(oA, dA, hA, DA, tbxA, hAr, DAr);
        const float wxAl = __shfl_up_sync(FULL, wxA, 1);
        const float eA = rb_cell_e<MODEL>(a, hA + dA, rb_star<MODEL>(DA, DZ, DB));
        if (upd1) pA = cell(dA, eA, a.Rb[oA], wxA, wxAl, wyAB, wyZA);
    }
    float tbx0, h0r, D0r;
    float wx1p = x1(oB, dB, hB, DB, tbx0, h0r, D0r);       // omega'_x(j0)
    float tby0 = a.tb[1][oB];
    float wy1p = rb_face<MODEL, false>(a, dB, d1, hB, h1, DB, D1, a.win[1][oB], tby0, u);  // omega'_y(j0+1/2)
    float r0 = a.Rb[oB];
    float p0 = dB;                                         // delta'(j0)
    {
        const float wxl = __shfl_up_sync(FULL, wx1p, 1);
        const float eB = rb_cell_e<MODEL>(a, hB + dB, rb_star<MODEL>(DB, DA, D1));
        if (upd1) p0 = cell(dB, eB, r0, wx1p, wxl, wy1p, wyAB);
    }
    float uy2b = 0.0f;
    float wy2b = rb_face<MODEL, CHECK>(a, pA, p0, hA, hB, DA, DB, wyAB, tbyA, uy2b);   // omega''_y(j0-1/2)
    if (j0 == 1 && upd2) a.wout[1][oA] = wy2b;
    float h0 = hB, D0 = DB, Dm1 = DA;

    // ---- march: level 1 of row s+1, level 2 of row s.  LIN, NONLIN: the x
    // and y faces of a level are one two-lane (f32x2) evaluation of the flux
    // arithmetic; the models with a coefficient field keep the scalar faces
    // (the packed ones did not reproduce the one-iteration kernel bit for bit
    // there).  (Packing the iteration parameters too, whose constant operands
    // scalar instructions take for free, was slower: 81.2 against 77.9 us.)
    constexpr bool PACKF = MODEL == LIN || MODEL == NONLIN;
    long long o = oC;   // offset of row s+1
    for (int s = j0; s < j1; ++s, o += sy) {
        float p1 = d1, wx1 = 0.0f, wy1 = 0.0f, r1 = 0.0f, h2 = h1, D2 = D1, tbx1 = 0.0f, tby1 = 0.0f;
        float h1r = h1, D1r = D1;
        if (s + 1 <= ny - 2) {   // row s+1 interior (uniform): level 1 there
            const float d2 = a.din[o + sy];
            h2 = a.Hf[o + sy];
            if (HASD) D2 = a.Df[o + sy];
            r1 = a.Rb[o];
            tbx1 = a.tb[0][o];
            tby1 = a.tb[1][o];
            const float d1r = __shfl_down_sync(FULL, d1, 1);
            h1r = __shfl_down_sync(FULL, h1, 1);
            if (HASD) D1r = __shfl_down_sync(FULL, D1, 1);
            if (PACKF) {
                float2 uu;
                const float2 w1 = rb_face2<MODEL, false>(a, f2(d1), f2(d1r, d2), f2(h1), f2(h1r, h2), f2(D1),
                                                         f2(D1r, D2), f2(a.win[0][o], a.win[1][o]), f2(tbx1, tby1), uu);
                wx1 = w1.x;
                wy1 = w1.y;
            } else {
                wx1 = rb_face<MODEL, false>(a, d1, d1r, h1, h1r, D1, D1r, a.win[0][o], tbx1, u);
                wy1 = rb_face<MODEL, false>(a, d1, d2, h1, h2, D1, D2, a.win[1][o], tby1, u);
            }
            const float wx1l = __shfl_up_sync(FULL, wx1, 1);
            const float e1 = rb_cell_e<MODEL>(a, h1 + d1, rb_star<MODEL>(D1, D0, D2));
            if (upd1) p1 = cell(d1, e1, r1, wx1, wx1l, wy1, wy1p);
            d1 = d2;
        }
        // level 2 of row s
        const float p0r = __shfl_down_sync(FULL, p0, 1);
        float wx2, wy2, ux2 = 0.0f, uy2 = 0.0f;
        if (PACKF) {
            float2 u2 = f2(0.0f);
            const float2 w2 = rb_face2<MODEL, CHECK>(a, f2(p0), f2(p0r, p1), f2(h0), f2(h0r, h1), f2(D0), f2(D0r, D1),
                                                     f2(wx1p, wy1p), f2(tbx0, tby0), u2);
            wx2 = w2.x;
            wy2 = w2.y;
            ux2 = u2.x;
            uy2 = u2.y;
        } else {
            wx2 = rb_face<MODEL, CHECK>(a, p0, p0r, h0, h0r, D0, D0r, wx1p, tbx0, ux2);
            wy2 = rb_face<MODEL, CHECK>(a, p0, p1, h0, h1, D0, D1, wy1p, tby0, uy2);
        }
        const float wx2l = __shfl_up_sync(FULL, wx2, 1);
        const float ux2l = CHECK ? __shfl_up_sync(FULL, ux2, 1) : 0.0f;
        const float e0 = rb_cell_e<MODEL>(a, h0 + p0, rb_star<MODEL>(D0, Dm1, D1));
        const long long os = o - sy;
        if (own_x) a.wout[0][os] = wx2;
        if (upd2) {
            const float q = cell(p0, e0, r0, wx2, wx2l, wy2, wy2b);
            a.dout[os] = q;
            a.wout[1][os] = wy2;
            if (CHECK) {
                const float divu = fmaf(uy2 - uy2b, s1, (ux2 - ux2l) * s0);
                accumulate_residual32(fmaf(-q, rdt, a.Cb[os] + divu), part, pmax);
            }
        }
        // shift the windows
        p0 = p1;
        wx1p = wx1;
        wy1p = wy1;
        tbx0 = tbx1;
        tby0 = tby1;
        r0 = r1;
        wy2b = wy2;
        uy2b = uy2;
        h0 = h1;
        h0r = h1r;
        h1 = h2;
        Dm1 = D0;
        D0 = D1;
        D0r = D1r;
        D1 = D2;
        if (CHECK && s == j1 - 1) warp_flush_residual32(a.acc, a.norm_max, part, pmax, lane, a.parts, slot);
    }
}

// ---------------------------------------------------------------------------
// 2D, two iterations per launch with two x-adjacent columns per lane (LIN,
// NONLIN): rb2d_tb2_body's march, operation for operation per column, with
// every field read and written as one 8-byte pair per lane and the faces of
// the same direction of a lane's two columns (x: the face between them and
// the face to the next lane's first column; y: both columns' faces) as one
// FP32x2 evaluation.  The kernel is bound by memory latency: a pair per lane
// doubles the bytes each load instruction has in flight and halves the
// loads, shuffles and address arithmetic per cell.  A warp covers the 64
// columns 60 t - 2 + q, q = 2L, 2L+1 on lane L (an even first column, so a
// pair is one aligned 8-byte access): level 1 updates q = 1..62, level 2
// q = 2..61 (60 columns per warp).
template <int MODEL, bool CHECK>
__device__ __forceinline__ void rb2d_tb2_pair_body(const RbArgs& a, int tile, int cy, int chunk, float& part,
                                                   unsigned& pmax, long long slot = 0)
{
    static_assert(MODEL == LIN || MODEL == NONLIN, "the pair kernel serves LIN and NONLIN");
    const int lane = threadIdx.x;
    const int nx = a.nx, ny = a.ny;
    const int j0 = 1 + cy * chunk;
    const int j1 = min(j0 + chunk, ny - 1);
    if (60 * tile > nx - 2 || j0 >= j1) {   // uniform over the warp
        if (CHECK && a.parts && lane == 0) a.parts[slot] = 0.0;
        return;
    }
    const int c0 = 60 * tile - 2 + 2 * lane;      // column of the lane's first cell
    // pairs left of the grid or past the row pitch are read at the nearest
    // pair: their values feed only faces and cells that are discarded
    const int cl = min(max(c0, 0), (int)a.sy - 2);
    const int q0 = 2 * lane;
    auto in_grid = [&](int c) { return c >= 1 && c <= nx - 2; };
    const bool u1a = q0 >= 1 && in_grid(c0), u1b = q0 + 1 <= 62 && in_grid(c0 + 1);          // level 1
    const bool u2a = q0 >= 2 && q0 <= 61 && in_grid(c0);                                      // level 2
    const bool u2b = q0 + 1 >= 2 && q0 + 1 <= 61 && in_grid(c0 + 1);
    // level-2 x faces (q -> q+1, evaluated for q = 1..61) stored: q = 1..60 (q = 61 is the next
    // tile's q = 1), and the grid's last face
    auto own_face = [&](int q, int c) {
        return q >= 1 && q <= 61 && c >= 0 && c <= nx - 2 && (q <= 60 || c == nx - 2);
    };
    const bool oxa = own_face(q0, c0), oxb = own_face(q0 + 1, c0 + 1);
    const long long sy = a.sy;
    const float2 s0 = f2(a.sig[0]), s1 = f2(a.sig[1]), rdt = f2(a.rdt);
    float2 u;
    auto ld2 = [&](const float* p, long long o) { return *reinterpret_cast<const float2*>(p + o); };
    auto st2 = [&](float* p, long long o, float2 v, bool ma, bool mb) {
        if (ma && mb) {
            *reinterpret_cast<float2*>(p + o) = v;
        } else {
            if (ma) p[o] = v.x;
            if (mb) p[o + 1] = v.y;
        }
    };
    // right neighbours of the lane's two columns: (second column, next lane's first)
    auto right = [&](float2 v) { return f2(v.y, __shfl_down_sync(FULL, v.x, 1)); };
    // left faces of the two columns from their right faces
    auto left = [&](float2 w) { return f2(__shfl_up_sync(FULL, w.y, 1), w.x); };
    auto cell_e2 = [&](float2 h, float2 d) {
        return f2(rb_cell_e<MODEL>(a, h.x + d.x, 0.0f), rb_cell_e<MODEL>(a, h.y + d.y, 0.0f));
    };
    // the update of rb2d_tb2_body's `cell`, both columns: d - e (d rdt + r + (wy - wyb) s1 + (wx - wxl) s0)
    auto cell2 = [&](float2 d, float2 e, float2 r, float2 wx, float2 wxl, float2 wy, float2 wyb) {
        return fma2(f2(-e.x, -e.y), fma2(d, rdt, add2(r, fma2(sub2(wy, wyb), s1, mul2(sub2(wx, wxl), s0)))), d);
    };
    auto sel = [](float2 v, float2 old, bool ma, bool mb) { return f2(ma ? v.x : old.x, mb ? v.y : old.y); };

    // ---- prologue: level 1 of rows j0-1 (A) and j0 (B), level-2 face j0-1/2
    const long long oA = (long long)(j0 - 1) * sy + cl, oB = oA + sy, oC = oB + sy;
    const float2 dA = ld2(a.din, oA), hA = ld2(a.Hf, oA);
    const float2 dB = ld2(a.din, oB), hB = ld2(a.Hf, oB);
    float2 d1 = ld2(a.din, oC), h1 = ld2(a.Hf, oC);   // row j0+1 <= ny-1
    const float2 tbyA = ld2(a.tb[1], oA);
    const float2 wyAB = rb_face2<MODEL, false>(a, dA, dB, hA, hB, f2(0.0f), f2(0.0f), ld2(a.win[1], oA), tbyA, u);
    float2 pA = dA;
    if (j0 >= 2) {   // row j0-1 is interior: level 1 there
        const long long oZ = oA - sy;
        const float2 dZ = ld2(a.din, oZ), hZ = ld2(a.Hf, oZ);
        const float2 wyZA = rb_face2<MODEL, false>(a, dZ, dA, hZ, hA, f2(0.0f), f2(0.0f), ld2(a.win[1], oZ),
                                                   ld2(a.tb[1], oZ), u);
        const float2 wxA = rb_face2<MODEL, false>(a, dA, right(dA), hA, right(hA), f2(0.0f), f2(0.0f),
                                                  ld2(a.win[0], oA), ld2(a.tb[0], oA), u);
        pA = sel(cell2(dA, cell_e2(hA, dA), ld2(a.Rb, oA), wxA, left(wxA), wyAB, wyZA), dA, u1a, u1b);
    }
    float2 h0r = right(hB);
    float2 tbx0 = ld2(a.tb[0], oB), tby0 = ld2(a.tb[1], oB), r0 = ld2(a.Rb, oB);
    float2 wx1p = rb_face2<MODEL, false>(a, dB, right(dB), hB, h0r, f2(0.0f), f2(0.0f), ld2(a.win[0], oB), tbx0, u);
    float2 wy1p = rb_face2<MODEL, false>(a, dB, d1, hB, h1, f2(0.0f), f2(0.0f), ld2(a.win[1], oB), tby0, u);
    float2 p0 = sel(cell2(dB, cell_e2(hB, dB), r0, wx1p, left(wx1p), wy1p, wyAB), dB, u1a, u1b);
    float2 uy2b = f2(0.0f);
    float2 wy2b = rb_face2<MODEL, CHECK>(a, pA, p0, hA, hB, f2(0.0f), f2(0.0f), wyAB, tbyA, uy2b);
    if (j0 == 1) st2(a.wout[1], oA, wy2b, u2a, u2b);
    float2 h0 = hB;

    // ---- march: level 1 of row s+1, level 2 of row s.  (Issuing a step's
    // loads one step ahead, in registers, was no faster: 66.6 against 66.4 us
    // per iteration at 4096^2, its 78 registers halving the resident warps.
    // Staging them through a per-warp shared-memory ring with cp.async, one to
    // three steps ahead, was slower at every launch shape that fills the GPU:
    // 67.5 / 68.6 / 90.5 us against 64.7 at the best shape, the shared loads
    // costing more issue slots than the hidden latency saved.  Capping the
    // registers at 48 for five CTAs per SM spilled 40 bytes and took 73 us.)
    long long o = oC;   // offset of row s+1
    for (int s = j0; s < j1; ++s, o += sy) {
        float2 p1 = d1, wx1 = f2(0.0f), wy1 = f2(0.0f), r1 = f2(0.0f), h2 = h1, tbx1 = f2(0.0f), tby1 = f2(0.0f);
        float2 h1r = h1;
        if (s + 1 <= ny - 2) {   // row s+1 interior (uniform): level 1 there
            const float2 d2 = ld2(a.din, o + sy);
            h2 = ld2(a.Hf, o + sy);
            r1 = ld2(a.Rb, o);
            tbx1 = ld2(a.tb[0], o);
            tby1 = ld2(a.tb[1], o);
            h1r = right(h1);
            wx1 = rb_face2<MODEL, false>(a, d1, right(d1), h1, h1r, f2(0.0f), f2(0.0f), ld2(a.win[0], o), tbx1, u);
            wy1 = rb_face2<MODEL, false>(a, d1, d2, h1, h2, f2(0.0f), f2(0.0f), ld2(a.win[1], o), tby1, u);
            p1 = sel(cell2(d1, cell_e2(h1, d1), r1, wx1, left(wx1), wy1, wy1p), d1, u1a, u1b);
            d1 = d2;
        }
        // level 2 of row s
        float2 ux2 = f2(0.0f), uy2 = f2(0.0f);
        const float2 wx2 = rb_face2<MODEL, CHECK>(a, p0, right(p0), h0, h0r, f2(0.0f), f2(0.0f), wx1p, tbx0, ux2);
        const float2 wy2 = rb_face2<MODEL, CHECK>(a, p0, p1, h0, h1, f2(0.0f), f2(0.0f), wy1p, tby0, uy2);
        const float2 q = cell2(p0, cell_e2(h0, p0), r0, wx2, left(wx2), wy2, wy2b);
        const long long os = o - sy;
        st2(a.wout[0], os, wx2, oxa, oxb);
        st2(a.dout, os, q, u2a, u2b);
        st2(a.wout[1], os, wy2, u2a, u2b);
        if (CHECK) {
            const float2 ux2l = left(ux2);
            const float2 divu = fma2(sub2(uy2, uy2b), s1, mul2(sub2(ux2, ux2l), s0));
            if (u2a) accumulate_residual32(fmaf(-q.x, rdt.x, a.Cb[os] + divu.x), part, pmax);
            if (u2b) accumulate_residual32(fmaf(-q.y, rdt.y, a.Cb[os + 1] + divu.y), part, pmax);
        }
        // shift the windows
        p0 = p1;
        wx1p = wx1;
        wy1p = wy1;
        tbx0 = tbx1;
        tby0 = tby1;
        r0 = r1;
        wy2b = wy2;
        uy2b = uy2;
        h0 = h1;
        h0r = h1r;
        h1 = h2;
        if (CHECK && s == j1 - 1) warp_flush_residual32(a.acc, a.norm_max, part, pmax, lane, a.parts, slot);
    }
}

// ---------------------------------------------------------------------------
// 3D: R warps as the y rows of an x-y tile, z march (ptd_pt_body.cuh).
template <int MODEL, bool CHECK, int R>
__device__ __forceinline__ void rb3d_body(const RbArgs& a, int bx, int by, int bz, int chunk, double& part,
                                          unsigned long long& pmax)
{
    constexpr bool LS = MODEL == LINSTEP;
    constexpr bool HASD = LS || MODEL == NONLIN_EXPM;   // a per-cell field in Df
    __shared__ float sd[2][R][32];
    __shared__ float sh[2][R][32];
    __shared__ float sw[2][R][32];
    __shared__ float su[CHECK ? 2 : 1][CHECK ? R : 1][32];
    __shared__ float sD[HASD ? 2 : 1][HASD ? R : 1][32];
    const int lane = threadIdx.x, r = threadIdx.y;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int i = 31 * bx + lane;
    const int j = (R - 1) * by + r;
    const int k0 = 1 + bz * chunk;
    const int k1 = min(k0 + chunk, nz - 1);
    if (k0 < k1) {   // uniform over the block
        const int ic = min(i, nx - 1), jc = min(j, ny - 1);
        const bool inner_x = i >= 1 && i <= nx - 2, inner_y = j >= 1 && j <= ny - 2;
        const bool xface = i <= nx - 2 && inner_y && r >= 1;
        const bool yface = j <= ny - 2 && inner_x;
        const bool upd = inner_x && inner_y && lane >= 1 && r >= 1;
        const bool own_x = xface && (lane >= 1 || bx == 0);
        const bool own_y = yface && lane >= 1 && (r >= 1 || by == 0);
        const bool top = r == R - 1, up_ok = jc + 1 < ny;
        const long long sy = a.sy, sz = a.sz;
        long long idx = (long long)k0 * sz + (long long)jc * sy + ic;
        float dc = a.din[idx], hc = a.Hf[idx];
        float Dc = HASD ? a.Df[idx] : 0.0f, Db = 0.0f;
        float wzb = 0.0f, uzb = 0.0f;
        if (upd) {
            Db = HASD ? a.Df[idx - sz] : 0.0f;
            wzb = rb_face<MODEL, CHECK>(a, a.din[idx - sz], dc, a.Hf[idx - sz], hc, Db, Dc, a.win[2][idx - sz],
                                        a.tb[2][idx - sz], uzb);
            if (k0 == 1) a.wout[2][idx - sz] = wzb;
        }
        int p = 0;
        sd[0][r][lane] = dc;
        sh[0][r][lane] = hc;
        if (HASD) sD[0][r][lane] = Dc;
        __syncthreads();
        for (int k = k0; k < k1; ++k, idx += sz) {
            const float dn = a.din[idx + sz], hn = a.Hf[idx + sz];
            const float wx = a.win[0][idx], wy = a.win[1][idx], wz = a.win[2][idx];
            const float tbx = a.tb[0][idx], tby = a.tb[1][idx], tbz = a.tb[2][idx], rb = a.Rb[idx];
            const float Dn = HASD ? a.Df[idx + sz] : 0.0f;
            float du, hu, Du = 0.0f;
            if (!top) {
                du = sd[p][r + 1][lane];
                hu = sh[p][r + 1][lane];
                if (HASD) Du = sD[p][r + 1][lane];
            } else {
                du = up_ok ? a.din[idx + sy] : dc;
                hu = up_ok ? a.Hf[idx + sy] : hc;
                if (HASD) Du = up_ok ? a.Df[idx + sy] : Dc;
            }
            const float Dd = (LS && r >= 1) ? sD[p][r - 1][lane] : 0.0f;
            float dr = __shfl_down_sync(FULL, dc, 1);
            float hr = __shfl_down_sync(FULL, hc, 1);
            float Dr = HASD ? __shfl_down_sync(FULL, Dc, 1) : 0.0f;
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                dr = ok ? a.din[idx + 1] : dc;
                hr = ok ? a.Hf[idx + 1] : hc;
                if (HASD) Dr = ok ? a.Df[idx + 1] : Dc;
            }
            float ux = 0.0f, uy = 0.0f, uz = 0.0f, wxn = 0.0f, wyn = 0.0f, wzn = 0.0f;
            if (xface) wxn = rb_face<MODEL, CHECK>(a, dc, dr, hc, hr, Dc, Dr, wx, tbx, ux);
            if (yface) wyn = rb_face<MODEL, CHECK>(a, dc, du, hc, hu, Dc, Du, wy, tby, uy);
            if (upd) wzn = rb_face<MODEL, CHECK>(a, dc, dn, hc, hn, Dc, Dn, wz, tbz, uz);
            if (own_x) a.wout[0][idx] = wxn;
            if (own_y) a.wout[1][idx] = wyn;
            if (upd) a.wout[2][idx] = wzn;
            const float wxl = __shfl_up_sync(FULL, wxn, 1);
            const float uxl = CHECK ? __shfl_up_sync(FULL, ux, 1) : 0.0f;
            const float Dl = HASD ? __shfl_up_sync(FULL, Dc, 1) : 0.0f;
            sw[p][r][lane] = wyn;
            if (CHECK) su[p][r][lane] = uy;
            sd[p ^ 1][r][lane] = dn;
            sh[p ^ 1][r][lane] = hn;
            if (HASD) sD[p ^ 1][r][lane] = Dn;
            __syncthreads();
            if (upd) {
                const float wyb = sw[p][r - 1][lane];
                const float e = rb_cell_e<MODEL>(
                    a, hc + dc, LS ? fmaxf(fmaxf(fmaxf(Dc, Dl), fmaxf(Dr, Du)), fmaxf(fmaxf(Dd, Db), Dn)) : Dc);
                const float div = fmaf(wzn - wzb, a.sig[2], fmaf(wyn - wyb, a.sig[1], (wxn - wxl) * a.sig[0]));
                const float dnew = fmaf(-e, fmaf(dc, a.rdt, rb + div), dc);
                a.dout[idx] = dnew;
                if (CHECK) {
                    const float uyb = su[p][r - 1][lane];
                    const float divu = fmaf(uz - uzb, a.sig[2], fmaf(uy - uyb, a.sig[1], (ux - uxl) * a.sig[0]));
                    // 3D: the FP64 pipe, otherwise idle in this kernel, forms and sums the
                    // residual from an FP64 base term (an FP32 residual, or an FP32 base term
                    // widened here, made the 512^3 step 7-16 ms longer)
                    accumulate_residual(a.Cb64[idx] + (double)divu - (double)dnew * (double)a.rdt, part, pmax);
                }
            }
            dc = dn;
            hc = hn;
            wzb = wzn;
            uzb = uz;
            if (HASD) {
                Db = Dc;
                Dc = Dn;
            }
            p ^= 1;
        }
    }
}

// ---------------------------------------------------------------------------
// 3D, two iterations per launch (temporal blocking in z, LIN and NONLIN).
// The tile is R warps (y rows) x 32 lanes (x columns): lane L <-> column
// 28 bx + L - 1, row r <-> row (R-4) by + r - 1.  The first iteration (level 1)
// updates lanes 1..30 x rows 1..R-2 and runs one plane ahead of the second
// (level 2), which updates lanes 2..29 x rows 2..R-3 (28 x (R-4) cells) from
// the level-1 values: x neighbours by shuffles, y neighbours through shared
// memory, z neighbours in registers.  Step k of the march does level 1 at
// plane k+1 and level 2 at plane k, with two barriers (after the level-1
// faces; after the level-2 faces); the march starts two planes below the
// chunk (one at the bottom boundary) so that level 1 is in place where level
// 2 needs it.  Each iteration's arithmetic is rb3d_body's, operation for
// operation, so a launch gives the iterates of two one-iteration launches.
// A launch reads and writes each field once for two iterations: 26 bytes per
// cell-iteration instead of 52.  Every row and lane evaluates both levels
// (the halo rows' results are discarded): measured at 512^3, 1225 us per
// iteration against 1244 us one iteration per launch -- the 28 x 12 of 32 x 16
// cells that a tile updates at level 2 make the launch issue-bound, which
// takes back almost all of the halved bytes.  (Skipping the halo rows' unused
// work per warp, with the x and y faces of a level as one FP32x2 evaluation,
// was slower: 1365 us.)
template <int MODEL, bool CHECK, int R>
__device__ __forceinline__ void rb3d_tb2_body(const RbArgs& a, int bx, int by, int bz, int chunk, double& part,
                                              unsigned long long& pmax)
{
    static_assert(MODEL == LIN || MODEL == NONLIN, "the 3D two-iteration kernel serves LIN and NONLIN");
    __shared__ float sdi[2][R][32];   // level-1 input delta of a plane (row above)
    __shared__ float shi[2][R][32];   // H_b (FP32) of a plane (row above)
    __shared__ float sd1[2][R][32];   // level-1 result delta' of a plane (row above)
    __shared__ float sy1[R][32];      // level-1 y face (row below)
    __shared__ float sy2[R][32];      // level-2 y face (row below)
    __shared__ float su2[CHECK ? R : 1][32];
    const int lane = threadIdx.x, r = threadIdx.y;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int i = 28 * bx + lane - 1, j = (R - 4) * by + r - 1;
    const int k0 = 1 + bz * chunk;
    const int k1 = min(k0 + chunk, nz - 1);
    if (k0 >= k1) return;   // uniform over the block
    const int ic = min(max(i, 0), nx - 1), jc = min(max(j, 0), ny - 1);
    const bool colin = i >= 1 && i <= nx - 2, rowin = j >= 1 && j <= ny - 2;
    const bool upd1 = colin && rowin && lane >= 1 && lane <= 30 && r >= 1 && r <= R - 2;
    const bool lv2 = lane >= 2 && lane <= 29 && r >= 2 && r <= R - 3;   // level-2 cell of the tile
    const bool upd2 = lv2 && colin && rowin;
    // level-2 faces stored: x faces of lanes 1..28 (lane 29's face is the next
    // tile's lane-1 face) and the grid's last face; y faces of rows 1..R-4
    // likewise; z faces of the level-2 cells
    const bool xf2 = i >= 0 && i <= nx - 2 && lane >= 1 && lane <= 29 && r >= 2 && r <= R - 3 && rowin;
    const bool own_x = xf2 && (lane <= 28 || i == nx - 2);
    const bool yf2 = j >= 0 && j <= ny - 2 && r >= 1 && r <= R - 3 && lane >= 2 && lane <= 29 && colin;
    const bool own_y = yf2 && (r <= R - 4 || j == ny - 2);
    const long long sz = a.sz;
    const long long col = (long long)jc * a.sy + ic;
    const float s0 = a.sig[0], s1 = a.sig[1], s2 = a.sig[2], rdt = a.rdt;
    const bool up = r < R - 1;
    float u;

    // ---- start state: planes ks and ks+1 (ks = k0-2, or 0 at the bottom)
    const int ks = k0 >= 2 ? k0 - 2 : 0;
    long long o0 = (long long)ks * sz + col;
    float p0 = a.din[o0];                 // delta' of plane ks: exact at the boundary plane, else unused
    float h0 = a.Hf[o0];
    float d1 = a.din[o0 + sz], h1 = a.Hf[o0 + sz];
    float tbz0 = a.tb[2][o0];
    float wz1b = rb_face<MODEL, false>(a, p0, d1, h0, h1, 0.0f, 0.0f, a.win[2][o0], tbz0, u);   // level 1, ks+1/2
    float wx1p = 0.0f, wy1p = 0.0f, tbx0 = 0.0f, tby0 = 0.0f, rb0 = 0.0f, hu0 = h0;
    float wz2b = 0.0f, uz2b = 0.0f;
    sdi[(ks + 1) & 1][r][lane] = d1;
    shi[(ks + 1) & 1][r][lane] = h1;
    sd1[ks & 1][r][lane] = p0;
    __syncthreads();
    for (int k = ks; k < k1; ++k, o0 += sz) {
        const int kn = k + 1;                 // level-1 plane
        const bool l1 = kn <= nz - 2;         // interior: updated at level 1, plane kn+1 exists
        const long long on = o0 + sz;
        // ---- A: inputs of plane kn, level-1 faces there
        float d2 = d1, h2 = h1;
        if (l1) {
            d2 = a.din[on + sz];
            h2 = a.Hf[on + sz];
        }
        const float wx = a.win[0][on], wy = a.win[1][on], wz = a.win[2][on];
        const float tbx1 = a.tb[0][on], tby1 = a.tb[1][on], tbz1 = a.tb[2][on], rb1 = a.Rb[on];
        const float du = up ? sdi[kn & 1][r + 1][lane] : d1;
        const float hu = up ? shi[kn & 1][r + 1][lane] : h1;
        const float d1r = __shfl_down_sync(FULL, d1, 1);
        const float h1r = __shfl_down_sync(FULL, h1, 1);
        const float wx1 = rb_face<MODEL, false>(a, d1, d1r, h1, h1r, 0.0f, 0.0f, wx, tbx1, u);
        const float wy1 = rb_face<MODEL, false>(a, d1, du, h1, hu, 0.0f, 0.0f, wy, tby1, u);
        const float wz1 = rb_face<MODEL, false>(a, d1, d2, h1, h2, 0.0f, 0.0f, wz, tbz1, u);   // kn+1/2
        sy1[r][lane] = wy1;
        sdi[(kn + 1) & 1][r][lane] = d2;
        shi[(kn + 1) & 1][r][lane] = h2;
        __syncthreads();
        // ---- B: level-1 update of plane kn; level-2 faces of plane k
        const float wy1b = r >= 1 ? sy1[r - 1][lane] : 0.0f;
        const float wx1l = __shfl_up_sync(FULL, wx1, 1);
        float p1 = d1;
        if (l1 && upd1) {
            const float e = rb_cell_e<MODEL>(a, h1 + d1, 0.0f);
            const float div = fmaf(wz1 - wz1b, s2, fmaf(wy1 - wy1b, s1, (wx1 - wx1l) * s0));
            p1 = fmaf(-e, fmaf(d1, rdt, rb1 + div), d1);
        }
        sd1[kn & 1][r][lane] = p1;
        const float p0r = __shfl_down_sync(FULL, p0, 1);
        const float h0r = __shfl_down_sync(FULL, h0, 1);
        const float p0u = up ? sd1[k & 1][r + 1][lane] : p0;
        float ux2 = 0.0f, uy2 = 0.0f, uz2 = 0.0f;
        const float wx2 = rb_face<MODEL, CHECK>(a, p0, p0r, h0, h0r, 0.0f, 0.0f, wx1p, tbx0, ux2);
        const float wy2 = rb_face<MODEL, CHECK>(a, p0, p0u, h0, hu0, 0.0f, 0.0f, wy1p, tby0, uy2);
        const float wz2 = rb_face<MODEL, CHECK>(a, p0, p1, h0, h1, 0.0f, 0.0f, wz1b, tbz0, uz2);   // k+1/2
        sy2[r][lane] = wy2;
        if (CHECK) su2[r][lane] = uy2;
        __syncthreads();
        // ---- C: level-2 update of plane k
        const float wx2l = __shfl_up_sync(FULL, wx2, 1);
        const float ux2l = CHECK ? __shfl_up_sync(FULL, ux2, 1) : 0.0f;
        if (k >= k0) {   // uniform over the block
            const float wy2b = r >= 1 ? sy2[r - 1][lane] : 0.0f;
            if (upd2) {
                const float e = rb_cell_e<MODEL>(a, h0 + p0, 0.0f);
                const float div = fmaf(wz2 - wz2b, s2, fmaf(wy2 - wy2b, s1, (wx2 - wx2l) * s0));
                const float q = fmaf(-e, fmaf(p0, rdt, rb0 + div), p0);
                a.dout[o0] = q;
                a.wout[2][o0] = wz2;
                if (CHECK) {
                    const float uy2b = su2[r - 1][lane];
                    const float divu = fmaf(uz2 - uz2b, s2, fmaf(uy2 - uy2b, s1, (ux2 - ux2l) * s0));
                    accumulate_residual(a.Cb64[o0] + (double)divu - (double)q * (double)rdt, part, pmax);
                }
            }
            if (own_x) a.wout[0][o0] = wx2;
            if (own_y) a.wout[1][o0] = wy2;
        } else if (k == 0 && upd2) {
            a.wout[2][o0] = wz2;   // the bottom boundary's face 1/2, owned by the first chunk
        }
        // ---- shift the planes
        p0 = p1;
        h0 = h1;
        d1 = d2;
        h1 = h2;
        hu0 = hu;
        wz1b = wz1;
        wx1p = wx1;
        wy1p = wy1;
        tbx0 = tbx1;
        tby0 = tby1;
        tbz0 = tbz1;
        rb0 = rb1;
        wz2b = wz2;
        uz2b = uz2;
    }
}

// ---------------------------------------------------------------------------
// Rebase, FP64.  Fold the changes of buffer parity `parity` into the base:
// H_b += delta, w_b += omega (positions that are never updated hold zeros),
// and clear both buffers, so that the next iteration may start on either.
struct RbFoldArgs {
    long long n;
    double* H;
    double* wb[3];
    float* d[2];
    float* w[3][2];
    int ndim;
};

__device__ __forceinline__ void rb_fold_elem(const RbFoldArgs& f, int parity, long long t)
{
    // both buffers cleared: the next iteration may start on either parity
    const float* dp = parity ? f.d[1] : f.d[0];
    f.H[t] += (double)dp[t];
    f.d[0][t] = 0.0f;
    f.d[1][t] = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d < f.ndim) {
            const float* wp = parity ? f.w[d][1] : f.w[d][0];
            f.wb[d][t] += (double)wp[t];
            f.w[d][0][t] = 0.0f;
            f.w[d][1][t] = 0.0f;
        }
    }
}

// Base quantities, FP64 (one thread per cell): t_b = w_b + u(H_b) for the
// face to +d of every cell, and for inner cells R_b = (H_b - Hold)/dt +
// div w_b, C_b = div u(H_b) - (H_b - Hold)/dt (its norm into acc64), plus
// H_b as FP32.
struct RbBaseArgs {
    int nx, ny, nz, ndim, model;
    long long sy, sz;
    double rdt;
    double sig[3];
    const double* H;
    const double* Hold;
    const double* wb[3];
    const double* D;
    float* tb[3];
    float* Rb;
    float* Cb;           // 1D, 2D: C_b rounded to FP32
    double* Cb64;        // 3D: C_b
    float* Hf;
    double* acc64;
    double* parts;      // per-block slots of the FP64 residual (NULL: atomics into acc64)
    int norm_max;
};

__device__ __forceinline__ double rb_u64(const RbBaseArgs& b, long long cL, long long cR)
{
    const double g = b.H[cR] - b.H[cL];
    if (b.model == LIN) return g;
    if (b.model == LINSTEP) return (b.D[cL] + b.D[cR]) * g;
    const double s = b.H[cL] + b.H[cR];
    if (b.model == NONLIN_EXPM) return (b.D[cL] + b.D[cR]) * (s * s * s) * g;
    return s * s * s * g;
}

// The base quantities of the cell (ix, iy, iz); its check residual goes into
// (part, pmax).
__device__ __forceinline__ void rb_base_cell(const RbBaseArgs& b, int ix, int iy, int iz, double& part,
                                             unsigned long long& pmax)
{
    const long long stp[3] = {1, b.sy, b.sz};
    const int co[3] = {ix, iy, iz};
    const int nn[3] = {b.nx, b.ny, b.nz};
    const long long c = iz * b.sz + iy * b.sy + ix;
    b.Hf[c] = __double2float_rn(b.H[c]);
    bool inner = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) inner = inner && (d >= b.ndim || (co[d] >= 1 && co[d] <= nn[d] - 2));
    double divw = 0.0, divu = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= b.ndim) continue;
        double ur = 0.0;
        if (co[d] <= nn[d] - 2) {
            ur = rb_u64(b, c, c + stp[d]);
            b.tb[d][c] = (float)(b.wb[d][c] + ur);
        }
        if (inner) {
            const double ul = rb_u64(b, c - stp[d], c);
            divw = fma(b.wb[d][c] - b.wb[d][c - stp[d]], b.sig[d], divw);
            divu = fma(ur - ul, b.sig[d], divu);
        }
    }
    if (inner) {
        const double dh = (b.H[c] - b.Hold[c]) * b.rdt;
        b.Rb[c] = (float)(dh + divw);
        const double cb = divu - dh;
        b.Cb[c] = (float)cb;
        accumulate_residual(cb, part, pmax);
    }
}

// ---------------------------------------------------------------------------
// Judges of one grid (one thread).  After each block of nchk iterations: the
// FP32 check err; the phase ends (skip) to confirm err <= tol in FP64, or once
// it has reduced the residual well below its start (the FP32 base quantities
// carry rounding relative to the phase-start residual, which bounds what a
// phase attains), after phase_cap iterations, or when no further check block
// fits before itmax.
__device__ __forceinline__ void rb_check_judge(RbDev* st, double* errhist, int errcap, int nchk, int itmax,
                                               double tol, double norm_den, int norm_max,
                                               int phase_cap = 0x7fffffff)
{
    if (st->skip || st->step_done) return;
    const double acc = st->acc;
    st->acc = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(norm_den);
    const int n = st->nchecks;
    if (errhist && n < errcap) errhist[n] = err;
    st->nchecks = n + 1;
    st->iter += nchk;
    st->phase_iter += nchk;
    st->err = err;
    if (err != err) {
        st->step_done = DONE_NAN;
        st->skip = 1;
        return;
    }
    if (!(err > tol) || err <= 1e-4 * st->err64 || st->phase_iter >= phase_cap) st->skip = 1;
    if (st->iter + nchk > itmax) {    // no further check block fits
        st->skip = 1;
        st->capped = 1;
    }
}

// After each rebase: the FP64 err of the base; the step stops when the last
// FP32 check and the rebased FP64 state are both at tol (or on NaN, or when
// the phase was capped), else the next phase starts.  Returns step_done.
__device__ __forceinline__ int rb_base_judge(RbDev* st, double tol, double norm_den, int norm_max)
{
    if (st->step_done) return st->step_done;
    const double acc = st->acc64;
    st->acc64 = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(norm_den);
    st->err64 = err;
    st->phase_iter = 0;
    if (err != err) {
        st->step_done = DONE_NAN;
        st->skip = 1;
    } else if (st->iter > 0 && !(st->err > tol) && !(err > tol)) {
        st->step_done = DONE_CONVERGED;
    } else if (st->capped) {
        st->step_done = DONE_CAP;
    } else {
        st->skip = 0;
    }
    return st->step_done;
}

__device__ __forceinline__ void rb_reset(RbDev* st)
{
    st->skip = 0;
    st->step_done = DONE_RUNNING;
    st->iter = 0;
    st->phase_iter = 0;
    st->nchecks = 0;
    st->capped = 0;
    st->phases = 0;
    st->blocks = 0;
    st->passes = 0;
    st->acc = 0.0;
    st->acc64 = 0.0;
    st->err = 0.0;
    st->err64 = 0.0;
}

}  // namespace ptd
