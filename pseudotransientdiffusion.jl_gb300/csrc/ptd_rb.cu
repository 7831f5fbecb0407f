// ptd_rb.cu -- FP32 PT iterations on the change since an FP64 base state
// (PTD_PREC_FP32_RB, "rebased" FP32 form).
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
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "ptd_internal.h"

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
    const double* Cb;     // base check residual (FP64: read on check iterations only)
    const float* Hf;      // H_b as FP32 (iteration parameters, u_d)
    const float* Df;      // LINSTEP: D, NONLIN_EXPM: exp(m), as FP32
    const int* skip;
    double* acc;
    int norm_max;
};

struct RbDev {
    int skip;         // PT kernels return at entry: the phase is over or the step done
    int step_done;    // DONE_* of the physical step
    int iter;         // PT iterations of this step
    int phase_iter;   // PT iterations of this phase (the buffer parity)
    int nchecks;
    int capped;
    int phases;       // phases run in this step (passes of the step graph's loop)
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
__device__ __forceinline__ void rb1d_body(const RbArgs& a, int bx, double& part, unsigned long long& pmax)
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
            accumulate_residual(a.Cb[i] + (double)((ur - ul) * a.sig[0]) - (double)dnew * (double)a.rdt, part,
                                pmax);
    }
}

// ---------------------------------------------------------------------------
// 2D: the tiling of ptd_pt_body.cuh (31 updated columns per warp, y march).
template <int MODEL, bool CHECK>
__device__ __forceinline__ void rb2d_body(const RbArgs& a, int tile, int cy, int chunk, double& part,
                                          unsigned long long& pmax)
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
                    accumulate_residual(a.Cb[idx] + (double)divu - (double)dnew * (double)a.rdt, part, pmax);
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
            if (CHECK && j == j1 - 1) warp_flush_residual(a.acc, a.norm_max, part, pmax, lane);
        }
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
__device__ __forceinline__ void rb2d_tb2_body(const RbArgs& a, int tile, int cy, int chunk, double& part,
                                              unsigned long long& pmax)
{
    constexpr bool HASD = MODEL == LINSTEP || MODEL == NONLIN_EXPM;
    const int lane = threadIdx.x;
    const int nx = a.nx, ny = a.ny;
    const int j0 = 1 + cy * chunk;
    const int j1 = min(j0 + chunk, ny - 1);
    if (28 * tile >= nx - 2 || j0 >= j1) return;   // uniform over the warp
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
                accumulate_residual(a.Cb[os] + (double)divu - (double)q * (double)rdt, part, pmax);
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
        if (CHECK && s == j1 - 1) warp_flush_residual(a.acc, a.norm_max, part, pmax, lane);
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
                    accumulate_residual(a.Cb[idx] + (double)divu - (double)dnew * (double)a.rdt, part, pmax);
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

template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) rb1d_kernel(RbArgs a)
{
    if (rb_skip(a.skip)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    rb1d_body<MODEL, CHECK>(a, blockIdx.x, part, pmax);
    if (CHECK) block_reduce_residual(a.acc, a.norm_max, part, pmax);
}

template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256) rb2d_kernel(RbArgs a, int chunk)
{
    if (rb_skip(a.skip)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    // the body flushes its check partials into a.acc (last step of its march)
    rb2d_body<MODEL, CHECK>(a, blockIdx.x * blockDim.y + threadIdx.y, blockIdx.y, chunk, part, pmax);
}

// The plain NONLIN variant is capped at 32 registers (8 CTAs of 256 threads
// per SM; ptxas spills 16 bytes): at its natural 40 the march, bound by
// memory latency, ran at most 48 of 64 warps per SM.  Measured at 4096^2:
// 77.9 -> 76.8 us per iteration.  A minimum of 0 blocks leaves the other
// variants' register allocation as without the bound.
template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(256, (MODEL == NONLIN && !CHECK) ? 8 : 0) rb2d_tb2_kernel(RbArgs a, int chunk)
{
    if (rb_skip(a.skip)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    // the body flushes its check partials into a.acc (last step of its march)
    rb2d_tb2_body<MODEL, CHECK>(a, blockIdx.x * blockDim.y + threadIdx.y, blockIdx.y, chunk, part, pmax);
}

template <int MODEL, bool CHECK>
__global__ void __launch_bounds__(512) rb3d_kernel(RbArgs a, int chunk)
{
    if (rb_skip(a.skip)) return;
    double part = 0.0;
    unsigned long long pmax = 0ull;
    rb3d_body<MODEL, CHECK, 16>(a, blockIdx.x, blockIdx.y, blockIdx.z, chunk, part, pmax);
    if (CHECK) block_reduce_residual(a.acc, a.norm_max, part, pmax);
}

// ---------------------------------------------------------------------------
// Rebase, FP64.  Fold the changes into the base: H_b += delta, w_b += omega
// (positions that are never updated hold zeros), and clear the buffers the
// next phase starts from (parity 0).  parity < 0: the buffers of the phase's
// own parity (RbDev::phase_iter, tb iterations per launch).
struct RbFoldArgs {
    long long n;
    double* H;
    double* wb[3];
    float* d[2];
    float* w[3][2];
    int ndim;
};

__global__ void rb_fold_kernel(RbFoldArgs f, const RbDev* st, int parity, int tb)
{
    if (parity < 0) {
        if (st->step_done) return;
        parity = (st->phase_iter / tb) & 1;   // one buffer swap per launch of tb iterations
    }
    const float* dp = parity ? f.d[1] : f.d[0];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < f.n;
         t += (long long)gridDim.x * blockDim.x) {
        f.H[t] += (double)dp[t];
        f.d[0][t] = 0.0f;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (d < f.ndim) {
                const float* wp = parity ? f.w[d][1] : f.w[d][0];
                f.wb[d][t] += (double)wp[t];
                f.w[d][0][t] = 0.0f;
            }
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
    double* Cb;
    float* Hf;
    double* acc64;
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

__global__ void __launch_bounds__(256) rb_base_kernel(RbBaseArgs b, const RbDev* st)
{
    if (st && st->step_done) return;
    const long long total = (long long)b.nx * b.ny * b.nz;
    const long long stp[3] = {1, b.sy, b.sz};
    double part = 0.0;
    unsigned long long pmax = 0ull;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(t % b.nx);
        const long long rest = t / b.nx;
        const int iy = (int)(rest % b.ny);
        const int iz = (int)(rest / b.ny);
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
            b.Cb[c] = cb;
            accumulate_residual(cb, part, pmax);
        }
    }
    block_reduce_residual(b.acc64, b.norm_max, part, pmax);
}

__global__ void rb_reset_kernel(RbDev* st)
{
    st->skip = 0;
    st->step_done = DONE_RUNNING;
    st->iter = 0;
    st->phase_iter = 0;
    st->nchecks = 0;
    st->capped = 0;
    st->phases = 0;
    st->acc = 0.0;
    st->acc64 = 0.0;
    st->err = 0.0;
    st->err64 = 0.0;
}

// After each block of nchk iterations: the FP32 check err.
__global__ void rb_check_judge_kernel(RbDev* st, double* errhist, int errcap, int nchk, int itmax, double tol,
                                      double norm_den, int norm_max)
{
    if (st->skip || st->step_done) return;
    const double acc = st->acc;
    st->acc = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(norm_den);
    const int n = st->nchecks;
    if (n < errcap) errhist[n] = err;
    st->nchecks = n + 1;
    st->iter += nchk;
    st->phase_iter += nchk;
    st->err = err;
    if (err != err) {
        st->step_done = DONE_NAN;
        st->skip = 1;
        return;
    }
    // rebase: to confirm err <= tol in FP64, or once the phase has reduced the
    // residual well below its start (the FP32 base quantities carry rounding
    // relative to the phase-start residual, which bounds what a phase attains)
    if (!(err > tol) || err <= 1e-4 * st->err64) st->skip = 1;
    if (st->iter + nchk > itmax) {    // no further check block fits
        st->skip = 1;
        st->capped = 1;
    }
}

// After each rebase: the FP64 err of the base.  In the body of the step
// graph's WHILE node (in_loop) it also counts the phase and ends the loop
// once the step has stopped.  Every phase adds at least one check block of
// nchk iterations (its first judge runs with skip clear) and a phase that
// leaves no room for another block before itmax ends the step (capped), so
// the loop ends within itmax/nchk passes.
__global__ void rb_base_judge_kernel(RbDev* st, double tol, double norm_den, int norm_max,
                                     cudaGraphConditionalHandle loop, int in_loop)
{
    if (in_loop) st->phases += 1;
    if (st->step_done) {
        if (in_loop) cudaGraphSetConditional(loop, 0);
        return;
    }
    const double acc = st->acc64;
    st->acc64 = 0.0;
    const double err = norm_max ? acc : sqrt(acc) / sqrt(norm_den);
    st->err64 = err;
    st->phase_iter = 0;
    if (err != err) {
        st->step_done = DONE_NAN;
        st->skip = 1;
    } else if (st->iter > 0 && !(st->err > tol) && !(err > tol)) {
        st->step_done = DONE_CONVERGED;   // the last check and the rebased FP64 state both at tol
    } else if (st->capped) {
        st->step_done = DONE_CAP;
    } else {
        st->skip = 0;
    }
    if (in_loop && st->step_done) cudaGraphSetConditional(loop, 0);
}

__global__ void rb_tofloat_kernel(const double* src, float* dst, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        dst[t] = __double2float_rn(src[t]);
}

// ---------------------------------------------------------------------------
struct RbState {
    ptd_params p;
    Derived dv;
    LaunchCfg cfg;
    ptd_ctx_base g;
    cudaStream_t s = nullptr;
    float* d[2] = {nullptr, nullptr};
    float* w[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    float* tb[3] = {nullptr, nullptr, nullptr};
    float* Rb = nullptr;
    double* Cb = nullptr;
    float* Hf = nullptr;
    float* Df = nullptr;
    double* H = nullptr;                          // owned by the context: the base H_b
    double* Hold = nullptr;                       // owned by the context
    double* wb[3] = {nullptr, nullptr, nullptr};  // owned by the context: the base fluxes
    const double* D = nullptr;                    // owned by the context (LINSTEP)
    RbDev* dev = nullptr;
    RbDev* h_dev = nullptr;
    int* zero_flag = nullptr;
    double* errhist = nullptr;
    int errcap = 0;
    int blocks_per_phase = 1;
    int tblk = 1;                                 // iterations per launch (2: temporal blocking, 2D)
    cudaGraphExec_t gphase = nullptr;
    int kernels_per_phase = 0;
    DcCounters k;
};

namespace {

#define RCK(call)                                                 \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);       \
    } while (0)

void rb_args(const RbState* rb, int parity, const int* skip, RbArgs& a)
{
    std::memset(&a, 0, sizeof(a));
    a.nx = rb->g.nx;
    a.ny = rb->g.ny;
    a.nz = rb->g.nz;
    a.sy = rb->g.sy;
    a.sz = rb->g.sz;
    a.rdt = (float)rb->dv.rdt;
    for (int d = 0; d < 3; ++d) a.sig[d] = (float)rb->dv.sig[d];
    a.c_lin = (float)rb->dv.c_lin;
    a.e_lin = (float)rb->dv.e_lin;
    a.f = fparams(rb->dv);
    a.din = rb->d[parity];
    a.dout = rb->d[parity ^ 1];
    for (int d = 0; d < 3; ++d) {
        const int dd = rb->w[d][0] ? d : 0;
        a.win[d] = rb->w[dd][parity];
        a.wout[d] = rb->w[dd][parity ^ 1];
        a.tb[d] = rb->tb[rb->tb[d] ? d : 0];
    }
    a.Rb = rb->Rb;
    a.Cb = rb->Cb;
    a.Hf = rb->Hf;
    a.Df = rb->Df;
    a.skip = skip;
    a.acc = &rb->dev->acc;
    a.norm_max = rb->p.norm == PTD_NORM_MAX;
}

template <int MODEL, bool CHECK>
cudaError_t rb_launch_model(const RbArgs& a, int ndim, const LaunchCfg& cfg, cudaStream_t s, int tb)
{
    if (ndim == 1) {
        rb1d_kernel<MODEL, CHECK><<<(a.nx + 255) / 256, 256, 0, s>>>(a);
    } else if (ndim == 2 && tb == 2) {
        // twice the configured rows per y march: the march starts with two
        // extra level-1 rows (4096^2 nonlinear, 2 warps: 87.2 us per
        // iteration at 16 rows, 85.9 at 32, 86.0 at 64)
        const int W = cfg.warps2d, chunk = 2 * cfg.chunk2d;
        const int tiles = (a.nx - 2 + 27) / 28;
        dim3 grid((tiles + W - 1) / W, (a.ny - 2 + chunk - 1) / chunk);
        rb2d_tb2_kernel<MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, chunk);
    } else if (ndim == 2) {
        const int W = cfg.warps2d;
        const int tiles = (a.nx - 2 + 30) / 31;
        dim3 grid((tiles + W - 1) / W, (a.ny - 2 + cfg.chunk2d - 1) / cfg.chunk2d);
        rb2d_kernel<MODEL, CHECK><<<grid, dim3(32, W), 0, s>>>(a, cfg.chunk2d);
    } else {
        const int tx = (a.nx - 2 + 30) / 31;
        dim3 grid(tx, (a.ny - 2 + 14) / 15, (a.nz - 2 + cfg.chunk3d - 1) / cfg.chunk3d);
        rb3d_kernel<MODEL, CHECK><<<grid, dim3(32, 16), 0, s>>>(a, cfg.chunk3d);
    }
    return cudaGetLastError();
}

// One launch of tb PT iterations (tb = 2: 2D only).
cudaError_t rb_launch(const RbArgs& a, int ndim, int model, bool check, const LaunchCfg& cfg, cudaStream_t s,
                      int tb = 1)
{
    switch (model * 2 + (check ? 1 : 0)) {
    case 0: return rb_launch_model<LIN, false>(a, ndim, cfg, s, tb);
    case 1: return rb_launch_model<LIN, true>(a, ndim, cfg, s, tb);
    case 2: return rb_launch_model<LINSTEP, false>(a, ndim, cfg, s, tb);
    case 3: return rb_launch_model<LINSTEP, true>(a, ndim, cfg, s, tb);
    case 4: return rb_launch_model<NONLIN, false>(a, ndim, cfg, s, tb);
    case 5: return rb_launch_model<NONLIN, true>(a, ndim, cfg, s, tb);
    case 6: return rb_launch_model<NONLIN_EXPM, false>(a, ndim, cfg, s, tb);
    case 7: return rb_launch_model<NONLIN_EXPM, true>(a, ndim, cfg, s, tb);
    }
    return cudaErrorInvalidValue;
}

// niter PT iterations without checks from buffer parity 0 (pairs per launch
// when temporal blocking is on); returns the parity of the result.
cudaError_t rb_run_plain(const RbState* rb, int32_t niter, const int* skip, int& par, long long& launches)
{
    par = 0;
    for (int32_t it = 0; it < niter;) {
        const int tb = (rb->tblk == 2 && niter - it >= 2) ? 2 : 1;
        RbArgs a;
        rb_args(rb, par, skip, a);
        cudaError_t e = rb_launch(a, rb->p.ndim, rb->p.model, false, rb->cfg, rb->s, tb);
        if (e != cudaSuccess) return e;
        par ^= 1;
        ++launches;
        it += tb;
    }
    return cudaSuccess;
}

RbFoldArgs fold_args(const RbState* rb)
{
    RbFoldArgs f;
    std::memset(&f, 0, sizeof(f));
    f.n = rb->g.nfield;
    f.H = rb->H;
    f.ndim = rb->p.ndim;
    f.d[0] = rb->d[0];
    f.d[1] = rb->d[1];
    for (int d = 0; d < rb->p.ndim; ++d) {
        f.wb[d] = rb->wb[d];
        f.w[d][0] = rb->w[d][0];
        f.w[d][1] = rb->w[d][1];
    }
    return f;
}

RbBaseArgs base_args(const RbState* rb)
{
    RbBaseArgs b;
    std::memset(&b, 0, sizeof(b));
    b.nx = rb->g.nx;
    b.ny = rb->g.ny;
    b.nz = rb->g.nz;
    b.ndim = rb->p.ndim;
    b.model = rb->p.model;
    b.sy = rb->g.sy;
    b.sz = rb->g.sz;
    b.rdt = rb->dv.rdt;
    for (int d = 0; d < 3; ++d) b.sig[d] = rb->dv.sig[d];
    b.H = rb->H;
    b.Hold = rb->Hold;
    for (int d = 0; d < rb->p.ndim; ++d) {
        b.wb[d] = rb->wb[d];
        b.tb[d] = rb->tb[d];
    }
    b.D = rb->D;
    b.Rb = rb->Rb;
    b.Cb = rb->Cb;
    b.Hf = rb->Hf;
    b.acc64 = &rb->dev->acc64;
    b.norm_max = rb->p.norm == PTD_NORM_MAX;
    return b;
}

// The rebased PT iteration of one physical step as one CUDA graph: a WHILE
// node whose body is one phase -- blocks of nchk iterations each followed by
// the FP32 judge, then the rebase (fold, base quantities, FP64 judge) -- and
// which the FP64 judge ends when the step stops.  Every phase starts from
// buffer parity 0.
int rb_capture(RbState* rb)
{
    cudaGraph_t g = nullptr;
    RCK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle loop;
    cudaError_t err = cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = loop;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (err == cudaSuccess) err = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    if (err != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err, "conditional graph node");
    }
    cudaGraph_t body = np.conditional.phGraph_out[0];
    err = cudaStreamBeginCaptureToGraph(rb->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (err != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err, "cudaStreamBeginCaptureToGraph");
    }
    int par = 0, nk = 0;
    const int nchk = rb->p.nchk;
    const int nl = nchk / rb->tblk;   // launches per check block (tb divides nchk)
    for (int b = 0; b < rb->blocks_per_phase && err == cudaSuccess; ++b) {
        for (int it = 0; it < nl && err == cudaSuccess; ++it) {
            RbArgs a;
            rb_args(rb, par, &rb->dev->skip, a);
            err = rb_launch(a, rb->p.ndim, rb->p.model, it == nl - 1, rb->cfg, rb->s, rb->tblk);
            par ^= 1;
            ++nk;
        }
        if (err == cudaSuccess) {
            rb_check_judge_kernel<<<1, 1, 0, rb->s>>>(rb->dev, rb->errhist, rb->errcap, nchk, rb->p.itmax,
                                                      rb->p.tol, rb->dv.norm_den, rb->p.norm == PTD_NORM_MAX);
            err = cudaGetLastError();
            ++nk;
        }
    }
    if (err == cudaSuccess) {
        rb_fold_kernel<<<fill_blocks(), 256, 0, rb->s>>>(fold_args(rb), rb->dev, -1, rb->tblk);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) {
        rb_base_kernel<<<fill_blocks(), 256, 0, rb->s>>>(base_args(rb), rb->dev);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) {
        rb_base_judge_kernel<<<1, 1, 0, rb->s>>>(rb->dev, rb->p.tol, rb->dv.norm_den, rb->p.norm == PTD_NORM_MAX,
                                                 loop, 1);
        err = cudaGetLastError();
    }
    nk += 3;
    cudaError_t e2 = cudaStreamEndCapture(rb->s, &body);
    if (err != cudaSuccess || e2 != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(err != cudaSuccess ? err : e2, "capture rebased phase");
    }
    cudaError_t e3 = cudaGraphInstantiate(&rb->gphase, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return cuda_fail(e3, "cudaGraphInstantiate");
    rb->kernels_per_phase = nk;
    return PTD_OK;
}

}  // namespace

int rb_create(const ptd_ctx_base& g, const ptd_params& p, const Derived& dv, cudaStream_t s, RbState** out)
{
    *out = nullptr;
    RbState* rb = new (std::nothrow) RbState();
    if (!rb) return set_error(PTD_ENOMEM, "rb_create: host allocation failed");
    rb->p = p;
    rb->dv = dv;
    rb->g = g;
    rb->s = s;
    rb->cfg = tuned_config(p);
    // a phase: the check blocks of ~200 PT iterations between two FP64 rebases
    rb->blocks_per_phase = std::max(1, (200 + p.nchk - 1) / p.nchk);
    rb->tblk = (p.ndim == 2 && p.nchk % 2 == 0 && !(p.flags & PTD_FLAG_DC_NO_TBLOCK)) ? 2 : 1;
    rb->errcap = (p.nchk <= p.itmax ? p.itmax / p.nchk : 0) + 2;
    const size_t fb = (size_t)g.nfield * sizeof(float);
    auto alloc = [&](void** ptr, size_t n) -> int {
        cudaError_t e = cudaMalloc(ptr, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(e == cudaErrorMemoryAllocation ? PTD_ENOMEM : PTD_ECUDA, "rb: cudaMalloc failed");
        }
        return PTD_OK;
    };
    int rc = alloc((void**)&rb->d[0], fb);
    if (!rc) rc = alloc((void**)&rb->d[1], fb);
    for (int d = 0; d < p.ndim && !rc; ++d) {
        for (int q = 0; q < 2 && !rc; ++q) rc = alloc((void**)&rb->w[d][q], fb);
        if (!rc) rc = alloc((void**)&rb->tb[d], fb);
    }
    if (!rc) rc = alloc((void**)&rb->Rb, fb);
    if (!rc) rc = alloc((void**)&rb->Cb, (size_t)g.nfield * sizeof(double));
    if (!rc) rc = alloc((void**)&rb->Hf, fb);
    if (!rc && (p.model == PTD_MODEL_LINSTEP || p.model == PTD_MODEL_NONLIN_EXPM)) rc = alloc((void**)&rb->Df, fb);
    if (!rc) rc = alloc((void**)&rb->dev, sizeof(RbDev));
    if (!rc) rc = alloc((void**)&rb->zero_flag, sizeof(int));
    if (!rc) rc = alloc((void**)&rb->errhist, (size_t)rb->errcap * sizeof(double));
    if (!rc && cudaMallocHost((void**)&rb->h_dev, sizeof(RbDev)) != cudaSuccess) {
        cudaGetLastError();
        rc = set_error(PTD_ENOMEM, "rb: cudaMallocHost failed");
    }
    if (!rc) {
        cudaError_t e = cudaMemsetAsync(rb->dev, 0, sizeof(RbDev), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(rb->zero_flag, 0, sizeof(int), s);
        for (int q = 0; q < 2 && e == cudaSuccess; ++q) e = cudaMemsetAsync(rb->d[q], 0, fb, s);
        for (int d = 0; d < p.ndim && e == cudaSuccess; ++d) {
            for (int q = 0; q < 2 && e == cudaSuccess; ++q) e = cudaMemsetAsync(rb->w[d][q], 0, fb, s);
            // faces past the last one of each direction are read (never used) by the halo lanes
            if (e == cudaSuccess) e = cudaMemsetAsync(rb->tb[d], 0, fb, s);
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(rb->Rb, 0, fb, s);
        if (e != cudaSuccess) rc = cuda_fail(e, "rb: cudaMemsetAsync");
    }
    if (rc) {
        rb_destroy(rb);
        return rc;
    }
    *out = rb;
    return PTD_OK;
}

void rb_destroy(RbState* rb)
{
    if (!rb) return;
    if (rb->s) cudaStreamSynchronize(rb->s);
    if (rb->gphase) cudaGraphExecDestroy(rb->gphase);
    cudaFree(rb->d[0]);
    cudaFree(rb->d[1]);
    for (int d = 0; d < 3; ++d) {
        cudaFree(rb->w[d][0]);
        cudaFree(rb->w[d][1]);
        cudaFree(rb->tb[d]);
    }
    cudaFree(rb->Rb);
    cudaFree(rb->Cb);
    cudaFree(rb->Hf);
    cudaFree(rb->Df);
    cudaFree(rb->dev);
    cudaFree(rb->zero_flag);
    cudaFree(rb->errhist);
    if (rb->h_dev) cudaFreeHost(rb->h_dev);
    delete rb;
}

// The context's FP64 fields become the base: H_b = H, w_b = W (zeroed by the
// caller), Hold; the FP32 changes start at zero.
int rb_set_state(RbState* rb, double* H, double* Hold, double* const* wb, const double* D, cudaStream_t s)
{
    rb->H = H;
    rb->Hold = Hold;
    for (int d = 0; d < rb->p.ndim; ++d) rb->wb[d] = wb[d];
    rb->D = D;
    const size_t fb = (size_t)rb->g.nfield * sizeof(float);
    for (int q = 0; q < 2; ++q) RCK(cudaMemsetAsync(rb->d[q], 0, fb, s));
    for (int d = 0; d < rb->p.ndim; ++d)
        for (int q = 0; q < 2; ++q) RCK(cudaMemsetAsync(rb->w[d][q], 0, fb, s));
    if (rb->Df) {
        rb_tofloat_kernel<<<fill_blocks(), 256, 0, s>>>(D, rb->Df, rb->g.nfield);
        RCK(cudaGetLastError());
    }
    if (!rb->gphase) {
        int rc = rb_capture(rb);
        if (rc) return rc;
    }
    return PTD_OK;
}

int rb_step(RbState* rb, int32_t* iters, double* err_hist, int32_t err_cap, int32_t* n_err, int* nan_flag,
            int* capped)
{
    rb_reset_kernel<<<1, 1, 0, rb->s>>>(rb->dev);
    RCK(cudaGetLastError());
    rb_base_kernel<<<fill_blocks(), 256, 0, rb->s>>>(base_args(rb), rb->dev);
    RCK(cudaGetLastError());
    rb_base_judge_kernel<<<1, 1, 0, rb->s>>>(rb->dev, rb->p.tol, rb->dv.norm_den, rb->p.norm == PTD_NORM_MAX,
                                             cudaGraphConditionalHandle{}, 0);
    RCK(cudaGetLastError());
    rb->k.launches += 3;
    rb->h_dev->step_done = DONE_RUNNING;
    rb->h_dev->iter = 0;
    rb->h_dev->nchecks = 0;
    if (rb->p.nchk <= rb->p.itmax) {
        // the whole step: phases until the FP64 judge stops it
        RCK(cudaGraphLaunch(rb->gphase, rb->s));
        RCK(cudaMemcpyAsync(rb->h_dev, rb->dev, sizeof(RbDev), cudaMemcpyDeviceToHost, rb->s));
        RCK(cudaStreamSynchronize(rb->s));
        rb->k.launches += (long long)rb->h_dev->phases * rb->kernels_per_phase;
    }
    const RbDev& st = *rb->h_dev;
    int32_t iter = st.iter;
    *nan_flag = st.step_done == DONE_NAN;
    *capped = st.step_done == DONE_CAP || st.step_done == DONE_RUNNING;
    if (*capped && iter < rb->p.itmax) {
        // no further check block fits (or nchk > itmax: the perf scripts'
        // fixed iterations): the remaining PT iterations up to itmax without
        // checks, from the folded base, then fold them in
        const int32_t tail = rb->p.itmax - iter;
        int par = 0;
        long long nl = 0;
        RCK(rb_run_plain(rb, tail, rb->zero_flag, par, nl));
        rb_fold_kernel<<<fill_blocks(), 256, 0, rb->s>>>(fold_args(rb), rb->dev, par, 1);
        RCK(cudaGetLastError());
        rb->k.launches += nl + 1;
        iter = rb->p.itmax;
    }
    *iters = iter;
    rb->k.iterations += iter;
    if (err_hist && st.nchecks > 0 && *n_err < err_cap) {
        const int k = std::min(st.nchecks, std::min(err_cap - *n_err, rb->errcap));
        RCK(cudaMemcpyAsync(err_hist + *n_err, rb->errhist, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost,
                            rb->s));
        *n_err += k;
    } else if (st.nchecks > 0 && *n_err < err_cap) {
        *n_err += std::min(st.nchecks, err_cap - *n_err);
    }
    RCK(cudaMemcpyAsync(rb->Hold, rb->H, (size_t)rb->g.nfield * sizeof(double), cudaMemcpyDeviceToDevice,
                        rb->s));
    RCK(cudaStreamSynchronize(rb->s));
    return PTD_OK;
}

// Fixed FP32 iterations without checks (perf protocol), then one rebase.
int rb_iterate(RbState* rb, int32_t niter)
{
    rb_base_kernel<<<fill_blocks(), 256, 0, rb->s>>>(base_args(rb), nullptr);
    RCK(cudaGetLastError());
    int par = 0;
    long long nl = 0;
    RCK(rb_run_plain(rb, niter, rb->zero_flag, par, nl));
    rb_fold_kernel<<<fill_blocks(), 256, 0, rb->s>>>(fold_args(rb), rb->dev, par, 1);
    RCK(cudaGetLastError());
    rb->k.launches += nl + 2;
    rb->k.iterations += niter;
    return PTD_OK;
}

int rb_set_config(RbState* rb, const LaunchCfg& cfg)
{
    rb->cfg = cfg;
    if (rb->gphase) {   // captured once the base fields are known (rb_set_state)
        cudaGraphExecDestroy(rb->gphase);
        rb->gphase = nullptr;
        return rb_capture(rb);
    }
    return PTD_OK;
}

DcCounters rb_counters(const RbState* rb) { return rb ? rb->k : DcCounters{}; }

}  // namespace ptd
