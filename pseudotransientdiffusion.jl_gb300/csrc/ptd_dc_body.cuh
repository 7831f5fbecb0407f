// ptd_dc_body.cuh -- FP32 inner PT iteration of the defect-correction solver
// (the linearised operator J = I/dt + d(div q)/dH applied to a correction),
// as bodies callable with explicit tile indices: one grid (ptd_dc.cu) or a
// batch of grids (ptd_batch.cu).  See ptd_dc.cu for the algorithm.
#pragma once

#include "ptd_device.cuh"
#include "ptd_kernels.h"

namespace ptd {

struct DcArgs {
    int nx, ny, nz;
    long long sy, sz;
    float rdt;
    float sig[3];
    float c_lin, e_lin;
    FParams f;
    const float* din;     // correction delta (iteration k)
    float* dout;          // correction delta (iteration k+1)
    const float* win[3];
    float* wout[3];
    const float* Hf;      // FP32 copy of H (linearisation point)
    const float* Df;      // LINSTEP: FP32 copy of D
    const float* r;       // FP32 copy of the FP64 residual
    const int* done;
    double* acc;
    double* parts;        // check-residual slots (fixed-order sum), or null: atomics into acc
    int norm_max;
};

// Control block of the inner solve (device), see DevState in ptd_kernels.h.
struct DcDev {
    int done;
    int nchecks;
    int iter;
    int best_at;       // check index of the smallest inner err so far
    double acc;        // inner residual accumulator
    double err;        // last inner err
    double best;       // smallest inner err so far
    double target;     // inner stopping threshold
    double outer_acc;  // FP64 residual accumulator
    double outer_err;  // FP64 residual norm
    unsigned long long hmax_bits;  // max |H| over the grid (bit pattern), for the FP32 floor
    int cap;           // inner iterations allowed to this inner solve (the step's remaining budget)
    int passes;        // passes of the inner solve graph's loop
};

// One face of the linearised flux (scaled like ptd_device.cuh):
// u = K_f (d_R - d_L) [+ 3 s^2 (h_R - h_L) (d_L + d_R)],  w <- w - c (w + u).
// Every operation explicit, so that the packed two-face form below rounds
// identically (D_f = (s/2)^3 = s^3/8 exactly).
template <int MODEL, bool U>
__device__ __forceinline__ float face32(const DcArgs& a, float dL, float dR, float hL, float hR, float DL,
                                        float DR, float w, float& u)
{
    const float gd = dR - dL;
    float uu, c;
    if (MODEL == LIN) {
        uu = gd;
        c = a.c_lin;
    } else if (MODEL == LINSTEP) {
        uu = __fmul_rn(DL + DR, gd);
        c = a.c_lin;
    } else {
        const float s = hL + hR;
        const float s2 = __fmul_rn(s, s);
        const float s3 = __fmul_rn(s2, s);
        uu = __fmaf_rn(__fmul_rn(__fmul_rn(3.0f, s2), hR - hL), dL + dR, __fmul_rn(s3, gd));
        c = face_c_rn(a.f, __fmul_rn(0.125f, s3));
    }
    if (U) u = uu;
    return __fmaf_rn(-c, w + uu, w);
}

// Two faces (LIN, NONLIN) with FP32x2 flux arithmetic; c stays scalar (its
// constant operands are free in scalar instructions).  3 s^2 is formed as
// (s^2 + s^2) + s^2, which rounds once like 3.0f * s^2.
template <int MODEL, bool U>
__device__ __forceinline__ float2 face32x2(const DcArgs& a, float2 dL, float2 dR, float2 hL, float2 hR, float2 w,
                                           float2& u)
{
    const float2 gd = sub2(dR, dL);
    float2 uu;
    float cx, cy;
    if (MODEL == LIN) {
        uu = gd;
        cx = cy = a.c_lin;
    } else {
        const float2 s = add2(hL, hR);
        const float2 s2 = mul2(s, s);
        const float2 s3 = mul2(s2, s);
        uu = fma2(mul2(add2(add2(s2, s2), s2), sub2(hR, hL)), add2(dL, dR), mul2(s3, gd));
        cx = face_c_rn(a.f, __fmul_rn(0.125f, s3.x));
        cy = face_c_rn(a.f, __fmul_rn(0.125f, s3.y));
    }
    if (U) u = uu;
    return fma2(f2(-cx, -cy), add2(w, uu), w);
}

template <int MODEL>
__device__ __forceinline__ float cell_e32(const DcArgs& a, float h, float dmax)
{
    if (MODEL == LIN) return a.e_lin;
    if (MODEL == LINSTEP) return linstep_cell_e(a.f, dmax);
    return nonlin_cell_e(a.f, h);
}

__device__ __forceinline__ bool dc_done(const int* done) { return __ldcg(done) != 0; }

// ---------------------------------------------------------------------------
template <int MODEL, bool CHECK>
__device__ __forceinline__ void dc1d_body(const DcArgs& a, int bx, float& part, unsigned& pmax)
{
    const int i = bx * blockDim.x + threadIdx.x;
    const int nx = a.nx;
    if (i < nx) {
        const float dc = a.din[i], hc = a.Hf[i];
        const float Dc = MODEL == LINSTEP ? a.Df[i] : 0.0f;
        float wr = 0.0f, ur = 0.0f, Dr = 0.0f;
        if (i <= nx - 2) {
            Dr = MODEL == LINSTEP ? a.Df[i + 1] : 0.0f;
            wr = face32<MODEL, CHECK>(a, dc, a.din[i + 1], hc, a.Hf[i + 1], Dc, Dr, a.win[0][i], ur);
            a.wout[0][i] = wr;
        }
        if (i >= 1 && i <= nx - 2) {
            const float Dl = MODEL == LINSTEP ? a.Df[i - 1] : 0.0f;
            float ul = 0.0f;
            const float wl = face32<MODEL, CHECK>(a, a.din[i - 1], dc, a.Hf[i - 1], hc, Dl, Dc, a.win[0][i - 1], ul);
            const float rr = a.r[i];
            const float e = cell_e32<MODEL>(a, hc, fmaxf(fmaxf(Dl, Dr), Dc));
            const float div = (wr - wl) * a.sig[0];
            const float dn = fmaf(-e, fmaf(dc, a.rdt, div - rr), dc);
            a.dout[i] = dn;
            if (CHECK) accumulate_residual32(fmaf(-dn, a.rdt, rr + (ur - ul) * a.sig[0]), part, pmax);
        }
    }
}

template <int MODEL, bool CHECK>
__device__ __forceinline__ void dc2d_body(const DcArgs& a, int tile, int cy, int chunk, float& part,
                                          unsigned& pmax, long long slot = 0)
{
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
        float Dc = MODEL == LINSTEP ? a.Df[idx] : 0.0f, Db = 0.0f;
        float wyb = 0.0f, uyb = 0.0f;
        if (upd) {
            Db = MODEL == LINSTEP ? a.Df[idx - sy] : 0.0f;
            wyb = face32<MODEL, CHECK>(a, a.din[idx - sy], dc, a.Hf[idx - sy], hc, Db, Dc, a.win[1][idx - sy], uyb);
            if (j0 == 1) a.wout[1][idx - sy] = wyb;
        }
        for (int j = j0; j < j1; ++j, idx += sy) {
            const float dn = a.din[idx + sy], hn = a.Hf[idx + sy];
            const float wx = a.win[0][idx], wy = a.win[1][idx], rr = a.r[idx];
            const float Dn = MODEL == LINSTEP ? a.Df[idx + sy] : 0.0f;
            float dr = __shfl_down_sync(FULL, dc, 1);
            float hr = __shfl_down_sync(FULL, hc, 1);
            float Dr = MODEL == LINSTEP ? __shfl_down_sync(FULL, Dc, 1) : 0.0f;
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                dr = ok ? a.din[idx + 1] : dc;
                hr = ok ? a.Hf[idx + 1] : hc;
                if (MODEL == LINSTEP) Dr = ok ? a.Df[idx + 1] : Dc;
            }
            float ux = 0.0f, uy = 0.0f, wxn = 0.0f, wyn = 0.0f;
            if (xface) wxn = face32<MODEL, CHECK>(a, dc, dr, hc, hr, Dc, Dr, wx, ux);
            if (upd) wyn = face32<MODEL, CHECK>(a, dc, dn, hc, hn, Dc, Dn, wy, uy);
            const float wxl = __shfl_up_sync(FULL, wxn, 1);
            const float uxl = CHECK ? __shfl_up_sync(FULL, ux, 1) : 0.0f;
            const float Dl = MODEL == LINSTEP ? __shfl_up_sync(FULL, Dc, 1) : 0.0f;
            if (own_x) a.wout[0][idx] = wxn;
            if (upd) {
                a.wout[1][idx] = wyn;
                const float e = cell_e32<MODEL>(a, hc, fmaxf(fmaxf(fmaxf(Dc, Dl), fmaxf(Dr, Db)), Dn));
                const float div = fmaf(wyn - wyb, a.sig[1], (wxn - wxl) * a.sig[0]);
                const float dnew = fmaf(-e, fmaf(dc, a.rdt, div - rr), dc);
                a.dout[idx] = dnew;
                if (CHECK) {
                    const float divu = fmaf(uy - uyb, a.sig[1], (ux - uxl) * a.sig[0]);
                    accumulate_residual32(fmaf(-dnew, a.rdt, rr + divu), part, pmax);
                }
            }
            dc = dn;
            hc = hn;
            wyb = wyn;
            uyb = uy;
            if (MODEL == LINSTEP) {
                Db = Dc;
                Dc = Dn;
            }
            if (CHECK && j == j1 - 1) warp_flush_residual32(a.acc, a.norm_max, part, pmax, lane, a.parts, slot);
        }
    } else if (CHECK && a.parts && lane == 0) {
        a.parts[slot] = 0.0;
    }
}

// One inner cell update: d - e*(d/dt + div w - r).
__device__ __forceinline__ float dc_update(const DcArgs& a, float d, float wx, float wxl, float wy, float wyb,
                                           float rr, float e)
{
    const float div = fmaf(wy - wyb, a.sig[1], (wx - wxl) * a.sig[0]);
    return fmaf(-e, fmaf(d, a.rdt, div - rr), d);
}

// ---------------------------------------------------------------------------
// 2D, two inner iterations per launch (temporal blocking, depth 2).
//
// The FP32 inner iteration moves 32 bytes per cell and is bound by HBM; doing
// two iterations per pass over memory halves that.  Iteration k+1 ("level 1")
// runs one row ahead of iteration k+2 ("level 2") in the y march, and only
// level-2 values are written: level-1 values live in registers (the rows the
// level-2 stencil needs) and in warp shuffles (the x neighbours).
//
// x: lane L of warp-tile t holds column i = 28t + L - 1.  Level-1 x faces
// are used on lanes 0..30 (the right neighbour is lane L+1's column, so no
// lane loads beyond its own), level-1 cells on lanes 1..30, level-2 x faces
// on lanes 1..29 and level-2 cells on lanes 2..29: each tile updates 28
// columns and stores the x faces of lanes 1..28, and of lane 29 when it is
// the last face (every face i+1/2, i = 0..nx-2, has one owner).  y: a chunk
// of level-2 rows [j0, j1) first recomputes level 1 for rows j0-1 and j0
// (the halo), then each march step s computes level 1 for row s+1 and
// level 2 for row s.  Boundary rows and columns are never updated (their
// level-1 and level-2 values are the input).  The check variant forms the
// mixed residual of the second iteration: undamped flux from the level-1
// state, time term from the level-2 state.
template <int MODEL>
__device__ __forceinline__ float dc_star(float Dc, float Db, float Dn)
{
    if (MODEL != LINSTEP) return 0.0f;
    const float Dr = __shfl_down_sync(FULL, Dc, 1);
    const float Dl = __shfl_up_sync(FULL, Dc, 1);
    return fmaxf(fmaxf(fmaxf(Dc, Dl), fmaxf(Dr, Db)), Dn);
}

template <int MODEL, bool CHECK>
__device__ __forceinline__ void dc2d_tb2_body(const DcArgs& a, int tile, int cy, int chunk, float& part,
                                              unsigned& pmax, long long slot = 0)
{
    constexpr bool LS = MODEL == LINSTEP;
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
    const bool colin = i >= 1 && i <= nx - 2;       // interior column
    const bool upd1 = colin && lane >= 1 && lane <= 30;
    const bool xf2 = i >= 0 && i <= nx - 2 && lane >= 1 && lane <= 29;
    const bool upd2 = colin && lane >= 2 && lane <= 29;
    const bool own_x = xf2 && (lane <= 28 || i == nx - 2);
    const long long sy = a.sy;
    float u;

    // level-1 x face of the row at offset o (flux of the input state)
    auto x1 = [&](long long o, float d, float h, float D) {
        const float dr = __shfl_down_sync(FULL, d, 1);
        const float hr = __shfl_down_sync(FULL, h, 1);
        const float Dr = LS ? __shfl_down_sync(FULL, D, 1) : 0.0f;
        return face32<MODEL, false>(a, d, dr, h, hr, D, Dr, a.win[0][o], u);
    };

    // ---- prologue: level 1 of rows j0-1 (A) and j0 (B), level-2 face (j0-1/2)
    const long long oA = (long long)(j0 - 1) * sy + ic, oB = oA + sy, oC = oB + sy;
    const float dA = a.din[oA], hA = a.Hf[oA];
    const float DA = LS ? a.Df[oA] : 0.0f;
    const float dB = a.din[oB], hB = a.Hf[oB];
    const float DB = LS ? a.Df[oB] : 0.0f;
    float d1 = a.din[oC], h1 = a.Hf[oC];   // row j0+1 <= ny-1
    float D1 = LS ? a.Df[oC] : 0.0f;
    const float wyAB = face32<MODEL, false>(a, dA, dB, hA, hB, DA, DB, a.win[1][oA], u);   // w'_y(j0-1/2)
    float pA = dA;   // delta'(j0-1)
    if (j0 >= 2) {   // row j0-1 is interior: level 1 there
        const long long oZ = oA - sy;
        const float dZ = a.din[oZ], hZ = a.Hf[oZ];
        const float DZ = LS ? a.Df[oZ] : 0.0f;
        const float wyZA = face32<MODEL, false>(a, dZ, dA, hZ, hA, DZ, DA, a.win[1][oZ], u);
        const float wxA = x1(oA, dA, hA, DA);
        const float wxAl = __shfl_up_sync(FULL, wxA, 1);
        const float eA = cell_e32<MODEL>(a, hA, dc_star<MODEL>(DA, DZ, DB));
        if (upd1) pA = dc_update(a, dA, wxA, wxAl, wyAB, wyZA, a.r[oA], eA);
    }
    float wx1p = x1(oB, dB, hB, DB);                                                  // w'_x(j0)
    float wy1p = face32<MODEL, false>(a, dB, d1, hB, h1, DB, D1, a.win[1][oB], u);     // w'_y(j0+1/2)
    float r0 = a.r[oB];
    float p0 = dB;                                                                    // delta'(j0)
    {
        const float wxl = __shfl_up_sync(FULL, wx1p, 1);
        const float eB = cell_e32<MODEL>(a, hB, dc_star<MODEL>(DB, DA, D1));
        if (upd1) p0 = dc_update(a, dB, wx1p, wxl, wy1p, wyAB, r0, eB);
    }
    float uy2b = 0.0f;
    float wy2b = face32<MODEL, CHECK>(a, pA, p0, hA, hB, DA, DB, wyAB, uy2b);   // w''_y(j0-1/2)
    if (j0 == 1 && upd2) a.wout[1][oA] = wy2b;
    float h0 = hB, D0 = DB, Dm1 = DA;

    // ---- march: level 1 of row s+1, level 2 of row s (LIN, NONLIN: the x
    // and y faces of a level as one FP32x2 evaluation)
    constexpr bool PACKF = MODEL == LIN || MODEL == NONLIN;
    long long o = oC;   // offset of row s+1
    for (int s = j0; s < j1; ++s, o += sy) {
        float p1 = d1, wx1 = 0.0f, wy1 = 0.0f, r1 = 0.0f, h2 = h1, D2 = D1;
        if (s + 1 <= ny - 2) {   // row s+1 interior (uniform): level 1 there
            const float d2 = a.din[o + sy];
            h2 = a.Hf[o + sy];
            if (LS) D2 = a.Df[o + sy];
            r1 = a.r[o];
            if (PACKF) {
                const float d1r = __shfl_down_sync(FULL, d1, 1);
                const float h1r = __shfl_down_sync(FULL, h1, 1);
                float2 uu;
                const float2 w1 = face32x2<MODEL, false>(a, f2(d1), f2(d1r, d2), f2(h1), f2(h1r, h2),
                                                         f2(a.win[0][o], a.win[1][o]), uu);
                wx1 = w1.x;
                wy1 = w1.y;
            } else {
                wx1 = x1(o, d1, h1, D1);
                wy1 = face32<MODEL, false>(a, d1, d2, h1, h2, D1, D2, a.win[1][o], u);
            }
            const float wx1l = __shfl_up_sync(FULL, wx1, 1);
            const float e1 = cell_e32<MODEL>(a, h1, dc_star<MODEL>(D1, D0, D2));
            if (upd1) p1 = dc_update(a, d1, wx1, wx1l, wy1, wy1p, r1, e1);
            d1 = d2;
        }
        // level 2 of row s
        const float p0r = __shfl_down_sync(FULL, p0, 1);
        const float h0r = __shfl_down_sync(FULL, h0, 1);
        const float D0r = LS ? __shfl_down_sync(FULL, D0, 1) : 0.0f;
        float ux2 = 0.0f, uy2 = 0.0f, wx2, wy2;
        if (PACKF) {
            float2 u2 = f2(0.0f);
            const float2 w2 = face32x2<MODEL, CHECK>(a, f2(p0), f2(p0r, p1), f2(h0), f2(h0r, h1), f2(wx1p, wy1p), u2);
            wx2 = w2.x;
            wy2 = w2.y;
            ux2 = u2.x;
            uy2 = u2.y;
        } else {
            wx2 = face32<MODEL, CHECK>(a, p0, p0r, h0, h0r, D0, D0r, wx1p, ux2);
            wy2 = face32<MODEL, CHECK>(a, p0, p1, h0, h1, D0, D1, wy1p, uy2);
        }
        const float wx2l = __shfl_up_sync(FULL, wx2, 1);
        const float ux2l = CHECK ? __shfl_up_sync(FULL, ux2, 1) : 0.0f;
        const float e0 = cell_e32<MODEL>(a, h0, dc_star<MODEL>(D0, Dm1, D1));
        const long long os = o - sy;
        if (own_x) a.wout[0][os] = wx2;
        if (upd2) {
            const float q = dc_update(a, p0, wx2, wx2l, wy2, wy2b, r0, e0);
            a.dout[os] = q;
            a.wout[1][os] = wy2;
            if (CHECK) {
                const float divu = fmaf(uy2 - uy2b, a.sig[1], (ux2 - ux2l) * a.sig[0]);
                accumulate_residual32(fmaf(-q, a.rdt, r0 + divu), part, pmax);
            }
        }
        // shift the windows
        p0 = p1;
        wx1p = wx1;
        wy1p = wy1;
        wy2b = wy2;
        uy2b = uy2;
        h0 = h1;
        h1 = h2;
        Dm1 = D0;
        D0 = D1;
        D1 = D2;
        r0 = r1;
        if (CHECK && s == j1 - 1) warp_flush_residual32(a.acc, a.norm_max, part, pmax, lane, a.parts, slot);
    }
}

template <int MODEL, bool CHECK, int R>
__device__ __forceinline__ void dc3d_body(const DcArgs& a, int bx, int by, int bz, int chunk, float& part,
                                          unsigned& pmax)
{
    __shared__ float sd[2][R][32];
    __shared__ float sh[2][R][32];
    __shared__ float sw[2][R][32];
    __shared__ float su[CHECK ? 2 : 1][CHECK ? R : 1][32];
    __shared__ float sD[MODEL == LINSTEP ? 2 : 1][MODEL == LINSTEP ? R : 1][32];
    const int lane = threadIdx.x, r = threadIdx.y;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int i = 31 * bx + lane;
    const int j = (R - 1) * by + r;
    const int k0 = 1 + bz * chunk;
    const int k1 = min(k0 + chunk, nz - 1);
    if (k0 < k1) {
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
        float Dc = MODEL == LINSTEP ? a.Df[idx] : 0.0f, Db = 0.0f;
        float wzb = 0.0f, uzb = 0.0f;
        if (upd) {
            Db = MODEL == LINSTEP ? a.Df[idx - sz] : 0.0f;
            wzb = face32<MODEL, CHECK>(a, a.din[idx - sz], dc, a.Hf[idx - sz], hc, Db, Dc, a.win[2][idx - sz], uzb);
            if (k0 == 1) a.wout[2][idx - sz] = wzb;
        }
        int p = 0;
        sd[0][r][lane] = dc;
        sh[0][r][lane] = hc;
        if (MODEL == LINSTEP) sD[0][r][lane] = Dc;
        __syncthreads();
        for (int k = k0; k < k1; ++k, idx += sz) {
            const float dn = a.din[idx + sz], hn = a.Hf[idx + sz];
            const float wx = a.win[0][idx], wy = a.win[1][idx], wz = a.win[2][idx], rr = a.r[idx];
            const float Dn = MODEL == LINSTEP ? a.Df[idx + sz] : 0.0f;
            float du, hu, Du = 0.0f;
            if (!top) {
                du = sd[p][r + 1][lane];
                hu = sh[p][r + 1][lane];
                if (MODEL == LINSTEP) Du = sD[p][r + 1][lane];
            } else {
                du = up_ok ? a.din[idx + sy] : dc;
                hu = up_ok ? a.Hf[idx + sy] : hc;
                if (MODEL == LINSTEP) Du = up_ok ? a.Df[idx + sy] : Dc;
            }
            const float Dd = (MODEL == LINSTEP && r >= 1) ? sD[p][r - 1][lane] : 0.0f;
            float dr = __shfl_down_sync(FULL, dc, 1);
            float hr = __shfl_down_sync(FULL, hc, 1);
            float Dr = MODEL == LINSTEP ? __shfl_down_sync(FULL, Dc, 1) : 0.0f;
            if (lane == 31) {
                const bool ok = ic + 1 < nx;
                dr = ok ? a.din[idx + 1] : dc;
                hr = ok ? a.Hf[idx + 1] : hc;
                if (MODEL == LINSTEP) Dr = ok ? a.Df[idx + 1] : Dc;
            }
            float ux = 0.0f, uy = 0.0f, uz = 0.0f, wxn = 0.0f, wyn = 0.0f, wzn = 0.0f;
            if (xface) wxn = face32<MODEL, CHECK>(a, dc, dr, hc, hr, Dc, Dr, wx, ux);
            if (yface) wyn = face32<MODEL, CHECK>(a, dc, du, hc, hu, Dc, Du, wy, uy);
            if (upd) wzn = face32<MODEL, CHECK>(a, dc, dn, hc, hn, Dc, Dn, wz, uz);
            if (own_x) a.wout[0][idx] = wxn;
            if (own_y) a.wout[1][idx] = wyn;
            if (upd) a.wout[2][idx] = wzn;
            const float wxl = __shfl_up_sync(FULL, wxn, 1);
            const float uxl = CHECK ? __shfl_up_sync(FULL, ux, 1) : 0.0f;
            const float Dl = MODEL == LINSTEP ? __shfl_up_sync(FULL, Dc, 1) : 0.0f;
            sw[p][r][lane] = wyn;
            if (CHECK) su[p][r][lane] = uy;
            sd[p ^ 1][r][lane] = dn;
            sh[p ^ 1][r][lane] = hn;
            if (MODEL == LINSTEP) sD[p ^ 1][r][lane] = Dn;
            __syncthreads();
            if (upd) {
                const float wyb = sw[p][r - 1][lane];
                const float e = cell_e32<MODEL>(
                    a, hc, fmaxf(fmaxf(fmaxf(Dc, Dl), fmaxf(Dr, Du)), fmaxf(fmaxf(Dd, Db), Dn)));
                const float div = fmaf(wzn - wzb, a.sig[2], fmaf(wyn - wyb, a.sig[1], (wxn - wxl) * a.sig[0]));
                const float dnew = fmaf(-e, fmaf(dc, a.rdt, div - rr), dc);
                a.dout[idx] = dnew;
                if (CHECK) {
                    const float uyb = su[p][r - 1][lane];
                    const float divu = fmaf(uz - uzb, a.sig[2], fmaf(uy - uyb, a.sig[1], (ux - uxl) * a.sig[0]));
                    accumulate_residual32(fmaf(-dnew, a.rdt, rr + divu), part, pmax);
                }
            }
            dc = dn;
            hc = hn;
            wzb = wzn;
            uzb = uz;
            if (MODEL == LINSTEP) {
                Db = Dc;
                Dc = Dn;
            }
            p ^= 1;
        }
    }
}

}  // namespace ptd
