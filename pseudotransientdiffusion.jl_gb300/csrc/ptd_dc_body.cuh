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
};

// One face of the linearised flux (scaled like ptd_device.cuh):
// u = K_f (d_R - d_L) [+ 3 s^2 (h_R - h_L) (d_L + d_R)],  w <- w - c (w + u).
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
        uu = (DL + DR) * gd;
        c = a.c_lin;
    } else {
        const float s = hL + hR;
        const float s2 = s * s;
        uu = s2 * s * gd;
        uu = fmaf(3.0f * s2 * (hR - hL), dL + dR, uu);
        c = nonlin_face_c(a.f, s);
    }
    if (U) u = uu;
    return fmaf(-c, w + uu, w);
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
__device__ __forceinline__ void dc1d_body(const DcArgs& a, int bx, double& part, unsigned long long& pmax)
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
            if (CHECK) accumulate_residual((double)fmaf(-dn, a.rdt, rr + (ur - ul) * a.sig[0]), part, pmax);
        }
    }
}

template <int MODEL, bool CHECK>
__device__ __forceinline__ void dc2d_body(const DcArgs& a, int tile, int cy, int chunk, double& part,
                                          unsigned long long& pmax)
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
                    accumulate_residual((double)fmaf(-dnew, a.rdt, rr + divu), part, pmax);
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
        }
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
// x: lane L of warp-tile t holds column i = 29t + L - 1.  Level-1 x faces are
// valid on lanes 0..31 (lane 31 loads its right neighbour), level-1 cells on
// lanes 1..31 (the left face comes from lane L-1), level-2 x faces on lanes
// 1..30 and level-2 cells on lanes 2..30: each tile updates 29 columns, and
// stores the x faces of lanes 1..29 (every face i+1/2, i = 0..nx-2, has one
// owner).  y: a chunk of level-2 rows [j0, j1) first recomputes level 1 for
// rows j0-1 and j0 (the halo), then each march step s computes level 1 for
// row s+1 and level 2 for row s.  Boundary rows and columns are never
// updated (their level-1 and level-2 values are the input).  The check
// variant forms the mixed residual of the second iteration: undamped flux
// from the level-1 state, time term from the level-2 state.
template <int MODEL, bool CHECK>
__device__ __forceinline__ void dc2d_tb2_body(const DcArgs& a, int tile, int cy, int chunk, double& part,
                                              unsigned long long& pmax)
{
    const int lane = threadIdx.x;
    const int nx = a.nx, ny = a.ny;
    const int j0 = 1 + cy * chunk;
    const int j1 = min(j0 + chunk, ny - 1);
    if (29 * tile >= nx - 1 || j0 >= j1) return;   // uniform over the warp
    const int i = 29 * tile + lane - 1;
    const int ic = min(max(i, 0), nx - 1);          // clamped column of this lane's loads
    const int icr = min(ic + 1, nx - 1);            // lane 31's right neighbour
    const bool colin = i >= 1 && i <= nx - 2;       // interior column
    const bool xf = i >= 0 && i <= nx - 2;          // face i+1/2 exists
    const bool upd1 = colin && lane >= 1;
    const bool xf2 = xf && lane >= 1 && lane <= 30;
    const bool upd2 = colin && lane >= 2 && lane <= 30;
    const bool own_x = xf && lane >= 1 && lane <= 29;
    const bool L31 = lane == 31;
    constexpr bool LS = MODEL == LINSTEP;
    const long long sy = a.sy;
    auto at = [&](int row) { return (long long)row * sy + ic; };
    auto atr = [&](int row) { return (long long)row * sy + icr; };

    // level-1 x face of row m (w' = face of the input state): all lanes
    auto x1 = [&](int m, float d, float h, float D) {
        float dr = __shfl_down_sync(FULL, d, 1);
        float hr = __shfl_down_sync(FULL, h, 1);
        float Dr = LS ? __shfl_down_sync(FULL, D, 1) : 0.0f;
        if (L31) {
            dr = a.din[atr(m)];
            hr = a.Hf[atr(m)];
            if (LS) Dr = a.Df[atr(m)];
        }
        float u;
        return xf ? face32<MODEL, false>(a, d, dr, h, hr, D, Dr, a.win[0][at(m)], u) : 0.0f;
    };
    // star maximum of D around a cell (LINSTEP's iteration parameter)
    auto dstar = [&](float Dc, float Db, float Dn, int m) {
        if (!LS) return 0.0f;
        float Dr = __shfl_down_sync(FULL, Dc, 1);
        const float Dl = __shfl_up_sync(FULL, Dc, 1);
        if (L31) Dr = a.Df[atr(m)];
        return fmaxf(fmaxf(fmaxf(Dc, Dl), fmaxf(Dr, Db)), Dn);
    };

    // ---- prologue: level 1 of rows j0-1 and j0, level-2 face (j0-1/2)
    const float dA = a.din[at(j0 - 1)], hA = a.Hf[at(j0 - 1)];
    const float DA = LS ? a.Df[at(j0 - 1)] : 0.0f;
    const float dB = a.din[at(j0)], hB = a.Hf[at(j0)];
    const float DB = LS ? a.Df[at(j0)] : 0.0f;
    float d1 = a.din[at(j0 + 1)], h1 = a.Hf[at(j0 + 1)];
    float D1 = LS ? a.Df[at(j0 + 1)] : 0.0f;
    float u;
    // w'_y(j0 - 1/2)
    const float wyAB = upd1 ? face32<MODEL, false>(a, dA, dB, hA, hB, DA, DB, a.win[1][at(j0 - 1)], u) : 0.0f;
    float pA = dA;   // delta'(j0 - 1)
    float DZ = 0.0f; // D(j0 - 2)
    if (j0 >= 2) {   // row j0 - 1 is interior: level 1 there
        const float dZ = a.din[at(j0 - 2)], hZ = a.Hf[at(j0 - 2)];
        DZ = LS ? a.Df[at(j0 - 2)] : 0.0f;
        const float wyZA = upd1 ? face32<MODEL, false>(a, dZ, dA, hZ, hA, DZ, DA, a.win[1][at(j0 - 2)], u) : 0.0f;
        const float wxA = x1(j0 - 1, dA, hA, DA);
        const float wxAl = __shfl_up_sync(FULL, wxA, 1);
        const float eA = cell_e32<MODEL>(a, hA, dstar(DA, DZ, DB, j0 - 1));
        if (upd1) pA = dc_update(a, dA, wxA, wxAl, wyAB, wyZA, a.r[at(j0 - 1)], eA);
    }
    // level 1 of row j0
    float wx1p = x1(j0, dB, hB, DB);                                         // w'_x(j0)
    float wy1p = upd1 ? face32<MODEL, false>(a, dB, d1, hB, h1, DB, D1, a.win[1][at(j0)], u) : 0.0f;  // w'_y(j0+1/2)
    float p0 = dB;                                                           // delta'(j0)
    {
        const float wxl = __shfl_up_sync(FULL, wx1p, 1);
        const float eB = cell_e32<MODEL>(a, hB, dstar(DB, DA, D1, j0));
        if (upd1) p0 = dc_update(a, dB, wx1p, wxl, wy1p, wyAB, a.r[at(j0)], eB);
    }
    // level-2 face w''_y(j0 - 1/2)
    float uy2b = 0.0f;
    float wy2b = upd2 ? face32<MODEL, CHECK>(a, pA, p0, hA, hB, DA, DB, wyAB, uy2b) : 0.0f;
    if (j0 == 1 && upd2) a.wout[1][at(0)] = wy2b;
    float h0 = hB, D0 = DB, Dm1 = DA;
    float r0 = a.r[at(j0)];

    // ---- march: level 1 of row s+1, level 2 of row s
    for (int s = j0; s < j1; ++s) {
        const int m = s + 1;
        float p1 = d1, wx1 = 0.0f, wy1 = 0.0f, r1 = 0.0f, h2 = h1, D2 = D1;
        if (m <= ny - 2) {   // interior: level 1 of row m
            const float d2 = a.din[at(m + 1)];
            h2 = a.Hf[at(m + 1)];
            if (LS) D2 = a.Df[at(m + 1)];
            r1 = a.r[at(m)];
            wx1 = x1(m, d1, h1, D1);
            wy1 = upd1 ? face32<MODEL, false>(a, d1, d2, h1, h2, D1, D2, a.win[1][at(m)], u) : 0.0f;
            const float wx1l = __shfl_up_sync(FULL, wx1, 1);
            const float e1 = cell_e32<MODEL>(a, h1, dstar(D1, D0, D2, m));
            if (upd1) p1 = dc_update(a, d1, wx1, wx1l, wy1, wy1p, r1, e1);
            d1 = d2;
        }
        // level 2 of row s
        const float p0r = __shfl_down_sync(FULL, p0, 1);
        const float h0r = __shfl_down_sync(FULL, h0, 1);
        const float D0r = LS ? __shfl_down_sync(FULL, D0, 1) : 0.0f;
        float ux2 = 0.0f, uy2 = 0.0f;
        const float wx2 = xf2 ? face32<MODEL, CHECK>(a, p0, p0r, h0, h0r, D0, D0r, wx1p, ux2) : 0.0f;
        const float wy2 = upd2 ? face32<MODEL, CHECK>(a, p0, p1, h0, h1, D0, D1, wy1p, uy2) : 0.0f;
        const float wx2l = __shfl_up_sync(FULL, wx2, 1);
        const float ux2l = CHECK ? __shfl_up_sync(FULL, ux2, 1) : 0.0f;
        const float e0 = cell_e32<MODEL>(a, h0, dstar(D0, Dm1, D1, s));
        if (own_x) a.wout[0][at(s)] = wx2;
        if (upd2) {
            const float q = dc_update(a, p0, wx2, wx2l, wy2, wy2b, r0, e0);
            a.dout[at(s)] = q;
            a.wout[1][at(s)] = wy2;
            if (CHECK) {
                const float divu = fmaf(uy2 - uy2b, a.sig[1], (ux2 - ux2l) * a.sig[0]);
                accumulate_residual((double)fmaf(-q, a.rdt, r0 + divu), part, pmax);
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
    }
}

template <int MODEL, bool CHECK, int R>
__device__ __forceinline__ void dc3d_body(const DcArgs& a, int bx, int by, int bz, int chunk, double& part,
                                          unsigned long long& pmax)
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
                    accumulate_residual((double)fmaf(-dnew, a.rdt, rr + divu), part, pmax);
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
