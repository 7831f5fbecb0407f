// ptd_pair_body.cuh -- the fused 2D PT iteration of the double-float forms
// (DF64, DFH) with two x-adjacent cells per lane.
//
// The arithmetic is the one of ptd_pt_body.cuh operation for operation (so the
// iterates are bit for bit those of the one-cell-per-lane kernels); what
// changes is how it maps onto the hardware.  The double-float kernels are
// bound by instruction issue, not by HBM: one cell's x and y faces packed
// into one FP32x2 evaluation left the cell update and the packing moves
// scalar.  Here a lane owns the cells 2L and 2L+1 of a 64-cell strip, loads
// every field as one 16-byte pair (128-bit loads), and evaluates the faces of
// the same direction of its two cells as one FP32x2 double-float computation
// (x: the face between its cells and the face to the next lane's first cell;
// y: the faces of both cells), and both cells' updates as one more.  Per cell
// that is 1.5 packed face evaluations (2 before) and a half packed update (1
// before): at 4096^2 (NONLIN) DF64 204 -> 175 us and DFH 214 -> 203 us per
// iteration, DFH now near its FP64-pipe limit (5 FP64 instructions per cell).
//
// Tiling: warp w of a tile covers cells c = 62 t + q, q = 0..63 (lane L holds
// q = 2L, 2L+1; the first cell of a pair is even, so a pair is one aligned
// 16-byte access); q = 1..62 are updated, q = 0 and q = 63 are the
// neighbours.  Tiles therefore advance by 62 cells.  Every x face q = 0..62
// is evaluated in the tile (face q lies between cells q and q+1); face q = 0
// of tile t is face q = 62 of tile t-1, evaluated from the same values by the
// same operations, so both tiles write the same bits.
#pragma once

#include "ptd_pt_body.cuh"

namespace ptd {

// H values of the two cells of a lane.
template <class N>
struct HP {
    typename N::HV a, b;
};

template <class N>
__device__ __forceinline__ HP<N> ldh2(const void* p, long long i);
template <>
__device__ __forceinline__ HP<DF64> ldh2<DF64>(const void* p, long long i)
{
    const float4 v = *reinterpret_cast<const float4*>(static_cast<const float2*>(p) + i);
    return HP<DF64>{make_float2(v.x, v.y), make_float2(v.z, v.w)};
}
template <>
__device__ __forceinline__ HP<DFH> ldh2<DFH>(const void* p, long long i)
{
    const double2 v = *reinterpret_cast<const double2*>(static_cast<const double*>(p) + i);
    return HP<DFH>{DFH::HV{v.x, split_bits(v.x)}, DFH::HV{v.y, split_bits(v.y)}};
}

// Hold of the two cells (as stored: float2 for DF64, double for DFH)
__device__ __forceinline__ void ldo2(DF64, const void* p, long long i, float2& o0, float2& o1)
{
    const float4 v = *reinterpret_cast<const float4*>(static_cast<const float2*>(p) + i);
    o0 = make_float2(v.x, v.y);
    o1 = make_float2(v.z, v.w);
}
__device__ __forceinline__ void ldo2(DFH, const void* p, long long i, double& o0, double& o1)
{
    const double2 v = *reinterpret_cast<const double2*>(static_cast<const double*>(p) + i);
    o0 = v.x;
    o1 = v.y;
}

// A double-float field (fluxes, D) at two cells as a packed pair.
__device__ __forceinline__ DF2 ldt2(const void* p, long long i)
{
    const float4 v = *reinterpret_cast<const float4*>(static_cast<const float2*>(p) + i);
    return DF2{make_float2(v.x, v.z), make_float2(v.y, v.w)};
}
// Store a packed pair: both cells, or one of them.
__device__ __forceinline__ void stt2(void* p, long long i, const DF2& v, bool m0, bool m1)
{
    float2* q = static_cast<float2*>(p) + i;
    if (m0 && m1) {
        *reinterpret_cast<float4*>(q) = make_float4(v.hi.x, v.lo.x, v.hi.y, v.lo.y);
    } else {
        if (m0) q[0] = make_float2(v.hi.x, v.lo.x);
        if (m1) q[1] = make_float2(v.hi.y, v.lo.y);
    }
}
__device__ __forceinline__ void sth2(DF64, void* p, long long i, const DF2& v, bool m0, bool m1) { stt2(p, i, v, m0, m1); }

// A double-float constant {hi, lo} in both components.
__device__ __forceinline__ DF2 dup2(float2 c) { return DF2{f2(c.x), f2(c.y)}; }
__device__ __forceinline__ DF2 df2_zero() { return DF2{f2(0.0f), f2(0.0f)}; }

// g = H_R - H_L of two faces (a: La -> Ra, b: Lb -> Rb)
__device__ __forceinline__ DF2 hdiffp(DF64, float2 La, float2 Ra, float2 Lb, float2 Rb)
{
    return df2_sub(df2_pack(Ra, Rb), df2_pack(La, Lb));
}
__device__ __forceinline__ DF2 hdiffp(DFH, const DFH::HV& La, const DFH::HV& Ra, const DFH::HV& Lb,
                                      const DFH::HV& Rb)
{
    return df2_pack(split_bits(Ra.d - La.d), split_bits(Rb.d - Lb.d));   // FP64 differences (DFH::hdiff)
}
__device__ __forceinline__ DF2 hsump(DF64, float2 La, float2 Ra, float2 Lb, float2 Rb)
{
    return df2_add(df2_pack(La, Lb), df2_pack(Ra, Rb));
}
__device__ __forceinline__ DF2 hsump(DFH, const DFH::HV& La, const DFH::HV& Ra, const DFH::HV& Lb,
                                     const DFH::HV& Rb)
{
    return df2_add(df2_pack(La.f, Lb.f), df2_pack(Ra.f, Rb.f));
}

// Two faces as one packed evaluation: face_t of ptd_pt_body.cuh with every
// operation on both faces at once.  DL, DR: the per-cell field (LINSTEP: D,
// NONLIN_EXPM: exp(m)) left and right of each face; hsa, hsb: H_L + H_R in
// FP32 for the iteration parameter.
template <class N, int MODEL, bool U>
__device__ __forceinline__ DF2 facep(const PTArgs& a, const typename N::HV& La, const typename N::HV& Ra,
                                     const typename N::HV& Lb, const typename N::HV& Rb, float hsa, float hsb,
                                     const DF2& DL, const DF2& DR, const DF2& w, DF2& u)
{
    const DF2 g = hdiffp(N(), La, Ra, Lb, Rb);
    if (MODEL == LIN) {
        if (U) u = g;
        return df2_nmadf(df2_add(g, w), f2(a.fc_lin), w);
    }
    float2 c;
    DF2 K;
    if (MODEL == LINSTEP) {
        K = df2_add(DL, DR);
        c = f2(a.fc_lin);
    } else if (MODEL == NONLIN) {
        const DF2 s = hsump(N(), La, Ra, Lb, Rb);
        K = df2_mul(df2_mul(s, s), s);
        c = f2(nonlin_face_c(a.f, hsa), nonlin_face_c(a.f, hsb));
    } else {   // NONLIN_EXPM
        const DF2 s = hsump(N(), La, Ra, Lb, Rb);
        const DF2 e2 = df2_add(DL, DR);
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

// H - Hold of both cells, and the update H - e*Rp of both cells.
__device__ __forceinline__ DF2 hdo2(DF64, const HP<DF64>& H, float2 o0, float2 o1)
{
    return df2_sub(df2_pack(H.a, H.b), df2_pack(o0, o1));
}
__device__ __forceinline__ DF2 hdo2(DFH, const HP<DFH>& H, double o0, double o1)
{
    return df2_pack(split_bits(H.a.d - o0), split_bits(H.b.d - o1));
}

// The updated pair: DF64 as a packed pair, DFH as two doubles.
struct HN64 {
    DF2 v;
};
struct HNH {
    double a, b;
};
__device__ __forceinline__ HN64 hstep2(DF64, const HP<DF64>& H, const DF2& rp, float2 e)
{
    return HN64{df2_nmadf(rp, e, df2_pack(H.a, H.b))};
}
__device__ __forceinline__ HNH hstep2(DFH, const HP<DFH>& H, const DF2& rp, float2 e)
{
    return HNH{DFH::hstep(H.a, df2_first(rp), e.x), DFH::hstep(H.b, df2_second(rp), e.y)};
}
__device__ __forceinline__ void sthn(void* p, long long i, const HN64& v, bool m0, bool m1) { stt2(p, i, v.v, m0, m1); }
__device__ __forceinline__ void sthn(void* p, long long i, const HNH& v, bool m0, bool m1)
{
    double* q = static_cast<double*>(p) + i;
    if (m0 && m1) {
        *reinterpret_cast<double2*>(q) = make_double2(v.a, v.b);
    } else {
        if (m0) q[0] = v.a;
        if (m1) q[1] = v.b;
    }
}
// H_new - Hold of both cells (the check residual's time term)
__device__ __forceinline__ DF2 hdn2(const HN64& h, float2 o0, float2 o1) { return df2_sub(h.v, df2_pack(o0, o1)); }
__device__ __forceinline__ DF2 hdn2(const HNH& h, double o0, double o1)
{
    return df2_pack(split_bits(h.a - o0), split_bits(h.b - o1));
}

template <class N>
struct PairTraits;
template <>
struct PairTraits<DF64> {
    using HN = HN64;
};
template <>
struct PairTraits<DFH> {
    using HN = HNH;
};

__device__ __forceinline__ float2 shfl_down_f2(float2 v) { return DF64::shfl_down(v, 1); }
__device__ __forceinline__ float2 shfl_up_f2(float2 v) { return DF64::shfl_up(v, 1); }

// The two cells' updated H from their flux differences (dx, dy[, dz] packed):
// h_update_sq / h_update of ptd_pt_body.cuh on both cells at once.
template <class N>
__device__ __forceinline__ typename PairTraits<N>::HN pair_update(const PTArgs& a, const HP<N>& Hc,
                                                                  typename N::HS o0, typename N::HS o1,
                                                                  const DF2& dsum_or_div, float e0, float e1)
{
    const DF2 hd = hdo2(N(), Hc, o0, o1);
    if (a.sq) {
        const DF2 rp = df2_mad(hd, dup2(a.rdt_sig_df), dsum_or_div);
        return hstep2(N(), Hc, rp, f2(e0 * a.fsig, e1 * a.fsig));
    }
    const DF2 rp = df2_mad(hd, dup2(a.rdt_df), dsum_or_div);
    return hstep2(N(), Hc, rp, f2(e0, e1));
}

// ---------------------------------------------------------------------------
// 2D: blockDim = (32, W); warp w of block b owns the 64-cell strip of tile
// t = b*W + w and marches rows j0 .. j1-1 of y chunk cy.  slot: the warp's
// slot in a.parts.
template <class N, int MODEL, bool CHECK>
__device__ __forceinline__ void pt2d_pair_body(const PTArgs& a, int tile, int cy, int chunk, double& part,
                                               unsigned long long& pmax, long long slot = 0)
{
    using HS = typename N::HS;
    using HN = typename PairTraits<N>::HN;
    constexpr bool HASD = ModelTraits<MODEL>::hasd;
    const int lane = threadIdx.x;
    const int nx = a.nx, ny = a.ny;
    const int c0 = 62 * tile + 2 * lane;   // first cell of the lane's pair
    const int j0 = 1 + cy * chunk;
    const int j1 = min(j0 + chunk, ny - 1);
    if ((62 * tile < nx - 2) && (j0 < j1)) {   // uniform over the warp
        const long long sy = a.sy;
        // a pair past the row pitch (cells >= nx only) is read at the row's
        // last pair: its values feed only faces and cells that are discarded
        const int cl = min(c0, (int)sy - 2);
        const bool u0 = lane >= 1 && c0 >= 1 && c0 <= nx - 2;           // cell q = 2L updated
        const bool u1 = lane <= 30 && c0 + 1 <= nx - 2;                // cell q = 2L+1 updated (c0+1 >= 1)
        const bool fa = c0 <= nx - 2;                                  // face (c0, c0+1) exists
        const bool fb = lane <= 30 && c0 + 1 <= nx - 2;                // face (c0+1, c0+2), in the tile
        const bool y0 = c0 <= nx - 1, y1 = c0 + 1 <= nx - 1;           // y faces of existing cells
        long long idx = (long long)j0 * sy + cl;

        HP<N> Hc = ldh2<N>(a.Hin, idx);
        float hc0 = N::hf(Hc.a), hc1 = N::hf(Hc.b);
        DF2 Dc = HASD ? ldt2(a.D, idx) : df2_zero();
        float2 dbf = f2(0.0f);   // LINSTEP: D of the row below (FP32)
        DF2 wyb, uyb = df2_zero();
        {
            // faces (j0 - 1/2) of both cells, owned by the chunk below unless j0 == 1
            const HP<N> Hb = ldh2<N>(a.Hin, idx - sy);
            const DF2 Db = HASD ? ldt2(a.D, idx - sy) : df2_zero();
            if (MODEL == LINSTEP) dbf = Db.hi;
            wyb = facep<N, MODEL, CHECK>(a, Hb.a, Hc.a, Hb.b, Hc.b, N::hf(Hb.a) + hc0, N::hf(Hb.b) + hc1, Db, Dc,
                                         ldt2(a.win[1], idx - sy), uyb);
            if (j0 == 1) stt2(a.wout[1], idx - sy, wyb, y0, y1);
        }
        for (int j = j0; j < j1; ++j, idx += sy) {
            const HP<N> Hn = ldh2<N>(a.Hin, idx + sy);
            const DF2 wx = ldt2(a.win[0], idx);
            const DF2 wy = ldt2(a.win[1], idx);
            HS o0, o1;
            ldo2(N(), a.Hold, idx, o0, o1);
            const DF2 Dn = HASD ? ldt2(a.D, idx + sy) : df2_zero();
            // the next lane's first cell
            const typename N::HV Hr = N::shfl_down_h(Hc.a, 1);
            const float hr = __shfl_down_sync(FULL, hc0, 1);
            const float2 Dr = HASD ? shfl_down_f2(df2_first(Dc)) : f2(0.0f);
            const float hn0 = N::hf(Hn.a), hn1 = N::hf(Hn.b);
            DF2 ux = df2_zero(), uy = df2_zero();
            const DF2 wxn = facep<N, MODEL, CHECK>(a, Hc.a, Hc.b, Hc.b, Hr, hc0 + hc1, hc1 + hr, Dc,
                                                   df2_pack(df2_second(Dc), Dr), wx, ux);
            const DF2 wyn = facep<N, MODEL, CHECK>(a, Hc.a, Hn.a, Hc.b, Hn.b, hc0 + hn0, hc1 + hn1, Dc, Dn, wy, uy);
            // the left face of cell 2L: the previous lane's face (c0-1, c0)
            const float2 wbl = shfl_up_f2(df2_second(wxn));
            const float2 ubl = CHECK ? shfl_up_f2(df2_second(ux)) : f2(0.0f);
            stt2(a.wout[0], idx, wxn, fa, fb);
            stt2(a.wout[1], idx, wyn, y0, y1);
            float dm0 = 0.0f, dm1 = 0.0f;   // LINSTEP: maxloc of D (star); NONLIN_EXPM: exp(m) of the cell
            if (MODEL == LINSTEP) {
                const float dl = __shfl_up_sync(FULL, Dc.hi.y, 1);
                dm0 = fmaxf(fmaxf(fmaxf(Dc.hi.x, dl), fmaxf(Dc.hi.y, dbf.x)), Dn.hi.x);
                dm1 = fmaxf(fmaxf(fmaxf(Dc.hi.y, Dc.hi.x), fmaxf(Dr.x, dbf.y)), Dn.hi.y);
            } else if (MODEL == NONLIN_EXPM) {
                dm0 = Dc.hi.x;
                dm1 = Dc.hi.y;
            }
            const float e0 = cell_e<MODEL>(a, hc0, dm0), e1 = cell_e<MODEL>(a, hc1, dm1);
            // flux differences of both cells: x (w_R - w_L), y (w_up - w_down)
            const DF2 dx = df2_sub(wxn, df2_pack(wbl, df2_first(wxn)));
            const DF2 dy = df2_sub(wyn, wyb);
            const DF2 s = a.sq ? df2_add(dy, dx)
                               : df2_mad(dy, dup2(a.sig_df[1]), df2_mul(dx, dup2(a.sig_df[0])));
            const HN Hnew = pair_update<N>(a, Hc, o0, o1, s, e0, e1);
            sthn(a.Hout, idx, Hnew, u0, u1);
            if (CHECK) {
                const DF2 dux = df2_sub(ux, df2_pack(ubl, df2_first(ux)));
                const DF2 duy = df2_sub(uy, uyb);
                const DF2 divu = df2_mad(duy, dup2(a.sig_df[1]), df2_mul(dux, dup2(a.sig_df[0])));
                const DF2 r = df2_sub(divu, df2_mul(hdn2(Hnew, o0, o1), dup2(a.rdt_df)));
                if (u0) accumulate_residual(DF64::to_d(df2_first(r)), part, pmax);
                if (u1) accumulate_residual(DF64::to_d(df2_second(r)), part, pmax);
                uyb = uy;
            }
            Hc = Hn;
            hc0 = hn0;
            hc1 = hn1;
            wyb = wyn;
            if (HASD) {
                if (MODEL == LINSTEP) dbf = Dc.hi;
                Dc = Dn;
            }
            if (CHECK && j == j1 - 1) warp_flush_residual(a.acc, a.norm_max, part, pmax, lane, a.parts, slot);
        }
    } else if (CHECK && a.parts && lane == 0) {
        a.parts[slot] = 0.0;   // a warp with no cells: its slot still holds this check's (empty) part
    }
}

}  // namespace ptd
