// ptd_tune.cu -- launch-shape choice for the fused kernels.
#include <mutex>

#include "ptd_internal.h"

namespace ptd {

int sm_count()
{
    static std::mutex mu;
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 152;   // only reached when no device is usable; launches then fail anyway
    }
    std::lock_guard<std::mutex> lk(mu);
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
            cudaGetLastError();
            n = 152;
        }
        cache[dev] = n;
    }
    return cache[dev];
}

// The z march length of a 3D launch of bxy CTAs per z chunk on `slots`
// resident CTA slots: the longest march (512..16) whose CTA count fills the
// slots in whole waves to >= 90 % (wave quantization), else the best filling
// one.
int z_chunk(long long bxy, int nz, long long slots)
{
    int best = 16;
    double best_eff = -1.0;
    for (int chunk = 512; chunk >= 16; chunk /= 2) {
        const long long nb = bxy * ((nz - 2 + chunk - 1) / chunk);
        const long long waves = (nb + slots - 1) / slots;
        const double eff = (double)nb / (double)(waves * slots);
        if (nb >= slots && eff >= 0.9) return chunk;
        if (eff > best_eff) {
            best_eff = eff;
            best = chunk;
        }
    }
    return best;
}

LaunchCfg tuned_config(const ptd_params& p)
{
    LaunchCfg c;
    if (p.ndim == 2) {
        // short y marches in small CTAs: many independent warps per SM hide
        // the memory latency of the march.  Measured at 4096^2 (NONLIN) over
        // warps {1,2,4,8} x rows {8,16,32,64}, us per iteration against the
        // former 2 warps x 16 rows: FP64 1 x 32 587.3 (598.5), DFH 1 x 8 199.0
        // (202.4), DF64 2 x 8 169.3 (173.4), FP32_RB 8 x 32 (two-iteration
        // marches of 64 rows) 64.6 (65.6); FP32_DC 2 x 16.
        switch (p.precision) {
        case PTD_PREC_FP64: c.warps2d = 1; c.chunk2d = 32; break;
        case PTD_PREC_DFH: c.warps2d = 1; c.chunk2d = 8; break;
        case PTD_PREC_DF64: c.warps2d = 2; c.chunk2d = 8; break;
        case PTD_PREC_FP32_RB: c.warps2d = 8; c.chunk2d = 32; break;
        default: c.warps2d = 2; c.chunk2d = 16; break;
        }
    } else if (p.ndim == 3) {
        // 512-thread CTAs of 31 x 15 updated cells, 3 resident per SM at <= 40
        // registers (456 slots on the 152 SMs of a GB300), short z marches:
        // at 512^3 over marches {16..512}, FP64 32 planes 6926 us (64: 7016,
        // 512: 7388), DF64 32: 2011 (64: 2043), FP32_RB 16: 1196 (64: 1236).
        // Grids too small for whole waves at that length take the longest
        // march that fills the slots best (wave quantization).
        const int rows = 16, tw = 31;
        const long long slots = 3LL * sm_count();
        const long long bxy = (long long)((p.nx - 2 + tw - 1) / tw) * ((p.ny - 2 + rows - 2) / (rows - 1));
        const int pref = p.precision == PTD_PREC_FP32_RB ? 16 : 32;
        const long long nb = bxy * ((p.nz - 2 + pref - 1) / pref);
        c.chunk3d = nb >= 4 * slots ? pref : z_chunk(bxy, p.nz, slots);
        c.rows3d = rows;
    }
    return c;
}

}  // namespace ptd
