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
        // short y marches in 2-warp CTAs: many independent warps per SM hide
        // the memory latency of the march.  Measured at 4096^2 over warps
        // {1,2,4,8} x rows {4..64}: 16 rows is the best or within 2 % of it
        // for every arithmetic form (FP64 -6 %, DFH -11 %, DF64 -16 % against
        // 4 warps x 64 rows); the one recomputed face below each march costs
        // 1/16 of the y faces.
        c.warps2d = 2;
        c.chunk2d = 16;
    } else if (p.ndim == 3) {
        // 512-thread CTAs of 31 x 15 updated cells, 3 resident per SM at <= 40
        // registers (456 slots on the 152 SMs of a GB300).
        const int rows = 16, tw = 31;
        const long long slots = 3LL * sm_count();
        const long long bxy = (long long)((p.nx - 2 + tw - 1) / tw) * ((p.ny - 2 + rows - 2) / (rows - 1));
        const int best = z_chunk(bxy, p.nz, slots);
        c.chunk3d = best;
        c.rows3d = rows;
    }
    return c;
}

}  // namespace ptd
