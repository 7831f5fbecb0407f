// ptd_tune.cu -- launch-shape choice for the fused kernels.
#include "ptd_internal.h"

namespace ptd {

LaunchCfg tuned_config(const ptd_params& p)
{
    LaunchCfg c;
    if (p.ndim == 2) {
        // enough y chunks for ~8 blocks per SM on 152 SMs, chunk >= 16 rows
        const int tiles = (p.nx - 2 + 30) / 31;
        const int bx = (tiles + c.warps2d - 1) / c.warps2d;
        int chunk = 128;
        while (chunk > 16 && (long long)bx * ((p.ny - 2 + chunk - 1) / chunk) < 152 * 8) chunk /= 2;
        c.chunk2d = chunk;
    } else if (p.ndim == 3) {
        const int rows = 16;
        const long long bxy = (long long)((p.nx - 2 + 30) / 31) * ((p.ny - 2 + rows - 2) / (rows - 1));
        int chunk = 256;
        while (chunk > 16 && bxy * ((p.nz - 2 + chunk - 1) / chunk) < 152 * 4) chunk /= 2;
        c.chunk3d = chunk;
        c.rows3d = rows;
    }
    return c;
}

}  // namespace ptd
