// ptd_dc.cu -- FP32 PT iterations inside an FP64 defect-correction loop.
#include "ptd_internal.h"

namespace ptd {

struct DcState {
    DcCounters k;
};

int dc_create(const ptd_ctx_base&, const ptd_params&, const Derived&, cudaStream_t, DcState**)
{
    return set_error(PTD_EINVAL, "precision FP32_DC is not available in this build");
}
void dc_destroy(DcState* dc) { delete dc; }
int dc_set_state(DcState*, const ptd_ctx_base&, double*, double*, const double*, cudaStream_t) { return PTD_EINVAL; }
int dc_step(DcState*, const ptd_ctx_base&, int32_t*, double*, int32_t, int32_t*, int*, int*) { return PTD_EINVAL; }
int dc_iterate(DcState*, const ptd_ctx_base&, int32_t) { return PTD_EINVAL; }
const double* dc_current(const DcState*) { return nullptr; }
DcCounters dc_counters(const DcState* dc) { return dc ? dc->k : DcCounters{}; }

}  // namespace ptd
