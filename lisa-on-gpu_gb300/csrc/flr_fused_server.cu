// The fused kernel's serving instances (mixed arithmetic; difference forms
// for XYZ outputs, the double-float form for AET / AE; per-unit or grouped
// TDI): items are claimed from a source list that the host appends to while
// the kernel runs (see the serving part of flr_fused_kernel.cuh and
// flr_server_* in flr_batch.cu), compiled apart so the build stays parallel.
#include "flr_fused_kernel.cuh"

namespace flr {

const void *fused_fn_server(bool grouped, bool d2) {
    if (d2)
        return grouped ? reinterpret_cast<const void *>(fused_kernel<true, false, true, false, true, true>)
                       : reinterpret_cast<const void *>(fused_kernel<true, false, false, false, true, true>);
    return grouped ? reinterpret_cast<const void *>(fused_kernel<true, false, true, false, false, true>)
                   : reinterpret_cast<const void *>(fused_kernel<true, false, false, false, false, true>);
}

}  // namespace flr
