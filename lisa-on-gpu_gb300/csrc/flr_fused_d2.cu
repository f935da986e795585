// The mixed kernel instances in difference form (second differences in the
// TDI stage, third differences in the link stage; see flr_fused_kernel.cuh),
// compiled apart from the other instances so the two compile in parallel.
#include "flr_fused_kernel.cuh"

namespace flr {

const void *fused_fn_d2(bool grouped, bool diag, bool inner) {
    if (inner)
        return grouped ? reinterpret_cast<const void *>(fused_kernel<true, false, true, true, true>)
                       : reinterpret_cast<const void *>(fused_kernel<true, false, false, true, true>);
    if (grouped)
        return diag ? reinterpret_cast<const void *>(fused_kernel<true, true, true, false, true>)
                    : reinterpret_cast<const void *>(fused_kernel<true, false, true, false, true>);
    return diag ? reinterpret_cast<const void *>(fused_kernel<true, true, false, false, true>)
                : reinterpret_cast<const void *>(fused_kernel<true, false, false, false, true>);
}

}  // namespace flr
