// The difference-form mixed instances for launches whose sources all start at
// t0 = +0 (kT0Zero in flr_fused_kernel.cuh: two FP64 operations fewer per
// sample time and per index split, the same bits), compiled apart from the
// other instances so the builds run in parallel.
#include "flr_fused_kernel.cuh"

namespace flr {

const void *fused_fn_t0(bool grouped) {
    return grouped
               ? reinterpret_cast<const void *>(fused_kernel<true, false, true, false, true, false, true>)
               : reinterpret_cast<const void *>(fused_kernel<true, false, false, false, true, false, true>);
}

}  // namespace flr
