// Batched, fused response + TDI: kernel instances and launches (device code
// in flr_fused_kernel.cuh; the difference-form instances in flr_fused_d2.cu).
#include <algorithm>

#include "flr_fused_kernel.cuh"

namespace flr {

size_t fused_smem_bytes(bool mixed, int win_max, int y_max) {
    return layout(mixed, win_max, y_max).total;
}

static const void *fused_fn(bool mixed, bool grouped, bool diag, bool inner, bool d2,
                            bool t0_zero = false) {
    if (mixed && d2 && t0_zero && !diag && !inner) return fused_fn_t0(grouped);
    if (mixed && d2) return fused_fn_d2(grouped, diag, inner);
    if (inner) {
        if (mixed && grouped)
            return reinterpret_cast<const void *>(fused_kernel<true, false, true, true, false>);
        if (mixed)
            return reinterpret_cast<const void *>(fused_kernel<true, false, false, true, false>);
        return reinterpret_cast<const void *>(fused_kernel<false, false, false, true, false>);
    }
    if (mixed && grouped)
        return diag ? reinterpret_cast<const void *>(fused_kernel<true, true, true, false, false>)
                    : reinterpret_cast<const void *>(fused_kernel<true, false, true, false, false>);
    if (mixed)
        return diag ? reinterpret_cast<const void *>(fused_kernel<true, true, false, false, false>)
                    : reinterpret_cast<const void *>(fused_kernel<true, false, false, false, false>);
    return diag ? reinterpret_cast<const void *>(fused_kernel<false, true, false, false, false>)
                : reinterpret_cast<const void *>(fused_kernel<false, false, false, false, false>);
}

cudaError_t fused_configure(bool mixed, bool grouped, size_t smem_bytes, int *blocks_per_sm) {
    // plain, diagnostics, inner products; both forms of the mixed flavour, and
    // the difference form's t0 = 0 instance
    for (int v = 0; v < (mixed ? 7 : 3); ++v) {
        cudaError_t err = cudaFuncSetAttribute(fused_fn(mixed, grouped, v % 3 == 1 && v < 6,
                                                        v % 3 == 2, v >= 3, v == 6),
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem_bytes);
        if (err != cudaSuccess) return err;
    }
    // the grid is sized for the fewest blocks per SM of the instances launched alone
    int per = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per, fused_fn(mixed, grouped, false, false, false), kThreads, smem_bytes);
    for (int v = 0; v < 2 && err == cudaSuccess && mixed; ++v) {
        int per2 = 0;
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per2, fused_fn(mixed, grouped, false, false, true, v == 1), kThreads, smem_bytes);
        per = std::min(per, per2);
    }
    *blocks_per_sm = per;
    return err;
}

cudaError_t launch_fused(bool mixed, bool grouped, bool diag, bool inner, bool d2, bool t0_zero,
                         const FusedArgs &a, int grid, size_t smem_bytes, cudaStream_t stream) {
    if (a.num_sources <= 0) return cudaSuccess;
    if (diag && inner) return cudaErrorInvalidValue;
    void *args[] = {const_cast<FusedArgs *>(&a)};
    return cudaLaunchKernel(fused_fn(mixed, grouped, diag, inner, d2, t0_zero), dim3(grid),
                            dim3(kThreads), args, smem_bytes, stream);
}

cudaError_t launch_fused_server(bool grouped, bool d2, const FusedArgs &a, int grid,
                                size_t smem_bytes, cudaStream_t stream) {
    const void *fn = fused_fn_server(grouped, d2);
    cudaError_t err =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (err != cudaSuccess) return err;
    void *args[] = {const_cast<FusedArgs *>(&a)};
    return cudaLaunchKernel(fn, dim3(grid), dim3(kThreads), args, smem_bytes, stream);
}

cudaError_t launch_inner_reduce(const FusedArgs &a, cudaStream_t stream) {
    if (a.num_sources <= 0) return cudaSuccess;
    const long threads = 6L * a.num_sources;
    inner_reduce_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, stream>>>(
        a.sources, a.tile_start, a.num_sources, a.partial);
    return cudaGetLastError();
}

}  // namespace flr
