// On-device galactic-binary waveforms for batches of sources, written to
// memory (sources with a waveform buffer; the others are generated by the
// fused kernel while it stages its input).  The models are those of
// flr_gbwave.cuh, at t_i = t0 + i dt.
//
// One persistent launch covers every source of a batch: work items are
// (source, chunk of kChunk samples), strided over the grid; the source of a
// chunk is found by binary search in the per-source chunk prefix sums.
#include <cuda_runtime.h>

#include "flr_fused.h"
#include "flr_gbwave.cuh"

namespace flr {
namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 2048;

__global__ void __launch_bounds__(kThreads)
gb_waveform_kernel(const FusedSource *src, const GbParams *par, const long *chunk_start,
                   int num_sources, double dt) {
    const long num_chunks = chunk_start[num_sources];
    for (long c = blockIdx.x; c < num_chunks; c += gridDim.x) {
        // source of chunk c: chunk_start is the exclusive prefix sum of chunks
        int lo = 0, hi = num_sources - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (chunk_start[mid] <= c)
                lo = mid;
            else
                hi = mid - 1;
        }
        const FusedSource &s = src[lo];
        if (s.h == nullptr) continue;  // generated inside the fused kernel instead
        const GbCoefs g = gb_coefs(par[lo]);
        const long i0 = (c - chunk_start[lo]) * kChunk;
        double2 *h = const_cast<double2 *>(s.h);
        for (long i = i0 + threadIdx.x; i < min(i0 + kChunk, s.n); i += kThreads)
            h[i] = gb_sample(g, s.t0 + (double)i * dt);
    }
}

}  // namespace

long gb_waveform_chunks(long n) { return (n + kChunk - 1) / kChunk; }

cudaError_t launch_gb_waveforms(const FusedSource *src, const GbParams *par,
                                const long *chunk_start, int num_sources, double dt, int grid,
                                cudaStream_t stream) {
    if (num_sources <= 0) return cudaSuccess;
    gb_waveform_kernel<<<grid, kThreads, 0, stream>>>(src, par, chunk_start, num_sources, dt);
    return cudaGetLastError();
}

}  // namespace flr
