// On-device galactic-binary waveforms for batches of sources.
//
// h(t) = hp + i hc with
//   Phi = phi0 + 2 pi (f t + fdot t^2 / 2),
//   hp0 = A (1 + cos^2 iota) cos Phi,   hc0 = -2 A cos iota sin Phi,
//   hp  = hp0 cos 2psi - hc0 sin 2psi,  hc  = hp0 sin 2psi + hc0 cos 2psi,
// at t_i = t0 + i dt, the drifting-monochromatic binary of the benchmark
// configurations.  Evaluated in FP64 in the operation order of the host
// generator (fastlisaresponse_gb300.waveforms.gb_waveform) with CUDA's double
// sincos, so it agrees with the host generator to a few ulp.
//
// One persistent launch covers every source of a batch: work items are
// (source, chunk of kChunk samples), strided over the grid; the source of a
// chunk is found by binary search in the per-source chunk prefix sums.
#include <cuda_runtime.h>

#include "flr_fused.h"

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
        const GbParams p = par[lo];
        const long i0 = (c - chunk_start[lo]) * kChunk;
        const double cosi = cos(p.iota);
        const double amp_p = p.A * (1.0 + cosi * cosi);
        const double amp_c = -2.0 * p.A * cosi;
        double s2, c2;
        sincos(2.0 * p.psi, &s2, &c2);
        double2 *h = const_cast<double2 *>(s.h);
        for (long i = i0 + threadIdx.x; i < min(i0 + kChunk, s.n); i += kThreads) {
            const double t = s.t0 + (double)i * dt;
            const double phase = p.phi0 + 6.283185307179586 * (p.f * t + 0.5 * p.fdot * t * t);
            double sp, cp;
            sincos(phase, &sp, &cp);
            const double hp0 = amp_p * cp;
            const double hc0 = amp_c * sp;
            h[i] = make_double2(hp0 * c2 - hc0 * s2, hp0 * s2 + hc0 * c2);
        }
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
