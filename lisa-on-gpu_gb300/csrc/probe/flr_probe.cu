// Arithmetic-pipe throughput probes of the benchmark (libflr_probe.so, not the
// product library).
//
// The response + TDI kernels are bound by the FP64 pipe, whose peak is not in
// the measured-peak table of the machine (it lists HBM bandwidth and bf16
// tensor throughput).  These kernels measure it the same way those peaks are
// measured -- a saturating loop timed with CUDA events -- so the roofline
// fraction of the response kernels has a measured denominator.
//
//   kind 0: FP64 fused multiply-add  (8 independent chains per thread)
//   kind 1: FP64 correctly rounded division (8 independent chains, x <- a/x)
//   kind 2: FP32 fused multiply-add  (8 independent chains)
//
// Every thread runs `iters` iterations of 8 operations; the chains are folded
// into `sink` so nothing is dead code.  Operation count = blocks * threads *
// iters * 8.
#include <cuda_runtime.h>

#include "flr_probe.h"

namespace {

__global__ void probe_dfma(long iters, double a, double b, double *sink) {
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = threadIdx.x * 1e-3 + c;
    for (long it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    if (s == 1.2345e300) sink[blockIdx.x] = s;
}

__global__ void probe_ddiv(long iters, double a, double b, double *sink) {
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = threadIdx.x * 1e-3 + c + 1.0;
    for (long it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = a / x[c];
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    if (s == 1.2345e300) sink[blockIdx.x] = s;
}

__global__ void probe_ffma(long iters, float a, float b, double *sink) {
    float x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = threadIdx.x * 1e-3f + c;
    for (long it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    if (s == 1.2345e30f) sink[blockIdx.x] = s;
}

}  // namespace

extern "C" int flr_probe_pipe_rate(int kind, long iters, int blocks, int threads, double *sink,
                                   float *elapsed_ms, void *stream) {
    if (kind < 0 || kind > 2 || iters < 1 || blocks < 1 || threads < 32 || threads > 1024 ||
        !sink || !elapsed_ms)
        return -1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return -2;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return -2;
    }
    cudaEventRecord(e0, s);
    if (kind == 0)
        probe_dfma<<<blocks, threads, 0, s>>>(iters, 0.999999, 1e-7, sink);
    else if (kind == 1)
        probe_ddiv<<<blocks, threads, 0, s>>>(iters, 0.75, 0.0, sink);
    else
        probe_ffma<<<blocks, threads, 0, s>>>(iters, 0.999999f, 1e-7f, sink);
    cudaEventRecord(e1, s);
    cudaError_t err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaEventElapsedTime(elapsed_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return err == cudaSuccess ? 0 : -2;
}
