// flr_probe.h -- arithmetic-pipe throughput probe of the benchmark (not part of
// the product library's C ABI; built into its own libflr_probe.so).
#ifndef FLR_PROBE_H
#define FLR_PROBE_H

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Runs blocks x threads threads, each `iters` iterations of 8 independent
 * operations of `kind` (0 = FP64 FMA, 1 = FP64 division, 2 = FP32 FMA), timed
 * with CUDA events on `stream`; synchronises.  The benchmark uses the rates as
 * the measured FP64-pipe peak of its roofline (the machine's measured-peak
 * table lists HBM bandwidth and bf16 tensor throughput only).  `sink` is a
 * device buffer of `blocks` doubles.  Returns 0, -1 (invalid argument) or
 * -2 (CUDA error).
 */
int flr_probe_pipe_rate(int kind, long iters, int blocks, int threads, double *sink,
                        float *elapsed_ms, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FLR_PROBE_H */
