// Internal launch interface between the C ABI (flr_capi.cu) and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "flr_device.cuh"

// Orbit handle of the C ABI (opaque to callers).
struct flr_orbits {
    int device;
    double dt;
    int N;
    double armlength;
    int links[6];
    int sc_r[6];
    int sc_e[6];
    void *block;          // one device allocation holding everything below
    double *ltt;          // [N][6]
    double *x;            // [N][9]
    double *ltt_slope;    // [N-1][6]
    double *x_slope;      // [N-1][9]
    unsigned *status;     // status word
};

namespace flr {

// Kernel-side view of an orbit handle.
OrbitTables device_tables(const flr_orbits *o);

struct ResponseArgs {
    OrbitTables orb;
    LagrangeTables lt;
    double *y_gw;            // [6][num_delays]
    const double *t_data;    // [num_delays]
    const double *k, *u, *v; // [3] each
    const double2 *input;    // [num_inputs] complex128
    long num_delays;
    long num_inputs;
    double fs;
    int start;               // projections_start_ind
};

struct TdiArgs {
    OrbitTables orb;
    LagrangeTables lt;
    double *out;             // [num_channels][num_delays], accumulated into
    const double *y;         // [6][num_inputs]
    long num_inputs;
    long num_delays;
    const double *t_arr;     // [num_delays]
    const int *unit_starts, *unit_lengths, *base_link, *combos, *channels;
    const double *signs;
    int num_units;
    int num_channels;
    double fs;
    int start;               // tdi_start_ind
    // optional epilogue (num_channels == 3): A, E, T (aet_rows 3) or A, E (2)
    // of the accumulated X, Y, Z, [aet_rows][num_delays]; NULL: none
    double *aet = nullptr;
    int aet_rows = 0;
};

cudaError_t launch_response_plain(const ResponseArgs &a, cudaStream_t stream);
cudaError_t launch_tdi_plain(const TdiArgs &a, cudaStream_t stream);
cudaError_t launch_response_indices(const ResponseArgs &a, int *d_rec, int *d_em,
                                    cudaStream_t stream);
cudaError_t launch_tdi_indices(const TdiArgs &a, int *d_out, cudaStream_t stream);
// Sets the text flr_last_error() returns on the calling thread.
void set_last_error(const std::string &msg);

cudaError_t launch_xyz_to_aet(const double *xyz, double *aet, long n, long start, int rows,
                              cudaStream_t stream);
cudaError_t launch_orbit_slopes(const double *tab, double *slope, long n, int stride, double dt,
                                cudaStream_t stream);

}  // namespace flr
