// C ABI of the library (declared in include/flr_gb300.h): argument checks,
// orbit-table ownership, and the launches of the plain FP64 kernels.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/flr_gb300.h"
#include "flr_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t err, const char *what) {
    cudaGetLastError();  // a handled error must not resurface in a later check
    return fail(FLR_E_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

bool aligned(const void *p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

int check_device(const flr_orbits *o) {
    if (!o) return fail(FLR_E_NO_ORBITS, "Must add orbits with add_orbit_information method.");
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return cuda_fail(err, "cudaGetDevice");
    if (dev != o->device)
        return fail(FLR_E_INVALID_ARGUMENT,
                    "orbit handle was created on device " + std::to_string(o->device) +
                        " but device " + std::to_string(dev) + " is current");
    return FLR_OK;
}

}  // namespace

flr::OrbitTables flr::device_tables(const flr_orbits *o) {
    flr::OrbitTables t;
    t.dt = o->dt;
    t.N = o->N;
    t.ltt = o->ltt;
    t.x = o->x;
    t.ltt_slope = o->ltt_slope;
    t.x_slope = o->x_slope;
    for (int s = 0; s < 6; ++s) {
        t.links[s] = o->links[s];
        t.sc_r[s] = o->sc_r[s];
        t.sc_e[s] = o->sc_e[s];
    }
    t.status = o->status;
    return t;
}

namespace {

int check_lagrange(int order, const double *A, double deps, int num_A, const double *E,
                   flr::LagrangeTables &lt) {
    int h = (order + 1) / 2;
    if (order < 1 || order > FLR_MAX_ORDER || h < 1)
        return fail(FLR_E_INVALID_ARGUMENT,
                    "order must be in [1, " + std::to_string(FLR_MAX_ORDER) + "], got " +
                        std::to_string(order));
    if (!A || num_A < 2) return fail(FLR_E_INVALID_ARGUMENT, "A_in must hold num_A >= 2 values");
    if (!(deps > 0.0)) return fail(FLR_E_INVALID_ARGUMENT, "deps must be positive");
    if (h > 1 && !E) return fail(FLR_E_INVALID_ARGUMENT, "E_in must not be NULL");
    lt.A = A;
    lt.E = E;
    lt.deps = deps;
    lt.num_A = num_A;
    lt.h = h;
    return FLR_OK;
}

}  // namespace

void flr::set_last_error(const std::string &msg) { g_last_error = msg; }

extern "C" {

const char *flr_version(void) { return "flr_gb300 0.1.0 sm_103a"; }

int flr_host_alloc(size_t bytes, void **out) {
    g_last_error.clear();
    if (!out) return fail(FLR_E_INVALID_ARGUMENT, "out must not be NULL");
    *out = nullptr;
    if (bytes == 0) return fail(FLR_E_INVALID_ARGUMENT, "bytes must be positive");
    cudaError_t err = cudaHostAlloc(out, bytes, cudaHostAllocPortable);
    if (err != cudaSuccess) {
        *out = nullptr;
        return cuda_fail(err, "allocating page-locked host memory");
    }
    return FLR_OK;
}

int flr_host_free(void *ptr) {
    g_last_error.clear();
    if (!ptr) return FLR_OK;
    cudaError_t err = cudaFreeHost(ptr);
    if (err != cudaSuccess) return cuda_fail(err, "releasing page-locked host memory");
    return FLR_OK;
}

const char *flr_last_error(void) { return g_last_error.c_str(); }

int flr_orbits_create(double dt, int N, const double *n_arr, const double *ltt_arr,
                      const double *x_arr, const int *links, const int *sc_r, const int *sc_e,
                      double armlength, flr_orbits **out) {
    (void)n_arr;  // unused by the response, as in the reference
    g_last_error.clear();
    if (!out) return fail(FLR_E_INVALID_ARGUMENT, "out must not be NULL");
    *out = nullptr;
    if (!(dt > 0.0)) return fail(FLR_E_INVALID_ARGUMENT, "dt must be positive");
    if (N < 2) return fail(FLR_E_INVALID_ARGUMENT, "orbit tables need N >= 2 knots");
    if (!ltt_arr || !x_arr || !links || !sc_r || !sc_e)
        return fail(FLR_E_INVALID_ARGUMENT, "orbit table pointers must not be NULL");

    flr_orbits *o = new (std::nothrow) flr_orbits();
    if (!o) return fail(FLR_E_INVALID_ARGUMENT, "out of host memory");
    o->dt = dt;
    o->N = N;
    o->armlength = armlength;
    cudaError_t err = cudaGetDevice(&o->device);
    if (err != cudaSuccess) {
        delete o;
        return cuda_fail(err, "cudaGetDevice");
    }
    err = cudaMemcpy(o->links, links, sizeof(o->links), cudaMemcpyDefault);
    if (err == cudaSuccess) err = cudaMemcpy(o->sc_r, sc_r, sizeof(o->sc_r), cudaMemcpyDefault);
    if (err == cudaSuccess) err = cudaMemcpy(o->sc_e, sc_e, sizeof(o->sc_e), cudaMemcpyDefault);
    if (err != cudaSuccess) {
        delete o;
        return cuda_fail(err, "copying link tables");
    }
    for (int s = 0; s < 6; ++s) {
        if (o->sc_r[s] < 1 || o->sc_r[s] > 3 || o->sc_e[s] < 1 || o->sc_e[s] > 3) {
            delete o;
            return fail(FLR_E_INVALID_ARGUMENT, "sc_r/sc_e must hold spacecraft numbers 1..3");
        }
    }

    const size_t n_ltt = (size_t)N * 6, n_x = (size_t)N * 9;
    const size_t n_ltt_s = (size_t)(N - 1) * 6, n_x_s = (size_t)(N - 1) * 9;
    const size_t bytes = (n_ltt + n_x + n_ltt_s + n_x_s) * sizeof(double) + 256;
    err = cudaMalloc(&o->block, bytes);
    if (err != cudaSuccess) {
        delete o;
        return cuda_fail(err, "cudaMalloc(orbit tables)");
    }
    double *p = static_cast<double *>(o->block);
    o->ltt = p;
    o->x = o->ltt + n_ltt;
    o->ltt_slope = o->x + n_x;
    o->x_slope = o->ltt_slope + n_ltt_s;
    o->status = reinterpret_cast<unsigned *>(o->x_slope + n_x_s);

    err = cudaMemcpy(o->ltt, ltt_arr, n_ltt * sizeof(double), cudaMemcpyDefault);
    if (err == cudaSuccess) err = cudaMemcpy(o->x, x_arr, n_x * sizeof(double), cudaMemcpyDefault);
    if (err == cudaSuccess) err = cudaMemset(o->status, 0, sizeof(unsigned));
    if (err == cudaSuccess)
        err = flr::launch_orbit_slopes(o->ltt, o->ltt_slope, (long)n_ltt_s, 6, dt, 0);
    if (err == cudaSuccess)
        err = flr::launch_orbit_slopes(o->x, o->x_slope, (long)n_x_s, 9, dt, 0);
    if (err == cudaSuccess) err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        cudaFree(o->block);
        delete o;
        return cuda_fail(err, "uploading orbit tables");
    }
    *out = o;
    return FLR_OK;
}

int flr_orbits_destroy(flr_orbits *orbits) {
    g_last_error.clear();
    if (!orbits) return FLR_OK;
    cudaError_t err = cudaFree(orbits->block);
    delete orbits;
    if (err != cudaSuccess) return cuda_fail(err, "cudaFree(orbit tables)");
    return FLR_OK;
}

int flr_orbits_status(flr_orbits *orbits, uint32_t *bits, int reset, void *stream) {
    g_last_error.clear();
    int rc = check_device(orbits);
    if (rc) return rc;
    if (!bits) return fail(FLR_E_INVALID_ARGUMENT, "bits must not be NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned host = 0;
    cudaError_t err = cudaMemcpyAsync(&host, orbits->status, sizeof(unsigned),
                                      cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess && reset) err = cudaMemsetAsync(orbits->status, 0, sizeof(unsigned), s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return cuda_fail(err, "reading the status word");
    *bits = host;
    if (host & FLR_STATUS_STAGING_LOST)
        g_last_error = "a staging copy of the batched kernel never completed: discard every "
                       "output of the batches run since the status was last cleared";
    else if (host & FLR_STATUS_STAGING)
        g_last_error = "a staging copy of the batched kernel completed late: the outputs of its "
                       "work item are NaN";
    return FLR_OK;
}

int flr_get_response(flr_orbits *orbits, double *y_gw, const double *t_data, const double *k_in,
                     const double *u_in, const double *v_in, double dt, int num_delays,
                     const void *input_in, int num_inputs, int order, double sampling_frequency,
                     int buffer_integer, const double *A_in, double deps, int num_A,
                     const double *E_in, int projections_start_ind, void *stream) {
    (void)dt;
    (void)buffer_integer;
    g_last_error.clear();
    int rc = check_device(orbits);
    if (rc) return rc;
    flr::ResponseArgs a;
    rc = check_lagrange(order, A_in, deps, num_A, E_in, a.lt);
    if (rc) return rc;
    if (!y_gw || !t_data || !k_in || !u_in || !v_in || !input_in)
        return fail(FLR_E_INVALID_ARGUMENT, "array arguments must not be NULL");
    if (num_delays < 1 || num_inputs < 1 || projections_start_ind < 0)
        return fail(FLR_E_INVALID_ARGUMENT, "num_delays/num_inputs must be positive and "
                                            "projections_start_ind non-negative");
    if (!aligned(input_in, 16))
        return fail(FLR_E_INVALID_ARGUMENT, "input_in (complex128) must be 16-byte aligned");
    if (!(sampling_frequency > 0.0))
        return fail(FLR_E_INVALID_ARGUMENT, "sampling_frequency must be positive");
    a.orb = flr::device_tables(orbits);
    a.y_gw = y_gw;
    a.t_data = t_data;
    a.k = k_in;
    a.u = u_in;
    a.v = v_in;
    a.input = static_cast<const double2 *>(input_in);
    a.num_delays = num_delays;
    a.num_inputs = num_inputs;
    a.fs = sampling_frequency;
    a.start = projections_start_ind;
    cudaError_t err = flr::launch_response_plain(a, static_cast<cudaStream_t>(stream));
    if (err != cudaSuccess) return cuda_fail(err, "launching the response kernel");
    return FLR_OK;
}

static int tdi_delays(flr_orbits *orbits, double *delayed_links, const double *input_links,
                      int num_inputs, int num_delays, const double *t_arr,
                      const int *unit_starts, const int *unit_lengths, const int *tdi_base_link,
                      const int *tdi_link_combinations, const double *tdi_signs,
                      const int *channels, int num_units, int num_channels, int order,
                      double sampling_frequency, const double *A_in, double deps, int num_A,
                      const double *E_in, int tdi_start_ind, double *aet, int aet_rows,
                      void *stream) {
    g_last_error.clear();
    int rc = check_device(orbits);
    if (rc) return rc;
    flr::TdiArgs a;
    rc = check_lagrange(order, A_in, deps, num_A, E_in, a.lt);
    if (rc) return rc;
    if (!delayed_links || !input_links || !t_arr || !unit_starts || !unit_lengths ||
        !tdi_base_link || !tdi_link_combinations || !tdi_signs || !channels)
        return fail(FLR_E_INVALID_ARGUMENT, "array arguments must not be NULL");
    if (num_delays < 1 || num_inputs < 1 || tdi_start_ind < 0 || num_units < 0 ||
        num_channels < 0 || num_channels > 65535)
        return fail(FLR_E_INVALID_ARGUMENT, "invalid sizes");
    if (aet && (num_channels != 3 || (aet_rows != 2 && aet_rows != 3)))
        return fail(FLR_E_INVALID_ARGUMENT, "A, E, T need num_channels 3 and aet_rows 2 or 3");
    a.aet = aet;
    a.aet_rows = aet ? aet_rows : 0;
    if (!(sampling_frequency > 0.0))
        return fail(FLR_E_INVALID_ARGUMENT, "sampling_frequency must be positive");
    a.orb = flr::device_tables(orbits);
    a.out = delayed_links;
    a.y = input_links;
    a.num_inputs = num_inputs;
    a.num_delays = num_delays;
    a.t_arr = t_arr;
    a.unit_starts = unit_starts;
    a.unit_lengths = unit_lengths;
    a.base_link = tdi_base_link;
    a.combos = tdi_link_combinations;
    a.signs = tdi_signs;
    a.channels = channels;
    a.num_units = num_units;
    a.num_channels = num_channels;
    a.fs = sampling_frequency;
    a.start = tdi_start_ind;
    cudaError_t err = flr::launch_tdi_plain(a, static_cast<cudaStream_t>(stream));
    if (err != cudaSuccess) return cuda_fail(err, "launching the TDI kernel");
    return FLR_OK;
}

int flr_get_tdi_delays(flr_orbits *orbits, double *delayed_links, const double *input_links,
                       int num_inputs, int num_delays, const double *t_arr,
                       const int *unit_starts, const int *unit_lengths, const int *tdi_base_link,
                       const int *tdi_link_combinations, const double *tdi_signs,
                       const int *channels, int num_units, int num_channels, int order,
                       double sampling_frequency, int buffer_integer, const double *A_in,
                       double deps, int num_A, const double *E_in, int tdi_start_ind,
                       void *stream) {
    (void)buffer_integer;
    return tdi_delays(orbits, delayed_links, input_links, num_inputs, num_delays, t_arr,
                      unit_starts, unit_lengths, tdi_base_link, tdi_link_combinations, tdi_signs,
                      channels, num_units, num_channels, order, sampling_frequency, A_in, deps,
                      num_A, E_in, tdi_start_ind, nullptr, 0, stream);
}

int flr_get_tdi_delays_aet(flr_orbits *orbits, double *delayed_links, const double *input_links,
                           int num_inputs, int num_delays, const double *t_arr,
                           const int *unit_starts, const int *unit_lengths,
                           const int *tdi_base_link, const int *tdi_link_combinations,
                           const double *tdi_signs, const int *channels, int num_units,
                           int num_channels, int order, double sampling_frequency,
                           int buffer_integer, const double *A_in, double deps, int num_A,
                           const double *E_in, int tdi_start_ind, double *aet, int aet_rows,
                           void *stream) {
    (void)buffer_integer;
    if (!aet) return fail(FLR_E_INVALID_ARGUMENT, "aet must not be NULL");
    return tdi_delays(orbits, delayed_links, input_links, num_inputs, num_delays, t_arr,
                      unit_starts, unit_lengths, tdi_base_link, tdi_link_combinations, tdi_signs,
                      channels, num_units, num_channels, order, sampling_frequency, A_in, deps,
                      num_A, E_in, tdi_start_ind, aet, aet_rows, stream);
}

int flr_response_delay_indices(flr_orbits *orbits, int *d_rec, int *d_em, const double *t_data,
                               const double *k_in, int num_delays, double sampling_frequency,
                               int projections_start_ind, void *stream) {
    g_last_error.clear();
    int rc = check_device(orbits);
    if (rc) return rc;
    if (!d_rec || !d_em || !t_data || !k_in)
        return fail(FLR_E_INVALID_ARGUMENT, "array arguments must not be NULL");
    if (num_delays < 1 || projections_start_ind < 0 || !(sampling_frequency > 0.0))
        return fail(FLR_E_INVALID_ARGUMENT, "invalid sizes");
    flr::ResponseArgs a{};
    a.orb = flr::device_tables(orbits);
    a.t_data = t_data;
    a.k = k_in;
    a.num_delays = num_delays;
    a.fs = sampling_frequency;
    a.start = projections_start_ind;
    cudaError_t err =
        flr::launch_response_indices(a, d_rec, d_em, static_cast<cudaStream_t>(stream));
    if (err != cudaSuccess) return cuda_fail(err, "launching the index kernel");
    return FLR_OK;
}

int flr_tdi_delay_indices(flr_orbits *orbits, int *d_tdi, int num_delays, const double *t_arr,
                          const int *unit_starts, const int *unit_lengths,
                          const int *tdi_link_combinations, int num_units,
                          double sampling_frequency, int tdi_start_ind, void *stream) {
    g_last_error.clear();
    int rc = check_device(orbits);
    if (rc) return rc;
    if (!d_tdi || !t_arr || !unit_starts || !unit_lengths || !tdi_link_combinations)
        return fail(FLR_E_INVALID_ARGUMENT, "array arguments must not be NULL");
    if (num_delays < 1 || tdi_start_ind < 0 || num_units < 0 || num_units > 65535 ||
        !(sampling_frequency > 0.0))
        return fail(FLR_E_INVALID_ARGUMENT, "invalid sizes");
    flr::TdiArgs a{};
    a.orb = flr::device_tables(orbits);
    a.num_delays = num_delays;
    a.t_arr = t_arr;
    a.unit_starts = unit_starts;
    a.unit_lengths = unit_lengths;
    a.combos = tdi_link_combinations;
    a.num_units = num_units;
    a.fs = sampling_frequency;
    a.start = tdi_start_ind;
    cudaError_t err = flr::launch_tdi_indices(a, d_tdi, static_cast<cudaStream_t>(stream));
    if (err != cudaSuccess) return cuda_fail(err, "launching the index kernel");
    return FLR_OK;
}

int flr_xyz_to_aet(const double *xyz, double *aet, int num_delays, int start, int num_rows,
                   void *stream) {
    g_last_error.clear();
    if (!xyz || !aet) return fail(FLR_E_INVALID_ARGUMENT, "array arguments must not be NULL");
    if (num_delays < 1 || start < 0 || (num_rows != 2 && num_rows != 3))
        return fail(FLR_E_INVALID_ARGUMENT, "need num_delays >= 1, start >= 0, num_rows 2 or 3");
    cudaError_t err = flr::launch_xyz_to_aet(xyz, aet, num_delays, start, num_rows,
                                             static_cast<cudaStream_t>(stream));
    if (err != cudaSuccess) return cuda_fail(err, "launching the AET kernel");
    return FLR_OK;
}

}  // extern "C"
