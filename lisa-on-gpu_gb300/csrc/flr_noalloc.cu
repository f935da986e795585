// flr_get_response_noalloc: the link-projection entry point for callers that
// must not allocate device memory.
//
// Who needs it: code that runs inside a framework which owns the GPU's memory
// (JAX/XLA and TensorFlow pre-allocate most of it, so a foreign cudaMalloc
// can fail), and samplers that call the response thousands of times per
// second from a tight loop (cudaMalloc/cudaFree synchronise the device and
// stall the other streams).  The regular
// entry point needs an orbit handle whose creation allocates the tables'
// derived segment slopes and the status word; this variant keeps those in a
// fixed-size array compiled into the library instead.
//
// The scratch is `g_noalloc_scratch`, a file-scope __device__ array that
// every GPU which loads this library holds until the process exits
// (FLR_NOALLOC_MAX_KNOTS orbit knots: (32768 - 1) * 15 doubles of slopes plus
// the status word, 3.9 MB).  Host code may not use the array's name as a
// device address (on the host it names a stand-in object), so the first call
// on each device, with that device current, looks the address up with
// cudaGetSymbolAddress and caches it; that first call may load the module
// and should therefore come before any stream capture.  Each call first
// rewrites the slopes and clears the status word, then runs the same response
// kernel as flr_get_response.  All calls share the one array: calls whose
// work overlaps on the GPU (different streams, no ordering between them)
// race on it.  Results of a call are identical, bit for bit, to
// flr_get_response with the same tables.
//
// The kernel's status bits (an interpolation window that leaves the input, an
// A-table index out of range) land in the array's status word, which the next
// call clears: flr_noalloc_status() reads it (and optionally clears it)
// without allocating, so it holds the result of the latest call only.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/flr_gb300.h"
#include "flr_internal.h"

namespace {

constexpr long kSlopeDoubles = (long)(FLR_NOALLOC_MAX_KNOTS - 1) * 15;
constexpr long kScratchDoubles = kSlopeDoubles + 32;  // slopes, then the status word

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
double *g_scratch_ptr[kMaxDevices] = {nullptr};

int noalloc_fail(int code, const std::string &msg) {
    // a handled CUDA error must not resurface in a later, unrelated check
    if (code == FLR_E_CUDA) cudaGetLastError();
    flr::set_last_error(msg);
    return code;
}

// Device address of the scratch array on the current device (looked up once
// per device).
cudaError_t scratch_address(double **out) {
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> guard(g_lock);
    if (!g_scratch_ptr[dev]) {
        double *p = nullptr;
        err = cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_noalloc_scratch);
        if (err != cudaSuccess) return err;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

// Segment slopes (hi - lo) / dt of both tables and a cleared status word.
__global__ void noalloc_prepare_kernel(const double *ltt, const double *x, int N, double dt,
                                       double *scratch) {
    const long n_ltt = (long)(N - 1) * 6, n_x = (long)(N - 1) * 9;
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < n_ltt) scratch[idx] = (ltt[idx + 6] - ltt[idx]) / dt;
    if (idx < n_x) scratch[n_ltt + idx] = (x[idx + 9] - x[idx]) / dt;
    if (idx == 0) *reinterpret_cast<unsigned *>(scratch + kSlopeDoubles) = 0u;
}

}  // namespace

extern "C" int flr_get_response_noalloc(double orbit_dt, int orbit_N, const double *ltt_arr,
                                        const double *x_arr, const int *links, const int *sc_r,
                                        const int *sc_e, double *y_gw, const double *t_data,
                                        const double *k_in, const double *u_in,
                                        const double *v_in, double dt, int num_delays,
                                        const void *input_in, int num_inputs, int order,
                                        double sampling_frequency, int buffer_integer,
                                        const double *A_in, double deps, int num_A,
                                        const double *E_in, int projections_start_ind,
                                        void *stream) {
    (void)dt;
    (void)buffer_integer;
    flr::set_last_error("");
    if (orbit_N < 2 || orbit_N > FLR_NOALLOC_MAX_KNOTS)
        return noalloc_fail(FLR_E_INVALID_ARGUMENT,
                            "orbit_N must be in [2, " + std::to_string(FLR_NOALLOC_MAX_KNOTS) +
                                "] for the allocation-free entry point, got " +
                                std::to_string(orbit_N));
    if (!(orbit_dt > 0.0)) return noalloc_fail(FLR_E_INVALID_ARGUMENT, "orbit_dt must be positive");
    if (!ltt_arr || !x_arr || !links || !sc_r || !sc_e || !y_gw || !t_data || !k_in || !u_in ||
        !v_in || !input_in || !A_in || (order > 2 && !E_in))
        return noalloc_fail(FLR_E_INVALID_ARGUMENT, "array arguments must not be NULL");
    if (order < 1 || order > FLR_MAX_ORDER || num_A < 2 || !(deps > 0.0) ||
        !(sampling_frequency > 0.0) || num_delays < 1 || num_inputs < 1 ||
        projections_start_ind < 0)
        return noalloc_fail(FLR_E_INVALID_ARGUMENT, "invalid order, table or size arguments");
    if (reinterpret_cast<uintptr_t>(input_in) % 16 != 0)
        return noalloc_fail(FLR_E_INVALID_ARGUMENT, "input_in (complex128) must be 16-byte aligned");
    for (int s = 0; s < 6; ++s)
        if (sc_r[s] < 1 || sc_r[s] > 3 || sc_e[s] < 1 || sc_e[s] > 3)
            return noalloc_fail(FLR_E_INVALID_ARGUMENT, "sc_r/sc_e must hold spacecraft numbers 1..3");

    double *scratch = nullptr;
    cudaError_t err = scratch_address(&scratch);
    if (err != cudaSuccess)
        return noalloc_fail(FLR_E_CUDA, std::string("cudaGetSymbolAddress: ") +
                                            cudaGetErrorString(err));

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long n_x = (long)(orbit_N - 1) * 9;
    noalloc_prepare_kernel<<<(unsigned)((n_x + 255) / 256), 256, 0, s>>>(ltt_arr, x_arr, orbit_N,
                                                                          orbit_dt, scratch);
    err = cudaGetLastError();
    if (err != cudaSuccess)
        return noalloc_fail(FLR_E_CUDA, std::string("launching the slope kernel: ") +
                                            cudaGetErrorString(err));

    flr::ResponseArgs a;
    a.orb.dt = orbit_dt;
    a.orb.N = orbit_N;
    a.orb.ltt = ltt_arr;
    a.orb.x = x_arr;
    a.orb.ltt_slope = scratch;
    a.orb.x_slope = scratch + (long)(orbit_N - 1) * 6;
    for (int i = 0; i < 6; ++i) {
        a.orb.links[i] = links[i];
        a.orb.sc_r[i] = sc_r[i];
        a.orb.sc_e[i] = sc_e[i];
    }
    a.orb.status = reinterpret_cast<unsigned *>(scratch + kSlopeDoubles);
    a.lt.A = A_in;
    a.lt.E = E_in;
    a.lt.deps = deps;
    a.lt.num_A = num_A;
    a.lt.h = (order + 1) / 2;
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
    err = flr::launch_response_plain(a, s);
    if (err != cudaSuccess)
        return noalloc_fail(FLR_E_CUDA, std::string("launching the response kernel: ") +
                                            cudaGetErrorString(err));
    return FLR_OK;
}

extern "C" int flr_noalloc_status(uint32_t *bits, int reset, void *stream) {
    flr::set_last_error("");
    if (!bits) return noalloc_fail(FLR_E_INVALID_ARGUMENT, "bits must not be NULL");
    double *scratch = nullptr;
    cudaError_t err = scratch_address(&scratch);
    if (err != cudaSuccess)
        return noalloc_fail(FLR_E_CUDA, std::string("cudaGetSymbolAddress: ") +
                                            cudaGetErrorString(err));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned *word = reinterpret_cast<unsigned *>(scratch + kSlopeDoubles);
    unsigned value = 0u;
    err = cudaMemcpyAsync(&value, word, sizeof(value), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess && reset) err = cudaMemsetAsync(word, 0, sizeof(unsigned), s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess)
        return noalloc_fail(FLR_E_CUDA, std::string("reading the status word: ") +
                                            cudaGetErrorString(err));
    *bits = value;
    return FLR_OK;
}
