// Plain FP64 response and TDI kernels (sm_103a).
//
// Compiled with --fmad=false (see flr_device.cuh): these kernels reproduce the
// reference's CPU arithmetic bit for bit.  Parallel layout:
//
//   response: one thread per (sample, link); a 1-D grid of ceil(n/256) * 6
//             blocks, the six links of a 256-sample tile in consecutive blocks
//             (they read the same input window, which L2 then serves).  Each
//             thread evaluates the geometry of its link at its sample and the
//             two complex Lagrange interpolations (LISAResponse.cu:431-672).
//   TDI:      one thread per (sample, channel); the channels of a tile in
//             consecutive blocks likewise (they read the same link windows).
//             The thread walks the units of its channel in unit order and
//             accumulates into a register, so the sum order is that of the
//             reference's CPU loop (LISAResponse.cu:300-396) and deterministic
//             (the reference's GPU kernel uses atomicAdd, LISAResponse.cu:389).
//
// Both are FP64-pipe bound: the tap loops issue two IEEE divisions per tap and
// component.  Inputs are read through the read-only data cache; a block's 256
// consecutive samples touch a contiguous input window of roughly
// 256 + 2h + (delay spread) samples, so each tap value is fetched from DRAM
// once and served from L1/L2 afterwards.
#include <cuda_runtime.h>

#include "flr_device.cuh"
#include "flr_internal.h"

namespace flr {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double quiet_nan() {
    return __longlong_as_double(0x7ff8000000000000ll);
}

__global__ void __launch_bounds__(kThreads)
response_plain_kernel(ResponseArgs a) {
    const int slot = (int)(blockIdx.x % kLinks);
    const long i = (long)a.start + (long)(blockIdx.x / kLinks) * kThreads + threadIdx.x;
    if (i >= a.num_delays - a.start) return;

    const double k[3] = {__ldg(a.k), __ldg(a.k + 1), __ldg(a.k + 2)};
    const double u[3] = {__ldg(a.u), __ldg(a.u + 1), __ldg(a.u + 2)};
    const double v[3] = {__ldg(a.v), __ldg(a.v + 1), __ldg(a.v + 2)};
    const double t = __ldg(a.t_data + i);
    const double t_first = __ldg(a.t_data);

    LinkGeometry g = link_geometry(a.orb, slot, t, t_first, a.fs, k, u, v);

    const int h = a.lt.h;
    const long lo = (long)min(g.d_rec, g.d_em) - (h - 1);
    const long hi = (long)max(g.d_rec, g.d_em) + h;
    double *out = a.y_gw + (size_t)slot * a.num_delays + i;
    if (lo < 0 || hi >= a.num_inputs) {
        raise_status(a.orb.status, kStatusTap);
        *out = quiet_nan();
        return;
    }
    double A_rec, A_em;
    bool ok = prefactor(a.lt, g.e_rec, A_rec);
    ok = prefactor(a.lt, g.e_em, A_em) && ok;
    if (!ok) {
        raise_status(a.orb.status, kStatusAIndex);
        *out = quiet_nan();
        return;
    }
    double hp_rec, hc_rec, hp_em, hc_em;
    const GlobalC128 src{a.input};
    lagrange_c128(src, g.d_rec, g.e_rec, A_rec, a.lt, hp_rec, hc_rec);
    lagrange_c128(src, g.d_em, g.e_em, A_em, a.lt, hp_em, hc_em);

    double pre = 1. / (1. - g.k_dot_n);
    double big = (hp_em - hp_rec) * g.xi_p + (hc_em - hc_rec) * g.xi_c;
    *out = pre * big;
}

// One thread per (sample, channel), the channel rows of a tile in
// consecutive blocks: for more than three channels.
__global__ void __launch_bounds__(kThreads)
tdi_plain_channel_kernel(TdiArgs a) {
    const int channel = (int)(blockIdx.x % (unsigned)a.num_channels);
    const long i =
        (long)a.start + (long)(blockIdx.x / (unsigned)a.num_channels) * kThreads + threadIdx.x;
    if (i >= a.num_delays - a.start) return;

    const double t = __ldg(a.t_arr + i);
    const double t_first = __ldg(a.t_arr);
    // L(t) of every link slot; the reference re-evaluates the same
    // interpolation for each list entry (LISAResponse.cu:331), which yields
    // these values.
    double L[kLinks];
#pragma unroll
    for (int s = 0; s < kLinks; ++s) L[s] = light_travel_time(a.orb, t, s);

    double *out = a.out + (size_t)channel * a.num_delays + i;
    double acc = *out;
    const int h = a.lt.h;
    for (int unit = 0; unit < a.num_units; ++unit) {
        const int ch = __ldg(a.channels + unit);
        if (ch < 0 || ch >= a.num_channels) {
            raise_status(a.orb.status, kStatusChannel);
            continue;
        }
        if (ch != channel) continue;
        double delay = t;
        bool link_ok = true;
        const int s0 = __ldg(a.unit_starts + unit), n_s = __ldg(a.unit_lengths + unit);
        for (int s = 0; s < n_s; ++s) {
            const int link = __ldg(a.combos + s0 + s);
            if (link == kNoLink) continue;
            const int slot = link_slot(a.orb, link);
            if (slot < 0) {
                link_ok = false;
                break;
            }
            delay -= L[slot];
        }
        const int base = link_slot(a.orb, __ldg(a.base_link + unit));
        if (!link_ok || base < 0) {
            raise_status(a.orb.status, kStatusLink);
            acc = quiet_nan();
            continue;
        }
        int d;
        double eps;
        split_delay(delay, t_first, a.fs, d, eps);
        if ((long)d - (h - 1) < 0 || (long)d + h >= a.num_inputs) {
            raise_status(a.orb.status, kStatusTap);
            acc = quiet_nan();
            continue;
        }
        double pre;
        if (!prefactor(a.lt, eps, pre)) {
            raise_status(a.orb.status, kStatusAIndex);
            acc = quiet_nan();
            continue;
        }
        const GlobalF64 row{a.y + (size_t)base * a.num_inputs};
        double val = lagrange_real(row, d, eps, pre, a.lt);
        val *= __ldg(a.signs + unit);
        acc += val;
    }
    *out = acc;
}

__global__ void __launch_bounds__(kThreads)
response_indices_kernel(ResponseArgs a, int *d_rec, int *d_em) {
    const int slot = blockIdx.y;
    const long i = (long)a.start + (long)blockIdx.x * kThreads + threadIdx.x;
    if (i >= a.num_delays - a.start) return;
    const double k[3] = {__ldg(a.k), __ldg(a.k + 1), __ldg(a.k + 2)};
    const double zero[3] = {0.0, 0.0, 0.0};
    LinkGeometry g = link_geometry(a.orb, slot, __ldg(a.t_data + i), __ldg(a.t_data), a.fs, k,
                                   zero, zero);
    d_rec[(size_t)slot * a.num_delays + i] = g.d_rec;
    d_em[(size_t)slot * a.num_delays + i] = g.d_em;
}

__global__ void __launch_bounds__(kThreads)
tdi_indices_kernel(TdiArgs a, int *d_out) {
    const int unit = blockIdx.y;
    const long i = (long)a.start + (long)blockIdx.x * kThreads + threadIdx.x;
    if (i >= a.num_delays - a.start) return;
    const double t = __ldg(a.t_arr + i);
    double delay = t;
    const int s0 = __ldg(a.unit_starts + unit), n_s = __ldg(a.unit_lengths + unit);
    for (int s = 0; s < n_s; ++s) {
        const int link = __ldg(a.combos + s0 + s);
        if (link == kNoLink) continue;
        delay -= light_travel_time(a.orb, t, link_slot(a.orb, link));
    }
    int d;
    double eps;
    split_delay(delay, __ldg(a.t_arr), a.fs, d, eps);
    d_out[(size_t)unit * a.num_delays + i] = d;
}

__global__ void orbit_slopes_kernel(const double *tab, double *slope, long n, int stride,
                                    double dt) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    slope[idx] = (tab[idx + stride] - tab[idx]) / dt;
}

dim3 sample_grid(long count, int rows) {
    return dim3((unsigned)((count + kThreads - 1) / kThreads), (unsigned)rows);
}

// 1-D grid: the `rows` rows of a tile in consecutive blocks
unsigned interleaved_grid(long count, int rows) {
    return (unsigned)(((count + kThreads - 1) / kThreads) * rows);
}

// XYZ -> lisaanalysistools' AET, (Z - X)/sqrt2, (X - 2Y + Z)/sqrt6,
// (X + Y + Z)/sqrt3, in NumPy's operation order with correctly rounded
// division (the values of the reference's AET on the same XYZ); `rows` = 2
// writes A and E only.
__device__ __forceinline__ void store_aet(double *aet, long n, long i, int rows, double X,
                                          double Y, double Z) {
    aet[i] = (Z - X) / 1.4142135623730951;
    aet[n + i] = (X - 2.0 * Y + Z) / 2.449489742783178;
    if (rows > 2) aet[2 * n + i] = (X + Y + Z) / 1.7320508075688772;
}

__global__ void __launch_bounds__(kThreads)
xyz_to_aet_kernel(const double *xyz, double *aet, long n, long start, int rows) {
    const long i = start + (long)blockIdx.x * kThreads + threadIdx.x;
    if (i >= n - start) return;
    store_aet(aet, n, i, rows, xyz[i], xyz[n + i], xyz[2 * n + i]);
}

// One thread per sample and all (at most three) channels: the six L(t) once
// per sample, each unit's interpolation added to its channel in unit order
// (the per-channel sums of the reference, bit for bit), the tap windows of a
// sample read by one thread; optional A, E, T epilogue.
__global__ void __launch_bounds__(kThreads)
tdi_plain_kernel(TdiArgs a) {
    const long i = (long)a.start + (long)blockIdx.x * kThreads + threadIdx.x;
    if (i >= a.num_delays - a.start) return;

    const double t = __ldg(a.t_arr + i);
    const double t_first = __ldg(a.t_arr);
    // L(t) of every link slot; the reference re-evaluates the same
    // interpolation for each list entry (LISAResponse.cu:331), which yields
    // these values.
    double L[kLinks];
#pragma unroll
    for (int s = 0; s < kLinks; ++s) L[s] = light_travel_time(a.orb, t, s);

    const int nc = a.num_channels;
    const size_t nd = (size_t)a.num_delays;
    double acc0 = a.out[i];
    double acc1 = (nc > 1) ? a.out[nd + i] : 0.0;
    double acc2 = (nc > 2) ? a.out[2 * nd + i] : 0.0;
    const int h = a.lt.h;
    for (int unit = 0; unit < a.num_units; ++unit) {
        const int ch = __ldg(a.channels + unit);
        if (ch < 0 || ch >= nc) {
            raise_status(a.orb.status, kStatusChannel);
            continue;
        }
        double delay = t;
        bool link_ok = true;
        const int s0 = __ldg(a.unit_starts + unit), n_s = __ldg(a.unit_lengths + unit);
        for (int s = 0; s < n_s; ++s) {
            const int link = __ldg(a.combos + s0 + s);
            if (link == kNoLink) continue;
            const int slot = link_slot(a.orb, link);
            if (slot < 0) {
                link_ok = false;
                break;
            }
            delay -= L[slot];
        }
        const int base = link_slot(a.orb, __ldg(a.base_link + unit));
        double val;
        if (!link_ok || base < 0) {
            raise_status(a.orb.status, kStatusLink);
            val = quiet_nan();
        } else {
            int d;
            double eps, pre;
            split_delay(delay, t_first, a.fs, d, eps);
            if ((long)d - (h - 1) < 0 || (long)d + h >= a.num_inputs) {
                raise_status(a.orb.status, kStatusTap);
                val = quiet_nan();
            } else if (!prefactor(a.lt, eps, pre)) {
                raise_status(a.orb.status, kStatusAIndex);
                val = quiet_nan();
            } else {
                const GlobalF64 row{a.y + (size_t)base * a.num_inputs};
                val = lagrange_real(row, d, eps, pre, a.lt);
                val *= __ldg(a.signs + unit);
            }
        }
        // an invalid unit makes its channel NaN (assigned, as the per-channel
        // form does; NaN stays NaN under later additions)
        const bool bad = val != val;
        if (ch == 0)
            acc0 = bad ? val : acc0 + val;
        else if (ch == 1)
            acc1 = bad ? val : acc1 + val;
        else
            acc2 = bad ? val : acc2 + val;
    }
    a.out[i] = acc0;
    if (nc > 1) a.out[nd + i] = acc1;
    if (nc > 2) a.out[2 * nd + i] = acc2;
    if (a.aet) store_aet(a.aet, a.num_delays, i, a.aet_rows, acc0, acc1, acc2);
}

}  // namespace

cudaError_t launch_response_plain(const ResponseArgs &a, cudaStream_t stream) {
    long count = a.num_delays - 2L * a.start;
    if (count <= 0) return cudaSuccess;
    response_plain_kernel<<<interleaved_grid(count, kLinks), kThreads, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_tdi_plain(const TdiArgs &a, cudaStream_t stream) {
    long count = a.num_delays - 2L * a.start;
    if (count <= 0 || a.num_channels <= 0) return cudaSuccess;
    if (a.num_channels <= 3)
        tdi_plain_kernel<<<interleaved_grid(count, 1), kThreads, 0, stream>>>(a);
    else
        tdi_plain_channel_kernel<<<interleaved_grid(count, a.num_channels), kThreads, 0,
                                   stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_response_indices(const ResponseArgs &a, int *d_rec, int *d_em,
                                    cudaStream_t stream) {
    long count = a.num_delays - 2L * a.start;
    if (count <= 0) return cudaSuccess;
    response_indices_kernel<<<sample_grid(count, kLinks), kThreads, 0, stream>>>(a, d_rec, d_em);
    return cudaGetLastError();
}

cudaError_t launch_tdi_indices(const TdiArgs &a, int *d_out, cudaStream_t stream) {
    long count = a.num_delays - 2L * a.start;
    if (count <= 0 || a.num_units <= 0) return cudaSuccess;
    tdi_indices_kernel<<<sample_grid(count, a.num_units), kThreads, 0, stream>>>(a, d_out);
    return cudaGetLastError();
}

cudaError_t launch_xyz_to_aet(const double *xyz, double *aet, long n, long start, int rows,
                              cudaStream_t stream) {
    const long count = n - 2 * start;
    if (count <= 0) return cudaSuccess;
    xyz_to_aet_kernel<<<(unsigned)((count + kThreads - 1) / kThreads), kThreads, 0, stream>>>(
        xyz, aet, n, start, rows);
    return cudaGetLastError();
}

cudaError_t launch_orbit_slopes(const double *tab, double *slope, long n, int stride, double dt,
                                cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    orbit_slopes_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(tab, slope, n, stride,
                                                                          dt);
    return cudaGetLastError();
}

}  // namespace flr
