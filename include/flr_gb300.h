/*
 * flr_gb300.h — C ABI of the GB300 (sm_103a) LISA time-domain response + TDI.
 *
 * This is the drop-in boundary for the reference's native layer
 * (mikekatz04/lisa-on-gpu, package fastlisaresponse).  The reference binds its
 * CUDA code to Python through pybind11 classes; each entry point below takes
 * the same arguments, in the same order and with the same meaning, as the
 * method it replaces, so a backend module can forward calls one to one:
 *
 *   OrbitsWrap{CPU,GPU}_responselisa(dt, N, n_arr, ltt_arr, x_arr, links,
 *       sc_r, sc_e, armlength)      src/fastlisaresponse/cutils/binding_flr.hpp:35-59
 *                                   -> flr_orbits_create / flr_orbits_destroy
 *   LISAResponseWrap.get_response_wrap(...)    binding_flr.cxx:38-58,
 *                                              LISAResponse.cu:674-718
 *                                   -> flr_get_response
 *   LISAResponseWrap.get_tdi_delays_wrap(...)  binding_flr.cxx:16-35,
 *                                              LISAResponse.cu:399-429
 *                                   -> flr_get_tdi_delays
 *
 * Conventions (all entry points):
 *   - Array arguments are device pointers (cudaMalloc'd, managed, or any
 *     pointer the GPU can dereference), borrowed for the duration of the call;
 *     flr_orbits_create also accepts host pointers (it copies the tables).
 *   - Work is enqueued on `stream` (a cudaStream_t; NULL = legacy default
 *     stream) and is NOT synchronised: results are ready when the stream is.
 *     The reference synchronises the whole device after each launch
 *     (LISAResponse.cu:420,704); call cudaStreamSynchronize for that.
 *   - Every function returns FLR_OK (0) or a negative FLR_E* code; the text of
 *     the last error on the calling thread is in flr_last_error().  Argument
 *     errors are reported before anything is enqueued (the reference's CPU
 *     binding throws std::invalid_argument -> ValueError for the same cases,
 *     binding_flr.hpp:66-69).
 *   - Out-of-range tap reads (a delay window that leaves the input, or an A
 *     table index outside [0, num_A-2]) are not performed: the kernel records
 *     FLR_STATUS_* bits in the orbit handle's status word and writes NaN for
 *     that output sample.  Read the word with flr_orbits_status().
 *   - Arithmetic: the kernels evaluate the reference's expressions as separately
 *     rounded IEEE-754 double operations in the reference's order (no fused
 *     multiply-add, correctly rounded division and square root), so integer
 *     delay indices and outputs equal those of the reference's CPU path built
 *     without floating-point contraction, bit for bit.
 */
#ifndef FLR_GB300_H
#define FLR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FLR_OK 0
#define FLR_E_INVALID_ARGUMENT (-1)
#define FLR_E_CUDA (-2)
#define FLR_E_NO_ORBITS (-3)
#define FLR_E_UNSUPPORTED (-4)

/* Bits of the per-orbit-handle status word (set by kernels, sticky). */
#define FLR_STATUS_TAP_OUT_OF_RANGE 0x1u   /* interpolation window left the input   */
#define FLR_STATUS_A_INDEX_OUT_OF_RANGE 0x2u /* eps/deps outside the A table        */
#define FLR_STATUS_BAD_LINK 0x4u           /* link number not in the orbit's links  */
#define FLR_STATUS_BAD_CHANNEL 0x8u        /* TDI channel outside [0,num_channels)  */
/* Batched kernel only: a work item's staging copy did not complete within its
 * first wait; it completed within a second one and that item's outputs are
 * NaN (the batch's other outputs are valid). */
#define FLR_STATUS_STAGING 0x10u
/* Batched kernel only: a staging copy did not complete within the second wait
 * either; the block that issued it left the launch with the copy in flight,
 * so every output of the launches since the status was last cleared is to be
 * discarded (flr_orbits_status also says so in flr_last_error()). */
#define FLR_STATUS_STAGING_LOST 0x20u

/* Largest Lagrange order accepted (h = (order+1)/2 <= 40, the reference's
 * MAX_ORDER E-table size, LISAResponse.cu:216). */
#define FLR_MAX_ORDER 79

typedef struct flr_orbits flr_orbits;

/* Version string of this library ("flr_gb300 <semver> sm_103a"). */
const char *flr_version(void);

/* Text of the last error raised on the calling thread ("" if none). */
const char *flr_last_error(void);

/* Page-locked host memory of exactly `bytes` bytes (cudaHostAlloc, portable
 * to every device), for the host buffers of asynchronous copies (no
 * reference counterpart; the Python HostArray uses it).  flr_host_free
 * releases it. */
int flr_host_alloc(size_t bytes, void **out);
int flr_host_free(void *ptr);

/*
 * Upload orbit tables and return a handle (replaces OrbitsWrap*_responselisa,
 * binding_flr.hpp:35-59).  Layout as lisaanalysistools' pycppdetector_args:
 *   n_arr  [N][6][3]  link unit vectors (kept for completeness, unused by the
 *                     response, as in the reference)
 *   ltt_arr[N][6]     light travel time of each link [s]
 *   x_arr  [N][3][3]  spacecraft positions [m]
 *   links  [6]        link numbers (12, 23, 31, 13, 32, 21 by default)
 *   sc_r   [6], sc_e [6]  receiver / emitter spacecraft of each link (1..3)
 * on the uniform grid t_k = k*dt, k = 0..N-1 (N >= 2).  Values are linearly
 * interpolated; times whose segment (int)(t/dt) lies outside [0, N-1] give a
 * light travel time of 0 and a zero position, the last segment serves t up to
 * and beyond (N-1)*dt.  Unlike the reference (which borrows the caller's
 * arrays), the tables are copied into device memory owned by the handle; host
 * or device pointers are accepted.  The handle also owns the status word.
 */
int flr_orbits_create(double dt, int N, const double *n_arr, const double *ltt_arr,
                      const double *x_arr, const int *links, const int *sc_r, const int *sc_e,
                      double armlength, flr_orbits **out);
int flr_orbits_destroy(flr_orbits *orbits);

/* Read (and with reset != 0, clear) the status word; synchronises `stream`. */
int flr_orbits_status(flr_orbits *orbits, uint32_t *bits, int reset, void *stream);

/*
 * Link projections y_gw (replaces LISAResponseWrap.get_response_wrap,
 * binding_flr.cxx:38-58 -> LISAResponse::get_response, LISAResponse.cu:674-718).
 *   y_gw      [6*num_delays] out, link-major; samples [projections_start_ind,
 *             num_delays - projections_start_ind) are written, others untouched
 *   t_data    [num_delays] sample times; t_data[0] is the time origin of input_in
 *   k_in, u_in, v_in [3] propagation direction and polarisation basis
 *   dt        sample spacing (unused by the kernel, as in the reference)
 *   input_in  [num_inputs] complex128 h+ + i hx, interleaved (re, im)
 *   order     Lagrange order; h = (order+1)/2 taps on each side
 *   sampling_frequency  1/dt
 *   buffer_integer      staging margin of the reference's GPU kernel; accepted
 *                       and ignored (this kernel has no fixed-size window)
 *   A_in [num_A], deps, E_in [(order+1)/2 - 1]  Lagrange tables (response.py:273-310)
 */
int flr_get_response(flr_orbits *orbits, double *y_gw, const double *t_data, const double *k_in,
                     const double *u_in, const double *v_in, double dt, int num_delays,
                     const void *input_in, int num_inputs, int order, double sampling_frequency,
                     int buffer_integer, const double *A_in, double deps, int num_A,
                     const double *E_in, int projections_start_ind, void *stream);

/*
 * TDI combinations (replaces LISAResponseWrap.get_tdi_delays_wrap,
 * binding_flr.cxx:16-35 -> LISAResponse::get_tdi_delays, LISAResponse.cu:399-429).
 *   delayed_links [num_channels*num_delays] in/out, channel-major (it must
 *             hold num_channels rows: every row is read and written); each sample
 *             in [tdi_start_ind, num_delays - tdi_start_ind) is ACCUMULATED
 *             into, unit by unit in unit order (callers zero it first, as the
 *             reference's caller does, response.py:592)
 *   input_links [6*num_inputs] link streams y_gw, rows in orbit link order
 *   t_arr     [num_delays] sample times
 *   unit_starts/unit_lengths [num_units]  slices of tdi_link_combinations
 *   tdi_base_link [num_units]  link whose stream the unit interpolates
 *   tdi_link_combinations [...]  link numbers whose L(t) the unit subtracts
 *                               (-11 = none)
 *   tdi_signs [num_units] (double), channels [num_units]
 *   The caller guarantees unit_starts[u] + unit_lengths[u] <= the length of
 *   tdi_link_combinations (the kernel cannot check it: the array's length is
 *   not an argument, as in the reference).
 * Unlike the reference GPU kernel (atomicAdd, LISAResponse.cu:389) the sum over
 * units is in a fixed order, so results are deterministic.  With up to three
 * channels one thread takes all channels of a sample (the six L(t) once, the
 * sample's tap windows read by one thread); with more, one thread per
 * (sample, channel).
 */
int flr_get_tdi_delays(flr_orbits *orbits, double *delayed_links, const double *input_links,
                       int num_inputs, int num_delays, const double *t_arr,
                       const int *unit_starts, const int *unit_lengths, const int *tdi_base_link,
                       const int *tdi_link_combinations, const double *tdi_signs,
                       const int *channels, int num_units, int num_channels, int order,
                       double sampling_frequency, int buffer_integer, const double *A_in,
                       double deps, int num_A, const double *E_in, int tdi_start_ind,
                       void *stream);

/*
 * flr_get_tdi_delays followed, in the same kernel, by the A, E (and T) of
 * flr_xyz_to_aet (below) of the accumulated X, Y, Z: needs num_channels 3;
 * aet [aet_rows][num_delays], aet_rows 3 (A, E, T) or 2 (A, E); the samples
 * [tdi_start_ind, num_delays - tdi_start_ind) are written, delayed_links as
 * flr_get_tdi_delays writes it.  The reference forms AET on the host after
 * the TDI call (response.py:659-673).
 */
int flr_get_tdi_delays_aet(flr_orbits *orbits, double *delayed_links, const double *input_links,
                           int num_inputs, int num_delays, const double *t_arr,
                           const int *unit_starts, const int *unit_lengths,
                           const int *tdi_base_link, const int *tdi_link_combinations,
                           const double *tdi_signs, const int *channels, int num_units,
                           int num_channels, int order, double sampling_frequency,
                           int buffer_integer, const double *A_in, double deps, int num_A,
                           const double *E_in, int tdi_start_ind, double *aet, int aet_rows,
                           void *stream);

/*
 * Diagnostics: the integer delay indices the two kernels above compute, from
 * the same device code.  d_rec/d_em [6*num_delays] receive, per (link, sample),
 * ceil((delay - t_data[0]) * fs) - 1 for the receiver and emitter times
 * (LISAResponse.cu:616-622); d_tdi [num_units*num_delays] the same per (unit,
 * sample) for the TDI delays (LISAResponse.cu:339-341).  Samples outside the
 * computed range are untouched.  No counterpart in the reference (its indices
 * are internal); used to show the indices are bit-exact.
 */
int flr_response_delay_indices(flr_orbits *orbits, int *d_rec, int *d_em, const double *t_data,
                               const double *k_in, int num_delays, double sampling_frequency,
                               int projections_start_ind, void *stream);
int flr_tdi_delay_indices(flr_orbits *orbits, int *d_tdi, int num_delays, const double *t_arr,
                          const int *unit_starts, const int *unit_lengths,
                          const int *tdi_link_combinations, int num_units,
                          double sampling_frequency, int tdi_start_ind, void *stream);

/*
 * A, E (and T) from X, Y, Z as lisaanalysistools' AET defines them:
 * (Z - X)/sqrt2, (X - 2Y + Z)/sqrt6, (X + Y + Z)/sqrt3, in NumPy's operation
 * order with correctly rounded division, for the samples [start,
 * num_delays - start) of channel-major rows (xyz [3][num_delays] in, aet
 * [num_rows][num_delays] out, num_rows 3 for AET or 2 for AE; other samples
 * untouched).  Replaces the reference's call of lisatools' AET on the TDI
 * output (response.py:659-673), which is host Python in the reference.
 */
int flr_xyz_to_aet(const double *xyz, double *aet, int num_delays, int start, int num_rows,
                   void *stream);

/*
 * ------------------------------------------------------------------------
 * Batched, fused response + TDI (no reference counterpart: the reference
 * evaluates one source per call, with two launches and a device
 * synchronisation each, LISAResponse.cu:399-429, 674-718).  One persistent
 * kernel evaluates many sources of different lengths; the link streams stay
 * in shared memory, so per output sample only the complex input is read and
 * the three channels are written.
 *
 * Arithmetic (per plan):
 *   FLR_PRECISION_FP64   every operation as in the plain path: outputs are
 *                        bit-identical to flr_get_response + flr_get_tdi_delays
 *                        (+ the XYZ->AET transform) on the same inputs;
 *   FLR_PRECISION_MIXED  delays, their integer/fractional split, orbit
 *                        interpolation and TDI delay sums in FP64 (integer
 *                        indices bit-exact), Lagrange taps, weights and
 *                        projections in double-float (pairs of FP32) arithmetic.
 * ------------------------------------------------------------------------
 */
#define FLR_PRECISION_FP64 0
#define FLR_PRECISION_MIXED 1
#define FLR_CHAN_XYZ 0
#define FLR_CHAN_AET 1 /* lisaanalysistools AET: (Z-X)/sqrt2, (X-2Y+Z)/sqrt6, (X+Y+Z)/sqrt3 */
#define FLR_CHAN_AE 2

/* One TDI combination, in the reference's table layout (response.py:372-433,
 * 619-633); HOST arrays, read at plan creation. */
typedef struct {
    int num_units;
    const int *unit_starts;           /* [num_units] */
    const int *unit_lengths;          /* [num_units] */
    const int *tdi_base_link;         /* [num_units] link numbers */
    const int *tdi_link_combinations; /* [num_combos] link numbers, -11 = no delay */
    const double *tdi_signs;          /* [num_units] */
    const int *channels;              /* [num_units] 0, 1, 2 */
    int num_combos;
} flr_tdi_units;

/* One source of a batch. */
typedef struct {
    const void *h;          /* [n] complex128 h+ + i hx, device, 16-byte aligned */
    double *out;            /* [3][n] float64, device: rows X,Y,Z (or A,E,T / A,E and
                               a zero row); every sample is written, zeros outside
                               [tdi_start, n - tdi_start) as in the reference */
    long long n;
    int projections_start;  /* link streams are zero outside [ps, n - ps) */
    int tdi_start;          /* first output sample (garbage margin) */
    double t0;              /* time of sample 0; sample i is at t0 + i * (1/fs) */
    double k[3], u[3], v[3];/* propagation direction and polarisation basis */
    int tdi_set;            /* index of the plan's TDI unit set */
    int reserved;
    /* Optional diagnostics (NULL = off), written for samples [tdi_start, n - tdi_start):
     *   y_out [6][n] the link streams (y_gw) the TDI stage used;
     *   d_rec_out, d_em_out [6][n] receiver / emitter integer delays (both or neither);
     *   d_tdi_out [num_units][n] integer TDI delays, units in the set's given order. */
    double *y_out;
    int *d_rec_out;
    int *d_em_out;
    int *d_tdi_out;
    /* Optional inner products (both NULL = off): data [3][n] float64 device
     * channels in the layout of out; inner [6] float64 device receives
     * <h_c|d_c> for c = 0, 1, 2 then <h_c|h_c>, summed over the computed samples
     * [tdi_start, n - tdi_start) in a fixed order (deterministic).  With inner
     * set, out may be NULL: the channels are then never written to memory.
     * Not available through batch graphs.  (The reference's consumer,
     * utils/utility.py:16-82, forms such products from the stored channels.) */
    const double *data;
    double *inner;
    /* Optional output range (out_end <= out_begin = all of [tdi_start, n -
     * tdi_start)): only the tiles overlapping [out_begin, out_end) are
     * computed, with the same bits as a whole-source run (sample i is still at
     * t0 + i / fs); the first and last tiles also write the zero edge zones.
     * The taps may read h anywhere within the delays' reach of the range. */
    long long out_begin, out_end;
} flr_batch_source;

typedef struct flr_batch_plan flr_batch_plan;

/* Plan for batches on `orbits`: Lagrange tables (device or host; copied),
 * 1..64 TDI unit sets, precision, tile = output samples per work item
 * (0 = 512).  A run on another stream than the previous run of the plan waits
 * (on the device) for that run, whose staging buffer it reuses. */
int flr_batch_plan_create(flr_orbits *orbits, int order, const double *A_in, double deps,
                          int num_A, const double *E_in, double sampling_frequency,
                          const flr_tdi_units *sets, int num_sets, int precision, int tile,
                          flr_batch_plan **out);
int flr_batch_plan_destroy(flr_batch_plan *plan);
/* info[0..11] = tile, y halo, input window capacity, link row capacity, shared
 * memory bytes per block, persistent grid size, precision, 1 when the mixed
 * kernel evaluates the TDI units in equal-delay groups (equal-arm orbits:
 * units with delay lists of equal length share one interpolation of their
 * combined link rows), the first outer tap j of the TDI interpolations that
 * the mixed kernel's double-float form evaluates in FP32 (its weights are
 * small enough; the half-width h when none), and 1 when the mixed kernel
 * evaluates the TDI interpolations in second-difference form (a double-float
 * linear part plus an FP32 sum over second differences; needs the reference's
 * Lagrange tables, else the double-float form is used), the threads per block
 * of the fused kernel (256) and its staging depth (input windows in flight
 * per block: 1).  Fewer entries are written when n_info is smaller. */
int flr_batch_plan_info(const flr_batch_plan *plan, int *info, int n_info);

/* Test hook (no reference counterpart): the bound, in mbarrier polls, of each
 * work item's first wait for its staging copy in the plan's later runs and
 * graphs (polls < 0 restores the default, 2^20).  With 0 every first wait
 * gives up at once, so the give-up path runs without a stalled copy: a second
 * wait with the full bound lets the copy land, the item's outputs become NaN
 * and FLR_STATUS_STAGING is raised. */
int flr_batch_plan_set_wait_limit(flr_batch_plan *plan, long long polls);

/* Evaluate `num_sources` sources (host array of descriptors) on `stream`. */
int flr_batch_run(flr_batch_plan *plan, const flr_batch_source *sources, int num_sources,
                  int chan, void *stream);

/* Galactic-binary parameters of a source whose waveform the library
 * generates (FP64, CUDA's sincos; t = t0 + i / fs), in one of two models:
 *   FLR_GB_MODEL_CONFIG (0): Phi = phi0 + 2 pi (f t + fdot t^2 / 2),
 *     h+ = A (1 + cos^2 iota) cos Phi, hx = -2 A cos iota sin Phi;
 *   FLR_GB_MODEL_GBWAVE (1): the reference test-suite's generator
 *     (tests/test_fastlisaresponse.py:34-63): fddot = 11/3 fdot^2 / f,
 *     Phi = 2 pi (f t + fdot t^2 / 2 + fddot t^3 / 6) - phi0,
 *     h+ = -A (1 + cos^2 iota) cos Phi, hx = -2 A cos iota sin Phi;
 * both rotated by the polarisation angle psi (h+ cos2psi - hx sin2psi,
 * h+ sin2psi + hx cos2psi).  Zero-initialised fields select model 0. */
#define FLR_GB_MODEL_CONFIG 0
#define FLR_GB_MODEL_GBWAVE 1
typedef struct {
    double A, f, fdot, iota, phi0, psi;
    int model;
    int reserved;
} flr_gb_params;

/* As flr_batch_run, with each source's waveform generated on the device at
 * t_i = t0 + i / fs: into sources[i].h when it is set (a device buffer of n
 * complex128 the caller provides; one waveform launch writes it, the fused
 * launch reads it), or, when sources[i].h is NULL, straight into the fused
 * kernel's staged input window, so that the waveform never reaches memory
 * (per output sample 24 B of HBM traffic: the channels). */
int flr_batch_run_gb(flr_batch_plan *plan, const flr_batch_source *sources,
                     const flr_gb_params *params, int num_sources, int chan, void *stream);

/*
 * Batch graphs: the staging copy and the kernel launches of a run, captured
 * once as a CUDA graph for up to `max_sources` sources and replayed by
 * flr_batch_graph_launch.  The kernels take the number of tiles (and waveform
 * chunks) of every source from the staged per-source prefix sums, so one graph
 * runs batches of any lengths and of up to max_sources sources; everything
 * per source (buffers, n, sky position, t0, TDI set, waveform parameters) is
 * staged per launch.  Results are bit-identical to flr_batch_run /
 * flr_batch_run_gb on the same sources.  Two pinned staging buffers alternate,
 * so a launch can be prepared while the previous one runs; a launch on
 * another stream than the previous one waits for it on the device.  Destroy
 * the graphs of a plan before the plan.  No counterpart in the reference.
 * flags: FLR_GRAPH_WAVEFORMS (generate waveforms as flr_batch_run_gb; params
 * required at launch) | FLR_GRAPH_DIAGNOSTICS (allow the diagnostics fields).
 */
#define FLR_GRAPH_WAVEFORMS 0x1
#define FLR_GRAPH_DIAGNOSTICS 0x2
typedef struct flr_batch_graph flr_batch_graph;
int flr_batch_graph_create(flr_batch_plan *plan, int max_sources, int flags, int chan,
                           flr_batch_graph **out);
int flr_batch_graph_launch(flr_batch_graph *graph, const flr_batch_source *sources,
                           const flr_gb_params *params, int num_sources, void *stream);
int flr_batch_graph_destroy(flr_batch_graph *graph);

/*
 * Link projections without any device allocation.  No counterpart in the
 * reference: for callers that cannot call cudaMalloc -- code running inside a
 * framework that has pre-allocated the GPU's memory, and samplers that must
 * not trigger the device-wide synchronisation of cudaMalloc/cudaFree in their
 * inner loop.  Same arguments and
 * results (bit for bit) as flr_get_response, except that the orbit tables are
 * passed directly instead of through an flr_orbits handle:
 *   orbit_dt, orbit_N       grid spacing and knot count, orbit_N <= FLR_NOALLOC_MAX_KNOTS
 *   ltt_arr [orbit_N][6], x_arr [orbit_N][3][3]   device pointers
 *   links, sc_r, sc_e [6]   HOST arrays (read during the call)
 * The derived segment slopes and the status word live in a fixed array inside
 * the library (3.9 MB of device memory on every GPU that loads it, held until
 * exit), rewritten and cleared by every call; out-of-range tap windows set
 * FLR_STATUS_* bits there (flr_noalloc_status reads them) and give NaN, as in
 * flr_get_response.  The first call on a device,
 * with that device current, looks up the array's device address; make it
 * before any stream capture.  Calls whose work can overlap on the GPU race on
 * the array.  Sizes beyond the limit return FLR_E_INVALID_ARGUMENT with the
 * reason in flr_last_error().
 */
#define FLR_NOALLOC_MAX_KNOTS 32768
int flr_get_response_noalloc(double orbit_dt, int orbit_N, const double *ltt_arr,
                             const double *x_arr, const int *links, const int *sc_r,
                             const int *sc_e, double *y_gw, const double *t_data,
                             const double *k_in, const double *u_in, const double *v_in,
                             double dt, int num_delays, const void *input_in, int num_inputs,
                             int order, double sampling_frequency, int buffer_integer,
                             const double *A_in, double deps, int num_A, const double *E_in,
                             int projections_start_ind, void *stream);

/*
 * Status word of the allocation-free entry point (FLR_STATUS_* bits, as
 * flr_orbits_status reports them for a handle), read from the same fixed
 * array without allocating; reset != 0 also clears it.  Every call of
 * flr_get_response_noalloc clears the word first, so it describes the latest
 * call on this device only.  Synchronises `stream`.  No counterpart in the
 * reference.
 */
int flr_noalloc_status(uint32_t *bits, int reset, void *stream);


/*
 * ------------------------------------------------------------------------
 * Device-resident serving (no reference counterpart).  A server holds a list
 * of up to `capacity` sources in page-locked host memory mapped into the
 * device; flr_server_submit appends one source (its descriptor, waveform
 * parameters and tile count) and publishes its tiles, and a persistent launch
 * of the plan's mixed fused kernel (flr_server_pump) claims published tiles
 * as they arrive, so requests submitted while it runs need no new launch.
 * The block that writes a source's last tile sets its done flag (host
 * memory, flr_server_done_flags; read with acquire loads).  The launch
 * leaves after `idle_seconds` without claimable work or once flr_server_stop
 * is called (after the work already published); flr_server_pump relaunches
 * it when sources are not done and none is running.  Every wait of the
 * kernel is bounded (the idle time and a poll count).  Sources are whole
 * (no out_begin/out_end, diagnostics or inner products); h NULL with
 * waveform parameters generates the waveform inside the kernel.  Results are
 * those of flr_batch_run_gb / flr_batch_run on the same sources.  Not
 * thread-safe: one host thread submits and pumps.
 */
typedef struct flr_server flr_server;
int flr_server_create(flr_batch_plan *plan, int capacity, int chan, double idle_seconds,
                      flr_server **out);
int flr_server_submit(flr_server *server, const flr_batch_source *source,
                      const flr_gb_params *params, int *slot);
int flr_server_pump(flr_server *server, void *stream);
/* info[0..4] = sources submitted, tiles published, lowest source not known
 * to be done, launches so far, 1 while a launch may be running. */
int flr_server_info(flr_server *server, long long *info, int n_info);
const unsigned *flr_server_done_flags(const flr_server *server);
int flr_server_stop(flr_server *server);
int flr_server_destroy(flr_server *server);

#ifdef __cplusplus
}
#endif

#endif /* FLR_GB300_H */
