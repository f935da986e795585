// Internal interface of the batched, fused response + TDI kernel.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "flr_device.cuh"

namespace flr {

constexpr int kFusedMaxUnits = 64;
constexpr int kFusedMaxCombos = 320;
constexpr int kFusedMaxDepth = 16;  // links per TDI delay list
constexpr int kFusedMaxH = 40;   // h = (order + 1) / 2 supported by the fused kernel
constexpr int kFusedMaxGroups = kFusedMaxDepth + 1;  // distinct delay-list lengths
// Bound on the mbarrier polls of one staging copy (the default of
// FusedArgs::wait_polls and the bound of the second wait, see the kernel).
constexpr long kFusedWaitPolls = 1L << 20;
// Threads per block of the fused kernel and input windows staged per block
// (one: an item's window copy is issued when the item starts; measured
// alternatives are in the plan report's documentation).
constexpr int kFusedThreads = 256;
constexpr int kFusedStagingDepth = 1;
// Bound of a serving block's polls for new work (each ~1 us of sleep), on top
// of the idle time: a block leaves after at most this many.
constexpr long kServerMaxPolls = 1L << 22;
// Status bits of the fused kernel (beside those of flr_device.cuh):
constexpr unsigned kStatusStaging = 0x10u;      // an item's copy missed its first wait:
                                                // that item's outputs are NaN
constexpr unsigned kStatusStagingLost = 0x20u;  // a copy never completed: a block left
                                                // the launch, whose outputs are all invalid

// One source of a batch (device copy of flr_batch_source plus derived values).
struct FusedSource {
    const double2 *h;   // [n] complex128 input
    double *out;        // [3][n] output channels, rows of length n
    long n;
    int ps;             // projections_start_ind: y is zero outside [ps, n - ps)
    int ts;             // tdi_start_ind: outputs are computed for [ts, n - ts)
    double t0;          // time of sample 0
    double k[3], u[3], v[3];
    int tdi_set;        // index into the TDI table sets
    int pad;
    // optional diagnostics (NULL = off), written for the output samples [ts, n - ts):
    double *y_out;      // [6][n] link streams
    int *d_rec_out;     // [6][n] receiver integer delays
    int *d_em_out;      // [6][n] emitter integer delays
    int *d_tdi_out;     // [num_units][n] TDI integer delays, in the caller's unit order
    // optional inner products (NULL = off): data [3][n]; inner [6] =
    // <h_c|d_c> (c = 0..2), then <h_c|h_c>, over [ts, n - ts)
    const double *data;
    double *inner;
};

// TDI unit tables with link numbers already mapped to link slots.
// Small integer fields in the narrowest types that hold their ranges (link
// slots 0-5, channels 0-2, list lengths <= kFusedMaxDepth, unit and entry
// counts <= kFusedMaxUnits / kFusedMaxCombos; the plan checks them): each
// block keeps the set in shared memory, where its size limits the tile.
struct FusedTdiSet {
    int num_units;
    int num_combos;
    double sign[kFusedMaxUnits];
    int16_t unit_start[kFusedMaxUnits];
    int16_t unit_len[kFusedMaxUnits];
    int8_t base_slot[kFusedMaxUnits];
    int8_t channel[kFusedMaxUnits];
    int8_t sign_code[kFusedMaxUnits];    // +1, -1, or 0 (general sign: multiply)
    // Delay lists in compact form: unit u subtracts L of link_slot[u][0..len-1]
    // (the "no delay" markers removed), and shares its first prefix_keep[u]
    // partial sums with unit u-1, whose partial sums are bitwise the ones u
    // would compute itself (same subtractions in the same order).
    int8_t delay_len[kFusedMaxUnits];
    int8_t prefix_keep[kFusedMaxUnits];
    int8_t orig_unit[kFusedMaxUnits];    // position of the unit in the caller's table
    int8_t delay_slot[kFusedMaxUnits][kFusedMaxDepth];
    int8_t combo_slot[kFusedMaxCombos];  // -1: no delay
    // Grouped form, for mixed arithmetic on equal-arm orbits, where every L(t)
    // is the same value and units with delay lists of equal length have
    // bitwise-equal delays.  Group g holds the units [group_start[g],
    // group_start[g + 1]) (lists of length group_len[g], ascending); by
    // linearity their sum on channel c is the interpolation, at that one
    // delay, of group_vsign[g][c] (+-1, 0: none) times the virtual row
    // group_vrow[g][c].  Virtual row r = vrow_ca[r] y[vrow_a[r]] +
    // vrow_cb[r] y[vrow_b[r]] (coefficients +-1 or 0) replaces the link rows
    // in shared memory once per tile.  grouped = 0 when the set does not take
    // this form (a group and channel combining more than two links or with a
    // coefficient other than +-1, or more than six distinct combinations).
    int grouped;
    int num_groups;
    int num_vrows;
    float group_vsign[kFusedMaxGroups][3];
    float vrow_ca[6], vrow_cb[6];
    int8_t group_len[kFusedMaxGroups];
    int8_t group_start[kFusedMaxGroups + 1];
    int8_t group_vrow[kFusedMaxGroups][3];
    int8_t vrow_a[6], vrow_b[6];
};
static_assert(kFusedMaxUnits <= 127 && kFusedMaxDepth <= 127 && kFusedMaxCombos <= 32767,
              "FusedTdiSet field types");
static_assert(sizeof(FusedTdiSet) % sizeof(int) == 0, "the set is copied as ints");

enum FusedChan { kChanXYZ = 0, kChanAET = 1, kChanAE = 2 };

struct GbParams;

struct FusedArgs {
    OrbitTables orb;
    LagrangeTables lt;
    const FusedSource *sources;
    // tile_start[s] = tiles of sources 0..s-1; tile_start[num_sources] = all
    // tiles of the run.  Work item w is tile w - tile_start[s] of the source s
    // with tile_start[s] <= w < tile_start[s + 1].  The total is read on the
    // device, so a captured launch can run batches of any lengths.
    const long *tile_start;
    // tile_base[s] = tile_start[s] - (index of the first tile source s computes),
    // so that work item w is tile w - tile_base[s] of its source
    const long *tile_base;
    // Work items after each block's first (blockIdx.x) are taken from this
    // counter in the staged image (zero when staged): item gridDim.x + the
    // counter's old value.  A block that runs faster takes more items, so no
    // SM idles while others finish.  NULL: static striding by gridDim.x.
    unsigned long long *work_next;
    // Device-resident serving (the server instances): sources, tile_start and
    // the waveform parameters are in page-locked host memory mapped into the
    // device and grow while the kernel runs; tile_start entries not yet
    // published hold INT64_MAX.  Blocks claim items below srv_published (a
    // CAS on work_next, which persists across launches), and leave after
    // srv_idle_ns without claimable work or once srv_stop is set with none
    // left.  The block that finishes a source's last tile sets srv_done.
    const unsigned long long *srv_published;  // work items published (mapped)
    const int *srv_stop;                      // mapped
    unsigned int *srv_tiles_done;             // per source, device memory
    unsigned int *srv_done;                   // per source, mapped
    long long srv_idle_ns;
    int num_sources;
    // per work item: the six partial inner products of its tile (inner-product
    // runs only; reduced per source by launch_inner_reduce)
    double *partial;
    const FusedTdiSet *sets;
    int num_sets;
    const float4 *a_tab;       // per A-table knot: (A hi, A lo, dA hi, dA lo), dA = A[k+1]-A[k]
    int h_df;                  // mixed TDI taps: j < h_df in double-float, the outer ones in FP32
    // Difference forms of the mixed interpolations available (d2 = 1; the
    // launch chooses them for XYZ outputs): per A-table segment, sigma(u) =
    // lerp(A)/A_exact - 1 = ((((c4 u + c3) u + c2) u + c1) u + c0 with
    // (c4, c3, c2, c1) = sig4[segment] and c0 = sig0[segment]
    int d2;
    const float4 *sig4;
    const float *sig0;
    int tile;                  // output samples per work item
    int y_halo;                // link-stream samples computed before a tile
    int y_halo_hi;             // and after it: TDI delays only look back, so the taps
                               // of a tile's last sample reach h samples past it
    long wait_polls;           // bound of an item's first wait for its staging copy
    // per-source waveform parameters of a run with waveforms (NULL otherwise):
    // a source whose h is NULL has its waveform generated into the staged
    // window instead of read from memory
    const GbParams *gb;
    int win_max;               // capacity of the staged input window [samples]
    int y_max;                 // capacity of one staged link row [samples]
    double fs;                 // sampling frequency
    double dt;                 // 1 / fs as the host computes it (t_i = t0 + i * dt)
    double inv_deps;           // 1 / deps
    double inv_orbit_dt;       // 1 / orbit dt
    int chan;                  // FusedChan
    // Receiving spacecraft: rx_sc[r] receives the links in slots rx_slot[r][0..1]
    // (rx_shared = 1 when the orbit's six links split that way).
    int rx_shared;
    int rx_sc[3];
    int rx_slot[3][2];
    // tx_slot[r]: a link spacecraft r + 1 emits on; trio = 1 when all three
    // emit and the six arms are equal at every orbit knot, so that all links
    // leaving a spacecraft share t_em (bit for bit)
    int trio;
    int tx_slot[3];
};

// Galactic-binary parameters of one source (on-device waveform generation).
struct GbParams {
    double A, f, fdot, iota, phi0, psi;
    int model;     // 0: the configurations' binary, 1: the reference tests' GBWave
    int reserved;
};

long gb_waveform_chunks(long n);
// chunk_start[s] = waveform chunks of sources 0..s-1 (num_sources + 1 entries;
// the last is the total, read on the device).
cudaError_t launch_gb_waveforms(const FusedSource *src, const GbParams *par,
                                const long *chunk_start, int num_sources, double dt, int grid,
                                cudaStream_t stream);

size_t fused_smem_bytes(bool mixed, int win_max, int y_max);
// grouped: the mixed instance for sets in grouped form (every set of the plan).
cudaError_t fused_configure(bool mixed, bool grouped, size_t smem_bytes, int *blocks_per_sm);
// Sum each source's per-tile partial inner products, tiles in order, into
// its inner[6] (sources without inner are skipped).
cudaError_t launch_inner_reduce(const FusedArgs &a, cudaStream_t stream);
// diag: the instance that writes the FusedSource diagnostics (more registers);
// inner: the instance that forms inner products (FusedArgs::partial set);
// d2: the mixed instance in difference form (FusedArgs::d2 tables required);
// t0_zero: every source of the launch has t0 = +0 (bit pattern 0), which
// selects the difference-form instance without the t0 operations (no
// diagnostics, no inner products; the other launches ignore it).
cudaError_t launch_fused(bool mixed, bool grouped, bool diag, bool inner, bool d2, bool t0_zero,
                         const FusedArgs &a, int grid, size_t smem_bytes, cudaStream_t stream);
// The difference-form mixed instances (flr_fused_d2.cu).
const void *fused_fn_d2(bool grouped, bool diag, bool inner);
// The difference-form mixed instances for sources that all start at t0 = +0
// (flr_fused_t0.cu).
const void *fused_fn_t0(bool grouped);
// Serving instances (mixed; d2: difference forms for XYZ outputs): a launch
// that claims published items until it is idle or stopped.  Sets the
// instance's shared-memory limit before launching.
const void *fused_fn_server(bool grouped, bool d2);
cudaError_t launch_fused_server(bool grouped, bool d2, const FusedArgs &a, int grid,
                                size_t smem_bytes, cudaStream_t stream);

}  // namespace flr
