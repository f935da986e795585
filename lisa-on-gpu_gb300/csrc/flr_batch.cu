// C ABI of the batched path: plans and runs of the fused response + TDI
// kernel over many sources (declarations in include/flr_gb300.h).
//
// A plan fixes what is common to a batch -- orbit tables, Lagrange order and
// tables, TDI unit sets, arithmetic, tile length -- derives the launch shape
// (halo and window sizes, shared memory, persistent grid from the occupancy of
// the kernel), and owns reusable device and pinned buffers for the per-run
// source descriptors.  A run copies the descriptors and the per-source tile
// (and waveform chunk) prefix sums with one asynchronous copy and launches one
// persistent kernel on the stream; the kernel resolves its (source, tile)
// items from the prefix sums.
//
// A batch graph is a CUDA graph of that copy and those launches for a fixed
// capacity of sources.  Its kernels read the number of sources' tiles from the
// copied prefix sums, so one graph runs batches of any lengths and up to its
// capacity of sources (the rest are empty descriptors); the per-source data
// (buffers, lengths, sky position, start time, TDI set, waveform parameters)
// are staging contents, not graph parameters.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/flr_gb300.h"
#include "flr_fused.h"
#include "flr_internal.h"

struct flr_batch_plan {
    int device;
    bool mixed;
    bool grouped;              // mixed, equal-arm orbits, every set in grouped form
    flr::FusedArgs base;
    size_t smem;
    int grid_max;
    int num_sets;
    int set_max_len;           // longest TDI delay list (links subtracted)
    void *d_tables;            // A, E and the TDI sets (device)
    unsigned char *d_stage;    // per-run descriptors, work items, waveform parameters
    size_t cap_device;
    int sms;
    unsigned char *h_stage;    // pinned staging for descriptors and prefix sums
    size_t cap_stage;
    cudaEvent_t stage_free;    // recorded after the staging copies of the last run
    bool stage_pending;
    cudaEvent_t done;          // recorded after the kernels of the last run
    double *d_partial;         // per-tile partial inner products (runs that ask for them)
    size_t cap_partial;
    bool done_pending;
};

// Device-resident serving: a source list in page-locked host memory mapped
// into the device, appended to by the host while a persistent launch of the
// fused kernel's serving instance claims its tiles (flr_fused_kernel.cuh).
struct flr_server {
    flr_batch_plan *plan = nullptr;
    int chan = 0;
    bool d2 = false;
    int cap = 0;
    long long idle_ns = 0;
    unsigned char *h_block = nullptr;        // the mapped block
    flr::FusedSource *h_src = nullptr, *d_src = nullptr;
    flr::GbParams *h_gb = nullptr, *d_gb = nullptr;
    long long *h_tile_start = nullptr, *d_tile_start = nullptr;  // cap + 1
    unsigned long long *h_published = nullptr, *d_published = nullptr;
    int *h_stop = nullptr, *d_stop = nullptr;
    unsigned *h_done = nullptr, *d_done = nullptr;
    unsigned long long *d_next = nullptr;   // claim counter (device)
    unsigned *d_tiles_done = nullptr;       // per source (device)
    int count = 0;                          // sources submitted
    long long items = 0;                    // tiles published
    int first_open = 0;                     // lowest source not known to be done
    long long launches = 0;
    cudaEvent_t ran = nullptr;              // recorded after the last launch
    bool launched = false;
};

struct flr_batch_graph {
    flr_batch_plan *plan;
    int cap;                   // sources per launch at most
    bool waveforms, diag;
    int chan;
    unsigned char *h_stage[2];  // pinned staging, alternated between launches
    unsigned char *d_stage;
    cudaGraphExec_t exec[2];    // exec[b] copies from h_stage[b]
    cudaGraphExec_t exec_t0[2]; // the same with the t0 = 0 instance (or null)
    cudaEvent_t done[2];        // recorded after the launch that used buffer b
    bool pending[2];
    int next;                   // buffer of the next launch
    int last;                   // buffer of the last launch (-1: none yet)
};

namespace {

int fail(int code, const std::string &msg) {
    flr::set_last_error(msg);
    return code;
}

int cuda_fail(cudaError_t err, const std::string &what) {
    cudaGetLastError();  // a handled error must not resurface in a later check
    return fail(FLR_E_CUDA, what + ": " + cudaGetErrorString(err));
}

int current_device_is(int dev) {
    int cur = -1;
    cudaError_t err = cudaGetDevice(&cur);
    if (err != cudaSuccess) return cuda_fail(err, "cudaGetDevice");
    if (cur != dev)
        return fail(FLR_E_INVALID_ARGUMENT, "plan was created on device " + std::to_string(dev) +
                                                " but device " + std::to_string(cur) +
                                                " is current");
    return FLR_OK;
}

int slot_of(const flr_orbits *o, int link) {
    for (int s = 0; s < 6; ++s)
        if (o->links[s] == link) return s;
    return -1;
}

void release(flr_batch_plan *p) {
    if (!p) return;
    if (p->d_tables) cudaFree(p->d_tables);
    if (p->d_stage) cudaFree(p->d_stage);
    if (p->d_partial) cudaFree(p->d_partial);
    if (p->h_stage) cudaFreeHost(p->h_stage);
    if (p->stage_free) cudaEventDestroy(p->stage_free);
    if (p->done) cudaEventDestroy(p->done);
    delete p;
}

// Grouped form of a set whose units are ordered by delay-list length (mixed
// arithmetic, equal-arm orbits): runs of equal length become groups; per group
// and channel the units' signed base links merge into at most two link rows
// with coefficients +-1, and the distinct combinations (up to sign) become the
// virtual rows, at most six.  Leaves grouped = 0 when a set does not fit.
void make_groups(flr::FusedTdiSet &s) {
    s.grouped = 0;
    s.num_vrows = 0;
    int ng = 0;
    for (int u = 0; u < s.num_units;) {
        int v = u;
        while (v < s.num_units && s.delay_len[v] == s.delay_len[u]) ++v;
        if (ng == flr::kFusedMaxGroups) return;
        double coef[3][6] = {};
        for (int w = u; w < v; ++w) coef[s.channel[w]][s.base_slot[w]] += s.sign[w];
        s.group_len[ng] = s.delay_len[u];
        s.group_start[ng] = u;
        for (int c = 0; c < 3; ++c) {
            int slot[2] = {0, 0}, terms = 0;
            float cf[2] = {0.f, 0.f};
            for (int k = 0; k < 6; ++k) {
                if (coef[c][k] == 0.0) continue;
                if (terms == 2 || (coef[c][k] != 1.0 && coef[c][k] != -1.0)) return;
                slot[terms] = k;
                cf[terms] = (float)coef[c][k];
                ++terms;
            }
            s.group_vrow[ng][c] = 0;
            s.group_vsign[ng][c] = 0.f;
            if (terms == 0) continue;
            // canonical combination: first coefficient +1, the sign kept apart
            const float sg = cf[0];
            const int b = (terms == 2) ? slot[1] : slot[0];
            const float ca = 1.f, cb = (terms == 2) ? cf[1] * sg : 0.f;
            int r = 0;
            while (r < s.num_vrows && !(s.vrow_a[r] == slot[0] && s.vrow_b[r] == b &&
                                        s.vrow_ca[r] == ca && s.vrow_cb[r] == cb))
                ++r;
            if (r == s.num_vrows) {
                if (r == 6) return;
                s.vrow_a[r] = slot[0];
                s.vrow_b[r] = b;
                s.vrow_ca[r] = ca;
                s.vrow_cb[r] = cb;
                ++s.num_vrows;
            }
            s.group_vrow[ng][c] = r;
            s.group_vsign[ng][c] = sg;
        }
        ++ng;
        u = v;
    }
    s.group_start[ng] = s.num_units;
    s.num_groups = ng;
    s.grouped = 1;
}

// The second-difference form of the mixed kernel's TDI interpolation needs
// S(eps) = lerp(A)(eps) / A_exact(eps), the ratio of the caller's A table
// (linearly interpolated, as the reference does) to the exact Lagrange
// prefactor A_exact(eps) = prod_{i=1}^{h-1} (i + eps)(i + 1 - eps) / ((h-1)! h!)
// of which the table is a sampling.  Per table segment [a deps, (a+1) deps]
// the deviation sigma = S - 1 (|sigma| <= ~2e-7, zero at the knots) is a
// smooth function of u = eps / deps - a, stored as a degree-4 polynomial in u
// with FP32 coefficients (c4, c3, c2, c1) and c0.  Fitted at five Chebyshev
// nodes in long double and checked at 17 points as the kernel evaluates it:
// false (the form is not used) when it misses sigma by more than 1e-13
// anywhere (the FP32 coefficients alone carry ~1e-14), or when the E table
// does not hold the weights whose sum is 1 / A_exact (a table other than the
// reference's).
bool fit_sigma_table(const std::vector<double> &A, const std::vector<double> &E, int h,
                     double deps, std::vector<float4> &c4, std::vector<float> &c0) {
    const int segs = (int)A.size() - 1;
    if (segs < 1 || h < 2) return false;
    long double fact_h1 = 1.0L;
    for (int i = 2; i <= h - 1; ++i) fact_h1 *= i;
    const long double fact_h = fact_h1 * h;
    auto a_exact = [&](long double e) {
        long double p = 1.0L;
        for (int i = 1; i < h; ++i) p *= (i + e) * (i + 1 - e);
        return p / (fact_h1 * fact_h);
    };
    // the unnormalised weights (1 - e, e, e (1 - e) E_j / (j + e), e (1 - e) E_j / (j + 1 - e))
    // must sum to 1 / A_exact
    for (int k = 1; k < 8; ++k) {
        const long double e = k / 8.0L;
        long double tail = 0.0L;
        for (int j = 1; j < h; ++j) tail += E[j - 1] * (1.0L / (j + e) + 1.0L / (j + 1 - e));
        const long double sum = 1.0L + e * (1 - e) * tail;
        if (std::fabs((double)(sum * a_exact(e) - 1.0L)) > 1e-13) return false;
    }
    c4.resize(segs);
    c0.resize(segs);
    constexpr int m = 5;
    long double node[m];
    for (int i = 0; i < m; ++i)
        node[i] = 0.5L - 0.5L * std::cos((2 * i + 1) * 3.14159265358979323846L / (2 * m));
    for (int a = 0; a < segs; ++a) {
        auto sigma = [&](long double u) {
            const long double lerp = A[a] + u * ((long double)A[a + 1] - (long double)A[a]);
            return lerp / a_exact((a + u) * (long double)deps) - 1.0L;
        };
        // Vandermonde system V c = sigma(node), c = (c0 .. c4), Gauss-Jordan elimination
        long double V[m][m + 1];
        for (int i = 0; i < m; ++i) {
            long double pw = 1.0L;
            for (int j = 0; j < m; ++j, pw *= node[i]) V[i][j] = pw;
            V[i][m] = sigma(node[i]);
        }
        for (int col = 0; col < m; ++col) {
            int piv = col;
            for (int r = col + 1; r < m; ++r)
                if (std::fabs((double)V[r][col]) > std::fabs((double)V[piv][col])) piv = r;
            for (int j = 0; j <= m; ++j) std::swap(V[col][j], V[piv][j]);
            for (int r = 0; r < m; ++r) {
                if (r == col) continue;
                const long double f = V[r][col] / V[col][col];
                for (int j = col; j <= m; ++j) V[r][j] -= f * V[col][j];
            }
        }
        float c[m];
        for (int j = 0; j < m; ++j) c[j] = (float)(V[j][m] / V[j][j]);
        for (int k = 0; k <= 16; ++k) {  // the FP32 polynomial as the kernel evaluates it
            const float u = k / 16.0f;
            const float v = std::fma(std::fma(std::fma(std::fma(c[4], u, c[3]), u, c[2]), u, c[1]),
                                     u, c[0]);
            if (std::fabs((double)((long double)v - sigma(u))) > 1e-13) return false;
        }
        c4[a] = make_float4(c[4], c[3], c[2], c[1]);
        c0[a] = c[0];
    }
    return true;
}

// Staging layout: descriptors | tile prefix sums | waveform parameters |
// chunk prefix sums, each part 256-byte aligned.
struct StageLayout {
    size_t tiles, base, gb, chunks, counter, bytes;
};

StageLayout stage_layout(int cap, bool waveforms) {
    auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
    StageLayout l;
    l.tiles = up(sizeof(flr::FusedSource) * (size_t)cap);
    l.base = up(l.tiles + sizeof(long) * ((size_t)cap + 1));
    l.gb = up(l.base + sizeof(long) * ((size_t)cap + 1));
    l.chunks = up(l.gb + (waveforms ? sizeof(flr::GbParams) * (size_t)cap : 0));
    l.counter = up(l.chunks + (waveforms ? sizeof(long) * ((size_t)cap + 1) : 0));
    l.bytes = l.counter + sizeof(unsigned long long);
    return l;
}

// Check the sources and write their staging image for `cap` descriptors
// (entries num_sources..cap-1 are empty: no tiles, no chunks).  `diag` is set
// when a source asks for diagnostics, `inner` when one asks for inner
// products; `total_tiles` receives the run's work items.
int fill_stage(const flr_batch_plan *plan, const flr_batch_source *sources, int num_sources,
               const flr_gb_params *gb, int cap, const StageLayout &lay, unsigned char *hs,
               bool *diag, bool *inner, long *total_tiles) {
    const int tile = plan->base.tile;
    flr::FusedSource *srcs = reinterpret_cast<flr::FusedSource *>(hs);
    long *tile_start = reinterpret_cast<long *>(hs + lay.tiles);
    long *tile_base = reinterpret_cast<long *>(hs + lay.base);
    long *chunk_start = reinterpret_cast<long *>(hs + lay.chunks);
    long tiles = 0, chunks = 0;
    *diag = false;
    *inner = false;
    for (int i = 0; i < num_sources; ++i) {
        const flr_batch_source &s = sources[i];
        if ((!s.h && !gb) || (!s.out && !s.inner) || s.n < 2 || s.projections_start < 0 ||
            s.tdi_start < s.projections_start || 2LL * s.tdi_start >= s.n ||
            s.n > (1LL << 31) - 1 || s.tdi_set < 0 || s.tdi_set >= plan->num_sets)
            return fail(FLR_E_INVALID_ARGUMENT,
                        "source " + std::to_string(i) +
                            ": need h (or waveform parameters), out (or inner), "
                            "0 <= projections_start <= tdi_start "
                            "< n/2, "
                            "n < 2^31 and a valid tdi_set");
        if (gb && (gb[i].model < 0 || gb[i].model > 1))
            return fail(FLR_E_INVALID_ARGUMENT,
                        "source " + std::to_string(i) + ": unknown waveform model");
        if (reinterpret_cast<uintptr_t>(s.h) % 16 != 0)
            return fail(FLR_E_INVALID_ARGUMENT, "source " + std::to_string(i) +
                                                    ": h (complex128) must be 16-byte aligned");
        if ((s.d_rec_out == nullptr) != (s.d_em_out == nullptr))
            return fail(FLR_E_INVALID_ARGUMENT, "d_rec_out and d_em_out go together");
        if ((s.data == nullptr) != (s.inner == nullptr))
            return fail(FLR_E_INVALID_ARGUMENT, "source " + std::to_string(i) +
                                                    ": data and inner go together");
        flr::FusedSource d{};
        d.h = static_cast<const double2 *>(s.h);
        d.out = s.out;
        d.n = (long)s.n;
        d.ps = s.projections_start;
        d.ts = s.tdi_start;
        d.t0 = s.t0;
        for (int c = 0; c < 3; ++c) {
            d.k[c] = s.k[c];
            d.u[c] = s.u[c];
            d.v[c] = s.v[c];
        }
        d.tdi_set = s.tdi_set;
        d.y_out = s.y_out;
        d.d_rec_out = s.d_rec_out;
        d.d_em_out = s.d_em_out;
        d.d_tdi_out = s.d_tdi_out;
        d.data = s.data;
        d.inner = s.inner;
        const long all_tiles = (long)((s.n - 2LL * s.tdi_start + tile - 1) / tile);
        long first = 0, count = all_tiles;
        if (s.out_end > s.out_begin) {
            if (s.out_begin < s.tdi_start || s.out_end > s.n - s.tdi_start)
                return fail(FLR_E_INVALID_ARGUMENT,
                            "source " + std::to_string(i) +
                                ": need tdi_start <= out_begin < out_end <= n - tdi_start");
            first = (long)((s.out_begin - s.tdi_start) / tile);
            count = (long)((s.out_end - s.tdi_start + tile - 1) / tile) - first;
        }
        tile_base[i] = tiles - first;
        *diag = *diag || s.y_out || s.d_rec_out || s.d_tdi_out;
        *inner = *inner || s.inner;
        std::memcpy(srcs + i, &d, sizeof(d));
        tile_start[i] = tiles;
        tiles += count;
        if (gb) {
            chunk_start[i] = chunks;
            chunks += flr::gb_waveform_chunks((long)s.n);
            flr::GbParams g{gb[i].A,    gb[i].f,   gb[i].fdot,  gb[i].iota,
                            gb[i].phi0, gb[i].psi, gb[i].model, 0};
            std::memcpy(reinterpret_cast<flr::GbParams *>(hs + lay.gb) + i, &g, sizeof(g));
        }
    }
    if (tiles > 0x7fffffffL) return fail(FLR_E_INVALID_ARGUMENT, "too many tiles");
    *total_tiles = tiles;
    if (cap > num_sources) {
        std::memset(srcs + num_sources, 0, sizeof(flr::FusedSource) * (size_t)(cap - num_sources));
        if (gb)
            std::memset(reinterpret_cast<flr::GbParams *>(hs + lay.gb) + num_sources, 0,
                        sizeof(flr::GbParams) * (size_t)(cap - num_sources));
    }
    for (int i = num_sources; i <= cap; ++i) {
        tile_start[i] = tiles;
        tile_base[i] = tiles;
        if (gb) chunk_start[i] = chunks;
    }
    // the work-item counter starts at zero in every run (the copy resets it)
    *reinterpret_cast<unsigned long long *>(hs + lay.counter) = 0ull;
    return FLR_OK;
}

// Whether every source starts at t0 = +0 (its bit pattern is 0): such
// launches may take the fused kernel's t0 = 0 instance.
bool all_t0_zero(const flr_batch_source *sources, int num_sources) {
    for (int i = 0; i < num_sources; ++i) {
        unsigned long long bits;
        std::memcpy(&bits, &sources[i].t0, sizeof(bits));
        if (bits != 0ull) return false;
    }
    return num_sources > 0;
}

// The copy of a staging image to `d_stage` and the kernels that read it
// (t0_zero: every staged source starts at t0 = +0).
cudaError_t enqueue(const flr_batch_plan *plan, const unsigned char *h_stage,
                    unsigned char *d_stage, const StageLayout &lay, int cap, bool waveforms,
                    bool diag, double *partial, int chan, bool t0_zero, cudaEvent_t copied,
                    cudaStream_t st) {
    cudaError_t err = cudaMemcpyAsync(d_stage, h_stage, lay.bytes, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess && copied) err = cudaEventRecord(copied, st);
    if (err != cudaSuccess) return err;
    const flr::FusedSource *d_src = reinterpret_cast<const flr::FusedSource *>(d_stage);
    if (waveforms) {
        err = flr::launch_gb_waveforms(
            d_src, reinterpret_cast<const flr::GbParams *>(d_stage + lay.gb),
            reinterpret_cast<const long *>(d_stage + lay.chunks), cap, plan->base.dt,
            plan->sms * 8, st);
        if (err != cudaSuccess) return err;
    }
    flr::FusedArgs a = plan->base;
    a.sources = d_src;
    a.tile_start = reinterpret_cast<const long *>(d_stage + lay.tiles);
    a.tile_base = reinterpret_cast<const long *>(d_stage + lay.base);
    a.work_next = reinterpret_cast<unsigned long long *>(d_stage + lay.counter);
    a.num_sources = cap;
    a.chan = chan;
    a.partial = partial;
    a.gb = waveforms ? reinterpret_cast<const flr::GbParams *>(d_stage + lay.gb) : nullptr;
    // the difference forms for XYZ outputs; AET / AE keep the double-float form,
    // whose absolute error stays ~1e-14 of the links: those channels are
    // combinations of X, Y, Z that can cancel to a small fraction of them
    const bool d2 = plan->mixed && plan->base.d2 && chan == FLR_CHAN_XYZ;
    err = flr::launch_fused(plan->mixed, plan->grouped, diag, partial != nullptr, d2, t0_zero, a,
                            plan->grid_max,
                            plan->smem, st);
    if (err == cudaSuccess && partial) err = flr::launch_inner_reduce(a, st);
    return err;
}

void release_graph(flr_batch_graph *g) {
    if (!g) return;
    for (int b = 0; b < 2; ++b) {
        if (g->exec[b]) cudaGraphExecDestroy(g->exec[b]);
        if (g->exec_t0[b]) cudaGraphExecDestroy(g->exec_t0[b]);
        if (g->h_stage[b]) cudaFreeHost(g->h_stage[b]);
        if (g->done[b]) cudaEventDestroy(g->done[b]);
    }
    if (g->d_stage) cudaFree(g->d_stage);
    delete g;
}

}  // namespace

extern "C" {

int flr_batch_plan_create(flr_orbits *orbits, int order, const double *A_in, double deps,
                          int num_A, const double *E_in, double sampling_frequency,
                          const flr_tdi_units *sets, int num_sets, int precision, int tile,
                          flr_batch_plan **out) {
    flr::set_last_error("");
    if (!out) return fail(FLR_E_INVALID_ARGUMENT, "out must not be NULL");
    *out = nullptr;
    if (!orbits) return fail(FLR_E_NO_ORBITS, "Must add orbits with add_orbit_information method.");
    int rc = current_device_is(orbits->device);
    if (rc) return rc;
    const int h = (order + 1) / 2;
    if (order < 1 || h > flr::kFusedMaxH)
        return fail(FLR_E_INVALID_ARGUMENT, "order must be in [1, " +
                                                std::to_string(2 * flr::kFusedMaxH - 1) + "]");
    if (!A_in || num_A < 2 || !(deps > 0.0) || (h > 1 && !E_in))
        return fail(FLR_E_INVALID_ARGUMENT, "invalid Lagrange tables");
    if (!(sampling_frequency > 0.0))
        return fail(FLR_E_INVALID_ARGUMENT, "sampling_frequency must be positive");
    if (!sets || num_sets < 1 || num_sets > 64)
        return fail(FLR_E_INVALID_ARGUMENT, "need 1..64 TDI unit sets");
    if (precision != FLR_PRECISION_FP64 && precision != FLR_PRECISION_MIXED)
        return fail(FLR_E_INVALID_ARGUMENT, "precision must be FLR_PRECISION_FP64 or _MIXED");
    if (tile == 0) tile = 512;
    if (tile < 32 || tile > 8192) return fail(FLR_E_INVALID_ARGUMENT, "tile must be in [32, 8192]");

    // largest light travel time of the orbit table; equal-arm tables (all six
    // links equal at every knot) give equal delays to lists of equal length
    std::vector<double> ltt((size_t)orbits->N * 6);
    cudaError_t err = cudaMemcpy(ltt.data(), orbits->ltt, ltt.size() * sizeof(double),
                                 cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_fail(err, "reading the orbit table");
    double lmax = 0.0;
    bool equal_arms = true;
    for (size_t i = 0; i < ltt.size(); ++i) {
        lmax = std::max(lmax, std::fabs(ltt[i]));
        if (ltt[i] != ltt[(i / 6) * 6]) equal_arms = false;
    }
    const bool mixed = (precision == FLR_PRECISION_MIXED);

    // TDI sets: map link numbers to slots, check sizes.  The FP64 flavour keeps
    // the reference's unit order (its per-channel sums are order-sensitive);
    // the mixed flavour on equal-arm orbits orders units by delay-list length
    // so that units with equal delays are adjacent and share the index split.
    std::vector<flr::FusedTdiSet> hsets(num_sets);
    int max_len = 0;
    for (int si = 0; si < num_sets; ++si) {
        const flr_tdi_units &in = sets[si];
        flr::FusedTdiSet &s = hsets[si];
        std::memset(&s, 0, sizeof(s));
        if (in.num_units < 1 || in.num_units > flr::kFusedMaxUnits || in.num_combos < 0 ||
            in.num_combos > flr::kFusedMaxCombos || !in.unit_starts || !in.unit_lengths ||
            !in.tdi_base_link || !in.tdi_link_combinations || !in.tdi_signs || !in.channels)
            return fail(FLR_E_INVALID_ARGUMENT,
                        "TDI set " + std::to_string(si) + ": 1.." +
                            std::to_string(flr::kFusedMaxUnits) + " units and at most " +
                            std::to_string(flr::kFusedMaxCombos) + " link entries");
        s.num_units = in.num_units;
        s.num_combos = in.num_combos;
        for (int c = 0; c < in.num_combos; ++c) {
            const int link = in.tdi_link_combinations[c];
            s.combo_slot[c] = (link == -11) ? -1 : slot_of(orbits, link);
            if (link != -11 && s.combo_slot[c] < 0)
                return fail(FLR_E_INVALID_ARGUMENT,
                            "TDI link " + std::to_string(link) + " is not an orbit link");
        }
        std::vector<int> order(in.num_units);
        for (int u = 0; u < in.num_units; ++u) order[u] = u;
        if (mixed && equal_arms) {
            auto list_len = [&](int u) {
                int len = 0;
                for (int c = in.unit_starts[u]; c < in.unit_starts[u] + in.unit_lengths[u]; ++c)
                    len += (c >= 0 && c < in.num_combos && in.tdi_link_combinations[c] != -11);
                return len;
            };
            std::stable_sort(order.begin(), order.end(),
                             [&](int a, int b) { return list_len(a) < list_len(b); });
        }
        for (int u = 0; u < in.num_units; ++u) {
            const int src_u = order[u];
            const int st = in.unit_starts[src_u], ln = in.unit_lengths[src_u];
            if (st < 0 || ln < 0 || st + ln > in.num_combos)
                return fail(FLR_E_INVALID_ARGUMENT, "unit_starts/unit_lengths outside the links");
            if (in.channels[src_u] < 0 || in.channels[src_u] > 2)
                return fail(FLR_E_INVALID_ARGUMENT, "channels must be 0, 1 or 2");
            s.unit_start[u] = st;
            s.unit_len[u] = ln;
            s.orig_unit[u] = src_u;
            s.base_slot[u] = slot_of(orbits, in.tdi_base_link[src_u]);
            if (s.base_slot[u] < 0)
                return fail(FLR_E_INVALID_ARGUMENT, "TDI base link is not an orbit link");
            s.channel[u] = in.channels[src_u];
            s.sign[u] = in.tdi_signs[src_u];
            s.sign_code[u] = (s.sign[u] == 1.0) ? 1 : (s.sign[u] == -1.0) ? -1 : 0;
            int len = 0;
            for (int c = st; c < st + ln; ++c) {
                if (s.combo_slot[c] < 0) continue;
                if (len == flr::kFusedMaxDepth)
                    return fail(FLR_E_INVALID_ARGUMENT,
                                "TDI delay lists may hold at most " +
                                    std::to_string(flr::kFusedMaxDepth) + " links");
                s.delay_slot[u][len++] = s.combo_slot[c];
            }
            s.delay_len[u] = len;
            int keep = 0;
            if (u > 0) {
                const int lim = std::min(len, (int)s.delay_len[u - 1]);
                if (mixed && equal_arms)
                    keep = lim;  // every L(t) is the same value: partial sums depend on length only
                else
                    while (keep < lim && s.delay_slot[u][keep] == s.delay_slot[u - 1][keep]) ++keep;
            }
            s.prefix_keep[u] = keep;
            max_len = std::max(max_len, len);
        }
        if (mixed && equal_arms) make_groups(s);
    }
    const bool grouped =
        mixed && equal_arms &&
        std::all_of(hsets.begin(), hsets.end(), [](const flr::FusedTdiSet &t) { return t.grouped; });


    flr_batch_plan *p = new flr_batch_plan();
    p->device = orbits->device;
    p->mixed = mixed;
    p->grouped = grouped;
    p->num_sets = num_sets;
    p->set_max_len = max_len;
    const int y_halo = (int)std::ceil(max_len * lmax * sampling_frequency) + h + 3;
    const int spread = (int)std::ceil(2.0 * lmax * sampling_frequency) + 2;
    p->base.tile = tile;
    p->base.y_halo = y_halo;
    p->base.y_halo_hi = std::min(y_halo, h + 3);
    p->base.y_max = tile + 2 * y_halo;
    p->base.win_max = tile + 2 * y_halo + 2 * h + spread + 2 * 4 + 16;
    p->smem = flr::fused_smem_bytes(p->mixed, p->base.win_max, p->base.y_max);

    // device copies of A, E, the double-float A table and the sets
    const size_t a_bytes = sizeof(double) * (size_t)num_A;
    const size_t e_bytes = sizeof(double) * (size_t)std::max(h - 1, 1);
    const size_t atab_off = (a_bytes + e_bytes + 255) & ~size_t(255);
    const size_t sig4_off = (atab_off + sizeof(float4) * (size_t)num_A + 255) & ~size_t(255);
    const size_t sig0_off = (sig4_off + sizeof(float4) * (size_t)num_A + 255) & ~size_t(255);
    const size_t set_off = (sig0_off + sizeof(float) * (size_t)num_A + 255) & ~size_t(255);
    std::vector<double> a_host(num_A);
    err = cudaMemcpy(a_host.data(), A_in, a_bytes, cudaMemcpyDefault);
    if (err != cudaSuccess) {
        release(p);
        return cuda_fail(err, "reading the A table");
    }
    std::vector<double> e_host(std::max(h - 1, 1), 0.0);
    if (h > 1) {
        err = cudaMemcpy(e_host.data(), E_in, sizeof(double) * (h - 1), cudaMemcpyDefault);
        if (err != cudaSuccess) {
            release(p);
            return cuda_fail(err, "reading the E table");
        }
    }
    std::vector<float4> a_tab(num_A);
    for (int i = 0; i < num_A; ++i) {
        const double a = a_host[i];
        const double da = (i + 1 < num_A) ? a_host[i + 1] - a_host[i] : 0.0;
        const float ah = (float)a, dah = (float)da;
        a_tab[i] = make_float4(ah, (float)(a - (double)ah), dah, (float)(da - (double)dah));
    }
    // second-difference TDI form (mixed flavour): the sigma table of the A table
    std::vector<float4> sig4;
    std::vector<float> sig0;
    const bool d2 = mixed && fit_sigma_table(a_host, e_host, h, deps, sig4, sig0);
    err = cudaMalloc(&p->d_tables, set_off + sizeof(flr::FusedTdiSet) * num_sets);
    if (err == cudaSuccess && d2)
        err = cudaMemcpy(static_cast<char *>(p->d_tables) + sig4_off, sig4.data(),
                         sizeof(float4) * sig4.size(), cudaMemcpyHostToDevice);
    if (err == cudaSuccess && d2)
        err = cudaMemcpy(static_cast<char *>(p->d_tables) + sig0_off, sig0.data(),
                         sizeof(float) * sig0.size(), cudaMemcpyHostToDevice);
    if (err == cudaSuccess)
        err = cudaMemcpy(static_cast<char *>(p->d_tables) + atab_off, a_tab.data(),
                         sizeof(float4) * (size_t)num_A, cudaMemcpyHostToDevice);
    if (err == cudaSuccess)
        err = cudaMemcpy(p->d_tables, A_in, a_bytes, cudaMemcpyDefault);
    if (err == cudaSuccess && h > 1)
        err = cudaMemcpy(static_cast<char *>(p->d_tables) + a_bytes, E_in,
                         sizeof(double) * (h - 1), cudaMemcpyDefault);
    if (err == cudaSuccess)
        err = cudaMemcpy(static_cast<char *>(p->d_tables) + set_off, hsets.data(),
                         sizeof(flr::FusedTdiSet) * num_sets, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->stage_free, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming);
    int smem_optin = 0;
    if (err == cudaSuccess)
        err = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                     p->device);
    if (err == cudaSuccess && p->smem > (size_t)smem_optin) {
        release(p);
        return fail(FLR_E_UNSUPPORTED, "tile " + std::to_string(tile) + " needs " +
                                           std::to_string(p->smem) +
                                           " B of shared memory per block; the device allows " +
                                           std::to_string(smem_optin));
    }
    int per_sm = 0;
    if (err == cudaSuccess) err = flr::fused_configure(p->mixed, p->grouped, p->smem, &per_sm);
    int sms = 0;
    if (err == cudaSuccess)
        err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
    if (err != cudaSuccess) {
        release(p);
        return cuda_fail(err, "creating the batch plan");
    }
    if (per_sm < 1) {
        release(p);
        return fail(FLR_E_UNSUPPORTED, "the fused kernel does not fit on an SM with " +
                                           std::to_string(p->smem) + " B of shared memory");
    }
    p->grid_max = sms * per_sm;
    p->sms = sms;

    flr::FusedArgs &b = p->base;
    b.orb = flr::device_tables(orbits);
    b.lt.A = static_cast<const double *>(p->d_tables);
    b.lt.E = reinterpret_cast<const double *>(static_cast<char *>(p->d_tables) + a_bytes);
    b.lt.deps = deps;
    b.lt.num_A = num_A;
    b.lt.h = h;
    // Outer TDI taps in FP32 (mixed flavour): with c = A eps (1 - eps) <= max A / 4
    // and both denominators j + eps, j + 1 - eps >= j, the taps j >= h_df weigh
    // at most 2 sum_j c_max |E_j| / j <= 5e-6 of the link values together, so
    // their FP32 evaluation (relative error ~2e-7) adds at most ~1e-12 of max|y|
    // to a unit's interpolation, against ~1e-14 from the double-float taps and
    // an error budget of ~1e-11 (1e-6 relative on a 2nd-generation channel at
    // 1e-4 Hz, 3e-4 of the link amplitude).  Order 25: taps 10..12; order 45:
    // 14..22.
    b.h_df = h;
    if (p->mixed) {
        double a_max = 0.0, outer = 0.0;
        for (int i = 0; i < num_A; ++i) a_max = std::max(a_max, std::fabs(a_host[i]));
        for (int j = h - 1; j >= 1; --j) {
            outer += 2.0 * 0.25 * a_max * std::fabs(e_host[j - 1]) / j;
            if (outer > 5e-6) break;
            b.h_df = j;
        }
    }
    b.sets = reinterpret_cast<const flr::FusedTdiSet *>(static_cast<char *>(p->d_tables) +
                                                       set_off);
    b.num_sets = num_sets;
    b.a_tab = reinterpret_cast<const float4 *>(static_cast<char *>(p->d_tables) + atab_off);
    b.d2 = d2 ? 1 : 0;
    b.sig4 = reinterpret_cast<const float4 *>(static_cast<char *>(p->d_tables) + sig4_off);
    b.sig0 = reinterpret_cast<const float *>(static_cast<char *>(p->d_tables) + sig0_off);
    b.wait_polls = flr::kFusedWaitPolls;
    b.fs = sampling_frequency;
    b.dt = 1.0 / sampling_frequency;
    b.inv_deps = 1.0 / deps;
    b.inv_orbit_dt = 1.0 / orbits->dt;
    // receiving spacecraft and their two links each (any LISA link table)
    b.rx_shared = 1;
    for (int r = 0; r < 3; ++r) {
        int found = 0;
        for (int slot = 0; slot < 6; ++slot) {
            if (orbits->sc_r[slot] != r + 1) continue;
            if (found < 2) b.rx_slot[r][found] = slot;
            ++found;
        }
        b.rx_sc[r] = r + 1;
        if (found != 2) b.rx_shared = 0;
    }
    b.trio = b.rx_shared && equal_arms;
    for (int r = 0; r < 3; ++r) {
        b.tx_slot[r] = -1;
        for (int slot = 5; slot >= 0; --slot)
            if (orbits->sc_e[slot] == r + 1) b.tx_slot[r] = slot;
        if (b.tx_slot[r] < 0) b.trio = 0;
    }
    *out = p;
    return FLR_OK;
}

int flr_batch_plan_destroy(flr_batch_plan *plan) {
    if (!plan) return FLR_OK;
    if (plan->stage_pending) cudaEventSynchronize(plan->stage_free);
    if (plan->done_pending) cudaEventSynchronize(plan->done);
    release(plan);
    return FLR_OK;
}

int flr_batch_plan_info(const flr_batch_plan *plan, int *info, int n_info) {
    if (!plan || !info) return fail(FLR_E_INVALID_ARGUMENT, "NULL argument");
    const int vals[] = {plan->base.tile, plan->base.y_halo, plan->base.win_max,
                        plan->base.y_max, (int)plan->smem, plan->grid_max,
                        plan->mixed ? FLR_PRECISION_MIXED : FLR_PRECISION_FP64,
                        plan->grouped ? 1 : 0, plan->base.h_df, plan->base.d2,
                        flr::kFusedThreads, flr::kFusedStagingDepth};
    for (int i = 0; i < n_info && i < (int)(sizeof(vals) / sizeof(int)); ++i) info[i] = vals[i];
    return FLR_OK;
}

int flr_batch_plan_set_wait_limit(flr_batch_plan *plan, long long polls) {
    flr::set_last_error("");
    if (!plan) return fail(FLR_E_INVALID_ARGUMENT, "plan must not be NULL");
    plan->base.wait_polls = (polls < 0) ? flr::kFusedWaitPolls
                                        : (long)std::min<long long>(polls, flr::kFusedWaitPolls);
    return FLR_OK;
}

static int batch_run(flr_batch_plan *plan, const flr_batch_source *sources, int num_sources,
                     const flr_gb_params *gb, int chan, void *stream) {
    flr::set_last_error("");
    if (!plan) return fail(FLR_E_INVALID_ARGUMENT, "plan must not be NULL");
    int rc = current_device_is(plan->device);
    if (rc) return rc;
    if (num_sources < 0 || (num_sources > 0 && !sources))
        return fail(FLR_E_INVALID_ARGUMENT, "invalid source list");
    if (chan != FLR_CHAN_XYZ && chan != FLR_CHAN_AET && chan != FLR_CHAN_AE)
        return fail(FLR_E_INVALID_ARGUMENT, "chan must be FLR_CHAN_XYZ, _AET or _AE");
    if (num_sources == 0) return FLR_OK;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t err = cudaSuccess;
    // the pinned staging buffer of the previous run must have been consumed
    if (plan->stage_pending) {
        err = cudaEventSynchronize(plan->stage_free);
        if (err != cudaSuccess) return cuda_fail(err, "waiting for the previous run's copies");
        plan->stage_pending = false;
    }
    const StageLayout lay = stage_layout(num_sources, gb != nullptr);
    if (lay.bytes > plan->cap_stage) {
        if (plan->h_stage) cudaFreeHost(plan->h_stage);
        plan->h_stage = nullptr;
        plan->cap_stage = 0;
        err = cudaMallocHost(&plan->h_stage, lay.bytes * 2);
        if (err != cudaSuccess) return cuda_fail(err, "allocating the staging buffer");
        plan->cap_stage = lay.bytes * 2;
    }
    bool diag = false, inner = false;
    long tiles = 0;
    rc = fill_stage(plan, sources, num_sources, gb, num_sources, lay, plan->h_stage, &diag, &inner,
                    &tiles);
    if (rc) return rc;
    if (diag && inner)
        return fail(FLR_E_INVALID_ARGUMENT, "diagnostics and inner products need separate runs");
    // the device staging buffer is reused: a previous run on another stream
    // must have finished reading it
    if (plan->done_pending) {
        err = cudaStreamWaitEvent(st, plan->done, 0);
        if (err != cudaSuccess) return cuda_fail(err, "ordering after the previous run");
    }
    if (lay.bytes > plan->cap_device) {
        if (plan->d_stage) {
            err = cudaStreamSynchronize(st);
            if (err == cudaSuccess) err = cudaFree(plan->d_stage);
            if (err != cudaSuccess) return cuda_fail(err, "releasing the staging buffer");
        }
        plan->d_stage = nullptr;
        plan->cap_device = 0;
        err = cudaMalloc(&plan->d_stage, lay.bytes * 2);
        if (err != cudaSuccess) return cuda_fail(err, "allocating the staging buffer");
        plan->cap_device = lay.bytes * 2;
    }
    const size_t partial_bytes = sizeof(double) * 6 * (size_t)tiles;
    if (inner && partial_bytes > plan->cap_partial) {
        if (plan->d_partial) {  // an earlier run may still read it
            err = cudaDeviceSynchronize();
            if (err == cudaSuccess) err = cudaFree(plan->d_partial);
            if (err != cudaSuccess) return cuda_fail(err, "releasing the inner-product buffer");
        }
        plan->d_partial = nullptr;
        plan->cap_partial = 0;
        err = cudaMalloc(&plan->d_partial, partial_bytes + partial_bytes / 2);
        if (err != cudaSuccess) return cuda_fail(err, "allocating the inner-product buffer");
        plan->cap_partial = partial_bytes + partial_bytes / 2;
    }
    err = enqueue(plan, plan->h_stage, plan->d_stage, lay, num_sources, gb != nullptr, diag,
                  inner ? plan->d_partial : nullptr, chan, all_t0_zero(sources, num_sources),
                  plan->stage_free, st);
    plan->stage_pending = true;
    if (err != cudaSuccess) return cuda_fail(err, "launching the batch");
    err = cudaEventRecord(plan->done, st);
    if (err != cudaSuccess) return cuda_fail(err, "recording the batch");
    plan->done_pending = true;
    return FLR_OK;
}

int flr_batch_run(flr_batch_plan *plan, const flr_batch_source *sources, int num_sources,
                  int chan, void *stream) {
    return batch_run(plan, sources, num_sources, nullptr, chan, stream);
}

int flr_batch_run_gb(flr_batch_plan *plan, const flr_batch_source *sources,
                     const flr_gb_params *params, int num_sources, int chan, void *stream) {
    if (num_sources > 0 && !params)
        return fail(FLR_E_INVALID_ARGUMENT, "params must not be NULL");
    return batch_run(plan, sources, num_sources, params, chan, stream);
}

int flr_batch_graph_create(flr_batch_plan *plan, int max_sources, int flags, int chan,
                           flr_batch_graph **out) {
    flr::set_last_error("");
    if (!out) return fail(FLR_E_INVALID_ARGUMENT, "out must not be NULL");
    *out = nullptr;
    if (!plan) return fail(FLR_E_INVALID_ARGUMENT, "plan must not be NULL");
    int rc = current_device_is(plan->device);
    if (rc) return rc;
    if (max_sources < 1 || max_sources > (1 << 20))
        return fail(FLR_E_INVALID_ARGUMENT, "max_sources must be in [1, 2^20]");
    if (flags & ~(FLR_GRAPH_WAVEFORMS | FLR_GRAPH_DIAGNOSTICS))
        return fail(FLR_E_INVALID_ARGUMENT, "unknown graph flags");
    if (chan != FLR_CHAN_XYZ && chan != FLR_CHAN_AET && chan != FLR_CHAN_AE)
        return fail(FLR_E_INVALID_ARGUMENT, "chan must be FLR_CHAN_XYZ, _AET or _AE");
    flr_batch_graph *g = new flr_batch_graph();
    g->plan = plan;
    g->cap = max_sources;
    g->waveforms = (flags & FLR_GRAPH_WAVEFORMS) != 0;
    g->diag = (flags & FLR_GRAPH_DIAGNOSTICS) != 0;
    g->chan = chan;
    g->last = -1;
    const StageLayout lay = stage_layout(g->cap, g->waveforms);
    cudaError_t err = cudaMalloc(&g->d_stage, lay.bytes);
    for (int b = 0; b < 2 && err == cudaSuccess; ++b) {
        err = cudaMallocHost(&g->h_stage[b], lay.bytes);
        if (err == cudaSuccess) std::memset(g->h_stage[b], 0, lay.bytes);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&g->done[b], cudaEventDisableTiming);
    }
    cudaStream_t cs = nullptr;
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    // per staging buffer, the general launch and (where the difference-form
    // instance runs) the one for sources that all start at t0 = +0
    const bool with_t0 = plan->mixed && plan->base.d2 && chan == FLR_CHAN_XYZ && !g->diag;
    for (int v = 0; v < (with_t0 ? 4 : 2) && err == cudaSuccess; ++v) {
        const int b = v & 1;
        err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) break;
        const cudaError_t e_enq = enqueue(plan, g->h_stage[b], g->d_stage, lay, g->cap,
                                          g->waveforms, g->diag, nullptr, chan, v >= 2, nullptr,
                                          cs);
        cudaGraph_t graph = nullptr;
        const cudaError_t e_end = cudaStreamEndCapture(cs, &graph);
        err = (e_enq != cudaSuccess) ? e_enq : e_end;
        if (err == cudaSuccess)
            err = cudaGraphInstantiate(v >= 2 ? &g->exec_t0[b] : &g->exec[b], graph, 0);
        if (graph) cudaGraphDestroy(graph);
    }
    if (cs) cudaStreamDestroy(cs);
    if (err != cudaSuccess) {
        release_graph(g);
        return cuda_fail(err, "capturing the batch graph");
    }
    *out = g;
    return FLR_OK;
}

int flr_batch_graph_launch(flr_batch_graph *g, const flr_batch_source *sources,
                           const flr_gb_params *params, int num_sources, void *stream) {
    flr::set_last_error("");
    if (!g) return fail(FLR_E_INVALID_ARGUMENT, "graph must not be NULL");
    int rc = current_device_is(g->plan->device);
    if (rc) return rc;
    if (num_sources < 0 || num_sources > g->cap || (num_sources > 0 && !sources))
        return fail(FLR_E_INVALID_ARGUMENT, "need 0.." + std::to_string(g->cap) + " sources");
    if (g->waveforms && num_sources > 0 && !params)
        return fail(FLR_E_INVALID_ARGUMENT, "this graph generates waveforms: params required");
    if (!g->waveforms && params)
        return fail(FLR_E_INVALID_ARGUMENT, "this graph has no waveform stage");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t err = cudaSuccess;
    const int b = g->next;
    if (g->pending[b]) {  // the launch that last used this staging buffer
        err = cudaEventSynchronize(g->done[b]);
        if (err != cudaSuccess) return cuda_fail(err, "waiting for an earlier launch");
        g->pending[b] = false;
    }
    const StageLayout lay = stage_layout(g->cap, g->waveforms);
    bool diag = false, inner = false;
    long tiles = 0;
    rc = fill_stage(g->plan, sources, num_sources, g->waveforms ? params : nullptr, g->cap, lay,
                    g->h_stage[b], &diag, &inner, &tiles);
    if (rc) return rc;
    if (inner)
        return fail(FLR_E_INVALID_ARGUMENT,
                    "inner products are not available through batch graphs: use flr_batch_run");
    if (diag && !g->diag)
        return fail(FLR_E_INVALID_ARGUMENT,
                    "diagnostics need a graph created with FLR_GRAPH_DIAGNOSTICS");
    if (g->last >= 0 && g->pending[g->last]) {  // the device staging buffer is shared
        err = cudaStreamWaitEvent(st, g->done[g->last], 0);
        if (err != cudaSuccess) return cuda_fail(err, "ordering after the previous launch");
    }
    const bool t0_zero = g->exec_t0[b] && all_t0_zero(sources, num_sources);
    err = cudaGraphLaunch(t0_zero ? g->exec_t0[b] : g->exec[b], st);
    if (err == cudaSuccess) err = cudaEventRecord(g->done[b], st);
    if (err != cudaSuccess) return cuda_fail(err, "launching the batch graph");
    g->pending[b] = true;
    g->last = b;
    g->next = 1 - b;
    return FLR_OK;
}

int flr_batch_graph_destroy(flr_batch_graph *g) {
    if (!g) return FLR_OK;
    for (int b = 0; b < 2; ++b)
        if (g->pending[b]) cudaEventSynchronize(g->done[b]);
    release_graph(g);
    return FLR_OK;
}


// ------------------------------------------------------------------ serving --

int flr_server_create(flr_batch_plan *plan, int capacity, int chan, double idle_seconds,
                      flr_server **out) {
    flr::set_last_error("");
    if (!plan || !out) return fail(FLR_E_INVALID_ARGUMENT, "plan and out must not be NULL");
    *out = nullptr;
    if (!plan->mixed) return fail(FLR_E_INVALID_ARGUMENT, "serving needs a mixed-precision plan");
    if (capacity < 1 || capacity > (1 << 24))
        return fail(FLR_E_INVALID_ARGUMENT, "capacity must be in [1, 2^24]");
    if (chan != FLR_CHAN_XYZ && chan != FLR_CHAN_AET && chan != FLR_CHAN_AE)
        return fail(FLR_E_INVALID_ARGUMENT, "chan must be FLR_CHAN_XYZ, _AET or _AE");
    if (!(idle_seconds > 0.0) || idle_seconds > 60.0)
        return fail(FLR_E_INVALID_ARGUMENT, "idle_seconds must be in (0, 60]");
    int rc = current_device_is(plan->device);
    if (rc) return rc;
    flr_server *sv = new flr_server();
    sv->plan = plan;
    sv->chan = chan;
    sv->d2 = plan->base.d2 && chan == FLR_CHAN_XYZ;
    sv->cap = capacity;
    sv->idle_ns = (long long)(idle_seconds * 1e9);
    auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t o_src = 0;
    const size_t o_gb = up(o_src + sizeof(flr::FusedSource) * (size_t)capacity);
    const size_t o_ts = up(o_gb + sizeof(flr::GbParams) * (size_t)capacity);
    const size_t o_pub = up(o_ts + sizeof(long long) * ((size_t)capacity + 1));
    const size_t o_stop = o_pub + 64;
    const size_t o_done = up(o_stop + 64);
    const size_t bytes = up(o_done + sizeof(unsigned) * (size_t)capacity);
    void *hb = nullptr, *db = nullptr;
    cudaError_t err = cudaHostAlloc(&hb, bytes, cudaHostAllocMapped | cudaHostAllocPortable);
    if (err == cudaSuccess) err = cudaHostGetDevicePointer(&db, hb, 0);
    if (err == cudaSuccess) err = cudaMalloc(&sv->d_next, sizeof(unsigned long long));
    if (err == cudaSuccess) err = cudaMalloc(&sv->d_tiles_done, sizeof(unsigned) * (size_t)capacity);
    if (err == cudaSuccess) err = cudaMemset(sv->d_next, 0, sizeof(unsigned long long));
    if (err == cudaSuccess) err = cudaMemset(sv->d_tiles_done, 0, sizeof(unsigned) * (size_t)capacity);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&sv->ran, cudaEventDisableTiming);
    sv->h_block = static_cast<unsigned char *>(hb);
    if (err != cudaSuccess) {
        flr_server_destroy(sv);
        return cuda_fail(err, "allocating the serving buffers");
    }
    unsigned char *h = sv->h_block, *d = static_cast<unsigned char *>(db);
    std::memset(h, 0, bytes);
    sv->h_src = reinterpret_cast<flr::FusedSource *>(h + o_src);
    sv->h_gb = reinterpret_cast<flr::GbParams *>(h + o_gb);
    sv->h_tile_start = reinterpret_cast<long long *>(h + o_ts);
    sv->h_published = reinterpret_cast<unsigned long long *>(h + o_pub);
    sv->h_stop = reinterpret_cast<int *>(h + o_stop);
    sv->h_done = reinterpret_cast<unsigned *>(h + o_done);
    sv->d_src = reinterpret_cast<flr::FusedSource *>(d + o_src);
    sv->d_gb = reinterpret_cast<flr::GbParams *>(d + o_gb);
    sv->d_tile_start = reinterpret_cast<long long *>(d + o_ts);
    sv->d_published = reinterpret_cast<unsigned long long *>(d + o_pub);
    sv->d_stop = reinterpret_cast<int *>(d + o_stop);
    sv->d_done = reinterpret_cast<unsigned *>(d + o_done);
    for (int i = 1; i <= capacity; ++i) sv->h_tile_start[i] = INT64_MAX;  // not yet published
    *out = sv;
    return FLR_OK;
}

int flr_server_submit(flr_server *sv, const flr_batch_source *source, const flr_gb_params *params,
                      int *slot) {
    flr::set_last_error("");
    if (!sv || !source || !slot) return fail(FLR_E_INVALID_ARGUMENT, "NULL argument");
    if (sv->count >= sv->cap)
        return fail(FLR_E_INVALID_ARGUMENT, "the server's source list is full");
    if (source->y_out || source->d_rec_out || source->d_em_out || source->d_tdi_out ||
        source->data || source->inner || source->out_end > source->out_begin)
        return fail(FLR_E_INVALID_ARGUMENT,
                    "serving takes whole sources without diagnostics or inner products");
    if (!source->out) return fail(FLR_E_INVALID_ARGUMENT, "out must not be NULL");
    // the batch path's checks and descriptor, for one source
    const StageLayout lay = stage_layout(1, params != nullptr);
    std::vector<unsigned char> stage(lay.bytes);
    bool diag = false, inner = false;
    long tiles = 0;
    int rc = fill_stage(sv->plan, source, 1, params, 1, lay, stage.data(), &diag, &inner, &tiles);
    if (rc) return rc;
    const int i = sv->count;
    std::memcpy(sv->h_src + i, stage.data(), sizeof(flr::FusedSource));
    if (params)
        std::memcpy(sv->h_gb + i, stage.data() + lay.gb, sizeof(flr::GbParams));
    else
        std::memset(sv->h_gb + i, 0, sizeof(flr::GbParams));
    sv->h_done[i] = 0u;
    const long long end = sv->items + tiles;
    sv->h_tile_start[i + 1] = end;
    // publish: the descriptor and prefix sum are visible before the count
    __atomic_store_n(sv->h_published, (unsigned long long)end, __ATOMIC_RELEASE);
    sv->items = end;
    sv->count = i + 1;
    *slot = i;
    return FLR_OK;
}

static void advance_first_open(flr_server *sv) {
    while (sv->first_open < sv->count &&
           __atomic_load_n(sv->h_done + sv->first_open, __ATOMIC_ACQUIRE) != 0u)
        ++sv->first_open;
}

int flr_server_pump(flr_server *sv, void *stream) {
    flr::set_last_error("");
    if (!sv) return fail(FLR_E_INVALID_ARGUMENT, "server must not be NULL");
    int rc = current_device_is(sv->plan->device);
    if (rc) return rc;
    advance_first_open(sv);
    if (sv->launched) {
        const cudaError_t q = cudaEventQuery(sv->ran);
        if (q == cudaErrorNotReady) return FLR_OK;  // still running: it will claim new items
        if (q != cudaSuccess) return cuda_fail(q, "querying the serving kernel");
        sv->launched = false;
    }
    advance_first_open(sv);
    if (sv->first_open >= sv->count || __atomic_load_n(sv->h_stop, __ATOMIC_RELAXED)) return FLR_OK;
    flr::FusedArgs a = sv->plan->base;
    a.sources = sv->d_src;
    a.tile_start = reinterpret_cast<const long *>(sv->d_tile_start);
    a.tile_base = reinterpret_cast<const long *>(sv->d_tile_start);
    a.gb = sv->d_gb;
    a.num_sources = sv->cap;
    a.chan = sv->chan;
    a.partial = nullptr;
    a.work_next = sv->d_next;
    a.srv_published = sv->d_published;
    a.srv_stop = sv->d_stop;
    a.srv_tiles_done = sv->d_tiles_done;
    a.srv_done = sv->d_done;
    a.srv_idle_ns = sv->idle_ns;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t err = flr::launch_fused_server(sv->plan->grouped, sv->d2, a, sv->plan->grid_max,
                                               sv->plan->smem, st);
    if (err == cudaSuccess) err = cudaEventRecord(sv->ran, st);
    if (err != cudaSuccess) return cuda_fail(err, "launching the serving kernel");
    sv->launched = true;
    ++sv->launches;
    return FLR_OK;
}

int flr_server_info(flr_server *sv, long long *info, int n_info) {
    if (!sv || !info) return fail(FLR_E_INVALID_ARGUMENT, "NULL argument");
    advance_first_open(sv);
    const long long vals[] = {sv->count, sv->items, sv->first_open, sv->launches,
                              sv->launched ? 1LL : 0LL};
    for (int i = 0; i < n_info && i < 5; ++i) info[i] = vals[i];
    return FLR_OK;
}

const unsigned *flr_server_done_flags(const flr_server *sv) { return sv ? sv->h_done : nullptr; }

int flr_server_stop(flr_server *sv) {
    flr::set_last_error("");
    if (!sv) return fail(FLR_E_INVALID_ARGUMENT, "server must not be NULL");
    __atomic_store_n(sv->h_stop, 1, __ATOMIC_RELEASE);
    if (sv->launched) {
        const cudaError_t err = cudaEventSynchronize(sv->ran);
        sv->launched = false;
        if (err != cudaSuccess) return cuda_fail(err, "waiting for the serving kernel");
    }
    return FLR_OK;
}

int flr_server_destroy(flr_server *sv) {
    if (!sv) return FLR_OK;
    if (sv->h_block) {
        __atomic_store_n(sv->h_stop, 1, __ATOMIC_RELEASE);
        if (sv->launched) cudaEventSynchronize(sv->ran);
    }
    if (sv->ran) cudaEventDestroy(sv->ran);
    if (sv->d_next) cudaFree(sv->d_next);
    if (sv->d_tiles_done) cudaFree(sv->d_tiles_done);
    if (sv->h_block) cudaFreeHost(sv->h_block);
    delete sv;
    return FLR_OK;
}

}  // extern "C"
