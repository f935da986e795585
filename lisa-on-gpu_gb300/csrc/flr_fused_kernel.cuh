// Batched, fused response + TDI (sm_103a): one persistent launch over the
// flattened (source, tile) items of a batch, resolved on the device from
// per-source tile prefix sums (no work list is uploaded).
//
// A work item is T consecutive output samples [o0, o1) of one source.  The CTA
//   1. finds the input window its link streams need (geometry at the two ends
//      of the stream range), and stages it into shared memory with one 1-D
//      bulk copy (cp.async.bulk, mbarrier completion, bounded wait);
//   2. computes the six link streams y for [o0 - halo, o1 + halo) into shared
//      memory: one (receiving spacecraft, sample) per thread iteration, or,
//      on equal arms, three lanes per sample sharing the emitter sides by
//      warp shuffles (one (link, sample) per iteration for other link tables);
//   3. computes the TDI channels of [o0, o1) from those streams (one output
//      sample, all units of all channels, per thread iteration; in the mixed
//      flavour on equal arms, units of equal delay evaluated as groups over
//      signed link-row combinations) and writes X/Y/Z (or A/E/T, A/E) to
//      global memory.
// The link streams never touch HBM: per output sample the kernel reads 16 B
// of input and writes 24 B (plus the halos).
//
// Two arithmetic flavours share this structure:
//   exact: every interpolation, geometry and index operation is the plain
//          path's (flr_device.cuh): outputs are bit-identical to the reference's
//          CPU arithmetic.  Bound by the FP64 pipe.
//   mixed: delays, their integer/fractional split, orbit interpolation and TDI
//          delay sums in FP64 with the same operation order (integer indices
//          bit-exact); the Lagrange taps, weights and projections in
//          double-float arithmetic (flr_df.cuh) on the FP32 pipe, with the tile's
//          input scaled by a power of two near 1/max|h|.  The link response is
//          formed by summation by parts, sum_k W_k x_k =
//          P_b x_b - sum_{k<b} P_k (x_{k+1} - x_k) with P the running weight
//          sums, so the cancellation between the emitter and receiver terms
//          happens on first differences of the input instead of on the input.
//
// Compiled with --fmad=false (required by both flavours).
//
// This header holds the device code; flr_fused.cu instantiates the FP64 and
// the double-float mixed kernels and dispatches launches, flr_fused_d2.cu the
// mixed kernels in difference form (compiled in parallel).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "flr_df.cuh"
#include "flr_device.cuh"
#include "flr_fused.h"
#include "flr_gbwave.cuh"

namespace flr {
namespace {

constexpr int kThreads = kFusedThreads;
constexpr int kWindowMargin = 4;  // samples added on each side of the window estimate

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000ll); }

// ------------------------------------------------------------ bulk copy ----

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared; src and dst 16-byte aligned, bytes a
// multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes,
                                              uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the bulk copy of the current phase (at most `polls`
// try_wait polls); true when it completed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, long polls) {
    for (long it = 0; it < polls; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ------------------------------------------------------- shared layout ----

struct Layout {
    size_t set, edf, hraw, hdf, dh, y, d2, total;
};

__host__ __device__ constexpr size_t align128(size_t x) { return (x + 127) & ~size_t(127); }

__host__ __device__ inline Layout layout(bool mixed, int win_max, int y_max) {
    Layout L{};
    size_t off = 640;  // mbarrier, scale, warp maxima, segment cache, window ends, source copy
    L.set = off;
    off = align128(off + sizeof(FusedTdiSet));
    L.edf = off;
    off = align128(off + sizeof(df::f2) * kFusedMaxH);
    if (mixed) {
        // the raw window is read only until its double-float copy and
        // differences exist, before the link stage writes its rows: it shares
        // their space; the TDI stage's second differences (6 * y_max floats
        // <= win_max * 32 bytes, since win_max >= y_max) and weight tables
        // then take the space of the window's copies
        L.hdf = off;
        off = align128(off + sizeof(float4) * (size_t)win_max);
        L.dh = off;
        off = align128(off + sizeof(float4) * (size_t)win_max);
        L.y = off;
        L.hraw = off;
        const size_t rows = sizeof(float2) * 6 * (size_t)y_max;
        const size_t raw = sizeof(double2) * (size_t)win_max;
        off = align128(off + (rows > raw ? rows : raw));
        L.d2 = L.hdf;
    } else {
        L.hraw = off;
        off = align128(off + sizeof(double2) * (size_t)win_max);
        L.hdf = L.dh = 0;
        L.y = off;
        off = align128(off + sizeof(double) * 6 * (size_t)y_max);
        L.d2 = L.hraw;
    }
    L.total = off;
    return L;
}

// ------------------------------------------------- mixed-path geometry ----

// Segment index of the orbit grid found by multiplication with 1/dt; equal to
// orbit_segment()'s (int)(t / dt) because the two quotients differ by a few
// ulp and the exact division is used whenever t/dt is that close to an
// integer.
__device__ __forceinline__ int orbit_segment_fast(const OrbitTables &o, double inv_dt, double t) {
    double q = t * inv_dt;
    double r = rint(q);
    int w = (fabs(q - r) <= 1e-9 * fmax(1.0, fabs(q))) ? (int)(t / o.dt) : (int)q;
    if (w < 0 || w > o.N - 1) return -1;
    return (w == o.N - 1) ? o.N - 2 : w;
}

// Orbit segments of one work item's times, decided from the bits of t (a
// positive double orders like its bit pattern): the item's times fall in at
// most three consecutive segments w0 .. w0 + 2; a time farther than 1e-12
// (relative) from their bounds is in segment w0 + (t >= b1) + (t >= b2),
// which is the exact (int)(t / dt) (the quotient is then at least 1e-12 w0
// from an integer, far more than its rounding); other times take the exact
// lookup.  base[k] = dt * (w0 + k), the product orbit_lerp forms, so lerps
// from it give the same bits.  The cache saves the FP64 pipe the segment
// search and that product (GB300's FP64 pipe is the mixed kernel's busiest).
struct SegCache {
    long long lo, hi, g1lo, g1hi, g2lo, g2hi;
    double base[3];
    int w0;  // -1: not usable (every lookup exact)
};

struct Seg {
    int w;        // segment, -1 outside the table
    double base;  // dt * w
};

__device__ __forceinline__ void seg_cache_setup(SegCache *c, const OrbitTables &o,
                                                double inv_dt, double t_lo, double t_hi) {
    c->w0 = -1;
    if (!(t_lo > 0.0)) return;
    const int w0 = orbit_segment_fast(o, inv_dt, t_lo);
    if (w0 < 1 || w0 + 2 > o.N - 2) return;
    const double b0 = o.dt * (double)w0, b1 = o.dt * (double)(w0 + 1),
                 b2 = o.dt * (double)(w0 + 2), b3 = o.dt * (double)(w0 + 3);
    if (!(t_hi < b3)) return;
    const double m = 1e-12;
    c->lo = __double_as_longlong(b0 * (1.0 + m));
    c->hi = __double_as_longlong(b3 * (1.0 - m));
    c->g1lo = __double_as_longlong(b1 * (1.0 - m));
    c->g1hi = __double_as_longlong(b1 * (1.0 + m));
    c->g2lo = __double_as_longlong(b2 * (1.0 - m));
    c->g2hi = __double_as_longlong(b2 * (1.0 + m));
    c->base[0] = b0;
    c->base[1] = b1;
    c->base[2] = b2;
    c->w0 = w0;
}

__device__ __forceinline__ Seg seg_of(const SegCache *c, const OrbitTables &o, double inv_dt,
                                      double t) {
    const long long b = __double_as_longlong(t);
    const int w0 = c->w0;
    if (w0 >= 0 && b > c->lo && b < c->hi && (b <= c->g1lo || b >= c->g1hi) &&
        (b <= c->g2lo || b >= c->g2hi)) {
        const int k = (int)(b >= c->g1hi) + (int)(b >= c->g2hi);
        return {w0 + k, c->base[k]};
    }
    const int w = orbit_segment_fast(o, inv_dt, t);
    return {w, (w < 0) ? 0.0 : o.dt * (double)w};
}

// orbit_lerp with the segment's base time given: m (t - base) + lo
__device__ __forceinline__ double orbit_lerp_b(const double *tab, const double *slope, int w,
                                               int stride, int col, double t, double base) {
    const double lo = __ldg(tab + (size_t)w * stride + col);
    const double m = __ldg(slope + (size_t)w * stride + col);
    return m * (t - base) + lo;
}

__device__ __forceinline__ void position_sb(const OrbitTables &o, Seg g, double t, int sc,
                                            double out[3]) {
    const int s = (sc >= 1 && sc <= 3) ? sc - 1 : -1;
    if (g.w < 0 || s < 0) {
        out[0] = out[1] = out[2] = 0.0;
        return;
    }
    const double dt_w = t - g.base;
#pragma unroll
    for (int c = 0; c < 3; ++c)
        out[c] = __ldg(o.x_slope + (size_t)g.w * 9 + 3 * s + c) * dt_w +
                 __ldg(o.x + (size_t)g.w * 9 + 3 * s + c);
}

__device__ __forceinline__ void position_seg(const OrbitTables &o, int w, double t, int sc,
                                             double out[3]) {
    int s = (sc >= 1 && sc <= 3) ? sc - 1 : -1;
    if (w < 0 || s < 0) {
        out[0] = out[1] = out[2] = 0.0;
        return;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) out[c] = orbit_lerp(o.x, o.x_slope, w, 9, 3 * s + c, t, o.dt);
}

// K * 2^-fb as a df value, for 0 < K < 2^fb and 22 <= fb <= 52: the floats
// are assembled from the bits of K (hi = its top 24 significant bits, lo the
// rest, truncated to 24 bits), so no FP64 or conversion instruction is used.
// Exact when K has at most 48 significant bits.
__device__ __forceinline__ df::f2 df_from_fixed(unsigned long long K, int fb) {
    const int len = 64 - __clzll((long long)K);  // 1..52
    const int sh = len - 24;
    const unsigned long long top = (sh >= 0) ? (K >> sh) : (K << -sh);
    const float hi = __int_as_float(((len - 1 - fb + 127) << 23) | (int)(top & 0x7fffffu));
    float lo = 0.f;
    if (sh > 0) {
        const unsigned long long rest = K & ((1ull << sh) - 1);
        if (rest != 0) {
            const int len2 = 64 - __clzll((long long)rest);
            const int sh2 = len2 - 24;
            const unsigned long long top2 = (sh2 >= 0) ? (rest >> sh2) : (rest << -sh2);
            lo = __int_as_float(((len2 - 1 - fb + 127) << 23) | (int)(top2 & 0x7fffffu));
        }
    }
    return {hi, lo};
}

// The mixed flavour's index split.  The reference's (LISAResponse.cu:339-341,
// 616-622) is d = (int)ceil(x) - 1, eps = (1 + d) - x for x = (t - t0) * fs,
// x computed in FP64 with the same operations; (1 + d) - x is exact, so eps is
// determined by the bits of x.  For 1 <= x < 2^31 the integer and fractional
// parts are read from those bits (x = (m >> fb) + (m & (2^fb - 1)) 2^-fb for
// the significand m and fb = 52 - exponent): the same d and the same value of
// eps, as a df, without FP64 conversions.  Other x take the FP64 route, the
// ceiling as a round-up conversion ((double)(d + 1) equals 1.0 + d).
// kT0Zero: t_first is +0 (every source of the launch starts at t0 = +0), and
// delayed_t - (+0) is delayed_t for every double, so the subtraction is left
// out: the same x with one FP64 operation fewer.
template <bool kT0Zero = false>
__device__ __forceinline__ void split_delay_df(double delayed_t, double t_first, double fs,
                                               int &d, df::f2 &eps) {
    const double x = (kT0Zero ? delayed_t : delayed_t - t_first) * fs;
    const long long b = __double_as_longlong(x);
    const int e = (int)(b >> 52) - 1023;  // negative x: e < -1023
    if (e >= 0 && e <= 30) {
        const int fb = 52 - e;
        const unsigned long long m = ((unsigned long long)b & 0xfffffffffffffull) | (1ull << 52);
        const unsigned long long frac = m & ((1ull << fb) - 1);
        const int ip = (int)(m >> fb);
        if (frac != 0) {
            d = ip;
            eps = df_from_fixed((1ull << fb) - frac, fb);
        } else {
            d = ip - 1;
            eps = {0.f, 0.f};
        }
        return;
    }
    const int c = __double2int_ru(x);
    d = c - 1;
    eps = df::from_double((double)c - x);
}

// k . x for a delay: ((a0 b0) + a1 b1) + a2 b2.  The reference's
// dot_product_1d (LISAResponse.cu:48-57) starts from 0 + a0 b0, which differs
// from a0 b0 only when a0 b0 is -0; the two sums then differ at most in the
// sign of a zero result, and t - (+-0) C^-1 is the same delayed time, so the
// index split gets the same bits with one FP64 addition fewer.
__device__ __forceinline__ double dot3_delay(const double *a, const double *b) {
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

// t0 + j dt, the reference's sample time; kT0Zero: t0 is +0 and j dt (never
// -0) is the sum's exact value.
template <bool kT0Zero>
__device__ __forceinline__ double sample_time(double t0, long long j, double dt) {
    return kT0Zero ? exact_double_of(j) * dt : t0 + exact_double_of(j) * dt;
}

struct MixedDelays {
    int d_rec, d_em;
    df::f2 e_rec, e_em;
    double x_rec[3], x_em[3];
};

// Receiver/emitter delays exactly as link_geometry() computes them (same
// operations, same order, so the integer indices are bit-identical), plus
// the spacecraft positions for the projection factors.
template <bool kT0Zero = false>
__device__ __forceinline__ MixedDelays link_delays_mixed(const OrbitTables &o, double inv_dt,
                                                         int slot, double t, double t_first,
                                                         double fs, const double k[3]) {
    MixedDelays g;
    int w = orbit_segment_fast(o, inv_dt, t);
    double L = (w < 0) ? 0.0 : orbit_lerp(o.ltt, o.ltt_slope, w, 6, slot, t, o.dt);
    double t_em = t - L;
    position_seg(o, w, t, o.sc_r[slot], g.x_rec);
    position_seg(o, orbit_segment_fast(o, inv_dt, t_em), t_em, o.sc_e[slot], g.x_em);
    double kx_rec = dot3_delay(k, g.x_rec);
    double kx_em = dot3_delay(k, g.x_em);
    split_delay_df<kT0Zero>(t - kx_rec * kCInv, t_first, fs, g.d_rec, g.e_rec);
    split_delay_df<kT0Zero>(t_em - kx_em * kCInv, t_first, fs, g.d_em, g.e_em);
    return g;
}

// The receiver side of link_delays_mixed(), shared by the two links a
// spacecraft receives: its position at t and the receiver delay's split
// (same operations as there, so the same bits).
struct ReceiverSide {
    Seg w;  // orbit segment of t
    int d_rec;
    df::f2 e_rec;
    double x_rec[3];
};

template <bool kT0Zero = false>
__device__ __forceinline__ ReceiverSide receiver_mixed(const OrbitTables &o, double inv_dt, int sc,
                                                       double t, double t_first, double fs,
                                                       const double k[3], const SegCache *sc_) {
    ReceiverSide r;
    r.w = seg_of(sc_, o, inv_dt, t);
    position_sb(o, r.w, t, sc, r.x_rec);
    split_delay_df<kT0Zero>(t - dot3_delay(k, r.x_rec) * kCInv, t_first, fs, r.d_rec, r.e_rec);
    return r;
}

// The emitter side of link_delays_mixed() for link `slot` given the segment
// of t: t_em = t - L(t), the emitter position at t_em and its delay's split.
struct EmitterSide {
    int d_em;
    df::f2 e_em;
    double x_em[3];
};

template <bool kT0Zero = false>
__device__ __forceinline__ EmitterSide emitter_mixed(const OrbitTables &o, double inv_dt, int slot,
                                                     Seg w, double t, double t_first, double fs,
                                                     const double k[3], const SegCache *sc_) {
    EmitterSide e;
    const double L =
        (w.w < 0) ? 0.0 : orbit_lerp_b(o.ltt, o.ltt_slope, w.w, 6, slot, t, w.base);
    const double t_em = t - L;
    position_sb(o, seg_of(sc_, o, inv_dt, t_em), t_em, o.sc_e[slot], e.x_em);
    split_delay_df<kT0Zero>(t_em - dot3_delay(k, e.x_em) * kCInv, t_first, fs, e.d_em, e.e_em);
    return e;
}

// The exact flavour's link geometry split into its receiver side (shared by
// the two links a spacecraft receives) and its emitter side: the operations
// of link_geometry() in the same order, so the same bits.
struct ReceiverF64 {
    int d_rec;
    double e_rec;
    double x_rec[3];
};

__device__ __forceinline__ ReceiverF64 receiver_f64(const OrbitTables &o, int sc, double t,
                                                    double t_first, double fs,
                                                    const double k[3]) {
    ReceiverF64 r;
    position(o, t, sc, r.x_rec);
    const double kx_rec = dot3(k, r.x_rec);
    const double delay_rec = t - kx_rec * kCInv;
    split_delay(delay_rec, t_first, fs, r.d_rec, r.e_rec);
    return r;
}

struct EmitterF64 {
    int d_em;
    double e_em;
    double xi_p, xi_c, k_dot_n;
};

// Polarisation projections and k.n of one link, n = (x_rec - x_em)/|x_rec - x_em|
// (link_geometry()'s operations in its order).
__device__ __forceinline__ void link_projection_f64(const double x_rec[3], const double x_em[3],
                                                    const double k[3], const double u[3],
                                                    const double v[3], double &xi_p,
                                                    double &xi_c, double &k_dot_n) {
    double n[3];
    double norm = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        n[c] = x_rec[c] - x_em[c];
        norm += n[c] * n[c];
    }
    norm = sqrt(norm);
#pragma unroll
    for (int c = 0; c < 3; ++c) n[c] = n[c] / norm;
    const double un = dot3(u, n), vn = dot3(v, n);
    xi_p = 0.5 * ((un * un) - (vn * vn));
    xi_c = un * vn;
    k_dot_n = dot3(k, n);
}

// Emission time, position and index split of spacecraft sc's side of a link
// with light travel time L (the emitter half of link_geometry()).
__device__ __forceinline__ void emitter_side_f64(const OrbitTables &o, int sc, double t, double L,
                                                 double t_first, double fs, const double k[3],
                                                 double x_em[3], int &d_em, double &e_em) {
    const double t_em = t - L;
    position(o, t_em, sc, x_em);
    const double kx_em = dot3(k, x_em);
    const double delay_em = t_em - kx_em * kCInv;
    split_delay(delay_em, t_first, fs, d_em, e_em);
}

__device__ __forceinline__ EmitterF64 emitter_f64(const OrbitTables &o, int slot, double t,
                                                  const double x_rec[3], double t_first,
                                                  double fs, const double k[3],
                                                  const double u[3], const double v[3]) {
    EmitterF64 e;
    double x_em[3];
    emitter_side_f64(o, o.sc_e[slot], t, light_travel_time(o, t, slot), t_first, fs, k, x_em,
                     e.d_em, e.e_em);
    link_projection_f64(x_rec, x_em, k, u, v, e.xi_p, e.xi_c, e.k_dot_n);
    return e;
}

// Exact complex interpolation at (d, eps) from the staged raw window when its
// taps lie in it, else from global memory (the same values); false when the
// taps leave the input.
__device__ __forceinline__ bool c128_any(const double2 *hraw, long wlo, int W, const HSrc &hg,
                                         long n, int d, double eps, double A,
                                         const LagrangeTables &lt, double &hp, double &hc) {
    const long lo = (long)d - (lt.h - 1), hi = (long)d + lt.h;
    if (lo >= wlo && hi < wlo + W) {
        lagrange_c128(SharedC128{hraw}, (int)(d - wlo), eps, A, lt, hp, hc);
        return true;
    }
    if (lo >= 0 && hi < n) {
        lagrange_c128(hg, d, eps, A, lt, hp, hc);
        return true;
    }
    return false;
}

// 1/sqrt(x) in df: hardware approximation and one Newton step,
// r = r0 + r0 (1 - x r0^2) / 2; relative error ~1e-14.
__device__ __forceinline__ df::f2 df_rsqrt(df::f2 x) {
    float r0;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(x.hi));
    const df::f2 xr2 = df::mul_raw(x, df::two_prod(r0, r0));
    const float t = (1.0f - xr2.hi) - xr2.lo;
    return df::fast_two_sum(r0, r0 * 0.5f * t);
}

__device__ __forceinline__ df::f2 df_dot3(const df::f2 a[3], const df::f2 b[3]) {
    return df::add(df::add(df::mul(a[0], b[0]), df::mul(a[1], b[1])), df::mul(a[2], b[2]));
}

struct DfProjection {
    df::f2 xi_p, xi_c, pre;  // polarisation projections and 1 / (1 - k.n)
};

// Projection factors of one link (LISAResponse.cu:581-606, 664) in df from the
// FP64 spacecraft positions: n = (x_rec - x_em) / |x_rec - x_em|,
// xi+ = ((u.n)^2 - (v.n)^2) / 2, xix = (u.n)(v.n), 1 / (1 - k.n).
__device__ __forceinline__ DfProjection df_projection_of(df::f2 n[3], const df::f2 k[3],
                                                         const df::f2 u[3], const df::f2 v[3]);

__device__ __forceinline__ DfProjection df_projection(const double x_rec[3], const double x_em[3],
                                                      const df::f2 k[3], const df::f2 u[3],
                                                      const df::f2 v[3]) {
    df::f2 n[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) n[c] = df::from_double_bits(x_rec[c] - x_em[c]);
    return df_projection_of(n, k, u, v);
}

// The same from double-float positions: the link vector as a double-float
// difference (~1e-13 of it, where the projection factors need ~1e-11), which
// takes three FP64 subtractions per link off the FP64 pipe.
__device__ __forceinline__ DfProjection df_projection_df(const df::f2 x_rec[3],
                                                         const df::f2 x_em[3], const df::f2 k[3],
                                                         const df::f2 u[3], const df::f2 v[3]) {
    df::f2 n[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) n[c] = df::sub(x_rec[c], x_em[c]);
    return df_projection_of(n, k, u, v);
}

// n: the link vector x_rec - x_em (overwritten)
__device__ __forceinline__ DfProjection df_projection_of(df::f2 n[3], const df::f2 k[3],
                                                         const df::f2 u[3], const df::f2 v[3]) {
    const df::f2 r = df_rsqrt(df_dot3(n, n));
#pragma unroll
    for (int c = 0; c < 3; ++c) n[c] = df::mul(n[c], r);
    const df::f2 un = df_dot3(u, n), vn = df_dot3(v, n), kn = df_dot3(k, n);
    DfProjection p;
    const df::f2 d = df::sub(df::mul(un, un), df::mul(vn, vn));
    p.xi_p = {0.5f * d.hi, 0.5f * d.lo};
    p.xi_c = df::mul(un, vn);
    p.pre = df::renorm(df::rcp(df::sub({1.0f, 0.0f}, kn)));
    return p;
}

// A(eps) from the df table: q = eps / deps, A = A[ind] + (q - ind) (A[ind+1] - A[ind]),
// the reference's lerp (LISAResponse.cu:114-117) rearranged; differs from it
// by rounding only.
__device__ __forceinline__ df::f2 prefactor_df(const float4 *tab, int num_A, df::f2 inv_deps,
                                               df::f2 e) {
    // normalised, so that |q.lo| <= ulp(q.hi) / 2 and floor(q.hi) (corrected
    // below when q.hi is a knot) is the segment of q itself: a q.hi a few
    // ulp under a knot would pick the previous segment and extrapolate it
    const df::f2 q = df::renorm(df::mul_raw(e, inv_deps));
    const float fl = floorf(q.hi);
    int ind = (int)fl;
    if (q.hi == fl && q.lo < 0.f) ind -= 1;
    ind = min(max(ind, 0), num_A - 2);
    const df::f2 frac = df::fast_two_sum(q.hi - (float)ind, q.lo);
    const float4 t = __ldg(tab + ind);
    // A >= 1 and the segment's change is ~1e-3 of it: no cancellation
    return df::add_raw({t.x, t.y}, df::mul_raw(frac, {t.z, t.w}));
}

// --------------------------------------------- double-float interpolation ----

// Tap weights of the reference's kernel (interp, LISAResponse.cu:149-207):
// W_{d+1} = A(1-e), W_d = A e, W_{d+1+j} = A e(1-e) E_j/(j+e),
// W_{d-j} = A e(1-e) E_j/(j+1-e), j = 1..h-1.
struct DfWeights {
    df::f2 A, e, ome, c;  // A, eps, 1 - eps, A eps (1 - eps)
};

__device__ __forceinline__ DfWeights df_weights(df::f2 A, df::f2 e) {
    DfWeights w;
    w.A = A;
    w.e = e;
    w.ome = df::one_minus(e);
    w.c = df::mul(df::mul(A, e), w.ome);
    return w;
}

// j: the tap's distance as a float (exact)
__device__ __forceinline__ df::f2 df_tail_up(const DfWeights &w, df::f2 Ej, float j) {
    return df::div_raw(df::mul_raw(w.c, Ej), df::add_big_float(j, w.e));
}

__device__ __forceinline__ df::f2 df_tail_dn(const DfWeights &w, df::f2 Ej, float j) {
    return df::div_raw(df::mul_raw(w.c, Ej), df::add_big_float(j, w.ome));
}

// Shared-memory df views of the staged input: value and first difference.
struct DfShared {
    using index_t = int;  // window offsets: 32-bit shared-memory addressing
    const float4 *x;      // (re_hi, re_lo, im_hi, im_lo)
    const float4 *dx;     // x[k+1] - x[k]
    __device__ __forceinline__ float4 val(int k) const { return x[k]; }
    __device__ __forceinline__ float4 diff(int k) const { return dx[k]; }
};

// The same views computed on the fly from global memory (used when a tap
// window falls outside the staged window).
struct DfGlobal {
    using index_t = long;
    HSrc h;
    double scale;
    __device__ __forceinline__ float4 val(long k) const {
        double2 v = h[k];
        df::f2 r = df::from_double(v.x * scale), i = df::from_double(v.y * scale);
        return make_float4(r.hi, r.lo, i.hi, i.lo);
    }
    __device__ __forceinline__ float4 diff(long k) const {
        double2 a = h[k], b = h[k + 1];
        df::f2 r = df::from_double((b.x - a.x) * scale), i = df::from_double((b.y - a.y) * scale);
        return make_float4(r.hi, r.lo, i.hi, i.lo);
    }
};

// Complex interpolation around sample d of the source, by summation by parts.
template <class Src>
__device__ __forceinline__ void df_interp_c128_sbp(const Src &src, typename Src::index_t d,
                                                   df::f2 A, df::f2 eps,
                                                   const df::f2 *edf, int h, df::f2 &re,
                                                   df::f2 &im) {
    const DfWeights w = df_weights(A, eps);
    df::f2 P = {0.f, 0.f};
    df::Acc sre, sim;
    df::acc_init(sre);
    df::acc_init(sim);
    using index_t = typename Src::index_t;
    auto step = [&](df::f2 W, index_t k) {
        P = df::add(P, W);
        float4 dx = src.diff(k);
        df::acc_fma(sre, P, {dx.x, dx.y});
        df::acc_fma(sim, P, {dx.z, dx.w});
    };
    {  // taps d - (h - 1) .. d - 1, j = h - 1 .. 1
        const df::f2 *Ej = edf + h - 2;
        float jf = (float)(h - 1);
        for (index_t k = d - (h - 1); k < d; ++k, --Ej, jf -= 1.f)
            step(df_tail_dn(w, *Ej, jf), k);
    }
    step(df::mul_raw(w.A, w.e), d);
    df::f2 W_last;
    index_t last;
    if (h == 1) {
        W_last = df::mul_raw(w.A, w.ome);
        last = d + 1;
    } else {
        step(df::mul_raw(w.A, w.ome), d + 1);
        const df::f2 *Ej = edf;  // taps d + 2 .. d + h - 1, j = 1 .. h - 2
        float jf = 1.f;
        for (index_t k = d + 2; k < d + h; ++k, ++Ej, jf += 1.f) step(df_tail_up(w, *Ej, jf), k);
        W_last = df_tail_up(w, edf[h - 2], (float)(h - 1));
        last = d + h;
    }
    P = df::add(P, W_last);
    float4 xb = src.val(last);
    re = df::sub(df::mul(P, {xb.x, xb.y}), df::acc_value(sre));
    im = df::sub(df::mul(P, {xb.z, xb.w}), df::acc_value(sim));
}

// Complex interpolation at (d, eps) from the staged window when its taps lie
// in it, else from global memory (the same df values); false when the taps
// leave the input.
__device__ __forceinline__ bool df_interp_c128_any(const float4 *hdf, const float4 *dh, long wlo,
                                                   int W, const HSrc &hg, double scale, long n,
                                                   int d, df::f2 A, df::f2 eps, const df::f2 *edf,
                                                   int h, df::f2 &re, df::f2 &im) {
    const long lo = (long)d - (h - 1), hi = (long)d + h;
    if (lo >= wlo && hi + 1 < wlo + W) {
        df_interp_c128_sbp(DfShared{hdf, dh}, (int)(d - wlo), A, eps, edf, h, re, im);
        return true;
    }
    if (lo >= 0 && hi + 1 < n) {
        df_interp_c128_sbp(DfGlobal{hg, scale}, d, A, eps, edf, h, re, im);
        return true;
    }
    return false;
}

// Real interpolation around sample d of a staged df link row, compensated dot
// products (Dot2).  The common factor c = A eps (1 - eps) of the outer taps
// is applied once to their sum, sum_j E_j (y_up/(j + eps) + y_dn/(j + 1 - eps)),
// whose terms are df quotients: per tap one division instead of a reciprocal
// and two products.
__device__ __forceinline__ df::f2 df_interp_real(const float2 *y, int d, df::f2 A, df::f2 eps,
                                                 const df::f2 *edf, int h, int h_df) {
    const DfWeights w = df_weights(A, eps);
    df::Acc acc, tail;
    df::acc_init(acc);
    df::acc_init(tail);
    float2 v = y[d + 1];
    df::acc_fma(acc, df::mul_raw(w.A, w.ome), {v.x, v.y});
    v = y[d];
    df::acc_fma(acc, df::mul_raw(w.A, w.e), {v.x, v.y});
    // taps j = 1 .. h_df - 1 at y[d + 1 + j] and y[d - j]; running pointers and
    // a float copy of j (exact) keep the loop free of index arithmetic
    const float2 *up = y + d + 2, *dn = y + d - 1;
    const df::f2 *Ej = edf;
    float jf = 1.f;
    for (int j = 1; j < h_df; ++j, ++up, --dn, ++Ej, jf += 1.f) {
        const float2 u = *up, v = *dn;
        df::acc_fma(tail, df::div_raw(*Ej, df::add_big_float(jf, w.e)), {u.x, u.y});
        df::acc_fma(tail, df::div_raw(*Ej, df::add_big_float(jf, w.ome)), {v.x, v.y});
    }
    // outer taps (j >= h_df, smallest first): weights E_j / (j + eps) small
    // enough that FP32 products and sums stay far below the df error budget
    float outer = 0.f;
    up = y + d + h;
    dn = y + d + 1 - h;
    Ej = edf + h - 2;
    jf = (float)(h - 1);
    for (int j = h - 1; j >= h_df; --j, --up, ++dn, --Ej, jf -= 1.f) {
        outer = __fmaf_rn(Ej->hi * df::rcp_approx(jf + w.e.hi), up->x, outer);
        outer = __fmaf_rn(Ej->hi * df::rcp_approx(jf + w.ome.hi), dn->x, outer);
    }
    df::acc_add(tail, {outer, 0.f});
    df::acc_add(acc, df::mul(w.c, df::acc_value(tail)));
    return df::acc_value(acc);
}

// Output sample i of the channels: X, Y, Z or lisaanalysistools' AET,
// (Z-X)/sqrt2, (X-2Y+Z)/sqrt6, (X+Y+Z)/sqrt3 (AE: a zero third row).
__device__ __forceinline__ void store_channels(double *out, long n, long i, int chan, double X,
                                               double Yc, double Z) {
    if (chan == kChanXYZ) {
        out[i] = X;
        out[n + i] = Yc;
        out[2 * n + i] = Z;
    } else {
        out[i] = (Z - X) / 1.4142135623730951;
        out[n + i] = (X - 2.0 * Yc + Z) / 2.449489742783178;
        out[2 * n + i] = (chan == kChanAET) ? (X + Yc + Z) / 1.7320508075688772 : 0.0;
    }
}

// Inner-product form of store_channels: the same channel values, added to
// lk[c] += value_c * data_c[i] and lk[3 + c] += value_c^2.
__device__ __forceinline__ void add_inner(double lk[6], const double *data, long n, long i,
                                          int chan, double X, double Yc, double Z) {
    double c0, c1, c2;
    if (chan == kChanXYZ) {
        c0 = X;
        c1 = Yc;
        c2 = Z;
    } else {
        c0 = (Z - X) / 1.4142135623730951;
        c1 = (X - 2.0 * Yc + Z) / 2.449489742783178;
        c2 = (chan == kChanAET) ? (X + Yc + Z) / 1.7320508075688772 : 0.0;
    }
    lk[0] += c0 * data[i];
    lk[1] += c1 * data[n + i];
    lk[2] += c2 * data[2 * n + i];
    lk[3] += c0 * c0;
    lk[4] += c1 * c1;
    lk[5] += c2 * c2;
}

// Grouped real interpolation: for each channel c the interpolation at one
// delay (d, eps) of the virtual row at shared offset off[c], times sg[c]
// (+-1; 0: the channel has no term here); the weights are computed once for
// the three channels.
__device__ __forceinline__ void df_interp_group(const float2 *y, const int off[3],
                                                const float sg[3], int d, df::f2 A, df::f2 eps,
                                                const df::f2 *edf, int h, int h_df,
                                                df::f2 out[3]) {
    const DfWeights w = df_weights(A, eps);
    // per channel: its virtual row around sample d; taps at row[k], k relative to d
    const float2 *row[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) row[c] = y + off[c] + d;
    df::Acc acc[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) df::acc_init(acc[c]);
    auto tap = [&](df::f2 W, int k) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 v = row[c][k];
            df::acc_fma(acc[c], W, {v.x, v.y});
        }
    };
    tap(df::mul_raw(w.A, w.ome), 1);
    tap(df::mul_raw(w.A, w.e), 0);
    const df::f2 *Ej = edf;
    float jf = 1.f;  // j as a float (exact)
    for (int j = 1; j < h_df; ++j, ++Ej, jf += 1.f) {
        const df::f2 cE = df::mul_raw(w.c, *Ej);  // unnormalised: mul_raw accepts it
        tap(df::div_raw(cE, df::add_big_float(jf, w.e)), 1 + j);
        tap(df::div_raw(cE, df::add_big_float(jf, w.ome)), -j);
    }
    // outer taps in FP32, smallest first (see df_interp_real)
    float outer[3] = {0.f, 0.f, 0.f};
    jf = (float)(h - 1);
    Ej = edf + h - 2;
    for (int j = h - 1; j >= h_df; --j, --Ej, jf -= 1.f) {
        const float cE = w.c.hi * Ej->hi;
        const float wu = cE * df::rcp_approx(jf + w.e.hi);
        const float wd = cE * df::rcp_approx(jf + w.ome.hi);
#pragma unroll
        for (int c = 0; c < 3; ++c)
            outer[c] = __fmaf_rn(wd, row[c][-j].x, __fmaf_rn(wu, row[c][1 + j].x, outer[c]));
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) df::acc_add(acc[c], {outer[c], 0.f});
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const df::f2 v = df::acc_value(acc[c]);
        out[c] = (sg[c] == 0.f) ? df::f2{0.f, 0.f} : df::f2{sg[c] * v.hi, sg[c] * v.lo};
    }
}

// ------------------------------------------- second-difference TDI form ----
//
// The reference's weights (interp_single, LISAResponse.cu:110-147) are
// W_k = A(eps) w_k with w_{d+1} = 1 - eps, w_d = eps, w_{d+1+j} = eps (1 - eps)
// E_j / (j + eps), w_{d-j} = eps (1 - eps) E_j / (j + 1 - eps), A the
// linearly interpolated table.  The unnormalised weights of Lagrange
// interpolation reproduce polynomials of degree < 2h: sum w_k = 1 / A_exact(eps)
// and sum k w_k = (1 - eps) / A_exact(eps) relative to d.  Writing each tap as
// the linear model through y_d, y_{d+1} plus a remainder that summation by
// parts (twice, from each end towards the centre) turns into second
// differences D_i = y_{i+1} - 2 y_i + y_{i-1},
//   sum W_k y_k = S(eps) (eps y_d + (1 - eps) y_{d+1}) + A(eps) sum_i U_i D_i,
// S = A / A_exact = 1 + sigma(eps), U_i = sum_{k > i} (k - i) w_k right of the
// centre (i >= 1) and sum_{k < i} (i - k) w_k left of it (i <= 0).  The linear
// part is a double-float product; sigma comes from a per-segment polynomial of
// the plan; D and the sum run in FP32.  For the smooth link streams the second
// differences are ~(2 pi f dt)^2 of the values, so the FP32 part's error is
// ~1e-7 (2 pi f dt)^2 |y|, which grows with frequency like the TDI channels
// themselves (~f^2 of the links): a few 1e-8 of the channels at any f.

struct D2Weights {
    float u;        // position in the A-table segment, [0, 1)
    float A;        // A(eps) (FP32)
    float sigma;    // S - 1
};

__device__ __forceinline__ D2Weights d2_weights(const FusedArgs &a, df::f2 inv_deps, df::f2 e) {
    D2Weights w;
    const df::f2 q = df::renorm(df::mul_raw(e, inv_deps));
    const float fl = floorf(q.hi);
    int ind = (int)fl;
    if (q.hi == fl && q.lo < 0.f) ind -= 1;
    ind = min(max(ind, 0), a.lt.num_A - 2);
    w.u = (q.hi - (float)ind) + q.lo;
    const float4 t = __ldg(a.a_tab + ind);
    w.A = __fmaf_rn(w.u, t.z, t.x);
    const float4 c = __ldg(a.sig4 + ind);
    w.sigma = __fmaf_rn(
        __fmaf_rn(__fmaf_rn(__fmaf_rn(c.x, w.u, c.y), w.u, c.z), w.u, c.w), w.u,
        __ldg(a.sig0 + ind));
    return w;
}

// eps y_d + (1 - eps) y_{d+1} of a df row (both weights positive: no cancellation)
__device__ __forceinline__ df::f2 d2_linear(const float2 *y, int d, df::f2 e, df::f2 ome) {
    const float2 y0 = y[d], y1 = y[d + 1];
    return df::add_raw(df::mul_raw(e, {y0.x, y0.y}), df::mul_raw(ome, {y1.x, y1.y}));
}

// S l + A acc as a df value: l + (sigma l + A acc), the correction in FP32
__device__ __forceinline__ df::f2 d2_combine(df::f2 l, const D2Weights &w, float acc) {
    const float corr = __fmaf_rn(w.A, acc, w.sigma * l.hi);
    const df::f2 s = df::two_sum(l.hi, corr);
    return df::fast_two_sum(s.hi, s.lo + l.lo);
}

// Real interpolation of one df row (y) around sample d with its second
// differences dd.  edf: E_j (df; the FP32 part uses .hi).
__device__ __forceinline__ df::f2 d2_interp_real(const float2 *y, const float *dd, int d,
                                                 df::f2 e, const D2Weights &w,
                                                 const df::f2 *edf, int h) {
    const df::f2 ome = df::one_minus(e);
    const df::f2 l = d2_linear(y, d, e, ome);
    const float e32 = e.hi, o32 = ome.hi + ome.lo, c = e32 * o32;
    float R = 0.f, UR = 0.f, L = 0.f, UL = 0.f, acc = 0.f;
    const float *up = dd + d + h - 1;  // D_{d+j}, j = h-1 .. 1
    const float *dn = dd + d + 2 - h;  // D_{d+1-j}
    const df::f2 *Ej = edf + h - 2;
    float jf = (float)(h - 1);
    for (int j = h - 1; j >= 1; --j, --up, ++dn, --Ej, jf -= 1.f) {
        const float cE = c * Ej->hi;
        R = __fmaf_rn(cE, df::rcp_approx(jf + e32), R);  // + w_{d+1+j}
        UR += R;
        acc = __fmaf_rn(UR, *up, acc);
        L = __fmaf_rn(cE, df::rcp_approx(jf + o32), L);  // + w_{d-j}
        UL += L;
        acc = __fmaf_rn(UL, *dn, acc);
    }
    return d2_combine(l, w, acc);
}

// The partial sums (UR_j, UL_j), j = h-1 .. 1, of the grouped form's FP32
// remainder weights: functions of e32 (eps rounded to FP32) alone.
__device__ __forceinline__ void d2_group_sums(float e32, const df::f2 *edf, int h, float2 *tab) {
    const float o32 = 1.0f - e32, c = e32 * o32;
    float R = 0.f, UR = 0.f, L = 0.f, UL = 0.f;
    const df::f2 *Ej = edf + h - 2;
    float jf = (float)(h - 1);
    for (int j = h - 1; j >= 1; --j, --Ej, jf -= 1.f) {
        const float cE = c * Ej->hi;
        R = __fmaf_rn(cE, df::rcp_approx(jf + e32), R);
        UR += R;
        L = __fmaf_rn(cE, df::rcp_approx(jf + o32), L);
        UL += L;
        tab[h - 1 - j] = make_float2(UR, UL);
    }
}

// The grouped form: the same weights for the virtual rows of the three
// channels (offsets off[c] into y / dd, signs sg[c], 0 = no term).  tab: the
// partial sums of d2_group_sums for this e32 when the caller has them (the
// same values), else nullptr.  Adds each channel's signed linear part
// (double-float) to lin[c] and its signed FP32 correction A acc + sigma l to
// corr[c]: the caller sums the corrections of all groups in FP32 and adds
// them to the double-float sum of the linear parts once.
__device__ __forceinline__ void d2_interp_group(const float2 *y, const float *dd, const int off[3],
                                                const float sg[3], int d, df::f2 e,
                                                const D2Weights &w, const df::f2 *edf, int h,
                                                const float2 *tab, df::f2 lin[3], float corr[3]) {
    const df::f2 ome = df::one_minus(e);
    float acc[3] = {0.f, 0.f, 0.f};
    const float *up[3], *dn[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        up[k] = dd + off[k] + d + h - 1;
        dn[k] = dd + off[k] + d + 2 - h;
    }
    if (tab != nullptr) {
        for (int o = 0; o < h - 1; ++o) {
            const float2 u = tab[o];
#pragma unroll
            for (int k = 0; k < 3; ++k)
                acc[k] = __fmaf_rn(u.y, dn[k][o], __fmaf_rn(u.x, up[k][-o], acc[k]));
        }
    } else {
        const float e32 = e.hi, o32 = 1.0f - e32, c = e32 * o32;
        float R = 0.f, UR = 0.f, L = 0.f, UL = 0.f;
        const df::f2 *Ej = edf + h - 2;
        float jf = (float)(h - 1);
        for (int j = h - 1; j >= 1; --j, --Ej, jf -= 1.f) {
            const float cE = c * Ej->hi;
            R = __fmaf_rn(cE, df::rcp_approx(jf + e32), R);
            UR += R;
            L = __fmaf_rn(cE, df::rcp_approx(jf + o32), L);
            UL += L;
            const int o = h - 1 - j;
#pragma unroll
            for (int k = 0; k < 3; ++k)
                acc[k] = __fmaf_rn(UL, dn[k][o], __fmaf_rn(UR, up[k][-o], acc[k]));
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (sg[k] == 0.f) continue;
        const df::f2 l = d2_linear(y + off[k], d, e, ome);
        lin[k] = df::add(lin[k], {sg[k] * l.hi, sg[k] * l.lo});
        corr[k] = __fmaf_rn(sg[k], __fmaf_rn(w.A, acc[k], w.sigma * l.hi), corr[k]);
    }
}

// b - a of two df values, exactly up to the low parts' FP32 rounding: the
// high parts' difference by TwoSum (an FP32 subtraction of the high parts
// alone is not exact where one value is much smaller than the other, near a
// zero crossing, and its error would be relative to the difference, not to
// the much smaller higher differences formed from it).  Not normalised.
__device__ __forceinline__ df::f2 df_diff(float ah, float al, float bh, float bl) {
    const df::f2 s = df::two_sum(bh, -ah);
    return {s.hi, s.lo + (bl - al)};
}

// Second differences of `rows` df rows of length Y (row stride ystride) into
// dd (same stride); D_0 = D_{Y-1} = 0 (never read: the taps of a TDI
// interpolation stay inside the row).  D is ~(2 pi f dt)^2 of the values and
// needs ~1e-7 of itself: first differences exact, their difference rounded
// once to FP32.
__device__ __forceinline__ void second_differences(const float2 *y, float *dd, int rows, int Y,
                                                   int ystride, int tid, int nthreads) {
    for (int it = tid; it < rows * Y; it += nthreads) {
        const int r = it / Y, j = it - r * Y;
        const float2 *row = y + r * ystride;
        float v = 0.f;
        if (j > 0 && j < Y - 1) {
            const float2 a = row[j - 1], b = row[j], c = row[j + 1];
            const df::f2 d0 = df_diff(a.x, a.y, b.x, b.y), d1 = df_diff(b.x, b.y, c.x, c.y);
            v = (d1.hi - d0.hi) + (d1.lo - d0.lo);
        }
        dd[r * ystride + j] = v;
    }
}

// ---------------------------------------- third-difference link interpolation ----
//
// The link streams need ~50x more absolute accuracy per interpolation than
// the TDI taps (the response is a difference of two interpolated values
// ~2 pi f L apart), so the complex interpolation of the input uses one order
// more: the quadratic through samples d-1, d, d+1 (its Lagrange weights
// -eps (1-eps)/2, eps (2-eps), (1-eps)(2-eps)/2 at x = d + 1 - eps, a
// double-float Dot2 of three taps) reproduced by the weights exactly, and the
// remainder of every other tap written, by summation by parts three times
// from each end, over the input's third differences
// T_i = h_{i+3} - 3 h_{i+2} + 3 h_{i+1} - h_i (FP32):
//   sum W_k h_k = S(eps) q(x) + A(eps) (sum_{i>=-1} V_i T_{d+i} - sum_{j>=2} V'_j T_{d-j}),
// V_i = sum_{k>=i+3} C(k-1-i, 2) w_k on the right, the mirror on the left.
// Its FP32 part's error is ~1e-7 (2 pi f dt)^3 |h|, growing with frequency as
// the link streams and their TDI combinations do.

// Third differences of the staged df input, exact up to one final FP32
// rounding (see df_diff), real and imaginary parts: t3[i] for i + 3 < W.
__device__ __forceinline__ float third_difference(float4 v0, float4 v1, float4 v2, float4 v3,
                                                  bool imag) {
    const float a0 = imag ? v0.z : v0.x, b0 = imag ? v0.w : v0.y;
    const float a1 = imag ? v1.z : v1.x, b1 = imag ? v1.w : v1.y;
    const float a2 = imag ? v2.z : v2.x, b2 = imag ? v2.w : v2.y;
    const float a3 = imag ? v3.z : v3.x, b3 = imag ? v3.w : v3.y;
    const df::f2 d0 = df_diff(a0, b0, a1, b1), d1 = df_diff(a1, b1, a2, b2),
                 d2 = df_diff(a2, b2, a3, b3);
    const df::f2 s0 = df_diff(d0.hi, d0.lo, d1.hi, d1.lo),
                 s1 = df_diff(d1.hi, d1.lo, d2.hi, d2.lo);
    return (s1.hi - s0.hi) + (s1.lo - s0.lo);
}

// The staged window's views for the third-difference form: df values and
// third differences.
struct D3Shared {
    using index_t = int;
    const float4 *x;   // (re_hi, re_lo, im_hi, im_lo)
    const float2 *t3;  // third differences (re, im)
    __device__ __forceinline__ float4 val(int k) const { return x[k]; }
    __device__ __forceinline__ float2 tdiff(int k) const { return t3[k]; }
};

// The same from global memory (taps outside the staged window).
struct D3Global {
    using index_t = long;
    HSrc h;
    double scale;
    __device__ __forceinline__ float4 val(long k) const {
        const double2 v = h[k];
        const df::f2 r = df::from_double(v.x * scale), i = df::from_double(v.y * scale);
        return make_float4(r.hi, r.lo, i.hi, i.lo);
    }
    __device__ __forceinline__ float2 tdiff(long k) const {
        const float4 v0 = val(k), v1 = val(k + 1), v2 = val(k + 2), v3 = val(k + 3);
        return make_float2(third_difference(v0, v1, v2, v3, false),
                           third_difference(v0, v1, v2, v3, true));
    }
};

template <class Src>
__device__ __forceinline__ void d3_interp_c128(const Src &src, typename Src::index_t d, df::f2 e,
                                               const D2Weights &w, const df::f2 *edf, int h,
                                               df::f2 &re, df::f2 &im) {
    // the quadratic part: Dot2 of samples d-1, d, d+1 with the quadratic's weights
    const df::f2 ome = df::one_minus(e);
    const df::f2 c = df::mul(e, ome);                                   // eps (1 - eps)
    const df::f2 two_m = df::add_big_float(2.0f, {-e.hi, -e.lo});      // 2 - eps
    const df::f2 wm = {-0.5f * c.hi, -0.5f * c.lo};
    const df::f2 w0 = df::mul_raw(e, two_m);
    const df::f2 w1p = df::mul_raw(ome, two_m);
    const df::f2 w1 = {0.5f * w1p.hi, 0.5f * w1p.lo};
    df::Acc qr, qi;
    df::acc_init(qr);
    df::acc_init(qi);
    const float4 vm = src.val(d - 1), v0 = src.val(d), v1 = src.val(d + 1);
    df::acc_fma(qr, w0, {v0.x, v0.y});
    df::acc_fma(qi, w0, {v0.z, v0.w});
    df::acc_fma(qr, w1, {v1.x, v1.y});
    df::acc_fma(qi, w1, {v1.z, v1.w});
    df::acc_fma(qr, wm, {vm.x, vm.y});
    df::acc_fma(qi, wm, {vm.z, vm.w});
    // the third-difference remainder in FP32
    const float e32 = e.hi, o32 = ome.hi + ome.lo, c32 = c.hi;
    float a1 = 0.f, a2 = 0.f, a3 = 0.f, b1 = 0.f, b2 = 0.f, b3 = 0.f;
    float accr = 0.f, acci = 0.f;
    const df::f2 *Ej = edf + h - 2;
    float jf = (float)(h - 1);
    using index_t = typename Src::index_t;
    for (int j = h - 1; j >= 1; --j, --Ej, jf -= 1.f) {
        const float cE = c32 * Ej->hi;
        a1 = __fmaf_rn(cE, df::rcp_approx(jf + e32), a1);  // + w_{d+1+j}
        a2 += a1;
        a3 += a2;
        const float2 tr = src.tdiff(d + (index_t)(j - 2));
        accr = __fmaf_rn(a3, tr.x, accr);
        acci = __fmaf_rn(a3, tr.y, acci);
        if (j >= 2) {
            b1 = __fmaf_rn(cE, df::rcp_approx(jf + o32), b1);  // + w_{d-j}
            b2 += b1;
            b3 += b2;
            const float2 tl = src.tdiff(d - (index_t)j);
            accr = __fmaf_rn(-b3, tl.x, accr);
            acci = __fmaf_rn(-b3, tl.y, acci);
        }
    }
    re = d2_combine(df::acc_value(qr), w, accr);
    im = d2_combine(df::acc_value(qi), w, acci);
}

// As df_interp_c128_any for the third-difference form.
__device__ __forceinline__ bool d3_interp_c128_any(const float4 *hdf, const float2 *t3, long wlo,
                                                   int W, const HSrc &hg, double scale, long n,
                                                   int d, df::f2 e, const D2Weights &w,
                                                   const df::f2 *edf, int h, df::f2 &re,
                                                   df::f2 &im) {
    const long lo = (long)d - (h - 1), hi = (long)d + h;
    if (lo >= wlo && hi + 1 < wlo + W) {
        d3_interp_c128(D3Shared{hdf, t3}, (int)(d - wlo), e, w, edf, h, re, im);
        return true;
    }
    if (lo >= 0 && hi + 1 < n) {
        d3_interp_c128(D3Global{hg, scale}, (long)d, e, w, edf, h, re, im);
        return true;
    }
    return false;
}

// The mixed flavour's complex interpolation at (d, eps): the third-difference
// form (kD2), else the double-float summation by parts; staged window or
// global memory; false when the taps leave the input.
template <bool kD2>
__device__ __forceinline__ bool mixed_interp_any(const FusedArgs &a, const float4 *hdf,
                                                 const float4 *dh, long wlo, int W,
                                                 const HSrc &hg, double scale, long n, int d,
                                                 df::f2 e, df::f2 inv_deps, const df::f2 *edf,
                                                 int h, df::f2 &re, df::f2 &im) {
    if (kD2)
        return d3_interp_c128_any(hdf, reinterpret_cast<const float2 *>(dh), wlo, W, hg, scale, n,
                                  d, e, d2_weights(a, inv_deps, e), edf, h, re, im);
    return df_interp_c128_any(hdf, dh, wlo, W, hg, scale, n, d,
                              prefactor_df(a.a_tab, a.lt.num_A, inv_deps, e), e, edf, h, re, im);
}

// -------------------------------------------------------------- the kernel ----

// Register budgets: the mixed instances are sized for three blocks per SM (80
// registers; the grouped one measured 3 % faster than at the compiler's 96
// registers and two blocks, and the plan's persistent grid is sized for the
// instances together); the FP64 and the diagnostics instances keep the
// compiler's choice (a minimum of 0 blocks leaves it unspecified).
// kInner: the instance that forms per-tile inner products with FusedSource
// data (FusedArgs::partial) and writes the channels only where out is set.
// kT0Zero: the instance for launches whose sources all start at t0 = +0: a
// sample time t0 + j dt is then j dt and a split's t - t0 is t, bit for bit
// (j dt is never -0), so the two FP64 operations are left out.
// ------------------------------------------------ device-resident serving ----
//
// The server instances run the same item code over a source list that the
// host appends to in mapped page-locked memory while the kernel runs.  Such
// memory is read with ld.relaxed/acquire.sys, never through the read-only
// cache, so a line cached before the host wrote it is not reused.

__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ long long ld_relaxed_sys(const long long *p) {
    long long v;
    asm volatile("ld.relaxed.sys.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Called by every thread of a block between items.  Thread 0 first reports
// the finished item (`done_source` >= 0: its source, with `done_tiles` tiles
// in all) -- every thread has fenced its outputs at system scope before the
// barrier, so the flag the last tile sets is seen after them -- then claims
// the next published item with a CAS on the counter, polling (bounded by
// kServerMaxPolls and srv_idle_ns) while none is published.  Returns the item,
// or -1: the block leaves.
__device__ long long server_next_item(const FusedArgs &a, long long *slot, int tid,
                                      int done_source, long long done_tiles) {
    __threadfence_system();
    __syncthreads();
    if (tid == 0) {
        if (done_source >= 0) {
            const unsigned old = atomicAdd(a.srv_tiles_done + done_source, 1u);
            if ((long long)old + 1 == done_tiles) {
                __threadfence_system();
                asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(a.srv_done + done_source),
                             "r"(1u)
                             : "memory");
            }
        }
        long long got = -1;
        const unsigned long long t_start = globaltimer_ns();
        for (long it = 0; it < kServerMaxPolls; ++it) {
            const unsigned long long pub = ld_acquire_sys(a.srv_published);
            unsigned long long c = atomicAdd(a.work_next, 0ull);
            while (c < pub) {
                const unsigned long long prev = atomicCAS(a.work_next, c, c + 1ull);
                if (prev == c) {
                    got = (long long)c;
                    break;
                }
                c = prev;
            }
            if (got >= 0) break;
            int stop;
            asm volatile("ld.relaxed.sys.global.s32 %0, [%1];" : "=r"(stop) : "l"(a.srv_stop) : "memory");
            if (stop != 0 || globaltimer_ns() - t_start > (unsigned long long)a.srv_idle_ns) break;
            __nanosleep(1000);
        }
        *slot = got;
    }
    __syncthreads();
    const long long w = *slot;
    __syncthreads();
    return w;
}

template <bool kMixed, bool kDiag, bool kGrouped, bool kInner, bool kD2, bool kServer = false,
          bool kT0Zero = false>
__global__ void __launch_bounds__(kThreads, (kMixed && !kDiag) ? 3 : 0)
    fused_kernel(const FusedArgs a) {
    static_assert(!kT0Zero || (kMixed && !kServer), "the t0 = 0 instances are mixed batch instances");
    static_assert(!kServer || (kMixed && !kDiag && !kInner), "serving runs the plain mixed instances");
    static_assert(kMixed || !kD2, "the difference forms are mixed-arithmetic forms");
    static_assert(kMixed || !kGrouped, "the grouped form is a mixed-arithmetic form");
    static_assert(!(kDiag && kInner), "diagnostics and inner products are separate instances");
    extern __shared__ __align__(128) unsigned char smem[];
    const Layout lay = layout(kMixed, a.win_max, a.y_max);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    double *scale_sm = reinterpret_cast<double *>(smem + 16);
    int *scale_exp_sm = reinterpret_cast<int *>(smem + 24);  // scale = 2^(*scale_exp_sm)
    SegCache *segc = reinterpret_cast<SegCache *>(smem + 128);  // the item's orbit segments
    double *warp_max = reinterpret_cast<double *>(smem + 64);
    int2 *ends_sm = reinterpret_cast<int2 *>(smem + 256);  // (min d, max d) per link end
    long long *next_sm = reinterpret_cast<long long *>(smem + 352);  // next item, 2 slots
    // serving: the item's source descriptor and waveform parameters, copied
    // from mapped memory
    FusedSource *src_sm = reinterpret_cast<FusedSource *>(smem + 384);
    GbParams *gb_sm = reinterpret_cast<GbParams *>(smem + 576);
    static_assert(sizeof(FusedSource) <= 192 && sizeof(GbParams) <= 64, "header layout");
    static_assert(sizeof(FusedSource) % 8 == 0 && sizeof(FusedSource) / 8 <= 32 &&
                      sizeof(GbParams) % 8 == 0,
                  "descriptor copies: whole 8-byte words, one per thread of a warp");
    static_assert(kThreads / 32 <= 8, "warp maxima: 8 slots");
    static_assert(sizeof(SegCache) <= 128, "segment cache: 128 bytes");
    FusedTdiSet *set = reinterpret_cast<FusedTdiSet *>(smem + lay.set);
    df::f2 *edf = reinterpret_cast<df::f2 *>(smem + lay.edf);
    double2 *hraw = reinterpret_cast<double2 *>(smem + lay.hraw);
    float4 *hdf = reinterpret_cast<float4 *>(smem + lay.hdf);
    float4 *dh = reinterpret_cast<float4 *>(smem + lay.dh);
    double *y64 = reinterpret_cast<double *>(smem + lay.y);
    float2 *y32 = reinterpret_cast<float2 *>(smem + lay.y);
    float *d2 = reinterpret_cast<float *>(smem + lay.d2);

    const int tid = threadIdx.x;
    const int h = a.lt.h;
    const df::f2 inv_deps_df = df::from_double(a.inv_deps);
    if (tid == 0) mbar_init(bar, 1);
    for (int j = tid; j < h - 1; j += kThreads) edf[j] = df::from_double(__ldg(a.lt.E + j));
    __syncthreads();

    uint32_t phase = 0;
    int loaded_set = -1;
    const long num_work = __ldg(a.tile_start + a.num_sources);
    int si = 0;
    int par = 0;  // slot of next_sm this item's successor is written to
    // The block's next item is fetched by thread 0 at the start of an item and
    // read by all after the item's last barrier (the loop increment; a
    // `continue` passes through it too); the two slots alternate, so a slot
    // is rewritten only after every thread has read it.
    // serving: the finished item's source and tile count, for its report
    int srv_src = -1;
    long long srv_tiles = 0;
    long wi0 = blockIdx.x;
    if (kServer) wi0 = (long)server_next_item(a, next_sm, tid, -1, 0);
    for (long wi = wi0; kServer ? wi >= 0 : wi < num_work;
         wi = kServer ? (long)server_next_item(a, next_sm + 1, tid, srv_src, srv_tiles)
                      : (long)next_sm[par],
              par ^= 1) {
        if (!kServer && tid == 0)
            next_sm[par] = a.work_next ? (long long)gridDim.x + (long long)atomicAdd(a.work_next, 1ull)
                                       : wi + gridDim.x;
        // source of item wi: the last s with tile_start[s] <= wi.  A block's
        // items only grow and mostly stay in one source, so the current
        // source is checked first; otherwise a binary search from the next.
        long tile_idx;
        if (kServer) {
            // claimed items grow and their sources are published (entries not
            // yet published read as INT64_MAX): gallop up from the last source,
            // then bisect
            const long long *ts_m = reinterpret_cast<const long long *>(a.tile_start);
            if (ld_relaxed_sys(ts_m + si + 1) <= wi) {
                int lo = si + 1, step = 1;
                while (lo + step < a.num_sources && ld_relaxed_sys(ts_m + lo + step) <= wi) {
                    lo += step;
                    step *= 2;
                }
                int hi = min(lo + step, a.num_sources) - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (ld_relaxed_sys(ts_m + mid) <= wi)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                si = lo;
            }
            const long long first = ld_relaxed_sys(ts_m + si);
            srv_src = si;
            srv_tiles = ld_relaxed_sys(ts_m + si + 1) - first;
            tile_idx = wi - first;
            // the descriptor and parameters into shared memory
            const long long *from = reinterpret_cast<const long long *>(a.sources + si);
            if (tid < (int)(sizeof(FusedSource) / 8))
                reinterpret_cast<long long *>(src_sm)[tid] = ld_relaxed_sys(from + tid);
            const long long *gfrom = reinterpret_cast<const long long *>(a.gb + si);
            if (tid >= 32 && tid < 32 + (int)(sizeof(GbParams) / 8))
                reinterpret_cast<long long *>(gb_sm)[tid - 32] = ld_relaxed_sys(gfrom + tid - 32);
            __syncthreads();
        } else {
            if (__ldg(a.tile_start + si + 1) <= wi) {
                ++si;
                int hi = a.num_sources - 1;
                while (si < hi) {
                    const int mid = (si + hi + 1) >> 1;
                    if (__ldg(a.tile_start + mid) <= wi)
                        si = mid;
                    else
                        hi = mid - 1;
                }
            }
            tile_idx = wi - __ldg(a.tile_base + si);
        }
        const FusedSource &src = kServer ? *src_sm : a.sources[si];
        const GbParams *gbp = kServer ? gb_sm : (a.gb ? a.gb + si : nullptr);
        // the input outside the staged window: the stored waveform, or the
        // source's generator when it has none
        const HSrc hsrc{src.h, gbp, src.t0, a.dt};
        const long n = src.n;
        const int ps = src.ps, ts = src.ts;
        const double t0 = src.t0;
        const double k[3] = {src.k[0], src.k[1], src.k[2]};
        const double u[3] = {src.u[0], src.u[1], src.u[2]};
        const double v[3] = {src.v[0], src.v[1], src.v[2]};
        df::f2 kdf[3], udf[3], vdf[3];
        if (kMixed) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                kdf[c] = df::from_double(k[c]);
                udf[c] = df::from_double(u[c]);
                vdf[c] = df::from_double(v[c]);
            }
        }

        if (src.tdi_set != loaded_set) {
            const int *from = reinterpret_cast<const int *>(a.sets + src.tdi_set);
            int *to = reinterpret_cast<int *>(set);
            for (int i = tid; i < (int)(sizeof(FusedTdiSet) / sizeof(int)); i += kThreads)
                to[i] = from[i];
            loaded_set = src.tdi_set;
        }

        const long o0 = ts + tile_idx * a.tile;
        const long o1 = min(o0 + (long)a.tile, n - ts);
        // the first and last tiles also write the zeros of the edge zones
        // [0, ts) and [n - ts, n), so outputs need no clearing beforehand
        if ((tile_idx == 0 || o1 == n - ts) && (!kInner || src.out)) {
            const long e0 = (tile_idx == 0) ? 0 : n - ts;
            for (int c = 0; c < 3; ++c)
                for (long i = e0 + tid; i < e0 + ts; i += kThreads) src.out[c * n + i] = 0.0;
            if (tile_idx == 0 && o1 == n - ts)
                for (int c = 0; c < 3; ++c)
                    for (long i = n - ts + tid; i < n; i += kThreads) src.out[c * n + i] = 0.0;
        }
        const long ya = max(o0 - a.y_halo, 0L);
        const long yb = min(o1 + a.y_halo_hi, n);
        const long yfirst = max(ya, (long)ps), ylast = min(yb, n - ps);  // y computed here
        const int Y = (int)(yb - ya);

        // 1. input window: delays at both ends of the computed stream range
        // (threads 0-11, one link end each) and, in parallel, the item's orbit
        // segments (thread 32: its link-stream times and their emission times
        // up to 100 s earlier); one barrier for both
        if (tid < 12) {
            int2 e = make_int2(0x7fffffff, -0x7fffffff);
            if (yfirst < ylast) {
                const int slot = tid % 6;
                const long j = (tid < 6) ? yfirst : ylast - 1;
                const double t = sample_time<kT0Zero>(t0, j, a.dt);
                int dr, de;
                if (kMixed) {
                    MixedDelays g = link_delays_mixed<kT0Zero>(a.orb, a.inv_orbit_dt, slot, t, t0, a.fs, k);
                    dr = g.d_rec;
                    de = g.d_em;
                } else {
                    LinkGeometry g = link_geometry(a.orb, slot, t, t0, a.fs, k, u, v);
                    dr = g.d_rec;
                    de = g.d_em;
                }
                e = make_int2(min(dr, de), max(dr, de));
            }
            ends_sm[tid] = e;
        } else if (kMixed && tid == 32) {
            seg_cache_setup(segc, a.orb, a.inv_orbit_dt, t0 + (double)ya * a.dt - 100.0,
                            t0 + (double)yb * a.dt);
        }
        __syncthreads();
        long wlo = 0;
        int W = 0;
        if (yfirst < ylast) {
            int dmin = 0x7fffffff, dmax = -0x7fffffff;
#pragma unroll
            for (int q = 0; q < 12; ++q) {
                const int2 e = ends_sm[q];
                dmin = min(dmin, e.x);
                dmax = max(dmax, e.y);
            }
            wlo = max((long)dmin - (h - 1) - kWindowMargin, 0L);
            const long whi = min((long)dmax + h + 1 + kWindowMargin, n);
            W = (int)max(0L, min(whi - wlo, (long)a.win_max));
        }

        // 2. stage the window: generated in place for a source without a stored
        // waveform, else one bulk copy
        if (W > 0 && src.h == nullptr) {
            const GbCoefs gc = gb_coefs(*gbp);
            for (int i = tid; i < W; i += kThreads)
                hraw[i] = gb_sample(gc, t0 + exact_double_of(wlo + i) * a.dt);
            __syncthreads();
        } else if (W > 0) {
            if (tid == 0) {
                fence_proxy_async();
                mbar_expect_tx(bar, (uint32_t)W * 16u);
                bulk_copy_g2s(hraw, src.h + wlo, (uint32_t)W * 16u, bar);
            }
            const bool done = mbar_wait_bounded(bar, phase, a.wait_polls);
            if (__syncthreads_or(!done)) {
                // the copy missed the first bound: wait again with the full bound,
                // so that it lands before this block reuses its shared memory
                const bool landed = mbar_wait_bounded(bar, phase, kFusedWaitPolls);
                if (__syncthreads_or(!landed)) {
                    // still in flight: the block cannot reuse its shared memory and
                    // leaves; its remaining items are never computed, so every
                    // output of the launch is to be discarded
                    if (tid == 0) raise_status(a.orb.status, kStatusStaging | kStatusStagingLost);
                    return;
                }
                phase ^= 1u;
                // the copy landed late: this item's outputs become NaN (it is not
                // computed) and the block goes on with its next item
                if (tid == 0) raise_status(a.orb.status, kStatusStaging);
                if (!kInner || src.out)
                    for (int c = 0; c < 3; ++c)
                        for (long i = o0 + tid; i < o1; i += kThreads) src.out[c * n + i] = qnan();
                if (kInner && tid < 6) a.partial[wi * 6 + tid] = qnan();
                __syncthreads();
                continue;
            }
            phase ^= 1u;
        }

        // 3. mixed: scale to ~1 by a power of two, split into df (from the bits:
        // the power of two goes into the exponent), first differences
        double scale = 1.0;
        int sexp = 0;
        if (kMixed) {
            // the window's largest magnitude, from the bits (non-negative
            // doubles order like their bit patterns; NaN is skipped as fmax
            // skips it): integer work instead of FP64 comparisons
            unsigned long long mb = 0ull;
            for (int i = tid; i < W; i += kThreads) {
                const double2 q = hraw[i];
                unsigned long long bx = (unsigned long long)__double_as_longlong(q.x) &
                                        0x7fffffffffffffffull;
                unsigned long long by = (unsigned long long)__double_as_longlong(q.y) &
                                        0x7fffffffffffffffull;
                if (bx > 0x7ff0000000000000ull) bx = 0ull;
                if (by > 0x7ff0000000000000ull) by = 0ull;
                mb = max(mb, max(bx, by));
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
                mb = max(mb, (unsigned long long)__shfl_xor_sync(0xffffffffu, mb, off));
            if ((tid & 31) == 0) warp_max[tid >> 5] = __longlong_as_double((long long)mb);
            __syncthreads();
            if (tid == 0) {
                double mm = 0.0;
                for (int i = 0; i < kThreads / 32; ++i) mm = fmax(mm, warp_max[i]);
                int ex = 0;
                if (mm > 0.0 && mm < 1e300) frexp(mm, &ex);
                *scale_sm = ldexp(1.0, -ex);
                *scale_exp_sm = -ex;
            }
            __syncthreads();
            scale = *scale_sm;
            sexp = *scale_exp_sm;
            for (int i = tid; i < W; i += kThreads) {
                const double2 q = hraw[i];
                const df::f2 r = df::from_double_bits(q.x, sexp), im = df::from_double_bits(q.y, sexp);
                hdf[i] = make_float4(r.hi, r.lo, im.hi, im.lo);
                if (!kD2 && i + 1 < W) {
                    const double2 q1 = hraw[i + 1];
                    df::f2 dr = df::from_double((q1.x - q.x) * scale);
                    df::f2 di = df::from_double((q1.y - q.y) * scale);
                    dh[i] = make_float4(dr.hi, dr.lo, di.hi, di.lo);
                }
            }
            if (kD2) {  // third differences of the window (in dh's space)
                __syncthreads();
                float2 *t3 = reinterpret_cast<float2 *>(dh);
                for (int i = tid; i + 3 < W; i += kThreads) {
                    const float4 v0 = hdf[i], v1 = hdf[i + 1], v2 = hdf[i + 2], v3 = hdf[i + 3];
                    t3[i] = make_float2(third_difference(v0, v1, v2, v3, false),
                                        third_difference(v0, v1, v2, v3, true));
                }
            }
        }
        __syncthreads();

        // 4. link streams y[slot][j - ya] for j in [ya, yb).  Mixed flavour,
        // two links per receiving spacecraft: one (receiver, sample) per thread
        // iteration, the receiver's position, index split and interpolation
        // shared by its two links (the same values the per-link form computes
        // twice).  Otherwise one (link, sample) per thread iteration.
        if (kGrouped && a.trio) {
            // Equal arms (the grouped form implies them): every link leaving a
            // spacecraft has the same t_em, so a sample needs three receiver
            // and three emitter interpolations.  Three lanes per sample (ten
            // samples per warp, lanes 30-31 idle): lane r computes spacecraft
            // r + 1's receiver and emitter sides and takes the emitter sides of
            // its two links from the other lanes of its trio.
            const int lane = tid & 31, sub = lane / 3, r = lane - 3 * sub;
            const int rr = (r < 3) ? r : 0;
            for (int base = (tid >> 5) * 10; base < Y; base += 10 * (kThreads / 32)) {
                const int jj = base + sub;
                const bool act = (sub < 10) && (jj < Y);
                const long j = ya + jj;
                const bool live = act && j >= yfirst && j < ylast;
                const double t = sample_time<kT0Zero>(t0, j, a.dt);
                ReceiverSide rs{};
                EmitterSide es{};
                df::f2 re_r = {0.f, 0.f}, im_r = {0.f, 0.f}, re_e = {0.f, 0.f}, im_e = {0.f, 0.f};
                df::f2 xr_df[3] = {}, xe_df[3] = {};  // positions for the projections
                bool ok_r = false, ok_e = false;
                if (live) {
                    rs = receiver_mixed<kT0Zero>(a.orb, a.inv_orbit_dt, rr + 1, t, t0, a.fs, k, segc);
                    ok_r = mixed_interp_any<kD2>(a, hdf, dh, wlo, W, hsrc, scale, n, rs.d_rec,
                                            rs.e_rec, inv_deps_df, edf, h, re_r, im_r);
                    es = emitter_mixed<kT0Zero>(a.orb, a.inv_orbit_dt, a.tx_slot[rr], rs.w, t, t0, a.fs, k,
                                       segc);
                    ok_e = mixed_interp_any<kD2>(a, hdf, dh, wlo, W, hsrc, scale, n, es.d_em,
                                            es.e_em, inv_deps_df, edf, h, re_e, im_e);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        xr_df[c] = df::from_double_bits(rs.x_rec[c]);
                        xe_df[c] = df::from_double_bits(es.x_em[c]);
                    }
                }
                const bool own = live && (j >= o0 && j < o1);  // diagnostics
                for (int q = 0; q < 2; ++q) {
                    const int slot = a.rx_slot[rr][q];
                    const int from = min(3 * sub + a.orb.sc_e[slot] - 1, 31);
                    const unsigned full = 0xffffffffu;
                    const df::f2 xre = {__shfl_sync(full, re_e.hi, from),
                                        __shfl_sync(full, re_e.lo, from)};
                    const df::f2 xim = {__shfl_sync(full, im_e.hi, from),
                                        __shfl_sync(full, im_e.lo, from)};
                    const bool xok = __shfl_sync(full, (int)ok_e, from) != 0;
                    df::f2 x_em[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        x_em[c] = {__shfl_sync(full, xe_df[c].hi, from),
                                   __shfl_sync(full, xe_df[c].lo, from)};
                    const int d_em = __shfl_sync(full, es.d_em, from);
                    if (!act) continue;
                    if (!live) {  // the reference's y_gw is zero there
                        y32[slot * a.y_max + jj] = make_float2(0.f, 0.f);
                        continue;
                    }
                    if (kDiag && own && src.d_rec_out) {
                        src.d_rec_out[(long)slot * n + j] = rs.d_rec;
                        src.d_em_out[(long)slot * n + j] = d_em;
                    }
                    if (!ok_r || !xok) {
                        raise_status(a.orb.status, kStatusTap);
                        y32[slot * a.y_max + jj] = make_float2(__int_as_float(0x7fc00000), 0.f);
                        continue;
                    }
                    const DfProjection pr = df_projection_df(xr_df, x_em, kdf, udf, vdf);
                    const df::f2 dre = df::sub(xre, re_r), dim = df::sub(xim, im_r);
                    df::f2 yv = df::add(df::mul(dre, pr.xi_p), df::mul(dim, pr.xi_c));
                    yv = df::mul(yv, pr.pre);
                    y32[slot * a.y_max + jj] = make_float2(yv.hi, yv.lo);
                    if (kDiag && own && src.y_out)
                        src.y_out[(long)slot * n + j] = df::to_double(yv) / scale;
                }
            }
        } else if (kMixed && a.rx_shared) {
            for (int it = tid; it < 3 * Y; it += kThreads) {
                const int r = it / Y;
                const int jj = it - r * Y;
                const long j = ya + jj;
                if (j < yfirst || j >= ylast) {  // the reference's y_gw is zero there
                    y32[a.rx_slot[r][0] * a.y_max + jj] = make_float2(0.f, 0.f);
                    y32[a.rx_slot[r][1] * a.y_max + jj] = make_float2(0.f, 0.f);
                    continue;
                }
                const double t = sample_time<kT0Zero>(t0, j, a.dt);
                const bool own = (j >= o0 && j < o1);  // this tile's outputs: diagnostics
                const ReceiverSide rs =
                    receiver_mixed<kT0Zero>(a.orb, a.inv_orbit_dt, a.rx_sc[r], t, t0, a.fs, k, segc);
                df::f2 re_r, im_r;
                const bool ok_r = mixed_interp_any<kD2>(a, hdf, dh, wlo, W, hsrc, scale, n, rs.d_rec,
                                                   rs.e_rec, inv_deps_df, edf, h, re_r, im_r);
                for (int q = 0; q < 2; ++q) {
                    const int slot = a.rx_slot[r][q];
                    const EmitterSide es =
                        emitter_mixed<kT0Zero>(a.orb, a.inv_orbit_dt, slot, rs.w, t, t0, a.fs, k, segc);
                    if (kDiag && own && src.d_rec_out) {
                        src.d_rec_out[(long)slot * n + j] = rs.d_rec;
                        src.d_em_out[(long)slot * n + j] = es.d_em;
                    }
                    df::f2 re_e, im_e;
                    const bool ok_e = mixed_interp_any<kD2>(a, hdf, dh, wlo, W, hsrc, scale, n,
                                                       es.d_em, es.e_em, inv_deps_df, edf, h,
                                                       re_e, im_e);
                    if (!ok_r || !ok_e) {
                        raise_status(a.orb.status, kStatusTap);
                        y32[slot * a.y_max + jj] = make_float2(__int_as_float(0x7fc00000), 0.f);
                        continue;
                    }
                    const DfProjection pr = df_projection(rs.x_rec, es.x_em, kdf, udf, vdf);
                    const df::f2 dre = df::sub(re_e, re_r), dim = df::sub(im_e, im_r);
                    df::f2 yv = df::add(df::mul(dre, pr.xi_p), df::mul(dim, pr.xi_c));
                    yv = df::mul(yv, pr.pre);
                    y32[slot * a.y_max + jj] = make_float2(yv.hi, yv.lo);
                    if (kDiag && own && src.y_out)
                        src.y_out[(long)slot * n + j] = df::to_double(yv) / scale;
                }
            }
        } else if (!kMixed && a.trio) {
            // exact flavour on equal arms: three lanes per sample as in the
            // mixed form; lane r computes spacecraft r + 1's receiver side and
            // the emitter side that every link leaving it shares (the same
            // L(t) bits on every link, hence the same t_em, position, split and
            // interpolation), and each link's projection from its two sides:
            // the per-link form's operations, 6 interpolations instead of 9
            const int lane = tid & 31, sub = lane / 3, r = lane - 3 * sub;
            const int rr = (r < 3) ? r : 0;
            for (int base = (tid >> 5) * 10; base < Y; base += 10 * (kThreads / 32)) {
                const int jj = base + sub;
                const bool act = (sub < 10) && (jj < Y);
                const long j = ya + jj;
                const bool live = act && j >= yfirst && j < ylast;
                const double t = sample_time<kT0Zero>(t0, j, a.dt);
                ReceiverF64 rs{};
                double x_em[3] = {0.0, 0.0, 0.0};
                int d_em = 0;
                double hp_r = 0.0, hc_r = 0.0, hp_e = 0.0, hc_e = 0.0;
                bool okA_r = false, okT_r = false, okA_e = false, okT_e = false;
                if (live) {
                    rs = receiver_f64(a.orb, rr + 1, t, t0, a.fs, k);
                    double A_r;
                    okA_r = prefactor(a.lt, rs.e_rec, A_r);
                    okT_r = okA_r && c128_any(hraw, wlo, W, hsrc, n, rs.d_rec, rs.e_rec, A_r,
                                              a.lt, hp_r, hc_r);
                    double e_em, A_e;
                    emitter_side_f64(a.orb, rr + 1, t, light_travel_time(a.orb, t, a.tx_slot[rr]),
                                     t0, a.fs, k, x_em, d_em, e_em);
                    okA_e = prefactor(a.lt, e_em, A_e);
                    okT_e = okA_e && c128_any(hraw, wlo, W, hsrc, n, d_em, e_em, A_e, a.lt,
                                              hp_e, hc_e);
                }
                const bool own = live && (j >= o0 && j < o1);  // diagnostics
                for (int q = 0; q < 2; ++q) {
                    const int slot = a.rx_slot[rr][q];
                    const int from = min(3 * sub + a.orb.sc_e[slot] - 1, 31);
                    const unsigned full = 0xffffffffu;
                    const double xhp = __shfl_sync(full, hp_e, from);
                    const double xhc = __shfl_sync(full, hc_e, from);
                    const bool xokA = __shfl_sync(full, (int)okA_e, from) != 0;
                    const bool xokT = __shfl_sync(full, (int)okT_e, from) != 0;
                    double xem[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) xem[c] = __shfl_sync(full, x_em[c], from);
                    const int xd_em = __shfl_sync(full, d_em, from);
                    if (!act) continue;
                    if (!live) {  // the reference's y_gw is zero there
                        y64[slot * a.y_max + jj] = 0.0;
                        continue;
                    }
                    if (kDiag && own && src.d_rec_out) {
                        src.d_rec_out[(long)slot * n + j] = rs.d_rec;
                        src.d_em_out[(long)slot * n + j] = xd_em;
                    }
                    double out;
                    if (!(okA_r && xokA)) {
                        raise_status(a.orb.status, kStatusAIndex);
                        out = qnan();
                    } else if (okT_r && xokT) {
                        double xi_p, xi_c, k_dot_n;
                        link_projection_f64(rs.x_rec, xem, k, u, v, xi_p, xi_c, k_dot_n);
                        double pre = 1. / (1. - k_dot_n);
                        double big = (xhp - hp_r) * xi_p + (xhc - hc_r) * xi_c;
                        out = pre * big;
                    } else {
                        raise_status(a.orb.status, kStatusTap);
                        out = qnan();
                    }
                    y64[slot * a.y_max + jj] = out;
                    if (kDiag && own && src.y_out) src.y_out[(long)slot * n + j] = out;
                }
            }
        } else if (!kMixed && a.rx_shared) {
            // exact flavour: one (receiver, sample) item, the receiver side
            // shared by its two links
            for (int it = tid; it < 3 * Y; it += kThreads) {
                const int r = it / Y;
                const int jj = it - r * Y;
                const long j = ya + jj;
                if (j < yfirst || j >= ylast) {  // the reference's y_gw is zero there
                    y64[a.rx_slot[r][0] * a.y_max + jj] = 0.0;
                    y64[a.rx_slot[r][1] * a.y_max + jj] = 0.0;
                    continue;
                }
                const double t = sample_time<kT0Zero>(t0, j, a.dt);
                const bool own = (j >= o0 && j < o1);
                const ReceiverF64 rs = receiver_f64(a.orb, a.rx_sc[r], t, t0, a.fs, k);
                double A_r, hp_r = 0.0, hc_r = 0.0;
                const bool okA_r = prefactor(a.lt, rs.e_rec, A_r);
                const bool okT_r = okA_r && c128_any(hraw, wlo, W, hsrc, n, rs.d_rec, rs.e_rec,
                                                     A_r, a.lt, hp_r, hc_r);
                for (int q = 0; q < 2; ++q) {
                    const int slot = a.rx_slot[r][q];
                    const EmitterF64 es = emitter_f64(a.orb, slot, t, rs.x_rec, t0, a.fs, k, u, v);
                    if (kDiag && own && src.d_rec_out) {
                        src.d_rec_out[(long)slot * n + j] = rs.d_rec;
                        src.d_em_out[(long)slot * n + j] = es.d_em;
                    }
                    double A_e, out;
                    const bool okA_e = prefactor(a.lt, es.e_em, A_e);
                    if (!(okA_r && okA_e)) {
                        raise_status(a.orb.status, kStatusAIndex);
                        out = qnan();
                    } else {
                        double hp_e, hc_e;
                        const bool okT_e = c128_any(hraw, wlo, W, hsrc, n, es.d_em, es.e_em,
                                                    A_e, a.lt, hp_e, hc_e);
                        if (okT_r && okT_e) {
                            double pre = 1. / (1. - es.k_dot_n);
                            double big = (hp_e - hp_r) * es.xi_p + (hc_e - hc_r) * es.xi_c;
                            out = pre * big;
                        } else {
                            raise_status(a.orb.status, kStatusTap);
                            out = qnan();
                        }
                    }
                    y64[slot * a.y_max + jj] = out;
                    if (kDiag && own && src.y_out) src.y_out[(long)slot * n + j] = out;
                }
            }
        } else
        for (int it = tid; it < 6 * Y; it += kThreads) {
            const int slot = it / Y;
            const int jj = it - slot * Y;
            const long j = ya + jj;
            if (j < yfirst || j >= ylast) {  // the reference's y_gw is zero there
                if (kMixed)
                    y32[slot * a.y_max + jj] = make_float2(0.f, 0.f);
                else
                    y64[slot * a.y_max + jj] = 0.0;
                continue;
            }
            const double t = sample_time<kT0Zero>(t0, j, a.dt);
            if (kMixed) {
                const MixedDelays g = link_delays_mixed<kT0Zero>(a.orb, a.inv_orbit_dt, slot, t, t0, a.fs, k);
                const bool own = (j >= o0 && j < o1);  // this tile's outputs: diagnostics
                if (kDiag && own && src.d_rec_out) {
                    src.d_rec_out[(long)slot * n + j] = g.d_rec;
                    src.d_em_out[(long)slot * n + j] = g.d_em;
                }
                const long lo = (long)min(g.d_rec, g.d_em) - (h - 1);
                const long hi = (long)max(g.d_rec, g.d_em) + h;
                const df::f2 e_r = g.e_rec, e_e = g.e_em;
                df::f2 re_r, im_r, re_e, im_e;
                if (kD2) {
                    if (!(lo >= 0 && hi + 1 < n)) {
                        raise_status(a.orb.status, kStatusTap);
                        y32[slot * a.y_max + jj] = make_float2(__int_as_float(0x7fc00000), 0.f);
                        continue;
                    }
                    mixed_interp_any<kD2>(a, hdf, dh, wlo, W, hsrc, scale, n, g.d_rec, e_r,
                                     inv_deps_df, edf, h, re_r, im_r);
                    mixed_interp_any<kD2>(a, hdf, dh, wlo, W, hsrc, scale, n, g.d_em, e_e,
                                     inv_deps_df, edf, h, re_e, im_e);
                } else if (lo >= wlo && hi + 1 < wlo + W) {
                    const df::f2 A_r = prefactor_df(a.a_tab, a.lt.num_A, inv_deps_df, e_r);
                    const df::f2 A_e = prefactor_df(a.a_tab, a.lt.num_A, inv_deps_df, e_e);
                    const DfShared s{hdf, dh};
                    df_interp_c128_sbp(s, (int)(g.d_rec - wlo), A_r, e_r, edf, h, re_r, im_r);
                    df_interp_c128_sbp(s, (int)(g.d_em - wlo), A_e, e_e, edf, h, re_e, im_e);
                } else if (lo >= 0 && hi + 1 < n) {
                    const df::f2 A_r = prefactor_df(a.a_tab, a.lt.num_A, inv_deps_df, e_r);
                    const df::f2 A_e = prefactor_df(a.a_tab, a.lt.num_A, inv_deps_df, e_e);
                    const DfGlobal s{hsrc, scale};
                    df_interp_c128_sbp(s, g.d_rec, A_r, e_r, edf, h, re_r, im_r);
                    df_interp_c128_sbp(s, g.d_em, A_e, e_e, edf, h, re_e, im_e);
                } else {
                    raise_status(a.orb.status, kStatusTap);
                    y32[slot * a.y_max + jj] = make_float2(__int_as_float(0x7fc00000), 0.f);
                    continue;
                }
                const DfProjection pr = df_projection(g.x_rec, g.x_em, kdf, udf, vdf);
                const df::f2 dre = df::sub(re_e, re_r), dim = df::sub(im_e, im_r);
                df::f2 yv = df::add(df::mul(dre, pr.xi_p), df::mul(dim, pr.xi_c));
                yv = df::mul(yv, pr.pre);
                y32[slot * a.y_max + jj] = make_float2(yv.hi, yv.lo);
                if (kDiag && own && src.y_out)
                    src.y_out[(long)slot * n + j] = df::to_double(yv) / scale;
            } else {
                const LinkGeometry g = link_geometry(a.orb, slot, t, t0, a.fs, k, u, v);
                const bool own = (j >= o0 && j < o1);
                if (kDiag && own && src.d_rec_out) {
                    src.d_rec_out[(long)slot * n + j] = g.d_rec;
                    src.d_em_out[(long)slot * n + j] = g.d_em;
                }
                const long lo = (long)min(g.d_rec, g.d_em) - (h - 1);
                const long hi = (long)max(g.d_rec, g.d_em) + h;
                double A_r, A_e, out;
                bool ok = prefactor(a.lt, g.e_rec, A_r);
                ok = prefactor(a.lt, g.e_em, A_e) && ok;
                if (!ok) {
                    raise_status(a.orb.status, kStatusAIndex);
                    out = qnan();
                } else if ((lo >= wlo && hi < wlo + W) || (lo >= 0 && hi < n)) {
                    double hp_r, hc_r, hp_e, hc_e;
                    if (lo >= wlo && hi < wlo + W) {
                        const SharedC128 s{hraw};
                        lagrange_c128(s, (int)(g.d_rec - wlo), g.e_rec, A_r, a.lt, hp_r, hc_r);
                        lagrange_c128(s, (int)(g.d_em - wlo), g.e_em, A_e, a.lt, hp_e, hc_e);
                    } else {
                        const HSrc &s = hsrc;
                        lagrange_c128(s, g.d_rec, g.e_rec, A_r, a.lt, hp_r, hc_r);
                        lagrange_c128(s, g.d_em, g.e_em, A_e, a.lt, hp_e, hc_e);
                    }
                    double pre = 1. / (1. - g.k_dot_n);
                    double big = (hp_e - hp_r) * g.xi_p + (hc_e - hc_r) * g.xi_c;
                    out = pre * big;
                } else {
                    raise_status(a.orb.status, kStatusTap);
                    out = qnan();
                }
                y64[slot * a.y_max + jj] = out;
                if (kDiag && own && src.y_out) src.y_out[(long)slot * n + j] = out;
            }
        }
        __syncthreads();

        // 4b. grouped form: the link rows become the set's virtual rows, in
        // place (each thread reads a sample's six rows before writing them)
        if (kGrouped) {
            for (int jj = tid; jj < Y; jj += kThreads) {
                df::f2 z[6];
#pragma unroll
                for (int r = 0; r < 6; ++r) {
                    if (r < set->num_vrows) {
                        const float ca = set->vrow_ca[r], cb = set->vrow_cb[r];
                        const float2 va = y32[set->vrow_a[r] * a.y_max + jj];
                        const float2 vb = y32[set->vrow_b[r] * a.y_max + jj];
                        z[r] = df::add({ca * va.x, ca * va.y}, {cb * vb.x, cb * vb.y});
                    }
                }
#pragma unroll
                for (int r = 0; r < 6; ++r)
                    if (r < set->num_vrows) y32[r * a.y_max + jj] = make_float2(z[r].hi, z[r].lo);
            }
            __syncthreads();
        }
        // 4c. second-difference form: the rows' second differences (the input
        // window's space is free now)
        // Equal-delay groups: a group's delay has the same fractional part at
        // every sample up to FP64 rounding (equal arms), so its eps rounded to
        // FP32 (what the FP32 remainder weights depend on) takes one value or
        // a neighbour of it across a tile.  The partial sums are tabulated
        // for the first output sample's value and its two FP32 neighbours;
        // samples with one of those values read them, the others compute
        // them: the same numbers either way.  The tables sit behind the
        // second differences in the input window's space.
        const size_t tab_off = lay.d2 + align128(sizeof(float) * 6 * (size_t)a.y_max);
        float *wkey = reinterpret_cast<float *>(smem + tab_off);
        float2 *was = reinterpret_cast<float2 *>(smem + tab_off + 256);  // (A, sigma) per key
        float2 *wtab = reinterpret_cast<float2 *>(smem + tab_off + 256 + 512);
        const bool use_tab = kGrouped && kD2 && o0 < o1 &&
                             tab_off + 768 + sizeof(float2) * 3 * kFusedMaxGroups * (h - 1) <=
                                 lay.y;
        if (kMixed && kD2) {
            second_differences(y32, d2, kGrouped ? set->num_vrows : 6, Y, a.y_max, tid, kThreads);
            if (use_tab && tid < 3 * set->num_groups) {
                const int g = tid / 3, v = tid - 3 * g;
                const double t = t0 + (double)o0 * a.dt;
                const Seg w = seg_of(segc, a.orb, a.inv_orbit_dt, t);
                const double L0 =
                    (w.w < 0) ? 0.0
                              : orbit_lerp_b(a.orb.ltt, a.orb.ltt_slope, w.w, 6, 0, t, w.base);
                double delay = t;
                for (int m = 0; m < set->group_len[g]; ++m) delay = delay - L0;
                int d;
                df::f2 e;
                split_delay_df(delay, t0, a.fs, d, e);
                // the neighbours of a non-negative float by its bits (below 0: a
                // NaN key, which no sample matches)
                const float key = __int_as_float(__float_as_int(e.hi) + (v - 1));
                wkey[tid] = key;
                const D2Weights wk = d2_weights(a, inv_deps_df, df::f2{key, 0.f});
                was[tid] = make_float2(wk.A, wk.sigma);
                d2_group_sums(key, edf, h, wtab + (size_t)tid * (h - 1));
            }
            __syncthreads();
        }

        // 5. TDI for the output samples [o0, o1)
        double lk[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};  // inner products (kInner)
        if (kGrouped) {
            for (long i = o0 + tid; i < o1; i += kThreads) {
                const double t = sample_time<kT0Zero>(t0, i, a.dt);
                const Seg w = seg_of(segc, a.orb, a.inv_orbit_dt, t);
                // every link has this L(t): the delay of a list of length m is t - L - ... - L
                const double L0 =
                    (w.w < 0) ? 0.0
                              : orbit_lerp_b(a.orb.ltt, a.orb.ltt_slope, w.w, 6, 0, t, w.base);
                df::f2 accdf[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
                float corr[3] = {0.f, 0.f, 0.f};  // the difference form's FP32 parts
                double delay = t;
                int depth = 0;
                for (int g = 0; g < set->num_groups; ++g) {
                    for (const int len = set->group_len[g]; depth < len; ++depth)
                        delay = delay - L0;
                    int d;
                    df::f2 e_df;
                    split_delay_df<kT0Zero>(delay, t0, a.fs, d, e_df);
                    if (kDiag && src.d_tdi_out)
                        for (int u = set->group_start[g]; u < set->group_start[g + 1]; ++u)
                            src.d_tdi_out[(long)set->orig_unit[u] * n + i] = d;
                    const long lo = (long)d - (h - 1), hi = (long)d + h;
                    if (lo < ya || hi >= yb) {
                        raise_status(a.orb.status, kStatusTap);
#pragma unroll
                        for (int c = 0; c < 3; ++c)
                            if (set->group_vsign[g][c] != 0.f)
                                accdf[c] = {__int_as_float(0x7fc00000), 0.f};
                        continue;
                    }
                    int off[3];
                    float sg[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        off[c] = set->group_vrow[g][c] * a.y_max;
                        sg[c] = set->group_vsign[g][c];
                    }
                    if (kD2) {
                        // the FP32 weights, A and sigma are functions of eps
                        // rounded to FP32 (tabulated per item, or computed)
                        const float k32 = e_df.hi;
                        int q = -1;
                        if (use_tab)
                            q = (k32 == wkey[3 * g + 1])   ? 3 * g + 1
                                : (k32 == wkey[3 * g])     ? 3 * g
                                : (k32 == wkey[3 * g + 2]) ? 3 * g + 2
                                                           : -1;
                        D2Weights w2;
                        if (q >= 0) {
                            const float2 as = was[q];
                            w2.A = as.x;
                            w2.sigma = as.y;
                        } else {
                            w2 = d2_weights(a, inv_deps_df, df::f2{k32, 0.f});
                        }
                        d2_interp_group(y32, d2, off, sg, (int)(d - ya), e_df, w2, edf, h,
                                        q >= 0 ? wtab + (size_t)q * (h - 1) : nullptr, accdf,
                                        corr);
                    } else {
                        df::f2 val[3];
                        const df::f2 A_df = prefactor_df(a.a_tab, a.lt.num_A, inv_deps_df, e_df);
                        df_interp_group(y32, off, sg, (int)(d - ya), A_df, e_df, edf, h, a.h_df,
                                        val);
#pragma unroll
                        for (int c = 0; c < 3; ++c) accdf[c] = df::add(accdf[c], val[c]);
                    }
                }
                if (kD2) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) accdf[c] = df::add(accdf[c], {corr[c], 0.f});
                }
                const double X = df::to_double_bits(accdf[0], -sexp);
                const double Yc = df::to_double_bits(accdf[1], -sexp);
                const double Z = df::to_double_bits(accdf[2], -sexp);
                if (!kInner || src.out) store_channels(src.out, n, i, a.chan, X, Yc, Z);
                if (kInner && src.data) add_inner(lk, src.data, n, i, a.chan, X, Yc, Z);
            }
        } else {
            for (long i = o0 + tid; i < o1; i += kThreads) {
                const double t = sample_time<kT0Zero>(t0, i, a.dt);
                double L[kLinks];
                if (kMixed) {
                    const Seg w = seg_of(segc, a.orb, a.inv_orbit_dt, t);
                    const double dt_w = t - w.base;
#pragma unroll
                    for (int s = 0; s < kLinks; ++s)
                        L[s] = (w.w < 0) ? 0.0
                                         : __ldg(a.orb.ltt_slope + (size_t)w.w * 6 + s) * dt_w +
                                               __ldg(a.orb.ltt + (size_t)w.w * 6 + s);
                } else {
#pragma unroll
                    for (int s = 0; s < kLinks; ++s) L[s] = light_travel_time(a.orb, t, s);
                }
                double acc64[3] = {0.0, 0.0, 0.0};
                df::f2 accdf[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
                double stack[kFusedMaxDepth + 1];  // partial delays t - L_1 - ... - L_s
                stack[0] = t;
                long long prev_bits = 0x7ff8dead00000000ll;  // a NaN no delay can equal
                int d = 0;
                double eps = 0.0;
                df::f2 e_df = {0.f, 0.f}, A_df = {0.f, 0.f};
                D2Weights w2{};
                for (int unit = 0; unit < set->num_units; ++unit) {
                    const int ch = set->channel[unit];
                    const int len = set->delay_len[unit];
                    for (int s = set->prefix_keep[unit]; s < len; ++s)
                        stack[s + 1] = stack[s] - L[set->delay_slot[unit][s]];
                    const double delay = stack[len];
                    if (kMixed) {
                        // consecutive units with bit-identical delays share the split
                        const long long bits = __double_as_longlong(delay);
                        if (bits != prev_bits) {
                            split_delay_df<kT0Zero>(delay, t0, a.fs, d, e_df);
                            if (kD2)
                                w2 = d2_weights(a, inv_deps_df, e_df);
                            else
                                A_df = prefactor_df(a.a_tab, a.lt.num_A, inv_deps_df, e_df);
                            prev_bits = bits;
                        }
                    } else {
                        split_delay(delay, t0, a.fs, d, eps);
                    }
                    if (kDiag && src.d_tdi_out)
                        src.d_tdi_out[(long)set->orig_unit[unit] * n + i] = d;
                    const int b = set->base_slot[unit];
                    const long lo = (long)d - (h - 1), hi = (long)d + h;
                    if (lo < ya || hi >= yb) {
                        raise_status(a.orb.status, kStatusTap);
                        acc64[ch] = qnan();
                        accdf[ch] = {__int_as_float(0x7fc00000), 0.f};
                        continue;
                    }
                    if (kMixed) {
                        df::f2 val =
                            kD2 ? d2_interp_real(y32 + b * a.y_max, d2 + b * a.y_max,
                                                  (int)(d - ya), e_df, w2, edf, h)
                                 : df_interp_real(y32 + b * a.y_max, (int)(d - ya), A_df, e_df,
                                                  edf, h, a.h_df);
                        const int sc = set->sign_code[unit];
                        if (sc == 1)
                            accdf[ch] = df::add(accdf[ch], val);
                        else if (sc == -1)
                            accdf[ch] = df::sub(accdf[ch], val);
                        else
                            accdf[ch] = df::add(accdf[ch],
                                                df::mul(val, df::from_double(set->sign[unit])));
                    } else {
                        double pre;
                        if (!prefactor(a.lt, eps, pre)) {
                            raise_status(a.orb.status, kStatusAIndex);
                            acc64[ch] = qnan();
                            continue;
                        }
                        const SharedF64 row{y64 + b * a.y_max};
                        double val = lagrange_real(row, (int)(d - ya), eps, pre, a.lt);
                        val *= set->sign[unit];
                        acc64[ch] += val;
                    }
                }
                double X, Yc, Z;
                if (kMixed) {
                    X = df::to_double_bits(accdf[0], -sexp);
                    Yc = df::to_double_bits(accdf[1], -sexp);
                    Z = df::to_double_bits(accdf[2], -sexp);
                } else {
                    X = acc64[0];
                    Yc = acc64[1];
                    Z = acc64[2];
                }
                if (!kInner || src.out) store_channels(src.out, n, i, a.chan, X, Yc, Z);
                if (kInner && src.data) add_inner(lk, src.data, n, i, a.chan, X, Yc, Z);
            }
        }
        if (kInner) {
            // the tile's six sums, reduced in a fixed order: lanes by xor
            // shuffles, then the warps in index order (deterministic)
#pragma unroll
            for (int q = 0; q < 6; ++q)
#pragma unroll
                for (int off = 16; off > 0; off >>= 1)
                    lk[q] += __shfl_xor_sync(0xffffffffu, lk[q], off);
            __syncthreads();  // the link rows are read no more: their space takes the warp sums
            double *red = reinterpret_cast<double *>(smem + lay.y);
            if ((tid & 31) == 0)
#pragma unroll
                for (int q = 0; q < 6; ++q) red[(tid >> 5) * 6 + q] = lk[q];
            __syncthreads();
            if (tid < 6) {
                double sum = 0.0;
                for (int w = 0; w < kThreads / 32; ++w) sum += red[w * 6 + tid];
                a.partial[wi * 6 + tid] = sum;
            }
        }
        __syncthreads();
    }
}

// One thread per (source, quantity): the source's per-tile partial sums added
// in tile order.
__global__ void inner_reduce_kernel(const FusedSource *src, const long *tile_start,
                                    int num_sources, const double *partial) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int s = (int)(idx / 6), q = (int)(idx - 6L * (idx / 6));
    if (s >= num_sources || src[s].inner == nullptr) return;
    double sum = 0.0;
    for (long w = tile_start[s]; w < tile_start[s + 1]; ++w) sum += partial[w * 6 + q];
    src[s].inner[q] = sum;
}

}  // namespace

}  // namespace flr
