// Device-side building blocks of the plain FP64 response + TDI path.
//
// Every function here evaluates the reference's expressions as separately
// rounded IEEE-754 double operations, in the order the reference writes them.
// The translation units that include this header are compiled with
// --fmad=false so nvcc cannot contract a*b+c into an FMA; division and square
// root are nvcc's correctly rounded defaults (-prec-div=true -prec-sqrt=true).
// That makes the integer delay indices and the outputs equal, bit for bit, to
// the reference's CPU code built without contraction.
#pragma once

#include <cstdint>

namespace flr {

constexpr double kCInv = 3.3356409519815204e-09;  // s/m, LISAResponse.hh:7
constexpr int kNoLink = -11;                      // "no delay" marker, response.py:390
constexpr int kLinks = 6;

// Status bits (mirror FLR_STATUS_* of include/flr_gb300.h).
constexpr unsigned kStatusTap = 0x1u;
constexpr unsigned kStatusAIndex = 0x2u;
constexpr unsigned kStatusLink = 0x4u;
constexpr unsigned kStatusChannel = 0x8u;

// Orbit tables resident in device memory, passed to kernels by value.
// Layout of lisaanalysistools' pycppdetector_args plus per-segment slopes
// ((hi - lo) / dt, precomputed once with the same IEEE division the
// interpolation formula performs, so using them changes no bit).
struct OrbitTables {
    double dt;
    int N;
    const double *ltt;        // [N][6]
    const double *x;          // [N][3][3]
    const double *ltt_slope;  // [N-1][6]
    const double *x_slope;    // [N-1][9]
    int links[kLinks];
    int sc_r[kLinks];         // receiver spacecraft number (1..3) per link slot
    int sc_e[kLinks];         // emitter spacecraft number (1..3) per link slot
    unsigned *status;         // sticky FLR_STATUS_* bits
};

// Lagrange interpolation tables (response.py:273-310).
struct LagrangeTables {
    const double *A;  // [num_A]   prefactor A(eps) on eps = k*deps
    const double *E;  // [h-1]     tail weights E_j
    double deps;
    int num_A;
    int h;            // (order + 1) / 2
};

__device__ __forceinline__ void raise_status(unsigned *status, unsigned bit) {
    if (status) atomicOr(status, bit);
}

__device__ __forceinline__ int link_slot(const OrbitTables &o, int link) {
#pragma unroll
    for (int s = 0; s < kLinks; ++s)
        if (o.links[s] == link) return s;
    return -1;
}

// Segment of the uniform orbit grid containing t, or -1 outside the table
// (lisaanalysistools Orbits window rule, restated; see the header comment of
// include/flr_gb300.h).
__device__ __forceinline__ int orbit_segment(const OrbitTables &o, double t) {
    int w = (int)(t / o.dt);
    if (w < 0 || w > o.N - 1) return -1;
    return (w == o.N - 1) ? o.N - 2 : w;
}

// slope * (t - dt * w) + lo: the linear-interpolation formula of the orbit
// tables, evaluated as the reference's dependency writes it.
__device__ __forceinline__ double orbit_lerp(const double *tab, const double *slope, int w,
                                             int stride, int col, double t, double dt) {
    double lo = __ldg(tab + (size_t)w * stride + col);
    double m = __ldg(slope + (size_t)w * stride + col);
    return m * (t - dt * (double)w) + lo;
}

__device__ __forceinline__ double light_travel_time(const OrbitTables &o, double t, int slot) {
    int w = orbit_segment(o, t);
    if (w < 0 || slot < 0) return 0.0;
    return orbit_lerp(o.ltt, o.ltt_slope, w, 6, slot, t, o.dt);
}

__device__ __forceinline__ void position(const OrbitTables &o, double t, int sc, double out[3]) {
    int w = orbit_segment(o, t);
    int s = (sc >= 1 && sc <= 3) ? sc - 1 : -1;
    if (w < 0 || s < 0) {
        out[0] = out[1] = out[2] = 0.0;
        return;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) out[c] = orbit_lerp(o.x, o.x_slope, w, 9, 3 * s + c, t, o.dt);
}

// ((0 + a0 b0) + a1 b1) + a2 b2, dot_product_1d, LISAResponse.cu:48-57.
__device__ __forceinline__ double dot3(const double *a, const double *b) {
    double acc = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) acc += a[c] * b[c];
    return acc;
}

// Integer index and fraction of a delayed time, LISAResponse.cu:339-341, 616-622.
__device__ __forceinline__ void split_delay(double delayed_t, double t_first, double fs, int &d,
                                            double &eps) {
    double x = delayed_t - t_first;
    d = (int)ceil(x * fs) - 1;
    eps = (1.0 + (double)d) - x * fs;
}

// A(eps) by linear interpolation in the table, LISAResponse.cu:114-117, 161-164.
// Returns false (and leaves `a` NaN) when the table index is out of range.
__device__ __forceinline__ bool prefactor(const LagrangeTables &lt, double eps, double &a) {
    int ind = (int)(eps / lt.deps);
    if (ind < 0 || ind > lt.num_A - 2) {
        a = __longlong_as_double(0x7ff8000000000000ll);
        return false;
    }
    double frac = (eps - (double)ind * lt.deps) / lt.deps;
    a = __ldg(lt.A + ind) * (1. - frac) + __ldg(lt.A + ind + 1) * frac;
    return true;
}

// Sample sources for the interpolation: read-only global memory through the
// texture path, or shared memory (staged windows).
struct GlobalF64 {
    const double *p;
    __device__ __forceinline__ double operator[](long i) const { return __ldg(p + i); }
};
struct GlobalC128 {
    const double2 *p;
    __device__ __forceinline__ double2 operator[](long i) const { return __ldg(p + i); }
};
struct SharedF64 {
    const double *p;
    __device__ __forceinline__ double operator[](long i) const { return p[i]; }
};
struct SharedC128 {
    const double2 *p;
    __device__ __forceinline__ double2 operator[](long i) const { return p[i]; }
};

// (double)j for an integer |j| < 2^52, assembled from the bits of j: the
// exact value the conversion instruction gives, without that instruction
// (conversions to FP64 take the FP64 pipe's issue slots).
__device__ __forceinline__ double exact_double_of(long long j) {
    const unsigned long long u = (unsigned long long)(j < 0 ? -j : j);
    const int e = 63 - __clzll((long long)u);  // u = 0: -1 (replaced below)
    const unsigned long long b = ((unsigned long long)(1023 + e) << 52) |
                                 ((u << (52 - e)) & 0xfffffffffffffull) |
                                 (j < 0 ? 0x8000000000000000ull : 0ull);
    return __longlong_as_double(u == 0 ? 0ll : (long long)b);
}

// Real 2h-point Lagrange interpolation of x around sample d (interp_single,
// LISAResponse.cu:110-147).  The caller guarantees d-h+1 >= 0 and d+h < n.
template <class Src>
__device__ __forceinline__ double lagrange_real(const Src &x, int d, double eps, double a,
                                                const LagrangeTables &lt) {
    double w_up = 1.0 - eps, w_dn = eps, w_tail = eps * (1.0 - eps);
    double tail = 0.0;
    for (int j = 1; j < lt.h; ++j) {
        const double jd = exact_double_of(j);
        double f = jd + eps;
        double g = jd + (1.0 - eps);
        double up = x[d + 1 + j];
        double dn = x[d - j];
        tail += __ldg(lt.E + j - 1) * (up / f + dn / g);
    }
    return a * (w_up * x[d + 1] + w_dn * x[d] + w_tail * tail);
}

// Complex version over interleaved complex128 samples (interp,
// LISAResponse.cu:149-207).
template <class Src>
__device__ __forceinline__ void lagrange_c128(const Src &x, int d, double eps, double a,
                                              const LagrangeTables &lt, double &re, double &im) {
    double w_up = 1.0 - eps, w_dn = eps, w_tail = eps * (1.0 - eps);
    double tail_re = 0.0, tail_im = 0.0;
    for (int j = 1; j < lt.h; ++j) {
        const double jd = exact_double_of(j);
        double f = jd + eps;
        double g = jd + (1.0 - eps);
        double2 up = x[d + 1 + j];
        double2 dn = x[d - j];
        double e = __ldg(lt.E + j - 1);
        tail_re += e * (up.x / f + dn.x / g);
        tail_im += e * (up.y / f + dn.y / g);
    }
    double2 up0 = x[d + 1];
    double2 dn0 = x[d];
    re = a * (w_up * up0.x + w_dn * dn0.x + w_tail * tail_re);
    im = a * (w_up * up0.y + w_dn * dn0.y + w_tail * tail_im);
}

// Geometry of one link at reception time t (LISAResponse.cu:565-622): the
// integer/fractional receiver and emitter delays and the projection factors.
struct LinkGeometry {
    int d_rec, d_em;
    double e_rec, e_em;
    double xi_p, xi_c, k_dot_n;
};

__device__ __forceinline__ LinkGeometry link_geometry(const OrbitTables &o, int slot, double t,
                                                      double t_first, double fs,
                                                      const double k[3], const double u[3],
                                                      const double v[3]) {
    LinkGeometry g;
    double L = light_travel_time(o, t, slot);
    double t_em = t - L;
    double x_rec[3], x_em[3], n[3];
    position(o, t, o.sc_r[slot], x_rec);
    position(o, t_em, o.sc_e[slot], x_em);

    double norm = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        n[c] = x_rec[c] - x_em[c];
        norm += n[c] * n[c];
    }
    norm = sqrt(norm);
#pragma unroll
    for (int c = 0; c < 3; ++c) n[c] = n[c] / norm;

    double un = dot3(u, n), vn = dot3(v, n);
    g.xi_p = 0.5 * ((un * un) - (vn * vn));
    g.xi_c = un * vn;
    g.k_dot_n = dot3(k, n);
    double kx_rec = dot3(k, x_rec);
    double kx_em = dot3(k, x_em);

    double delay_rec = t - kx_rec * kCInv;
    double delay_em = t_em - kx_em * kCInv;
    split_delay(delay_rec, t_first, fs, g.d_rec, g.e_rec);
    split_delay(delay_em, t_first, fs, g.d_em, g.e_em);
    return g;
}

}  // namespace flr
