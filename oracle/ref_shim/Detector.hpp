// Test infrastructure: build shim for compiling the reference's CPU branch.
//
// The reference response code calls an `Orbits` class that lives in the
// lisaanalysistools package (Detector.hpp / Detector.cu, pinned by the
// reference at lisaanalysistools>=1.2.8, pyproject.toml:9).  That source is not
// available here, so this header restates the behaviour the reference relies on
// (call sites LISAResponse.cu:311,326,331,499-507,565-576):
//
//   * tables on a uniform time grid t_k = k*dt, k = 0..N-1, laid out as the
//     `pycppdetector_args` arrays (binding_flr.hpp:35-51):
//       ltt_arr[k*6 + link_slot], x_arr[(k*3 + sc_slot)*3 + coord],
//       n_arr[(k*6 + link_slot)*3 + coord]
//   * linear interpolation between the two knots that bracket t, in slope form
//       value = ((hi - lo) / dt) * (t - dt*w) + lo,  w = (int)(t / dt)
//   * w < 0 or w > N-1 is "outside the table": light travel time 0 and a zero
//     position; w == N-1 uses the last segment (no read past the table);
//   * link numbers (12, 23, 31, 13, 32, 21 by default) map to the slot where
//     they appear in `links`; spacecraft numbers 1..3 map to slots 0..2.
//
// The CPU oracle (oracle/flr_oracle.c) and the CUDA kernels implement the same
// rules, so the three agree bit for bit; agreement with lisaanalysistools'
// own interpolation is not pinned (its source is absent).
#ifndef ORACLE_REF_SHIM_DETECTOR_HPP
#define ORACLE_REF_SHIM_DETECTOR_HPP

#include "cuda_complex.hpp"

class Vec {
  public:
    double x;
    double y;
    double z;
    Vec(double x_, double y_, double z_) : x(x_), y(y_), z(z_) {}
};

class OrbitsCPU {
  public:
    double dt;
    int N;
    double *n_arr;
    double *ltt_arr;
    double *x_arr;
    int *links;
    int *sc_r;
    int *sc_e;
    double armlength;

    OrbitsCPU(double dt_, int N_, double *n_arr_, double *ltt_arr_, double *x_arr_,
              int *links_, int *sc_r_, int *sc_e_, double armlength_)
        : dt(dt_), N(N_), n_arr(n_arr_), ltt_arr(ltt_arr_), x_arr(x_arr_),
          links(links_), sc_r(sc_r_), sc_e(sc_e_), armlength(armlength_) {}

    int get_link_ind(int link) const {
        for (int s = 0; s < 6; ++s)
            if (links[s] == link) return s;
        return -1;
    }

    int get_sc_ind(int sc) const { return (sc >= 1 && sc <= 3) ? sc - 1 : -1; }

    // Segment index for time t, or -1 when t is outside the table.
    int segment(double t) const {
        int w = (int)(t / dt);
        if (w < 0 || w > N - 1) return -1;
        return (w == N - 1) ? N - 2 : w;
    }

    double lerp(const double *tab, int w, long stride, long col, double t) const {
        double lo = tab[(long)w * stride + col];
        double hi = tab[(long)(w + 1) * stride + col];
        return ((hi - lo) / dt) * (t - dt * w) + lo;
    }

    double get_light_travel_time(double t, int link) const {
        int w = segment(t);
        int s = get_link_ind(link);
        if (w < 0 || s < 0) return 0.0;
        return lerp(ltt_arr, w, 6, s, t);
    }

    Vec get_pos(double t, int sc) const {
        int w = segment(t);
        int s = get_sc_ind(sc);
        if (w < 0 || s < 0) return Vec(0.0, 0.0, 0.0);
        return Vec(lerp(x_arr, w, 9, s * 3 + 0, t),
                   lerp(x_arr, w, 9, s * 3 + 1, t),
                   lerp(x_arr, w, 9, s * 3 + 2, t));
    }
};

#endif
