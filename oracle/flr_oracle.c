/*
 * CPU oracle for the LISA response + TDI hot path — TEST INFRASTRUCTURE ONLY.
 * See flr_oracle.h for what may use it and what it restates.
 *
 * Build with -ffp-contract=off (oracle/Makefile): the oracle evaluates every
 * expression as separately rounded IEEE-754 double operations in the order the
 * reference's source writes them, which is what makes its integer delay indices
 * and its outputs reproducible bit for bit on x86-64, aarch64 and the GPU.
 */
#include "flr_oracle.h"

#include <math.h>
#include <stddef.h>

/* Speed-of-light reciprocal [s/m], LISAResponse.hh:7. */
#define ORC_C_INV 3.3356409519815204e-09
#define ORC_NO_LINK (-11) /* "no delay" marker in the TDI link lists, response.py:390 */

/* ---------------------------------------------------------------- orbits -- */

static int orc_link_slot(const orc_orbits *o, int link)
{
    for (int s = 0; s < 6; ++s)
        if (o->links[s] == link) return s;
    return -1;
}

static int orc_sc_slot(int sc) { return (sc >= 1 && sc <= 3) ? sc - 1 : -1; }

/* Segment of the uniform grid holding t; -1 outside the table. */
static int orc_segment(const orc_orbits *o, double t)
{
    int w = (int)(t / o->dt);
    if (w < 0 || w > o->N - 1) return -1;
    return (w == o->N - 1) ? o->N - 2 : w;
}

static double orc_lerp(const orc_orbits *o, const double *tab, int w, int stride, int col, double t)
{
    double lo = tab[(size_t)w * stride + col];
    double hi = tab[(size_t)(w + 1) * stride + col];
    double slope = (hi - lo) / o->dt;
    return slope * (t - o->dt * (double)w) + lo;
}

double orc_light_travel_time(const orc_orbits *o, double t, int link)
{
    int w = orc_segment(o, t);
    int s = orc_link_slot(o, link);
    if (w < 0 || s < 0) return 0.0;
    return orc_lerp(o, o->ltt, w, 6, s, t);
}

void orc_position(const orc_orbits *o, double t, int sc, double out[3])
{
    int w = orc_segment(o, t);
    int s = orc_sc_slot(sc);
    for (int c = 0; c < 3; ++c)
        out[c] = (w < 0 || s < 0) ? 0.0 : orc_lerp(o, o->x, w, 9, 3 * s + c, t);
}

/* ------------------------------------------------------ small geometry -- */

/* dot_product_1d, LISAResponse.cu:48-57: accumulated from 0.0, left to right. */
static double orc_dot3(const double *a, const double *b)
{
    double acc = 0.0;
    for (int c = 0; c < 3; ++c) acc += a[c] * b[c];
    return acc;
}

/* Integer sample index and fractional offset of a delayed time,
 * LISAResponse.cu:339-341 and 616-622. */
static void orc_split_delay(double delayed_t, double t_first, double fs, int *d, double *eps)
{
    double x = delayed_t - t_first;
    int di = (int)ceil(x * fs) - 1;
    *d = di;
    *eps = (1.0 + (double)di) - x * fs;
}

/* Lagrange prefactor A(eps) from the tabulated values by linear interpolation,
 * LISAResponse.cu:114-117 / 161-164. */
static double orc_prefactor(double eps, const double *A, double deps)
{
    int ind = (int)(eps / deps);
    double frac = (eps - (double)ind * deps) / deps;
    return A[ind] * (1. - frac) + A[ind + 1] * frac;
}

/* Real 2h-point Lagrange fractional-delay interpolation around sample d,
 * interp_single, LISAResponse.cu:110-147. */
static double orc_lagrange_real(const double *x, int h, int d, double eps, const double *A,
                                double deps, const double *E)
{
    double pre = orc_prefactor(eps, A, deps);
    double w_up = 1.0 - eps, w_dn = eps, w_tail = eps * (1.0 - eps);
    double tail = 0.0;
    for (int j = 1; j < h; ++j) {
        double f = (double)j + eps;
        double g = (double)j + (1.0 - eps);
        tail += E[j - 1] * (x[d + 1 + j] / f + x[d - j] / g);
    }
    return pre * (w_up * x[d + 1] + w_dn * x[d] + w_tail * tail);
}

/* Complex version over interleaved (re, im) samples, interp, LISAResponse.cu:149-207. */
static void orc_lagrange_c128(const double *x, int h, int d, double eps, const double *A,
                              double deps, const double *E, double *re, double *im)
{
    double pre = orc_prefactor(eps, A, deps);
    double w_up = 1.0 - eps, w_dn = eps, w_tail = eps * (1.0 - eps);
    double tail_re = 0.0, tail_im = 0.0;
    for (int j = 1; j < h; ++j) {
        double f = (double)j + eps;
        double g = (double)j + (1.0 - eps);
        const double *up = x + 2 * (ptrdiff_t)(d + 1 + j);
        const double *dn = x + 2 * (ptrdiff_t)(d - j);
        tail_re += E[j - 1] * (up[0] / f + dn[0] / g);
        tail_im += E[j - 1] * (up[1] / f + dn[1] / g);
    }
    const double *up0 = x + 2 * (ptrdiff_t)(d + 1);
    const double *dn0 = x + 2 * (ptrdiff_t)d;
    *re = pre * (w_up * up0[0] + w_dn * dn0[0] + w_tail * tail_re);
    *im = pre * (w_up * up0[1] + w_dn * dn0[1] + w_tail * tail_im);
}

/* ------------------------------------------------------------- response -- */

/* One (link, sample) projection, the body of the sample loop of response(),
 * LISAResponse.cu:559-668. */
static double orc_link_sample(const orc_orbits *o, int slot, double t, double t_first,
                              const double *k, const double *u, const double *v,
                              const double *input, int h, double fs, const double *A,
                              double deps, const double *E, int *d_rec_out, int *d_em_out)
{
    double L = orc_light_travel_time(o, t, o->links[slot]);
    double t_em = t - L;
    double x_rec[3], x_em[3], n[3];
    orc_position(o, t, o->sc_r[slot], x_rec);
    orc_position(o, t_em, o->sc_e[slot], x_em);

    double norm = 0.0;
    for (int c = 0; c < 3; ++c) {
        n[c] = x_rec[c] - x_em[c];
        norm += n[c] * n[c];
    }
    norm = sqrt(norm);
    for (int c = 0; c < 3; ++c) n[c] = n[c] / norm;

    /* xi_projections, LISAResponse.cu:59-67 */
    double un = orc_dot3(u, n), vn = orc_dot3(v, n);
    double xi_p = 0.5 * ((un * un) - (vn * vn));
    double xi_c = un * vn;

    double kn = orc_dot3(k, n);
    double kx_rec = orc_dot3(k, x_rec);
    double kx_em = orc_dot3(k, x_em);

    double delay_rec = t - kx_rec * ORC_C_INV;
    double delay_em = t_em - kx_em * ORC_C_INV;

    int d_rec, d_em;
    double e_rec, e_em;
    orc_split_delay(delay_rec, t_first, fs, &d_rec, &e_rec);
    orc_split_delay(delay_em, t_first, fs, &d_em, &e_em);
    if (d_rec_out) *d_rec_out = d_rec;
    if (d_em_out) *d_em_out = d_em;

    double hp_rec, hc_rec, hp_em, hc_em;
    orc_lagrange_c128(input, h, d_rec, e_rec, A, deps, E, &hp_rec, &hc_rec);
    orc_lagrange_c128(input, h, d_em, e_em, A, deps, E, &hp_em, &hc_em);

    double pre = 1. / (1. - kn);
    double big = (hp_em - hp_rec) * xi_p + (hc_em - hc_rec) * xi_c;
    return pre * big;
}

void orc_get_response_range(const orc_orbits *o, double *y_gw, const double *t_data,
                            const double *k, const double *u, const double *v, int num_delays,
                            const double *input_c128, int order, double sampling_frequency,
                            const double *A, double deps, const double *E, int start,
                            int *d_rec, int *d_em, int i0, int i1)
{
    int h = (order + 1) / 2;
    double t_first = t_data[0];
    int lo = i0 > start ? i0 : start;
    int hi = i1 < num_delays - start ? i1 : num_delays - start;
    for (int slot = 0; slot < 6; ++slot) {
        for (int i = lo; i < hi; ++i) {
            size_t at = (size_t)slot * num_delays + i;
            y_gw[at] = orc_link_sample(o, slot, t_data[i], t_first, k, u, v, input_c128, h,
                                       sampling_frequency, A, deps, E,
                                       d_rec ? d_rec + at : NULL, d_em ? d_em + at : NULL);
        }
    }
}

void orc_get_response(const orc_orbits *o, double *y_gw, const double *t_data, const double *k,
                      const double *u, const double *v, int num_delays,
                      const double *input_c128, int order, double sampling_frequency,
                      const double *A, double deps, const double *E, int start,
                      int *d_rec, int *d_em)
{
    orc_get_response_range(o, y_gw, t_data, k, u, v, num_delays, input_c128, order,
                           sampling_frequency, A, deps, E, start, d_rec, d_em, start,
                           num_delays - start);
}

/* ------------------------------------------------------------------ TDI -- */

void orc_get_tdi_delays_range(const orc_orbits *o, double *delayed_links,
                              const double *input_links, int num_inputs, int num_delays,
                              const double *t_arr, const int *unit_starts,
                              const int *unit_lengths, const int *tdi_base_link,
                              const int *tdi_link_combinations, const double *tdi_signs,
                              const int *channels, int num_units, int order,
                              double sampling_frequency, const double *A, double deps,
                              const double *E, int start, int *d_out, int i0, int i1)
{
    int h = (order + 1) / 2;
    double t_first = t_arr[0];
    int lo = i0 > start ? i0 : start;
    int hi = i1 < num_delays - start ? i1 : num_delays - start;
    for (int i = lo; i < hi; ++i) {
        double t = t_arr[i];
        for (int unit = 0; unit < num_units; ++unit) {
            /* delay = t - sum of L(t) over the unit's link list, all L taken at
             * the same t, LISAResponse.cu:314-333 */
            double delay = t;
            for (int s = 0; s < unit_lengths[unit]; ++s) {
                int link = tdi_link_combinations[unit_starts[unit] + s];
                if (link != ORC_NO_LINK) delay -= orc_light_travel_time(o, t, link);
            }
            int d;
            double eps;
            orc_split_delay(delay, t_first, sampling_frequency, &d, &eps);
            if (d_out) d_out[(size_t)unit * num_delays + i] = d;

            const double *row = input_links + (size_t)orc_link_slot(o, tdi_base_link[unit]) * num_inputs;
            double val = orc_lagrange_real(row, h, d, eps, A, deps, E);
            val *= tdi_signs[unit];
            delayed_links[(size_t)channels[unit] * num_delays + i] += val;
        }
    }
}

void orc_get_tdi_delays(const orc_orbits *o, double *delayed_links, const double *input_links,
                        int num_inputs, int num_delays, const double *t_arr,
                        const int *unit_starts, const int *unit_lengths,
                        const int *tdi_base_link, const int *tdi_link_combinations,
                        const double *tdi_signs, const int *channels, int num_units,
                        int order, double sampling_frequency, const double *A, double deps,
                        const double *E, int start, int *d_out)
{
    orc_get_tdi_delays_range(o, delayed_links, input_links, num_inputs, num_delays, t_arr,
                             unit_starts, unit_lengths, tdi_base_link, tdi_link_combinations,
                             tdi_signs, channels, num_units, order, sampling_frequency, A, deps,
                             E, start, d_out, start, num_delays - start);
}
