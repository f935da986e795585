/*
 * CPU oracle for the LISA time-domain response + TDI hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py may load this library, and only as the checker
 * or as the timed CPU baseline.  The product (the CUDA library and its Python
 * host layer) never calls it.
 *
 * It restates, in plain C and in the reference's operation order, the CPU
 * branch of the reference kernels:
 *   response()  ............ src/fastlisaresponse/cutils/LISAResponse.cu:431-672
 *   TDI_delay() ............ LISAResponse.cu:218-397
 *   interp() / interp_single()  LISAResponse.cu:149-207 / 110-147
 *   dot_product_1d(), xi_projections()  LISAResponse.cu:48-67
 * and the orbit-table evaluation of lisaanalysistools' Orbits class (restated;
 * that source is absent, see oracle/ref_shim/Detector.hpp for the rules).
 *
 * Pinned bit-for-bit against the reference's own CPU code compiled from the
 * reference checkout with the shim headers (oracle/Makefile, target `ref`) and
 * against golden fixtures generated by driving the reference's Python layer
 * (tests/golden/make_golden.py).
 */
#ifndef FLR_ORACLE_H
#define FLR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Orbit tables in the lisaanalysistools `pycppdetector_args` layout. */
typedef struct {
    double dt;            /* grid spacing of the tables [s]          */
    int N;                /* number of knots                         */
    const double *ltt;    /* [N][6] light travel times [s]           */
    const double *x;      /* [N][3][3] spacecraft positions [m]      */
    const int *links;     /* [6] link numbers, e.g. 12 23 31 13 32 21 */
    const int *sc_r;      /* [6] receiver spacecraft per link (1..3)  */
    const int *sc_e;      /* [6] emitter spacecraft per link (1..3)   */
} orc_orbits;

double orc_light_travel_time(const orc_orbits *o, double t, int link);
void orc_position(const orc_orbits *o, double t, int sc, double out[3]);

/* LISAResponse::get_response (LISAResponse.cu:674-718), CPU branch.
 * y_gw[6*num_delays] (link-major) is written for i in [start, num_delays-start).
 * If d_rec / d_em are non-NULL they receive the integer delays per (link, i)
 * (same layout as y_gw; untouched outside the computed range). */
void orc_get_response(const orc_orbits *o, double *y_gw, const double *t_data, const double *k,
                      const double *u, const double *v, int num_delays,
                      const double *input_c128, int order, double sampling_frequency,
                      const double *A, double deps, const double *E, int start,
                      int *d_rec, int *d_em);

/* LISAResponse::get_tdi_delays (LISAResponse.cu:399-429), CPU branch.
 * delayed_links[num_channels*num_delays] is accumulated into (callers zero it).
 * If d_out is non-NULL it receives the integer delay per (unit, i), laid out
 * [num_units][num_delays]. */
void orc_get_tdi_delays(const orc_orbits *o, double *delayed_links, const double *input_links,
                        int num_inputs, int num_delays, const double *t_arr,
                        const int *unit_starts, const int *unit_lengths,
                        const int *tdi_base_link, const int *tdi_link_combinations,
                        const double *tdi_signs, const int *channels, int num_units,
                        int order, double sampling_frequency, const double *A, double deps,
                        const double *E, int start, int *d_out);

/* The same, restricted to samples i in [max(start, i0), min(num_delays-start, i1)):
 * each output sample depends only on its own time and the inputs around its
 * delays, so a range is exactly the corresponding slice of the full result. */
void orc_get_response_range(const orc_orbits *o, double *y_gw, const double *t_data,
                            const double *k, const double *u, const double *v, int num_delays,
                            const double *input_c128, int order, double sampling_frequency,
                            const double *A, double deps, const double *E, int start,
                            int *d_rec, int *d_em, int i0, int i1);
void orc_get_tdi_delays_range(const orc_orbits *o, double *delayed_links,
                              const double *input_links, int num_inputs, int num_delays,
                              const double *t_arr, const int *unit_starts,
                              const int *unit_lengths, const int *tdi_base_link,
                              const int *tdi_link_combinations, const double *tdi_signs,
                              const int *channels, int num_units, int order,
                              double sampling_frequency, const double *A, double deps,
                              const double *E, int start, int *d_out, int i0, int i1);

#ifdef __cplusplus
}
#endif

#endif
