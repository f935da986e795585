// Test infrastructure: a flat C entry point over the reference's own CPU
// implementation (LISAResponse.cu compiled as C++ with the shim headers in this
// folder).  Used only to pin the oracle restatement and to generate golden
// fixtures; never linked into the product.
//
// The argument lists are those of the reference's pybind11 wrappers
// (binding_flr.cxx:16-58) with the orbit tables of OrbitsWrap
// (binding_flr.hpp:35-51) in front.
#include "LISAResponse.hh"

extern "C" {

int flr_ref_get_response(double orb_dt, int orb_N, double *n_arr, double *ltt_arr, double *x_arr,
                         int *links, int *sc_r, int *sc_e, double armlength,
                         double *y_gw, double *t_data, double *k_in, double *u_in, double *v_in,
                         double dt, int num_delays, void *input_in, int num_inputs, int order,
                         double sampling_frequency, int buffer_integer, double *A_in, double deps,
                         int num_A, double *E_in, int projections_start_ind)
{
    OrbitsCPU orbits(orb_dt, orb_N, n_arr, ltt_arr, x_arr, links, sc_r, sc_e, armlength);
    LISAResponseCPU response(&orbits);
    response.get_response(y_gw, t_data, k_in, u_in, v_in, dt, num_delays,
                          static_cast<cmplx *>(input_in), num_inputs, order, sampling_frequency,
                          buffer_integer, A_in, deps, num_A, E_in, projections_start_ind);
    return 0;
}

int flr_ref_get_tdi_delays(double orb_dt, int orb_N, double *n_arr, double *ltt_arr, double *x_arr,
                           int *links, int *sc_r, int *sc_e, double armlength,
                           double *delayed_links, double *input_links, int num_inputs,
                           int num_delays, double *t_arr, int *unit_starts, int *unit_lengths,
                           int *tdi_base_link, int *tdi_link_combinations, double *tdi_signs_in,
                           int *channels, int num_units, int num_channels, int order,
                           double sampling_frequency, int buffer_integer, double *A_in,
                           double deps, int num_A, double *E_in, int tdi_start_ind)
{
    OrbitsCPU orbits(orb_dt, orb_N, n_arr, ltt_arr, x_arr, links, sc_r, sc_e, armlength);
    LISAResponseCPU response(&orbits);
    response.get_tdi_delays(delayed_links, input_links, num_inputs, num_delays, t_arr, unit_starts,
                            unit_lengths, tdi_base_link, tdi_link_combinations, tdi_signs_in,
                            channels, num_units, num_channels, order, sampling_frequency,
                            buffer_integer, A_in, deps, num_A, E_in, tdi_start_ind);
    return 0;
}

}  // extern "C"
