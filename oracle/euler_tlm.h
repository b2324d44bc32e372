/* Host tangent-linear model of the Euler time step (TEST INFRASTRUCTURE ONLY).
 *
 * Forward-mode derivative of the reference's step with dt held fixed, in
 * plain C (euler_tlm.c): each function carries a state and a tangent of the
 * same layout as euler_oracle.h (5 host arrays per bundle, layout_left).
 * Values are computed exactly as the oracle computes them, so a tangent run
 * follows the oracle's trajectory bit for bit.  At exact ties of the HLLC
 * flux (equal min/max arguments, ustar == 0 in the subsonic case) the
 * tangent is the mean of the two one-sided tangents, as a central difference
 * measures.
 */
#ifndef EULER_TLM_H
#define EULER_TLM_H

#ifdef __cplusplus
extern "C" {
#endif

void oracle_tlm_prim_to_cons_f64(double const* const* prim, double const* const* dprim, double* const* cons,
                                 double* const* dcons, int n0, int n1, int n2, double gamma);
void oracle_tlm_cons_to_prim_f64(double const* const* cons, double const* const* dcons, double* const* prim,
                                 double* const* dprim, int n0, int n1, int n2, double gamma);
void oracle_tlm_godunov_f64(double const* const* prim, double const* const* dprim, double* const* cons,
                            double* const* dcons, int n0, int n1, int n2, double gamma, double dx0, double dx1,
                            double dx2, double dt);
/* cons = prim_to_cons(prim), then nsteps of godunov(dts[n]) + cons_to_prim,
 * value and tangent; prim/dprim hold the initial state on entry and the
 * final one on exit. */
void oracle_tlm_simulate_f64(double* const* prim, double* const* dprim, double* const* cons, double* const* dcons,
                             int n0, int n1, int n2, double gamma, double dx0, double dx1, double dx2,
                             double const* dts, int nsteps);

#ifdef __cplusplus
}
#endif

#endif
