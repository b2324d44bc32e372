/* CPU oracle for the Euler operators (TEST INFRASTRUCTURE ONLY).
 *
 * Declarations of the C restatement in euler_oracle.c.  Bundles are 5 host
 * pointers in the reference's field order: prim = (d, p, ux0, ux1, ux2) and
 * cons = (d, e, mx0, mx1, mx2), each layout_left over n0*n1*n2 cells.
 */
#ifndef EULER_ORACLE_H
#define EULER_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define EULER_ORACLE_DECLARE(SUF, REAL)                                                            \
    void oracle_init_implode_##SUF(REAL* const* prim, int n0, int n1, int n2, REAL dx0, REAL dx1, REAL dx2); \
    void oracle_init_step_##SUF(REAL* const* prim, int n0, int n1, int n2, double dx0, double dx1, double dx2,   \
                                double c, double rho_in, double p_in, double rho_out, double p_out);      \
    void oracle_prim_to_cons_##SUF(REAL const* const* prim, REAL* const* cons, int n0, int n1, int n2, REAL gamma); \
    void oracle_cons_to_prim_##SUF(REAL const* const* cons, REAL* const* prim, int n0, int n1, int n2, REAL gamma); \
    REAL oracle_time_step_##SUF(REAL const* const* prim, int n0, int n1, int n2, REAL gamma, REAL dx0, REAL dx1, REAL dx2); \
    void oracle_godunov_##SUF(REAL const* const* prim, REAL* const* cons, int n0, int n1, int n2, REAL gamma,   \
                              REAL dx0, REAL dx1, REAL dx2, REAL dt);                            \
    REAL oracle_step_##SUF(REAL* const* prim, REAL* const* cons, int n0, int n1, int n2, REAL gamma, REAL dx0, \
                           REAL dx1, REAL dx2, REAL cfl);                                        \
    void oracle_simulate_##SUF(REAL* const* prim, REAL* const* cons, int n0, int n1, int n2, REAL gamma,       \
                               REAL dx0, REAL dx1, REAL dx2, REAL cfl, int nsteps, double* t_out);          \
    void oracle_hllc_face_##SUF(int dir, REAL gamma, REAL const* qL, REAL const* qR, REAL* f);

EULER_ORACLE_DECLARE(f64, double)
EULER_ORACLE_DECLARE(f32, float)

#undef EULER_ORACLE_DECLARE

int oracle_omp_threads(void);

#ifdef __cplusplus
}
#endif

#endif
