/* CPU oracle for the Euler operators (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference operator headers (euler_operators/), used by the
 * tests, the smoke check and bench.py's CPU-baseline leg as the parity reference.  It is
 * pinned bit-for-bit against the reference itself (oracle/_ref, built from the
 * reference headers by oracle/Makefile) and against the golden fixtures under
 * tests/golden/.  Build: see oracle/Makefile (-O2 -ffp-contract=off -fopenmp).
 */
#include <float.h>
#include <math.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "euler_oracle.h"

#define REAL double
#define SUF f64
#define SQRT sqrt
#define FABS fabs
#define REAL_MAX DBL_MAX
#include "euler_oracle_body.h"
#undef REAL
#undef SUF
#undef SQRT
#undef FABS
#undef REAL_MAX

#define REAL float
#define SUF f32
#define SQRT sqrtf
#define FABS fabsf
#define REAL_MAX FLT_MAX
#include "euler_oracle_body.h"
#undef REAL
#undef SUF
#undef SQRT
#undef FABS
#undef REAL_MAX

/* The number of OpenMP threads a parallel region of this library uses. */
int oracle_omp_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
