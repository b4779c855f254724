/* Oracle build shim (test infrastructure): predict.c and driftfac.c include
 * <gsl/gsl_math.h> but use nothing from it beyond <math.h>. */
#ifndef CUCO_ORACLE_GSL_MATH_SHIM_H
#define CUCO_ORACLE_GSL_MATH_SHIM_H
#include <math.h>
#endif
