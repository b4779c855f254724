/* Oracle build shim (test infrastructure): begrun.c includes <gsl/gsl_rng.h> and
 * uses nothing from it. */
#ifndef CUCO_ORACLE_GSL_RNG_SHIM_H
#define CUCO_ORACLE_GSL_RNG_SHIM_H
#endif
