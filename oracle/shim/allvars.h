/* Oracle build shim (test infrastructure, never shipped in the product path).
 *
 * The reference fixes the PM mesh size at compile time (allvars.h:9,
 * `#define PMGRID 64`).  The oracle recipe compiles the reference sources where
 * they lie, with `-I-` so that this directory is searched before the source
 * directory; this header pulls in the reference's own allvars.h by path and then
 * swaps PMGRID for the value the recipe asks for (CUCO_PMGRID).  Nothing else in
 * the reference header changes. */
#ifndef CUCO_ORACLE_ALLVARS_SHIM_H
#define CUCO_ORACLE_ALLVARS_SHIM_H
#include CUCO_REF_ALLVARS
#undef PMGRID
#define PMGRID CUCO_PMGRID
#endif
