/* Oracle build shim (test infrastructure).
 *
 * Pulls in the reference's proto.cuh by path, then repairs the one defect that
 * keeps the reference CPU short-range path from running: the linked-list arrays
 * `ll` and `ihoc` are file-static pointers in gravlist.cpp whose mallocs are
 * commented out (gravlist.cpp:25-26,53-54), so gravity_linklist() dereferences
 * NULL.  The macros below turn every use of those two names in gravlist.cpp into
 * a call that returns storage owned by the oracle harness (sized NumPart and
 * PMGRID^3 ints).  The declaration `static int * ll;` becomes a redeclaration of
 * the static function defined here, so the source file itself is untouched. */
#ifndef CUCO_ORACLE_PROTO_CUH_SHIM_H
#define CUCO_ORACLE_PROTO_CUH_SHIM_H
#include CUCO_REF_PROTO_CUH
#ifdef __cplusplus
extern "C" {
#endif
int *cuco_ref_ll_storage(void);
int *cuco_ref_ihoc_storage(void);
static int *cuco_ref_ll(void) { return cuco_ref_ll_storage(); }
static int *cuco_ref_ihoc(void) { return cuco_ref_ihoc_storage(); }
#ifdef __cplusplus
}
#endif
#define ll (cuco_ref_ll())
#define ihoc (cuco_ref_ihoc())
#endif
