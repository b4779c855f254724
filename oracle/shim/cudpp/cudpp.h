/* Oracle build shim (test infrastructure): the CUDPP names that the reference's
 * radixsort.h mentions.  The CPU oracle never sorts on a device, so the plan
 * calls are no-ops that report success. */
#ifndef CUCO_ORACLE_CUDPP_SHIM_H
#define CUCO_ORACLE_CUDPP_SHIM_H
typedef unsigned long CUDPPHandle;
typedef int CUDPPResult;
enum CUDPPAlgorithm { CUDPP_SCAN = 0 };
enum CUDPPDatatype { CUDPP_UINT = 0 };
enum CUDPPOperator { CUDPP_ADD = 0 };
enum CUDPPOption { CUDPP_OPTION_FORWARD = 1, CUDPP_OPTION_EXCLUSIVE = 4 };
typedef struct {
    int algorithm;
    int datatype;
    int op;
    unsigned int options;
} CUDPPConfiguration;
#ifdef __cplusplus
extern "C" {
#endif
CUDPPResult cudppPlan(CUDPPHandle *plan, CUDPPConfiguration config, size_t n, size_t rows, size_t pitch);
CUDPPResult cudppDestroyPlan(CUDPPHandle plan);
#ifdef __cplusplus
}
#endif
#endif
