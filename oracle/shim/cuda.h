/* Oracle build shim (test infrastructure): pm_periodic.c includes <cuda.h> but
 * uses nothing from it beyond what cuda_runtime_api.h declares. */
#ifndef CUCO_ORACLE_CUDA_SHIM_H
#define CUCO_ORACLE_CUDA_SHIM_H
#include "cuda_runtime_api.h"
#endif
