/* Oracle build shim (test infrastructure). */
#ifndef CUCO_ORACLE_CUDA_RUNTIME_SHIM_H
#define CUCO_ORACLE_CUDA_RUNTIME_SHIM_H
#include "cuda_runtime_api.h"
#endif
