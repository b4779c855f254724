/* Oracle build shim (test infrastructure): the cuFFT API subset that
 * pm_periodic.c calls (cufftPlan3d, cufftExecR2C, cufftExecC2R), implemented on
 * the CPU in oracle/shim_impl.c with cuFFT's conventions: unnormalised
 * transforms, forward sign e^{-i}, inverse e^{+i}, row-major [nx][ny][nz] with the
 * last dimension halved to nz/2+1 complex values (padded to 2(nz/2+1) reals for
 * the in-place layout the reference uses). */
#ifndef CUCO_ORACLE_CUFFT_SHIM_H
#define CUCO_ORACLE_CUFFT_SHIM_H
#include "cuda_runtime_api.h"
typedef float cufftReal;
typedef struct { float x, y; } cufftComplex;
typedef int cufftHandle;
typedef int cufftResult;
typedef enum { CUFFT_R2C = 0x2a, CUFFT_C2R = 0x2c, CUFFT_C2C = 0x29 } cufftType;
#ifdef __cplusplus
extern "C" {
#endif
cufftResult cufftPlan3d(cufftHandle *plan, int nx, int ny, int nz, cufftType type);
cufftResult cufftExecR2C(cufftHandle plan, cufftReal *idata, cufftComplex *odata);
cufftResult cufftExecC2R(cufftHandle plan, cufftComplex *idata, cufftReal *odata);
#ifdef __cplusplus
}
#endif
#endif
