/* Oracle build shim (test infrastructure): the few CUDA runtime declarations the
 * reference's host code names.  The oracle build runs on the CPU only; the
 * definitions in oracle/shim_impl.c back "device" memory with host memory. */
#ifndef CUCO_ORACLE_CUDA_RUNTIME_API_SHIM_H
#define CUCO_ORACLE_CUDA_RUNTIME_API_SHIM_H
#include <stddef.h>
typedef unsigned int uint;
typedef int cudaError_t;
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3
};
#ifdef __cplusplus
extern "C" {
#endif
cudaError_t cudaMalloc(void **ptr, size_t size);
cudaError_t cudaFree(void *ptr);
cudaError_t cudaMemcpy(void *dst, const void *src, size_t size, enum cudaMemcpyKind kind);
#ifdef __cplusplus
}
#endif
#endif
