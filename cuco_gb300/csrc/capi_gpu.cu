// Reference-named GPU helpers (gravlist.cu:18-183, radixsort.h:47-81).
//
// These keep the reference's signatures and its void/abort error behaviour
// (cutilSafeCall prints and exits), work on the legacy default stream like the
// reference, and run the engine's kernels underneath.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "common.cuh"

namespace cuco {

struct CapiState {
    SIMPARAM sim;
    SOFTPARAM soft;
    bool have_sim = false;
    bool have_soft = false;
    float *table = nullptr;  // device copy of sim.shortrange_table
    int grid = 64;           // cell grid of calcHash (PMGRID in the reference)
};

CapiState &capi() {
    static CapiState s;
    return s;
}

void capi_set_grid(int G) { capi().grid = G; }

[[noreturn]] void capi_fail(const char *where, const char *what) {
    fprintf(stderr, "cuco_gb300: %s failed: %s\n", where, what);
    exit(1);
}

void capi_check(cudaError_t e, const char *where) {
    if (e != cudaSuccess) capi_fail(where, cudaGetErrorString(e));
}

void capi_status(cuco_status_t s, const char *where) {
    if (s != CUCO_OK) capi_fail(where, last_error());
}

}  // namespace cuco

using namespace cuco;

extern "C" {

void cudaInit(void) {
    int dev = 0;
    const char *env = getenv("CUCO_DEVICE");
    if (env) dev = atoi(env);
    capi_check(cudaSetDevice(dev), "cudaInit");
}

void allocateArray(void **devPtr, size_t size) { capi_check(cudaMalloc(devPtr, size), "allocateArray"); }

void freeArray(void *devPtr) { capi_check(cudaFree(devPtr), "freeArray"); }

void copyArrayFromDevice(void *host, void *device, int size) {
    capi_check(cudaMemcpy(host, device, (size_t)size, cudaMemcpyDeviceToHost), "copyArrayFromDevice");
}

void copyArrayToDevice(void *device, void *host, int offset, int size) {
    capi_check(cudaMemcpy((char *)device + offset, host, (size_t)size, cudaMemcpyHostToDevice),
               "copyArrayToDevice");
}

void setSimParam(SIMPARAM *p) {
    CapiState &s = capi();
    s.sim = *p;
    s.have_sim = true;
    if (!s.table) capi_check(cudaMalloc(&s.table, sizeof(float) * kNTab), "setSimParam");
    capi_check(cudaMemcpy(s.table, p->shortrange_table, sizeof(float) * kNTab, cudaMemcpyHostToDevice),
               "setSimParam");
}

void setSoftParam(SOFTPARAM *p) {
    capi().soft = *p;
    capi().have_soft = true;
}

void calcHash(uint *gridParticleHash, uint *gridParticleIndex, float *pos, uint numParticles) {
    CapiState &s = capi();
    if (!s.have_sim) capi_fail("calcHash", "setSimParam has not been called");
    capi_status(launch_cell_keys((const float4 *)pos, gridParticleHash, gridParticleIndex,
                                 numParticles, s.sim.to_grid_fac, s.grid, 0),
                "calcHash");
}

void reorderDataAndFindCellStart(uint *cellStart, uint *cellEnd, float *sortedPos,
                                 uint *gridParticleHash, uint *gridParticleIndex, float *oldPos,
                                 uint numParticles, uint numCells) {
    capi_status(launch_reorder_start_end(cellStart, cellEnd, (float4 *)sortedPos, gridParticleHash,
                                         gridParticleIndex, (const float4 *)oldPos, numParticles,
                                         numCells, 0),
                "reorderDataAndFindCellStart");
}

void cudaForceEvaluateShortrange(float *gravAccel, float *sortedPos, uint *gridParticleIndex,
                                 uint *cellStart, uint *cellEnd, uint numParticles, uint numCells) {
    CapiState &s = capi();
    if (!s.have_sim || !s.have_soft)
        capi_fail("cudaForceEvaluateShortrange", "setSimParam/setSoftParam have not been called");
    int G = (int)llround(cbrt((double)numCells));
    if ((uint)(G * G * G) != numCells) capi_fail("cudaForceEvaluateShortrange", "numCells is not a cube");
    ShortRangeParams p{};
    p.boxsize = s.sim.boxsize;
    p.gridfac = s.sim.to_grid_fac;
    p.cellw = s.sim.boxsize / G;
    p.rcut = s.sim.rcut;
    p.rcut2 = s.sim.rcut2;
    p.asmthfac = s.sim.asmthfac;
    // gravlist.cpp:67 keeps asmthfac in double; SIMPARAM carries Asmth itself
    p.asmthfac_d = 0.5 / (double)s.sim.asmth * (kNTab / 3.0);
    p.mass = s.sim.mass;
    p.G = s.sim.G;
    p.h = s.soft.h;
    p.hinv = s.soft.h_inv;
    p.h3inv = s.soft.h3_inv;
    p.grid = G;
    p.n = numParticles;
    KickArgs k{};
    // the work plan's scratch, grown on demand (like the reference's device
    // arrays, held until exit)
    static SRWork w{};
    if (w.seg_cap < numCells || w.heavy_cap < shortrange_heavy_cap(numParticles)) {
        cudaFree(w.heavy);
        cudaFree(w.seg_nt);
        cudaFree(w.ctl);
        w = SRWork{};
        const uint32_t hc = shortrange_heavy_cap(numParticles);
        capi_check(cudaMalloc(&w.heavy, sizeof(uint2) * hc), "cudaForceEvaluateShortrange");
        capi_check(cudaMalloc(&w.seg_nt, sizeof(uint32_t) * numCells), "cudaForceEvaluateShortrange");
        capi_check(cudaMalloc(&w.ctl, kSRCtlWords * sizeof(uint32_t)), "cudaForceEvaluateShortrange");
        capi_check(cudaMemset(w.ctl, 0, kSRCtlWords * sizeof(uint32_t)), "cudaForceEvaluateShortrange");
        w.heavy_cap = hc;
        w.seg_cap = numCells;
    }
    capi_status(launch_shortrange(p, (const float4 *)sortedPos, gridParticleIndex, cellStart, cellEnd,
                                  kCellStartEnd, s.table, (float4 *)gravAccel, k, w, 0),
                "cudaForceEvaluateShortrange");
    capi_status(shortrange_check(w.ctl, 0), "cudaForceEvaluateShortrange");
}

void radixSort(uint *keys, uint *values, uint *tempKeys, uint *tempValues, uint *counters,
               uint *countersSum, uint *blockOffsets, CUDPPHandle scanPlan, uint numElements,
               uint keyBits, bool flipBits) {
    (void)countersSum;
    (void)blockOffsets;
    (void)scanPlan;
    if (flipBits) capi_fail("radixSort", "flipBits is not supported");
    bool in_alt = false;
    int launches = 0;
    capi_status(sort_pairs(keys, values, values, tempKeys, tempValues, counters, numElements,
                           (int)keyBits, 6, 0, &in_alt, &launches),
                "radixSort");
    if (in_alt) {
        capi_check(cudaMemcpyAsync(keys, tempKeys, sizeof(uint) * numElements, cudaMemcpyDeviceToDevice, 0),
                   "radixSort");
        capi_check(cudaMemcpyAsync(values, tempValues, sizeof(uint) * numElements,
                                   cudaMemcpyDeviceToDevice, 0),
                   "radixSort");
    }
}

void radixSortKeysOnly(uint *keys, uint *tempKeys, uint *counters, uint *countersSum,
                       uint *blockOffsets, CUDPPHandle scanPlan, uint numElements, uint keyBits,
                       bool flipBits) {
    (void)countersSum;
    (void)blockOffsets;
    (void)scanPlan;
    if (flipBits) capi_fail("radixSortKeysOnly", "flipBits is not supported");
    bool in_alt = false;
    int launches = 0;
    capi_status(sort_pairs(keys, nullptr, nullptr, tempKeys, nullptr, counters, numElements,
                           (int)keyBits, 6, 0, &in_alt, &launches),
                "radixSortKeysOnly");
    if (in_alt)
        capi_check(cudaMemcpyAsync(keys, tempKeys, sizeof(uint) * numElements, cudaMemcpyDeviceToDevice, 0),
                   "radixSortKeysOnly");
}

// radixSortFloatKeys / radixSortFloatKeysOnly: order-preserving map of
// signed floats to unsigned keys and back (an involution pair: sign bit set
// -> all bits inverted, else sign bit set).
}  // extern "C"

namespace {
__global__ void k_float_to_key(uint32_t *__restrict__ k, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t u = k[i];
        k[i] = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    }
}
__global__ void k_key_to_float(uint32_t *__restrict__ k, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t u = k[i];
        k[i] = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    }
}
void float_keys(float *keys, uint32_t n, bool to_key, const char *where) {
    if (n == 0) return;
    const unsigned blocks = (n + 255) / 256;
    if (to_key)
        k_float_to_key<<<blocks, 256>>>(reinterpret_cast<uint32_t *>(keys), n);
    else
        k_key_to_float<<<blocks, 256>>>(reinterpret_cast<uint32_t *>(keys), n);
    capi_check(cudaGetLastError(), where);
}
}  // namespace

extern "C" {

void radixSortFloatKeys(float *keys, uint *values, float *tempKeys, uint *tempValues, uint *counters,
                        uint *countersSum, uint *blockOffsets, CUDPPHandle scanPlan, uint numElements,
                        uint keyBits, bool negativeKeys) {
    if (negativeKeys) float_keys(keys, numElements, true, "radixSortFloatKeys");
    radixSort(reinterpret_cast<uint *>(keys), values, reinterpret_cast<uint *>(tempKeys), tempValues, counters,
              countersSum, blockOffsets, scanPlan, numElements, keyBits, false);
    if (negativeKeys) float_keys(keys, numElements, false, "radixSortFloatKeys");
}

void radixSortFloatKeysOnly(float *keys, float *tempKeys, uint *counters, uint *countersSum,
                            uint *blockOffsets, CUDPPHandle scanPlan, uint numElements, uint keyBits,
                            bool negativeKeys) {
    if (negativeKeys) float_keys(keys, numElements, true, "radixSortFloatKeysOnly");
    radixSortKeysOnly(reinterpret_cast<uint *>(keys), reinterpret_cast<uint *>(tempKeys), counters, countersSum,
                      blockOffsets, scanPlan, numElements, keyBits, false);
    if (negativeKeys) float_keys(keys, numElements, false, "radixSortFloatKeysOnly");
}

void cuco_radixsort_overflow(uint numElements, uint maxElements) {
    char msg[128];
    snprintf(msg, sizeof msg, "%u elements exceed the %u this RadixSort was created for", numElements,
             maxElements);
    capi_fail("RadixSort::sort", msg);
}

void initDeviceParameters(void) {}

void checkCudaError(const char *msg) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) capi_fail(msg ? msg : "checkCudaError", cudaGetErrorString(e));
}

}  // extern "C"
