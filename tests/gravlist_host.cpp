// A host program written the way the reference's gravlist.cpp drives the GPU
// short-range pipeline (gravlist.cpp:48-115 linklist_init allocations and
// `sorter = new RadixSort(numParticles)`, gravlist.cpp:148-193 calcHash ->
// sorter->sort -> reorderDataAndFindCellStart), compiled against this
// library's include/radixsort.h and include/cuco_gb300.h only (no CUDA
// headers, no CUDPP).  tests/test_gpu_radixsort_host.py builds it with g++,
// runs it and compares what it writes with the oracle.
//
// usage: gravlist_host <in.bin> <out.bin>
//   in.bin : int32 n, int32 G, float32 boxsize, float32 pos[n][3],
//            float32 fkeys[n] (float keys for the RadixSort float overload)
//   out.bin: uint32 hash[n], uint32 index[n], uint32 cellStart[G^3],
//            uint32 cellEnd[G^3], float32 sortedPos[n][4],
//            uint32 keysOnly[n] (the hashes sorted with values = NULL),
//            float32 fkeys_sorted[n], uint32 fvals[n]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cuco_gb300.h"
#include "radixsort.h"

static void die(const char *m) {
    fprintf(stderr, "gravlist_host: %s\n", m);
    exit(2);
}

int main(int argc, char **argv) {
    if (argc != 3) die("usage: gravlist_host in.bin out.bin");
    FILE *f = fopen(argv[1], "rb");
    if (!f) die("cannot open input");
    int n = 0, G = 0;
    float L = 0;
    if (fread(&n, 4, 1, f) != 1 || fread(&G, 4, 1, f) != 1 || fread(&L, 4, 1, f) != 1) die("short header");
    std::vector<float> pos(3 * (size_t)n), fkeys(n);
    if (fread(pos.data(), 4, pos.size(), f) != pos.size()) die("short positions");
    if (fread(fkeys.data(), 4, fkeys.size(), f) != fkeys.size()) die("short float keys");
    fclose(f);
    const unsigned numParticles = (unsigned)n, numGridCells = (unsigned)(G * G * G);

    cudaInit();
    cuco_dropin_configure(G, G);

    // gravlist.cpp:56-67,100-114: the constants calcHash uses (the table is
    // not needed for keys and the sort)
    SIMPARAM sim;
    memset(&sim, 0, sizeof sim);
    sim.boxsize = L;
    sim.boxhalf = 0.5f * L;
    sim.to_grid_fac = (float)G / L;
    setSimParam(&sim);

    // gravlist.cpp:88-98: host staging, device arrays and the sorter
    std::vector<float> hPos4(4 * (size_t)n);
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) hPos4[4 * (size_t)i + d] = pos[3 * (size_t)i + d];
    float *dPos = 0, *dSorted = 0;
    unsigned *dHash = 0, *dIndex = 0, *dStart = 0, *dEnd = 0;
    allocateArray((void **)&dPos, 16 * (size_t)n);
    allocateArray((void **)&dSorted, 16 * (size_t)n);
    allocateArray((void **)&dHash, 4 * (size_t)n);
    allocateArray((void **)&dIndex, 4 * (size_t)n);
    allocateArray((void **)&dStart, 4 * (size_t)numGridCells);
    allocateArray((void **)&dEnd, 4 * (size_t)numGridCells);
    delete sorter;  // the library's own linklist_init may have made one
    sorter = new RadixSort(numParticles);

    // gravlist.cpp:155-178
    copyArrayToDevice(dPos, hPos4.data(), 0, 16 * n);
    calcHash(dHash, dIndex, dPos, numParticles);
    sorter->sort(dHash, dIndex, numParticles, 18);
    reorderDataAndFindCellStart(dStart, dEnd, dSorted, dHash, dIndex, dPos, numParticles, numGridCells);
    checkCudaError("gravlist_host pipeline");

    std::vector<unsigned> hash(n), index(n), start(numGridCells), end(numGridCells), keys_only(n), fvals(n);
    std::vector<float> sorted(4 * (size_t)n), fsorted(n);
    copyArrayFromDevice(hash.data(), dHash, 4 * n);
    copyArrayFromDevice(index.data(), dIndex, 4 * n);
    copyArrayFromDevice(start.data(), dStart, 4 * (int)numGridCells);
    copyArrayFromDevice(end.data(), dEnd, 4 * (int)numGridCells);
    copyArrayFromDevice(sorted.data(), dSorted, 16 * n);

    // keys only (values = NULL): the unsorted hashes again
    calcHash(dHash, dIndex, dPos, numParticles);
    sorter->sort(dHash, (unsigned *)0, numParticles, 18);
    copyArrayFromDevice(keys_only.data(), dHash, 4 * n);

    // the float-key overload with signed keys and values 0..n-1
    float *dF = 0;
    allocateArray((void **)&dF, 4 * (size_t)n);
    for (int i = 0; i < n; ++i) fvals[i] = (unsigned)i;
    copyArrayToDevice(dF, fkeys.data(), 0, 4 * n);
    copyArrayToDevice(dIndex, fvals.data(), 0, 4 * n);
    sorter->sort(dF, dIndex, numParticles, 32, true);
    copyArrayFromDevice(fsorted.data(), dF, 4 * n);
    copyArrayFromDevice(fvals.data(), dIndex, 4 * n);
    checkCudaError("gravlist_host float keys");

    delete sorter;
    sorter = 0;
    freeArray(dF);
    freeArray(dPos);
    freeArray(dSorted);
    freeArray(dHash);
    freeArray(dIndex);
    freeArray(dStart);
    freeArray(dEnd);

    FILE *o = fopen(argv[2], "wb");
    if (!o) die("cannot open output");
    fwrite(hash.data(), 4, n, o);
    fwrite(index.data(), 4, n, o);
    fwrite(start.data(), 4, numGridCells, o);
    fwrite(end.data(), 4, numGridCells, o);
    fwrite(sorted.data(), 4, 4 * (size_t)n, o);
    fwrite(keys_only.data(), 4, n, o);
    fwrite(fsorted.data(), 4, n, o);
    fwrite(fvals.data(), 4, n, o);
    fclose(o);
    printf("gravlist_host ok: %d particles, %u cells\n", n, numGridCells);
    return 0;
}
