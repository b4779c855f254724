/* radixsort.h - the RadixSort class of the reference's radixsort.h:129-297,
 * over libcuco_gb300's stable LSD radix sort, with no CUDPP.
 *
 * The reference's short-range host code (gravlist.cpp:98, 164-167) creates
 * `sorter = new RadixSort(numParticles)` in linklist_init and calls
 * `sorter->sort(dGridParticleHash, dGridParticleIndex, numParticles, 18)`
 * every force evaluation; `RadixSort *sorter` itself is defined by the GPU
 * side (gravlist.cu:20, here libcuco_gb300.so).  A host that keeps
 * gravlist.cpp compiles against this header unchanged.
 *
 * What the class holds: temporary keys and values (maxElements words each;
 * values only when keysOnly is false) and the per-tile digit histogram the
 * library's radixSort reads through its `counters` argument
 * (32 * ceil(maxElements / 1024) words, the reference's own counter
 * allocation, radixsort.h:271-275).  The reference's countersSum and
 * blockOffsets buffers and its CUDPP scan plan are not needed: the library
 * turns the histogram into offsets in place.  Storage comes from
 * allocateArray/freeArray (gravlist.cu:33-43), which abort with a message on
 * failure as the reference's cutilSafeCall does.
 *
 * Semantics are the reference's: sort() orders (keys, values) stably by the
 * low keyBits bits of the keys, in place, on the legacy default stream; every
 * key must be below 2^keyBits (bits above keyBits are not masked: a pass may
 * cover a few bits more than keyBits, and such bits would take part in the
 * order, as they would in the reference's CUDPP sort).  values may be NULL
 * (keys only).  numElements must not exceed maxElements. */
#ifndef CUCO_RADIXSORT_H
#define CUCO_RADIXSORT_H

#include "cuco_gb300.h"

#ifdef __cplusplus

class RadixSort {
public:
    /* radixsort.h:142-152 */
    RadixSort(unsigned int maxElements, bool keysOnly = false)
        : mScanPlan(0), mNumElements(0), mTempKeys(0), mTempValues(0), mCounters(0), mCountersSum(0),
          mBlockOffsets(0) {
        initialize(maxElements, keysOnly);
    }

    /* radixsort.h:157-160 */
    ~RadixSort() { finalize(); }

    /* radixsort.h:170-187: unsigned keys, optional values */
    void sort(unsigned int *keys, unsigned int *values, unsigned int numElements, unsigned int keyBits) {
        checkCount(numElements);
        if (values == 0)
            radixSortKeysOnly(keys, mTempKeys, mCounters, mCountersSum, mBlockOffsets, mScanPlan, numElements,
                              keyBits, false);
        else
            radixSort(keys, values, mTempKeys, mTempValues, mCounters, mCountersSum, mBlockOffsets, mScanPlan,
                      numElements, keyBits, false);
    }

    /* radixsort.h:199-218: float keys (negativeKeys: signed floats), optional values */
    void sort(float *keys, unsigned int *values, unsigned int numElements, unsigned int keyBits,
              bool negativeKeys) {
        checkCount(numElements);
        if (values == 0)
            radixSortFloatKeysOnly(keys, (float *)mTempKeys, mCounters, mCountersSum, mBlockOffsets, mScanPlan,
                                   numElements, keyBits, negativeKeys);
        else
            radixSortFloatKeys(keys, values, (float *)mTempKeys, mTempValues, mCounters, mCountersSum,
                               mBlockOffsets, mScanPlan, numElements, keyBits, negativeKeys);
    }

    /* radixsort.h:221-222 */
    static const unsigned int CTA_SIZE = 256;
    static const unsigned int WARP_SIZE = 32;

protected:
    CUDPPHandle mScanPlan;       /* kept for layout; no plan is made */
    unsigned int mNumElements;   /* capacity of the temporaries */
    unsigned int *mTempKeys;
    unsigned int *mTempValues;
    unsigned int *mCounters;     /* per-tile digit histogram */
    unsigned int *mCountersSum;  /* unused (NULL) */
    unsigned int *mBlockOffsets; /* unused (NULL) */

    /* radixsort.h:251-280 */
    void initialize(unsigned int numElements, bool keysOnly) {
        initDeviceParameters();
        mNumElements = numElements;
        const unsigned int blocks = (numElements + CTA_SIZE * 4 - 1) / (CTA_SIZE * 4);
        const size_t words = numElements ? numElements : 1;
        allocateArray((void **)&mTempKeys, words * sizeof(unsigned int));
        if (!keysOnly) allocateArray((void **)&mTempValues, words * sizeof(unsigned int));
        allocateArray((void **)&mCounters, (size_t)WARP_SIZE * (blocks ? blocks : 1) * sizeof(unsigned int));
        checkCudaError("RadixSort::initialize()");
    }

    /* radixsort.h:285-296 */
    void finalize() {
        if (mTempKeys) freeArray(mTempKeys);
        if (mTempValues) freeArray(mTempValues);
        if (mCounters) freeArray(mCounters);
        mTempKeys = mTempValues = mCounters = 0;
        checkCudaError("RadixSort::finalize()");
    }

    void checkCount(unsigned int numElements) const {
        if (numElements > mNumElements) cuco_radixsort_overflow(numElements, mNumElements);
    }

private:
    RadixSort(const RadixSort &);
    RadixSort &operator=(const RadixSort &);
};

/* gravlist.cu:20 (declared in proto.cuh:60); defined by libcuco_gb300.so and
 * created by linklist_init, as gravlist.cpp:98 does. */
extern RadixSort *sorter;

#endif /* __cplusplus */
#endif
