// Allocation-free variant of the stable radix sort.
//
// cuco_radix_sort_noalloc sorts (keys, values) like radixSort but takes its
// scratch - the alternate key/value buffers and the per-tile digit histogram -
// from one fixed array compiled into this library, so a call never allocates
// device memory.  It exists for callers that must not allocate on the path
// where they sort: cudaMalloc/cudaFree can synchronize the device and stall
// every other stream (the serving loop interleaves many jobs on one GPU), and
// a host that hands each job a fixed slice of HBM up front (an admission
// budget, or a framework's caching allocator owning the device memory) cannot
// let a library grow its footprint in the middle of a run.
//
// Limits and sharing:
//   * at most kNoAllocMaxN = 2^20 elements per call; larger calls are rejected
//     with CUCO_ERR_INVALID before anything is launched;
//   * the array takes 8.25 MiB of device memory on every GPU where this
//     library's kernels are loaded, held until the process exits;
//   * every call on a device uses the same array, which keeps whatever the
//     last call left in it.  Nothing in it needs to start at zero: each pass
//     rewrites every histogram entry it reads and every buffer word it reads
//     back.  Calls whose work overlaps on the GPU (different streams, or
//     different host threads, without ordering between them) race on the
//     array and corrupt each other's results: order them on one stream;
//   * host code cannot pass the array's name to a kernel (in host code the
//     name is a host-side stand-in, not a device address).  The first call on
//     each device, with that device current, looks the address up with
//     cudaGetSymbolAddress and caches it; make that first call before
//     capturing any work on that device into a stream capture.  The cached
//     address lives as long as the device's context: a cudaDeviceReset after
//     the first call is not supported (the address would be stale);
//   * keys must be below 2^key_bits: the passes split key_bits into equal
//     digits of 4 to 8 bits, which may cover a few bits above key_bits, and
//     bits set there would take part in the order.
#include <mutex>

#include "common.cuh"

namespace cuco {
namespace {

constexpr uint32_t kNoAllocMaxN = 1u << 20;
constexpr uint32_t kTile = 4096;  // keys per sort tile (sort.cu)
constexpr size_t kHistWords = 256u * ((kNoAllocMaxN + kTile - 1) / kTile);
constexpr size_t kScratchWords = 2u * kNoAllocMaxN + kHistWords;

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
uint32_t *g_scratch_ptr[kMaxDevices] = {};

}  // namespace

// The scratch array: alternate keys, alternate values, digit histogram.
static __device__ __align__(256) uint32_t g_sort_scratch[kScratchWords];

}  // namespace cuco

using namespace cuco;

extern "C" cuco_status_t cuco_radix_sort_noalloc(uint32_t *keys, uint32_t *values, uint32_t n,
                                                 uint32_t key_bits, void *stream) {
    if (n > kNoAllocMaxN) {
        set_error("cuco_radix_sort_noalloc: " + std::to_string(n) +
                  " elements exceed the fixed scratch limit of " + std::to_string(kNoAllocMaxN));
        return CUCO_ERR_INVALID;
    }
    if ((n && !keys) || key_bits < 1 || key_bits > 32) {
        set_error("cuco_radix_sort_noalloc: null keys or key_bits outside 1..32");
        return CUCO_ERR_INVALID;
    }
    if (n == 0) return CUCO_OK;
    int dev = 0;
    CUCO_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("cuco_radix_sort_noalloc: device ordinal beyond the supported 64");
        return CUCO_ERR_INVALID;
    }
    uint32_t *scratch;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_scratch_ptr[dev]) {
            void *p = nullptr;
            CUCO_TRY_CUDA(cudaGetSymbolAddress(&p, g_sort_scratch));
            g_scratch_ptr[dev] = static_cast<uint32_t *>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    uint32_t *tmp_keys = scratch;
    uint32_t *tmp_vals = scratch + kNoAllocMaxN;
    uint32_t *hist = scratch + 2u * kNoAllocMaxN;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    bool in_alt = false;
    int launches = 0;
    // digits of at most 8 bits: the histogram holds 2^8 * ceil(n/4096) words
    CUCO_TRY(sort_pairs(keys, values, values, tmp_keys, values ? tmp_vals : nullptr, hist, n,
                        (int)key_bits, 8, s, &in_alt, &launches));
    if (in_alt) {
        CUCO_TRY_CUDA(cudaMemcpyAsync(keys, tmp_keys, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
        if (values)
            CUCO_TRY_CUDA(cudaMemcpyAsync(values, tmp_vals, sizeof(uint32_t) * n,
                                          cudaMemcpyDeviceToDevice, s));
    }
    return CUCO_OK;
}
