// Cell keys, stable LSD radix sort, and the reorder / cell-bound kernels.
//
// Reference: calcHashD (gravlist_kernel.cu:92-118), RadixSort::sort ->
// radixSort (radixsort.h:170-187, radixsort.cu:1048-1145), and
// reorderDataAndFindCellStartD (gravlist_kernel.cu:121-160).
//
// The sort is a three-kernel-per-pass LSD radix sort designed for sm_103a:
//   1. k_sort_hist:   per 4096-key tile, a digit histogram (warp match_any
//                     aggregation into shared-memory counters);
//   2. k_sort_scan:   one CTA per digit turns its tile counts into inclusive
//                     prefixes over the tiles (the digit's total is the last);
//   3. k_sort_scatter: each tile ranks its keys stably with warp ballots
//                     (the lanes sharing a digit are found from RB ballots, the
//                     rank is a popcount below the lane), takes each run's
//                     global offset from the digit totals and its own
//                     prefix, stages the tile in digit order in shared memory
//                     and writes out digit runs with coalesced stores.
// Digits are 4..8 bits; a pass count of ceil(bits/8) with equal digit widths
// is used (18-bit keys: three 6-bit passes).
#include "common.cuh"

namespace cuco {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys
constexpr int kSortWarps = kSortThreads / 32;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int cell_coord(float t, int G) {
    int c = (int)t;  // truncation toward zero (cvt.rzi), as calcHashD's int3 assignment
    c = c < 0 ? 0 : c;
    return c >= G ? G - 1 : c;
}

__global__ void k_cell_keys(const float4 *__restrict__ pos, uint32_t *__restrict__ keys,
                            uint32_t *__restrict__ idx, uint32_t n, float gridfac, int G) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = pos[i];
        int ix = cell_coord(__fmul_rn(gridfac, p.x), G);
        int iy = cell_coord(__fmul_rn(gridfac, p.y), G);
        int iz = cell_coord(__fmul_rn(gridfac, p.z), G);
        keys[i] = ((uint32_t)ix * G + iy) * G + iz;
        if (idx) idx[i] = i;
    }
}

template <int RB>
__global__ void __launch_bounds__(kSortThreads)
    k_sort_hist(const uint32_t *__restrict__ keys, uint32_t n, int shift,
                uint32_t *__restrict__ hist, uint32_t tiles) {
    constexpr int RADIX = 1 << RB;
    __shared__ uint32_t h[RADIX];
    for (int d = threadIdx.x; d < RADIX; d += kSortThreads) h[d] = 0;
    __syncthreads();
    const uint32_t tile = blockIdx.x;
    const uint32_t base = tile * kSortTile;
    const int lane = threadIdx.x & 31;
#pragma unroll 4
    for (int k = 0; k < kSortItems; ++k) {
        uint32_t i = base + k * kSortThreads + threadIdx.x;
        bool valid = i < n;
        uint32_t d = valid ? (keys[i] >> shift) & (RADIX - 1) : (uint32_t)RADIX;
        uint32_t peers = __match_any_sync(kFull, d);
        if (valid && lane == __ffs(peers) - 1) atomicAdd(&h[d], (uint32_t)__popc(peers));
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += kSortThreads) hist[d * tiles + tile] = h[d];
}

// hist[d*tiles + t] (count of digit d in tile t) -> the inclusive prefix of
// those counts over the tiles, one CTA per digit.  A digit's total is then its
// last entry, and the scatter derives every run's global offset from these
// (no second pass over the table, no scratch beyond it).
// zero_next (or null): the next pass's histogram, whose row of this digit is
// cleared here for the scatter to count into.
__global__ void __launch_bounds__(kSortThreads) k_sort_scan(uint32_t *__restrict__ hist, uint32_t tiles,
                                                            uint32_t *__restrict__ zero_next) {
    __shared__ uint32_t wsum[kSortWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t *h = hist + (size_t)blockIdx.x * tiles;
    if (zero_next)
        for (uint32_t t = threadIdx.x; t < tiles; t += kSortThreads) zero_next[(size_t)blockIdx.x * tiles + t] = 0u;
    uint32_t carry = 0;
    for (uint32_t t0 = 0; t0 < tiles; t0 += kSortThreads) {
        const uint32_t t = t0 + threadIdx.x;
        const uint32_t v = t < tiles ? h[t] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, incl, off);
            if (lane >= off) incl += y;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        uint32_t before = 0, all = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t x = wsum[w];
            before += w < warp ? x : 0u;
            all += x;
        }
        if (t < tiles) h[t] = carry + before + incl;
        carry += all;
        __syncthreads();  // wsum is rewritten by the next round
    }
}

// NEXT: also count the next pass's digit (at next_shift) of every key placed,
// per destination tile, into next_hist (cleared by this pass's scan): the
// histogram the next pass would build from this pass's output.
template <int RB, bool WITH_VALS, bool SINGLE_TILE, bool NEXT>
__global__ void __launch_bounds__(kSortThreads, 4)
    k_sort_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                   uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, uint32_t n,
                   int shift, const uint32_t *__restrict__ hist, uint32_t tiles,
                   uint32_t *__restrict__ next_hist, int next_shift) {
    constexpr int RADIX = 1 << RB;
    __shared__ uint32_t wcnt[kSortWarps][RADIX];
    __shared__ uint32_t dstart[RADIX];
    __shared__ uint32_t gbase[RADIX];
    __shared__ uint32_t skeys[kSortTile];
    __shared__ uint32_t svals[WITH_VALS ? kSortTile : 1];

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tile = blockIdx.x;
    const uint32_t base = tile * kSortTile;
    const uint32_t lt = (1u << lane) - 1u;
    for (int e = threadIdx.x; e < kSortWarps * RADIX; e += kSortThreads) (&wcnt[0][0])[e] = 0;
    __syncthreads();

    // Warp w owns tile elements [w*512, w*512+512); item k covers 32 of them in
    // lane order, so (k, lane) order is input order and the ranks are stable.
    // The ranks (below 4096) are kept two to a register; keys and values are
    // read again when they are placed, so few registers stay live.
    uint32_t rank2[kSortItems / 2];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t i = base + warp * (32 * kSortItems) + k * 32 + lane;
        const bool valid = i < n;
        const uint32_t key = valid ? kin[i] : 0xffffffffu;
        const uint32_t d = (key >> shift) & (RADIX - 1);
        uint32_t peers = __ballot_sync(kFull, valid);
#pragma unroll
        for (int b = 0; b < RB; ++b) {
            const uint32_t bit = (d >> b) & 1u;
            const uint32_t m = __ballot_sync(kFull, bit);
            peers &= bit ? m : ~m;
        }
        const uint32_t cnt = wcnt[warp][d];
        const uint32_t r = cnt + __popc(peers & lt);
        if (k & 1)
            rank2[k >> 1] |= r << 16;
        else
            rank2[k >> 1] = r;
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = cnt + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += kSortThreads) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            uint32_t c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
        dstart[d] = run;
    }
    __syncthreads();
    if (warp == 0) {
        // exclusive scan of this tile's digit counts; and, over the digits,
        // of the digit totals (the last tile's inclusive prefixes)
        constexpr int PER = (RADIX + 31) / 32;
        uint32_t v[PER], tv[PER], s = 0, ts = 0;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int d = lane * PER + j;
            v[j] = d < RADIX ? dstart[d] : 0;
            tv[j] = (!SINGLE_TILE && d < RADIX) ? hist[(size_t)d * tiles + tiles - 1] : 0;
            s += v[j];
            ts += tv[j];
        }
        uint32_t incl = s, tincl = ts;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, incl, off), ty = __shfl_up_sync(kFull, tincl, off);
            if (lane >= off) incl += y, tincl += ty;
        }
        uint32_t run = incl - s, trun = tincl - ts;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int d = lane * PER + j;
            if (d < RADIX) {
                dstart[d] = run;
                // the run of digit d from this tile starts after the lower
                // digits' totals and this digit's runs from earlier tiles
                gbase[d] = SINGLE_TILE ? run : trun + hist[(size_t)d * tiles + tile] - v[j];
                run += v[j];
                trun += tv[j];
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t i = base + warp * (32 * kSortItems) + k * 32 + lane;
        if (i < n) {
            const uint32_t key = kin[i];
            const uint32_t d = (key >> shift) & (RADIX - 1);
            const uint32_t lp = dstart[d] + wcnt[warp][d] + ((rank2[k >> 1] >> (16 * (k & 1))) & 0xffffu);
            skeys[lp] = key;
            if (WITH_VALS) svals[lp] = vin ? vin[i] : i;
        }
    }
    __syncthreads();
    const uint32_t tile_n = min((uint32_t)kSortTile, n - base);
    // (the loop's trip count is the same for every lane of a warp: tile_n
    // only cuts the last warp's lanes, which still vote)
    for (uint32_t j0 = 0; j0 < (uint32_t)kSortTile; j0 += kSortThreads) {
        const uint32_t j = j0 + threadIdx.x;
        const bool in = j < tile_n;
        uint32_t kk = 0, o = 0;
        if (in) {
            kk = skeys[j];
            const uint32_t d = (kk >> shift) & (RADIX - 1);
            o = gbase[d] + j - dstart[d];
            kout[CUCO_IDX(o, n)] = kk;
            if (WITH_VALS) vout[CUCO_IDX(o, n)] = svals[j];
        }
        if (NEXT) {
            // one atomic per (digit, destination tile) group of the warp
            const uint32_t slot = in ? ((kk >> next_shift) & (RADIX - 1)) * tiles + o / kSortTile : 0xffffffffu;
            const uint32_t peers = __match_any_sync(kFull, slot);
            if (in && (threadIdx.x & 31) == __ffs(peers) - 1)
                atomicAdd(&next_hist[CUCO_IDX(slot, (uint32_t)RADIX * tiles)], (uint32_t)__popc(peers));
        }
    }
}

// One pass.  hist_ready: `hist` already holds this pass's histogram (counted
// by the previous pass's scatter); next_hist (or null): count the next pass's
// digits at next_shift into it.
template <int RB>
cuco_status_t sort_pass(const uint32_t *kin, const uint32_t *vin, uint32_t *kout, uint32_t *vout,
                        bool with_vals, uint32_t *hist, uint32_t n, int shift,
                        cudaStream_t stream, int *launches, bool hist_ready = false,
                        uint32_t *next_hist = nullptr, int next_shift = 0) {
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    if (tiles == 1) {
        if (with_vals)
            k_sort_scatter<RB, true, true, false><<<1, kSortThreads, 0, stream>>>(kin, vin, kout, vout, n, shift,
                                                                                 hist, tiles, nullptr, 0);
        else
            k_sort_scatter<RB, false, true, false><<<1, kSortThreads, 0, stream>>>(kin, vin, kout, vout, n, shift,
                                                                                  hist, tiles, nullptr, 0);
        *launches += 1;
    } else {
        if (!hist_ready) {
            k_sort_hist<RB><<<tiles, kSortThreads, 0, stream>>>(kin, n, shift, hist, tiles);
            *launches += 1;
        }
        k_sort_scan<<<1u << RB, kSortThreads, 0, stream>>>(hist, tiles, next_hist);
        if (next_hist) {
            if (with_vals)
                k_sort_scatter<RB, true, false, true><<<tiles, kSortThreads, 0, stream>>>(
                    kin, vin, kout, vout, n, shift, hist, tiles, next_hist, next_shift);
            else
                k_sort_scatter<RB, false, false, true><<<tiles, kSortThreads, 0, stream>>>(
                    kin, vin, kout, vout, n, shift, hist, tiles, next_hist, next_shift);
        } else {
            if (with_vals)
                k_sort_scatter<RB, true, false, false><<<tiles, kSortThreads, 0, stream>>>(
                    kin, vin, kout, vout, n, shift, hist, tiles, nullptr, 0);
            else
                k_sort_scatter<RB, false, false, false><<<tiles, kSortThreads, 0, stream>>>(
                    kin, vin, kout, vout, n, shift, hist, tiles, nullptr, 0);
        }
        *launches += 2;
    }
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

void split_bits(int key_bits, int max_radix_bits, int *passes, int *rb) {
    if (key_bits < 1) key_bits = 1;
    if (max_radix_bits > 8) max_radix_bits = 8;
    if (max_radix_bits < 4) max_radix_bits = 4;
    *passes = (key_bits + max_radix_bits - 1) / max_radix_bits;
    *rb = (key_bits + *passes - 1) / *passes;
    if (*rb < 4) *rb = 4;
}

__global__ void k_reorder_start_end(uint32_t *__restrict__ cell_start, uint32_t *__restrict__ cell_end,
                                    float4 *__restrict__ sorted_pos,
                                    const uint32_t *__restrict__ skeys,
                                    const uint32_t *__restrict__ perm,
                                    const float4 *__restrict__ pos, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t k = skeys[i];
    if (i == 0 || k != skeys[i - 1]) {
        cell_start[k] = i;
        if (i > 0) cell_end[skeys[i - 1]] = i;
    }
    if (i == n - 1) cell_end[k] = i + 1;
    sorted_pos[i] = pos[perm[i]];
}

__global__ void k_reorder_offsets(uint32_t *__restrict__ cell_off, float4 *__restrict__ sorted_pos,
                                  const uint32_t *__restrict__ skeys,
                                  const uint32_t *__restrict__ perm,
                                  const float4 *__restrict__ pos, uint32_t n, uint32_t ncells) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    // cells (prev, cur] start at i; thread n closes the tail up to ncells
    uint32_t prev = i == 0 ? 0u : skeys[i - 1] + 1u;
    uint32_t cur = i == n ? ncells : skeys[i];
    for (uint32_t c = prev; c <= cur; ++c) cell_off[c] = i;
    if (i < n && sorted_pos) sorted_pos[i] = pos[perm[i]];
}

// A stable counting sort of each cell's particles by z slice.  A lane's
// slice is spelled out by four ballots (three slice bits and "no particle"),
// so the lanes of each slice, their counts and each lane's rank among equal
// slices are popcounts of the ballots masked to the cell's lanes, and one
// lane per slice keeps the slice's running offset.  The order is fixed by the
// input order alone.  A warp takes four consecutive cells: eight lanes per
// cell, eight particles at a time, which keeps four cells' dependent loads
// (bounds, permutation, position) in flight where cells hold a few particles
// (one warp per cell left most lanes idle waiting on them); where one of the
// four holds more than 32, the warp sorts them one after the other with all
// 32 lanes, so a dense cell does not leave three groups of lanes idle.
constexpr uint32_t kSubLanes = 8;  // lanes per cell in the four-cell mode
static_assert(kZSub == (int)kSubLanes, "one lane per slice within a cell's lanes");

// The cell box of cell c: `one`, or the box of a many-box launch holding c.
__device__ __forceinline__ CellBox cell_box(uint32_t c, const CellBox &one, const CellBox *__restrict__ boxes,
                                            int nbox) {
    if (!boxes) return one;
    int lo = 0, hi = nbox;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&boxes[mid].cell_base) <= c)
            lo = mid;
        else
            hi = mid;
    }
    return boxes[lo];
}

// slice of z within cell cz: plain, of the key rule's product G/L * z (in
// [cz, cz + 1) but for the clamped top face); fixed point, the three bits
// below the cell index of z * G / 2^32
__device__ __forceinline__ uint32_t z_slice(float4 p, const CellBox &d, uint32_t cz, int fixed) {
    if (fixed) return (uint32_t)(((uint64_t)__float_as_uint(p.z) * d.G) >> (32 - kZSubBits)) & (kZSub - 1);
    const float t = __fmul_rn(p.z, d.gridfac);
    const int s = __float2int_rd(__fmul_rn(__fsub_rn(t, (float)cz), (float)kZSub));
    return (uint32_t)min(max(s, 0), kZSub - 1);
}

// One cell [a, b) sorted by the lanes of gmask (W = 8 or 32 consecutive
// lanes; gl = lane within them); every lane of the warp calls it together.
// `valid`: whether this lane's group has a cell (c < ncells).
template <uint32_t W>
__device__ __forceinline__ void subsort_cell(bool valid, uint32_t c, uint32_t a, uint32_t b, const CellBox &d,
                                             uint32_t gmask, uint32_t gl, const uint32_t *__restrict__ perm,
                                             const float4 *__restrict__ pos, float4 *__restrict__ sorted_pos,
                                             uint32_t *__restrict__ perm_s, uint4 *__restrict__ slices,
                                             int fixed) {
    const uint32_t lane = threadIdx.x & 31, lt = (1u << lane) - 1u;
    const uint32_t n_cell = b - a;
    const uint32_t cz = valid ? (c - d.cell_base) % d.G : 0u;
    // lanes gl < kZSub write the cell's inclusive slice counts as u16
    uint16_t *sl = reinterpret_cast<uint16_t *>(slices + (valid ? c : 0u));
    auto put_counts = [&](uint32_t incl) {
        if (valid && gl < kZSub) sl[gl] = n_cell >= 0xffffu ? (uint16_t)0xffffu : (uint16_t)incl;
    };
    // the lanes of gmask holding slice k (k = kZSub: no particle)
    auto lanes_of = [&](uint32_t k, uint32_t b0, uint32_t b1, uint32_t b2, uint32_t none) {
        return ((k & 1) ? b0 : ~b0) & ((k & 2) ? b1 : ~b1) & ((k & 4) ? b2 : ~b2) & ~none & gmask;
    };
    // inclusive scan over the group's first kZSub lanes
    auto scan = [&](uint32_t v) {
#pragma unroll
        for (uint32_t off = 1; off < (uint32_t)kZSub; off <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, v, off, W);
            if (gl >= off) v += u;
        }
        return v;
    };
    const uint32_t chunks = (n_cell + W - 1) / W;
    const uint32_t chunks_max = __reduce_max_sync(0xffffffffu, chunks);
    const bool multi = chunks > 1;
    if (n_cell == 0) put_counts(0);
    const uint32_t gbase = lane - gl;  // the group's first lane
    uint32_t base = 0;                  // lane gl < kZSub: slice gl's next offset in the cell
    if (__any_sync(0xffffffffu, multi)) {
        // cells of more than one chunk count their slices first
        for (uint32_t j = 0; j < chunks_max; ++j) {
            const uint32_t i = a + j * W + gl;
            const uint32_t s = multi && i < b ? z_slice(pos[perm[i]], d, cz, fixed) : (uint32_t)kZSub;
            const uint32_t b0 = __ballot_sync(0xffffffffu, s & 1), b1 = __ballot_sync(0xffffffffu, s & 2),
                           b2 = __ballot_sync(0xffffffffu, s & 4), none = __ballot_sync(0xffffffffu, s == kZSub);
            if (gl < kZSub) base += __popc(lanes_of(gl, b0, b1, b2, none));
        }
        const uint32_t incl = scan(base);
        if (multi) put_counts(incl);
        base = incl - base;
    }
    for (uint32_t j = 0; j < chunks_max; ++j) {
        const uint32_t i = a + j * W + gl;
        uint32_t o = 0, s = kZSub;
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < b) {
            o = perm[i];
            p = pos[o];
            s = z_slice(p, d, cz, fixed);
        }
        const uint32_t b0 = __ballot_sync(0xffffffffu, s & 1), b1 = __ballot_sync(0xffffffffu, s & 2),
                       b2 = __ballot_sync(0xffffffffu, s & 4), none = __ballot_sync(0xffffffffu, s == kZSub);
        const uint32_t mine = lanes_of(s, b0, b1, b2, none);
        const uint32_t cnt = gl < kZSub ? __popc(lanes_of(gl, b0, b1, b2, none)) : 0u;
        const uint32_t incl = scan(cnt);
        if (!multi && j == 0) {
            // one chunk: the offsets are the exclusive scan of its counts
            if (n_cell) put_counts(incl);
            base = incl - cnt;
        }
        const uint32_t at = __shfl_sync(0xffffffffu, base, gbase + (s & (kZSub - 1))) + __popc(mine & lt);
        if (i < b) {
            sorted_pos[CUCO_IDX(a + at, b)] = make_float4(p.x, p.y, p.z, (float)s);
            perm_s[CUCO_IDX(a + at, b)] = o;
        }
        base += cnt;
    }
}

__global__ void k_cell_subsort(const uint32_t *__restrict__ cell_off, const uint32_t *__restrict__ perm,
                               const float4 *__restrict__ pos, float4 *__restrict__ sorted_pos,
                               uint32_t *__restrict__ perm_s, uint4 *__restrict__ slices, uint32_t ncells,
                               const __grid_constant__ CellBox one, const CellBox *__restrict__ boxes, int nbox,
                               int fixed) {
    constexpr uint32_t kCells = 32 / kSubLanes;
    const uint32_t lane = threadIdx.x & 31, grp = lane / kSubLanes;
    const uint32_t c0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kCells;
    if (c0 >= ncells) return;  // warp-uniform
    const uint32_t c = c0 + grp;
    const bool valid = c < ncells;
    const uint32_t a = valid ? cell_off[c] : 0u, b = valid ? cell_off[c + 1] : 0u;
    if (__any_sync(0xffffffffu, b - a > 32u)) {
        // the four cells one after the other, all 32 lanes on each
        for (uint32_t g = 0; g < kCells; ++g) {
            const uint32_t cg = c0 + g;
            if (cg >= ncells) break;  // warp-uniform
            const uint32_t ag = __shfl_sync(0xffffffffu, a, g * kSubLanes), bg = __shfl_sync(0xffffffffu, b, g * kSubLanes);
            subsort_cell<32>(true, cg, ag, bg, cell_box(cg, one, boxes, nbox), 0xffffffffu, lane, perm, pos,
                             sorted_pos, perm_s, slices, fixed);
        }
    } else {
        const CellBox d = valid ? cell_box(c, one, boxes, nbox) : one;
        subsort_cell<kSubLanes>(valid, c, a, b, d, 0xffu << (grp * kSubLanes), lane % kSubLanes, perm, pos,
                                sorted_pos, perm_s, slices, fixed);
    }
}

}  // namespace

cuco_status_t launch_cell_subsort(const uint32_t *cell_off, const uint32_t *perm, const float4 *pos,
                                  float4 *sorted_pos, uint32_t *perm_s, uint4 *slices, uint32_t ncells,
                                  const CellBox &one, const CellBox *boxes, int nbox, bool fixed,
                                  cudaStream_t stream) {
    if (ncells == 0) return CUCO_OK;
    const uint64_t threads = 32ull * ((ncells + 32 / kSubLanes - 1) / (32 / kSubLanes));
    k_cell_subsort<<<(unsigned)((threads + 255) / 256), 256, 0, stream>>>(
        cell_off, perm, pos, sorted_pos, perm_s, slices, ncells, one, boxes, nbox, fixed ? 1 : 0);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

size_t sort_hist_entries(uint32_t n, int key_bits, int max_radix_bits) {
    int passes, rb;
    split_bits(key_bits, max_radix_bits, &passes, &rb);
    size_t tiles = (n + kSortTile - 1) / kSortTile;
    return (size_t)(1u << rb) * (tiles ? tiles : 1);
}

cuco_status_t sort_pairs(uint32_t *keys, uint32_t *vals, const uint32_t *vals_in,
                         uint32_t *keys_alt, uint32_t *vals_alt, uint32_t *hist, uint32_t n,
                         int key_bits, int max_radix_bits, cudaStream_t stream,
                         bool *result_in_alt, int *launches, uint32_t *hist2) {
    int passes, rb;
    split_bits(key_bits, max_radix_bits, &passes, &rb);
    bool with_vals = vals != nullptr;
    *result_in_alt = false;
    if (n == 0) return CUCO_OK;
    uint32_t *kbuf[2] = {keys, keys_alt};
    uint32_t *vbuf[2] = {vals, vals_alt};
    uint32_t *hbuf[2] = {hist, hist2 ? hist2 : hist};
    int cur = 0;
    for (int p = 0; p < passes; ++p) {
        const uint32_t *vin = (p == 0) ? vals_in : vbuf[cur];
        const int shift = p * rb;
        // with two histograms, pass p uses hbuf[p & 1] and counts pass p+1's
        // digits into the other
        const bool fused = hist2 != nullptr;
        uint32_t *h = hbuf[fused ? (p & 1) : 0];
        uint32_t *hn = fused && p + 1 < passes ? hbuf[(p + 1) & 1] : nullptr;
        const bool ready = fused && p > 0;
        cuco_status_t s;
        switch (rb) {
#define CUCO_SORT_PASS(R)                                                                                    \
    s = sort_pass<R>(kbuf[cur], vin, kbuf[cur ^ 1], vbuf[cur ^ 1], with_vals, h, n, shift, stream, launches, \
                     ready, hn, shift + rb)
            case 4: CUCO_SORT_PASS(4); break;
            case 5: CUCO_SORT_PASS(5); break;
            case 6: CUCO_SORT_PASS(6); break;
            case 7: CUCO_SORT_PASS(7); break;
            default: CUCO_SORT_PASS(8); break;
#undef CUCO_SORT_PASS
        }
        if (s != CUCO_OK) return s;
        cur ^= 1;
    }
    *result_in_alt = cur == 1;
    return CUCO_OK;
}

cuco_status_t launch_cell_keys(const float4 *pos, uint32_t *keys, uint32_t *idx, uint32_t n,
                               float gridfac, int G, cudaStream_t stream) {
    if (n == 0) return CUCO_OK;
    int blocks = (int)((n + 255) / 256);
    k_cell_keys<<<blocks, 256, 0, stream>>>(pos, keys, idx, n, gridfac, G);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

cuco_status_t launch_reorder_start_end(uint32_t *cell_start, uint32_t *cell_end,
                                       float4 *sorted_pos, const uint32_t *sorted_keys,
                                       const uint32_t *perm, const float4 *pos, uint32_t n,
                                       uint32_t ncells, cudaStream_t stream) {
    CUCO_TRY_CUDA(cudaMemsetAsync(cell_start, 0xff, sizeof(uint32_t) * ncells, stream));
    if (n == 0) return CUCO_OK;
    k_reorder_start_end<<<(n + 255) / 256, 256, 0, stream>>>(cell_start, cell_end, sorted_pos,
                                                           sorted_keys, perm, pos, n);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

cuco_status_t launch_reorder_offsets(uint32_t *cell_off, float4 *sorted_pos,
                                     const uint32_t *sorted_keys, const uint32_t *perm,
                                     const float4 *pos, uint32_t n, uint32_t ncells,
                                     cudaStream_t stream) {
    k_reorder_offsets<<<(n + 1 + 255) / 256, 256, 0, stream>>>(cell_off, sorted_pos, sorted_keys,
                                                             perm, pos, n, ncells);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

uint32_t bounds_violations_sort() { return bounds_violations_take(); }

}  // namespace cuco
