// Shared declarations of the GB300 force engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "../../include/cuco_gb300.h"

namespace cuco {

constexpr uint32_t kEmptyCell = 0xffffffffu;
constexpr int kNTab = CUCO_NTAB;

// ---------------------------------------------------------------- errors

void set_error(const std::string &msg);
const char *last_error();

#define CUCO_TRY_CUDA(expr)                                                         \
    do {                                                                            \
        cudaError_t _e = (expr);                                                    \
        if (_e != cudaSuccess) {                                                    \
            ::cuco::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));  \
            return CUCO_ERR_CUDA;                                                   \
        }                                                                           \
    } while (0)

#define CUCO_TRY(expr)                         \
    do {                                       \
        cuco_status_t _s = (expr);             \
        if (_s != CUCO_OK) return _s;          \
    } while (0)

// ---------------------------------------------------- debug bounds checks

// Debug builds (compiled with -DCUCO_BOUNDS_CHECK) check the index of the
// main global and shared memory accesses of the kernels against its bound.  A
// failed check adds one to this translation unit's violation counter and the
// access goes to the last in-bounds element instead, so the kernel keeps
// running and the host reads the count afterwards
// (cuco_debug_bounds_violations).  Release builds compile the checks away.
#ifdef CUCO_BOUNDS_CHECK
static __device__ unsigned int g_bounds_violations;
__device__ __forceinline__ uint32_t bounds_checked(uint32_t i, uint32_t limit) {
    if (i >= limit) {
        atomicAdd(&g_bounds_violations, 1u);
        return limit ? limit - 1u : 0u;
    }
    return i;
}
#define CUCO_IDX(i, limit) ::cuco::bounds_checked((uint32_t)(i), (uint32_t)(limit))
// this translation unit's count, read and reset (host)
static inline uint32_t bounds_violations_take() {
    unsigned int v = 0, zero = 0;
    cudaMemcpyFromSymbol(&v, g_bounds_violations, sizeof v);
    cudaMemcpyToSymbol(g_bounds_violations, &zero, sizeof zero);
    return v;
}
#else
#define CUCO_IDX(i, limit) (i)
static inline uint32_t bounds_violations_take() { return 0; }
#endif
uint32_t bounds_violations_sort();
uint32_t bounds_violations_pm();
uint32_t bounds_violations_shortrange();

// -------------------------------------------------------------- sorting

// Scratch a sort of n keys needs: alternate key/value buffers and the per-tile
// digit histogram (radix * tiles entries).
size_t sort_hist_entries(uint32_t n, int key_bits, int max_radix_bits);

// Stable LSD radix sort of (keys, vals) by the low key_bits bits.  vals_in may
// be null: the values are then the input positions 0..n-1.  The sorted data
// ends in (keys, vals) when `result_in_alt` comes back false, else in
// (keys_alt, vals_alt).  max_radix_bits bounds the digit width (4..8).
// hist2: a second histogram of the same size, or null.  With it each pass's
// scatter also counts the next pass's digits of the keys it places (into the
// other histogram, cleared by the pass's scan), so only the first pass runs a
// histogram kernel; the result is the same.
cuco_status_t sort_pairs(uint32_t *keys, uint32_t *vals, const uint32_t *vals_in,
                         uint32_t *keys_alt, uint32_t *vals_alt, uint32_t *hist, uint32_t n,
                         int key_bits, int max_radix_bits, cudaStream_t stream,
                         bool *result_in_alt, int *launches, uint32_t *hist2 = nullptr);

// Cell keys of float4 positions (calcHashD rule); idx gets 0..n-1 when non-null.
cuco_status_t launch_cell_keys(const float4 *pos, uint32_t *keys, uint32_t *idx, uint32_t n,
                               float gridfac, int G, cudaStream_t stream);

// Reference cell-bound format (cellStart/cellEnd, empty start = 0xffffffff) and
// the sorted-position gather.
cuco_status_t launch_reorder_start_end(uint32_t *cell_start, uint32_t *cell_end,
                                       float4 *sorted_pos, const uint32_t *sorted_keys,
                                       const uint32_t *perm, const float4 *pos, uint32_t n,
                                       uint32_t ncells, cudaStream_t stream);

// Engine cell-bound format: cell_off[c] = first sorted index with key >= c,
// for c in [0, ncells], plus the gather (none when sorted_pos is null).
cuco_status_t launch_reorder_offsets(uint32_t *cell_off, float4 *sorted_pos,
                                     const uint32_t *sorted_keys, const uint32_t *perm,
                                     const float4 *pos, uint32_t n, uint32_t ncells,
                                     cudaStream_t stream);

// A box's cell grid within a concatenated cell numbering (cells
// cell_base .. cell_base + G^3 - 1).
struct CellBox {
    uint32_t G, cell_base;
    float boxsize, gridfac;  // gridfac = (float)G / L, the key rule's factor
};

// Each cell's particles ordered by z slice: kZSub slices of the cell along z,
// stable within a slice.  From the cell-sorted permutation `perm` (cell_off:
// the cells' first sorted indices) it gathers sorted_pos in that order, with
// w = the slice as a float, and perm_s = its map to original indices.
// slices[c] holds eight u16: entry j = the cell's particles in slices 0..j
// (all 0xffff for a cell of 65535 or more).  Boxes: one (boxes null, `one`)
// or nbox descriptors sorted by cell_base.  fixed: positions are 32-bit fixed
// point.
constexpr int kZSubBits = 3;
constexpr int kZSub = 1 << kZSubBits;
cuco_status_t launch_cell_subsort(const uint32_t *cell_off, const uint32_t *perm, const float4 *pos,
                                  float4 *sorted_pos, uint32_t *perm_s, uint4 *slices, uint32_t ncells,
                                  const CellBox &one, const CellBox *boxes, int nbox, bool fixed,
                                  cudaStream_t stream);

// ----------------------------------------------------------- short range

struct ShortRangeParams {
    float boxsize;
    float gridfac;   // G / L in float, the key rule's factor
    float cellw;     // L / G
    float rcut, rcut2;
    float asmthfac;  // 0.5 / asmth * NTAB / 3
    double asmthfac_d;  // the same in double (gravlist.cpp:67), for bin-edge pairs
    float mass;      // source mass
    float G;         // gravitational constant (applied once per target)
    float h, hinv, h3inv;
    int grid;        // G
    uint32_t n;
    bool fixed;      // positions are 32-bit fixed point (bit patterns in the float4s)
    float fscale;    // L / 2^32
    uint32_t cell_base;  // first cell of this box in a multi-box cell array (0 otherwise)
    // pair-law bounds, filled in by the short-range launch from the above:
    // fast-path cut and flag cut (plain: a band around rcut^2 decided in
    // double), the softening bound below which the spline applies, the bin
    // factor scaled down and up by the bin-edge band, rcut^2 in double
    float rc2_lo, rc2_hi, hmin2, alo, ahi;
    double rcut2_d;
    // the z-slice counts of the cells (launch_cell_subsort), indexed by cell
    // id; null when the sources are not in slice order or the per-segment
    // table would not fit in shared memory
    const uint4 *slices;
};

// Which cell-bound format the kernel reads.
enum CellFormat { kCellOffsets = 0, kCellStartEnd = 1 };

// Kick applied in the short-range epilogue (null vel: no kick).
struct KickArgs {
    float4 *vel;              // original order
    const float4 *acc_pm_s;   // PM acceleration in sorted order (may be null)
    float4 *acc_pm_out;       // PM acceleration scattered to original order (may be null)
    double kick_pp, kick_pm;
    const float4 *acc_pm_o;   // PM acceleration in original order (used when acc_pm_s is null)
};

// Device scratch of a launch's work plan: each segment's target count, the
// slices of segments denser than one unit, and two counters.  seg_cap must
// cover the launch's segments (G^3 is always enough), heavy_cap
// shortrange_heavy_cap(n).
struct SRWork {
    uint2 *heavy;
    uint32_t heavy_cap;
    uint32_t *seg_nt;
    uint32_t seg_cap;
    uint32_t *ctl;  // kSRCtlWords: [0] dense slices listed, [1] next unit (both reset per
                    // launch), [2] nonzero once a staging wait gave up (kept until read)
};
uint32_t shortrange_heavy_cap(uint32_t n);
constexpr int kSRCtlWords = 4;
// Reads and clears the short range's timeout word (ctl[2]) after the work on
// `stream` is done: CUCO_ERR_TIMEOUT when a staging wait gave up.
cuco_status_t shortrange_check(uint32_t *ctl, cudaStream_t stream);
// Runs the staging wait's timeout path with a barrier that never completes
// and a limit of `limit_cycles`: returns what shortrange_check then reports.
cuco_status_t shortrange_timeout_probe(uint32_t *ctl, long long limit_cycles, cudaStream_t stream);

// pair_counter: when non-null, the launch adds its in-range pair count to it.
// late_stream (with plan_done, an event of the caller's): the persistent grid
// is split, one CTA per SM fewer on `stream` and the rest queued on
// late_stream behind whatever that stream runs first (the PM); both parts
// take units from the same counter, so work left when the late part starts
// spreads over both.  The launch is complete when both streams have run it.
cuco_status_t launch_shortrange(const ShortRangeParams &p, const float4 *sorted_pos,
                                const uint32_t *perm, const uint32_t *cell_a,
                                const uint32_t *cell_b, CellFormat fmt, const float *table,
                                float4 *acc_out, const KickArgs &kick, const SRWork &work, cudaStream_t stream,
                                unsigned long long *pair_counter = nullptr, cudaStream_t late_stream = nullptr,
                                cudaEvent_t plan_done = nullptr);

// Many boxes in one launch (the batched form).  A box's descriptor holds its
// parameters and neighbour-column set; shortrange_desc_fill writes one (in
// host memory, shortrange_desc_bytes() long) and returns the box's segment
// count and shared memory.  kicks[b] = (kick_pp, kick_pm) of box b.
size_t shortrange_desc_bytes();
cuco_status_t shortrange_desc_fill(const ShortRangeParams &p, void *desc, uint32_t *segments, size_t *smem);
// uniform_law_desc (host memory, or null): a descriptor whose pair law every
// box shares (shortrange_descs_uniform_law said so); the launch then reads
// the law from its parameters instead of each box's descriptor.
bool shortrange_descs_uniform_law(const void *host_descs, int nbox);
cuco_status_t launch_shortrange_multi(const void *descs, const double2 *kicks, const uint32_t *seg_base,
                                      int nbox, uint32_t segments, size_t smem, bool fixed,
                                      const float4 *sorted_pos, const uint32_t *perm, const uint32_t *cell_off,
                                      const float *table, float4 *acc_out, const KickArgs &kick,
                                      const SRWork &work, cudaStream_t stream, unsigned long long *pair_counter,
                                      const void *uniform_law_desc = nullptr);

// ------------------------------------------------------------------- PM

struct PMPlan {
    int M;
    bool fixed;         // positions are 32-bit fixed point (units of L / 2^32)
    float boxsize;
    float to_slab_fac;  // M / L in float (pm_periodic.c:42)
    float mass;
    float fd_fac;       // G/(pi L) * M/(2L) (pm_periodic.c:85-86)
    float *rho;         // M^3 real grid: the potential
    unsigned long long *rho64;  // M^3 deposited mass in units of m / 2^32
    bool rho64_dirty;   // rho64 may hold sums (the z pass clears what it reads)
    float2 *spec;       // M*M*(M/2+1) complex grid
    float *green1d;     // M/2+1: exp(-k^2 a) / sinc(pi k/M)^4
    float2 *twiddle;    // M: exp(-2 pi i t / M)
};

// Meshes the FFT supports: even, 8..1024, no prime factor above 5.
bool pm_mesh_supported(int M);
cuco_status_t pm_plan_create(PMPlan *plan, int M, float boxsize, float asmth, float mass,
                             double G, bool fixed = false);
void pm_plan_destroy(PMPlan *plan);
// Long-range acceleration of n positions (any order) into acc (same order).
cuco_status_t pm_forces(PMPlan &plan, const float4 *pos, uint32_t n, float4 *acc,
                        cudaStream_t stream, cudaEvent_t *ev_deposit_done,
                        cudaEvent_t *ev_fft_done, int *launches);

// Many boxes' meshes in one launch per PM phase (the batched form).
struct PMBoxDesc {
    int M, P, B;         // mesh; z-pass row pairs and axis-pass columns per CTA
    float to_slab_fac, mass, fd_fac;
    float *rho;          // this box's M^3 real grid (the potential)
    unsigned long long *rho64;  // its deposited mass, units of m / 2^32
    float mscale;        // m / 2^32
    float2 *spec;        // its M*M*(M/2+1) half spectrum
    const float *green1d;
    const float2 *twiddle;
};
struct PMMulti {
    int nbox;
    bool fixed;
    const PMBoxDesc *boxes;   // device
    const uint32_t *pbeg;     // device, nbox+1: each box's first particle
    const uint2 *map_z;       // device: (box, block) per CTA of the z passes
    const uint2 *map_axis;    // device: (box, block) per CTA of the y/x passes
    uint32_t nz_blocks, naxis_blocks;
    size_t smz, sma;          // dynamic shared memory of the z and axis passes
    unsigned long long *rho64_all;  // all boxes' deposit grids, contiguous (one memset)
    size_t rho_all_count;
    bool big;  // some box's transforms need the large register kernels (pm_big_fft)
};
// Whether a box of mesh M with transform batches P, B takes the large (32-point)
// register transforms, which run in kernels of their own.
bool pm_big_fft(int M, int P, int B);
bool pm_fft_batches_ok(int M, int P, int B);
int pm_batch_z(int M);
int pm_batch_axis(int M);
size_t pm_smem_z(int M, int P);
size_t pm_smem_axis(int M, int B);
void pm_tables(int M, float boxsize, float asmth, float *green1d, float2 *twiddle);
float pm_fd_fac(int M, float boxsize, double G);
// PM accelerations of n positions laid out box after box (pbeg), into acc.
cuco_status_t pm_forces_multi(const PMMulti &m, const float4 *pos, uint32_t n, float4 *acc,
                              cudaStream_t stream, int *launches);

// Index of the box whose range [pbeg[b], pbeg[b+1]) holds i (pbeg[0] = 0).
__device__ __forceinline__ int find_box(const uint32_t *__restrict__ pbeg, int nbox, uint32_t i) {
    int lo = 0, hi = nbox;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&pbeg[mid]) <= i)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// ------------------------------------------------------------ integrator

cuco_status_t launch_drift_keys(float4 *pos, const float4 *vel, double drift, float boxsize,
                                bool do_drift, uint32_t *keys, uint32_t n, float gridfac, int G,
                                cudaStream_t stream);

// Fixed-point positions (uint32 per axis, units of L / 2^32, bit patterns in
// the float4 slots) from and to float triplets; float triplets <-> float4.
cuco_status_t to_fixed(const float *a, float4 *b, uint32_t n, float boxsize, cudaStream_t stream);
cuco_status_t from_fixed(const float4 *b, float *a, uint32_t n, float boxsize, cudaStream_t stream);
cuco_status_t pack3to4(const float *a, float4 *b, uint32_t n, cudaStream_t stream);
cuco_status_t unpack4to3(const float4 *b, float *a, uint32_t n, cudaStream_t stream);

// The reference's erfc split table T[i] (gravlist.cpp:56-67), FP64 -> float.
void shortrange_table(float *t);

// Host FP64 cosmological integrals.
double cosmo_integral(double a0, double a1, double omega0, double omega_lambda, double hubble,
                      int power);

}  // namespace cuco
