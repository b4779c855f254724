// Short-range P3M pair force on the cell grid.
//
// Reference: cudaForceEvaluateShortrangeD + calcForce (gravlist_kernel.cu:20-88,
// 162-234) and the CPU force_evaluate_shortrange (gravlist.cpp:216-338).  The
// pair law is the reference's: minimum-image separation, cut at r^2 > rcut^2,
// 1/r^2 outside the spline softening length h and GADGET's spline inside,
// times the nearest-bin erfc split factor T[(int)(asmthfac*r)] (NTAB = 1000).
//
// Work layout (GB300-first rather than one thread per particle over a full
// cube of cells):
//   * a segment is S consecutive cells along z (ix, iy, iz0..iz0+S-1); its
//     targets are one contiguous range of the cell order.  A unit of work is a
//     segment, or a slice of at most kTMax targets of a denser one; a plan
//     kernel lists each segment's targets and the dense slices, and a
//     persistent grid (the CTAs that fit on the GPU) pulls units from a
//     counter, dense slices first;
//   * the sources are the neighbour columns (dx, dy) within rcut of the
//     segment in xy, over z-cells iz0-R .. iz0+S-1+R.  A column's cells are
//     consecutive keys, so it is at most two contiguous runs of the cell order
//     (two when the z range wraps); the unit's threads find every cell's
//     staged offset with one block scan, each thread issues one run as a
//     bulk copy (cp.async.bulk, completing on one mbarrier) into shared
//     memory, and the staged sources are then moved relative to an integer
//     origin at the segment corner, with the periodic image shift applied
//     once per run (in chunks of kMaxStage sources; every target runs
//     against each chunk, its sums carried in shared memory);
//   * two consecutive targets per warp: lane k culls column k against the
//     pair's bounding box in xy and narrows it to the z range
//     sqrt(rcut^2 - d_xy^2) reaches, trimmed in the two end cells to the z
//     slices it reaches (the cells' particles are ordered by slice, with
//     per-cell slice counts); the column ranges, concatenated by a warp scan,
//     are walked 32 candidates at a time, every lane on one staged source
//     that it evaluates against both targets in packed FP32 (float2
//     add/mul/fma, one instruction for the two targets);
//   * the pair law runs without branches on the common path and flags the
//     rest (bin-edge and cut-edge pairs decided in double, the spline); the
//     windows holding a flagged pair are revisited after the last window;
//   * the warp reduces its lanes' six partial sums (3 components x 2
//     targets) with a transpose-reduce of xor shuffles (the precision form
//     compensated by error-free splitting);
//   * the warp's lanes scatter the forces to original particle order and, in
//     the engine's step, kick the velocities (timestep.c:56-59,86-91).
//
// Precision of the plain path.  A float computation of asmthfac*r lands in the
// neighbouring table bin for ~3e-5 of the pairs, and at high redshift (net
// force a small residual of cancelling pair terms) that alone costs ~1.6e-4
// rms against the reference's double path.  Coordinates relative to an integer
// origin make the image shift exact (origin -/+ L is an exact float for
// L < 2^23) and dx exact for ~97% of pairs; pairs whose r^2 lies within
// 8e-7 (relative) of rcut^2 or whose asmthfac*r lies within 4e-7 (relative)
// of a bin edge are decided in double as gravlist.cpp:298-320 does.
#include <algorithm>
#include <cstring>

#include "common.cuh"

namespace cuco {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxStage = 2048;  // staged sources per chunk (32 KB)
constexpr int kMaxR = 8;         // neighbour reach in cells (the reference's G = PMGRID needs 6)
constexpr int kMaxCols = (2 * kMaxR + 1) * (2 * kMaxR + 1);
constexpr int kMaxSeg = 8;
// A unit of work is at most kTMax targets: a segment with that many, or a
// kTMax slice of a denser segment.
constexpr int kTMax = 128;
// the split table in shared memory, padded to a power of two
constexpr int kTabPad = 1024;
static_assert(kTabPad >= kNTab && (kTabPad & (kTabPad - 1)) == 0, "table padding");
constexpr unsigned kFull = 0xffffffffu;
// CTAs per SM the register allocation is sized for (65536 / (256 * 4) = 64
// registers a thread at 4)
#ifndef CUCO_SR_MIN_BLOCKS
#define CUCO_SR_MIN_BLOCKS 4
#endif
constexpr int kMinBlocks = CUCO_SR_MIN_BLOCKS;

struct ColumnSet {
    int ncols;
    int R;
    int S;
    int c00;       // the column (0, 0)
    float margin;  // culling slack for the float cell assignment (length units)
    signed char dx[kMaxCols];
    signed char dy[kMaxCols];
};

// One box of a multi-box launch.
struct SRBoxDesc {
    ShortRangeParams p;
    ColumnSet cs;
};

struct Run {
    uint32_t gsrc;  // first sorted index
    uint32_t soff;  // first staged index (stencil order)
    uint32_t cnt;
    float sx, sy, sz;
};

// Dynamic shared memory, in order: staged sources and one sentinel source,
// split table, column xy bounds, per-(column, z-cell) staged offsets, cell
// starts and counts, column runs, column totals.
__host__ __device__ inline size_t smem_base_bytes(int ncols, int nz) {
    const size_t b = sizeof(float4) * (kMaxStage + 1) + sizeof(float) * kTabPad + sizeof(float4) * (size_t)ncols +
                     sizeof(uint32_t) * (size_t)ncols * (nz + 1) + 2 * sizeof(uint32_t) * (size_t)ncols * nz +
                     sizeof(Run) * 2 * (size_t)ncols + sizeof(uint32_t) * (size_t)ncols;
    return (b + 15) & ~(size_t)15;
}
// ... then, with z slices, every (column, z-cell)'s slice counts
__host__ __device__ inline size_t smem_bytes(int ncols, int nz, bool zs) {
    return smem_base_bytes(ncols, nz) + (zs ? sizeof(uint4) * (size_t)ncols * nz : 0);
}
// The slice table is used where it adds at most this much shared memory.
constexpr size_t kMaxSliceTable = 16384;

// A staged source this far away is beyond any cut: list positions past the
// end of a target's candidates read it instead of branching.
constexpr float kSentinel = 1e15f;

template <CellFormat FMT>
__device__ __forceinline__ void cell_range(const uint32_t *__restrict__ a,
                                           const uint32_t *__restrict__ b, uint32_t c,
                                           uint32_t *start, uint32_t *count) {
    if (FMT == kCellOffsets) {
        uint32_t s = a[c];
        *start = s;
        *count = a[c + 1] - s;
    } else {
        uint32_t s = a[c];
        if (s == kEmptyCell) {
            *start = 0;
            *count = 0;
        } else {
            *start = s;
            *count = b[c] - s;
        }
    }
}

// s + e = a + b exactly (Knuth's two-sum; the intrinsics keep the compiler
// from contracting or reordering it).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// 1 << k for k < 32, else 0: PTX clamps a shift count above the width, so
// this is one shift with no compare and select.
__device__ __forceinline__ uint32_t bit_at(uint32_t k) {
    uint32_t b;
    asm("shl.b32 %0, %1, %2;" : "=r"(b) : "r"(1u), "r"(k));
    return b;
}

// The hardware reciprocal square root, flushing subnormal inputs (the fast
// path only sees r^2 well above them; without the flush the compiler wraps
// the instruction in a subnormal rescale).
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// r^2 with a fixed operation order: the candidate test and the force pass
// must agree on it bit for bit.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// ---- Bulk copies of contiguous source runs into shared memory (the tensor
// memory accelerator's untiled global -> shared copy, completing on an
// mbarrier).  One barrier per CTA, reused phase after phase; its waits are
// bounded (kWaitCycles), after which the CTA reports a timeout and stops.
constexpr long long kWaitCycles = 1ll << 31;  // ~1 s at 2 GHz
__shared__ __align__(8) uint64_t g_stage_bar;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one arrival that also expects `bytes` of copies in this phase
__device__ __forceinline__ void bar_arrive_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool bar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Wait for the phase with parity `parity` to complete, at most `limit`
// clock cycles.
__device__ __forceinline__ bool bar_wait_bounded(uint64_t *bar, uint32_t parity, long long limit = kWaitCycles) {
    const long long t0 = clock64();
    for (;;) {
        if (bar_try_wait(bar, parity)) return true;
        if (clock64() - t0 > limit) return false;
    }
}

// The staging wait's timeout path on its own: one CTA arms the barrier for
// 16 bytes of copies that are never issued, waits at most `limit` cycles (the
// staging wait, with a shorter limit), and reports through the same timeout
// word the short range uses.  No copy is in flight when it gives up.
__global__ void k_staging_timeout_probe(uint32_t *__restrict__ err, long long limit) {
    if (threadIdx.x == 0) bar_init(&g_stage_bar);
    __syncthreads();
    if (threadIdx.x == 0) bar_arrive_expect(&g_stage_bar, 16u);
    __syncthreads();
    const bool ok = bar_wait_bounded(&g_stage_bar, 0u, limit);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(err, 1u);
}

// bytes (a multiple of 16) from global src to shared dst, both 16-byte aligned
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// orders this thread's earlier shared-memory accesses (and, after a CTA
// barrier, the CTA's) before later bulk copies into shared memory
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// The body for one unit: the targets [slice_lo, slice_hi) (counted from the
// segment's first target) of segment `seg` of one box (p, cs); kick_pp/kick_pm
// are that box's kick factors.  A unit has at most kTMax targets.
// Returns false when a staging wait gave up (the error word is set; the CTA
// must stop).  `phase` is the parity of the CTA's staging barrier.
// `law`: the pair law's constants (rc2_lo, rc2_hi, hmin2, alo, ahi, rcut2_d,
// asmthfac_d, h, hinv, h3inv): the box's own (p), or the launch's when every
// box of a many-box launch has the same (read from the kernel's parameters).
// PIN_LAW: the law lives in global memory (a many-box launch's descriptor):
// its three range bounds are held in registers for a pair's windows, where the
// compiler would otherwise reload them in every window.
template <CellFormat FMT, bool KICK, bool COUNT, bool FIXED, bool PIN_LAW = false>
__device__ __forceinline__ bool shortrange_segment(
    const ShortRangeParams &p, const ShortRangeParams &law, const ColumnSet &cs, const int seg,
    const uint32_t slice_lo,
    const uint32_t slice_hi, const double kick_pp, const double kick_pm, const float4 *__restrict__ spos,
    const uint32_t *__restrict__ perm, const uint32_t *__restrict__ ca, const uint32_t *__restrict__ cb,
    const float *__restrict__ table_g, float4 *__restrict__ acc_out, const KickArgs &kick,
    unsigned long long *__restrict__ pair_counter, uint32_t &phase, uint32_t *__restrict__ err) {
    extern __shared__ float4 smem_f4[];
    __shared__ uint32_t s_total, s_tbegin, s_tend;
    __shared__ uint32_t s_wdelta[kWarps][32];
    __shared__ uint32_t s_wsum[kWarps];
    __shared__ float s_acc[6][kTMax];  // per-target sums (multi-chunk units: and FIXED error terms)
    __shared__ float4 s_tpos[kTMax];   // the unit's target positions

    const int G = p.grid;
    const int S = cs.S, R = cs.R, nz = S + 2 * R, ncols = cs.ncols;
    const int zst = nz + 1;  // coff stride per column
    float4 *src = smem_f4;
    float *tab = reinterpret_cast<float *>(src + kMaxStage + 1);
    float4 *cgeo = reinterpret_cast<float4 *>(tab + kTabPad);  // x0, x1, y0, y1
    uint32_t *coff = reinterpret_cast<uint32_t *>(cgeo + ncols);
    uint32_t *cst = coff + ncols * zst;
    uint32_t *ccn = cst + ncols * nz;
    Run *runs = reinterpret_cast<Run *>(ccn + ncols * nz);
    uint32_t *coltot = reinterpret_cast<uint32_t *>(runs + 2 * ncols);
    // (column, z-cell) -> eight u16 slice counts of that cell
    uint4 *s_sl = reinterpret_cast<uint4 *>(reinterpret_cast<char *>(smem_f4) + smem_base_bytes(ncols, nz));
    const uint16_t *sl16 = reinterpret_cast<const uint16_t *>(s_sl);

    const int segs = G / S;
    const int ix = seg / (G * segs);
    const int iy = (seg / segs) % G;
    const int iz0 = (seg % segs) * S;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float L = p.boxsize;
    const bool ZS = p.slices != nullptr;  // sources in z-slice order within cells, with slice counts

    // every (column, z-cell) range, loaded in parallel; e = col * nz + zc
    // (the float quotient is exact here: (e + 1/2) / nz is at least 1/(2 nz)
    // from an integer)
    const float inv_nz = 1.0f / (float)nz;
    auto col_of = [&](int e) { return (int)(((float)e + 0.5f) * inv_nz); };
    for (int e = tid; e < ncols * nz; e += kThreads) {
        const int col = col_of(e), zc = e - col * nz;
        int cxu = ix + cs.dx[col], cyu = iy + cs.dy[col], czu = iz0 - R + zc;
        int cx = cxu < 0 ? cxu + G : (cxu >= G ? cxu - G : cxu);
        int cy = cyu < 0 ? cyu + G : (cyu >= G ? cyu - G : cyu);
        int cz = czu < 0 ? czu + G : (czu >= G ? czu - G : czu);
        uint32_t st, cn;
        const uint32_t cell = p.cell_base + ((uint32_t)cx * G + cy) * G + cz;
        cell_range<FMT>(ca, cb, cell, &st, &cn);
        cst[e] = st;
        ccn[e] = cn;
        if (ZS) s_sl[e] = p.slices[cell];
    }
    __syncthreads();
    uint32_t t_begin, t_end, total;
    if (FMT == kCellOffsets) {
        // The segment's targets are cells R .. R+S-1 of column (0, 0):
        // consecutive keys, so one range of the cell order.
        const int e00 = cs.c00 * nz + R;
        const uint32_t t_seg = cst[e00], t_seg_end = cst[e00 + S - 1] + ccn[e00 + S - 1];
        t_begin = t_seg + min(slice_lo, t_seg_end - t_seg);
        t_end = t_seg + min(slice_hi, t_seg_end - t_seg);
        if (t_begin >= t_end) return true;  // uniform over the CTA
        // staged offsets: an exclusive scan of the cell counts in (column,
        // z-cell) order, each thread over a run of consecutive entries
        const int ne = ncols * nz;
        const int per = (ne + kThreads - 1) / kThreads;
        const int e0 = min(tid * per, ne), e1 = min(e0 + per, ne);
        uint32_t loc = 0;
        for (int e = e0; e < e1; ++e) loc += ccn[e];
        uint32_t inc = loc;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t v = __shfl_up_sync(kFull, inc, off);
            if (lane >= off) inc += v;
        }
        if (lane == 31) s_wsum[warp] = inc;
        __syncthreads();
        uint32_t run = inc - loc;
        total = 0;
        for (int k = 0; k < kWarps; ++k) {
            const uint32_t v = s_wsum[k];
            if (k < warp) run += v;
            total += v;
        }
        for (int e = e0; e < e1; ++e) {
            const int col = col_of(e);
            coff[col * zst + e - col * nz] = run;
            run += ccn[e];
        }
        __syncthreads();
        // per column: its end offset, its xy bounds and its (at most two)
        // runs of z-cells with one periodic shift, each one contiguous range
        // of the cell order (consecutive keys; the offset of an empty cell is
        // where the next cell starts)
        for (int col = tid; col < ncols; col += kThreads) {
            const uint32_t cend = col + 1 < ncols ? coff[(col + 1) * zst] : total;
            coff[col * zst + nz] = cend;
            const int cxu = ix + cs.dx[col], cyu = iy + cs.dy[col];
            const float x0 = __fmul_rn((float)cxu, p.cellw), y0 = __fmul_rn((float)cyu, p.cellw);
            cgeo[col] = make_float4(x0, __fadd_rn(x0, p.cellw), y0, __fadd_rn(y0, p.cellw));
            const float sx = cxu < 0 ? -L : (cxu >= G ? L : 0.0f);
            const float sy = cyu < 0 ? -L : (cyu >= G ? L : 0.0f);
            const int z0 = iz0 - R;
            // z-cells before the wrap (below z = 0 or from z = G on), if any
            const int zw = z0 < 0 ? -z0 : (z0 + nz > G ? G - z0 : nz);
            Run &r0 = runs[col * 2], &r1 = runs[col * 2 + 1];
            r0.gsrc = cst[col * nz];
            r0.soff = coff[col * zst];
            r0.cnt = (zw < nz ? coff[col * zst + zw] : cend) - r0.soff;
            r0.sx = sx;
            r0.sy = sy;
            r0.sz = z0 < 0 ? -L : 0.0f;
            r1.cnt = 0;
            if (zw < nz) {
                r1.gsrc = cst[col * nz + zw];
                r1.soff = coff[col * zst + zw];
                r1.cnt = cend - r1.soff;
                r1.sx = sx;
                r1.sy = sy;
                r1.sz = z0 < 0 ? 0.0f : L;
            }
        }
        __syncthreads();
    } else {
        if (tid == 0) {
            // the segment's cells are column (0, 0), z-cells R .. R+S-1
            const int c00 = cs.c00;
            uint32_t tb = 0, te = 0;
            bool found = false;
            for (int k = 0; k < S; ++k) {
                const uint32_t st = cst[c00 * nz + R + k], cn = ccn[c00 * nz + R + k];
                if (cn) {
                    if (!found) tb = st;
                    found = true;
                    te = st + cn;
                }
            }
            s_tbegin = tb;
            s_tend = found ? te : tb;
        }
        __syncthreads();
        const uint32_t t_seg = s_tbegin, t_seg_end = s_tend;
        t_begin = t_seg + min(slice_lo, t_seg_end - t_seg);
        t_end = t_seg + min(slice_hi, t_seg_end - t_seg);
        if (t_begin >= t_end) return true;

        // per column: staged offsets of its z-cells, runs of consecutive cells with one shift
        for (int col = tid; col < ncols; col += kThreads) {
            int cxu = ix + cs.dx[col], cyu = iy + cs.dy[col];
            const float x0 = __fmul_rn((float)cxu, p.cellw), y0 = __fmul_rn((float)cyu, p.cellw);
            cgeo[col] = make_float4(x0, __fadd_rn(x0, p.cellw), y0, __fadd_rn(y0, p.cellw));
            float sx = cxu < 0 ? -L : (cxu >= G ? L : 0.0f);
            float sy = cyu < 0 ? -L : (cyu >= G ? L : 0.0f);
            uint32_t acc = 0;
            int nrun = 0;
            int prev_wrap = -2;
            for (int zc = 0; zc < nz; ++zc) {
                int czu = iz0 - R + zc;
                int wrap = czu < 0 ? -1 : (czu >= G ? 1 : 0);
                const uint32_t st = cst[col * nz + zc], cn = ccn[col * nz + zc];
                coff[col * zst + zc] = acc;  // relative, made absolute below
                if (wrap != prev_wrap) {
                    Run &r = runs[col * 2 + (nrun < 2 ? nrun : 1)];
                    r.gsrc = 0xffffffffu;
                    r.soff = acc;
                    r.cnt = 0;
                    r.sx = sx;
                    r.sy = sy;
                    r.sz = wrap * L;
                    nrun++;
                    prev_wrap = wrap;
                }
                if (cn) {
                    Run &r = runs[col * 2 + (nrun - 1 < 1 ? nrun - 1 : 1)];
                    if (r.gsrc == 0xffffffffu) r.gsrc = st;
                    r.cnt += cn;
                }
                acc += cn;
            }
            coff[col * zst + nz] = acc;
            if (nrun < 2) runs[col * 2 + 1].cnt = 0;
            coltot[col] = acc;
        }
        __syncthreads();
        if (tid == 0) {
            uint32_t run = 0;
            for (int col = 0; col < ncols; ++col) {
                uint32_t t = coltot[col];
                coltot[col] = run;
                run += t;
            }
            s_total = run;
        }
        __syncthreads();
        for (int e = tid; e < ncols * zst; e += kThreads) coff[e] += coltot[e / zst];
        for (int col = tid; col < ncols; col += kThreads) {
            runs[col * 2].soff += coltot[col];
            runs[col * 2 + 1].soff += coltot[col];
        }
        __syncthreads();
        total = s_total;
    }
    const bool single_chunk = total <= (uint32_t)kMaxStage;
    // every column and z-cell of the stencil inside the box: no run carries a
    // periodic image shift
    const bool no_wrap = ix >= R && ix + R < G && iy >= R && iy + R < G && iz0 >= R && iz0 + S + R <= G;

    const uint32_t nt = t_end - t_begin;
    const float w = p.cellw;
    const float rc2m = (p.rcut + cs.margin) * (p.rcut + cs.margin);
    const float zbase = (float)(iz0 - R);
    const float winv = 1.0f / w;
    // integer origin at the segment corner (see the file comment)
    const float ox = floorf(ix * w), oy = floorf(iy * w), oz = floorf(iz0 * w);
    // Fixed-point positions: the origin is the segment corner on the 2^32
    // grid, and an int32 difference from it is the periodic image for free
    // (every staged source lies within S + R < G/2 cells of it).
    const uint32_t oxu = (uint32_t)(((uint64_t)ix << 32) / (uint32_t)G);
    const uint32_t oyu = (uint32_t)(((uint64_t)iy << 32) / (uint32_t)G);
    const uint32_t ozu = (uint32_t)(((uint64_t)iz0 << 32) / (uint32_t)G);
    const float fs = p.fscale;
    // __fmul_rn: a target's coordinates must equal its own staged copy bit
    // for bit (the self pair then has r = 0 exactly), so the product may not
    // be contracted into the later subtraction
    auto rel = [&](float4 a) {
        return make_float4(__fmul_rn((float)(int32_t)(__float_as_uint(a.x) - oxu), fs),
                           __fmul_rn((float)(int32_t)(__float_as_uint(a.y) - oyu), fs),
                           __fmul_rn((float)(int32_t)(__float_as_uint(a.z) - ozu), fs), 0.f);
    };
    uint32_t npairs = 0;
    uint32_t *wdelta = s_wdelta[warp];
    const uint32_t lt_mask = (1u << lane) - 1u, le_mask = lt_mask | (1u << lane);

    // The pair law, in two parts.  pair_fast2 takes the common case - inside
    // the cut, away from a table-bin edge and from the cut, outside the
    // softening length - without a branch, and reports the rest (its
    // contribution there is zero): a candidate whose bin or cut decision is
    // made in double and the spline inside h (the self pair, r = 0, adds
    // nothing and is skipped).  pair_slow applies the full law to those.  Both add into the same
    // accumulators in the same order as a single law would.
    // The bounds (law.rc2_lo, law.hmin2, law.rc2_hi) are read into registers
    // once per chunk; where they come from a box's descriptor in global memory
    // (PIN_LAW), an empty asm statement keeps them there instead of a reload
    // in every window.
    // bin = floor(asmthfac * r): a round-toward-zero fma onto 2^23 leaves the
    // floor in the mantissa, with no conversion instruction.  Plain: the bins
    // of r * asmthfac * (1 -/+ kEdge) differ when r lies within kEdge
    // (relative) of a bin edge, and such a pair is decided in double.  The
    // table is padded to kTabPad entries with its last value, so a bin index
    // masked to the padding is the clamped one (fast pairs have bins below
    // kNTab; others read a padding value they do not use).
    // The two targets of a warp's pair are evaluated together in packed FP32
    // (each float2 holds target A in .x and B in .y; Blackwell's paired
    // add/mul/fma issue one instruction for both), with the targets' negated
    // coordinates held in registers, so d = s + (-t) = s - t exactly.  Every
    // element is rounded as the scalar law rounds it: the result is the
    // scalar law's, bit for bit, for each target.
    const float2 alo2 = make_float2(law.alo, law.alo), ahi2 = make_float2(law.ahi, law.ahi);
    const float2 magic2 = make_float2(8388608.0f, 8388608.0f);
    // acc = false: the flags alone (the revisit of a window with rare-case
    // pairs), nothing added or counted.
    auto pair_fast2 = [&](float4 s, float2 ntx, float2 nty, float2 ntz, float2 &ax, float2 &ay, float2 &az,
                          bool &slow_a, bool &slow_b, bool acc, float rc2_lo, float hmin2, float rc2_hi) {
        const float2 dx = __fadd2_rn(make_float2(s.x, s.x), ntx);
        const float2 dy = __fadd2_rn(make_float2(s.y, s.y), nty);
        const float2 dz = __fadd2_rn(make_float2(s.z, s.z), ntz);
        // dist2's order: dz^2 + (dy^2 + dx^2)
        const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
        // r2 = 0 gives rinv = inf and r = NaN: not fast (r2 < hmin2), not flagged
        const float2 rinv = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
        const float2 r = __fmul2_rn(r2, rinv);
        const float2 xl = __ffma2_rz(r, alo2, magic2);
        bool edge_a = false, edge_b = false;
        if (!FIXED) {
            const float2 xh = __ffma2_rz(r, ahi2, magic2);
            edge_a = xl.x != xh.x;
            edge_b = xl.y != xh.y;
        }
        // the bin is the mantissa's low bits (2^23's own are zero)
        const float2 t = make_float2(tab[__float_as_uint(xl.x) & (kTabPad - 1)],
                                     tab[__float_as_uint(xl.y) & (kTabPad - 1)]);
        const bool fast_a = r2.x <= rc2_lo && r2.x >= hmin2 && !edge_a;
        const bool fast_b = r2.y <= rc2_lo && r2.y >= hmin2 && !edge_b;
        const float2 f = __fmul2_rn(__fmul2_rn(__fmul2_rn(rinv, rinv), rinv), t);
        const float2 fac = make_float2(fast_a ? f.x : 0.f, fast_b ? f.y : 0.f);
        if (acc) {
            ax = __ffma2_rn(dx, fac, ax);
            ay = __ffma2_rn(dy, fac, ay);
            az = __ffma2_rn(dz, fac, az);
            if (COUNT) npairs += fast_a + fast_b;
        }
        // r2 == 0 (the self pair, or a coincident source) adds dx*fac = 0:
        // not flagged, so the rare-case branch is not taken once per target
        slow_a = r2.x <= rc2_hi && r2.x != 0.f && !fast_a;
        slow_b = r2.y <= rc2_hi && r2.y != 0.f && !fast_b;
    };
    auto pair_slow = [&](float4 s, float tx, float ty, float tz, float &ax, float &ay, float &az) {
        const float dx = s.x - tx, dy = s.y - ty, dz = s.z - tz;
        const float r2 = dist2(dx, dy, dz);
        bool ok = r2 <= law.rc2_hi && r2 != 0.f;
        const float rinv = rsqrtf(ok ? r2 : 1.f);
        const float r = r2 * rinv;
        const float xl = __fmaf_rz(r, law.alo, 8388608.0f);
        int ti = __float_as_int(xl) - 0x4B000000;
        float fac = rinv * rinv * rinv;
        if (!FIXED && (xl != __fmaf_rz(r, law.ahi, 8388608.0f) || r2 > law.rc2_lo)) {
            // decided in double as the reference's CPU path computes it
            const double dd = (double)dx * dx + (double)dy * dy + (double)dz * dz;
            ok = ok && dd <= law.rcut2_d;
            ti = (int)(law.asmthfac_d * sqrt(dd));
        }
        if (r < law.h) {
            const float u = r * law.hinv;
            const float h3inv = law.h3inv;
            if (u < 0.5f)
                fac = __fmul_rn(h3inv, __fmaf_rn(__fmul_rn(u, u), __fmaf_rn(32.0f, u, -38.4f), 10.66667f));
            else
                fac = __fmul_rn(h3inv, __fsub_rn(__fmaf_rn(u, __fmaf_rn(u, __fmaf_rn(-10.66667f, u, 38.4f), -48.0f),
                                                           21.33333f),
                                                 __fdiv_rn(0.06667f, __fmul_rn(__fmul_rn(u, u), u))));
        }
        fac = ok ? fac * tab[min(ti, kNTab - 1)] : 0.f;
        ax = __fmaf_rn(dx, fac, ax);
        ay = __fmaf_rn(dy, fac, ay);
        az = __fmaf_rn(dz, fac, az);
        if (COUNT) npairs += ok;
    };

    // Two targets per warp: the warp culls the columns once for the pair
    // (lane k takes column k, k+32, ...: the column against the pair's bounding
    // box), concatenates the surviving column ranges into one candidate list,
    // and walks it 32 candidates at a time, every lane on one staged source
    // that it evaluates against both targets.  The pair shares the cull, the
    // list mapping and the source loads; each target keeps its own sums.
    // Chunk-major: each chunk of staged sources is staged once, and every
    // target of the unit runs against it; with more than one chunk the
    // targets' sums are carried in shared memory from chunk to chunk.
    const uint32_t npair = (nt + 1) / 2;
    const uint32_t rounds = (npair + kWarps - 1) / kWarps;
    const float mg = p.mass * p.G;

    // The forces on targets A and B from the sources of chunk [c0, c1),
    // warp-reduced (lane 0 holds them); FIXED: compensated, with the error
    // terms in e*.  lo/hi: the pair's bounding box (absolute), ta/tb: the
    // targets origin-relative (a missing B sits at the sentinel: it adds and
    // counts nothing).
    auto pair_chunk = [&](float4 lo, float4 hi, float4 ta, float4 tb, uint32_t c0, uint32_t c1, float &ax,
                          float &ay, float &az, float &eax, float &eay, float &eaz, float &bx, float &by, float &bz,
                          float &ebx, float &eby, float &ebz) {
        // the pair's sums (A in .x, B in .y) and negated coordinates
        float2 sx = make_float2(0.f, 0.f), sy = sx, sz = sx;
        float b_lo = law.rc2_lo, b_h = law.hmin2, b_hi = law.rc2_hi;
        if (PIN_LAW) asm volatile("" : "+f"(b_lo), "+f"(b_h), "+f"(b_hi));
        const float2 ntx = make_float2(-ta.x, -tb.x), nty = make_float2(-ta.y, -tb.y),
                     ntz = make_float2(-ta.z, -tb.z);
        for (int cb = 0; cb < ncols; cb += 32) {
            const int col = cb + lane;
            uint32_t b = 0, e = 0;
            if (col < ncols) {
                const float4 g = cgeo[col];
                const float ddx = fmaxf(fmaxf(g.x - hi.x, lo.x - g.y), 0.f);
                const float ddy = fmaxf(fmaxf(g.z - hi.y, lo.y - g.w), 0.f);
                // explicit roundings: the candidate set (hence the lane each
                // candidate lands on) must not depend on how the compiler
                // contracts this expression in a given instantiation
                const float q = __fsub_rn(rc2m, __fmaf_rn(ddy, ddy, __fmul_rn(ddx, ddx)));
                if (q >= 0.f) {
                    // half-height of the cut disc over this column (an
                    // approximate square root: the margin covers it), in
                    // cells from the column's first z-cell
                    const float hz = __fmul_rn(q, rsqrt_ftz(fmaxf(q, 1e-30f)));
                    const float ul = __fmaf_rn(lo.z - hz, winv, -zbase), uh = __fmaf_rn(hi.z + hz, winv, -zbase);
                    const int fl = __float2int_rd(ul), fh = __float2int_rd(uh);
                    const int zlo = max(fl, 0), zhi = min(fh, nz - 1);
                    if (zlo <= zhi) {
                        b = coff[col * zst + zlo];
                        e = coff[col * zst + zhi + 1];
                        if (ZS) {
                            // the end cells hold their sources by z slice: drop
                            // the slices below ul and above uh (a cell whose
                            // counts saturated, 0xffff, is kept whole)
                            if (fl >= 0) {
                                const int kl = __float2int_rd(__fmul_rn(__fsub_rn(ul, (float)fl), (float)kZSub));
                                if (kl > 0) {
                                    const uint32_t o = sl16[(col * nz + zlo) * kZSub + min(kl, kZSub) - 1];
                                    if (o != 0xffffu) b += o;
                                }
                            }
                            if (fh <= nz - 1) {
                                const int kh = __float2int_rd(__fmul_rn(__fsub_rn(uh, (float)fh), (float)kZSub));
                                if (kh < kZSub - 1) {
                                    const uint32_t o = sl16[(col * nz + zhi) * kZSub + max(kh, 0)];
                                    if (o != 0xffffu) e = coff[col * zst + zhi] + o;
                                }
                            }
                        }
                        b = max(b, c0);
                        e = min(e, c1);
                    }
                }
            }
            // The column ranges, concatenated, form one candidate list of
            // length T; ps is this lane's column start in it.
            const uint32_t len = b < e ? e - b : 0u;
            uint32_t ps = len;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t v = __shfl_up_sync(kFull, ps, off);
                if (lane >= off) ps += v;
            }
            const uint32_t T = __shfl_sync(kFull, ps, 31);
            ps -= len;
            if (T == 0) continue;
            // the k-th non-empty column's shift from list to staged index
            const uint32_t nonempty = __ballot_sync(kFull, len > 0);
            if (len > 0) wdelta[__popc(nonempty & lt_mask)] = b - c0 - ps;
            if (len == 0) ps = 0xffffffffu;  // marks no start
            __syncwarp();
            // Each window of 32 candidates: one bit per column start, so a
            // lane's column is (columns started before the window) +
            // (starts at or below its position) - 1.  Positions at or past
            // T read the sentinel.
            auto window_source = [&](uint32_t base, uint32_t before, uint32_t &m0) {
                m0 = __reduce_or_sync(kFull, bit_at(ps - base));
                const uint32_t k0 = base + lane;
                const uint32_t d0 = wdelta[before + __popc(m0 & le_mask) - 1];
                return src[CUCO_IDX(k0 < T ? k0 + d0 : (uint32_t)kMaxStage, kMaxStage + 1)];
            };
            // The windows with a rare-case pair are only marked here (at most
            // 64: T <= kMaxStage) and revisited after the last one, so the
            // loop carries none of the rare-case law's code.
            // (two windows per iteration: their loads and laws interleave)
            uint64_t wslow = 0, wbit = 1;
            uint32_t before = 0;
#pragma unroll 2
            for (uint32_t base = 0; base < T; base += 32, wbit <<= 1) {
                uint32_t m0;
                const float4 s0 = window_source(base, before, m0);
                bool xa, xb;
                pair_fast2(s0, ntx, nty, ntz, sx, sy, sz, xa, xb, true, b_lo, b_h, b_hi);
                if (__any_sync(kFull, xa || xb)) wslow |= wbit;
                before += __popc(m0);
            }
            // the rare-case pairs, window by window: the lane's candidate
            // again, its flags, and the full law for the flagged targets
            while (wslow) {
                const uint32_t w = (uint32_t)__ffsll((long long)wslow) - 1u;
                wslow &= wslow - 1;
                const uint32_t base = 32u * w;
                uint32_t m0;
                const float4 s0 = window_source(base, __popc(__ballot_sync(kFull, ps < base)), m0);
                bool xa, xb;
                float2 unused = make_float2(0.f, 0.f);
                pair_fast2(s0, ntx, nty, ntz, unused, unused, unused, xa, xb, false, b_lo, b_h, b_hi);
                if (xa) pair_slow(s0, ta.x, ta.y, ta.z, sx.x, sy.x, sz.x);
                if (xb) pair_slow(s0, tb.x, tb.y, tb.z, sx.y, sy.y, sz.y);
            }
            __syncwarp();
        }
        // The six sums (A.x A.y A.z B.x B.y B.z) over the warp in five
        // exchanges, each halving the values a lane holds: afterwards lane
        // 16 t + 4 c + j (j < 4) holds component c of target t in ax (c = 3:
        // nothing).  FIXED: compensated by error-free splitting.  With V a
        // power of two above every lane's partial sum of a target, each
        // partial is split against the quantum q = V / 2^18 into a multiple
        // of q (h = (v + C) - C, C = 1.5 * 2^23 q) and an exact remainder
        // l = v - h (|l| <= q/2).  The 32 multiples of q add exactly in any
        // order (any partial sum is at most 32 V = 2^23 q); the remainders
        // add in float, their error far below q.  The lane's result is then
        // the normalised pair (ax, eax) = (sum of the h, sum of the l).
        float h[6] = {sx.x, sy.x, sz.x, sx.y, sy.y, sz.y}, l[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (FIXED) {
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                const float m = fmaxf(fmaxf(fabsf(h[3 * t]), fabsf(h[3 * t + 1])), fabsf(h[3 * t + 2]));
                const uint32_t eb = __reduce_max_sync(kFull, __float_as_uint(m) >> 23);  // V = 2^(eb - 126)
                const float C = __uint_as_float(((eb + 6u) << 23) | 0x400000u);       // 1.5 * 2^5 V
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float v = h[3 * t + c], hv = __fsub_rn(__fadd_rn(v, C), C);
                    l[3 * t + c] = __fsub_rn(v, hv);
                    h[3 * t + c] = hv;
                }
            }
        }
        auto xchg = [&](float keep, float send, int off) {
            return __fadd_rn(keep, __shfl_xor_sync(kFull, send, off));
        };
        const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
        float k[2][3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            k[0][c] = xchg(h16 ? h[3 + c] : h[c], h16 ? h[c] : h[3 + c], 16);
            if (FIXED) k[1][c] = xchg(h16 ? l[3 + c] : l[c], h16 ? l[c] : l[3 + c], 16);
        }
        float v[2];
#pragma unroll
        for (int j = 0; j < (FIXED ? 2 : 1); ++j) {
            const float m0 = xchg(h8 ? k[j][2] : k[j][0], h8 ? k[j][0] : k[j][2], 8);
            const float m1 = xchg(h8 ? 0.f : k[j][1], h8 ? k[j][1] : 0.f, 8);
            float u = xchg(h4 ? m1 : m0, h4 ? m0 : m1, 4);
            u = xchg(u, u, 2);
            v[j] = xchg(u, u, 1);
        }
        ax = v[0];
        eax = 0.f;
        if (FIXED) two_sum(v[0], v[1], ax, eax);
        (void)ay, (void)az, (void)bx, (void)by, (void)bz, (void)eay, (void)eaz, (void)ebx, (void)eby, (void)ebz;
    };
    // the lane that writes a reduced sum, its target (0: A, 1: B) and
    // component
    const int red_c = (lane >> 2) & 3, red_t = lane >> 4;
    const bool red_w = (lane & 3) == 0 && red_c < 3;

    // a target's coordinates: absolute float (for the culling; fixed point
    // rounded to float, which the culling margin covers) and origin-relative
    // (for the pair law)
    auto load_target = [&](float4 praw, float4 &rel_out) {
        float4 pt = praw;
        if (FIXED) {
            pt = make_float4(__fmul_rn((float)__float_as_uint(praw.x), fs),
                             __fmul_rn((float)__float_as_uint(praw.y), fs),
                             __fmul_rn((float)__float_as_uint(praw.z), fs), 0.f);
            rel_out = rel(praw);
        } else {
            rel_out = make_float4(pt.x - ox, pt.y - oy, pt.z - oz, 0.f);
        }
        return pt;
    };

    // the pair (2q, 2q + 1) of round `round`: bounding box and relative
    // coordinates; a missing second target sits at the sentinel
    auto load_pair = [&](uint32_t q, float4 &lo, float4 &hi, float4 &ta, float4 &tb, bool &has_b) {
        const uint32_t t = 2 * q;
        has_b = t + 1 < nt;
        const float4 pa = load_target(s_tpos[t], ta);
        float4 pb = pa;
        tb = make_float4(kSentinel, kSentinel, kSentinel, 0.f);
        if (has_b) pb = load_target(s_tpos[t + 1], tb);
        lo = make_float4(fminf(pa.x, pb.x), fminf(pa.y, pb.y), fminf(pa.z, pb.z), 0.f);
        hi = make_float4(fmaxf(pa.x, pb.x), fmaxf(pa.y, pb.y), fmaxf(pa.z, pb.z), 0.f);
    };

    // force (already scaled by m G) to original order, PM scatter and kick
    auto epilogue = [&](uint32_t t, float4 a) {
        const uint32_t i = t_begin + t;
        const uint32_t o = perm[i];
        acc_out[o] = a;
        float4 gpm = make_float4(0.f, 0.f, 0.f, 0.f);
        const bool with_pm = kick.acc_pm_s || kick.acc_pm_o;
        if (kick.acc_pm_s) {
            gpm = kick.acc_pm_s[i];
            if (kick.acc_pm_out) kick.acc_pm_out[o] = gpm;
        } else if (kick.acc_pm_o) {
            gpm = kick.acc_pm_o[o];
        }
        if (KICK) {
            float4 v = kick.vel[o];
            // vel += GravAccel*dt; vel += GravPM*dt (timestep.c:57-58,88), in
            // float (the reference rounds each product to float first)
            const float kp = (float)kick_pp, km = (float)kick_pm;
            v.x += __fmul_rn(a.x, kp);
            v.y += __fmul_rn(a.y, kp);
            v.z += __fmul_rn(a.z, kp);
            if (with_pm) {
                v.x = __fmaf_rn(gpm.x, km, v.x);
                v.y = __fmaf_rn(gpm.y, km, v.y);
                v.z = __fmaf_rn(gpm.z, km, v.z);
            }
            kick.vel[o] = v;
        }
    };

    // stage [c0, c1): each run's part is one bulk copy into shared memory,
    // issued by one thread (run rr by thread rr mod kThreads); after the
    // barrier's phase completes, the staged sources are shifted in place to
    // the origin: all with one shift where no run is a periodic image (and in
    // fixed point, where the int32 offsets from the corner are the image),
    // else run by run, one warp per run.  Entered by all threads after a CTA
    // barrier.
    auto stage = [&](uint32_t c0, uint32_t c1) -> bool {
        if (tid == 0) bar_arrive_expect(&g_stage_bar, (c1 - c0) * (uint32_t)sizeof(float4));
        __syncthreads();
        for (int rr = tid; rr < ncols * 2; rr += kThreads) {
            const Run &r = runs[rr];
            const uint32_t lo = max(r.soff, c0), hi = min(r.soff + r.cnt, c1);
            if (r.cnt && hi > lo) {
#ifdef CUCO_BOUNDS_CHECK
                // the run lies inside the staging area (a skipped copy also
                // leaves the staging wait to time out)
                if (CUCO_IDX(hi - c0 - 1, kMaxStage) != hi - c0 - 1) continue;
#endif
                fence_async_smem();
                bulk_copy_g2s(src + (lo - c0), spos + r.gsrc + (lo - r.soff), (hi - lo) * (uint32_t)sizeof(float4),
                              &g_stage_bar);
            }
        }
        bool ok = bar_wait_bounded(&g_stage_bar, phase);
        if (!ok) ok = bar_wait_bounded(&g_stage_bar, phase);  // the copies still in flight, bounded again
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(err, 1u);
            return false;
        }
        if (FIXED || no_wrap) {
            // one shift for every staged source (fixed point: the int32
            // offset is the periodic image whatever the run)
            for (uint32_t i = tid; i < c1 - c0; i += kThreads) {
                const float4 a = src[i];
                src[i] = FIXED ? rel(a) : make_float4(a.x - ox, a.y - oy, a.z - oz, 0.f);
            }
        } else {
            for (int rr = warp; rr < ncols * 2; rr += kWarps) {
                const Run r = runs[rr];
                if (r.cnt == 0) continue;
                const float cx = ox - r.sx, cy = oy - r.sy, cz = oz - r.sz;
                const uint32_t lo = max(r.soff, c0), hi = min(r.soff + r.cnt, c1);
                for (uint32_t s0 = lo + lane; s0 < hi; s0 += 32) {
                    const float4 a = src[s0 - c0];
                    src[s0 - c0] = make_float4(a.x - cx, a.y - cy, a.z - cz, 0.f);
                }
            }
        }
        return true;
    };

    // the unit's targets, read by every round (and chunk) from shared memory
    for (uint32_t t = tid; t < nt; t += kThreads) s_tpos[t] = spos[t_begin + t];

    if (single_chunk) {
        if (!stage(0, total)) return false;
        __syncthreads();
        for (uint32_t round = 0; round < rounds; ++round) {
            const uint32_t q = round * kWarps + warp;
            if (q >= npair) break;  // warp-uniform
            float4 lo, hi, ta, tb;
            bool has_b;
            load_pair(q, lo, hi, ta, tb, has_b);
            float ax, ay, az, eax, eay, eaz, bx, by, bz, ebx, eby, ebz;
            pair_chunk(lo, hi, ta, tb, 0, total, ax, ay, az, eax, eay, eaz, bx, by, bz, ebx, eby, ebz);
            if (FIXED) ax = __fadd_rn(ax, eax);
            if (red_w && (red_t == 0 || has_b)) s_acc[red_c][2 * q + red_t] = ax * mg;
        }
        // the warp's epilogues side by side: lane 2r + j takes target j of
        // its round r pair
        __syncwarp();
        const uint32_t t = 2 * ((lane >> 1) * kWarps + warp) + (lane & 1);
        if ((lane >> 1) < rounds && t < nt) epilogue(t, make_float4(s_acc[0][t], s_acc[1][t], s_acc[2][t], 0.f));
    } else {
        for (uint32_t t = tid; t < nt; t += kThreads)
            for (int k = 0; k < 6; ++k) s_acc[k][t] = 0.f;
        // component c of target t's running sum (only the warp of t's pair
        // touches it)
        auto carry = [&](uint32_t t, int c, float x, float ex) {
            if (FIXED) {
                float e;
                two_sum(s_acc[c][t], x, s_acc[c][t], e);
                s_acc[3 + c][t] = __fadd_rn(s_acc[3 + c][t], __fadd_rn(ex, e));
            } else {
                s_acc[c][t] += x;
            }
        };
        for (uint32_t c0 = 0; c0 < total; c0 += kMaxStage) {
            const uint32_t c1 = min(total, c0 + (uint32_t)kMaxStage);
            __syncthreads();  // the previous chunk is no longer read; s_acc zeroed
            if (!stage(c0, c1)) return false;
            __syncthreads();
            for (uint32_t round = 0; round < rounds; ++round) {
                const uint32_t q = round * kWarps + warp;
                if (q >= npair) break;
                float4 lo, hi, ta, tb;
                bool has_b;
                load_pair(q, lo, hi, ta, tb, has_b);
                float ax, ay, az, eax, eay, eaz, bx, by, bz, ebx, eby, ebz;
                pair_chunk(lo, hi, ta, tb, c0, c1, ax, ay, az, eax, eay, eaz, bx, by, bz, ebx, eby, ebz);
                if (red_w && (red_t == 0 || has_b)) carry(2 * q + red_t, red_c, ax, eax);
            }
        }
        __syncthreads();
        for (uint32_t t = tid; t < nt; t += kThreads) {
            float ax = s_acc[0][t], ay = s_acc[1][t], az = s_acc[2][t];
            if (FIXED) {
                ax = __fadd_rn(ax, s_acc[3][t]);
                ay = __fadd_rn(ay, s_acc[4][t]);
                az = __fadd_rn(az, s_acc[5][t]);
            }
            epilogue(t, make_float4(ax * mg, ay * mg, az * mg, 0.f));
        }
    }
    if (COUNT) {
        uint32_t wsum = npairs;
        for (int off = 16; off > 0; off >>= 1) wsum += __shfl_xor_sync(kFull, wsum, off);
        if (lane == 0 && wsum) atomicAdd(pair_counter, (unsigned long long)wsum);
    }
    return true;
}

// The work plan of one launch: each segment's target count, and the kTMax
// slices of the segments that have more (appended in any order: which CTA
// computes a target does not change its result).
template <CellFormat FMT>
__device__ __forceinline__ void plan_segment(const ShortRangeParams &p, int S, uint32_t seg, uint32_t gseg,
                                             const uint32_t *__restrict__ ca, const uint32_t *__restrict__ cb,
                                             const SRWork &w) {
    const int G = p.grid, segs = G / S;
    const int ix = seg / (G * segs), iy = (seg / segs) % G, iz0 = (seg % segs) * S;
    uint32_t tb = 0, te = 0;
    bool found = false;
    for (int k = 0; k < S; ++k) {
        uint32_t st, cn;
        cell_range<FMT>(ca, cb, p.cell_base + ((uint32_t)ix * G + iy) * G + iz0 + k, &st, &cn);
        if (cn) {
            if (!found) tb = st;
            found = true;
            te = st + cn;
        }
    }
    const uint32_t nt = found ? te - tb : 0u;
    w.seg_nt[gseg] = nt;
    if (nt > (uint32_t)kTMax) {
        const uint32_t c = (nt + kTMax - 1) / kTMax;
        const uint32_t o = atomicAdd(&w.ctl[0], c);
        for (uint32_t k = 0; k < c; ++k)
            if (o + k < w.heavy_cap) w.heavy[o + k] = make_uint2(gseg, k);
    }
}

template <CellFormat FMT>
__global__ void k_sr_plan(const __grid_constant__ ShortRangeParams p, int S, uint32_t nseg,
                          const uint32_t *__restrict__ ca, const uint32_t *__restrict__ cb,
                          const __grid_constant__ SRWork w) {
    const uint32_t seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg < nseg) plan_segment<FMT>(p, S, seg, seg, ca, cb, w);
}

// The next unit for a persistent CTA: the dense segments' slices first (the
// longest work), then every other non-empty segment whole.  Returns false
// when none is left; `skip` for a segment that is empty or dense.
__device__ __forceinline__ bool next_unit(const SRWork &w, uint32_t nseg, uint32_t *seg, uint32_t *lo,
                                          bool *skip) {
    __shared__ uint32_t s_item;
    __syncthreads();  // the previous unit's shared memory is no longer read
    if (threadIdx.x == 0) s_item = atomicAdd(&w.ctl[1], 1u);
    __syncthreads();
    const uint32_t item = s_item, nh = min(w.ctl[0], w.heavy_cap);
    *skip = false;
    if (item < nh) {
        const uint2 h = w.heavy[item];
        *seg = h.x;
        *lo = h.y * kTMax;
        return true;
    }
    *seg = item - nh;
    if (*seg >= nseg) return false;
    const uint32_t c = w.seg_nt[*seg];
    *skip = c == 0 || c > (uint32_t)kTMax;
    *lo = 0;
    return true;
}

// The split table and the sentinel source, once per CTA: every unit reads
// them (the first unit's barrier orders these writes).
__device__ __forceinline__ void load_table(const float *__restrict__ table_g) {
    extern __shared__ float4 smem_f4[];
    float *tab = reinterpret_cast<float *>(smem_f4 + kMaxStage + 1);
    for (int i = threadIdx.x; i < kTabPad; i += kThreads) tab[i] = table_g[min(i, kNTab - 1)];
    if (threadIdx.x == 0) {
        smem_f4[kMaxStage] = make_float4(kSentinel, kSentinel, kSentinel, 0.f);
        bar_init(&g_stage_bar);
    }
}

// Persistent: as many CTAs as fit on the GPU, each taking units until none
// is left, so a few dense segments no longer leave most SMs idle.
template <CellFormat FMT, bool KICK, bool COUNT, bool FIXED>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    k_shortrange(const __grid_constant__ ShortRangeParams p, const __grid_constant__ ColumnSet cs, uint32_t nseg,
                 const __grid_constant__ SRWork w, const float4 *__restrict__ spos,
                 const uint32_t *__restrict__ perm, const uint32_t *__restrict__ ca,
                 const uint32_t *__restrict__ cb, const float *__restrict__ table_g,
                 float4 *__restrict__ acc_out, const __grid_constant__ KickArgs kick,
                 unsigned long long *__restrict__ pair_counter) {
    uint32_t seg, lo, phase = 0;
    bool skip;
    load_table(table_g);
    while (next_unit(w, nseg, &seg, &lo, &skip)) {
        if (skip) continue;
        if (!shortrange_segment<FMT, KICK, COUNT, FIXED>(p, p, cs, (int)seg, lo, lo + kTMax, kick.kick_pp,
                                                         kick.kick_pm, spos, perm, ca, cb, table_g, acc_out, kick,
                                                         pair_counter, phase, w.ctl + 2))
            return;
    }
}

// Many boxes in one launch: segments numbered box after box (seg_base, nbox+1
// entries); particles, cells (p.cell_base) and outputs are the concatenated
// arrays of all boxes.
__global__ void k_sr_plan_multi(const SRBoxDesc *__restrict__ boxes, const uint32_t *__restrict__ seg_base,
                                int nbox, uint32_t nseg, const uint32_t *__restrict__ cell_off,
                                const __grid_constant__ SRWork w) {
    const uint32_t gseg = blockIdx.x * blockDim.x + threadIdx.x;
    if (gseg >= nseg) return;
    const int b = find_box(seg_base, nbox, gseg);
    const SRBoxDesc &d = boxes[b];
    plan_segment<kCellOffsets>(d.p, d.cs.S, gseg - seg_base[b], gseg, cell_off, nullptr, w);
}

// UNIFORM: every box has the pair law of `law` (a kernel parameter, read as
// constant-bank operands); else each box's own from its descriptor.
template <bool KICK, bool COUNT, bool FIXED, bool UNIFORM>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    k_shortrange_multi(const SRBoxDesc *__restrict__ boxes, const double2 *__restrict__ kicks,
                       const uint32_t *__restrict__ seg_base, int nbox, uint32_t nseg,
                       const __grid_constant__ SRWork w, const float4 *__restrict__ spos,
                       const uint32_t *__restrict__ perm, const uint32_t *__restrict__ cell_off,
                       const float *__restrict__ table_g, float4 *__restrict__ acc_out,
                       const __grid_constant__ KickArgs kick, unsigned long long *__restrict__ pair_counter,
                       const __grid_constant__ ShortRangeParams law) {
    uint32_t seg, lo, phase = 0;
    bool skip;
    load_table(table_g);
    while (next_unit(w, nseg, &seg, &lo, &skip)) {
        if (skip) continue;
        const int b = find_box(seg_base, nbox, seg);
        const SRBoxDesc &d = boxes[b];
        const double2 k = KICK ? kicks[b] : make_double2(0.0, 0.0);
        if (!shortrange_segment<kCellOffsets, KICK, COUNT, FIXED, !UNIFORM>(d.p, UNIFORM ? law : d.p, d.cs,
                                                                  (int)(seg - seg_base[b]), lo, lo + kTMax, k.x, k.y,
                                                                  spos, perm, cell_off, nullptr, table_g, acc_out,
                                                                  kick, pair_counter, phase, w.ctl + 2))
            return;
    }
}

// CTAs a persistent launch of `kernel` keeps resident on this device.
// The persistent grid of a kernel: SMs x its resident CTAs per SM.
struct PersistentGrid {
    unsigned sms, per;
};
template <typename K>
PersistentGrid persistent_grid(K kernel, size_t smem) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kThreads, smem) != cudaSuccess || per < 1)
        per = 1;
    return {(unsigned)std::max(sms, 1), (unsigned)per};
}

// Neighbour columns (dx, dy) whose xy cell distance is within rcut (+margin).
bool build_columns(const ShortRangeParams &p, ColumnSet *cs) {
    const double w = (double)p.boxsize / p.grid;
    const double margin = 1e-5 * (double)p.boxsize + 1e-4 * w;
    const double rc = (double)p.rcut + margin;
    int R = (int)ceil(rc / w);
    if (R > kMaxR) return false;
    if (2.0 * p.rcut >= p.boxsize) return false;
    // segment length: a power of two dividing G, with the S + 2R z-cells of a
    // column at most G (so a column's z range wraps at most once)
    int S = kMaxSeg;
    // fixed point also needs every staged source within G/2 cells of the
    // segment corner (the int32 difference is the periodic image)
    auto bad = [&](int s) { return p.grid % s || p.grid < s + 2 * R || (p.fixed && 2 * (s + R) >= p.grid); };
    while (S > 1 && bad(S)) S >>= 1;
    if (bad(S)) return false;
    cs->R = R;
    cs->S = S;
    cs->margin = (float)margin;
    int n = 0;
    for (int dx = -R; dx <= R; ++dx)
        for (int dy = -R; dy <= R; ++dy) {
            double ex = fmax(abs(dx) - 1, 0) * w, ey = fmax(abs(dy) - 1, 0) * w;
            if (ex * ex + ey * ey > rc * rc) continue;
            if (dx == 0 && dy == 0) cs->c00 = n;
            cs->dx[n] = (signed char)dx;
            cs->dy[n] = (signed char)dy;
            n++;
        }
    cs->ncols = n;
    return true;
}

}  // namespace

template <CellFormat FMT, bool KICK, bool FIXED>
void launch_fmt_kick(cudaStream_t stream, cudaStream_t late_stream, const ShortRangeParams &p, const ColumnSet &cs,
                     uint32_t nseg, const SRWork &work, const float4 *sorted_pos, const uint32_t *perm,
                     const uint32_t *cell_a, const uint32_t *cell_b, const float *table,
                     float4 *acc_out, const KickArgs &kick, unsigned long long *counter) {
    const size_t sm = smem_bytes(cs.ncols, cs.S + 2 * cs.R, p.slices != nullptr);
    static const size_t sm_max = smem_base_bytes(kMaxCols, kMaxSeg + 2 * kMaxR) + kMaxSliceTable;
    static bool attr = [] {
        cudaFuncSetAttribute(k_shortrange<FMT, KICK, true, FIXED>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_max);
        cudaFuncSetAttribute(k_shortrange<FMT, KICK, false, FIXED>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_max);
        return true;
    }();
    (void)attr;
    auto launch = [&](auto kernel) {
        const PersistentGrid g = persistent_grid(kernel, sm);
        const unsigned late = late_stream && g.per > 1 ? g.sms : 0u;
        kernel<<<g.sms * g.per - late, kThreads, sm, stream>>>(p, cs, nseg, work, sorted_pos, perm, cell_a, cell_b,
                                                              table, acc_out, kick, counter);
        if (late)
            kernel<<<late, kThreads, sm, late_stream>>>(p, cs, nseg, work, sorted_pos, perm, cell_a, cell_b, table,
                                                        acc_out, kick, counter);
    };
    if (counter)
        launch(k_shortrange<FMT, KICK, true, FIXED>);
    else
        launch(k_shortrange<FMT, KICK, false, FIXED>);
}

uint32_t shortrange_heavy_cap(uint32_t n) { return 2u * (n / kTMax) + 16u; }

cuco_status_t shortrange_timeout_probe(uint32_t *ctl, long long limit_cycles, cudaStream_t stream) {
    k_staging_timeout_probe<<<1, kThreads, 0, stream>>>(ctl + 2, limit_cycles);
    CUCO_TRY_CUDA(cudaGetLastError());
    return shortrange_check(ctl, stream);
}

cuco_status_t shortrange_check(uint32_t *ctl, cudaStream_t stream) {
    uint32_t flag = 0;
    CUCO_TRY_CUDA(cudaMemcpyAsync(&flag, ctl + 2, sizeof flag, cudaMemcpyDeviceToHost, stream));
    CUCO_TRY_CUDA(cudaStreamSynchronize(stream));
    if (flag) {
        CUCO_TRY_CUDA(cudaMemsetAsync(ctl + 2, 0, sizeof(uint32_t), stream));
        set_error("short range: a bulk-copy wait into shared memory gave up after ~1 s; forces are invalid");
        return CUCO_ERR_TIMEOUT;
    }
    return CUCO_OK;
}

// The pair-law bounds the kernel reads from its parameters.
static void finish_pair_law(ShortRangeParams &p) {
    const float kEdge = 4e-7f;
    // plain: cut-edge band decided in double; fixed: the float cut
    p.rc2_lo = p.fixed ? p.rcut2 : p.rcut2 * (1.f - 2.f * kEdge);
    p.rc2_hi = p.fixed ? p.rcut2 : p.rcut2 * (1.f + 2.f * kEdge);
    const float hmin = std::max(p.h, 1e-9f);
    p.hmin2 = hmin * hmin;
    p.alo = p.fixed ? p.asmthfac : p.asmthfac * (1.f - kEdge);
    p.ahi = p.fixed ? p.asmthfac : p.asmthfac * (1.f + kEdge);
    p.rcut2_d = (double)p.rcut * (double)p.rcut;
}

// The slice table where the sources are in slice order and it fits.
static bool use_slices(const ShortRangeParams &p, const ColumnSet &cs) {
    return p.slices != nullptr && sizeof(uint4) * (size_t)cs.ncols * (cs.S + 2 * cs.R) <= kMaxSliceTable;
}

cuco_status_t launch_shortrange(const ShortRangeParams &p_in, const float4 *sorted_pos,
                                const uint32_t *perm, const uint32_t *cell_a,
                                const uint32_t *cell_b, CellFormat fmt, const float *table,
                                float4 *acc_out, const KickArgs &kick, const SRWork &work, cudaStream_t stream,
                                unsigned long long *pair_counter, cudaStream_t late_stream, cudaEvent_t plan_done) {
    ColumnSet cs;
    ShortRangeParams p = p_in;
    finish_pair_law(p);
    if (!build_columns(p, &cs)) {
        set_error("short range: cell grid does not fit rcut (need rcut <= 8 cell widths, "
                  "rcut < L/2 and at least S+2R cells per dimension)");
        return CUCO_ERR_UNSUPPORTED;
    }
    if (p.n == 0) return CUCO_OK;
    const int G = p.grid;
    const uint32_t nseg = (uint32_t)G * G * (G / cs.S);
    if (nseg > work.seg_cap || work.heavy_cap < shortrange_heavy_cap(p.n)) {
        set_error("short range: work-plan scratch too small for this grid or particle count");
        return CUCO_ERR_INVALID;
    }
    const bool kick_on = kick.vel != nullptr;
    if (fmt != kCellOffsets || !use_slices(p, cs)) p.slices = nullptr;
    if (p.fixed && fmt != kCellOffsets) {
        set_error("short range: fixed-point positions need the engine's cell-offset format");
        return CUCO_ERR_UNSUPPORTED;
    }
    CUCO_TRY_CUDA(cudaMemsetAsync(work.ctl, 0, 2 * sizeof(uint32_t), stream));
    if (fmt == kCellOffsets)
        k_sr_plan<kCellOffsets><<<(nseg + 255) / 256, 256, 0, stream>>>(p, cs.S, nseg, cell_a, cell_b, work);
    else
        k_sr_plan<kCellStartEnd><<<(nseg + 255) / 256, 256, 0, stream>>>(p, cs.S, nseg, cell_a, cell_b, work);
    if (late_stream) {
        if (!plan_done) {
            set_error("short range: a split launch needs the caller's plan event");
            return CUCO_ERR_INVALID;
        }
        CUCO_TRY_CUDA(cudaEventRecord(plan_done, stream));
        CUCO_TRY_CUDA(cudaStreamWaitEvent(late_stream, plan_done, 0));
    }
    if (p.fixed) {
        if (kick_on)
            launch_fmt_kick<kCellOffsets, true, true>(stream, late_stream, p, cs, nseg, work, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
        else
            launch_fmt_kick<kCellOffsets, false, true>(stream, late_stream, p, cs, nseg, work, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
    } else if (fmt == kCellOffsets) {
        if (kick_on)
            launch_fmt_kick<kCellOffsets, true, false>(stream, late_stream, p, cs, nseg, work, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
        else
            launch_fmt_kick<kCellOffsets, false, false>(stream, late_stream, p, cs, nseg, work, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
    } else {
        if (kick_on)
            launch_fmt_kick<kCellStartEnd, true, false>(stream, late_stream, p, cs, nseg, work, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
        else
            launch_fmt_kick<kCellStartEnd, false, false>(stream, late_stream, p, cs, nseg, work, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
    }
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

size_t shortrange_desc_bytes() { return sizeof(SRBoxDesc); }

cuco_status_t shortrange_desc_fill(const ShortRangeParams &p, void *desc, uint32_t *segments, size_t *smem) {
    SRBoxDesc d{};
    d.p = p;
    finish_pair_law(d.p);
    if (!build_columns(p, &d.cs)) {
        set_error("short range: cell grid does not fit rcut (need rcut <= 8 cell widths, "
                  "rcut < L/2 and at least S+2R cells per dimension)");
        return CUCO_ERR_UNSUPPORTED;
    }
    if (!use_slices(d.p, d.cs)) d.p.slices = nullptr;
    memcpy(desc, &d, sizeof d);
    *segments = (uint32_t)p.grid * p.grid * (p.grid / d.cs.S);
    *smem = smem_bytes(d.cs.ncols, d.cs.S + 2 * d.cs.R, d.p.slices != nullptr);
    return CUCO_OK;
}

bool shortrange_descs_uniform_law(const void *host_descs, int nbox) {
    const SRBoxDesc *d = static_cast<const SRBoxDesc *>(host_descs);
    for (int b = 1; b < nbox; ++b) {
        const ShortRangeParams &x = d[0].p, &y = d[b].p;
        if (x.rc2_lo != y.rc2_lo || x.rc2_hi != y.rc2_hi || x.hmin2 != y.hmin2 || x.alo != y.alo ||
            x.ahi != y.ahi || x.rcut2_d != y.rcut2_d || x.asmthfac_d != y.asmthfac_d || x.h != y.h ||
            x.hinv != y.hinv || x.h3inv != y.h3inv)
            return false;
    }
    return nbox > 0;
}

cuco_status_t launch_shortrange_multi(const void *descs, const double2 *kicks, const uint32_t *seg_base,
                                      int nbox, uint32_t segments, size_t smem, bool fixed,
                                      const float4 *sorted_pos, const uint32_t *perm, const uint32_t *cell_off,
                                      const float *table, float4 *acc_out, const KickArgs &kick,
                                      const SRWork &work, cudaStream_t stream, unsigned long long *pair_counter,
                                      const void *uniform_law_desc) {
    static const size_t sm_max = smem_base_bytes(kMaxCols, kMaxSeg + 2 * kMaxR) + kMaxSliceTable;
    static bool attr = [] {
#define CUCO_SR_MULTI_ATTR(K, C, F, U) \
    cudaFuncSetAttribute(k_shortrange_multi<K, C, F, U>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_max)
        CUCO_SR_MULTI_ATTR(true, true, true, false);
        CUCO_SR_MULTI_ATTR(true, false, true, false);
        CUCO_SR_MULTI_ATTR(false, true, true, false);
        CUCO_SR_MULTI_ATTR(false, false, true, false);
        CUCO_SR_MULTI_ATTR(true, true, false, false);
        CUCO_SR_MULTI_ATTR(true, false, false, false);
        CUCO_SR_MULTI_ATTR(false, true, false, false);
        CUCO_SR_MULTI_ATTR(false, false, false, false);
        CUCO_SR_MULTI_ATTR(true, true, true, true);
        CUCO_SR_MULTI_ATTR(true, false, true, true);
        CUCO_SR_MULTI_ATTR(false, true, true, true);
        CUCO_SR_MULTI_ATTR(false, false, true, true);
        CUCO_SR_MULTI_ATTR(true, true, false, true);
        CUCO_SR_MULTI_ATTR(true, false, false, true);
        CUCO_SR_MULTI_ATTR(false, true, false, true);
        CUCO_SR_MULTI_ATTR(false, false, false, true);
#undef CUCO_SR_MULTI_ATTR
        return true;
    }();
    (void)attr;
    if (!segments) return CUCO_OK;
    if (segments > work.seg_cap) {
        set_error("short range: work-plan scratch too small for the ensemble's segments");
        return CUCO_ERR_INVALID;
    }
    const SRBoxDesc *d = static_cast<const SRBoxDesc *>(descs);
    const bool kick_on = kick.vel != nullptr;
    CUCO_TRY_CUDA(cudaMemsetAsync(work.ctl, 0, 2 * sizeof(uint32_t), stream));
    k_sr_plan_multi<<<(segments + 255) / 256, 256, 0, stream>>>(d, seg_base, nbox, segments, cell_off, work);
    // the shared law (any box's, all being equal) or, unused, box 0's shape
    ShortRangeParams law{};
    const bool uniform = uniform_law_desc != nullptr;
    if (uniform) law = static_cast<const SRBoxDesc *>(uniform_law_desc)->p;
#define CUCO_SR_MULTI_U(K, C, F, U)                                                                     \
    do {                                                                                                \
        const PersistentGrid g = persistent_grid(k_shortrange_multi<K, C, F, U>, smem);                  \
        k_shortrange_multi<K, C, F, U><<<g.sms * g.per, kThreads, smem, stream>>>(                       \
            d, kicks, seg_base, nbox, segments, work, sorted_pos, perm, cell_off, table, acc_out, kick,     \
            pair_counter, law);                                                                         \
    } while (0)
#define CUCO_SR_MULTI(K, C, F)                 \
    do {                                       \
        if (uniform)                           \
            CUCO_SR_MULTI_U(K, C, F, true);    \
        else                                   \
            CUCO_SR_MULTI_U(K, C, F, false);   \
    } while (0)
    if (fixed) {
        if (kick_on) {
            if (pair_counter) CUCO_SR_MULTI(true, true, true); else CUCO_SR_MULTI(true, false, true);
        } else {
            if (pair_counter) CUCO_SR_MULTI(false, true, true); else CUCO_SR_MULTI(false, false, true);
        }
    } else {
        if (kick_on) {
            if (pair_counter) CUCO_SR_MULTI(true, true, false); else CUCO_SR_MULTI(true, false, false);
        } else {
            if (pair_counter) CUCO_SR_MULTI(false, true, false); else CUCO_SR_MULTI(false, false, false);
        }
    }
#undef CUCO_SR_MULTI
#undef CUCO_SR_MULTI_U
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

uint32_t bounds_violations_shortrange() { return bounds_violations_take(); }

}  // namespace cuco
