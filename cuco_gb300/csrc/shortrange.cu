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
//   * one CTA per z-segment of S consecutive cells (ix, iy, iz0..iz0+S-1); its
//     targets are one contiguous range of the cell-sorted particles;
//   * the sources are the neighbour columns (dx, dy) within rcut of the
//     segment in xy, over z-cells iz0-R .. iz0+S-1+R.  A column's cells are
//     consecutive keys, so it is at most two contiguous runs of sorted
//     particles (two when the z range wraps); warps copy the runs into shared
//     memory relative to an integer origin at the segment corner, with the
//     periodic image shift applied once per run;
//   * each target has one lane, or a power-of-two group of lanes when the
//     segment is sparse; its lanes cull columns by the target's xy distance,
//     narrow each column to the z-cells within sqrt(rcut^2 - d_xy^2), and walk
//     those sources (lane k of the group takes every tpt-th one, so the group
//     reads consecutive staged sources);
//   * the pair law runs without branches on the common path (a candidate
//     beyond the cut gets a zero factor), two candidates per iteration into
//     two accumulator sets for instruction-level parallelism.  Lanes of a warp
//     hold different targets, so any per-candidate branch would be taken by
//     some lane and cost the whole warp anyway;
//   * 256-thread CTAs over 8-cell segments keep 8+ warps per scheduler on the
//     shared memory a segment needs;
//   * the lanes of a target add their partial sums with xor shuffles;
//   * the epilogue scatters the force to original particle order and, in the
//     engine's step, kicks the velocity (timestep.c:56-59,86-91).
//
// Precision of the plain path.  A float computation of asmthfac*r lands in the
// neighbouring table bin for ~3e-5 of the pairs, and at high redshift (net
// force a small residual of cancelling pair terms) that alone costs ~1.6e-4
// rms against the reference's double path.  Coordinates relative to an integer
// origin make the image shift exact (origin -/+ L is an exact float for
// L < 2^23) and dx exact for ~97% of pairs; pairs whose r^2 lies within
// 4e-7 of rcut^2 or whose asmthfac*r lies within 4e-7 (relative) of a bin edge
// are decided in double as gravlist.cpp:298-320 does.
#include "common.cuh"

namespace cuco {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxStage = 2048;  // staged sources per chunk (32 KB)
constexpr int kMaxR = 8;         // neighbour reach in cells (the reference's G = PMGRID needs 6)
constexpr int kMaxCols = (2 * kMaxR + 1) * (2 * kMaxR + 1);
constexpr int kMaxSeg = 8;
constexpr unsigned kFull = 0xffffffffu;

struct ColumnSet {
    int ncols;
    int R;
    int S;
    float margin;  // culling slack for the float cell assignment (length units)
    signed char dx[kMaxCols];
    signed char dy[kMaxCols];
};

struct Run {
    uint32_t gsrc;  // first sorted index
    uint32_t soff;  // first staged index (stencil order)
    uint32_t cnt;
    float sx, sy, sz;
};

// Dynamic shared memory, in order: staged sources, split table,
// per-(column, z-cell) staged offsets, cell starts and counts, column runs,
// column totals.
__host__ __device__ inline size_t smem_bytes(int ncols, int nz) {
    return sizeof(float4) * kMaxStage + sizeof(float) * kNTab + sizeof(uint32_t) * (size_t)ncols * (nz + 1) +
           2 * sizeof(uint32_t) * (size_t)ncols * nz + sizeof(Run) * 2 * (size_t)ncols +
           sizeof(uint32_t) * (size_t)ncols;
}

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

// r^2 with a fixed operation order: the candidate test and the force pass
// must agree on it bit for bit.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

template <CellFormat FMT, bool KICK, bool COUNT>
__global__ void __launch_bounds__(kThreads, 4)
    k_shortrange(ShortRangeParams p, ColumnSet cs, const float4 *__restrict__ spos,
                 const uint32_t *__restrict__ perm, const uint32_t *__restrict__ ca,
                 const uint32_t *__restrict__ cb, const float *__restrict__ table_g,
                 float4 *__restrict__ acc_out, KickArgs kick,
                 unsigned long long *__restrict__ pair_counter) {
    extern __shared__ float4 smem_f4[];
    __shared__ uint32_t s_total, s_tbegin, s_tend;

    const int G = p.grid;
    const int S = cs.S, R = cs.R, nz = S + 2 * R, ncols = cs.ncols;
    const int zst = nz + 1;  // coff stride per column
    float4 *src = smem_f4;
    float *tab = reinterpret_cast<float *>(src + kMaxStage);
    uint32_t *coff = reinterpret_cast<uint32_t *>(tab + kNTab);
    uint32_t *cst = coff + ncols * zst;
    uint32_t *ccn = cst + ncols * nz;
    Run *runs = reinterpret_cast<Run *>(ccn + ncols * nz);
    uint32_t *coltot = reinterpret_cast<uint32_t *>(runs + 2 * ncols);

    const int segs = G / S;
    const int seg = blockIdx.x;
    const int ix = seg / (G * segs);
    const int iy = (seg / segs) % G;
    const int iz0 = (seg % segs) * S;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float L = p.boxsize;

    // every (column, z-cell) range, loaded in parallel
    for (int e = tid; e < ncols * nz; e += kThreads) {
        const int col = e / nz, zc = e % nz;
        int cxu = ix + cs.dx[col], cyu = iy + cs.dy[col], czu = iz0 - R + zc;
        int cx = cxu < 0 ? cxu + G : (cxu >= G ? cxu - G : cxu);
        int cy = cyu < 0 ? cyu + G : (cyu >= G ? cyu - G : cyu);
        int cz = czu < 0 ? czu + G : (czu >= G ? czu - G : czu);
        uint32_t st, cn;
        cell_range<FMT>(ca, cb, ((uint32_t)cx * G + cy) * G + cz, &st, &cn);
        cst[e] = st;
        ccn[e] = cn;
    }
    __syncthreads();
    if (tid == 0) {
        // the segment's cells are column (0, 0), z-cells R .. R+S-1
        int c00 = -1;
        for (int col = 0; col < ncols; ++col)
            if (cs.dx[col] == 0 && cs.dy[col] == 0) c00 = col;
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
    const uint32_t t_begin = s_tbegin, t_end = s_tend;
    if (t_begin == t_end) return;

    for (int i = tid; i < kNTab; i += kThreads) tab[i] = table_g[i];

    // per column: staged offsets of its z-cells, runs of consecutive cells with one shift
    for (int col = tid; col < ncols; col += kThreads) {
        int cxu = ix + cs.dx[col], cyu = iy + cs.dy[col];
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
    const uint32_t total = s_total;
    const bool single_chunk = total <= (uint32_t)kMaxStage;

    // lanes per target (a power of two): sparse segments give a target
    // several lanes, which take interleaved sources of each of its ranges
    const uint32_t nt = t_end - t_begin;
    int tpt = 1;
    while (tpt < 32 && (uint32_t)(tpt * 2) * nt <= (uint32_t)kThreads) tpt *= 2;
    const int tpc = kThreads / tpt;
    const int sub = tid & (tpt - 1);

    const float w = p.cellw;
    const float rc2m = (p.rcut + cs.margin) * (p.rcut + cs.margin);
    const float zbase = (float)(iz0 - R);
    const float winv = 1.0f / w;
    // integer origin at the segment corner (see the file comment)
    const float ox = floorf(ix * w), oy = floorf(iy * w), oz = floorf(iz0 * w);
    const float kEdge = 4e-7f;
    const float rc2_lo = p.rcut2 * (1.f - 2.f * kEdge), rc2_hi = p.rcut2 * (1.f + 2.f * kEdge);
    const double rcut2_d = (double)p.rcut * (double)p.rcut;
    bool staged = false;
    uint32_t npairs = 0;

    float tx = 0.f, ty = 0.f, tz = 0.f;  // the current target, origin-relative

    // Kernel parameters used per candidate, held in registers.
    const float asmf = p.asmthfac, hh = p.h, hinv = p.hinv, h3inv = p.h3inv;
    const double asmd = p.asmthfac_d;

    // The pair law for one candidate.  The common case (inside the cut, away
    // from a table-bin edge, outside the softening length) has no branch; the
    // rare cases - a bin or cut edge decided in double, the spline inside h -
    // share one branch.  A candidate beyond the cut gets a zero factor.
    auto pair = [&](float4 s, float &ax, float &ay, float &az) {
        const float dx = s.x - tx, dy = s.y - ty, dz = s.z - tz;
        const float r2 = dist2(dx, dy, dz);
        bool ok = r2 <= rc2_hi && r2 != 0.f;
        const float rinv = rsqrtf(ok ? r2 : 1.f);
        const float r = r2 * rinv;
        // bin = floor(asmthfac * r) without a conversion instruction: a
        // round-toward-zero add of 2^23 leaves floor(x) in the mantissa
        const float xt = asmf * r;
        const float xf = __fadd_rz(xt, 8388608.0f);
        int ti = __float_as_int(xf) - 0x4B000000;
        const float frac = xt - (xf - 8388608.0f);
        float fac = rinv * rinv * rinv;
        const bool edge = fabsf(frac - 0.5f) > __fmaf_rn(-kEdge, xt, 0.5f) || r2 > rc2_lo;
        if (ok && (edge || r < hh)) {
            if (edge) {
                // decided in double as the reference's CPU path computes it
                const double dd = (double)dx * dx + (double)dy * dy + (double)dz * dz;
                ok = dd <= rcut2_d;
                ti = (int)(asmd * sqrt(dd));
            }
            if (r < hh) {
                const float u = r * hinv;
                if (u < 0.5f)
                    fac = h3inv * (10.66667f + u * u * (32.0f * u - 38.4f));
                else
                    fac = h3inv * (21.33333f - 48.0f * u + 38.4f * u * u - 10.66667f * u * u * u -
                                   0.06667f / (u * u * u));
            }
        }
        fac = ok ? fac * tab[min(ti, kNTab - 1)] : 0.f;
        ax = __fmaf_rn(dx, fac, ax);
        ay = __fmaf_rn(dy, fac, ay);
        az = __fmaf_rn(dz, fac, az);
        if (COUNT) npairs += ok;
    };

    for (uint32_t tb = 0; tb < nt; tb += tpc) {
        const uint32_t t = tb + tid / tpt;
        const bool active = t < nt;
        const float4 pt = active ? spos[t_begin + t] : make_float4(0.f, 0.f, 0.f, 0.f);
        tx = pt.x - ox;
        ty = pt.y - oy;
        tz = pt.z - oz;
        // two accumulator sets: the unrolled candidate pairs are independent
        float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
        for (uint32_t c0 = 0; c0 < total; c0 += kMaxStage) {
            const uint32_t c1 = min(total, c0 + (uint32_t)kMaxStage);
            if (!(single_chunk && staged)) {
                __syncthreads();
                // stage [c0, c1): warp per run
                for (int rr = warp; rr < ncols * 2; rr += kWarps) {
                    const Run r = runs[rr];
                    if (r.cnt == 0) continue;
                    const float cx = ox - r.sx, cy = oy - r.sy, cz = oz - r.sz;
                    uint32_t lo = max(r.soff, c0), hi = min(r.soff + r.cnt, c1);
                    for (uint32_t s0 = lo + lane; s0 < hi; s0 += 64) {
                        const uint32_t s1 = s0 + 32;
                        const float4 a0 = spos[r.gsrc + (s0 - r.soff)];
                        float4 a1 = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (s1 < hi) a1 = spos[r.gsrc + (s1 - r.soff)];
                        src[s0 - c0] = make_float4(a0.x - cx, a0.y - cy, a0.z - cz, 0.f);
                        if (s1 < hi) src[s1 - c0] = make_float4(a1.x - cx, a1.y - cy, a1.z - cz, 0.f);
                    }
                }
                __syncthreads();
                staged = true;
            }
            if (!active) continue;
            for (int col = 0; col < ncols; ++col) {
                const float x0 = (ix + cs.dx[col]) * w, y0 = (iy + cs.dy[col]) * w;
                const float ddx = fmaxf(fmaxf(x0 - pt.x, pt.x - (x0 + w)), 0.f);
                const float ddy = fmaxf(fmaxf(y0 - pt.y, pt.y - (y0 + w)), 0.f);
                const float d2 = ddx * ddx + ddy * ddy;
                if (d2 > rc2m) continue;
                const float hz = sqrtf(rc2m - d2);
                const int zlo = max((int)floorf((pt.z - hz) * winv - zbase), 0);
                const int zhi = min((int)floorf((pt.z + hz) * winv - zbase), nz - 1);
                if (zlo > zhi) continue;
                const uint32_t b = max(coff[col * zst + zlo], c0);
                const uint32_t e = min(coff[col * zst + zhi + 1], c1);
                uint32_t j = b + sub;
                for (; j + 3 * tpt < e; j += 4 * tpt) {
                    const float4 s0 = src[j - c0];
                    const float4 s1 = src[j + tpt - c0];
                    const float4 s2 = src[j + 2 * tpt - c0];
                    const float4 s3 = src[j + 3 * tpt - c0];
                    pair(s0, ax, ay, az);
                    pair(s1, bx, by, bz);
                    pair(s2, ax, ay, az);
                    pair(s3, bx, by, bz);
                }
                for (; j < e; j += tpt) pair(src[j - c0], ax, ay, az);
            }
        }
        ax += bx;
        ay += by;
        az += bz;
        if (COUNT) {
            uint32_t wsum = npairs;
            for (int off = 16; off > 0; off >>= 1) wsum += __shfl_xor_sync(kFull, wsum, off);
            if (lane == 0 && wsum) atomicAdd(pair_counter, (unsigned long long)wsum);
            npairs = 0;
        }
        for (int off = tpt >> 1; off > 0; off >>= 1) {
            ax += __shfl_xor_sync(kFull, ax, off);
            ay += __shfl_xor_sync(kFull, ay, off);
            az += __shfl_xor_sync(kFull, az, off);
        }
        if (active && sub == 0) {
            const uint32_t i = t_begin + t;
            const uint32_t o = perm[i];
            const float mg = p.mass * p.G;
            const float4 a = make_float4(ax * mg, ay * mg, az * mg, 0.f);
            acc_out[o] = a;
            float4 gpm = make_float4(0.f, 0.f, 0.f, 0.f);
            if (kick.acc_pm_s) {
                gpm = kick.acc_pm_s[i];
                if (kick.acc_pm_out) kick.acc_pm_out[o] = gpm;
            }
            if (KICK) {
                float4 v = kick.vel[o];
                // vel += GravAccel*dt; vel += GravPM*dt (timestep.c:57-58,88), in
                // float (the reference rounds each product to float first)
                const float kp = (float)kick.kick_pp, km = (float)kick.kick_pm;
                v.x += __fmul_rn(a.x, kp);
                v.y += __fmul_rn(a.y, kp);
                v.z += __fmul_rn(a.z, kp);
                if (kick.acc_pm_s) {
                    v.x = __fmaf_rn(gpm.x, km, v.x);
                    v.y = __fmaf_rn(gpm.y, km, v.y);
                    v.z = __fmaf_rn(gpm.z, km, v.z);
                }
                kick.vel[o] = v;
            }
        }
    }
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
    while (S > 1 && (p.grid % S || p.grid < S + 2 * R)) S >>= 1;
    if (p.grid < S + 2 * R) return false;
    cs->R = R;
    cs->S = S;
    cs->margin = (float)margin;
    int n = 0;
    for (int dx = -R; dx <= R; ++dx)
        for (int dy = -R; dy <= R; ++dy) {
            double ex = fmax(abs(dx) - 1, 0) * w, ey = fmax(abs(dy) - 1, 0) * w;
            if (ex * ex + ey * ey > rc * rc) continue;
            cs->dx[n] = (signed char)dx;
            cs->dy[n] = (signed char)dy;
            n++;
        }
    cs->ncols = n;
    return true;
}

}  // namespace

template <CellFormat FMT, bool KICK>
void launch_fmt_kick(unsigned blocks, cudaStream_t stream, const ShortRangeParams &p,
                     const ColumnSet &cs, const float4 *sorted_pos, const uint32_t *perm,
                     const uint32_t *cell_a, const uint32_t *cell_b, const float *table,
                     float4 *acc_out, const KickArgs &kick, unsigned long long *counter) {
    const size_t sm = smem_bytes(cs.ncols, cs.S + 2 * cs.R);
    static const size_t sm_max = smem_bytes(kMaxCols, kMaxSeg + 2 * kMaxR);
    static bool attr = [] {
        cudaFuncSetAttribute(k_shortrange<FMT, KICK, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_max);
        cudaFuncSetAttribute(k_shortrange<FMT, KICK, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_max);
        return true;
    }();
    (void)attr;
    if (counter)
        k_shortrange<FMT, KICK, true><<<blocks, kThreads, sm, stream>>>(
            p, cs, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, counter);
    else
        k_shortrange<FMT, KICK, false><<<blocks, kThreads, sm, stream>>>(
            p, cs, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, counter);
}

cuco_status_t launch_shortrange(const ShortRangeParams &p, const float4 *sorted_pos,
                                const uint32_t *perm, const uint32_t *cell_a,
                                const uint32_t *cell_b, CellFormat fmt, const float *table,
                                float4 *acc_out, const KickArgs &kick, cudaStream_t stream,
                                unsigned long long *pair_counter) {
    ColumnSet cs;
    if (!build_columns(p, &cs)) {
        set_error("short range: cell grid does not fit rcut (need rcut <= 8 cell widths, "
                  "rcut < L/2 and at least S+2R cells per dimension)");
        return CUCO_ERR_UNSUPPORTED;
    }
    if (p.n == 0) return CUCO_OK;
    const int G = p.grid;
    const unsigned blocks = (unsigned)G * G * (G / cs.S);
    const bool kick_on = kick.vel != nullptr;
    if (fmt == kCellOffsets) {
        if (kick_on)
            launch_fmt_kick<kCellOffsets, true>(blocks, stream, p, cs, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
        else
            launch_fmt_kick<kCellOffsets, false>(blocks, stream, p, cs, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
    } else {
        if (kick_on)
            launch_fmt_kick<kCellStartEnd, true>(blocks, stream, p, cs, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
        else
            launch_fmt_kick<kCellStartEnd, false>(blocks, stream, p, cs, sorted_pos, perm, cell_a, cell_b, table, acc_out, kick, pair_counter);
    }
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

}  // namespace cuco
