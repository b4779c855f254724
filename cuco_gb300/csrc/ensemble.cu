// Batched form: many independent boxes advanced together, one launch per
// phase.  No counterpart in the reference, which runs one box per process.
//
// Layout.  All boxes' particles are concatenated (box b owns [pbeg[b],
// pbeg[b+1])), and so are their cells: a particle's key is the box's first
// cell (cell_base) plus its cell in the box.  One stable radix sort of those
// keys therefore sorts every box at once and keeps each box's particles in
// its own range; one reorder builds every box's cell offsets.  Each PM phase
// is one launch over all boxes' meshes (a per-CTA (box, block) map), and the
// short range is one launch over all boxes' segments (a segment prefix
// table).  The per-step factors of every box (drift, kicks) sit in a small
// device array refreshed from pinned host memory by a copy queued before each
// step, so the rest of the step is one CUDA graph; the pinned factors have two
// slots used in turn, and the host waits only for the copy of two steps back,
// never for the step in flight.
//
// Autotuning.  A box's short-range cell grid G (cell_grid = 0) and its FFT
// batching (columns per CTA) are chosen by timing candidates on a scratch box
// of the same particle count and mesh with uniform positions; results are
// cached per (n, M, mode), since R = ceil(rcut / w) depends only on G / M.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "common.cuh"

namespace cuco {

namespace {

using DriftBox = CellBox;  // a box's cell grid: drift, keys and the z-slice order

struct StepFactors {
    float units_per_time;  // fixed point: drift * 2^32 / L; plain: the drift factor
    float pad;
    double kick_pp, kick_pm;
};

__global__ void k_drift_keys_multi(float4 *__restrict__ pos, const float4 *__restrict__ vel,
                                   uint32_t *__restrict__ keys, uint32_t n, const uint32_t *__restrict__ pbeg,
                                   int nbox, const DriftBox *__restrict__ boxes,
                                   const StepFactors *__restrict__ f, int do_drift, int fixed) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = find_box(pbeg, nbox, i);
    const DriftBox d = boxes[b];
    const float4 p = pos[i];
    uint32_t k[3];
    if (fixed) {
        // the precision form's drift: one rounding to the 2^-32 L grid, then a
        // modular add (exact periodic wrap); key floor(x * G / 2^32)
        uint32_t c[3] = {__float_as_uint(p.x), __float_as_uint(p.y), __float_as_uint(p.z)};
        if (do_drift) {
            const float4 v = vel[i];
            const float vv[3] = {v.x, v.y, v.z};
            const float upt = f[b].units_per_time;
#pragma unroll
            for (int a = 0; a < 3; ++a) c[a] += (uint32_t)__float2ll_rn(vv[a] * upt);
            pos[i] = make_float4(__uint_as_float(c[0]), __uint_as_float(c[1]), __uint_as_float(c[2]), p.w);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) k[a] = (uint32_t)(((uint64_t)c[a] * d.G) >> 32);
    } else {
        // the plain form's drift and wrap (predict.c:19,34-38) and key rule
        // (gravlist_kernel.cu:108-113), as the single-box engine does them
        float c[3] = {p.x, p.y, p.z};
        if (do_drift) {
            const float4 v = vel[i];
            const float vv[3] = {v.x, v.y, v.z};
            const float dt = f[b].units_per_time;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                float x = __fmaf_rn(vv[a], dt, c[a]);
                for (int it = 0; it < 8 && x < 0.f; ++it) x = __fadd_rn(x, d.boxsize);
                for (int it = 0; it < 8 && x >= d.boxsize; ++it) x = __fsub_rn(x, d.boxsize);
                c[a] = x;
            }
            pos[i] = make_float4(c[0], c[1], c[2], p.w);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            int v = (int)__fmul_rn(d.gridfac, c[a]);
            v = v < 0 ? 0 : v;
            k[a] = (uint32_t)(v >= (int)d.G ? d.G - 1 : v);
        }
    }
    keys[i] = d.cell_base + (k[0] * d.G + k[1]) * d.G + k[2];
}

int key_bits(uint64_t ncells) {
    int b = 1;
    while ((1ull << b) < ncells) ++b;
    return b;
}

template <typename T>
cuco_status_t dalloc(T **p, size_t count) {
    cudaError_t e = cudaMalloc(p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return CUCO_ERR_NOMEM;
    }
    return CUCO_OK;
}

// Ensemble arrays come from the device's stream-ordered pool, which keeps
// freed memory for reuse (release threshold raised once per device): a
// serving loop rebuilds its ensemble whenever jobs join or leave, and must not
// pay cudaMalloc/cudaFree each time.
void pool_keep_memory(int device) {
    static std::mutex mu;
    static bool done[64] = {};
    std::lock_guard<std::mutex> lk(mu);
    if (device < 0 || device >= 64 || done[device]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    done[device] = true;
}

template <typename T>
cuco_status_t palloc(T **p, size_t count, cudaStream_t s) {
    cudaError_t e = cudaMallocAsync((void **)p, sizeof(T) * (count ? count : 1), s);
    if (e != cudaSuccess) {
        set_error(std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
        return CUCO_ERR_NOMEM;
    }
    return CUCO_OK;
}

ShortRangeParams sr_params(const cuco_config_t &c, uint32_t n, uint32_t cell_base, const uint4 *slices) {
    ShortRangeParams p{};
    p.boxsize = c.boxsize;
    p.gridfac = (float)c.cell_grid / c.boxsize;
    p.cellw = c.boxsize / c.cell_grid;
    p.rcut = c.rcut;
    p.rcut2 = c.rcut * c.rcut;
    p.asmthfac_d = 0.5 / (double)c.asmth * (kNTab / 3.0);
    p.asmthfac = (float)p.asmthfac_d;
    p.mass = c.mass;
    p.G = (float)c.G;
    p.h = c.softening;
    p.hinv = (float)(1.0 / (double)c.softening);
    p.h3inv = p.hinv * p.hinv * p.hinv;
    p.grid = c.cell_grid;
    p.n = n;
    p.fixed = c.mode == CUCO_MODE_FIXED;
    p.fscale = ldexpf(c.boxsize, -32);
    p.cell_base = cell_base;
    p.slices = slices;
    return p;
}

// ------------------------------------------------------------ autotuner

struct Tuned {
    int cell_grid, P, B;
};

std::mutex g_tune_mu;
std::map<std::tuple<int64_t, int, int>, Tuned> g_tune_cache;

// Shortest measured short-range time among the admissible cell grids.
int tune_cell_grid(const cuco_config_t &c0, cudaStream_t stream) {
    std::vector<int> cand;
    for (int div : {2, 3, 4, 5, 6, 8}) {
        const int G = std::max(8, c0.pm_grid / div);
        if (std::find(cand.begin(), cand.end(), G) == cand.end()) cand.push_back(G);
    }
    const uint32_t n = (uint32_t)c0.n;
    std::vector<float> pos(3 * (size_t)n);
    uint64_t s = 0x9E3779B97F4A7C15ull ^ (uint64_t)n;
    for (auto &x : pos) {  // seeded uniform positions (xorshift)
        s ^= s << 13, s ^= s >> 7, s ^= s << 17;
        x = (float)((double)(s >> 11) * (1.0 / 9007199254740992.0) * c0.boxsize);
        if (x >= c0.boxsize) x = 0.f;
    }
    int best = -1;
    float best_ms = 1e30f;
    for (int G : cand) {
        cuco_config_t c = c0;
        c.cell_grid = G;
        cuco_box_t *b = nullptr;
        if (cuco_box_create(&c, &b) != CUCO_OK) continue;
        float ms = 1e30f;
        if (cuco_box_set_state(b, pos.data(), nullptr, 0) == CUCO_OK && cuco_box_enable_timing(b, 1) == CUCO_OK) {
            bool ok = cuco_box_forces(b, 0, 1) == CUCO_OK;  // warm-up
            for (int r = 0; ok && r < 2; ++r) {
                float t[8];
                ok = cuco_box_forces(b, 0, 1) == CUCO_OK && cuco_box_timings(b, t) == CUCO_OK;
                if (ok) ms = std::min(ms, t[6]);
            }
        }
        cuco_box_destroy(b);
        if (ms < best_ms) best_ms = ms, best = G;
    }
    (void)stream;
    return best;
}

// FFT batching (columns per CTA) by timing one-box multi launches.
void tune_fft(int M, float boxsize, float asmth, cudaStream_t stream, int *P_out, int *B_out) {
    *P_out = pm_batch_z(M);
    *B_out = pm_batch_axis(M);
    const size_t Mh = M / 2 + 1;
    float *rho = nullptr, *green = nullptr;
    unsigned long long *rho64 = nullptr;
    float2 *spec = nullptr, *tw = nullptr;
    PMBoxDesc *dd = nullptr;
    uint32_t *pbeg = nullptr;
    uint2 *mz = nullptr, *ma = nullptr;
    bool ok = dalloc(&rho, (size_t)M * M * M) == CUCO_OK && dalloc(&rho64, (size_t)M * M * M) == CUCO_OK &&
              dalloc(&spec, (size_t)M * M * Mh) == CUCO_OK &&
              dalloc(&green, Mh) == CUCO_OK && dalloc(&tw, (size_t)M) == CUCO_OK && dalloc(&dd, 1) == CUCO_OK &&
              dalloc(&pbeg, 2) == CUCO_OK && dalloc(&mz, (size_t)M * M) == CUCO_OK &&
              dalloc(&ma, (size_t)M * Mh) == CUCO_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ok) {
        std::vector<float> g(Mh);
        std::vector<float2> t(M);
        pm_tables(M, boxsize, asmth, g.data(), t.data());
        cudaMemcpy(green, g.data(), sizeof(float) * Mh, cudaMemcpyHostToDevice);
        cudaMemcpy(tw, t.data(), sizeof(float2) * M, cudaMemcpyHostToDevice);
        cudaMemset(rho, 0, sizeof(float) * (size_t)M * M * M);
        const uint32_t pb[2] = {0, 0};
        cudaMemcpy(pbeg, pb, sizeof pb, cudaMemcpyHostToDevice);
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best = 1e30f;
        for (int P : {1, 2, 4, 8, 16}) {
            if (P > M / 2 || (M * M / 2) % P || pm_smem_z(M, P) > 200 * 1024) continue;
            for (int B : {4, 8, 16}) {
                if (pm_smem_axis(M, B) > 200 * 1024 || !pm_fft_batches_ok(M, P, B)) continue;
                PMBoxDesc d{M, P, B, 1.f, 0.f, 0.f, rho, rho64, 1.f, spec, green, tw};
                cudaMemcpy(dd, &d, sizeof d, cudaMemcpyHostToDevice);
                const uint32_t nz = (uint32_t)(M * M / (2 * P)), nbx = (uint32_t)((Mh + B - 1) / B),
                               na = nbx * M;
                std::vector<uint2> vz(nz), va(na);
                for (uint32_t k = 0; k < nz; ++k) vz[k] = make_uint2(0, k);
                for (uint32_t k = 0; k < na; ++k) va[k] = make_uint2(0, k);
                cudaMemcpy(mz, vz.data(), sizeof(uint2) * nz, cudaMemcpyHostToDevice);
                cudaMemcpy(ma, va.data(), sizeof(uint2) * na, cudaMemcpyHostToDevice);
                PMMulti m{1, false, dd, pbeg, mz, ma, nz, na, pm_smem_z(M, P), pm_smem_axis(M, B), rho64,
                          (size_t)M * M * M};
                m.big = pm_big_fft(M, P, B);
                if (pm_forces_multi(m, nullptr, 0, nullptr, stream, nullptr) != CUCO_OK) continue;  // warm-up
                cudaEventRecord(e0, stream);
                for (int r = 0; r < 3; ++r) pm_forces_multi(m, nullptr, 0, nullptr, stream, nullptr);
                cudaEventRecord(e1, stream);
                if (cudaEventSynchronize(e1) != cudaSuccess) continue;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best) best = ms, *P_out = P, *B_out = B;
            }
        }
    }
    cudaGetLastError();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(rho), cudaFree(rho64), cudaFree(spec), cudaFree(green), cudaFree(tw), cudaFree(dd), cudaFree(pbeg), cudaFree(mz),
        cudaFree(ma);
}

}  // namespace
}  // namespace cuco

using namespace cuco;

struct cuco_ensemble {
    int nbox = 0;
    int device = 0;
    bool fixed = false;
    cudaStream_t stream = nullptr;
    std::vector<cuco_config_t> cfg;
    std::vector<uint32_t> pbeg;  // host copy, nbox+1
    std::vector<int> P, B;
    uint32_t n = 0;
    uint64_t ncells = 0;
    int key_bits = 0;
    // particles, concatenated
    float4 *pos = nullptr, *vel = nullptr, *acc_pp = nullptr, *acc_pm = nullptr, *spos = nullptr,
           *acc_pm_s = nullptr;
    uint32_t *keys = nullptr, *perm = nullptr, *keys_alt = nullptr, *perm_alt = nullptr, *hist = nullptr,
             *hist2 = nullptr,
             *cell_off = nullptr, *sorted_perm = nullptr;
    uint4 *cell_sl = nullptr;  // per cell: z-slice counts
    float *stage3 = nullptr;
    // meshes, concatenated
    float *rho = nullptr, *green = nullptr, *table = nullptr;
    unsigned long long *rho64 = nullptr;
    float2 *spec = nullptr, *tw = nullptr;
    // descriptors
    uint32_t *d_pbeg = nullptr, *d_segbase = nullptr;
    DriftBox *d_drift = nullptr;
    PMBoxDesc *d_pm = nullptr;
    uint2 *d_mapz = nullptr, *d_mapa = nullptr;
    char *d_sr = nullptr;
    double2 *d_kicks = nullptr;
    StepFactors *d_factors = nullptr;
    // per-step factors in pinned host memory, two slots used in turn: a step
    // fills one slot while the copy from the other may still be queued, and
    // waits only for the copy of two steps back (up_done), so the host
    // prepares step t+1 while the GPU runs step t
    StepFactors *h_factors[2] = {nullptr, nullptr};
    double2 *h_kicks[2] = {nullptr, nullptr};
    cudaEvent_t up_done[2] = {nullptr, nullptr};
    bool up_pending[2] = {false, false};
    int slot = 0;
    PMMulti pm{};
    uint32_t segments = 0;
    size_t sr_smem = 0;
    // box 0's short-range descriptor (host copy) when every box has its pair
    // law, so the launch reads the law from its parameters
    std::vector<char> sr_law;
    unsigned long long *pair_counter = nullptr;
    bool count_pairs = false;
    bool has_state = false;
    int launches = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    // the PM's stream beside the sort (forked after the keys, joined before
    // the short range; both branches are captured into the step's graph)
    cudaStream_t pm_stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    // capacities (elements) of the grow-only arrays
    size_t cap_n = 0, cap_hist = 0, cap_hist2 = 0, cap_cells = 0, cap_stage3 = 0, cap_mesh = 0, cap_mesh64 = 0, cap_spec = 0,
           cap_green = 0, cap_tw = 0, cap_table = 0, cap_pbeg = 0, cap_segbase = 0, cap_drift = 0, cap_pm = 0,
           cap_kicks = 0, cap_factors = 0, cap_counter = 0, cap_sr = 0, cap_hfactors[2] = {0, 0},
           cap_hkicks[2] = {0, 0},
           cap_mapz = 0, cap_mapa = 0, cap_heavy = 0, cap_segnt = 0, cap_ctl = 0, cap_cellsl = 0;
    // the short range's work-plan scratch
    uint2 *sr_heavy = nullptr;
    uint32_t *sr_segnt = nullptr, *sr_ctl = nullptr;
};

namespace {

// One force pass (and kicks when kick != 0), enqueued on e->stream.
cuco_status_t ensemble_pass(cuco_ensemble *e, int do_drift, bool kick) {
    e->launches = 0;
    if (e->n) {
        k_drift_keys_multi<<<(e->n + 255) / 256, 256, 0, e->stream>>>(e->pos, e->vel, e->keys, e->n, e->d_pbeg,
                                                                     e->nbox, e->d_drift, e->d_factors, do_drift,
                                                                     e->fixed ? 1 : 0);
        CUCO_TRY_CUDA(cudaGetLastError());
        e->launches++;
    }
    // The PM reads the positions and writes its accelerations in original
    // order (order-independent results), beside the sort and the cell order.
    CUCO_TRY_CUDA(cudaEventRecord(e->fork, e->stream));
    CUCO_TRY_CUDA(cudaStreamWaitEvent(e->pm_stream, e->fork, 0));
    CUCO_TRY(pm_forces_multi(e->pm, e->pos, e->n, e->acc_pm, e->pm_stream, &e->launches));
    CUCO_TRY_CUDA(cudaEventRecord(e->join, e->pm_stream));
    bool in_alt = false;
    CUCO_TRY(sort_pairs(e->keys, e->perm, nullptr, e->keys_alt, e->perm_alt, e->hist, e->n, e->key_bits, 8,
                        e->stream, &in_alt, &e->launches, e->hist2));
    const uint32_t *skeys = in_alt ? e->keys_alt : e->keys;
    e->sorted_perm = in_alt ? e->perm_alt : e->perm;
    CUCO_TRY(launch_reorder_offsets(e->cell_off, nullptr, skeys, e->sorted_perm, e->pos, e->n, (uint32_t)e->ncells,
                                    e->stream));
    // cells refined by z slice, as for one box; the map to original indices
    // goes to the sort's spare buffer
    uint32_t *perm_s = in_alt ? e->perm : e->perm_alt;
    CUCO_TRY(launch_cell_subsort(e->cell_off, e->sorted_perm, e->pos, e->spos, perm_s, e->cell_sl,
                                 (uint32_t)e->ncells, CellBox{}, e->d_drift, e->nbox, e->fixed, e->stream));
    e->launches += 2;
    CUCO_TRY_CUDA(cudaStreamWaitEvent(e->stream, e->join, 0));
    KickArgs k{};
    k.vel = kick ? e->vel : nullptr;
    k.acc_pm_o = e->acc_pm;
    SRWork w{e->sr_heavy, (uint32_t)e->cap_heavy, e->sr_segnt, (uint32_t)e->cap_segnt, e->sr_ctl};
    CUCO_TRY(launch_shortrange_multi(e->d_sr, e->d_kicks, e->d_segbase, e->nbox, e->segments, e->sr_smem, e->fixed,
                                     e->spos, perm_s, e->cell_off, e->table, e->acc_pp, k, w, e->stream,
                                     e->count_pairs ? e->pair_counter : nullptr,
                                     e->sr_law.empty() ? nullptr : e->sr_law.data()));
    e->launches += 2;  // work plan + persistent short range
    return CUCO_OK;
}

// The factors of slot k to the device, stream-ordered before the step that
// reads them; up_done[k] marks when slot k may be written again.
cuco_status_t upload_factors(cuco_ensemble *e, int k) {
    CUCO_TRY_CUDA(cudaMemcpyAsync(e->d_factors, e->h_factors[k], sizeof(StepFactors) * e->nbox,
                                  cudaMemcpyHostToDevice, e->stream));
    CUCO_TRY_CUDA(cudaMemcpyAsync(e->d_kicks, e->h_kicks[k], sizeof(double2) * e->nbox, cudaMemcpyHostToDevice,
                                  e->stream));
    CUCO_TRY_CUDA(cudaEventRecord(e->up_done[k], e->stream));
    e->up_pending[k] = true;
    return CUCO_OK;
}

void drop_graph(cuco_ensemble *e) {
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    e->exec = nullptr;
    e->graph = nullptr;
}

cuco_status_t validate_boxes(const cuco_config_t *boxes, int nbox, int mode, int device) {
    for (int b = 0; b < nbox; ++b) {
        const cuco_config_t &c = boxes[b];
        if ((int)c.mode != mode || c.device != device) {
            set_error("ensemble: all boxes share one mode and one device");
            return CUCO_ERR_INVALID;
        }
        if (c.n < 0 || !(c.boxsize > 0) || !(c.rcut > 0) || !(c.asmth > 0) || !(c.softening > 0) ||
            c.cell_grid < 0 || c.cell_grid > 1024) {
            set_error("ensemble: invalid box configuration");
            return CUCO_ERR_INVALID;
        }
        if (!pm_mesh_supported(c.pm_grid)) {
            set_error("ensemble: a mesh is not even, in [8, 1024] and 5-smooth");
            return CUCO_ERR_UNSUPPORTED;
        }
    }
    return CUCO_OK;
}

// Device array that only grows (25% headroom), reallocated without keeping
// its contents; the stream-ordered pool makes the reallocation cheap.
template <typename T>
cuco_status_t grow(T *&p, size_t &cap, size_t need, cudaStream_t s) {
    if (p && need <= cap) return CUCO_OK;
    const size_t ncap = std::max(need ? need : 1, cap + cap / 4);
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    cap = 0;
    CUCO_TRY(palloc(&p, ncap, s));
    cap = ncap;
    return CUCO_OK;
}

template <typename T>
cuco_status_t grow_pinned(T *&p, size_t &cap, size_t need) {
    if (p && need <= cap) return CUCO_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    if (cudaMallocHost(&p, sizeof(T) * need) != cudaSuccess) {
        set_error("ensemble: pinned allocation failed");
        return CUCO_ERR_NOMEM;
    }
    memset(p, 0, sizeof(T) * need);
    cap = need;
    return CUCO_OK;
}

// (Re)build the ensemble for a set of boxes: autotuned plans, offsets, array
// capacities, descriptors and CTA maps.  carry[b] = the box of the previous
// layout whose positions and velocities box b keeps (-1: set by the caller
// afterwards); null when there is no previous layout to keep.
cuco_status_t ensemble_layout(cuco_ensemble *e, const cuco_config_t *boxes, int nbox, const int *carry) {
    cudaStream_t st = e->stream;
    drop_graph(e);
    std::vector<cuco_config_t> cfg(boxes, boxes + nbox);
    std::vector<int> P(nbox), B(nbox);
    // autotune: cell grid and FFT batching per (n, M, mode)
    for (int b = 0; b < nbox; ++b) {
        cuco_config_t &c = cfg[b];
        const auto key = std::make_tuple(c.n, c.pm_grid, (int)c.mode);
        Tuned t{};
        bool cached;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune_cache.find(key);
            cached = it != g_tune_cache.end();
            if (cached) t = it->second;
        }
        if (!cached) {
            t.cell_grid = tune_cell_grid(c, st);
            tune_fft(c.pm_grid, c.boxsize, c.asmth, st, &t.P, &t.B);
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tune_cache[key] = t;
        }
        if (c.cell_grid <= 0) {
            if (t.cell_grid <= 0) {
                set_error("ensemble: no admissible cell grid for a box");
                return CUCO_ERR_UNSUPPORTED;
            }
            c.cell_grid = t.cell_grid;
        }
        P[b] = t.P;
        B[b] = t.B;
    }
    // sizes and offsets
    std::vector<uint32_t> pbeg(nbox + 1, 0);
    std::vector<uint64_t> cbase(nbox + 1, 0), mbase(nbox + 1, 0), sbase(nbox + 1, 0), gbase(nbox + 1, 0),
        tbase(nbox + 1, 0);
    size_t maxn = 0;
    for (int b = 0; b < nbox; ++b) {
        const cuco_config_t &c = cfg[b];
        const uint64_t M = c.pm_grid, G = c.cell_grid;
        pbeg[b + 1] = pbeg[b] + (uint32_t)c.n;
        cbase[b + 1] = cbase[b] + G * G * G;
        mbase[b + 1] = mbase[b] + M * M * M;
        sbase[b + 1] = sbase[b] + M * M * (M / 2 + 1);
        gbase[b + 1] = gbase[b] + (M / 2 + 1);
        tbase[b + 1] = tbase[b] + M;
        maxn = std::max(maxn, (size_t)c.n);
    }
    if (cbase[nbox] >= 0xffffffffull || (uint64_t)pbeg[nbox] > 0xfffffff0ull) {
        set_error("ensemble: more than 2^32 cells or particles in total");
        return CUCO_ERR_UNSUPPORTED;
    }
    const size_t n = pbeg[nbox];
    const uint64_t ncells = cbase[nbox];
    const int kbits = key_bits(ncells);
    cuco_status_t s;
    // particle state: carried boxes move to their new offsets device to device
    if (carry && e->pos) {
        if (n > e->cap_n) {
            float4 *pos2 = nullptr, *vel2 = nullptr;
            const size_t ncap = std::max(n, e->cap_n + e->cap_n / 4);
            if ((s = palloc(&pos2, ncap, st)) || (s = palloc(&vel2, ncap, st))) {
                if (pos2) cudaFreeAsync(pos2, st);
                return s;
            }
            for (int b = 0; b < nbox; ++b)
                if (carry[b] >= 0) {
                    const size_t nb = cfg[b].n, o = e->pbeg[carry[b]];
                    CUCO_TRY_CUDA(cudaMemcpyAsync(pos2 + pbeg[b], e->pos + o, sizeof(float4) * nb,
                                                  cudaMemcpyDeviceToDevice, st));
                    CUCO_TRY_CUDA(cudaMemcpyAsync(vel2 + pbeg[b], e->vel + o, sizeof(float4) * nb,
                                                  cudaMemcpyDeviceToDevice, st));
                }
            cudaFreeAsync(e->pos, st);
            cudaFreeAsync(e->vel, st);
            e->pos = pos2;
            e->vel = vel2;
            size_t cap = e->cap_n;  // the other per-particle arrays follow
            for (float4 **q : {&e->acc_pp, &e->acc_pm, &e->spos, &e->acc_pm_s}) {
                size_t c2 = cap;
                CUCO_TRY(grow(*q, c2, ncap, st));
            }
            for (uint32_t **q : {&e->keys, &e->perm, &e->keys_alt, &e->perm_alt}) {
                size_t c2 = cap;
                CUCO_TRY(grow(*q, c2, ncap, st));
            }
            e->cap_n = ncap;
        } else {
            // through the sorted-copy arrays (scratch between steps), then swap
            for (int b = 0; b < nbox; ++b)
                if (carry[b] >= 0) {
                    const size_t nb = cfg[b].n, o = e->pbeg[carry[b]];
                    CUCO_TRY_CUDA(cudaMemcpyAsync(e->spos + pbeg[b], e->pos + o, sizeof(float4) * nb,
                                                  cudaMemcpyDeviceToDevice, st));
                    CUCO_TRY_CUDA(cudaMemcpyAsync(e->acc_pm_s + pbeg[b], e->vel + o, sizeof(float4) * nb,
                                                  cudaMemcpyDeviceToDevice, st));
                }
            std::swap(e->pos, e->spos);
            std::swap(e->vel, e->acc_pm_s);
        }
    } else if (n > e->cap_n || !e->pos) {
        const size_t ncap = std::max(n ? n : 1, e->cap_n + e->cap_n / 4);
        for (float4 **q : {&e->pos, &e->vel, &e->acc_pp, &e->acc_pm, &e->spos, &e->acc_pm_s}) {
            size_t c2 = e->cap_n;
            CUCO_TRY(grow(*q, c2, ncap, st));
        }
        for (uint32_t **q : {&e->keys, &e->perm, &e->keys_alt, &e->perm_alt}) {
            size_t c2 = e->cap_n;
            CUCO_TRY(grow(*q, c2, ncap, st));
        }
        e->cap_n = ncap;
        CUCO_TRY_CUDA(cudaMemsetAsync(e->pos, 0, sizeof(float4) * ncap, st));
        CUCO_TRY_CUDA(cudaMemsetAsync(e->vel, 0, sizeof(float4) * ncap, st));
    }
    const size_t nbc = (size_t)nbox + 1;
    if ((s = grow(e->hist, e->cap_hist, sort_hist_entries((uint32_t)n, kbits, 8), st)) ||
        (s = grow(e->hist2, e->cap_hist2, sort_hist_entries((uint32_t)n, kbits, 8), st)) ||
        (s = grow(e->cell_off, e->cap_cells, ncells + 1, st)) || (s = grow(e->cell_sl, e->cap_cellsl, ncells, st)) || (s = grow(e->stage3, e->cap_stage3, 3 * maxn, st)) ||
        (s = grow(e->rho, e->cap_mesh, mbase[nbox], st)) ||
        (s = grow(e->rho64, e->cap_mesh64, mbase[nbox], st)) || (s = grow(e->spec, e->cap_spec, sbase[nbox], st)) ||
        (s = grow(e->green, e->cap_green, gbase[nbox], st)) || (s = grow(e->tw, e->cap_tw, tbase[nbox], st)) ||
        (s = grow(e->table, e->cap_table, (size_t)kNTab, st)) || (s = grow(e->d_pbeg, e->cap_pbeg, nbc, st)) ||
        (s = grow(e->d_segbase, e->cap_segbase, nbc, st)) || (s = grow(e->d_drift, e->cap_drift, nbc, st)) ||
        (s = grow(e->d_pm, e->cap_pm, nbc, st)) || (s = grow(e->d_kicks, e->cap_kicks, nbc, st)) ||
        (s = grow(e->d_factors, e->cap_factors, nbc, st)) || (s = grow(e->pair_counter, e->cap_counter, 1, st)) ||
        (s = grow(e->d_sr, e->cap_sr, shortrange_desc_bytes() * nbc, st)) ||
        (s = grow_pinned(e->h_factors[0], e->cap_hfactors[0], nbc)) ||
        (s = grow_pinned(e->h_kicks[0], e->cap_hkicks[0], nbc)) ||
        (s = grow_pinned(e->h_factors[1], e->cap_hfactors[1], nbc)) ||
        (s = grow_pinned(e->h_kicks[1], e->cap_hkicks[1], nbc)))
        return s;
    // tables and descriptors
    std::vector<float> tab(kNTab);
    shortrange_table(tab.data());
    std::vector<DriftBox> drift(nbox);
    std::vector<PMBoxDesc> pmd(nbox);
    std::vector<char> srd(shortrange_desc_bytes() * nbox);
    std::vector<uint32_t> segbase(nbox + 1, 0);
    std::vector<uint2> mapz, mapa;
    std::vector<float> green(gbase[nbox]);
    std::vector<float2> tw(tbase[nbox]);
    size_t smz = 0, sma = 0, sr_smem = 0;
    for (int b = 0; b < nbox; ++b) {
        const cuco_config_t &c = cfg[b];
        const int M = c.pm_grid, Mh = M / 2 + 1;
        drift[b] = DriftBox{(uint32_t)c.cell_grid, (uint32_t)cbase[b], c.boxsize, (float)c.cell_grid / c.boxsize};
        pm_tables(M, c.boxsize, c.asmth, green.data() + gbase[b], tw.data() + tbase[b]);
        pmd[b] = PMBoxDesc{M, P[b], B[b], (float)M / c.boxsize, c.mass, pm_fd_fac(M, c.boxsize, c.G),
                           e->rho + mbase[b], e->rho64 + mbase[b], ldexpf(c.mass, -32), e->spec + sbase[b],
                           e->green + gbase[b], e->tw + tbase[b]};
        const uint32_t nz = (uint32_t)(M * M / (2 * P[b]));
        for (uint32_t k = 0; k < nz; ++k) mapz.push_back(make_uint2(b, k));
        const uint32_t na = (uint32_t)((Mh + B[b] - 1) / B[b]) * M;
        for (uint32_t k = 0; k < na; ++k) mapa.push_back(make_uint2(b, k));
        smz = std::max(smz, pm_smem_z(M, P[b]));
        sma = std::max(sma, pm_smem_axis(M, B[b]));
        uint32_t nseg = 0;
        size_t sm = 0;
        if ((s = shortrange_desc_fill(sr_params(c, (uint32_t)c.n, (uint32_t)cbase[b], e->cell_sl),
                                      srd.data() + b * shortrange_desc_bytes(), &nseg, &sm)))
            return s;
        segbase[b + 1] = segbase[b] + nseg;
        sr_smem = std::max(sr_smem, sm);
    }
    if ((s = grow(e->d_mapz, e->cap_mapz, mapz.size(), st)) || (s = grow(e->d_mapa, e->cap_mapa, mapa.size(), st)) ||
        (s = grow(e->sr_heavy, e->cap_heavy, (size_t)shortrange_heavy_cap((uint32_t)n) + 16u * nbox, st)) ||
        (s = grow(e->sr_segnt, e->cap_segnt, (size_t)segbase[nbox], st)) || (s = grow(e->sr_ctl, e->cap_ctl, kSRCtlWords, st)))
        return s;
    if (cudaStreamSynchronize(st) != cudaSuccess ||
        cudaMemcpy(e->table, tab.data(), sizeof(float) * kNTab, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->green, green.data(), sizeof(float) * green.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->tw, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->d_pbeg, pbeg.data(), sizeof(uint32_t) * (nbox + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->d_segbase, segbase.data(), sizeof(uint32_t) * (nbox + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->d_drift, drift.data(), sizeof(DriftBox) * nbox, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->d_pm, pmd.data(), sizeof(PMBoxDesc) * nbox, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->d_sr, srd.data(), srd.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->d_mapz, mapz.data(), sizeof(uint2) * mapz.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->d_mapa, mapa.data(), sizeof(uint2) * mapa.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(e->pair_counter, 0, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(e->sr_ctl, 0, sizeof(uint32_t) * kSRCtlWords) != cudaSuccess) {
        set_error("ensemble: descriptor upload failed");
        return CUCO_ERR_CUDA;
    }
    for (int k = 0; k < 2; ++k) {
        memset(e->h_factors[k], 0, sizeof(StepFactors) * nbox);
        memset(e->h_kicks[k], 0, sizeof(double2) * nbox);
    }
    e->nbox = nbox;
    e->cfg = cfg;
    e->P = P;
    e->B = B;
    e->pbeg = pbeg;
    e->n = (uint32_t)n;
    e->ncells = ncells;
    e->key_bits = kbits;
    e->segments = segbase[nbox];
    e->sr_smem = sr_smem;
    e->sr_law.clear();
    if (shortrange_descs_uniform_law(srd.data(), nbox))
        e->sr_law.assign(srd.begin(), srd.begin() + shortrange_desc_bytes());
    e->pm = PMMulti{nbox, e->fixed, e->d_pm, e->d_pbeg, e->d_mapz, e->d_mapa, (uint32_t)mapz.size(),
                    (uint32_t)mapa.size(), smz, sma, e->rho64, (size_t)mbase[nbox]};
    for (int b = 0; b < nbox; ++b) e->pm.big = e->pm.big || pm_big_fft(cfg[b].pm_grid, P[b], B[b]);
    e->has_state = e->has_state || carry != nullptr;
    return CUCO_OK;
}

}  // namespace

extern "C" {

cuco_status_t cuco_ensemble_create(const cuco_config_t *boxes, int nbox, cuco_ensemble_t **out) {
    if (!boxes || nbox <= 0 || !out) {
        set_error("cuco_ensemble_create: need at least one box");
        return CUCO_ERR_INVALID;
    }
    CUCO_TRY(validate_boxes(boxes, nbox, boxes[0].mode, boxes[0].device));
    CUCO_TRY_CUDA(cudaSetDevice(boxes[0].device));
    cuco_ensemble *e = new cuco_ensemble();
    e->device = boxes[0].device;
    e->fixed = boxes[0].mode == CUCO_MODE_FIXED;
    // the sort's stream first, the PM's on the SMs it leaves (as for one box)
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithPriority(&e->stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        delete e;
        return CUCO_ERR_CUDA;
    }
    if (cudaStreamCreateWithPriority(&e->pm_stream, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->join, cudaEventDisableTiming) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        cuco_ensemble_destroy(e);
        return CUCO_ERR_CUDA;
    }
    cudaEventCreate(&e->t0);
    cudaEventCreate(&e->t1);
    for (int k = 0; k < 2; ++k)
        if (cudaEventCreateWithFlags(&e->up_done[k], cudaEventDisableTiming) != cudaSuccess) {
            set_error("cudaEventCreate failed");
            cuco_ensemble_destroy(e);
            return CUCO_ERR_CUDA;
        }
    pool_keep_memory(e->device);
    cuco_status_t s = ensemble_layout(e, boxes, nbox, nullptr);
    if (s != CUCO_OK) {
        cuco_ensemble_destroy(e);
        return s;
    }
    *out = e;
    return CUCO_OK;
}

cuco_status_t cuco_ensemble_reshape(cuco_ensemble_t *e, const cuco_config_t *boxes, int nbox, const int *carry) {
    if (!e || !boxes || nbox <= 0) {
        set_error("cuco_ensemble_reshape: need at least one box");
        return CUCO_ERR_INVALID;
    }
    CUCO_TRY(validate_boxes(boxes, nbox, e->fixed ? CUCO_MODE_FIXED : CUCO_MODE_PLAIN, e->device));
    if (carry)
        for (int b = 0; b < nbox; ++b) {
            const int o = carry[b];
            if (o < -1 || o >= e->nbox || (o >= 0 && (e->cfg[o].n != boxes[b].n ||
                                                      e->cfg[o].boxsize != boxes[b].boxsize))) {
                set_error("cuco_ensemble_reshape: a carried box differs in size or box length");
                return CUCO_ERR_INVALID;
            }
        }
    CUCO_TRY_CUDA(cudaSetDevice(e->device));
    CUCO_TRY_CUDA(cudaStreamSynchronize(e->stream));
    return ensemble_layout(e, boxes, nbox, carry);
}

cuco_status_t cuco_ensemble_destroy(cuco_ensemble_t *e) {
    if (!e) return CUCO_OK;
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->pm_stream) cudaStreamSynchronize(e->pm_stream);  // a pass that stopped before its join
    drop_graph(e);
    for (void *p : {(void *)e->pos, (void *)e->vel, (void *)e->acc_pp, (void *)e->acc_pm, (void *)e->spos,
                    (void *)e->acc_pm_s, (void *)e->keys, (void *)e->perm, (void *)e->keys_alt, (void *)e->perm_alt,
                    (void *)e->hist, (void *)e->hist2, (void *)e->cell_off, (void *)e->cell_sl, (void *)e->stage3, (void *)e->rho, (void *)e->rho64,
                    (void *)e->spec,
                    (void *)e->green, (void *)e->tw, (void *)e->table, (void *)e->d_pbeg, (void *)e->d_segbase,
                    (void *)e->d_drift, (void *)e->d_pm, (void *)e->d_mapz, (void *)e->d_mapa, (void *)e->d_sr,
                    (void *)e->d_kicks, (void *)e->d_factors, (void *)e->pair_counter, (void *)e->sr_heavy,
                    (void *)e->sr_segnt, (void *)e->sr_ctl})
        if (p && e->stream) cudaFreeAsync(p, e->stream);
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (int k = 0; k < 2; ++k) {
        if (e->h_factors[k]) cudaFreeHost(e->h_factors[k]);
        if (e->h_kicks[k]) cudaFreeHost(e->h_kicks[k]);
        if (e->up_done[k]) cudaEventDestroy(e->up_done[k]);
    }
    if (e->t0) cudaEventDestroy(e->t0);
    if (e->t1) cudaEventDestroy(e->t1);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->join) cudaEventDestroy(e->join);
    if (e->pm_stream) cudaStreamDestroy(e->pm_stream);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return CUCO_OK;
}

cuco_status_t cuco_ensemble_cell_grid(cuco_ensemble_t *e, int box, int *cell_grid, int *fft_p, int *fft_b) {
    if (!e || box < 0 || box >= e->nbox) {
        set_error("cuco_ensemble_cell_grid: no such box");
        return CUCO_ERR_INVALID;
    }
    if (cell_grid) *cell_grid = e->cfg[box].cell_grid;
    if (fft_p) *fft_p = e->P[box];
    if (fft_b) *fft_b = e->B[box];
    return CUCO_OK;
}

cuco_status_t cuco_ensemble_set_state(cuco_ensemble_t *e, int box, const float *pos, const float *vel) {
    if (!e || box < 0 || box >= e->nbox || !pos) {
        set_error("cuco_ensemble_set_state: invalid argument");
        return CUCO_ERR_INVALID;
    }
    const uint32_t b0 = e->pbeg[box], nb = e->pbeg[box + 1] - b0;
    const size_t bytes = sizeof(float) * 3 * nb;
    CUCO_TRY_CUDA(cudaMemcpyAsync(e->stage3, pos, bytes, cudaMemcpyHostToDevice, e->stream));
    if (e->fixed)
        CUCO_TRY(to_fixed(e->stage3, e->pos + b0, nb, e->cfg[box].boxsize, e->stream));
    else
        CUCO_TRY(pack3to4(e->stage3, e->pos + b0, nb, e->stream));
    if (vel) {
        CUCO_TRY_CUDA(cudaMemcpyAsync(e->stage3, vel, bytes, cudaMemcpyHostToDevice, e->stream));
        CUCO_TRY(pack3to4(e->stage3, e->vel + b0, nb, e->stream));
    }
    CUCO_TRY_CUDA(cudaStreamSynchronize(e->stream));
    e->has_state = true;
    return CUCO_OK;
}

cuco_status_t cuco_ensemble_get_state(cuco_ensemble_t *e, int box, float *pos, float *vel, float *acc_pp,
                                      float *acc_pm) {
    if (!e || box < 0 || box >= e->nbox) {
        set_error("cuco_ensemble_get_state: invalid argument");
        return CUCO_ERR_INVALID;
    }
    const uint32_t b0 = e->pbeg[box], nb = e->pbeg[box + 1] - b0;
    float *dst[4] = {pos, vel, acc_pp, acc_pm};
    float4 *src[4] = {e->pos, e->vel, e->acc_pp, e->acc_pm};
    for (int k = 0; k < 4; ++k) {
        if (!dst[k]) continue;
        if (k == 0 && e->fixed)
            CUCO_TRY(from_fixed(src[k] + b0, e->stage3, nb, e->cfg[box].boxsize, e->stream));
        else
            CUCO_TRY(unpack4to3(src[k] + b0, e->stage3, nb, e->stream));
        CUCO_TRY_CUDA(cudaMemcpyAsync(dst[k], e->stage3, sizeof(float) * 3 * nb, cudaMemcpyDeviceToHost, e->stream));
        CUCO_TRY_CUDA(cudaStreamSynchronize(e->stream));
    }
    return CUCO_OK;
}

cuco_status_t cuco_ensemble_forces(cuco_ensemble_t *e) {
    if (!e || !e->has_state) {
        set_error("cuco_ensemble_forces: no state uploaded");
        return CUCO_ERR_STATE;
    }
    CUCO_TRY(ensemble_pass(e, 0, false));
    CUCO_TRY_CUDA(cudaStreamSynchronize(e->stream));
    return CUCO_OK;
}

cuco_status_t cuco_ensemble_step(cuco_ensemble_t *e, const double *drift, const double *kick_pp,
                                 const double *kick_pm) {
    if (!e || !e->has_state || !drift || !kick_pp || !kick_pm) {
        set_error("cuco_ensemble_step: no state uploaded or null factors");
        return CUCO_ERR_STATE;
    }
    // slot k was last copied two steps ago: wait for that copy only, not for
    // the steps in flight
    const int k = e->slot;
    if (e->up_pending[k]) {
        CUCO_TRY_CUDA(cudaEventSynchronize(e->up_done[k]));
        e->up_pending[k] = false;
    }
    for (int b = 0; b < e->nbox; ++b) {
        const double L = e->cfg[b].boxsize;
        e->h_factors[k][b].units_per_time = (float)(e->fixed ? drift[b] * 4294967296.0 / L : drift[b]);
        e->h_kicks[k][b] = make_double2(kick_pp[b], kick_pm[b]);
    }
    e->slot ^= 1;
    CUCO_TRY(upload_factors(e, k));
    if (!e->exec) {
        // first step: run once outside capture (one-time kernel attributes),
        // then capture the step (without the factor upload, which precedes
        // every launch) as a graph for the following ones
        CUCO_TRY(ensemble_pass(e, 1, true));
        CUCO_TRY_CUDA(cudaStreamSynchronize(e->stream));
        CUCO_TRY_CUDA(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        cuco_status_t s2 = ensemble_pass(e, 1, true);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        if (s2 != CUCO_OK) {
            if (g) cudaGraphDestroy(g);
            return s2;
        }
        CUCO_TRY_CUDA(ce);
        e->graph = g;
        CUCO_TRY_CUDA(cudaGraphInstantiate(&e->exec, e->graph, 0));
        return CUCO_OK;
    }
    CUCO_TRY_CUDA(cudaGraphLaunch(e->exec, e->stream));
    return CUCO_OK;
}

cuco_status_t cuco_ensemble_sync(cuco_ensemble_t *e) {
    if (!e) return CUCO_ERR_INVALID;
    CUCO_TRY_CUDA(cudaStreamSynchronize(e->stream));
    return e->sr_ctl ? shortrange_check(e->sr_ctl, e->stream) : CUCO_OK;
}

cuco_status_t cuco_ensemble_timer(cuco_ensemble_t *e, int op, float *ms) {
    if (!e) return CUCO_ERR_INVALID;
    if (op == 0) {
        CUCO_TRY_CUDA(cudaEventRecord(e->t0, e->stream));
    } else {
        CUCO_TRY_CUDA(cudaEventRecord(e->t1, e->stream));
        CUCO_TRY_CUDA(cudaEventSynchronize(e->t1));
        CUCO_TRY_CUDA(cudaEventElapsedTime(ms, e->t0, e->t1));
    }
    return CUCO_OK;
}

cuco_status_t cuco_ensemble_count_pairs(cuco_ensemble_t *e, int enable, uint64_t *pairs) {
    if (!e) return CUCO_ERR_INVALID;
    CUCO_TRY_CUDA(cudaStreamSynchronize(e->stream));
    if (pairs) CUCO_TRY_CUDA(cudaMemcpy(pairs, e->pair_counter, sizeof(uint64_t), cudaMemcpyDeviceToHost));
    CUCO_TRY_CUDA(cudaMemset(e->pair_counter, 0, sizeof(unsigned long long)));
    if ((bool)enable != e->count_pairs) drop_graph(e);  // the captured launch differs
    e->count_pairs = enable != 0;
    return CUCO_OK;
}

int cuco_ensemble_launches_per_step(cuco_ensemble_t *e) { return e ? e->launches : 0; }

cuco_status_t cuco_ensemble_copy_state(cuco_ensemble_t *dst, int dst_box, cuco_ensemble_t *src, int src_box) {
    if (!dst || !src || dst_box < 0 || dst_box >= dst->nbox || src_box < 0 || src_box >= src->nbox ||
        dst->cfg[dst_box].n != src->cfg[src_box].n || dst->fixed != src->fixed ||
        dst->cfg[dst_box].boxsize != src->cfg[src_box].boxsize) {
        set_error("cuco_ensemble_copy_state: boxes differ in size, box length or mode");
        return CUCO_ERR_INVALID;
    }
    CUCO_TRY_CUDA(cudaStreamSynchronize(src->stream));
    const size_t nb = src->cfg[src_box].n;
    const uint32_t s0 = src->pbeg[src_box], d0 = dst->pbeg[dst_box];
    CUCO_TRY_CUDA(cudaMemcpyAsync(dst->pos + d0, src->pos + s0, sizeof(float4) * nb, cudaMemcpyDeviceToDevice,
                                  dst->stream));
    CUCO_TRY_CUDA(cudaMemcpyAsync(dst->vel + d0, src->vel + s0, sizeof(float4) * nb, cudaMemcpyDeviceToDevice,
                                  dst->stream));
    CUCO_TRY_CUDA(cudaStreamSynchronize(dst->stream));
    dst->has_state = true;
    return CUCO_OK;
}

cuco_status_t cuco_ensemble_footprint(const cuco_config_t *boxes, int nbox, uint64_t *bytes) {
    if (!boxes || nbox < 0 || !bytes) {
        set_error("cuco_ensemble_footprint: invalid argument");
        return CUCO_ERR_INVALID;
    }
    uint64_t b = 0, maxn = 0, ntot = 0;
    for (int k = 0; k < nbox; ++k) {
        const uint64_t n = (uint64_t)boxes[k].n, M = (uint64_t)boxes[k].pm_grid;
        ntot += n;
        const uint64_t G = boxes[k].cell_grid > 0 ? (uint64_t)boxes[k].cell_grid : M / 2;  // the largest tuned grid
        b += n * (6 * sizeof(float4) + 4 * sizeof(uint32_t));    // state, sorted copies, keys
        b += 4 * (G * G * G + 1) + 16 * G * G * G;               // cell offsets, z-slice counts
        b += 12 * M * M * M + 8 * M * M * (M / 2 + 1);           // deposit + real grid + half spectrum
        b += 12 * (M / 2 + 1) + 8 * M + 2048 + 16 * (M * M);    // tables, descriptors, CTA maps
        maxn = std::max(maxn, n);
    }
    b += 12 * maxn + 4 * (uint64_t)kNTab;
    b += 2 * 4 * 256 * (ntot / 4096 + 1);  // the sort's two digit histograms (digits of at most 8 bits)
    *bytes = b;
    return CUCO_OK;
}

}  // extern "C"
