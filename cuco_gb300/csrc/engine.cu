// Engine: one resident simulation box per handle and its force/step pipeline.
//
// A step (run.c:11-20 for a global timestep) is, on one stream:
//   k_drift_keys      drift + periodic wrap + cell key (predict.c:10-41,
//                     gravlist_kernel.cu:92-118), fused
//   sort_pairs        stable LSD radix sort of (key, index)
//   reorder           cell offsets + gather of positions into cell order
//   pm_forces         PM long-range force on the cell-ordered particles
//   shortrange        P3M short-range force; its epilogue scatters both forces
//                     to original order and kicks the velocities
// Particle state (pos, vel, forces) is kept in original particle order so that
// the permutation the sort produces is the reference's (stable sort of the keys
// of P[] in index order).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace cuco {

static thread_local std::string g_error;

void set_error(const std::string &msg) { g_error = msg; }
const char *last_error() { return g_error.c_str(); }

namespace {

__global__ void k_drift_keys(float4 *__restrict__ pos, const float4 *__restrict__ vel,
                             double drift, float boxsize, int do_drift,
                             uint32_t *__restrict__ keys, uint32_t n, float gridfac, int G) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    float c[3] = {p.x, p.y, p.z};
    if (do_drift) {
        float4 v = vel[i];
        float vv[3] = {v.x, v.y, v.z};
        const float dt = (float)drift;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            // P.Pos += P.Vel * dt_drift (predict.c:19) as one fused float
            // operation (FP64 runs at 1/64 rate here; the reference's double
            // product differs by at most one float rounding), then the wrap
            // loops of do_box_wrapping (predict.c:34-38): a float add of L
            // equals the reference's double add rounded to float.
            float x = __fmaf_rn(vv[d], dt, c[d]);
            for (int it = 0; it < 8 && x < 0.f; ++it) x = __fadd_rn(x, boxsize);
            for (int it = 0; it < 8 && x >= boxsize; ++it) x = __fsub_rn(x, boxsize);
            c[d] = x;
        }
        pos[i] = make_float4(c[0], c[1], c[2], p.w);
    }
    int k[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int v = (int)__fmul_rn(gridfac, c[d]);
        v = v < 0 ? 0 : v;
        k[d] = v >= G ? G - 1 : v;
    }
    keys[i] = ((uint32_t)k[0] * G + k[1]) * G + k[2];
}

// Fixed-point form: positions are uint32 per axis in units of L / 2^32 (bit
// patterns in the float4 slots).  The drift adds the displacement rounded
// once to that grid; the uint32 add wraps modulo 2^32, i.e. modulo L, so the
// periodic wrap is exact and needs no loop.  The key is floor(x * G / 2^32),
// an exact integer product.
__global__ void k_drift_keys_fixed(float4 *__restrict__ pos, const float4 *__restrict__ vel,
                                   float units_per_time, int do_drift, uint32_t *__restrict__ keys,
                                   uint32_t n, int G) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    uint32_t c[3] = {__float_as_uint(p.x), __float_as_uint(p.y), __float_as_uint(p.z)};
    if (do_drift) {
        const float4 v = vel[i];
        const float vv[3] = {v.x, v.y, v.z};
#pragma unroll
        for (int d = 0; d < 3; ++d) c[d] += (uint32_t)__float2ll_rn(vv[d] * units_per_time);
        pos[i] = make_float4(__uint_as_float(c[0]), __uint_as_float(c[1]), __uint_as_float(c[2]), p.w);
    }
    uint32_t k[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) k[d] = (uint32_t)(((uint64_t)c[d] * (uint32_t)G) >> 32);
    keys[i] = (k[0] * G + k[1]) * G + k[2];
}

// float positions (any real value) -> fixed point, wrapped into [0, L)
__global__ void k_to_fixed(const float *__restrict__ a, float4 *__restrict__ b, uint32_t n, double units_per_length) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t c[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) c[d] = (uint32_t)(unsigned long long)__double2ll_rn((double)a[3 * i + d] * units_per_length);
    b[i] = make_float4(__uint_as_float(c[0]), __uint_as_float(c[1]), __uint_as_float(c[2]), 0.f);
}

// fixed point -> float positions in [0, L)
__global__ void k_from_fixed(const float4 *__restrict__ b, float *__restrict__ a, uint32_t n, double length_per_unit) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = b[i];
    a[3 * i + 0] = (float)((double)__float_as_uint(v.x) * length_per_unit);
    a[3 * i + 1] = (float)((double)__float_as_uint(v.y) * length_per_unit);
    a[3 * i + 2] = (float)((double)__float_as_uint(v.z) * length_per_unit);
}

__global__ void k_scatter4(const float4 *__restrict__ src_sorted, const uint32_t *__restrict__ perm,
                           float4 *__restrict__ dst, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[perm[i]] = src_sorted[i];
}

// The PM half of the kick, after the short range's epilogue applied the PP
// half: vel += GravPM * dt (timestep.c:58,88), rounded as the epilogue rounds
// it when it applies both.
__global__ void k_kick_pm(float4 *__restrict__ vel, const float4 *__restrict__ acc_pm, uint32_t n, float km) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float4 v = vel[i];
        const float4 g = acc_pm[i];
        v.x = __fmaf_rn(g.x, km, v.x);
        v.y = __fmaf_rn(g.y, km, v.y);
        v.z = __fmaf_rn(g.z, km, v.z);
        vel[i] = v;
    }
}

__global__ void k_pack3to4(const float *__restrict__ a, float4 *__restrict__ b, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = make_float4(a[3 * i], a[3 * i + 1], a[3 * i + 2], 0.f);
}

__global__ void k_unpack4to3(const float4 *__restrict__ b, float *__restrict__ a, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float4 v = b[i];
        a[3 * i] = v.x;
        a[3 * i + 1] = v.y;
        a[3 * i + 2] = v.z;
    }
}

// FMA throughput probe: 8 independent dependency chains per thread.
__global__ void k_fma_probe(float *out, int iters, float m) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3f + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], m, 1e-7f);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int bits_for(uint32_t ncells) {
    int b = 1;
    while (b < 32 && (1ull << b) < ncells) ++b;
    return b;
}

// ----------------------------------------------------------- FP64 quadrature

struct GL20 {
    double x[20], w[20];
    GL20() {
        const int n = 20;
        for (int i = 0; i < n; ++i) {
            double t = cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
            for (int it = 0; it < 100; ++it) {
                double p0 = 1.0, p1 = t;
                for (int k = 2; k <= n; ++k) {
                    double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
                    p0 = p1;
                    p1 = p2;
                }
                dp = n * (t * p1 - p0) / (t * t - 1.0);
                double dx = p1 / dp;
                t -= dx;
                if (fabs(dx) < 1e-16) break;
            }
            x[i] = t;
            w[i] = 2.0 / ((1.0 - t * t) * dp * dp);
        }
    }
};

const GL20 &gl20() {
    static GL20 g;
    return g;
}

struct Integrand {
    double om, ol, hub;
    int power;
    double operator()(double a) const {
        double h = om / (a * a * a) + (1 - om - ol) / (a * a) + ol;
        h = hub * sqrt(h);
        return power == 3 ? 1 / (h * a * a * a) : 1 / (h * a * a);
    }
};

double gl_rule(const Integrand &f, double a, double b) {
    const GL20 &g = gl20();
    double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0.0;
    for (int i = 0; i < 20; ++i) s += g.w[i] * f(c + h * g.x[i]);
    return s * h;
}

double gl_adapt(const Integrand &f, double a, double b, double whole, double tol, int depth) {
    double c = 0.5 * (a + b);
    double l = gl_rule(f, a, c), r = gl_rule(f, c, b);
    if (depth > 40 || fabs(l + r - whole) <= tol) return l + r;
    return gl_adapt(f, a, c, l, 0.5 * tol, depth + 1) + gl_adapt(f, c, b, r, 0.5 * tol, depth + 1);
}

}  // namespace

double cosmo_integral(double a0, double a1, double omega0, double omega_lambda, double hubble,
                      int power) {
    Integrand f{omega0, omega_lambda, hubble, power};
    if (a1 == a0) return 0.0;
    double whole = gl_rule(f, a0, a1);
    return gl_adapt(f, a0, a1, whole, 1e-13 * fabs(whole) + 1e-300, 0);
}

cuco_status_t launch_drift_keys(float4 *pos, const float4 *vel, double drift, float boxsize,
                                bool do_drift, uint32_t *keys, uint32_t n, float gridfac, int G,
                                cudaStream_t stream) {
    if (!n) return CUCO_OK;
    k_drift_keys<<<(n + 255) / 256, 256, 0, stream>>>(pos, vel, drift, boxsize, do_drift ? 1 : 0,
                                                      keys, n, gridfac, G);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

cuco_status_t launch_drift_keys_fixed(float4 *pos, const float4 *vel, double drift, float boxsize,
                                      bool do_drift, uint32_t *keys, uint32_t n, int G, cudaStream_t stream) {
    if (!n) return CUCO_OK;
    const float upt = (float)(drift * 4294967296.0 / (double)boxsize);
    k_drift_keys_fixed<<<(n + 255) / 256, 256, 0, stream>>>(pos, vel, upt, do_drift ? 1 : 0, keys, n, G);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

cuco_status_t to_fixed(const float *a, float4 *b, uint32_t n, float boxsize, cudaStream_t stream) {
    if (!n) return CUCO_OK;
    k_to_fixed<<<(n + 255) / 256, 256, 0, stream>>>(a, b, n, 4294967296.0 / (double)boxsize);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

cuco_status_t from_fixed(const float4 *b, float *a, uint32_t n, float boxsize, cudaStream_t stream) {
    if (!n) return CUCO_OK;
    k_from_fixed<<<(n + 255) / 256, 256, 0, stream>>>(b, a, n, (double)boxsize / 4294967296.0);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

cuco_status_t scatter4(const float4 *src_sorted, const uint32_t *perm, float4 *dst, uint32_t n,
                       cudaStream_t stream) {
    if (!n) return CUCO_OK;
    k_scatter4<<<(n + 255) / 256, 256, 0, stream>>>(src_sorted, perm, dst, n);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

cuco_status_t pack3to4(const float *a, float4 *b, uint32_t n, cudaStream_t stream) {
    if (!n) return CUCO_OK;
    k_pack3to4<<<(n + 255) / 256, 256, 0, stream>>>(a, b, n);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

cuco_status_t unpack4to3(const float4 *b, float *a, uint32_t n, cudaStream_t stream) {
    if (!n) return CUCO_OK;
    k_unpack4to3<<<(n + 255) / 256, 256, 0, stream>>>(b, a, n);
    CUCO_TRY_CUDA(cudaGetLastError());
    return CUCO_OK;
}

void shortrange_table(float *t) {
    for (int i = 0; i < kNTab; ++i) {
        double u = 3.0 / kNTab * (i + 0.5);
        t[i] = (float)(erfc(u) + 2.0 * u / sqrt(M_PI) * exp(-u * u));
    }
}

}  // namespace cuco

using namespace cuco;

constexpr int kPhaseEvents = 10;

struct cuco_box {
    cuco_config_t cfg;
    uint32_t n = 0;
    int M = 0, G = 0;
    uint32_t ncells = 0;
    int key_bits = 0;
    float gridfac = 0.f;
    cudaStream_t stream = nullptr;
    // the PM runs on its own stream beside the sort and the cell order,
    // forked after the positions are final; joined before the short range in
    // a small box, after it in a large one (whose short range it runs beside)
    cudaStream_t pm_stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, sr_plan = nullptr;
    uint32_t split_min = 0;  // particles from which the short range runs beside the PM
    float4 *pos = nullptr, *vel = nullptr, *acc_pp = nullptr, *acc_pm = nullptr;
    float4 *spos = nullptr;
    uint32_t *keys = nullptr, *perm = nullptr, *keys_alt = nullptr, *perm_alt = nullptr;
    uint32_t *hist = nullptr, *hist2 = nullptr, *cell_off = nullptr;
    uint4 *cell_sl = nullptr;  // per cell: z-slice counts
    uint32_t *sorted_keys = nullptr, *sorted_perm = nullptr;  // where the last sort ended
    uint32_t *perm_s = nullptr;  // the z-slice order's map to original indices (the sort's spare buffer)
    float *table = nullptr;
    float *stage3 = nullptr;  // n x 3 staging for host/device float3 transfers
    PMPlan pm{};
    bool has_state = false;
    bool timing = false;
    bool count_pairs = false;
    // phase events, two sets: a step records into ev[ev_cur] and the set of
    // the step before is read then, so timing never waits on the step just
    // enqueued.  0 start, 1 positions and keys done (the PM fork), 2 sort
    // done, 3 cell order done, 4/5/6 deposit/FFT/interpolation done (PM
    // stream), 8 short range starts (after the join), 7 end.
    cudaEvent_t ev[2][kPhaseEvents] = {};
    int ev_cur = 0;
    bool ev_pending = false;  // ev[ev_cur ^ 1] holds a recorded step not yet read
    float last_ms[8] = {};
    float acc_ms[8] = {};     // phase sums since timing was enabled (or reset)
    int launches = 0;
    unsigned long long *pair_counter = nullptr;
    cudaEvent_t tstart = nullptr, tstop = nullptr;
    SRWork work{};  // the short range's work-plan scratch
};

namespace {

template <typename T>
cuco_status_t alloc(T **p, size_t count) {
    cudaError_t e = cudaMalloc(p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return CUCO_ERR_NOMEM;
    }
    return CUCO_OK;
}

ShortRangeParams make_sr_params(const cuco_box *b) {
    ShortRangeParams p{};
    p.boxsize = b->cfg.boxsize;
    p.gridfac = b->gridfac;
    p.cellw = b->cfg.boxsize / b->G;
    p.rcut = b->cfg.rcut;
    p.rcut2 = b->cfg.rcut * b->cfg.rcut;
    p.asmthfac_d = 0.5 / (double)b->cfg.asmth * (kNTab / 3.0);
    p.asmthfac = (float)p.asmthfac_d;
    p.mass = b->cfg.mass;
    p.G = (float)b->cfg.G;
    p.h = b->cfg.softening;
    p.hinv = (float)(1.0 / (double)b->cfg.softening);
    p.h3inv = p.hinv * p.hinv * p.hinv;
    p.grid = b->G;
    p.n = b->n;
    p.fixed = b->cfg.mode == CUCO_MODE_FIXED;
    p.fscale = ldexpf(b->cfg.boxsize, -32);
    p.slices = b->cell_sl;
    return p;
}

cuco_status_t drift_keys(cuco_box *b, double drift, bool do_drift) {
    if (b->cfg.mode == CUCO_MODE_FIXED)
        return launch_drift_keys_fixed(b->pos, b->vel, drift, b->cfg.boxsize, do_drift, b->keys, b->n, b->G,
                                       b->stream);
    return launch_drift_keys(b->pos, b->vel, drift, b->cfg.boxsize, do_drift, b->keys, b->n, b->gridfac, b->G,
                             b->stream);
}

void record(cuco_box *b, int i, cudaStream_t s = nullptr) {
    if (b->timing) cudaEventRecord(b->ev[b->ev_cur][i], s ? s : b->stream);
}

// Particle count from which the short range runs beside the PM (a split
// launch) rather than after it; CUCO_SPLIT_MIN_PARTICLES, read when a box is
// created, overrides it (the two schedules give the same results: the tests
// compare them).
constexpr uint32_t kSplitMinParticles = 1u << 20;

uint32_t split_min_particles() {
    const char *env = getenv("CUCO_SPLIT_MIN_PARTICLES");
    if (!env || !*env) return kSplitMinParticles;
    char *end = nullptr;
    const unsigned long long v = strtoull(env, &end, 10);
    return end && *end == '\0' && v <= 0xffffffffull ? (uint32_t)v : kSplitMinParticles;
}

// The box's stream waits for everything enqueued on the PM's stream so far.
cuco_status_t join_pm(cuco_box *b) {
    CUCO_TRY_CUDA(cudaEventRecord(b->join, b->pm_stream));
    CUCO_TRY_CUDA(cudaStreamWaitEvent(b->stream, b->join, 0));
    return CUCO_OK;
}

// keys must already be in b->keys; runs sort, reorder, PM, short range (+kick)
cuco_status_t forces_after_keys(cuco_box *b, int pm, int pp, const KickArgs *kick) {
    // The PM reads the positions in original order and writes its
    // accelerations in original order (its results do not depend on the
    // order: integer deposit sums, one interpolation per particle), so it
    // needs nothing from the sort and runs beside it.
    if (pm) {
        CUCO_TRY_CUDA(cudaEventRecord(b->fork, b->stream));
        CUCO_TRY_CUDA(cudaStreamWaitEvent(b->pm_stream, b->fork, 0));
        CUCO_TRY(pm_forces(b->pm, b->pos, b->n, b->acc_pm, b->pm_stream,
                           b->timing ? &b->ev[b->ev_cur][4] : nullptr, b->timing ? &b->ev[b->ev_cur][5] : nullptr,
                           &b->launches));
        record(b, 6, b->pm_stream);
    } else {
        record(b, 4);
        record(b, 5);
        record(b, 6);
    }
    bool in_alt = false;
    CUCO_TRY(sort_pairs(b->keys, b->perm, nullptr, b->keys_alt, b->perm_alt, b->hist, b->n,
                        b->key_bits, 8, b->stream, &in_alt, &b->launches, b->hist2));
    b->sorted_keys = in_alt ? b->keys_alt : b->keys;
    b->sorted_perm = in_alt ? b->perm_alt : b->perm;
    record(b, 2);
    CUCO_TRY(launch_reorder_offsets(b->cell_off, nullptr, b->sorted_keys, b->sorted_perm, b->pos,
                                    b->n, b->ncells, b->stream));
    // the cell order refined by z slice (the short range trims its column
    // ranges to the slices a target reaches); its map to original indices
    // goes to the sort's spare buffer
    uint32_t *perm_s = in_alt ? b->perm : b->perm_alt;
    b->perm_s = perm_s;
    const CellBox cb{(uint32_t)b->G, 0u, b->cfg.boxsize, b->gridfac};
    CUCO_TRY(launch_cell_subsort(b->cell_off, b->sorted_perm, b->pos, b->spos, perm_s, b->cell_sl, b->ncells, cb,
                                 nullptr, 1, b->cfg.mode == CUCO_MODE_FIXED, b->stream));
    b->launches += 2;
    record(b, 3);
    // The short range needs nothing from the PM: in a large box it starts
    // when the cell order is ready, one CTA per SM short of a full persistent
    // grid, so the PM's remaining kernels keep running beside it; its last
    // CTAs are queued on the PM's stream behind the PM and take the units
    // left then, and the PM half of the kick follows once both are done.  A
    // small box's step is launch-bound: its short range waits for the PM and
    // applies both halves of the kick in its epilogue (fewer launches).
    const bool split = pm && b->n >= b->split_min;
    if (pm && !split) CUCO_TRY(join_pm(b));
    record(b, 8);
    const bool kick_on = kick && kick->vel;
    if (pp) {
        KickArgs k{};
        if (kick) k = *kick;
        k.acc_pm_s = nullptr;
        k.acc_pm_out = nullptr;
        k.acc_pm_o = pm && !split ? b->acc_pm : nullptr;
        CUCO_TRY(launch_shortrange(make_sr_params(b), b->spos, perm_s, b->cell_off,
                                   nullptr, kCellOffsets, b->table, b->acc_pp, k, b->work, b->stream,
                                   b->count_pairs ? b->pair_counter : nullptr, split ? b->pm_stream : nullptr,
                                   b->sr_plan));
        b->launches += split ? 3 : 2;  // work plan + persistent short range (in two parts beside the PM)
    }
    if (split) CUCO_TRY(join_pm(b));
    record(b, 9);  // the short range done (both parts)
    if (split && pp && kick_on && b->n) {
        k_kick_pm<<<(b->n + 255) / 256, 256, 0, b->stream>>>(kick->vel, b->acc_pm, b->n, (float)kick->kick_pm);
        CUCO_TRY_CUDA(cudaGetLastError());
        b->launches += 1;
    }
    if (pm && !pp) CUCO_TRY(join_pm(b));
    record(b, 7);
    return CUCO_OK;
}

// Phase times of the pending set into last_ms and acc_ms.
cuco_status_t read_pending(cuco_box *b) {
    if (!b->ev_pending) return CUCO_OK;
    b->ev_pending = false;
    cudaEvent_t *e = b->ev[b->ev_cur ^ 1];
    CUCO_TRY_CUDA(cudaEventSynchronize(e[7]));
    // drift+keys, sort, cell order; the PM's three phases from the fork (they
    // overlap the sort, the cell order and the start of the short range); the
    // short range from the cell order to the end of both parts of its launch;
    // the whole pass
    static const int from[8] = {0, 1, 2, 1, 4, 5, 8, 0}, to[8] = {1, 2, 3, 4, 5, 6, 9, 7};
    for (int i = 0; i < 8; ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e[from[i]], e[to[i]]);
        b->last_ms[i] = ms;
        b->acc_ms[i] += ms;
    }
    return CUCO_OK;
}

// End of a timed force pass: read the step before (done, or nearly, by the
// time this one is enqueued), leave this one pending, switch sets.
cuco_status_t finish_timing(cuco_box *b) {
    if (!b->timing) return CUCO_OK;
    CUCO_TRY(read_pending(b));
    b->ev_pending = true;
    b->ev_cur ^= 1;
    return CUCO_OK;
}

}  // namespace

extern "C" {

const char *cuco_last_error(void) { return cuco::last_error(); }
const char *cuco_version(void) { return "cuco_gb300 0.1 (sm_103a)"; }

cuco_status_t cuco_config_reference(cuco_config_t *cfg) {
    if (!cfg || cfg->pm_grid <= 0 || !(cfg->boxsize > 0)) {
        set_error("cuco_config_reference: pm_grid and boxsize must be set");
        return CUCO_ERR_INVALID;
    }
    // pm_periodic.c:27-28: All.Asmth and All.Rcut are float
    float asmth = (float)(CUCO_ASMTH * (double)cfg->boxsize / cfg->pm_grid);
    cfg->asmth = asmth;
    cfg->rcut = (float)(CUCO_RCUT * (double)asmth);
    if (cfg->cell_grid <= 0) cfg->cell_grid = cfg->pm_grid / 4 < 8 ? 8 : cfg->pm_grid / 4;
    return CUCO_OK;
}

cuco_status_t cuco_box_create(const cuco_config_t *cfg, cuco_box_t **out) {
    if (!cfg || !out) {
        set_error("cuco_box_create: null argument");
        return CUCO_ERR_INVALID;
    }
    if (cfg->n < 0 || cfg->n > 0xfffffff0ll || cfg->cell_grid < 4 || cfg->cell_grid > 1024 ||
        !(cfg->boxsize > 0) || !(cfg->rcut > 0) || !(cfg->asmth > 0) || !(cfg->softening > 0)) {
        set_error("cuco_box_create: invalid configuration");
        return CUCO_ERR_INVALID;
    }
    if (cfg->mode != CUCO_MODE_PLAIN && cfg->mode != CUCO_MODE_FIXED) {
        set_error("cuco_box_create: unknown mode");
        return CUCO_ERR_INVALID;
    }
    CUCO_TRY_CUDA(cudaSetDevice(cfg->device));
    cuco_box *b = new cuco_box();
    b->cfg = *cfg;
    b->n = (uint32_t)cfg->n;
    b->M = cfg->pm_grid;
    b->G = cfg->cell_grid;
    b->ncells = (uint32_t)b->G * b->G * b->G;
    b->key_bits = bits_for(b->ncells);
    b->gridfac = (float)b->G / cfg->boxsize;  // float division as gravlist.cpp:61
    b->split_min = split_min_particles();
    cuco_status_t s = CUCO_OK;
    auto fail = [&](cuco_status_t st) {
        cuco_box_destroy(b);
        return st;
    };
    // The box's stream has the higher priority: while the PM runs beside the
    // sort and the cell order, their CTAs are scheduled first and the PM
    // takes the SMs they leave idle (measured faster than the reverse, whose
    // sort passes waited behind the PM's transform CTAs).
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithPriority(&b->stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        delete b;
        return CUCO_ERR_CUDA;
    }
    if (cudaStreamCreateWithPriority(&b->pm_stream, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->sr_plan, cudaEventDisableTiming) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        return fail(CUCO_ERR_CUDA);
    }
    const size_t n = b->n;
    if ((s = alloc(&b->pos, n)) || (s = alloc(&b->vel, n)) || (s = alloc(&b->acc_pp, n)) ||
        (s = alloc(&b->acc_pm, n)) || (s = alloc(&b->spos, n)) ||
        (s = alloc(&b->keys, n)) || (s = alloc(&b->perm, n)) || (s = alloc(&b->keys_alt, n)) ||
        (s = alloc(&b->perm_alt, n)) ||
        (s = alloc(&b->hist, sort_hist_entries(b->n, b->key_bits, 8))) ||
        (s = alloc(&b->hist2, sort_hist_entries(b->n, b->key_bits, 8))) ||
        (s = alloc(&b->cell_off, (size_t)b->ncells + 1)) || (s = alloc(&b->cell_sl, (size_t)b->ncells)) ||
        (s = alloc(&b->table, kNTab)) ||
        (s = alloc(&b->stage3, 3 * n)) || (s = alloc(&b->pair_counter, 1)) ||
        (s = alloc(&b->work.heavy, shortrange_heavy_cap(b->n))) || (s = alloc(&b->work.seg_nt, b->ncells)) ||
        (s = alloc(&b->work.ctl, kSRCtlWords)))
        return fail(s);
    cudaMemset(b->work.ctl, 0, sizeof(uint32_t) * kSRCtlWords);
    b->work.heavy_cap = shortrange_heavy_cap(b->n);
    b->work.seg_cap = b->ncells;  // G^3 covers every segment length
    cudaMemset(b->pair_counter, 0, sizeof(unsigned long long));
    std::vector<float> t(kNTab);
    shortrange_table(t.data());
    if (cudaMemcpy(b->table, t.data(), sizeof(float) * kNTab, cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("table upload failed");
        return fail(CUCO_ERR_CUDA);
    }
    if ((s = pm_plan_create(&b->pm, b->M, cfg->boxsize, cfg->asmth, cfg->mass, cfg->G,
                            cfg->mode == CUCO_MODE_FIXED)))
        return fail(s);
    cudaMemsetAsync(b->acc_pp, 0, sizeof(float4) * (n ? n : 1), b->stream);
    cudaMemsetAsync(b->acc_pm, 0, sizeof(float4) * (n ? n : 1), b->stream);
    cudaMemsetAsync(b->vel, 0, sizeof(float4) * (n ? n : 1), b->stream);
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < kPhaseEvents; ++i) cudaEventCreate(&b->ev[k][i]);
    cudaEventCreate(&b->tstart);
    cudaEventCreate(&b->tstop);
    *out = b;
    return CUCO_OK;
}

cuco_status_t cuco_box_destroy(cuco_box_t *b) {
    if (!b) return CUCO_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->pm_stream) cudaStreamSynchronize(b->pm_stream);  // a pass that stopped before its join
    cudaFree(b->pos);
    cudaFree(b->vel);
    cudaFree(b->acc_pp);
    cudaFree(b->acc_pm);
    cudaFree(b->spos);
    cudaFree(b->keys);
    cudaFree(b->perm);
    cudaFree(b->keys_alt);
    cudaFree(b->perm_alt);
    cudaFree(b->hist);
    cudaFree(b->hist2);
    cudaFree(b->cell_off);
    cudaFree(b->cell_sl);
    cudaFree(b->table);
    cudaFree(b->stage3);
    cudaFree(b->pair_counter);
    cudaFree(b->work.heavy);
    cudaFree(b->work.seg_nt);
    cudaFree(b->work.ctl);
    if (b->tstart) cudaEventDestroy(b->tstart);
    if (b->tstop) cudaEventDestroy(b->tstop);
    if (b->pm.rho) pm_plan_destroy(&b->pm);
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < kPhaseEvents; ++i)
            if (b->ev[k][i]) cudaEventDestroy(b->ev[k][i]);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    if (b->sr_plan) cudaEventDestroy(b->sr_plan);
    if (b->pm_stream) cudaStreamDestroy(b->pm_stream);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return CUCO_OK;
}

}  // extern "C"

namespace state_check {
__global__ void k_count_nonfinite(const float *__restrict__ v, size_t n, uint32_t *__restrict__ count) {
    uint32_t bad = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        bad += !isfinite(v[i]);
    bad = __reduce_add_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(count, bad);
}

// The staged triplets (b->stage3) must all be finite: a state with a NaN or
// an infinity is refused before it reaches the box (CUCO_ERR_INVALID).
cuco_status_t check_finite(cuco_box_t *b, const char *what) {
    uint32_t *count = b->work.ctl + 3;  // the plan's spare control word
    CUCO_TRY_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t), b->stream));
    const size_t n = 3 * (size_t)b->n;
    if (n) {
        const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
        k_count_nonfinite<<<blocks, 256, 0, b->stream>>>(b->stage3, n, count);
        CUCO_TRY_CUDA(cudaGetLastError());
    }
    uint32_t bad = 0;
    CUCO_TRY_CUDA(cudaMemcpyAsync(&bad, count, sizeof bad, cudaMemcpyDeviceToHost, b->stream));
    CUCO_TRY_CUDA(cudaStreamSynchronize(b->stream));
    if (bad) {
        set_error(std::string("cuco_box_set_state: ") + std::to_string(bad) + " " + what +
                  " components are not finite");
        return CUCO_ERR_INVALID;
    }
    return CUCO_OK;
}
}  // namespace state_check

using state_check::check_finite;

extern "C" {

cuco_status_t cuco_box_set_state(cuco_box_t *b, const float *pos, const float *vel, int on_device) {
    if (!b || !pos) {
        set_error("cuco_box_set_state: null argument");
        return CUCO_ERR_INVALID;
    }
    const size_t bytes = sizeof(float) * 3 * b->n;
    cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    CUCO_TRY_CUDA(cudaMemcpyAsync(b->stage3, pos, bytes, kind, b->stream));
    CUCO_TRY(check_finite(b, "position"));
    if (b->cfg.mode == CUCO_MODE_FIXED)
        CUCO_TRY(to_fixed(b->stage3, b->pos, b->n, b->cfg.boxsize, b->stream));
    else
        CUCO_TRY(pack3to4(b->stage3, b->pos, b->n, b->stream));
    if (vel) {
        CUCO_TRY_CUDA(cudaMemcpyAsync(b->stage3, vel, bytes, kind, b->stream));
        CUCO_TRY(check_finite(b, "velocity"));
        CUCO_TRY(pack3to4(b->stage3, b->vel, b->n, b->stream));
    }
    b->has_state = true;
    return CUCO_OK;
}

cuco_status_t cuco_box_get_state(cuco_box_t *b, float *pos, float *vel, float *acc_pp,
                                 float *acc_pm, int on_device) {
    if (!b) {
        set_error("cuco_box_get_state: null box");
        return CUCO_ERR_INVALID;
    }
    const size_t bytes = sizeof(float) * 3 * b->n;
    cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    float *dst[4] = {pos, vel, acc_pp, acc_pm};
    float4 *src[4] = {b->pos, b->vel, b->acc_pp, b->acc_pm};
    for (int k = 0; k < 4; ++k) {
        if (!dst[k]) continue;
        if (k == 0 && b->cfg.mode == CUCO_MODE_FIXED)
            CUCO_TRY(from_fixed(src[k], b->stage3, b->n, b->cfg.boxsize, b->stream));
        else
            CUCO_TRY(unpack4to3(src[k], b->stage3, b->n, b->stream));
        CUCO_TRY_CUDA(cudaMemcpyAsync(dst[k], b->stage3, bytes, kind, b->stream));
    }
    CUCO_TRY_CUDA(cudaStreamSynchronize(b->stream));
    return shortrange_check(b->work.ctl, b->stream);
}

cuco_status_t cuco_box_set_state_fixed(cuco_box_t *b, const uint32_t *pos, const float *vel, int on_device) {
    if (!b || !pos || b->cfg.mode != CUCO_MODE_FIXED) {
        set_error("cuco_box_set_state_fixed: null argument or not a fixed-point box");
        return CUCO_ERR_INVALID;
    }
    const size_t bytes = sizeof(float) * 3 * b->n;
    cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    // the uint32 triplets move as bit patterns: pack3to4 only copies words
    CUCO_TRY_CUDA(cudaMemcpyAsync(b->stage3, pos, bytes, kind, b->stream));
    CUCO_TRY(pack3to4(b->stage3, b->pos, b->n, b->stream));
    if (vel) {
        CUCO_TRY_CUDA(cudaMemcpyAsync(b->stage3, vel, bytes, kind, b->stream));
        CUCO_TRY(check_finite(b, "velocity"));
        CUCO_TRY(pack3to4(b->stage3, b->vel, b->n, b->stream));
    }
    b->has_state = true;
    return CUCO_OK;
}

cuco_status_t cuco_box_get_state_fixed(cuco_box_t *b, uint32_t *pos, int on_device) {
    if (!b || !pos || b->cfg.mode != CUCO_MODE_FIXED) {
        set_error("cuco_box_get_state_fixed: null argument or not a fixed-point box");
        return CUCO_ERR_INVALID;
    }
    CUCO_TRY(unpack4to3(b->pos, b->stage3, b->n, b->stream));
    CUCO_TRY_CUDA(cudaMemcpyAsync(pos, b->stage3, sizeof(float) * 3 * b->n,
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, b->stream));
    CUCO_TRY_CUDA(cudaStreamSynchronize(b->stream));
    return CUCO_OK;
}

cuco_status_t cuco_box_set_softening(cuco_box_t *b, float h) {
    if (!b || !(h > 0)) {
        set_error("cuco_box_set_softening: invalid argument");
        return CUCO_ERR_INVALID;
    }
    b->cfg.softening = h;
    return CUCO_OK;
}

cuco_status_t cuco_box_forces(cuco_box_t *b, int pm, int pp) {
    if (!b || !b->has_state) {
        set_error("cuco_box_forces: no state uploaded");
        return CUCO_ERR_STATE;
    }
    b->launches = 0;
    record(b, 0);
    CUCO_TRY(drift_keys(b, 0.0, false));
    b->launches += 1;
    record(b, 1);
    CUCO_TRY(forces_after_keys(b, pm, pp, nullptr));
    CUCO_TRY(finish_timing(b));
    return CUCO_OK;
}

cuco_status_t cuco_box_step(cuco_box_t *b, double drift, double kick_pp, double kick_pm) {
    if (!b || !b->has_state) {
        set_error("cuco_box_step: no state uploaded");
        return CUCO_ERR_STATE;
    }
    b->launches = 0;
    record(b, 0);
    CUCO_TRY(drift_keys(b, drift, drift != 0.0));
    b->launches += 1;
    record(b, 1);
    KickArgs k{};
    k.vel = b->vel;
    k.kick_pp = kick_pp;
    k.kick_pm = kick_pm;
    CUCO_TRY(forces_after_keys(b, 1, 1, &k));
    CUCO_TRY(finish_timing(b));
    return CUCO_OK;
}

cuco_status_t cuco_box_run(cuco_box_t *b, int nsteps, const double *drift, const double *kick_pp,
                           const double *kick_pm) {
    if (!b || nsteps < 0 || (nsteps && (!drift || !kick_pp || !kick_pm))) {
        set_error("cuco_box_run: invalid argument");
        return CUCO_ERR_INVALID;
    }
    for (int s = 0; s < nsteps; ++s) CUCO_TRY(cuco_box_step(b, drift[s], kick_pp[s], kick_pm[s]));
    return CUCO_OK;
}

cuco_status_t cuco_debug_bounds_violations(uint64_t *count) {
#ifdef CUCO_BOUNDS_CHECK
    CUCO_TRY_CUDA(cudaDeviceSynchronize());
    const uint64_t v = (uint64_t)bounds_violations_sort() + bounds_violations_pm() + bounds_violations_shortrange();
    if (count) *count = v;
    return CUCO_OK;
#else
    (void)count;
    set_error("cuco_debug_bounds_violations: this library is a release build (no bounds checks)");
    return CUCO_ERR_UNSUPPORTED;
#endif
}

cuco_status_t cuco_box_selftest_timeout(cuco_box_t *b, double seconds) {
    if (!b || !(seconds > 0) || seconds > 1.0) {
        set_error("cuco_box_selftest_timeout: null box or a limit outside (0, 1] s");
        return CUCO_ERR_INVALID;
    }
    int dev = 0, khz = 0;
    CUCO_TRY_CUDA(cudaGetDevice(&dev));
    CUCO_TRY_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
    const long long cycles = (long long)(seconds * 1e3 * (khz > 0 ? khz : 2000000));
    return shortrange_timeout_probe(b->work.ctl, cycles, b->stream);
}

cuco_status_t cuco_box_sync(cuco_box_t *b) {
    if (!b) return CUCO_ERR_INVALID;
    CUCO_TRY_CUDA(cudaStreamSynchronize(b->stream));
    return shortrange_check(b->work.ctl, b->stream);
}

cuco_status_t cuco_box_stream(cuco_box_t *b, void **stream) {
    if (!b || !stream) return CUCO_ERR_INVALID;
    *stream = (void *)b->stream;
    return CUCO_OK;
}

cuco_status_t cuco_box_enable_timing(cuco_box_t *b, int enable) {
    if (!b) return CUCO_ERR_INVALID;
    CUCO_TRY(read_pending(b));
    b->timing = enable != 0;
    memset(b->acc_ms, 0, sizeof(b->acc_ms));
    return CUCO_OK;
}

cuco_status_t cuco_box_timings(cuco_box_t *b, float *ms) {
    if (!b || !ms) return CUCO_ERR_INVALID;
    CUCO_TRY(read_pending(b));
    memcpy(ms, b->last_ms, sizeof(b->last_ms));
    return CUCO_OK;
}

cuco_status_t cuco_box_phase_totals(cuco_box_t *b, float *ms, int reset) {
    if (!b || !ms) return CUCO_ERR_INVALID;
    CUCO_TRY(read_pending(b));
    memcpy(ms, b->acc_ms, sizeof(b->acc_ms));
    if (reset) memset(b->acc_ms, 0, sizeof(b->acc_ms));
    return CUCO_OK;
}

cuco_status_t cuco_box_debug(cuco_box_t *b, uint32_t *sorted_keys, uint32_t *perm,
                             uint32_t *cell_start, uint32_t *cell_end) {
    if (!b || !b->sorted_keys) {
        set_error("cuco_box_debug: no forces computed yet");
        return CUCO_ERR_STATE;
    }
    CUCO_TRY_CUDA(cudaStreamSynchronize(b->stream));
    const size_t n = b->n;
    if (sorted_keys) CUCO_TRY_CUDA(cudaMemcpy(sorted_keys, b->sorted_keys, 4 * n, cudaMemcpyDeviceToHost));
    if (perm) CUCO_TRY_CUDA(cudaMemcpy(perm, b->sorted_perm, 4 * n, cudaMemcpyDeviceToHost));
    if (cell_start || cell_end) {
        std::vector<uint32_t> off(b->ncells + 1);
        CUCO_TRY_CUDA(cudaMemcpy(off.data(), b->cell_off, 4 * off.size(), cudaMemcpyDeviceToHost));
        for (uint32_t c = 0; c < b->ncells; ++c) {
            bool empty = off[c] == off[c + 1];
            if (cell_start) cell_start[c] = empty ? kEmptyCell : off[c];
            if (cell_end) cell_end[c] = empty ? kEmptyCell : off[c + 1];
        }
    }
    return CUCO_OK;
}

cuco_status_t cuco_box_cell_order(cuco_box_t *b, uint32_t *perm_s, float *slice) {
    if (!b || !b->perm_s) {
        set_error("cuco_box_cell_order: no forces computed yet");
        return CUCO_ERR_STATE;
    }
    CUCO_TRY_CUDA(cudaStreamSynchronize(b->stream));
    if (perm_s) CUCO_TRY_CUDA(cudaMemcpy(perm_s, b->perm_s, 4 * (size_t)b->n, cudaMemcpyDeviceToHost));
    if (slice && b->n)
        CUCO_TRY_CUDA(cudaMemcpy2D(slice, sizeof(float), &b->spos[0].w, sizeof(float4), sizeof(float), b->n,
                                   cudaMemcpyDeviceToHost));
    return CUCO_OK;
}

int cuco_box_launches_per_step(cuco_box_t *b) { return b ? b->launches : 0; }

cuco_status_t cuco_box_count_pairs(cuco_box_t *b, int enable) {
    if (!b) return CUCO_ERR_INVALID;
    b->count_pairs = enable != 0;
    return CUCO_OK;
}

cuco_status_t cuco_box_pair_count(cuco_box_t *b, uint64_t *pairs, int reset) {
    if (!b || !pairs) return CUCO_ERR_INVALID;
    CUCO_TRY_CUDA(cudaStreamSynchronize(b->stream));
    unsigned long long v = 0;
    CUCO_TRY_CUDA(cudaMemcpy(&v, b->pair_counter, sizeof(v), cudaMemcpyDeviceToHost));
    *pairs = v;
    if (reset) CUCO_TRY_CUDA(cudaMemset(b->pair_counter, 0, sizeof(v)));
    return CUCO_OK;
}

cuco_status_t cuco_box_timer(cuco_box_t *b, int op, float *ms) {
    if (!b) return CUCO_ERR_INVALID;
    if (op == 0) {
        CUCO_TRY_CUDA(cudaEventRecord(b->tstart, b->stream));
        return CUCO_OK;
    }
    CUCO_TRY_CUDA(cudaEventRecord(b->tstop, b->stream));
    CUCO_TRY_CUDA(cudaEventSynchronize(b->tstop));
    float t = 0.f;
    CUCO_TRY_CUDA(cudaEventElapsedTime(&t, b->tstart, b->tstop));
    if (ms) *ms = t;
    return CUCO_OK;
}

cuco_status_t cuco_pinned_alloc(size_t bytes, void **ptr) {
    if (!ptr) return CUCO_ERR_INVALID;
    CUCO_TRY_CUDA(cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault));
    return CUCO_OK;
}

cuco_status_t cuco_pinned_free(void *ptr) {
    CUCO_TRY_CUDA(cudaFreeHost(ptr));
    return CUCO_OK;
}

cuco_status_t cuco_fp32_peak(int device, double *tflops) {
    if (!tflops) return CUCO_ERR_INVALID;
    CUCO_TRY_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    CUCO_TRY_CUDA(cudaGetDeviceProperties(&prop, device));
    const int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 4096;
    float *out = nullptr;
    CUCO_TRY_CUDA(cudaMalloc(&out, sizeof(float) * blocks * threads));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0);
        k_fma_probe<<<blocks, threads>>>(out, iters, 1.0f + 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) {
        set_error(cudaGetErrorString(e));
        return CUCO_ERR_CUDA;
    }
    // 8 independent chains x iters FMAs x 2 flops per thread
    double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return CUCO_OK;
}

// Internal (hidden) helpers for the drop-in layer in the same library.
__attribute__((visibility("hidden"))) cuco_status_t cuco_box_internal_arrays(
    cuco_box_t *b, float4 **pos, float4 **vel, float4 **acc_pp, float4 **acc_pm, void **stream,
    uint32_t **keys, uint32_t **perm, float4 **spos) {
    *pos = b->pos;
    *vel = b->vel;
    *acc_pp = b->acc_pp;
    *acc_pm = b->acc_pm;
    *stream = (void *)b->stream;
    *keys = b->keys;
    *perm = b->perm;
    *spos = b->spos;
    return CUCO_OK;
}

__attribute__((visibility("hidden"))) cuco_status_t cuco_box_mark_state(cuco_box_t *b) {
    b->has_state = true;
    return CUCO_OK;
}

}  // extern "C"

// ---- .cuco snapshot / initial-conditions files (read_ic.c:9-45, io.c:9-40):
// HEADER (32 bytes) then PARTICLE[NumPart] (60 bytes each), raw, host order.
namespace snapshot_io {

__global__ void k_records_to_state(const PARTICLE *__restrict__ rec, uint32_t n, float vscale,
                                   float *__restrict__ pos3, float *__restrict__ vel3) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const PARTICLE r = rec[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        pos3[3 * (size_t)i + d] = r.Pos[d];
        vel3[3 * (size_t)i + d] = vscale == 1.0f ? r.Vel[d] : __fmul_rn(r.Vel[d], vscale);
    }
}

__global__ void k_state_to_records(const float *__restrict__ pos3, const float *__restrict__ vel3,
                                   const float *__restrict__ app3, const float *__restrict__ apm3, float mass,
                                   uint32_t n, PARTICLE *__restrict__ rec) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PARTICLE r;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        r.Pos[d] = pos3[3 * (size_t)i + d];
        r.Vel[d] = vel3[3 * (size_t)i + d];
        r.GravAccel[d] = app3[3 * (size_t)i + d];
        r.GravPM[d] = apm3[3 * (size_t)i + d];
    }
    r.Mass = mass;
    r.Ti_endstep = 0;
    r.Ti_begstep = 0;
    rec[i] = r;
}

struct DeviceScratch {
    void *p[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    ~DeviceScratch() {
        for (void *q : p) cudaFree(q);
    }
};

struct HostFile {
    FILE *f = nullptr;
    ~HostFile() {
        if (f) fclose(f);
    }
};

}  // namespace snapshot_io

using namespace snapshot_io;

extern "C" {

cuco_status_t cuco_box_load_snapshot(cuco_box_t *b, const char *path, int initial_conditions, HEADER *header) {
    if (!b || !path) {
        set_error("cuco_box_load_snapshot: null argument");
        return CUCO_ERR_INVALID;
    }
    HostFile hf;
    hf.f = fopen(path, "rb");
    if (!hf.f) {
        set_error(std::string("cuco_box_load_snapshot: cannot open ") + path);
        return CUCO_ERR_INVALID;
    }
    HEADER h;
    if (fread(&h, sizeof h, 1, hf.f) != 1) {
        set_error("cuco_box_load_snapshot: short header");
        return CUCO_ERR_INVALID;
    }
    if (h.NumPart < 0 || (int64_t)h.NumPart != b->n) {
        set_error("cuco_box_load_snapshot: the file holds " + std::to_string(h.NumPart) +
                  " particles, the box " + std::to_string(b->n));
        return CUCO_ERR_INVALID;
    }
    const size_t n = (size_t)b->n;
    std::vector<PARTICLE> rec(n);
    if (n && fread(rec.data(), sizeof(PARTICLE), n, hf.f) != n) {
        set_error("cuco_box_load_snapshot: the file ends before its " + std::to_string(n) + " particles");
        return CUCO_ERR_INVALID;
    }
    if (header) *header = h;
    if (!n) return CUCO_OK;
    // init.c:30 scales an IC file's velocities by a^(3/2) into the
    // integrator's variable; a snapshot stores that variable already
    const float vscale = initial_conditions ? (float)(sqrt((double)h.Time) * (double)h.Time) : 1.0f;
    DeviceScratch ds;
    CUCO_TRY_CUDA(cudaMalloc(&ds.p[0], sizeof(PARTICLE) * n));
    CUCO_TRY_CUDA(cudaMalloc(&ds.p[1], sizeof(float) * 3 * n));
    CUCO_TRY_CUDA(cudaMalloc(&ds.p[2], sizeof(float) * 3 * n));
    CUCO_TRY_CUDA(cudaMemcpyAsync(ds.p[0], rec.data(), sizeof(PARTICLE) * n, cudaMemcpyHostToDevice, b->stream));
    k_records_to_state<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(
        static_cast<const PARTICLE *>(ds.p[0]), (uint32_t)n, vscale, static_cast<float *>(ds.p[1]),
        static_cast<float *>(ds.p[2]));
    CUCO_TRY_CUDA(cudaGetLastError());
    CUCO_TRY(cuco_box_set_state(b, static_cast<float *>(ds.p[1]), static_cast<float *>(ds.p[2]), 1));
    CUCO_TRY_CUDA(cudaStreamSynchronize(b->stream));
    return CUCO_OK;
}

cuco_status_t cuco_box_save_snapshot(cuco_box_t *b, const char *path, const HEADER *header) {
    if (!b || !path || !header) {
        set_error("cuco_box_save_snapshot: null argument");
        return CUCO_ERR_INVALID;
    }
    if (!b->has_state) {
        set_error("cuco_box_save_snapshot: the box has no state");
        return CUCO_ERR_STATE;
    }
    const size_t n = (size_t)b->n;
    HEADER h = *header;
    h.NumPart = (int)b->n;
    std::vector<PARTICLE> rec(n);
    if (n) {
        DeviceScratch ds;
        CUCO_TRY_CUDA(cudaMalloc(&ds.p[0], sizeof(PARTICLE) * n));
        for (int k = 1; k <= 4; ++k) CUCO_TRY_CUDA(cudaMalloc(&ds.p[k], sizeof(float) * 3 * n));
        float *f[4] = {static_cast<float *>(ds.p[1]), static_cast<float *>(ds.p[2]), static_cast<float *>(ds.p[3]),
                       static_cast<float *>(ds.p[4])};
        CUCO_TRY(cuco_box_get_state(b, f[0], f[1], f[2], f[3], 1));
        k_state_to_records<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(
            f[0], f[1], f[2], f[3], header->Mass, (uint32_t)n, static_cast<PARTICLE *>(ds.p[0]));
        CUCO_TRY_CUDA(cudaGetLastError());
        CUCO_TRY_CUDA(cudaMemcpyAsync(rec.data(), ds.p[0], sizeof(PARTICLE) * n, cudaMemcpyDeviceToHost, b->stream));
        CUCO_TRY_CUDA(cudaStreamSynchronize(b->stream));
    }
    HostFile hf;
    hf.f = fopen(path, "wb");
    if (!hf.f) {
        set_error(std::string("cuco_box_save_snapshot: cannot create ") + path);
        return CUCO_ERR_INVALID;
    }
    if (fwrite(&h, sizeof h, 1, hf.f) != 1 || (n && fwrite(rec.data(), sizeof(PARTICLE), n, hf.f) != n)) {
        set_error(std::string("cuco_box_save_snapshot: write failed on ") + path);
        return CUCO_ERR_INVALID;
    }
    return CUCO_OK;
}

cuco_status_t cuco_cosmo_factors(double a0, double a1, double omega0, double omega_lambda,
                                 double hubble, double *drift, double *kick) {
    if (!(a0 > 0) || !(a1 > 0)) {
        set_error("cuco_cosmo_factors: scale factors must be positive");
        return CUCO_ERR_INVALID;
    }
    if (drift) *drift = cosmo_integral(a0, a1, omega0, omega_lambda, hubble, 3);
    if (kick) *kick = cosmo_integral(a0, a1, omega0, omega_lambda, hubble, 2);
    return CUCO_OK;
}

}  // extern "C"
