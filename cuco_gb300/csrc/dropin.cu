// Drop-in replacements for the reference's host force and integrator functions,
// working on its globals (allvars.h:120-142).
//
// The reference host program keeps P[] (array of PARTICLE) in host memory and
// calls these functions from begrun()/run().  Where the device reads and
// writes pageable host memory coherently (a Grace host over NVLink-C2C), the
// kernels of each call work on P[] in place and write back only the fields
// the call changes; elsewhere each call copies P[] to a device mirror, runs
// the same kernels on it, and copies it back.  Either way the host sees the
// reference's fields updated in place when the call returns:
//   pm_init_periodic / long_range_init   pm_periodic.c:25-43, longrange.c:8-12
//   pmforce_periodic / long_range_force  pm_periodic.c:67-314, longrange.c:14-22
//   set_softenings / linklist_init       gravlist.cpp:28-115
//   gravity_linklist_cuda                gravlist.cpp:148-193
//   compute_accelerations                accel.c:8-23 (one round trip for wrap+PM+PP)
//   move_particles / do_box_wrapping     predict.c:10-41
//   advance_and_find_timesteps           timestep.c:11-94 (individual power-of-two
//                                        steps, evaluated per particle on the device)
//   get_timestep                         timestep.c:96-138
//   init_drift_table, get_*_factor       driftfac.c:14-126 (tables in FP64)
// The globals themselves are defined weakly here so that the library loads on
// its own (tests drive it through these symbols); a host program's own
// allvars.c definitions take precedence.
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "radixsort.h"

extern "C" {
__attribute__((weak)) unsigned int NumPart;
__attribute__((weak)) PARTICLE *P;
__attribute__((weak)) HEADER header;
__attribute__((weak)) ALL All;
__attribute__((weak)) float DriftTable[CUCO_DRIFT_TABLE_LENGTH];
__attribute__((weak)) float GravKickTable[CUCO_DRIFT_TABLE_LENGTH];
__attribute__((weak)) unsigned int numParticles;
__attribute__((weak)) unsigned int numGridCells;
__attribute__((weak)) float *hPos;
__attribute__((weak)) float *hGravAccel;
__attribute__((weak)) float *dOldPos;
__attribute__((weak)) float *dSortedPos;
__attribute__((weak)) float *dGravAccel;
__attribute__((weak)) unsigned int *dGridParticleHash;
__attribute__((weak)) unsigned int *dGridParticleIndex;
__attribute__((weak)) unsigned int *dCellStart;
__attribute__((weak)) unsigned int *dCellEnd;
}

/* gravlist.cu:20.  linklist_init creates it as gravlist.cpp:98 does, so a host
 * that keeps the reference's gravlist.cpp finds it; the drop-in's own
 * gravity_linklist_cuda sorts inside the engine and does not use it. */
RadixSort *sorter;

namespace cuco {
void capi_set_grid(int G);
[[noreturn]] void capi_fail(const char *where, const char *what);
void capi_check(cudaError_t e, const char *where);
void capi_status(cuco_status_t s, const char *where);
cuco_status_t scatter4(const float4 *src_sorted, const uint32_t *perm, float4 *dst, uint32_t n,
                       cudaStream_t stream);
void shortrange_table(float *t);
}  // namespace cuco

using namespace cuco;

namespace {

struct DropinState {
    int pmgrid = 64;
    int cellgrid = 0;
    cuco_box_t *box = nullptr;
    uint32_t box_n = 0;
    char *dP = nullptr;  // device mirror of P[]
    size_t dP_n = 0;
    int *dflag = nullptr;  // timestep error flag + particle
    double *dtab = nullptr;  // FP64 kick table on the device
    bool dtab_valid = false;
    double drift64[CUCO_DRIFT_TABLE_LENGTH];
    double kick64[CUCO_DRIFT_TABLE_LENGTH];
    double logTimeBegin = 0, logTimeMax = 0;
    bool tables = false;
    SOFTPARAM soft{};
    // short-range constants as gravlist.cpp keeps them
    double h = 0, h_inv = 0, h3_inv = 0;
    int direct = -1;  // kernels work on the host P[] in place (1) or on dP (0)
    int min_endstep = 0;  // min P[].Ti_endstep written by advance_and_find_timesteps
    bool min_valid = false;
    const void *min_P = nullptr;  // the P[] and NumPart it was taken over
    unsigned min_n = 0;
};

DropinState &ds() {
    static DropinState s;
    return s;
}

// Grid of calcHash and of the cellStart/cellEnd arrays: PMGRID, as the
// reference fixes it (gravlist_kernel.cu:114), unless configured.
int cell_grid() { return ds().cellgrid > 0 ? ds().cellgrid : ds().pmgrid; }

// Grid of the drop-in's own short-range pass: PMGRID/4 (cell width 4 mesh
// cells, rcut = 1.4 cells), unless configured.  The forces do not depend on it.
int engine_grid() {
    if (ds().cellgrid > 0) return ds().cellgrid;
    int g = ds().pmgrid / 4;
    return g < 8 ? 8 : g;
}

// ---------------------------------------------------------------- kernels
//
// Each drop-in call applies per-particle operations to P[].  An operation is a
// functor `bool op(PARTICLE &q, uint32_t i, int &endstep)` that returns
// whether it changed q.  It runs on the device mirror in place (k_apply) or on
// the host's P[] through shared memory (k_apply_staged): a CTA reads its
// contiguous run of records with coalesced 16-byte loads, applies the
// operation, and writes the run back whole, with coalesced stores, if any
// record changed.  The host link then carries full 16-byte words in both
// directions at once instead of scattered 4-byte fields.

constexpr int kRecThreads = 256;
constexpr int kRecBytes = kRecThreads * (int)sizeof(PARTICLE);  // 15360 = 960 x 16
static_assert(kRecBytes % 16 == 0, "a CTA's records are whole 16-byte words");

// warp minimum of endstep into *min_end (INT_MAX: nothing to report)
__device__ __forceinline__ void min_endstep(int endstep, int *min_end) {
    const int m = __reduce_min_sync(0xffffffffu, endstep);
    if (min_end && (threadIdx.x & 31) == 0 && m != INT_MAX) atomicMin(min_end, m);
}

template <class Op>
__global__ void __launch_bounds__(kRecThreads) k_apply(PARTICLE *__restrict__ p, uint32_t n, Op op,
                                                      int *__restrict__ min_end) {
    const uint32_t i = blockIdx.x * kRecThreads + threadIdx.x;
    int endstep = INT_MAX;
    if (i < n) op(p[i], i, endstep);
    min_endstep(endstep, min_end);
}

template <class Op>
__global__ void __launch_bounds__(kRecThreads) k_apply_staged(PARTICLE *__restrict__ p, uint32_t n, Op op,
                                                             int *__restrict__ min_end) {
    __shared__ uint4 buf[kRecBytes / 16];
    __shared__ int changed;
    const uint32_t tid = threadIdx.x;
    const uint32_t first = blockIdx.x * kRecThreads;
    const uint32_t cnt = min(n - first, (uint32_t)kRecThreads);
    const uint32_t bytes = cnt * (uint32_t)sizeof(PARTICLE);
    const uint32_t words = bytes / 16, tail = (bytes % 16) / 4;  // whole words, then 4-byte words
    // p is 16-byte aligned (checked by the caller) and first * 60 is a multiple of 16
    uint4 *g = reinterpret_cast<uint4 *>(reinterpret_cast<char *>(p) + (size_t)first * sizeof(PARTICLE));
    for (uint32_t w = tid; w < words; w += kRecThreads) buf[w] = g[w];
    if (tid < tail) reinterpret_cast<uint32_t *>(buf + words)[tid] = reinterpret_cast<const uint32_t *>(g + words)[tid];
    if (tid == 0) changed = 0;
    __syncthreads();
    int endstep = INT_MAX;
    if (tid < cnt && op(reinterpret_cast<PARTICLE *>(buf)[tid], first + tid, endstep)) changed = 1;
    __syncthreads();
    if (changed) {
        for (uint32_t w = tid; w < words; w += kRecThreads) g[w] = buf[w];
        if (tid < tail) reinterpret_cast<uint32_t *>(g + words)[tid] = reinterpret_cast<const uint32_t *>(buf + words)[tid];
    }
    min_endstep(endstep, min_end);
}

// The same streaming from the records at src to those at dst (either may be
// the host's P[] or the device mirror): every record is written to dst,
// changed or not.  compute_accelerations reads P[] once into the mirror and,
// after the forces, writes the mirror's records with their new fields back
// whole, so the host link carries P[] once each way instead of reading it
// again to merge the force fields.
template <class Op>
__global__ void __launch_bounds__(kRecThreads) k_apply_staged_to(const PARTICLE *__restrict__ src,
                                                                PARTICLE *__restrict__ dst, uint32_t n, Op op) {
    __shared__ uint4 buf[kRecBytes / 16];
    const uint32_t tid = threadIdx.x;
    const uint32_t first = blockIdx.x * kRecThreads;
    const uint32_t cnt = min(n - first, (uint32_t)kRecThreads);
    const uint32_t bytes = cnt * (uint32_t)sizeof(PARTICLE);
    const uint32_t words = bytes / 16, tail = (bytes % 16) / 4;
    const uint4 *gs = reinterpret_cast<const uint4 *>(reinterpret_cast<const char *>(src) + (size_t)first * sizeof(PARTICLE));
    uint4 *gd = reinterpret_cast<uint4 *>(reinterpret_cast<char *>(dst) + (size_t)first * sizeof(PARTICLE));
    for (uint32_t w = tid; w < words; w += kRecThreads) buf[w] = gs[w];
    if (tid < tail) reinterpret_cast<uint32_t *>(buf + words)[tid] = reinterpret_cast<const uint32_t *>(gs + words)[tid];
    __syncthreads();
    int endstep = INT_MAX;
    if (tid < cnt) op(reinterpret_cast<PARTICLE *>(buf)[tid], first + tid, endstep);
    __syncthreads();
    for (uint32_t w = tid; w < words; w += kRecThreads) gd[w] = buf[w];
    if (tid < tail) reinterpret_cast<uint32_t *>(gd + words)[tid] = reinterpret_cast<const uint32_t *>(buf + words)[tid];
}

// positions (and velocities) to the engine's float4 arrays
struct UnpackOp {
    float4 *pos, *vel;
    __device__ bool operator()(PARTICLE &q, uint32_t i, int &) const {
        pos[i] = make_float4(q.Pos[0], q.Pos[1], q.Pos[2], 0.f);
        if (vel) vel[i] = make_float4(q.Vel[0], q.Vel[1], q.Vel[2], 0.f);
        return false;
    }
};

enum { kPackPos = 1, kPackVel = 2, kPackPP = 4, kPackPM = 8 };

// engine results into the particle's fields
struct PackOp {
    const float4 *pos, *vel, *app, *apm;
    int what;
    __device__ bool operator()(PARTICLE &q, uint32_t i, int &) const {
        if (what & kPackPos) {
            const float4 v = pos[i];
            q.Pos[0] = v.x, q.Pos[1] = v.y, q.Pos[2] = v.z;
        }
        if (what & kPackVel) {
            const float4 v = vel[i];
            q.Vel[0] = v.x, q.Vel[1] = v.y, q.Vel[2] = v.z;
        }
        if (what & kPackPP) {
            const float4 v = app[i];
            q.GravAccel[0] = v.x, q.GravAccel[1] = v.y, q.GravAccel[2] = v.z;
        }
        if (what & kPackPM) {
            const float4 v = apm[i];
            q.GravPM[0] = v.x, q.GravPM[1] = v.y, q.GravPM[2] = v.z;
        }
        return what != 0;
    }
};

// predict.c:10-41: drift (no wrap) and/or wrap; optionally the resulting
// positions to the engine
struct DriftWrapOp {
    double dt, boxsize;
    int drift, wrap;
    float4 *pos_out;
    __device__ bool operator()(PARTICLE &q, uint32_t i, int &) const {
        float out[3];
        bool ch = false;
        for (int j = 0; j < 3; ++j) {
            const float x0 = q.Pos[j];
            float x = x0;
            if (drift) x = (float)((double)x + (double)q.Vel[j] * dt);
            if (wrap) {
                for (int it = 0; it < 64 && x < 0; ++it) x = (float)((double)x + boxsize);
                for (int it = 0; it < 64 && x >= (float)boxsize; ++it) x = (float)((double)x - boxsize);
            }
            if (__float_as_uint(x) != __float_as_uint(x0)) {
                q.Pos[j] = x;
                ch = true;
            }
            out[j] = x;
        }
        if (pos_out) pos_out[i] = make_float4(out[0], out[1], out[2], 0.f);
        return ch;
    }
};

struct TimestepArgs {
    double fac1, atime, hubble_a, dt_displacement;
    double errtol, softening_table, min_timestep, timebase_interval;
    double loga0, loga1;
    int ti_current;
    int pm_kick;         // PM kick due this call
    double pm_dt;        // its factor
};

__device__ double table_factor(const double *T, double loga0, double loga1, double tbi, int t0,
                               int t1) {
    const int n = CUCO_DRIFT_TABLE_LENGTH;
    double a1 = loga0 + t0 * tbi, a2 = loga0 + t1 * tbi;
    double u1 = (a1 - loga0) / (loga1 - loga0) * n, u2 = (a2 - loga0) / (loga1 - loga0) * n;
    int i1 = (int)u1, i2 = (int)u2;
    if (i1 >= n) i1 = n - 1;
    if (i2 >= n) i2 = n - 1;
    double df1 = i1 < 1 ? u1 * T[0] : T[i1 - 1] + (T[i1] - T[i1 - 1]) * (u1 - i1);
    double df2 = i2 < 1 ? u2 * T[0] : T[i2 - 1] + (T[i2] - T[i2 - 1]) * (u2 - i2);
    return df2 - df1;
}

// timestep.c:26-61 and 86-91 per particle; endstep = Ti_endstep after the
// update, for the scan of find_next_sync_point_and_drift (run.c:35-40).
struct TimestepOp {
    TimestepArgs a;
    const double *kick_table;
    int *flag;  // [0] error, [1] particle, [2] its ti_step
    __device__ bool operator()(PARTICLE &q, uint32_t i, int &endstep) const {
        const int TIMEBASE = CUCO_TIMEBASE;
        int beg = q.Ti_begstep, end = q.Ti_endstep;
        bool bad = false, kicked = false, stepped = false;
        float vel[3] = {q.Vel[0], q.Vel[1], q.Vel[2]};
        if (end == a.ti_current) {
            // get_timestep (timestep.c:96-138)
            double ax = a.fac1 * q.GravAccel[0], ay = a.fac1 * q.GravAccel[1], az = a.fac1 * q.GravAccel[2];
            ax += a.fac1 * q.GravPM[0];
            ay += a.fac1 * q.GravPM[1];
            az += a.fac1 * q.GravPM[2];
            double ac = sqrt(ax * ax + ay * ay + az * az);
            if (ac == 0) ac = 1.0e-30;
            double dt = sqrt(2 * a.errtol * a.atime * a.softening_table / ac);
            dt *= a.hubble_a;
            if (dt >= a.dt_displacement) dt = a.dt_displacement;
            if (dt < a.min_timestep) dt = a.min_timestep;
            int ti_step = (int)(dt / a.timebase_interval);
            if (!(ti_step > 0 && ti_step < TIMEBASE)) {
                if (atomicCAS(&flag[0], 0, 1) == 0) {
                    flag[1] = (int)i;
                    flag[2] = ti_step;
                }
                bad = true;
            } else {
                int ti_min = TIMEBASE;
                while (ti_min > ti_step) ti_min >>= 1;
                ti_step = ti_min;
                if (ti_step > (end - beg)) {
                    if (((TIMEBASE - end) % ti_step) > 0) ti_step = end - beg;
                }
                if (a.ti_current == TIMEBASE) ti_step = 0;
                if ((TIMEBASE - a.ti_current) < ti_step) ti_step = TIMEBASE - a.ti_current;
                const int tstart = (beg + end) / 2;
                const int tend = end + ti_step / 2;
                const double dt_gravkick =
                    table_factor(kick_table, a.loga0, a.loga1, a.timebase_interval, tstart, tend);
                beg = end;
                end = beg + ti_step;
                stepped = true;
                for (int j = 0; j < 3; ++j) vel[j] += (float)(q.GravAccel[j] * dt_gravkick);
                kicked = true;
            }
        }
        if (!bad && a.pm_kick) {
            for (int j = 0; j < 3; ++j) vel[j] = (float)((double)vel[j] + (double)q.GravPM[j] * a.pm_dt);
            kicked = true;
        }
        if (!bad) {
            if (kicked)
                for (int j = 0; j < 3; ++j) q.Vel[j] = vel[j];
            if (stepped) {
                q.Ti_begstep = beg;
                q.Ti_endstep = end;
            }
        }
        endstep = end;
        return !bad && (kicked || stepped);
    }
};

// --------------------------------------------------------------- helpers

cuco_config_t dropin_config() {
    cuco_config_t c{};
    c.n = NumPart;
    c.pm_grid = ds().pmgrid;
    c.cell_grid = engine_grid();
    c.boxsize = All.BoxSize;
    c.mass = header.Mass;
    c.G = All.G;
    c.asmth = All.Asmth;
    c.rcut = All.Rcut;
    c.softening = ds().h > 0 ? (float)ds().h : (All.ForceSoftening > 0 ? All.ForceSoftening : 1.0f);
    c.mode = CUCO_MODE_PLAIN;
    c.device = 0;
    cudaGetDevice(&c.device);
    return c;
}

void ensure_box() {
    DropinState &s = ds();
    if (s.box && s.box_n == NumPart) return;
    if (s.box) cuco_box_destroy(s.box);
    s.box = nullptr;
    cuco_config_t c = dropin_config();
    capi_status(cuco_box_create(&c, &s.box), "drop-in engine set-up");
    s.box_n = NumPart;
    if (s.dP_n < NumPart) {
        cudaFree(s.dP);
        capi_check(cudaMalloc(&s.dP, sizeof(PARTICLE) * (NumPart ? NumPart : 1)), "drop-in P[] mirror");
        s.dP_n = NumPart;
    }
    if (!s.dflag) capi_check(cudaMalloc(&s.dflag, sizeof(int) * 4), "drop-in flag");
}

struct BoxView {
    float4 *pos, *vel, *acc_pp, *acc_pm;
    cudaStream_t stream;
};

}  // namespace

// engine internals the drop-in reaches into (same library, not exported)
extern "C" cuco_status_t cuco_box_internal_arrays(cuco_box_t *b, float4 **pos, float4 **vel,
                                                  float4 **acc_pp, float4 **acc_pm,
                                                  void **stream, uint32_t **keys, uint32_t **perm,
                                                  float4 **spos);

namespace {

BoxView view() {
    BoxView v;
    void *st = nullptr;
    uint32_t *k, *pm;
    float4 *sp;
    cuco_box_internal_arrays(ds().box, &v.pos, &v.vel, &v.acc_pp, &v.acc_pm, &st, &k, &pm, &sp);
    v.stream = (cudaStream_t)st;
    return v;
}

// Whether kernels may read and write the host's P[] in place.  That needs a
// device that accesses pageable host memory coherently (Grace hosts over
// NVLink-C2C, or HMM) and a 16-byte aligned P[] (what malloc returns).
// CUCO_DROPIN_MIRROR=1 forces the mirror path (a full cudaMemcpy of P[] in and
// out around each call) on such devices too.
bool direct_access() {
    DropinState &s = ds();
    if (s.direct < 0) {
        int dev = 0, attr = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&attr, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) attr = 0;
        s.direct = attr == 1 ? 1 : 0;
    }
    const char *env = getenv("CUCO_DROPIN_MIRROR");
    return s.direct == 1 && !(env && env[0] == '1') && ((uintptr_t)P & 15) == 0;
}

// P[] as the kernels of one call see it: the host array itself, or the device
// mirror after a copy of the current P[].
PARTICLE *particles_in() {
    ensure_box();
    DropinState &s = ds();
    if (direct_access()) return P;
    capi_check(cudaMemcpyAsync(s.dP, P, sizeof(PARTICLE) * NumPart, cudaMemcpyHostToDevice, view().stream),
               "P[] upload");
    return (PARTICLE *)s.dP;
}

// Makes the kernels' writes to P[] visible to the host and waits for them.
void particles_out(PARTICLE *pp) {
    DropinState &s = ds();
    BoxView v = view();
    if (pp != P)
        capi_check(cudaMemcpyAsync(P, s.dP, sizeof(PARTICLE) * NumPart, cudaMemcpyDeviceToHost, v.stream),
                   "P[] download");
    capi_check(cudaStreamSynchronize(v.stream), "P[] download");
}

template <class Op>
void apply(PARTICLE *pp, const Op &op, const char *where, int *min_end = nullptr) {
    if (!NumPart) return;
    BoxView v = view();
    const unsigned blocks = (NumPart + kRecThreads - 1) / kRecThreads;
    if (pp == P)
        k_apply_staged<<<blocks, kRecThreads, 0, v.stream>>>(pp, NumPart, op, min_end);
    else
        k_apply<<<blocks, kRecThreads, 0, v.stream>>>(pp, NumPart, op, min_end);
    capi_check(cudaGetLastError(), where);
}

void unpack(PARTICLE *pp, bool with_vel) {
    BoxView v = view();
    apply(pp, UnpackOp{v.pos, with_vel ? v.vel : nullptr}, "P[] unpack");
}

void pack(PARTICLE *pp, int what) {
    BoxView v = view();
    apply(pp, PackOp{v.pos, v.vel, v.acc_pp, v.acc_pm, what}, "P[] pack");
}

void drift_wrap(PARTICLE *pp, double dt, bool drift, bool wrap, bool to_engine = false) {
    BoxView v = view();
    apply(pp, DriftWrapOp{dt, (double)All.BoxSize, drift ? 1 : 0, wrap ? 1 : 0, to_engine ? v.pos : nullptr},
          "drift/wrap");
}

}  // namespace

extern "C" cuco_status_t cuco_box_mark_state(cuco_box_t *b);


extern "C" {

void cuco_dropin_configure(int pmgrid, int cellgrid) {
    if (pmgrid < 8 || (pmgrid & (pmgrid - 1)) || pmgrid > 1024) capi_fail("cuco_dropin_configure", "pmgrid must be a power of two in [8, 1024]");
    ds().pmgrid = pmgrid;
    ds().cellgrid = cellgrid;
    capi_set_grid(cell_grid());
}

// read_ic.c:9-45: HEADER then PARTICLE[NumPart] into the globals; exits on a
// missing or short file as the reference does (it does not check fread).
void read_ic(char *fname) {
    FILE *fp = fopen(fname, "rb");
    if (!fp) {
        printf("Cannot open initial condition file %s!\n", fname);
        exit(1);
    }
    HEADER h;
    if (fread(&h, sizeof(HEADER), 1, fp) != 1 || h.NumPart < 0) {
        printf("Initial condition file %s has no valid header!\n", fname);
        exit(1);
    }
    header = h;
    NumPart = (unsigned)h.NumPart;
    P = (PARTICLE *)malloc(sizeof(PARTICLE) * (NumPart ? NumPart : 1));
    if (!P || fread(P, sizeof(PARTICLE), NumPart, fp) != NumPart) {
        printf("Initial condition file %s ends before its %u particles!\n", fname, NumPart);
        exit(1);
    }
    fclose(fp);
    All.NumPart = (int)NumPart;
    All.BoxSize = header.BoxSize;
    All.Mass = header.Mass;
    printf("IC file %s: %u particles, box %g kpc/h, mass %g x 1e10 Msun/h, z = %g\n", fname, NumPart,
           header.BoxSize, header.Mass, header.Redshift);
}

// io.c:9-40: <OutputDir>/<SnapshotFileBase>_<num>.cuco with the header's
// time and redshift from All.Time.
void savepositions(int num) {
    char path[2 * CUCO_MAXLEN_FILENAME + 32];
    snprintf(path, sizeof path, "%s/%s_%d.cuco", All.OutputDir, All.SnapshotFileBase, num);
    FILE *fp = fopen(path, "wb");
    if (!fp) {
        printf("Cannot open snapshot file %d!\n", num);
        exit(1);
    }
    HEADER h = header;
    h.Time = All.Time;
    h.Redshift = 1 / All.Time - 1;
    if (fwrite(&h, sizeof(HEADER), 1, fp) != 1 || fwrite(P, sizeof(PARTICLE), NumPart, fp) != NumPart) {
        printf("Cannot write snapshot file %d!\n", num);
        exit(1);
    }
    fclose(fp);
    printf("write output file %d: a = %g z = %g\n", num, All.Time, h.Redshift);
}

void pm_init_periodic(void) {
    All.Asmth = (float)(CUCO_ASMTH * (double)All.BoxSize / ds().pmgrid);
    All.Rcut = (float)(CUCO_RCUT * (double)All.Asmth);
    capi_set_grid(cell_grid());
}

void long_range_init(void) { pm_init_periodic(); }

void pm_init_periodic_allocate(void) { ensure_box(); }

void pm_init_periodic_free(void) {}

void pmforce_periodic(void) {
    PARTICLE *pp = particles_in();
    unpack(pp, false);
    cuco_box_mark_state(ds().box);
    capi_status(cuco_box_forces(ds().box, 1, 0), "pmforce_periodic");
    pack(pp, kPackPM);
    particles_out(pp);
}

void long_range_force(void) { pmforce_periodic(); }

void set_softenings(void) {
    if (All.SofteningHalo * All.Time > All.SofteningHaloMaxPhys)
        All.SofteningTable = All.SofteningHaloMaxPhys / All.Time;
    else
        All.SofteningTable = All.SofteningHalo;
    All.ForceSoftening = (float)(2.8 * All.SofteningTable);
    DropinState &s = ds();
    s.h = All.ForceSoftening;
    s.h_inv = 1.0 / s.h;
    s.h3_inv = s.h_inv * s.h_inv * s.h_inv;
    s.soft.h = (float)s.h;
    s.soft.h_inv = (float)s.h_inv;
    s.soft.h3_inv = (float)s.h3_inv;
    if (s.box) cuco_box_set_softening(s.box, s.soft.h);
}

void linklist_init(void) {
    DropinState &s = ds();
    SIMPARAM sim;
    shortrange_table(sim.shortrange_table);
    const int G = cell_grid();
    double to_grid_fac = (float)G / All.BoxSize;
    sim.boxsize = All.BoxSize;
    sim.boxhalf = (float)(All.BoxSize / 2.0);
    sim.to_grid_fac = (float)to_grid_fac;
    sim.rcut = All.Rcut;
    sim.rcut2 = (float)((double)All.Rcut * All.Rcut);
    sim.asmth = All.Asmth;
    sim.asmthfac = (float)(0.5 / (double)All.Asmth * (CUCO_NTAB / 3.0));
    sim.mass = header.Mass;
    sim.G = (float)All.G;
    numParticles = NumPart;
    numGridCells = (unsigned)G * G * G;
    delete sorter;
    sorter = new RadixSort(numParticles);
    if (s.h <= 0) set_softenings();
    ensure_box();
    float4 *pos, *vel, *app, *apm, *spos;
    uint32_t *keys, *perm;
    void *st;
    cuco_box_internal_arrays(s.box, &pos, &vel, &app, &apm, &st, &keys, &perm, &spos);
    dOldPos = (float *)pos;
    dSortedPos = (float *)spos;
    dGravAccel = (float *)app;
    dGridParticleHash = keys;
    dGridParticleIndex = perm;
    setSimParam(&sim);
}

void copyPosToDevice(void) {
    unpack(particles_in(), false);
    capi_check(cudaStreamSynchronize(view().stream), "copyPosToDevice");
}

void copyAccelFromDevice(void) {
    PARTICLE *pp = particles_in();
    pack(pp, kPackPP);
    particles_out(pp);
}

void gravity_linklist_cuda(void) {
    set_softenings();
    PARTICLE *pp = particles_in();
    unpack(pp, false);
    cuco_box_mark_state(ds().box);
    capi_status(cuco_box_forces(ds().box, 0, 1), "gravity_linklist_cuda");
    pack(pp, kPackPP);
    particles_out(pp);
}

void do_box_wrapping(void) {
    PARTICLE *pp = particles_in();
    drift_wrap(pp, 0.0, false, true);
    particles_out(pp);
}

void move_particles(int time0, int time1) {
    double dt = get_drift_factor(time0, time1);
    PARTICLE *pp = particles_in();
    drift_wrap(pp, dt, true, false);
    particles_out(pp);
}

void compute_accelerations(void) {
    set_softenings();
    PARTICLE *pp = particles_in();
    const int pm = All.PM_Ti_endstep == All.Ti_Current;
    if (pp == P && NumPart) {
        // P[] in place: one read of the records into the mirror (wrapped,
        // positions to the engine), the forces, one write of the records back
        DropinState &s = ds();
        BoxView v = view();
        const unsigned blocks = (NumPart + kRecThreads - 1) / kRecThreads;
        k_apply_staged_to<<<blocks, kRecThreads, 0, v.stream>>>(
            P, (PARTICLE *)s.dP, NumPart, DriftWrapOp{0.0, (double)All.BoxSize, 0, 1, v.pos});
        capi_check(cudaGetLastError(), "compute_accelerations");
        cuco_box_mark_state(s.box);
        capi_status(cuco_box_forces(s.box, pm, 1), "compute_accelerations");
        k_apply_staged_to<<<blocks, kRecThreads, 0, v.stream>>>(
            (const PARTICLE *)s.dP, P, NumPart, PackOp{v.pos, v.vel, v.acc_pp, v.acc_pm, kPackPP | (pm ? kPackPM : 0)});
        capi_check(cudaGetLastError(), "compute_accelerations");
        particles_out(pp);
        return;
    }
    drift_wrap(pp, 0.0, false, true, true);  // wrap, and the positions to the engine
    cuco_box_mark_state(ds().box);
    capi_status(cuco_box_forces(ds().box, pm, 1), "compute_accelerations");
    pack(pp, kPackPP | (pm ? kPackPM : 0));
    particles_out(pp);
}

int get_timestep(int p) {
    double fac1 = 1 / (All.Time * All.Time);
    double atime = All.Time;
    double hubble_a = All.Omega0 / (atime * atime * atime) +
                      (1 - All.Omega0 - All.OmegaLambda) / (atime * atime) + All.OmegaLambda;
    hubble_a = All.Hubble * sqrt(hubble_a);
    double ax = fac1 * P[p].GravAccel[0], ay = fac1 * P[p].GravAccel[1], az = fac1 * P[p].GravAccel[2];
    ax += fac1 * P[p].GravPM[0];
    ay += fac1 * P[p].GravPM[1];
    az += fac1 * P[p].GravPM[2];
    double ac = sqrt(ax * ax + ay * ay + az * az);
    if (ac == 0) ac = 1.0e-30;
    double dt = sqrt(2 * All.ErrTolIntAccuracy * atime * All.SofteningTable / ac);
    dt *= hubble_a;
    if (dt >= All.MaxSizeTimestep) dt = All.MaxSizeTimestep;
    if (dt < All.MinSizeTimestep) {
        printf("warning: Timestep will be below the limit of MinSizeTimestep!\n");
        dt = All.MinSizeTimestep;
    }
    int ti_step = (int)(dt / All.Timebase_interval);
    if (!(ti_step > 0 && ti_step < CUCO_TIMEBASE)) {
        printf("Error: a timestep of size zero was assigned on the integer timeline!\n");
        printf("ti_step: %d\n", ti_step);
        exit(1);
    }
    return ti_step;
}

void advance_and_find_timesteps(void) {
    DropinState &s = ds();
    if (!s.tables) init_drift_table();
    if (!s.dtab_valid) {
        const size_t bytes = sizeof(double) * CUCO_DRIFT_TABLE_LENGTH;
        if (!s.dtab) capi_check(cudaMalloc(&s.dtab, bytes), "advance_and_find_timesteps");
        capi_check(cudaMemcpy(s.dtab, s.kick64, bytes, cudaMemcpyHostToDevice), "advance_and_find_timesteps");
        s.dtab_valid = true;
    }
    PARTICLE *pp = particles_in();
    BoxView v = view();
    TimestepArgs a;
    a.fac1 = 1 / (All.Time * All.Time);
    a.atime = All.Time;
    double h = All.Omega0 / (a.atime * a.atime * a.atime) +
               (1 - All.Omega0 - All.OmegaLambda) / (a.atime * a.atime) + All.OmegaLambda;
    a.hubble_a = All.Hubble * sqrt(h);
    a.dt_displacement = All.MaxSizeTimestep;
    a.errtol = All.ErrTolIntAccuracy;
    a.softening_table = All.SofteningTable;
    a.min_timestep = All.MinSizeTimestep;
    a.timebase_interval = All.Timebase_interval;
    a.loga0 = s.logTimeBegin;
    a.loga1 = s.logTimeMax;
    a.ti_current = All.Ti_Current;
    a.pm_kick = 0;
    a.pm_dt = 0;
    // global PM step (timestep.c:63-93), scalar on the host
    if (All.PM_Ti_endstep == All.Ti_Current) {
        int ti_step = CUCO_TIMEBASE;
        while (ti_step > (a.dt_displacement / All.Timebase_interval)) ti_step >>= 1;
        if (ti_step > (All.PM_Ti_endstep - All.PM_Ti_begstep)) {
            if (((CUCO_TIMEBASE - All.PM_Ti_endstep) % ti_step) > 0)
                ti_step = All.PM_Ti_endstep - All.PM_Ti_begstep;
        }
        if (All.Ti_Current == CUCO_TIMEBASE) ti_step = 0;
        int tstart = (All.PM_Ti_begstep + All.PM_Ti_endstep) / 2;
        int tend = All.PM_Ti_endstep + ti_step / 2;
        a.pm_dt = get_gravkick_factor(tstart, tend);
        a.pm_kick = 1;
        All.PM_Ti_begstep = All.PM_Ti_endstep;
        All.PM_Ti_endstep = All.PM_Ti_begstep + ti_step;
    }
    capi_check(cudaMemsetAsync(s.dflag, 0, sizeof(int) * 3, v.stream), "timesteps");
    capi_check(cudaMemsetAsync(s.dflag + 3, 0x7f, sizeof(int), v.stream), "timesteps");
    apply(pp, TimestepOp{a, s.dtab, s.dflag}, "advance_and_find_timesteps", s.dflag + 3);
    int flag[4];
    capi_check(cudaMemcpyAsync(flag, s.dflag, sizeof(flag), cudaMemcpyDeviceToHost, v.stream), "timesteps");
    particles_out(pp);
    s.min_endstep = flag[3];
    s.min_valid = NumPart > 0 && !flag[0];
    s.min_P = P;
    s.min_n = NumPart;
    if (flag[0]) {
        printf("Error: a timestep of size zero was assigned on the integer timeline!\n");
        printf("ti_step: %d\n", flag[2]);
        printf("timebase interval: %g\n", All.Timebase_interval);
        printf("particle: %d\n", flag[1]);
        exit(1);
    }
}

int cuco_dropin_host_access(void) {
    ensure_box();
    return direct_access() ? 1 : 0;
}

int cuco_dropin_min_ti_endstep(void) {
    DropinState &s = ds();
    if (s.min_valid && s.min_P == P && s.min_n == NumPart) return s.min_endstep;
    // the host scan of find_next_sync_point_and_drift (run.c:35-40)
    int m = NumPart ? P[0].Ti_endstep : 0;
    for (unsigned i = 1; i < NumPart; ++i)
        if (P[i].Ti_endstep < m) m = P[i].Ti_endstep;
    return m;
}

double drift_integ(double a, void *param) {
    (void)param;
    double h = All.Omega0 / (a * a * a) + (1 - All.Omega0 - All.OmegaLambda) / (a * a) + All.OmegaLambda;
    h = All.Hubble * sqrt(h);
    return 1 / (h * a * a * a);
}

double gravkick_integ(double a, void *param) {
    (void)param;
    double h = All.Omega0 / (a * a * a) + (1 - All.Omega0 - All.OmegaLambda) / (a * a) + All.OmegaLambda;
    h = All.Hubble * sqrt(h);
    return 1 / (h * a * a);
}

void init_drift_table(void) {
    DropinState &s = ds();
    // in C the float argument is promoted to double (driftfac.c:23-24); C++
    // would pick the float overload of log
    s.logTimeBegin = log((double)All.TimeBegin);
    s.logTimeMax = log((double)All.TimeMax);
    const int n = CUCO_DRIFT_TABLE_LENGTH;
    double a0 = exp(s.logTimeBegin);
    for (int i = 0; i < n; ++i) {
        double a1 = exp(s.logTimeBegin + ((s.logTimeMax - s.logTimeBegin) / n) * (i + 1));
        s.drift64[i] = cosmo_integral(a0, a1, All.Omega0, All.OmegaLambda, All.Hubble, 3);
        s.kick64[i] = cosmo_integral(a0, a1, All.Omega0, All.OmegaLambda, All.Hubble, 2);
        DriftTable[i] = (float)s.drift64[i];
        GravKickTable[i] = (float)s.kick64[i];
    }
    s.tables = true;
    s.dtab_valid = false;  // uploaded by the next advance_and_find_timesteps
}

static double host_table_factor(const double *T, int t0, int t1) {
    DropinState &s = ds();
    const int n = CUCO_DRIFT_TABLE_LENGTH;
    double a1 = s.logTimeBegin + t0 * All.Timebase_interval;
    double a2 = s.logTimeBegin + t1 * All.Timebase_interval;
    double u1 = (a1 - s.logTimeBegin) / (s.logTimeMax - s.logTimeBegin) * n;
    double u2 = (a2 - s.logTimeBegin) / (s.logTimeMax - s.logTimeBegin) * n;
    int i1 = (int)u1, i2 = (int)u2;
    if (i1 >= n) i1 = n - 1;
    if (i2 >= n) i2 = n - 1;
    double df1 = i1 < 1 ? u1 * T[0] : T[i1 - 1] + (T[i1] - T[i1 - 1]) * (u1 - i1);
    double df2 = i2 < 1 ? u2 * T[0] : T[i2 - 1] + (T[i2] - T[i2 - 1]) * (u2 - i2);
    return df2 - df1;
}

double get_drift_factor(int time0, int time1) {
    if (!ds().tables) init_drift_table();
    return host_table_factor(ds().drift64, time0, time1);
}

double get_gravkick_factor(int time0, int time1) {
    if (!ds().tables) init_drift_table();
    return host_table_factor(ds().kick64, time0, time1);
}

}  // extern "C"
