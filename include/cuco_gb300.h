/* cuco_gb300.h - C ABI of libcuco_gb300.so, the GB300 (sm_103a) force engine.
 *
 * Two groups of entry points:
 *
 * 1. The reference's own names and signatures (liulei/cuco), so that its host
 *    program links against this library in place of gravlist.cu, radixsort.cu,
 *    gravlist.cpp, pm_periodic.c, longrange.c, accel.c, predict.c, timestep.c
 *    and driftfac.c.  Each declaration cites the reference function it
 *    replaces.  The GPU-side helpers take plain device pointers and sizes; the
 *    host-side force/integrator functions work on the reference's globals
 *    (P, NumPart, All, header, DriftTable, GravKickTable), which the host
 *    program defines (allvars.c) - the library carries weak fallbacks of them.
 *    As in the reference these functions return void and abort on a CUDA error
 *    (cutilSafeCall semantics); the message is printed first.
 *
 * 2. The engine API (cuco_*): one resident simulation box per handle, status
 *    returns, explicit configuration, host or device buffers.  The drop-in
 *    functions are built on it.
 *
 * Device state stays resident between calls; nothing is copied between host
 * and device except where a function says so. */
#ifndef CUCO_GB300_H
#define CUCO_GB300_H

#include <stddef.h>
#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#include "cuco_allvars.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned int uint;
typedef size_t CUDPPHandle; /* accepted and ignored: the sort needs no CUDPP plan */

/* ------------------------------------------------------------------------
 * 1a. GPU-side helpers of gravlist.cu and radixsort.cu (reference names)
 * ---------------------------------------------------------------------- */

/* gravlist.cu:25-31.  Selects device 0 (CUCO_DEVICE overrides). */
void cudaInit(void);
/* gravlist.cu:33-37 */
void allocateArray(void **devPtr, size_t size);
/* gravlist.cu:39-43 */
void freeArray(void *devPtr);
/* gravlist.cu:45-49 */
void copyArrayFromDevice(void *host, void *device, int size);
/* gravlist.cu:51-54 */
void copyArrayToDevice(void *device, void *host, int offset, int size);
/* gravlist.cu:173-177: table, box, cut and mass constants for the kernels below */
void setSimParam(SIMPARAM *pHostSimParam);
/* gravlist.cu:179-181: spline softening constants */
void setSoftParam(SOFTPARAM *pHostSoftParam);
/* gravlist.cu:56-68: P[i].Pos -> dOldPos (float4) */
void copyPosToDevice(void);
/* gravlist.cu:70-83: dGravAccel (float4) -> P[i].GravAccel */
void copyAccelFromDevice(void);

/* gravlist.cu:85-104 + gravlist_kernel.cu:92-118.  Cell key of each particle on
 * a G^3 grid, G = cbrt of the cell count last set by setSimParam's
 * to_grid_fac and cuco_dropin_configure (64 by default):
 * key = (ix*G+iy)*G+iz, i = (int)(to_grid_fac*p) in float32; index = i.
 * Unlike the reference every particle is keyed for any numParticles, and a
 * coordinate whose product rounds to G is clamped to cell G-1. */
void calcHash(uint *gridParticleHash, uint *gridParticleIndex, float *pos, uint numParticles);

/* gravlist.cu:108-142 + gravlist_kernel.cu:121-160.  cellStart[c] = first
 * sorted index of cell c (0xffffffff when empty), cellEnd[c] = one past the
 * last; sortedPos[i] = oldPos[gridParticleIndex[i]] (float4). */
void reorderDataAndFindCellStart(uint *cellStart, uint *cellEnd, float *sortedPos,
                                 uint *gridParticleHash, uint *gridParticleIndex,
                                 float *oldPos, uint numParticles, uint numCells);

/* gravlist.cu:144-171 + gravlist_kernel.cu:20-88,162-234.  Short-range P3M
 * force on every sorted particle from all particles within rcut, with the
 * constants of setSimParam/setSoftParam; gravAccel[gridParticleIndex[i]] =
 * (ax, ay, az, 0).  numCells = G^3 of the grid the keys were made on. */
void cudaForceEvaluateShortrange(float *gravAccel, float *sortedPos, uint *gridParticleIndex,
                                 uint *cellStart, uint *cellEnd, uint numParticles,
                                 uint numCells);

/* radixsort.h:47-58 / radixsort.cu:1048-1145.  Stable LSD sort of
 * (keys, values) by the low keyBits bits, in place.  Every key must be below
 * 2^keyBits: the passes split keyBits into equal digits of 4 to 6 bits
 * (18 bits: three 6-bit passes; 1 bit: one 4-bit pass), which may cover a few
 * bits above keyBits, and bits set there would take part in the order (the
 * reference's CUDPP sort makes the same assumption).  tempKeys/tempValues hold numElements
 * entries each; `counters` holds at least 32*ceil(n/1024) entries (the
 * reference RadixSort's allocation, radixsort.h:271-275) and is used as the
 * per-tile digit histogram; countersSum, blockOffsets and scanPlan are not
 * used.  flipBits must be false. */
void radixSort(uint *keys, uint *values, uint *tempKeys, uint *tempValues, uint *counters,
               uint *countersSum, uint *blockOffsets, CUDPPHandle scanPlan, uint numElements,
               uint keyBits, bool flipBits);
/* radixsort.h:73-81: key-only variant of radixSort. */
void radixSortKeysOnly(uint *keys, uint *tempKeys, uint *counters, uint *countersSum,
                       uint *blockOffsets, CUDPPHandle scanPlan, uint numElements,
                       uint keyBits, bool flipBits);
/* radixsort.h:60-71, 83-92: float keys.  With negativeKeys the keys are
 * mapped to order-preserving unsigned integers before the sort (sign bit set:
 * all bits inverted; else the sign bit set) and mapped back after it; without
 * it non-negative floats already order as their bit patterns.  The sort is
 * radixSort's over the low keyBits bits of the mapped keys (32 for a full
 * float order). */
void radixSortFloatKeys(float *keys, uint *values, float *tempKeys, uint *tempValues, uint *counters,
                        uint *countersSum, uint *blockOffsets, CUDPPHandle scanPlan, uint numElements,
                        uint keyBits, bool negativeKeys);
void radixSortFloatKeysOnly(float *keys, float *tempKeys, uint *counters, uint *countersSum,
                            uint *blockOffsets, CUDPPHandle scanPlan, uint numElements, uint keyBits,
                            bool negativeKeys);
/* No counterpart in the reference (whose RadixSort::sort does not check its
 * capacity): RadixSort::sort calls this, which prints a message and exits,
 * when asked to sort more elements than the object was created for. */
void cuco_radixsort_overflow(uint numElements, uint maxElements);
/* radixsort.h:47: no device-specific tuning is needed on sm_103a; kept for linkage. */
void initDeviceParameters(void);
/* radixsort.h:46: aborts with `msg` if a CUDA error is pending. */
void checkCudaError(const char *msg);

/* ------------------------------------------------------------------------
 * 1b. Host force / integrator functions over the reference's globals
 * ---------------------------------------------------------------------- */

/* Mesh size PMGRID (allvars.h:9) and short-range cell grid of the drop-in.
 * The reference fixes both at compile time (G = PMGRID); call before
 * pm_init_periodic().  Defaults: pmgrid 64, cellgrid = pmgrid. */
void cuco_dropin_configure(int pmgrid, int cellgrid);

/* longrange.c:8-12 */
void long_range_init(void);
/* longrange.c:14-22: zero GravPM, then pmforce_periodic() */
void long_range_force(void);
/* pm_periodic.c:25-43: All.Asmth, All.Rcut; mesh buffers */
void pm_init_periodic(void);
/* pm_periodic.c:45-65 (mesh buffers live on the device and are kept) */
void pm_init_periodic_allocate(void);
void pm_init_periodic_free(void);
/* pm_periodic.c:67-314: P[i].GravPM for every particle, on the device */
void pmforce_periodic(void);
/* gravlist.cpp:28-45 */
void set_softenings(void);
/* gravlist.cpp:48-115: split table, device arrays, SIMPARAM */
void linklist_init(void);
/* gravlist.cpp:148-193: P[i].GravAccel for every particle, on the device */
void gravity_linklist_cuda(void);
/* accel.c:8-23 */
void compute_accelerations(void);
/* predict.c:10-22 */
void move_particles(int time0, int time1);
/* predict.c:24-41 */
void do_box_wrapping(void);
/* timestep.c:11-94 */
void advance_and_find_timesteps(void);
/* timestep.c:96-138 */
int get_timestep(int p);
/* No counterpart in the reference.  min over P[i].Ti_endstep: the scan that
 * find_next_sync_point_and_drift does on the host (run.c:35-40).  Right after
 * advance_and_find_timesteps it returns the minimum that call computed on the
 * device, without reading P[]; otherwise (or when P / NumPart changed since)
 * it scans P[] on the host as run.c does.  A host that writes Ti_endstep
 * itself must call it only before its own writes or after the next
 * advance_and_find_timesteps. */
int cuco_dropin_min_ti_endstep(void);
/* No counterpart in the reference.  1 when the drop-in's kernels read and
 * write the host's P[] in place (the device accesses pageable host memory
 * coherently, e.g. a Grace host over NVLink-C2C, and CUCO_DROPIN_MIRROR is not
 * "1"); 0 when each call copies P[] whole to a device mirror and back. */
int cuco_dropin_host_access(void);
/* read_ic.c:9-45: HEADER then PARTICLE[NumPart] of an IC file into header, P
 * (malloc'ed here), NumPart and All.NumPart/BoxSize/Mass; exits on a missing
 * or short file. */
void read_ic(char *fname);
/* io.c:9-40: header (with Time = All.Time, Redshift = 1/All.Time - 1) and
 * P[0..NumPart) to <All.OutputDir>/<All.SnapshotFileBase>_<num>.cuco. */
void savepositions(int num);
/* driftfac.c:14-42 (tables integrated in FP64; the float tables DriftTable /
 * GravKickTable are filled too) */
void init_drift_table(void);
/* driftfac.c:44-64 */
double drift_integ(double a, void *param);
double gravkick_integ(double a, void *param);
/* driftfac.c:66-126 */
double get_drift_factor(int time0, int time1);
double get_gravkick_factor(int time0, int time1);

/* ------------------------------------------------------------------------
 * 2. Engine API
 * ---------------------------------------------------------------------- */

typedef enum {
    CUCO_OK = 0,
    CUCO_ERR_INVALID = 1,     /* bad argument or configuration */
    CUCO_ERR_NOMEM = 2,       /* device allocation failed */
    CUCO_ERR_CUDA = 3,        /* a CUDA call failed; see cuco_last_error() */
    CUCO_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
    CUCO_ERR_STATE = 5,       /* call out of order (e.g. no state uploaded) */
    CUCO_ERR_UNSUPPORTED = 6  /* configuration the library does not handle */
} cuco_status_t;

typedef enum {
    CUCO_MODE_PLAIN = 0, /* float32 positions, the reference's arithmetic */
    CUCO_MODE_FIXED = 1  /* uint32 fixed-point positions, compensated sums */
} cuco_mode_t;

typedef struct {
    int64_t n;        /* particles */
    int pm_grid;      /* PM mesh size M (even, 8..1024, no prime factor above 5) */
    int cell_grid;    /* short-range cell grid G (cell width >= rcut/2) */
    float boxsize;    /* L, internal length units */
    float mass;       /* particle mass */
    double G;         /* gravitational constant, internal units */
    float asmth;      /* split scale r_s (All.Asmth), length units */
    float rcut;       /* short-range cutoff (All.Rcut), length units */
    float softening;  /* spline softening length h = 2.8 eps (All.ForceSoftening) */
    int mode;         /* cuco_mode_t */
    int device;       /* CUDA device ordinal */
} cuco_config_t;

typedef struct cuco_box cuco_box_t;

/* Fill `cfg` with the reference's derived constants for a box:
 * asmth = ASMTH*L/M and rcut = RCUT*asmth rounded to float as pm_periodic.c:27-28
 * stores them; cell_grid = M/4 (cell width 4 mesh cells, rcut = 1.4 cells)
 * unless already set.  Any cell grid with rcut <= 8 cell widths gives the
 * same forces; the reference's own grid is cell_grid = M. */
cuco_status_t cuco_config_reference(cuco_config_t *cfg);

cuco_status_t cuco_box_create(const cuco_config_t *cfg, cuco_box_t **box);
cuco_status_t cuco_box_destroy(cuco_box_t *box);

/* State in original particle order, n x 3 floats each.  `on_device` selects
 * whether the pointers are device (1) or host (0) memory.  vel is the
 * integrator's variable a^2 dx/dt (the reference's P[].Vel after init.c:30). */
cuco_status_t cuco_box_set_state(cuco_box_t *box, const float *pos, const float *vel,
                                 int on_device);
cuco_status_t cuco_box_get_state(cuco_box_t *box, float *pos, float *vel, float *acc_pp,
                                 float *acc_pm, int on_device);
/* CUCO_MODE_FIXED boxes only: positions as uint32 x,y,z per particle in units
 * of boxsize / 2^32 (exact; cuco_box_set_state converts floats by rounding to
 * that grid, cuco_box_get_state rounds back to float). */
cuco_status_t cuco_box_set_state_fixed(cuco_box_t *box, const uint32_t *pos, const float *vel,
                                       int on_device);
cuco_status_t cuco_box_get_state_fixed(cuco_box_t *box, uint32_t *pos, int on_device);
/* The reference's IC/snapshot file format (read_ic.c:9-45, io.c:9-40): HEADER
 * then PARTICLE[NumPart], raw.  load: the file's NumPart must equal the box's
 * n; positions and velocities become the box's state (with
 * initial_conditions != 0 the velocities are scaled by Time^(3/2) into the
 * integrator's variable, as init.c:30 does for an IC file; a snapshot stores
 * that variable already); the header is returned when `header` is not NULL.
 * save: writes `header` (NumPart set to n) and one record per particle with
 * Pos, Vel, Mass = header->Mass, GravAccel = the last short-range force,
 * GravPM = the last PM force, Ti_endstep = Ti_begstep = 0 (the engine keeps
 * no individual timeline).  Both go through device memory they allocate for
 * the call. */
cuco_status_t cuco_box_load_snapshot(cuco_box_t *box, const char *path, int initial_conditions,
                                     HEADER *header);
cuco_status_t cuco_box_save_snapshot(cuco_box_t *box, const char *path, const HEADER *header);

/* Spline softening length h (changes with time when softening is physical). */
cuco_status_t cuco_box_set_softening(cuco_box_t *box, float h);

/* Forces at the current positions: keys, sort, reorder, then the PM force
 * (when pm != 0) and the short-range force (when pp != 0). */
cuco_status_t cuco_box_forces(cuco_box_t *box, int pm, int pp);

/* One step of the leapfrog in the reference's kick-drift-kick form (run.c:11-20
 * with timestep.c:26-93 for a global step): positions drift by `drift` and wrap,
 * forces are recomputed, velocities kick by acc_pp*kick_pp + acc_pm*kick_pm.
 * The factors are cosmological integrals (cuco_cosmo_factors). */
cuco_status_t cuco_box_step(cuco_box_t *box, double drift, double kick_pp, double kick_pm);

/* Run `nsteps` steps with per-step factors (arrays of nsteps), enqueued
 * back to back on the box's stream. */
cuco_status_t cuco_box_run(cuco_box_t *box, int nsteps, const double *drift,
                           const double *kick_pp, const double *kick_pm);

cuco_status_t cuco_box_sync(cuco_box_t *box);
/* No counterpart in the reference.  Exercises the short range's timeout
 * path without a fault: one CTA waits, at most `seconds` (<= 1), on a staging
 * barrier that is armed for copies never issued, gives up, and sets the
 * box's timeout word; the call then returns CUCO_ERR_TIMEOUT as cuco_box_sync
 * would after a real staging wait gave up, and clears the word.  The box
 * stays usable. */
cuco_status_t cuco_box_selftest_timeout(cuco_box_t *box, double seconds);
/* No counterpart in the reference.  In a debug build of the library
 * (libcuco_gb300_debug.so, compiled with CUCO_BOUNDS_CHECK) the kernels check
 * the index of their main memory accesses (sort scatter, cell order, deposit,
 * interpolation, short-range staging and source reads); a failed check is
 * counted and the access clamped in bounds.  Waits for the device, returns
 * the count since the last call in *count and resets it.  A release build
 * returns CUCO_ERR_UNSUPPORTED. */
cuco_status_t cuco_debug_bounds_violations(uint64_t *count);
/* The box's CUDA stream (cudaStream_t).  Every pass is ordered on it: the
 * PM's second stream forks from it after the keys and joins it again after
 * the short range (whose last CTAs it runs behind the PM), so work enqueued
 * on this stream before or after a pass is ordered with all of the pass. */
cuco_status_t cuco_box_stream(cuco_box_t *box, void **stream);

/* Device time (ms) of each phase of the last cuco_box_forces/cuco_box_step:
 * [0] drift+keys, [1] sort, [2] reorder (cell bounds and z-slice order),
 * [3] PM deposit, [4] PM FFT+Green, [5] PM gradient+interpolation,
 * [6] short range (with the PP half of the kick), [7] total.  The PM runs on
 * a second stream from the end of [0], beside the sort, the reorder and the
 * start of the short range, whose last CTAs it runs after itself; [6] spans
 * the short range's whole launch, from the end of [2] until both of its
 * parts are done.  [0] + [1] + [2] + [6] + the PM half of the kick (after
 * [6]) is [7].  Only filled when phase timing is enabled. */
cuco_status_t cuco_box_enable_timing(cuco_box_t *box, int enable);
cuco_status_t cuco_box_timings(cuco_box_t *box, float *ms /* 8 */);
/* Sums of the phase times since timing was enabled (or the last reset).  A
 * timed step does not wait for itself, only for the step before, so a run of
 * timed steps keeps the GPU busy; this call waits for the last one. */
cuco_status_t cuco_box_phase_totals(cuco_box_t *box, float *ms /* 8 */, int reset);

/* Copies of internal arrays for inspection (device -> host): keys and the
 * sort permutation in sorted order, cell bounds.  Any pointer may be NULL. */
cuco_status_t cuco_box_debug(cuco_box_t *box, uint32_t *sorted_keys, uint32_t *perm,
                             uint32_t *cell_start, uint32_t *cell_end);

/* The order the short range reads its sources in (no counterpart in the
 * reference): the sort's cells, each refined by z slice (8 slices of the cell
 * along z, stable within a slice).  perm_s[i] is the original index of the
 * i-th particle in that order, slice[i] its slice.  Either pointer may be NULL. */
cuco_status_t cuco_box_cell_order(cuco_box_t *box, uint32_t *perm_s, float *slice);

/* Number of kernel launches one cuco_box_step issues. */
int cuco_box_launches_per_step(cuco_box_t *box);

/* In-range pair count (r^2 <= rcut^2, self excluded) of the short-range
 * launches since the last reset, counted only while cuco_box_count_pairs is
 * enabled (the counting kernel is slightly slower; no counterpart in the
 * reference). */
cuco_status_t cuco_box_count_pairs(cuco_box_t *box, int enable);
cuco_status_t cuco_box_pair_count(cuco_box_t *box, uint64_t *pairs, int reset);

/* Device-time bracket on the box's stream: op 0 records the start event,
 * op 1 records the stop event, waits for it and returns the elapsed ms. */
cuco_status_t cuco_box_timer(cuco_box_t *box, int op, float *ms);

/* Page-locked host memory for transfers (cudaHostAlloc / cudaFreeHost). */
cuco_status_t cuco_pinned_alloc(size_t bytes, void **ptr);
cuco_status_t cuco_pinned_free(void *ptr);

/* ---- Batched form (no counterpart in the reference) ---------------------
 * Many independent boxes advanced together: every phase of a step (drift and
 * keys, sort, reorder, each PM pass, short range and kick) is one launch over
 * all boxes, and cuco_ensemble_step replays the whole step as one CUDA graph.
 * Each box is described by a cuco_config_t (all boxes share mode and device;
 * meshes even, 8..1024, no prime factor above 5).  cell_grid = 0 lets the
 * autotuner pick the box's short-range cell grid by timing candidates on a
 * scratch box of the same size; FFT batching is always tuned.  Tuning results
 * are cached per (n, pm_grid, mode) for the life of the process. */
typedef struct cuco_ensemble cuco_ensemble_t;
cuco_status_t cuco_ensemble_create(const cuco_config_t *boxes, int nbox, cuco_ensemble_t **ensemble);
cuco_status_t cuco_ensemble_destroy(cuco_ensemble_t *ensemble);
/* Re-lay the ensemble out for a new set of boxes (same mode and device),
 * reusing its device arrays, which only grow: how a serving loop admits and
 * retires jobs without reallocating.  carry[b] = the current box whose
 * positions and velocities new box b keeps (same n and box length), or -1
 * for a box whose state the caller then sets with cuco_ensemble_set_state;
 * carry may be NULL when nothing is kept.  Synchronizes the ensemble's stream;
 * the next step captures a new graph. */
cuco_status_t cuco_ensemble_reshape(cuco_ensemble_t *ensemble, const cuco_config_t *boxes, int nbox,
                                    const int *carry);
/* the cell grid and FFT batching (z-pass row pairs, axis-pass columns per CTA) in use */
cuco_status_t cuco_ensemble_cell_grid(cuco_ensemble_t *ensemble, int box, int *cell_grid, int *fft_p,
                                      int *fft_b);
/* host float triplets, as cuco_box_set_state / cuco_box_get_state */
cuco_status_t cuco_ensemble_set_state(cuco_ensemble_t *ensemble, int box, const float *pos, const float *vel);
cuco_status_t cuco_ensemble_get_state(cuco_ensemble_t *ensemble, int box, float *pos, float *vel,
                                      float *acc_pp, float *acc_pm);
/* forces at the current positions (synchronous) */
cuco_status_t cuco_ensemble_forces(cuco_ensemble_t *ensemble);
/* one step of every box: drift[b], kick_pp[b], kick_pm[b] as cuco_box_step
 * (asynchronous; the first call also captures the graph).  The factors are
 * copied from one of two pinned slots used in turn, so a call waits at most
 * for the copy queued two calls back, not for the steps in flight. */
cuco_status_t cuco_ensemble_step(cuco_ensemble_t *ensemble, const double *drift, const double *kick_pp,
                                 const double *kick_pm);
cuco_status_t cuco_ensemble_sync(cuco_ensemble_t *ensemble);
/* op 0: mark a start on the ensemble's stream; op 1: ms since the mark */
cuco_status_t cuco_ensemble_timer(cuco_ensemble_t *ensemble, int op, float *ms);
/* returns (and resets) the in-range pairs counted so far; enable turns the
 * in-kernel count on or off for the following passes */
cuco_status_t cuco_ensemble_count_pairs(cuco_ensemble_t *ensemble, int enable, uint64_t *pairs);
int cuco_ensemble_launches_per_step(cuco_ensemble_t *ensemble);
/* the positions and velocities of src's box to dst's box (same n, box length
 * and mode), device to device: how a serving loop carries a running job into
 * a rebuilt ensemble */
cuco_status_t cuco_ensemble_copy_state(cuco_ensemble_t *dst, int dst_box, cuco_ensemble_t *src, int src_box);
/* device bytes an ensemble of these boxes holds (an upper bound: a box with
 * cell_grid 0 is counted at the largest grid the autotuner may pick) */
cuco_status_t cuco_ensemble_footprint(const cuco_config_t *boxes, int nbox, uint64_t *bytes);

/* Stable sort of (keys, values) by the low key_bits bits, in place, that
 * allocates no device memory (no counterpart in the reference).  For callers
 * that must not allocate where they sort: cudaMalloc/cudaFree can synchronize
 * the device and stall other streams, and hosts that give each job a fixed HBM
 * slice up front cannot let a library grow mid-run.  Scratch comes from one
 * array compiled into the library: at most 2^20 elements per call (larger n is
 * rejected with CUCO_ERR_INVALID); 8.25 MiB held on every GPU that loads the
 * library, until exit.  All calls on a device share that array, so calls that
 * overlap on the GPU race; order them on one stream.  The first call on a
 * device (with it current) looks up the array's device address and keeps it
 * for the life of the device's context; make it before any stream capture on
 * that device, and do not reset the device afterwards.  Every key must be
 * below 2^key_bits (as for radixSort).  values may be NULL (keys only);
 * stream is a cudaStream_t (NULL: legacy default stream). */
cuco_status_t cuco_radix_sort_noalloc(uint32_t *keys, uint32_t *values, uint32_t n,
                                      uint32_t key_bits, void *stream);

/* Measured FP32 FMA throughput of `device` in TFLOP/s (2 flops per FMA): a
 * register-resident FMA chain on every SM, timed with CUDA events. */
cuco_status_t cuco_fp32_peak(int device, double *tflops);

/* Drift and kick factors between scale factors a0 < a1 in FP64:
 * drift = int da/(H a^3), kick = int da/(H a^2), H = hubble*sqrt(Om/a^3 +
 * (1-Om-OL)/a^2 + OL) (driftfac.c:44-64). */
cuco_status_t cuco_cosmo_factors(double a0, double a1, double omega0, double omega_lambda,
                                 double hubble, double *drift, double *kick);

/* Message of the last failed call on this thread. */
const char *cuco_last_error(void);
const char *cuco_version(void);

#ifdef __cplusplus
}
#endif
#endif
