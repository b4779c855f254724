/* Oracle harness around the reference's CPU force path (test infrastructure).
 *
 * Linked with the reference's own sources (compiled where they lie by
 * oracle/Makefile, one library per PMGRID) and oracle/shim_impl.c.  It replaces
 * only what the reference reads from files or hardcodes:
 *   - read_parameter_file (begrun.c:31-63) -> cref_begrun() takes the parameters;
 *   - the IC file (read_ic.c) is written by the caller in the reference's own
 *     wire format and read back by the reference's init() (init.c:8-39);
 * and then runs the reference's set_units, init, long_range_init, linklist_init
 * and init_drift_table in begrun's order (begrun.c:10-27).
 *
 * The force entry points call the reference functions unchanged:
 *   cref_pm()  -> long_range_force()            (longrange.c:14-22, pm_periodic.c:67-314)
 *   cref_pp()  -> set_softenings(); build_linklist(); force_evaluate_shortrange(i)
 *                 for every particle (gravlist.cpp:195-214, 216-338), split over
 *                 threads when asked: force_evaluate_shortrange reads globals and
 *                 writes only P[target], so the split does not change any result.
 *   cref_step() -> one pass of the reference's run loop (run.c:11-20) with the CPU
 *                 short-range path in place of the GPU one (accel.c:21 vs 22). */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "allvars.h"
#include "proto.h"

void cuco_ref_set_threads(int n);
int cuco_ref_get_threads(void);

/* ---------------------------------------- storage for gravlist.cpp's ll/ihoc */

static int *g_ll = NULL;
static size_t g_ll_n = 0;
static int *g_ihoc = NULL;

int *cuco_ref_ll_storage(void) {
    if (g_ll_n < NumPart) {
        free(g_ll);
        g_ll = (int *)malloc(sizeof(int) * (NumPart ? NumPart : 1));
        g_ll_n = NumPart;
    }
    return g_ll;
}

int *cuco_ref_ihoc_storage(void) {
    if (!g_ihoc) g_ihoc = (int *)malloc(sizeof(int) * (size_t)PMGRID * PMGRID * PMGRID);
    return g_ihoc;
}

/* ------------------------------------------------------------------ set-up */

int cref_pmgrid(void) { return PMGRID; }
int cref_sizeof_particle(void) { return (int)sizeof(PARTICLE); }
int cref_sizeof_header(void) { return (int)sizeof(HEADER); }

/* Parameters as read_parameter_file sets them (begrun.c:33-50), with the run's
 * own values for what the configurations vary.  `ic_path` is an IC file in the
 * reference's format (HEADER + PARTICLE[NumPart], read_ic.c:19-33). */
int cref_begrun(const char *ic_path, double a_begin, double a_max, double soft_comoving,
                double soft_maxphys, double omega0, double omega_lambda, double hubble_param,
                double max_dloga, double errtol) {
    All.UnitLength_in_m = 3.085678e19;
    All.UnitMass_in_kg = 1.98892e40;
    All.UnitVelocity_in_m_per_s = 1e3;
    All.Omega0 = (float)omega0;
    All.OmegaLambda = (float)omega_lambda;
    All.OmegaBaryon = 0.04f;
    All.HubbleParam = (float)hubble_param;
    All.BoxSize = 10000.0f;
    All.ErrTolIntAccuracy = (float)errtol;
    All.MaxSizeTimestep = (float)max_dloga;
    All.MinSizeTimestep = 0.0f;
    All.SofteningHalo = (float)soft_comoving;
    All.SofteningHaloMaxPhys = (float)soft_maxphys;
    All.TimeBegin = (float)a_begin;
    All.TimeMax = (float)a_max;
    strncpy(All.InitCondFile, ic_path, MAXLEN_FILENAME - 1);
    strcpy(All.OutputDir, ".");
    strcpy(All.SnapshotFileBase, "snapshot");
    All.OutputListLength = 0;

    set_units();
    init();
    cudaInit();
    long_range_init();
    linklist_init();
    init_drift_table();
    All.Ti_nextoutput = find_next_outputtime(All.Ti_Current);
    return 0;
}

double cref_G(void) { return All.G; }
double cref_hubble(void) { return All.Hubble; }
double cref_asmth(void) { return All.Asmth; }
double cref_rcut(void) { return All.Rcut; }
double cref_timebase_interval(void) { return All.Timebase_interval; }
int cref_ti_current(void) { return All.Ti_Current; }
double cref_time(void) { return All.Time; }
double cref_force_softening(void) { return All.ForceSoftening; }
unsigned int cref_numpart(void) { return NumPart; }

void cref_get_tables(float *drift, float *kick) {
    memcpy(drift, DriftTable, sizeof(float) * DRIFT_TABLE_LENGTH);
    memcpy(kick, GravKickTable, sizeof(float) * DRIFT_TABLE_LENGTH);
}

double cref_drift_factor(int t0, int t1) { return get_drift_factor(t0, t1); }
double cref_kick_factor(int t0, int t1) { return get_gravkick_factor(t0, t1); }

/* The constant block linklist_init uploads (SIMPARAM, proto.cuh:7-18). */
const void *cuco_ref_simparam(void);
const void *cuco_ref_softparam(void);
void cref_simparam(float *out /* NTAB + 9 */) { memcpy(out, cuco_ref_simparam(), sizeof(float) * (NTAB + 9)); }
void cref_softparam(float *out /* 3 */) { memcpy(out, cuco_ref_softparam(), sizeof(float) * 3); }

/* ------------------------------------------------------------ state access */

void cref_set_pos(const float *pos /* n x 3 */) {
    for (unsigned int i = 0; i < NumPart; ++i)
        for (int d = 0; d < 3; ++d) P[i].Pos[d] = pos[3 * i + d];
}

void cref_set_vel(const float *vel) {
    for (unsigned int i = 0; i < NumPart; ++i)
        for (int d = 0; d < 3; ++d) P[i].Vel[d] = vel[3 * i + d];
}

void cref_get(float *pos, float *vel, float *acc_pp, float *acc_pm) {
    for (unsigned int i = 0; i < NumPart; ++i)
        for (int d = 0; d < 3; ++d) {
            if (pos) pos[3 * i + d] = P[i].Pos[d];
            if (vel) vel[3 * i + d] = P[i].Vel[d];
            if (acc_pp) acc_pp[3 * i + d] = P[i].GravAccel[d];
            if (acc_pm) acc_pm[3 * i + d] = P[i].GravPM[d];
        }
}

void cref_get_particles(void *out /* NumPart * sizeof(PARTICLE) */) {
    memcpy(out, P, sizeof(PARTICLE) * NumPart);
}

void cref_get_timeline(int *ti_beg, int *ti_end, int *pm_ti) {
    for (unsigned int i = 0; i < NumPart; ++i) {
        ti_beg[i] = P[i].Ti_begstep;
        ti_end[i] = P[i].Ti_endstep;
    }
    pm_ti[0] = All.PM_Ti_begstep;
    pm_ti[1] = All.PM_Ti_endstep;
    pm_ti[2] = All.Ti_Current;
}

/* ----------------------------------------------------------------- forces */

void cref_wrap(void) { do_box_wrapping(); }

void cref_pm(void) { long_range_force(); }

typedef struct {
    int t, nt;
} pp_job;

static void *pp_worker(void *arg) {
    pp_job *jb = (pp_job *)arg;
    for (unsigned int i = (unsigned int)jb->t; i < NumPart; i += (unsigned int)jb->nt)
        force_evaluate_shortrange((int)i);
    return NULL;
}

/* Short-range force for every particle.  nthreads == 1 runs the reference's own
 * gravity_linklist() after marking every particle active; more threads split
 * the same per-target calls. */
void cref_pp(int nthreads) {
    if (nthreads <= 1) {
        for (unsigned int i = 0; i < NumPart; ++i) P[i].Ti_endstep = All.Ti_Current;
        gravity_linklist();
        return;
    }
    set_softenings();
    build_linklist();
    pthread_t th[256];
    pp_job jobs[256];
    if (nthreads > 256) nthreads = 256;
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].t = t;
        jobs[t].nt = nthreads;
        pthread_create(&th[t], NULL, pp_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
}

void cref_set_threads(int n) { cuco_ref_set_threads(n); }

typedef struct {
    int t, nt;
} step_job;

static void *active_worker(void *arg) {
    step_job *jb = (step_job *)arg;
    for (unsigned int i = (unsigned int)jb->t; i < NumPart; i += (unsigned int)jb->nt)
        if (P[i].Ti_endstep == All.Ti_Current) force_evaluate_shortrange((int)i);
    return NULL;
}

/* One pass of run() (run.c:11-20): drift to the next sync point, forces (PM when
 * due, then the CPU short-range path for the active particles), kick and new
 * timesteps.  Returns the new Ti_Current. */
int cref_step(int nthreads) {
    find_next_sync_point_and_drift();
    do_box_wrapping();
    if (All.PM_Ti_endstep == All.Ti_Current) long_range_force();
    if (nthreads <= 1) {
        gravity_linklist();
    } else {
        set_softenings();
        build_linklist();
        pthread_t th[256];
        step_job jobs[256];
        if (nthreads > 256) nthreads = 256;
        for (int t = 0; t < nthreads; ++t) {
            jobs[t].t = t;
            jobs[t].nt = nthreads;
            pthread_create(&th[t], NULL, active_worker, &jobs[t]);
        }
        for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    }
    advance_and_find_timesteps();
    All.NumCurrentTiStep++;
    return All.Ti_Current;
}

/* Snapshot in the reference's format (io.c:9-40), into All.OutputDir. */
void cref_set_output(const char *dir, const char *base) {
    strncpy(All.OutputDir, dir, MAXLEN_FILENAME - 1);
    strncpy(All.SnapshotFileBase, base, MAXLEN_FILENAME - 1);
}

void cref_save_snapshot(int num) { savepositions(num); }

/* Layout of the reference's global structs, for the ABI checks of the drop-in
 * headers: sizeof(ALL) and the offsets of fields the drop-in reads/writes. */
#include <stddef.h>
void cref_layout(long *out /* 16 */) {
    out[0] = (long)sizeof(ALL);
    out[1] = (long)offsetof(ALL, G);
    out[2] = (long)offsetof(ALL, Hubble);
    out[3] = (long)offsetof(ALL, Time);
    out[4] = (long)offsetof(ALL, Timebase_interval);
    out[5] = (long)offsetof(ALL, Ti_Current);
    out[6] = (long)offsetof(ALL, PM_Ti_endstep);
    out[7] = (long)offsetof(ALL, Asmth);
    out[8] = (long)offsetof(ALL, ForceSoftening);
    out[9] = (long)offsetof(ALL, OutputListTimes);
    out[10] = (long)offsetof(ALL, InitCondFile);
    out[11] = (long)sizeof(PARTICLE);
    out[12] = (long)sizeof(HEADER);
    out[13] = (long)offsetof(PARTICLE, GravPM);
    out[14] = (long)offsetof(PARTICLE, Ti_endstep);
    out[15] = (long)offsetof(ALL, SofteningTable);
}
