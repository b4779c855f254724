/* CPU oracle for the force path (test infrastructure only).
 *
 * A plain-C restatement of the reference's algorithms, used by the tests as the
 * checker and by bench.py as the timed CPU baseline ("port").  The product never
 * links or calls it.  Each function cites the reference file:line it follows.
 *
 * Parity status: pinned.  tests/test_oracle_ref.py checks every function here
 * against the reference's own CPU code compiled from its sources
 * (oracle/_ref/libcucoref_pm<M>.so, built by oracle/Makefile) on seeded inputs,
 * and tests/golden/ holds fixtures generated from that build. */
#ifndef CUCO_ORACLE_H
#define CUCO_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters of one force evaluation, in the reference's types. */
typedef struct {
    float boxsize;    /* All.BoxSize (allvars.h:61) */
    float mass;       /* header.Mass / P[i].Mass (equal masses) */
    double G;         /* All.G (begrun.c:69) */
    float asmth;      /* All.Asmth = ASMTH*L/PMGRID (pm_periodic.c:27) */
    float rcut;       /* All.Rcut = RCUT*Asmth (pm_periodic.c:28) */
    float softening;  /* All.ForceSoftening = 2.8*SofteningTable (gravlist.cpp:36) */
} op_params;

/* Cell key of every particle, float32 arithmetic as calcHashD
 * (gravlist_kernel.cu:103-117): i = (int)(gridfac*p), key = (ix*G+iy)*G+iz.
 * Coordinates with gridfac*p rounding to G are clamped to G-1 (the reference
 * does not clamp; see the engine's design notes). */
void op_keys(const float *pos, int stride, int64_t n, float gridfac, int G, uint32_t *keys);

/* Stable sort by key (the permutation RadixSort::sort produces from an identity
 * value array, radixsort.h:170-187): counting sort, ties in input order. */
void op_stable_sort(const uint32_t *keys, int64_t n, uint32_t nkeys, uint32_t *sorted_keys,
                    uint32_t *perm);

/* cellStart/cellEnd as reorderDataAndFindCellStartD (gravlist_kernel.cu:121-160):
 * start = 0xffffffff for empty cells, end left at 0xffffffff for them. */
void op_cell_bounds(const uint32_t *sorted_keys, int64_t n, uint32_t ncells, uint32_t *start,
                    uint32_t *end);

/* The short-range split table (gravlist.cpp:56-59). */
void op_shortrange_table(float *table /* 1000 */);

/* Short-range force of every particle (force_evaluate_shortrange,
 * gravlist.cpp:216-338), on a G^3 linked-list grid (the reference uses
 * G = PMGRID, gravlist.cpp:117-146).  FP64 accumulation; acc is n x 3. */
void op_pp(const float *pos, int64_t n, const op_params *p, int G, int nthreads, float *acc);

/* op_pp for the listed targets only (acc is n x 3; other rows untouched). */
void op_pp_targets(const float *pos, int64_t n, const int64_t *targets, int64_t nt,
                   const op_params *p, int G, int nthreads, float *acc);

/* Number of ordered pairs (i != j) with float-computed r^2 <= rcut^2, as the
 * reference's pair test (gravlist_kernel.cu:46-55). */
int64_t op_pair_count(const float *pos, int64_t n, const op_params *p, int G, int nthreads);

/* Long-range PM force (pmforce_periodic, pm_periodic.c:67-314) on an M^3 mesh:
 * CIC deposit, FFT, Green's function with smoothing and deconvolution, FD4
 * gradient, CIC interpolation.  acc is n x 3. */
void op_pm(const float *pos, int64_t n, const op_params *p, int M, int nthreads, float *acc);

/* Drift and kick tables in FP64 (driftfac.c:14-42 stores them as float);
 * n entries at log a = log a0 + (log a1 - log a0)/n*(i+1). */
void op_drift_tables(double a0, double a1, double omega0, double omega_lambda, double hubble,
                     int n, double *drift, double *kick);

/* get_drift_factor / get_gravkick_factor (driftfac.c:66-126) over FP64 tables. */
double op_table_factor(const double *table, int n, double loga0, double loga1,
                       double timebase_interval, int t0, int t1);

/* FP64 Ewald-summed periodic acceleration (Hernquist, Bouchet & Suto 1991) on
 * `nt` targets from all n sources of equal mass, with a uniform neutralising
 * background.  Pairs closer than the spline softening length h (min image) get
 * the reference's spline force in place of 1/r^2 (gravlist.cpp:307-316), so the
 * result is the softened periodic force that PM + short range approximate.
 * A source at exactly a target's position is the target itself and is skipped.
 * src and targets are n x 3 / nt x 3 doubles; acc is nt x 3. */
void op_ewald(const double *src, int64_t n, double mass, double G, double boxsize,
              double softening, const double *targets, int64_t nt, int nthreads, double *acc);

/* op_ewald with the split parameter alpha = alpha_l / boxsize given (>= 11.5,
 * so the real-space cut 5.5/alpha stays below L/2); alpha_l <= 0 picks the one
 * that balances the real and Fourier work for n sources and nt targets.  The
 * result does not depend on alpha beyond the ~1e-12 truncation of either sum. */
void op_ewald_alpha(const double *src, int64_t n, double mass, double G, double boxsize,
                    double softening, const double *targets, int64_t nt, int nthreads,
                    double alpha_l, double *acc);

#ifdef __cplusplus
}
#endif
#endif
