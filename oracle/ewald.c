/* CPU oracle: FP64 Ewald summation of the periodic softened gravitational
 * acceleration (test infrastructure only; see oracle.h).
 *
 * Method: Hernquist, Bouchet & Suto (1991), ApJS 75, 231, eqs. 2.14-2.15, the
 * splitting of the periodic 1/r potential (with a uniform neutralising
 * background) into an erfc-screened real-space image sum and a Fourier sum:
 *   a(x_t) = G m sum_j [ sum_n e/|e|^3 (erfc(alpha|e|) + 2 alpha|e|/sqrt(pi) exp(-alpha^2|e|^2))
 *                        + 4 pi/L^3 sum_{k!=0} k/k^2 exp(-k^2/(4 alpha^2)) sin(k.d) ],
 * with d = x_j - x_t and e = d + nL.
 *
 * Truncation: the real sum stops at |e| = 5.5/alpha (the screened pair term
 * there is below 5e-13 of the Newtonian one) and the Fourier sum at
 * k^2/(4 alpha^2) = 30 (exp factor below 1e-13).  The split parameter
 * alpha only moves work between the two sums; the result does not depend on
 * it beyond those truncations, which the tests check by evaluating the same
 * targets at two values.  Cost: the real sum runs over a cell list of width
 * >= 5.5/alpha (27 neighbour cells, each image at most once since the cut is
 * below L/2), the Fourier sum through structure factors S(k) = sum_j
 * exp(i k.x_j), O(N N_k) + O(N_t N_k).  With alpha chosen automatically the
 * two parts are balanced for the given source and target counts. */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define EW_REAL_CUT 5.5     /* alpha * r_cut */
#define EW_KFAC 30.0        /* k_cut^2 / (4 alpha^2) */

typedef struct {
    const double *src;
    int64_t n;
    double L, alpha, rc2, h, hinv, h3inv;
    const double *tg;
    int64_t nt;
    int H;           /* |h| <= H */
    int nk;          /* wave vectors in the half space */
    const int *kx;   /* per (hx, hy) row: hx, hy, hz range */
    const int *rows; /* nrows x 4: hx, hy, hz0, hz1 (inclusive), row start in kc */
    int nrows;
    const double *kc;
    double *S;       /* nk x 2 */
    double *Spart;
    double *acc;
    int nthreads;
    /* cell list of the sources */
    int nc;
    const int64_t *cstart; /* nc^3 + 1 */
    const int64_t *cidx;
} ew_ctx;

typedef struct {
    ew_ctx *c;
    int t;
} ew_job;

/* exp(i h th) for h = -H..H into e[2*(h+H)] (re, im) by direct evaluation */
static void phases(double th, int H, double *e) {
    for (int h = 0; h <= H; ++h) {
        double c = cos(h * th), s = sin(h * th);
        e[2 * (H + h)] = c;
        e[2 * (H + h) + 1] = s;
        e[2 * (H - h)] = c;
        e[2 * (H - h) + 1] = -s;
    }
}

static void *sf_worker(void *arg) {
    ew_job *j = (ew_job *)arg;
    ew_ctx *c = j->c;
    const int H = c->H;
    double *S = c->Spart + (size_t)j->t * 2 * c->nk;
    memset(S, 0, sizeof(double) * 2 * c->nk);
    double *ex = (double *)malloc(sizeof(double) * 6 * (2 * H + 1));
    double *ey = ex + 2 * (2 * H + 1), *ez = ey + 2 * (2 * H + 1);
    const double th0 = 2.0 * M_PI / c->L;
    for (int64_t i = j->t; i < c->n; i += c->nthreads) {
        phases(th0 * c->src[3 * i], H, ex);
        phases(th0 * c->src[3 * i + 1], H, ey);
        phases(th0 * c->src[3 * i + 2], H, ez);
        for (int r = 0; r < c->nrows; ++r) {
            const int *row = c->rows + 5 * r;
            const double *a = ex + 2 * (row[0] + H), *b = ey + 2 * (row[1] + H);
            const double re = a[0] * b[0] - a[1] * b[1], im = a[0] * b[1] + a[1] * b[0];
            double *s = S + 2 * row[4];
            for (int hz = row[2]; hz <= row[3]; ++hz, s += 2) {
                const double *e = ez + 2 * (hz + H);
                s[0] += re * e[0] - im * e[1];
                s[1] += re * e[1] + im * e[0];
            }
        }
    }
    free(ex);
    return NULL;
}

static void real_pair(const ew_ctx *c, const double *d, double *acc) {
    /* d is the minimum image; the real sum needs only that image (cut < L/2) */
    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (r2 == 0.0) return; /* the target itself */
    if (r2 <= c->rc2) {
        const double r = sqrt(r2), a = c->alpha;
        const double f = (erfc(a * r) + 2.0 * a / sqrt(M_PI) * r * exp(-a * a * r2)) / (r2 * r);
        acc[0] += f * d[0];
        acc[1] += f * d[1];
        acc[2] += f * d[2];
    }
    if (r2 < c->h * c->h) { /* spline softening of the nearest image (gravlist.cpp:307-316) */
        const double r = sqrt(r2), u = r * c->hinv;
        double fs;
        if (u < 0.5)
            fs = c->h3inv * (10.66667 + u * u * (32.0 * u - 38.4));
        else
            fs = c->h3inv * (21.33333 - 48.0 * u + 38.4 * u * u - 10.66667 * u * u * u - 0.06667 / (u * u * u));
        const double corr = fs - 1.0 / (r2 * r);
        acc[0] += corr * d[0];
        acc[1] += corr * d[1];
        acc[2] += corr * d[2];
    }
}

static void *tg_worker(void *arg) {
    ew_job *j = (ew_job *)arg;
    ew_ctx *c = j->c;
    const double L = c->L;
    const int H = c->H, nc = c->nc;
    double *ex = (double *)malloc(sizeof(double) * 6 * (2 * H + 1));
    double *ey = ex + 2 * (2 * H + 1), *ez = ey + 2 * (2 * H + 1);
    const double th0 = 2.0 * M_PI / L;
    for (int64_t t = j->t; t < c->nt; t += c->nthreads) {
        const double *x = c->tg + 3 * t;
        double acc[3] = {0, 0, 0};
        /* real space over the 27 neighbour cells (each image at most once) */
        int ci[3];
        for (int k = 0; k < 3; ++k) {
            double u = x[k] / L;
            u -= floor(u);
            ci[k] = (int)(u * nc);
            if (ci[k] >= nc) ci[k] = nc - 1;
        }
        for (int ox = -1; ox <= 1; ++ox)
            for (int oy = -1; oy <= 1; ++oy)
                for (int oz = -1; oz <= 1; ++oz) {
                    const int cx = (ci[0] + ox + nc) % nc, cy = (ci[1] + oy + nc) % nc, cz = (ci[2] + oz + nc) % nc;
                    const int cell = (cx * nc + cy) * nc + cz;
                    for (int64_t q = c->cstart[cell]; q < c->cstart[cell + 1]; ++q) {
                        const int64_t s = c->cidx[q];
                        double d[3];
                        for (int k = 0; k < 3; ++k) {
                            d[k] = c->src[3 * s + k] - x[k];
                            d[k] -= L * nearbyint(d[k] / L);
                        }
                        real_pair(c, d, acc);
                    }
                }
        /* Fourier space: Im(exp(-i k.x_t) S(k)) */
        phases(th0 * x[0], H, ex);
        phases(th0 * x[1], H, ey);
        phases(th0 * x[2], H, ez);
        for (int r = 0; r < c->nrows; ++r) {
            const int *row = c->rows + 5 * r;
            const double *a = ex + 2 * (row[0] + H), *b = ey + 2 * (row[1] + H);
            const double re = a[0] * b[0] - a[1] * b[1], im = a[0] * b[1] + a[1] * b[0];
            const double *s = c->S + 2 * row[4];
            const double *w = c->kc + row[4];
            double fx = 0, fy = 0, fz = 0;
            for (int hz = row[2]; hz <= row[3]; ++hz, s += 2, ++w) {
                const double *e = ez + 2 * (hz + H);
                const double pr = re * e[0] - im * e[1], pi = re * e[1] + im * e[0];
                /* exp(-i phi) S = (pr - i pi)(S_re + i S_im); its imaginary part */
                const double v = *w * (pr * s[1] - pi * s[0]);
                fx += v;
                fz += v * hz;
            }
            fy = fx * row[1];
            fx *= row[0];
            acc[0] += th0 * fx;
            acc[1] += th0 * fy;
            acc[2] += th0 * fz;
        }
        c->acc[3 * t] = acc[0];
        c->acc[3 * t + 1] = acc[1];
        c->acc[3 * t + 2] = acc[2];
    }
    free(ex);
    return NULL;
}

static void run_threads(ew_ctx *c, void *(*fn)(void *)) {
    pthread_t th[256];
    ew_job jobs[256];
    for (int t = 0; t < c->nthreads; ++t) {
        jobs[t].c = c;
        jobs[t].t = t;
        pthread_create(&th[t], NULL, fn, &jobs[t]);
    }
    for (int t = 0; t < c->nthreads; ++t) pthread_join(th[t], NULL);
}

void op_ewald_alpha(const double *src, int64_t n, double mass, double G, double boxsize, double softening,
                    const double *targets, int64_t nt, int nthreads, double alpha_l, double *acc) {
    ew_ctx c;
    memset(&c, 0, sizeof(c));
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (alpha_l <= 0) {
        /* balance nt*n*(4pi/3)(5.5/x)^3 real pairs (~10x the cost of a
         * Fourier term) against (n+nt)*(2pi/3)(1.743 x)^3 Fourier terms */
        const double ratio = 10.0 * (double)nt * (double)n * 696.9 / (((double)n + (double)nt) * 11.09);
        alpha_l = pow(ratio, 1.0 / 6.0);
        if (alpha_l < 12.0) alpha_l = 12.0; /* keeps the real cut below L/2 */
        if (alpha_l > 40.0) alpha_l = 40.0;
    }
    if (alpha_l < 11.5) alpha_l = 11.5;
    c.src = src;
    c.n = n;
    c.L = boxsize;
    c.alpha = alpha_l / boxsize;
    const double rcut = EW_REAL_CUT / c.alpha;
    c.rc2 = rcut * rcut;
    c.h = softening;
    c.hinv = 1.0 / softening;
    c.h3inv = c.hinv * c.hinv * c.hinv;
    c.tg = targets;
    c.nt = nt;
    c.acc = acc;
    c.nthreads = nthreads;
    /* cell list: nc cells per dimension of width >= max(rcut, h) */
    const double wmin = rcut > softening ? rcut : softening;
    int nc = (int)floor(boxsize / wmin);
    if (nc < 3) nc = 3; /* rcut < L/2 keeps three cells of width >= rcut */
    if (nc > 256) nc = 256;
    c.nc = nc;
    const int64_t ncell = (int64_t)nc * nc * nc;
    int64_t *cstart = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
    int64_t *cidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int *cof = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) {
        int ci[3];
        for (int k = 0; k < 3; ++k) {
            double u = src[3 * i + k] / boxsize;
            u -= floor(u);
            ci[k] = (int)(u * nc);
            if (ci[k] >= nc) ci[k] = nc - 1;
        }
        cof[i] = (ci[0] * nc + ci[1]) * nc + ci[2];
        cstart[cof[i] + 1]++;
    }
    for (int64_t k = 0; k < ncell; ++k) cstart[k + 1] += cstart[k];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)ncell);
    memcpy(fill, cstart, sizeof(int64_t) * (size_t)ncell);
    for (int64_t i = 0; i < n; ++i) cidx[fill[cof[i]]++] = i;
    free(fill);
    free(cof);
    c.cstart = cstart;
    c.cidx = cidx;
    /* half-space wave vectors, 0 < k^2 <= 4 alpha^2 EW_KFAC, by (hx, hy) rows */
    const double kmax = 2.0 * c.alpha * sqrt(EW_KFAC);
    const int H = (int)floor(kmax * boxsize / (2.0 * M_PI));
    c.H = H;
    const double hmax2 = (kmax * boxsize / (2.0 * M_PI)) * (kmax * boxsize / (2.0 * M_PI));
    int *rows = (int *)malloc(sizeof(int) * 5 * (size_t)(H + 1) * (2 * H + 1));
    double *kc = (double *)malloc(sizeof(double) * (size_t)(H + 1) * (2 * H + 1) * (2 * H + 1));
    int nrows = 0, nk = 0;
    const double L3 = boxsize * boxsize * boxsize, dk = 2.0 * M_PI / boxsize;
    for (int hx = 0; hx <= H; ++hx)
        for (int hy = -H; hy <= H; ++hy) {
            const double rem = hmax2 - (double)hx * hx - (double)hy * hy;
            if (rem < 0) continue;
            int hz1 = (int)floor(sqrt(rem)), hz0 = -hz1;
            if (hx == 0 && hy < 0) continue;
            if (hx == 0 && hy == 0) hz0 = 1; /* half space, k != 0 */
            if (hz0 > hz1) continue;
            int *row = rows + 5 * nrows;
            row[0] = hx;
            row[1] = hy;
            row[2] = hz0;
            row[3] = hz1;
            row[4] = nk;
            for (int hz = hz0; hz <= hz1; ++hz) {
                const double k2 = dk * dk * ((double)hx * hx + (double)hy * hy + (double)hz * hz);
                /* factor 2: the k and -k terms are equal */
                kc[nk++] = 2.0 * 4.0 * M_PI / L3 * exp(-k2 / (4.0 * c.alpha * c.alpha)) / k2;
            }
            nrows++;
        }
    c.rows = rows;
    c.nrows = nrows;
    c.nk = nk;
    c.kc = kc;
    c.S = (double *)calloc((size_t)2 * nk, sizeof(double));
    c.Spart = (double *)malloc(sizeof(double) * 2 * (size_t)nk * nthreads);
    run_threads(&c, sf_worker);
    for (int t = 0; t < nthreads; ++t)
        for (int k = 0; k < 2 * nk; ++k) c.S[k] += c.Spart[(size_t)t * 2 * nk + k];
    run_threads(&c, tg_worker);
    for (int64_t t = 0; t < 3 * nt; ++t) acc[t] *= G * mass;
    free(rows);
    free(kc);
    free(c.S);
    free(c.Spart);
    free(cstart);
    free(cidx);
}

void op_ewald(const double *src, int64_t n, double mass, double G, double boxsize, double softening,
              const double *targets, int64_t nt, int nthreads, double *acc) {
    op_ewald_alpha(src, n, mass, G, boxsize, softening, targets, nt, nthreads, 0.0, acc);
}
