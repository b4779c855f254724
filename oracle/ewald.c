/* CPU oracle: FP64 Ewald summation of the periodic softened gravitational
 * acceleration (test infrastructure only; see oracle.h).
 *
 * Method: Hernquist, Bouchet & Suto (1991), ApJS 75, 231, eqs. 2.14-2.15, the
 * splitting of the periodic 1/r potential (with a uniform neutralising
 * background) into an erfc-screened real-space image sum and a Fourier sum:
 *   a(x_t) = G m sum_j [ sum_n e/|e|^3 (erfc(alpha|e|) + 2 alpha|e|/sqrt(pi) exp(-alpha^2|e|^2))
 *                        + 4 pi/L^3 sum_{k!=0} k/k^2 exp(-k^2/(4 alpha^2)) sin(k.d) ],
 * with d = x_j - x_t and e = d + nL.  The Fourier part uses structure factors
 * S(k) = sum_j exp(i k.x_j), so its cost is O(N N_k) + O(N_t N_k).  With
 * alpha L = 8 the real sum is cut at |e| < 6/alpha (erfc < 3e-17) over the 27
 * nearest images and the Fourier sum at |h| <= 15 (exp factor < 1e-15). */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

typedef struct {
    const double *src;
    int64_t n;
    double L, alpha, rc2, h, hinv, h3inv;
    const double *tg;
    int64_t nt;
    int nk;
    const int *kv;     /* nk x 3 integer wave vectors (half space) */
    const double *kc;  /* nk coefficients */
    double *S;         /* nk x 2 structure factor (re, im) */
    double *Spart;     /* per thread partial S */
    double *acc;
    int nthreads;
} ew_ctx;

typedef struct {
    ew_ctx *c;
    int t;
} ew_job;

static void *sf_worker(void *arg) {
    ew_job *j = (ew_job *)arg;
    ew_ctx *c = j->c;
    int H = 15;
    double *S = c->Spart + (size_t)j->t * 2 * c->nk;
    memset(S, 0, sizeof(double) * 2 * c->nk);
    double ex[2 * 16], ey[2 * 31], ez[2 * 31];
    for (int64_t i = j->t; i < c->n; i += c->nthreads) {
        double th[3];
        for (int d = 0; d < 3; ++d) th[d] = 2.0 * M_PI * c->src[3 * i + d] / c->L;
        for (int h = 0; h <= H; ++h) {
            ex[2 * h] = cos(h * th[0]);
            ex[2 * h + 1] = sin(h * th[0]);
        }
        for (int h = -H; h <= H; ++h) {
            ey[2 * (h + H)] = cos(h * th[1]);
            ey[2 * (h + H) + 1] = sin(h * th[1]);
            ez[2 * (h + H)] = cos(h * th[2]);
            ez[2 * (h + H) + 1] = sin(h * th[2]);
        }
        for (int k = 0; k < c->nk; ++k) {
            const double *a = ex + 2 * c->kv[3 * k];
            const double *b = ey + 2 * (c->kv[3 * k + 1] + H);
            const double *e = ez + 2 * (c->kv[3 * k + 2] + H);
            double re = a[0] * b[0] - a[1] * b[1], im = a[0] * b[1] + a[1] * b[0];
            S[2 * k] += re * e[0] - im * e[1];
            S[2 * k + 1] += re * e[1] + im * e[0];
        }
    }
    return NULL;
}

static void *tg_worker(void *arg) {
    ew_job *j = (ew_job *)arg;
    ew_ctx *c = j->c;
    double L = c->L, a = c->alpha, twoa_sqpi = 2.0 * a / sqrt(M_PI);
    for (int64_t t = j->t; t < c->nt; t += c->nthreads) {
        const double *x = c->tg + 3 * t;
        double ax = 0, ay = 0, az = 0;
        for (int64_t s = 0; s < c->n; ++s) {
            double d[3];
            for (int k = 0; k < 3; ++k) {
                d[k] = c->src[3 * s + k] - x[k];
                d[k] -= L * nearbyint(d[k] / L);
            }
            double dm2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (dm2 == 0.0) continue; /* the target itself */
            for (int nx = -1; nx <= 1; ++nx)
                for (int ny = -1; ny <= 1; ++ny)
                    for (int nz = -1; nz <= 1; ++nz) {
                        double ex = d[0] + nx * L, ey = d[1] + ny * L, ez = d[2] + nz * L;
                        double r2 = ex * ex + ey * ey + ez * ez;
                        if (r2 > c->rc2) continue;
                        double r = sqrt(r2);
                        double f = (erfc(a * r) + twoa_sqpi * r * exp(-a * a * r2)) / (r2 * r);
                        ax += f * ex;
                        ay += f * ey;
                        az += f * ez;
                    }
            if (dm2 < c->h * c->h) { /* spline softening of the nearest image */
                double r = sqrt(dm2), u = r * c->hinv, fs;
                if (u < 0.5)
                    fs = c->h3inv * (10.66667 + u * u * (32.0 * u - 38.4));
                else
                    fs = c->h3inv * (21.33333 - 48.0 * u + 38.4 * u * u - 10.66667 * u * u * u -
                                     0.06667 / (u * u * u));
                double corr = fs - 1.0 / (dm2 * r);
                ax += corr * d[0];
                ay += corr * d[1];
                az += corr * d[2];
            }
        }
        double th0 = 2.0 * M_PI / L;
        for (int k = 0; k < c->nk; ++k) {
            double kx = th0 * c->kv[3 * k], ky = th0 * c->kv[3 * k + 1], kz = th0 * c->kv[3 * k + 2];
            double ph = kx * x[0] + ky * x[1] + kz * x[2];
            /* Im(exp(-i k.x_t) S(k)) */
            double im = cos(ph) * c->S[2 * k + 1] - sin(ph) * c->S[2 * k];
            double w = c->kc[k] * im;
            ax += w * kx;
            ay += w * ky;
            az += w * kz;
        }
        c->acc[3 * t] = ax;
        c->acc[3 * t + 1] = ay;
        c->acc[3 * t + 2] = az;
    }
    return NULL;
}

void op_ewald(const double *src, int64_t n, double mass, double G, double boxsize,
              double softening, const double *targets, int64_t nt, int nthreads, double *acc) {
    const int H = 15;
    ew_ctx c;
    memset(&c, 0, sizeof(c));
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    c.src = src;
    c.n = n;
    c.L = boxsize;
    c.alpha = 8.0 / boxsize;
    c.rc2 = (6.0 / c.alpha) * (6.0 / c.alpha);
    c.h = softening;
    c.hinv = 1.0 / softening;
    c.h3inv = c.hinv * c.hinv * c.hinv;
    c.tg = targets;
    c.nt = nt;
    c.acc = acc;
    c.nthreads = nthreads;
    /* half-space wave vectors with 0 < |h| <= H */
    int cap = (2 * H + 1) * (2 * H + 1) * (H + 1);
    int *kv = (int *)malloc(sizeof(int) * 3 * cap);
    double *kc = (double *)malloc(sizeof(double) * cap);
    int nk = 0;
    double L3 = boxsize * boxsize * boxsize;
    for (int hx = 0; hx <= H; ++hx)
        for (int hy = -H; hy <= H; ++hy)
            for (int hz = -H; hz <= H; ++hz) {
                int h2 = hx * hx + hy * hy + hz * hz;
                if (h2 == 0 || h2 > H * H) continue;
                if (hx == 0 && (hy < 0 || (hy == 0 && hz < 0))) continue;
                double k2 = (2.0 * M_PI / boxsize) * (2.0 * M_PI / boxsize) * h2;
                kv[3 * nk] = hx;
                kv[3 * nk + 1] = hy;
                kv[3 * nk + 2] = hz;
                /* factor 2: the k and -k terms are equal */
                kc[nk] = 2.0 * 4.0 * M_PI / L3 * exp(-k2 / (4.0 * c.alpha * c.alpha)) / k2;
                nk++;
            }
    c.nk = nk;
    c.kv = kv;
    c.kc = kc;
    c.S = (double *)calloc((size_t)2 * nk, sizeof(double));
    c.Spart = (double *)malloc(sizeof(double) * 2 * nk * (size_t)nthreads);
    pthread_t th[256];
    ew_job jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].c = &c;
        jobs[t].t = t;
        pthread_create(&th[t], NULL, sf_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    for (int t = 0; t < nthreads; ++t)
        for (int k = 0; k < 2 * nk; ++k) c.S[k] += c.Spart[(size_t)t * 2 * nk + k];
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, tg_worker, &jobs[t]);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    for (int64_t t = 0; t < 3 * nt; ++t) acc[t] *= G * mass;
    free(kv);
    free(kc);
    free(c.S);
    free(c.Spart);
}
