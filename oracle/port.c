/* CPU oracle: plain-C restatement of the reference's force path
 * (test infrastructure only; declarations and the parity status in oracle.h).
 *
 * The arithmetic follows the reference statement by statement, including its
 * mix of float and double, so that results agree with the reference's own CPU
 * build to the last bit or within one float rounding. */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define NTAB 1000

/* ------------------------------------------------------------ thread helper */

typedef void (*range_fn)(void *ctx, int64_t begin, int64_t end, int tid);

typedef struct {
    range_fn fn;
    void *ctx;
    int64_t begin, end;
    int tid;
} range_job;

static void *range_worker(void *arg) {
    range_job *j = (range_job *)arg;
    j->fn(j->ctx, j->begin, j->end, j->tid);
    return NULL;
}

/* Split [0, n) into contiguous chunks, one per thread. */
static void parallel_for(int64_t n, int nthreads, range_fn fn, void *ctx) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (nthreads == 1 || n < 2 * nthreads) {
        fn(ctx, 0, n, 0);
        return;
    }
    pthread_t th[256];
    range_job jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].begin = n * t / nthreads;
        jobs[t].end = n * (t + 1) / nthreads;
        jobs[t].tid = t;
        pthread_create(&th[t], NULL, range_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------- keys */

void op_keys(const float *pos, int stride, int64_t n, float gridfac, int G, uint32_t *keys) {
    for (int64_t i = 0; i < n; ++i) {
        const float *p = pos + i * stride;
        int c[3];
        for (int d = 0; d < 3; ++d) {
            float t = gridfac * p[d]; /* float32 product, truncated (gravlist_kernel.cu:109-111) */
            int ic = (int)t;
            if (ic >= G) ic = G - 1;
            if (ic < 0) ic = 0;
            c[d] = ic;
        }
        keys[i] = ((uint32_t)c[0] * (uint32_t)G + (uint32_t)c[1]) * (uint32_t)G + (uint32_t)c[2];
    }
}

void op_stable_sort(const uint32_t *keys, int64_t n, uint32_t nkeys, uint32_t *sorted_keys,
                    uint32_t *perm) {
    uint32_t *count = (uint32_t *)calloc((size_t)nkeys + 1, sizeof(uint32_t));
    for (int64_t i = 0; i < n; ++i) count[keys[i] + 1]++;
    for (uint32_t k = 0; k < nkeys; ++k) count[k + 1] += count[k];
    for (int64_t i = 0; i < n; ++i) {
        uint32_t at = count[keys[i]]++;
        sorted_keys[at] = keys[i];
        perm[at] = (uint32_t)i;
    }
    free(count);
}

void op_cell_bounds(const uint32_t *sorted_keys, int64_t n, uint32_t ncells, uint32_t *start,
                    uint32_t *end) {
    for (uint32_t c = 0; c < ncells; ++c) {
        start[c] = 0xffffffffu;
        end[c] = 0xffffffffu;
    }
    for (int64_t i = 0; i < n; ++i) {
        if (i == 0 || sorted_keys[i] != sorted_keys[i - 1]) {
            start[sorted_keys[i]] = (uint32_t)i;
            if (i > 0) end[sorted_keys[i - 1]] = (uint32_t)i;
        }
        if (i == n - 1) end[sorted_keys[i]] = (uint32_t)(i + 1);
    }
}

/* ----------------------------------------------------------- short range */

void op_shortrange_table(float *table) {
    for (int i = 0; i < NTAB; ++i) {
        double u = 3.0 / NTAB * (i + 0.5);
        table[i] = (float)(erfc(u) + 2.0 * u / sqrt(M_PI) * exp(-u * u));
    }
}

typedef struct {
    const float *pos;
    int64_t n;
    int G;
    double to_grid_fac, rcut, rcut2, asmthfac, h, h_inv, h3_inv, mass, Gconst;
    float boxsize, boxhalf;
    float table[NTAB];
    int *ll, *ihoc;
    float *acc;
    int64_t *pair_counts; /* per thread, when counting */
} pp_ctx;

static void pp_setup(pp_ctx *c, const float *pos, int64_t n, const op_params *p, int G) {
    c->pos = pos;
    c->n = n;
    c->G = G;
    c->to_grid_fac = (double)((float)G / p->boxsize); /* gravlist.cpp:61, float division */
    c->rcut = p->rcut;
    c->rcut2 = c->rcut * c->rcut;
    c->asmthfac = 0.5 / (double)p->asmth * (NTAB / 3.0);
    c->boxsize = p->boxsize;
    c->boxhalf = (float)(p->boxsize / 2.0);
    c->h = p->softening;
    c->h_inv = 1.0 / c->h;
    c->h3_inv = c->h_inv * c->h_inv * c->h_inv;
    c->mass = p->mass;
    c->Gconst = p->G;
    op_shortrange_table(c->table);
    /* build_linklist (gravlist.cpp:117-146): the head of each cell's chain is the
     * last particle inserted into it */
    size_t ncell = (size_t)G * G * G;
    c->ll = (int *)malloc(sizeof(int) * (size_t)(n ? n : 1));
    c->ihoc = (int *)malloc(sizeof(int) * ncell);
    for (size_t i = 0; i < ncell; ++i) c->ihoc[i] = -1;
    for (int64_t i = 0; i < n; ++i) {
        int ix = (int)(c->to_grid_fac * pos[3 * i + 0]);
        int iy = (int)(c->to_grid_fac * pos[3 * i + 1]);
        int iz = (int)(c->to_grid_fac * pos[3 * i + 2]);
        if (ix >= G) ix = G - 1;
        if (iy >= G) iy = G - 1;
        if (iz >= G) iz = G - 1;
        int ibox = ix * G * G + iy * G + iz;
        c->ll[i] = c->ihoc[ibox];
        c->ihoc[ibox] = (int)i;
    }
}

static void pp_free(pp_ctx *c) {
    free(c->ll);
    free(c->ihoc);
}

/* force_evaluate_shortrange (gravlist.cpp:216-338) for one target; when
 * `count` is non-NULL it also counts the in-range pairs. */
static void pp_target(const pp_ctx *c, int64_t target, float *out, int64_t *count) {
    const float *P = c->pos;
    const int G = c->G;
    double acc_x = 0, acc_y = 0, acc_z = 0;
    double pos_x = P[3 * target + 0], pos_y = P[3 * target + 1], pos_z = P[3 * target + 2];
    double mass = c->mass;
    int xl = (int)(c->to_grid_fac * (pos_x - c->rcut) + G);
    xl -= G;
    int xr = (int)(c->to_grid_fac * (pos_x + c->rcut));
    int yl = (int)(c->to_grid_fac * (pos_y - c->rcut) + G);
    yl -= G;
    int yr = (int)(c->to_grid_fac * (pos_y + c->rcut));
    int zl = (int)(c->to_grid_fac * (pos_z - c->rcut) + G);
    zl -= G;
    int zr = (int)(c->to_grid_fac * (pos_z + c->rcut));
    int64_t npairs = 0;
    for (int ix = xl; ix <= xr; ++ix)
        for (int iy = yl; iy <= yr; ++iy)
            for (int iz = zl; iz <= zr; ++iz) {
                int iix = ix, iiy = iy, iiz = iz;
                while (iix < 0) iix += G;
                while (iix >= G) iix -= G;
                while (iiy < 0) iiy += G;
                while (iiy >= G) iiy -= G;
                while (iiz < 0) iiz += G;
                while (iiz >= G) iiz -= G;
                int no = c->ihoc[iix * G * G + iiy * G + iiz];
                while (no != -1) {
                    if (no == target) {
                        no = c->ll[no];
                        continue;
                    }
                    double dx = P[3 * no + 0] - pos_x;
                    double dy = P[3 * no + 1] - pos_y;
                    double dz = P[3 * no + 2] - pos_z;
                    if (dx > c->boxhalf) dx -= c->boxsize;
                    if (dx < -c->boxhalf) dx += c->boxsize;
                    if (dy > c->boxhalf) dy -= c->boxsize;
                    if (dy < -c->boxhalf) dy += c->boxsize;
                    if (dz > c->boxhalf) dz -= c->boxsize;
                    if (dz < -c->boxhalf) dz += c->boxsize;
                    double r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 > c->rcut2) {
                        no = c->ll[no];
                        continue;
                    }
                    npairs++;
                    double r = sqrt(r2), fac;
                    if (r >= c->h) {
                        fac = mass / (r2 * r);
                    } else {
                        double u = r * c->h_inv;
                        if (u < 0.5)
                            fac = mass * c->h3_inv * (10.66667 + u * u * (32.0 * u - 38.4));
                        else
                            fac = mass * c->h3_inv *
                                  (21.33333 - 48.0 * u + 38.4 * u * u - 10.66667 * u * u * u -
                                   0.06667 / (u * u * u));
                    }
                    int tabindex = (int)(c->asmthfac * r);
                    if (tabindex < NTAB) {
                        fac *= c->table[tabindex];
                        acc_x += dx * fac;
                        acc_y += dy * fac;
                        acc_z += dz * fac;
                    }
                    no = c->ll[no];
                }
            }
    if (out) {
        out[3 * target + 0] = (float)(acc_x * c->Gconst);
        out[3 * target + 1] = (float)(acc_y * c->Gconst);
        out[3 * target + 2] = (float)(acc_z * c->Gconst);
    }
    if (count) *count += npairs;
}

static void pp_range(void *ctx, int64_t b, int64_t e, int tid) {
    pp_ctx *c = (pp_ctx *)ctx;
    int64_t cnt = 0;
    for (int64_t i = b; i < e; ++i) pp_target(c, i, c->acc, c->pair_counts ? &cnt : NULL);
    if (c->pair_counts) c->pair_counts[tid] = cnt;
}

void op_pp(const float *pos, int64_t n, const op_params *p, int G, int nthreads, float *acc) {
    pp_ctx *c = (pp_ctx *)malloc(sizeof(pp_ctx));
    pp_setup(c, pos, n, p, G);
    c->acc = acc;
    c->pair_counts = NULL;
    parallel_for(n, nthreads, pp_range, c);
    pp_free(c);
    free(c);
}

typedef struct {
    pp_ctx *c;
    const int64_t *targets;
} pp_sub_ctx;

static void pp_sub_range(void *ctx, int64_t b, int64_t e, int tid) {
    (void)tid;
    pp_sub_ctx *s = (pp_sub_ctx *)ctx;
    for (int64_t i = b; i < e; ++i) pp_target(s->c, s->targets[i], s->c->acc, NULL);
}

void op_pp_targets(const float *pos, int64_t n, const int64_t *targets, int64_t nt,
                   const op_params *p, int G, int nthreads, float *acc) {
    pp_ctx *c = (pp_ctx *)malloc(sizeof(pp_ctx));
    pp_setup(c, pos, n, p, G);
    c->acc = acc;
    c->pair_counts = NULL;
    pp_sub_ctx s = {c, targets};
    parallel_for(nt, nthreads, pp_sub_range, &s);
    pp_free(c);
    free(c);
}

int64_t op_pair_count(const float *pos, int64_t n, const op_params *p, int G, int nthreads) {
    pp_ctx *c = (pp_ctx *)malloc(sizeof(pp_ctx));
    int64_t counts[256] = {0};
    pp_setup(c, pos, n, p, G);
    c->acc = NULL;
    c->pair_counts = counts;
    parallel_for(n, nthreads, pp_range, c);
    int64_t total = 0;
    for (int t = 0; t < 256; ++t) total += counts[t];
    pp_free(c);
    free(c);
    return total;
}

/* --------------------------------------------------------------- PM (FFT) */

typedef struct {
    double re, im;
} dcpx;

/* In-place transform of n points `stride` apart: radix-2 for a power of two,
 * else the DFT by its definition, X_k = sum_j a_j w^(j k mod n) (the meshes
 * the reference supports are powers of two; the others serve the engine's
 * batched form, whose meshes are 2 x the particle grid). */
static void fft_line(dcpx *a, int n, int64_t stride, int sign, dcpx *buf, const dcpx *tw) {
    for (int i = 0; i < n; ++i) buf[i] = a[i * stride];
    if (n & (n - 1)) {
        for (int k = 0; k < n; ++k) {
            double re = 0, im = 0;
            for (int j = 0; j < n; ++j) {
                dcpx w = tw[(int)(((int64_t)j * k) % n)];
                if (sign > 0) w.im = -w.im;
                re += buf[j].re * w.re - buf[j].im * w.im;
                im += buf[j].re * w.im + buf[j].im * w.re;
            }
            a[k * stride].re = re;
            a[k * stride].im = im;
        }
        return;
    }
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            dcpx t = buf[i];
            buf[i] = buf[j];
            buf[j] = t;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int step = n / len;
        for (int k = 0; k < len / 2; ++k) {
            dcpx w = tw[k * step];
            if (sign > 0) w.im = -w.im;
            for (int i = 0; i < n; i += len) {
                dcpx u = buf[i + k], v = buf[i + k + len / 2];
                dcpx x = {v.re * w.re - v.im * w.im, v.re * w.im + v.im * w.re};
                buf[i + k].re = u.re + x.re;
                buf[i + k].im = u.im + x.im;
                buf[i + k + len / 2].re = u.re - x.re;
                buf[i + k + len / 2].im = u.im - x.im;
            }
        }
    }
    for (int i = 0; i < n; ++i) a[i * stride] = buf[i];
}

typedef struct {
    dcpx *a;
    int M, axis, sign;
    const dcpx *tw;
} fft_ctx;

static void fft_range(void *ctx, int64_t b, int64_t e, int tid) {
    (void)tid;
    fft_ctx *c = (fft_ctx *)ctx;
    int M = c->M;
    dcpx *buf = (dcpx *)malloc(sizeof(dcpx) * M);
    for (int64_t l = b; l < e; ++l) {
        dcpx *base;
        int64_t stride;
        if (c->axis == 0) {
            base = c->a + l;
            stride = (int64_t)M * M;
        } else if (c->axis == 1) {
            base = c->a + (l / M) * M * M + (l % M);
            stride = M;
        } else {
            base = c->a + l * M;
            stride = 1;
        }
        fft_line(base, M, stride, c->sign, buf, c->tw);
    }
    free(buf);
}

static void fft3(dcpx *a, int M, int sign, int nthreads) {
    dcpx *tw = (dcpx *)malloc(sizeof(dcpx) * M);
    for (int k = 0; k < M; ++k) {
        tw[k].re = cos(2.0 * M_PI * k / M);
        tw[k].im = -sin(2.0 * M_PI * k / M);
    }
    fft_ctx c = {a, M, 0, sign, tw};
    for (int axis = 2; axis >= 0; --axis) {
        c.axis = axis;
        parallel_for((int64_t)M * M, nthreads, fft_range, &c);
    }
    free(tw);
}

typedef struct {
    const float *pos;
    int64_t n;
    int M, dim;
    float to_slab_fac;
    double fac;
    const float *rho; /* padded potential grid */
    float *force;     /* M^3 */
    float *acc;
    float *cgrid;     /* complex half grid, interleaved */
    double asmth2;
} pm_ctx;

static void green_range(void *ctx, int64_t b, int64_t e, int tid) {
    (void)tid;
    pm_ctx *c = (pm_ctx *)ctx;
    int M = c->M, Mh = M / 2 + 1;
    for (int64_t xy = b; xy < e; ++xy) {
        int x = (int)(xy / M), y = (int)(xy % M);
        for (int z = 0; z < Mh; ++z) {
            double kx = x > M / 2 ? x - M : x;
            double ky = y > M / 2 ? y - M : y;
            double kz = z > M / 2 ? z - M : z;
            double k2 = kx * kx + ky * ky + kz * kz;
            if (k2 > 0) {
                double smth = -exp(-k2 * c->asmth2) / k2;
                double fx = 1, fy = 1, fz = 1;
                if (kx != 0) {
                    fx = (M_PI * kx) / M;
                    fx = sin(fx) / fx;
                }
                if (ky != 0) {
                    fy = (M_PI * ky) / M;
                    fy = sin(fy) / fy;
                }
                if (kz != 0) {
                    fz = (M_PI * kz) / M;
                    fz = sin(fz) / fz;
                }
                double ff = 1 / (fx * fy * fz);
                smth *= ff * ff * ff * ff;
                int64_t ip = (int64_t)M * Mh * x + (int64_t)Mh * y + z;
                c->cgrid[2 * ip + 0] = (float)(c->cgrid[2 * ip + 0] * smth);
                c->cgrid[2 * ip + 1] = (float)(c->cgrid[2 * ip + 1] * smth);
            }
        }
    }
}

static void fd4_range(void *ctx, int64_t b, int64_t e, int tid) {
    (void)tid;
    pm_ctx *c = (pm_ctx *)ctx;
    int M = c->M, dimy = M, dimz = 2 * (M / 2 + 1);
    const float *r = c->rho;
    for (int64_t xy = b; xy < e; ++xy) {
        int x = (int)(xy / M), y = (int)(xy % M);
        for (int z = 0; z < M; ++z) {
            int xl = x, xr = x, xll = x, xrr = x, yl = y, yr = y, yll = y, yrr = y;
            int zl = z, zr = z, zll = z, zrr = z;
            if (c->dim == 0) {
                xr = (x + 1) % M;
                xrr = (x + 2) % M;
                xl = (x - 1 + M) % M;
                xll = (x - 2 + M) % M;
            } else if (c->dim == 1) {
                yr = (y + 1) % M;
                yrr = (y + 2) % M;
                yl = (y - 1 + M) % M;
                yll = (y - 2 + M) % M;
            } else {
                zr = (z + 1) % M;
                zrr = (z + 2) % M;
                zl = (z - 1 + M) % M;
                zll = (z - 2 + M) % M;
            }
            c->force[((int64_t)x * M + y) * M + z] =
                (float)(c->fac * ((4.0 / 3) * (r[((int64_t)xl * dimy + yl) * dimz + zl] -
                                               r[((int64_t)xr * dimy + yr) * dimz + zr]) -
                                  (1.0 / 6) * (r[((int64_t)xll * dimy + yll) * dimz + zll] -
                                               r[((int64_t)xrr * dimy + yrr) * dimz + zrr])));
        }
    }
}

/* slab index and CIC fraction exactly as pm_periodic.c:99-121 */
static inline void cic_axis(float to_slab_fac, float p, int M, int *s, int *ss, double *d) {
    float t = to_slab_fac * p;
    int sl = (int)t;
    if (sl >= M) sl = M - 1;
    float frac = t - (float)sl;
    *d = frac;
    *s = sl;
    *ss = sl + 1 >= M ? sl + 1 - M : sl + 1;
}

static void interp_range(void *ctx, int64_t b, int64_t e, int tid) {
    (void)tid;
    pm_ctx *c = (pm_ctx *)ctx;
    int M = c->M;
    const float *F = c->force;
    for (int64_t i = b; i < e; ++i) {
        int sx, sxx, sy, syy, sz, szz;
        double dx, dy, dz;
        cic_axis(c->to_slab_fac, c->pos[3 * i + 0], M, &sx, &sxx, &dx);
        cic_axis(c->to_slab_fac, c->pos[3 * i + 1], M, &sy, &syy, &dy);
        cic_axis(c->to_slab_fac, c->pos[3 * i + 2], M, &sz, &szz, &dz);
#define FG(a, b, cc) ((double)F[((int64_t)(a) * M + (b)) * M + (cc)])
        double acc = FG(sx, sy, sz) * (1.0 - dx) * (1.0 - dy) * (1.0 - dz);
        acc += FG(sx, syy, sz) * (1.0 - dx) * dy * (1.0 - dz);
        acc += FG(sx, sy, szz) * (1.0 - dx) * (1.0 - dy) * dz;
        acc += FG(sx, syy, szz) * (1.0 - dx) * dy * dz;
        acc += FG(sxx, sy, sz) * (dx) * (1.0 - dy) * (1.0 - dz);
        acc += FG(sxx, syy, sz) * (dx)*dy * (1.0 - dz);
        acc += FG(sxx, sy, szz) * (dx) * (1.0 - dy) * dz;
        acc += FG(sxx, syy, szz) * (dx)*dy * dz;
#undef FG
        c->acc[3 * i + c->dim] = (float)acc;
    }
}

void op_pm(const float *pos, int64_t n, const op_params *p, int M, int nthreads, float *acc) {
    int Mh = M / 2 + 1, dimy = M, dimz = 2 * Mh;
    pm_ctx c;
    memset(&c, 0, sizeof(c));
    c.pos = pos;
    c.n = n;
    c.M = M;
    c.to_slab_fac = (float)M / p->boxsize; /* pm_periodic.c:42, float division */
    c.asmth2 = (2 * M_PI) * (double)p->asmth / (double)p->boxsize;
    c.asmth2 *= c.asmth2;
    c.fac = p->G / (M_PI * (double)p->boxsize);
    c.fac *= (double)(1.0f / (2.0f * p->boxsize / (float)M)); /* pm_periodic.c:86, float */
    c.acc = acc;

    size_t fftsize = (size_t)M * M * dimz;
    float *rho = (float *)calloc(fftsize, sizeof(float));
    /* CIC deposit in particle order, float grid += double weight (pm_periodic.c:97-132) */
    for (int64_t i = 0; i < n; ++i) {
        int sx, sxx, sy, syy, sz, szz;
        double dx, dy, dz, m = p->mass;
        cic_axis(c.to_slab_fac, pos[3 * i + 0], M, &sx, &sxx, &dx);
        cic_axis(c.to_slab_fac, pos[3 * i + 1], M, &sy, &syy, &dy);
        cic_axis(c.to_slab_fac, pos[3 * i + 2], M, &sz, &szz, &dz);
#define RG(a, b, cc) rho[((int64_t)(a) * dimy + (b)) * dimz + (cc)]
        RG(sx, sy, sz) = (float)(RG(sx, sy, sz) + m * (1.0 - dx) * (1.0 - dy) * (1.0 - dz));
        RG(sx, syy, sz) = (float)(RG(sx, syy, sz) + m * (1.0 - dx) * dy * (1.0 - dz));
        RG(sx, sy, szz) = (float)(RG(sx, sy, szz) + m * (1.0 - dx) * (1.0 - dy) * dz);
        RG(sx, syy, szz) = (float)(RG(sx, syy, szz) + m * (1.0 - dx) * dy * dz);
        RG(sxx, sy, sz) = (float)(RG(sxx, sy, sz) + m * dx * (1.0 - dy) * (1.0 - dz));
        RG(sxx, syy, sz) = (float)(RG(sxx, syy, sz) + m * dx * dy * (1.0 - dz));
        RG(sxx, sy, szz) = (float)(RG(sxx, sy, szz) + m * dx * (1.0 - dy) * dz);
        RG(sxx, syy, szz) = (float)(RG(sxx, syy, szz) + m * dx * dy * dz);
#undef RG
    }
    /* R2C (cuFFT layout: in place, unnormalised, forward e^{-i}) */
    dcpx *a = (dcpx *)malloc(sizeof(dcpx) * (size_t)M * M * M);
    for (int64_t xy = 0; xy < (int64_t)M * M; ++xy)
        for (int z = 0; z < M; ++z) {
            a[xy * M + z].re = rho[xy * dimz + z];
            a[xy * M + z].im = 0;
        }
    fft3(a, M, -1, nthreads);
    float *cg = rho; /* complex view of the same buffer, [M][M][Mh] */
    for (int64_t xy = 0; xy < (int64_t)M * M; ++xy)
        for (int z = 0; z < Mh; ++z) {
            cg[2 * (xy * Mh + z) + 0] = (float)a[xy * M + z].re;
            cg[2 * (xy * Mh + z) + 1] = (float)a[xy * M + z].im;
        }
    c.cgrid = cg;
    parallel_for((int64_t)M * M, nthreads, green_range, &c);
    cg[0] = cg[1] = 0.0f;
    /* C2R */
    for (int x = 0; x < M; ++x)
        for (int y = 0; y < M; ++y)
            for (int z = 0; z < M; ++z) {
                int64_t dst = ((int64_t)x * M + y) * M + z;
                if (z < Mh) {
                    int64_t s = ((int64_t)x * M + y) * Mh + z;
                    a[dst].re = cg[2 * s];
                    a[dst].im = cg[2 * s + 1];
                } else {
                    int64_t s = ((int64_t)((M - x) % M) * M + (M - y) % M) * Mh + (M - z);
                    a[dst].re = cg[2 * s];
                    a[dst].im = -cg[2 * s + 1];
                }
            }
    fft3(a, M, +1, nthreads);
    for (int64_t xy = 0; xy < (int64_t)M * M; ++xy)
        for (int z = 0; z < M; ++z) rho[xy * dimz + z] = (float)a[xy * M + z].re;
    free(a);
    /* FD4 gradient and CIC interpolation per dimension (pm_periodic.c:205-310) */
    float *force = (float *)malloc(sizeof(float) * (size_t)M * M * M);
    c.rho = rho;
    c.force = force;
    for (int dim = 0; dim < 3; ++dim) {
        c.dim = dim;
        parallel_for((int64_t)M * M, nthreads, fd4_range, &c);
        parallel_for(n, nthreads, interp_range, &c);
    }
    free(force);
    free(rho);
}

/* ------------------------------------------------------- drift/kick tables */

static double gl_x[20], gl_w[20];
static int gl_ready = 0;

static void gl_init(void) {
    const int n = 20;
    for (int i = 0; i < n; ++i) {
        double x = cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = x;
            for (int k = 2; k <= n; ++k) {
                double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (x * p1 - p0) / (x * x - 1.0);
            double dx = p1 / dp;
            x -= dx;
            if (fabs(dx) < 1e-16) break;
        }
        gl_x[i] = x;
        gl_w[i] = 2.0 / ((1.0 - x * x) * dp * dp);
    }
    gl_ready = 1;
}

typedef struct {
    double om, ol, hub;
    int power; /* integrand 1/(H a^power) */
} cosmo_fn;

static double integrand(const cosmo_fn *f, double a) {
    double h = f->om / (a * a * a) + (1 - f->om - f->ol) / (a * a) + f->ol;
    h = f->hub * sqrt(h);
    return f->power == 3 ? 1 / (h * a * a * a) : 1 / (h * a * a);
}

static double gl_rule(const cosmo_fn *f, double a, double b) {
    double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0.0;
    for (int i = 0; i < 20; ++i) s += gl_w[i] * integrand(f, c + h * gl_x[i]);
    return s * h;
}

static double gl_adapt(const cosmo_fn *f, double a, double b, double whole, double tol, int depth) {
    double c = 0.5 * (a + b);
    double l = gl_rule(f, a, c), r = gl_rule(f, c, b);
    if (depth > 40 || fabs(l + r - whole) <= tol) return l + r;
    return gl_adapt(f, a, c, l, 0.5 * tol, depth + 1) + gl_adapt(f, c, b, r, 0.5 * tol, depth + 1);
}

static double integrate(const cosmo_fn *f, double a, double b) {
    if (!gl_ready) gl_init();
    double whole = gl_rule(f, a, b);
    return gl_adapt(f, a, b, whole, 1e-13 * fabs(whole) + 1e-300, 0);
}

void op_drift_tables(double a0, double a1, double omega0, double omega_lambda, double hubble,
                     int n, double *drift, double *kick) {
    double l0 = log(a0), l1 = log(a1);
    cosmo_fn fd = {omega0, omega_lambda, hubble, 3}, fk = {omega0, omega_lambda, hubble, 2};
    for (int i = 0; i < n; ++i) {
        double b = exp(l0 + ((l1 - l0) / n) * (i + 1));
        drift[i] = integrate(&fd, exp(l0), b);
        kick[i] = integrate(&fk, exp(l0), b);
    }
}

double op_table_factor(const double *T, int n, double loga0, double loga1,
                       double timebase_interval, int t0, int t1) {
    double a1 = loga0 + t0 * timebase_interval, a2 = loga0 + t1 * timebase_interval;
    double u1 = (a1 - loga0) / (loga1 - loga0) * n, u2 = (a2 - loga0) / (loga1 - loga0) * n;
    int i1 = (int)u1, i2 = (int)u2;
    if (i1 >= n) i1 = n - 1;
    if (i2 >= n) i2 = n - 1;
    double df1 = i1 < 1 ? u1 * T[0] : T[i1 - 1] + (T[i1] - T[i1 - 1]) * (u1 - i1);
    double df2 = i2 < 1 ? u2 * T[0] : T[i2 - 1] + (T[i2] - T[i2 - 1]) * (u2 - i2);
    return df2 - df1;
}
