/* Oracle build shim implementations (test infrastructure only).
 *
 * This file is linked into the CPU build of the reference sources that the
 * oracle recipe (oracle/Makefile) makes under oracle/_ref/.  It supplies what
 * the reference links against but this image does not have:
 *   - CUDA runtime memory calls, backed by host memory (the reference's PM code
 *     round-trips its grid through "device" memory, pm_periodic.c:138-142,199-203);
 *   - cuFFT's 3D R2C / C2R transforms, computed on the CPU in double precision
 *     with cuFFT's conventions (unnormalised, forward e^{-i}, inverse e^{+i},
 *     in-place padded layout, pm_periodic.c:34-35,140,201);
 *   - GSL's gsl_integration_qag, as adaptive Gauss-Legendre (driftfac.c:31-37);
 *   - CUDPP plan calls and the GPU entry points of gravlist.cu, as stubs: the CPU
 *     oracle never runs the reference's device path (it does not build on CUDA 13).
 * Nothing here is part of the product; the product must never load this code. */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cuda_runtime_api.h"
#include "cufft.h"
#include "cudpp/cudpp.h"
#include "gsl/gsl_integration.h"

/* ------------------------------------------------------------------ threads */

static int g_threads = 1;

void cuco_ref_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int cuco_ref_get_threads(void) { return g_threads; }

/* ------------------------------------------------------------- CUDA runtime */

cudaError_t cudaMalloc(void **ptr, size_t size) {
    *ptr = calloc(size ? size : 1, 1);
    return *ptr ? 0 : 2;
}

cudaError_t cudaFree(void *ptr) {
    free(ptr);
    return 0;
}

cudaError_t cudaMemcpy(void *dst, const void *src, size_t size, enum cudaMemcpyKind kind) {
    (void)kind;
    if (dst != src) memmove(dst, src, size);
    return 0;
}

/* --------------------------------------------------------------------- FFT */

typedef struct { double re, im; } cpx;

typedef struct {
    int nx, ny, nz;
    int type;
} fft_plan;

#define MAX_PLANS 1024
static fft_plan g_plans[MAX_PLANS];
static int g_nplans = 0;

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

cufftResult cufftPlan3d(cufftHandle *plan, int nx, int ny, int nz, cufftType type) {
    if (g_nplans >= MAX_PLANS || !is_pow2(nx) || !is_pow2(ny) || !is_pow2(nz)) {
        fprintf(stderr, "oracle cuFFT shim: unsupported plan %dx%dx%d\n", nx, ny, nz);
        return 1;
    }
    g_plans[g_nplans].nx = nx;
    g_plans[g_nplans].ny = ny;
    g_plans[g_nplans].nz = nz;
    g_plans[g_nplans].type = (int)type;
    *plan = g_nplans++;
    return 0;
}

/* In-place iterative radix-2 transform of n points spaced `stride` apart. */
static void fft1d(cpx *a, int n, int stride, int sign, cpx *scratch) {
    int i, j, k, len;
    for (i = 0; i < n; ++i) scratch[i] = a[(size_t)i * stride];
    for (i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            cpx t = scratch[i];
            scratch[i] = scratch[j];
            scratch[j] = t;
        }
    }
    for (len = 2; len <= n; len <<= 1) {
        double ang = sign * 2.0 * M_PI / len;
        for (k = 0; k < len / 2; ++k) {
            double c = cos(ang * k), s = sin(ang * k);
            for (i = 0; i < n; i += len) {
                cpx u = scratch[i + k], v = scratch[i + k + len / 2];
                cpx w = {v.re * c - v.im * s, v.re * s + v.im * c};
                scratch[i + k].re = u.re + w.re;
                scratch[i + k].im = u.im + w.im;
                scratch[i + k + len / 2].re = u.re - w.re;
                scratch[i + k + len / 2].im = u.im - w.im;
            }
        }
    }
    for (i = 0; i < n; ++i) a[(size_t)i * stride] = scratch[i];
}

typedef struct {
    cpx *a;
    int nx, ny, nz, axis, sign, t, nt;
} fft_job;

static void *fft_axis_worker(void *arg) {
    fft_job *jb = (fft_job *)arg;
    int nx = jb->nx, ny = jb->ny, nz = jb->nz;
    int n = jb->axis == 0 ? nx : jb->axis == 1 ? ny : nz;
    cpx *scratch = (cpx *)malloc(sizeof(cpx) * n);
    long lines = jb->axis == 0 ? (long)ny * nz : jb->axis == 1 ? (long)nx * nz : (long)nx * ny;
    for (long l = jb->t; l < lines; l += jb->nt) {
        cpx *base;
        int stride;
        if (jb->axis == 0) {
            base = jb->a + l; /* l = y*nz+z */
            stride = ny * nz;
        } else if (jb->axis == 1) {
            long x = l / nz, z = l % nz;
            base = jb->a + (size_t)x * ny * nz + z;
            stride = nz;
        } else {
            base = jb->a + (size_t)l * nz;
            stride = 1;
        }
        fft1d(base, n, stride, jb->sign, scratch);
    }
    free(scratch);
    return NULL;
}

static void fft3d(cpx *a, int nx, int ny, int nz, int sign) {
    int nt = g_threads;
    pthread_t th[256];
    fft_job jobs[256];
    if (nt > 256) nt = 256;
    for (int axis = 2; axis >= 0; --axis) {
        for (int t = 0; t < nt; ++t) {
            jobs[t].a = a;
            jobs[t].nx = nx;
            jobs[t].ny = ny;
            jobs[t].nz = nz;
            jobs[t].axis = axis;
            jobs[t].sign = sign;
            jobs[t].t = t;
            jobs[t].nt = nt;
            if (nt > 1)
                pthread_create(&th[t], NULL, fft_axis_worker, &jobs[t]);
            else
                fft_axis_worker(&jobs[t]);
        }
        if (nt > 1)
            for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
    }
}

cufftResult cufftExecR2C(cufftHandle plan, cufftReal *idata, cufftComplex *odata) {
    fft_plan p = g_plans[plan];
    int nx = p.nx, ny = p.ny, nz = p.nz, nzh = nz / 2 + 1, nzp = 2 * nzh;
    cpx *a = (cpx *)malloc(sizeof(cpx) * (size_t)nx * ny * nz);
    for (long xy = 0; xy < (long)nx * ny; ++xy)
        for (int z = 0; z < nz; ++z) {
            a[xy * nz + z].re = idata[xy * nzp + z];
            a[xy * nz + z].im = 0.0;
        }
    fft3d(a, nx, ny, nz, -1);
    for (long xy = 0; xy < (long)nx * ny; ++xy)
        for (int z = 0; z < nzh; ++z) {
            odata[xy * nzh + z].x = (float)a[xy * nz + z].re;
            odata[xy * nzh + z].y = (float)a[xy * nz + z].im;
        }
    free(a);
    return 0;
}

cufftResult cufftExecC2R(cufftHandle plan, cufftComplex *idata, cufftReal *odata) {
    fft_plan p = g_plans[plan];
    int nx = p.nx, ny = p.ny, nz = p.nz, nzh = nz / 2 + 1, nzp = 2 * nzh;
    cpx *a = (cpx *)malloc(sizeof(cpx) * (size_t)nx * ny * nz);
    for (int x = 0; x < nx; ++x)
        for (int y = 0; y < ny; ++y)
            for (int z = 0; z < nz; ++z) {
                long dst = ((long)x * ny + y) * nz + z;
                if (z < nzh) {
                    cufftComplex c = idata[((long)x * ny + y) * nzh + z];
                    a[dst].re = c.x;
                    a[dst].im = c.y;
                } else { /* Hermitian extension of the half spectrum */
                    int xs = (nx - x) % nx, ys = (ny - y) % ny;
                    cufftComplex c = idata[((long)xs * ny + ys) * nzh + (nz - z)];
                    a[dst].re = c.x;
                    a[dst].im = -c.y;
                }
            }
    fft3d(a, nx, ny, nz, +1);
    for (long xy = 0; xy < (long)nx * ny; ++xy)
        for (int z = 0; z < nz; ++z) odata[xy * nzp + z] = (float)a[xy * nz + z].re;
    free(a);
    return 0;
}

/* ------------------------------------------------------------------- CUDPP */

CUDPPResult cudppPlan(CUDPPHandle *plan, CUDPPConfiguration config, size_t n, size_t rows, size_t pitch) {
    (void)config;
    (void)n;
    (void)rows;
    (void)pitch;
    *plan = 1;
    return 0;
}

CUDPPResult cudppDestroyPlan(CUDPPHandle plan) {
    (void)plan;
    return 0;
}

/* --------------------------------------------------------------------- GSL */

static double gl_x[20], gl_w[20];
static int gl_ready = 0;

/* 20-point Gauss-Legendre nodes and weights by Newton iteration on P_20. */
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

static double gl_rule(const gsl_function *f, double a, double b) {
    double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0.0;
    for (int i = 0; i < 20; ++i) s += gl_w[i] * f->function(c + h * gl_x[i], f->params);
    return s * h;
}

static double gl_adapt(const gsl_function *f, double a, double b, double whole, double tol, int depth) {
    double c = 0.5 * (a + b);
    double l = gl_rule(f, a, c), r = gl_rule(f, c, b);
    if (depth > 40 || fabs(l + r - whole) <= tol) return l + r;
    return gl_adapt(f, a, c, l, 0.5 * tol, depth + 1) + gl_adapt(f, c, b, r, 0.5 * tol, depth + 1);
}

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n) {
    gsl_integration_workspace *w = (gsl_integration_workspace *)malloc(sizeof(*w));
    w->limit = n;
    return w;
}

void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }

int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs,
                        double epsrel, size_t limit, int key,
                        gsl_integration_workspace *workspace, double *result,
                        double *abserr) {
    (void)epsabs;
    (void)epsrel;
    (void)limit;
    (void)key;
    (void)workspace;
    if (!gl_ready) gl_init();
    double whole = gl_rule(f, a, b);
    /* Integrate to 1e-13 relative regardless of the caller's (looser) request. */
    double res = gl_adapt(f, a, b, whole, 1e-13 * fabs(whole) + 1e-300, 0);
    *result = res;
    *abserr = 1e-13 * fabs(res);
    return 0;
}

/* ------------------------------------------- gravlist.cu entry points (stubs) */

void *sorter = 0; /* `RadixSort *sorter`, gravlist.cu:20 */

static void gpu_path_unavailable(const char *name) {
    fprintf(stderr, "oracle build: %s is part of the reference's GPU path, which the CPU oracle does not run\n", name);
    abort();
}

void cudaInit(void) {}
void allocateArray(void **devPtr, size_t size) { cudaMalloc(devPtr, size); }
void freeArray(void *devPtr) { free(devPtr); }
void copyArrayFromDevice(void *host, void *device, int size) { memmove(host, device, (size_t)size); }
void copyArrayToDevice(void *device, void *host, int offset, int size) {
    memmove((char *)device + offset, host, (size_t)size);
}

static unsigned char g_simparam[8192];
static unsigned char g_softparam[64];
void setSimParam(void *p) { memcpy(g_simparam, p, 4 * 1000 + 9 * 4); }
void setSoftParam(void *p) { memcpy(g_softparam, p, 3 * 4); }
const void *cuco_ref_simparam(void) { return g_simparam; }
const void *cuco_ref_softparam(void) { return g_softparam; }

void copyPosToDevice(void) { gpu_path_unavailable("copyPosToDevice"); }
void copyAccelFromDevice(void) { gpu_path_unavailable("copyAccelFromDevice"); }
void calcHash(void) { gpu_path_unavailable("calcHash"); }
void reorderDataAndFindCellStart(void) { gpu_path_unavailable("reorderDataAndFindCellStart"); }
void cudaForceEvaluateShortrange(void) { gpu_path_unavailable("cudaForceEvaluateShortrange"); }
void radixSort(void) { gpu_path_unavailable("radixSort"); }
void radixSortKeysOnly(void) { gpu_path_unavailable("radixSortKeysOnly"); }
void radixSortFloatKeys(void) { gpu_path_unavailable("radixSortFloatKeys"); }
void radixSortFloatKeysOnly(void) { gpu_path_unavailable("radixSortFloatKeysOnly"); }
void initDeviceParameters(void) {}
void checkCudaError(const char *msg) { (void)msg; }
