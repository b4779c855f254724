// Long-range PM force: CIC deposit, 3D real FFT with the Green's function,
// FD4 gradient and CIC interpolation, all on the device.
//
// Reference: pmforce_periodic (pm_periodic.c:67-314), which deposits and
// interpolates on the host and round-trips the grid through cuFFT.  Here:
//   k_deposit      CIC mass assignment (pm_periodic.c:97-132): each weight as
//                  the integer w * 2^32, added with 64-bit integer atomics into
//                  an M^3 grid, so the grid is the same whatever order the
//                  particles land in (float atomics are not associative).  One
//                  box deposits in original particle order (it runs beside the
//                  sort), the ensemble cell-sorted.
//   k_fft_z_r2c    real->complex along z; its load converts the integer sums to
//                  mass (one rounding) and writes zero back, so the grid is
//                  clean for the next deposit.  Two real rows are packed as the
//                  real and imaginary parts of one complex row, transformed
//                  together and separated (X1 = (Z + conj Z_-k)/2,
//                  X2 = (Z - conj Z_-k)/2i).
//   k_fft_axis     complex transforms along y, and along x fused with the
//                  Green's-function multiply and the inverse x transform: the
//                  x pass is the last forward and the first inverse pass, so the
//                  spectrum is multiplied in shared memory and never stored.
//   k_fft_z_c2r    the inverse of k_fft_z_r2c (Hermitian extension of each row,
//                  imaginary parts of the self-conjugate points dropped).
//   k_interp       the FD4 gradient of the potential (pm_periodic.c:205-270) at
//                  the 8 CIC corners of each particle and the CIC interpolation
//                  (pm_periodic.c:272-309), fused: the three force grids the
//                  reference builds are never materialised.
// All transforms are unnormalised with cuFFT's sign conventions.  Power-of-two
// meshes up to 1024 use a two-level transform with the points in registers
// (RegFFT; the one-box axis passes with their column batch fixed at compile
// time, fft_axis_reg_fixed); other meshes M = 2^a 3^b 5^c use a shared-memory
// Stockham FFT over a batch of columns with radix-4/2/3/5 stages.  Twiddles
// come from an FP64-built table.
// The Green's function factorises: smth(k) = -g(kx) g(ky) g(kz) / k^2 with
// g(k) = exp(-k^2 (2 pi asmth / L)^2) / sinc(pi k / M)^4, built in FP64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace cuco {

namespace {

constexpr int kFFTThreads = 256;
constexpr int kLoadBatch = 8;  // global loads issued per thread before use

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Stage radix for the remaining length: 4, 2, 3 or 5 (M = 2^a 3^b 5^c).
__host__ __device__ __forceinline__ int stage_radix(int rem) {
    return (rem & 3) == 0 ? 4 : (rem & 1) == 0 ? 2 : rem % 3 == 0 ? 3 : 5;
}

// Division by a runtime d without a divide instruction: j / d is
// umulhi(j, ceil(2^32 / d)), exact for j, d < 2^16 (checked exhaustively for
// d <= 2048; every index here is below 2^16).
struct FastDiv {
    uint32_t d, inv;
    __device__ __forceinline__ explicit FastDiv(uint32_t d_) : d(d_), inv(d_ > 1 ? (uint32_t)((0x100000000ull + d_ - 1) / d_) : 0u) {}
    __device__ __forceinline__ uint32_t div(uint32_t j) const { return d > 1 ? __umulhi(j, inv) : j; }
};

template <int R>
__device__ __forceinline__ void dft_small(float2 (&v)[R], int sign) {
    if (R == 4) {
        const float2 a0 = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
        const float2 a1 = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
        const float2 a2 = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
        const float2 d = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
        // (v1 - v3) * (sign * i)
        const float2 a3 = sign < 0 ? make_float2(d.y, -d.x) : make_float2(-d.y, d.x);
        v[0] = make_float2(a0.x + a2.x, a0.y + a2.y);
        v[1] = make_float2(a1.x + a3.x, a1.y + a3.y);
        v[2] = make_float2(a0.x - a2.x, a0.y - a2.y);
        v[3] = make_float2(a1.x - a3.x, a1.y - a3.y);
    } else if (R == 2) {
        const float2 a = v[0], b = v[1];
        v[0] = make_float2(a.x + b.x, a.y + b.y);
        v[1] = make_float2(a.x - b.x, a.y - b.y);
    } else if (R == 3) {
        // y1,2 = v0 - (v1+v2)/2 +- i s (v1-v2), s = sign sqrt(3)/2
        const float s3 = sign * 0.866025403784438647f;
        const float2 t = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
        const float2 d = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
        const float2 m = make_float2(v[0].x - 0.5f * t.x, v[0].y - 0.5f * t.y);
        v[0] = make_float2(v[0].x + t.x, v[0].y + t.y);
        v[1] = make_float2(m.x - s3 * d.y, m.y + s3 * d.x);
        v[2] = make_float2(m.x + s3 * d.y, m.y - s3 * d.x);
    } else {
        // five-point DFT by the conjugate pairs (1,4), (2,3)
        const float c1 = 0.309016994374947424f, c2 = -0.809016994374947424f;
        const float s1 = sign * 0.951056516295153572f, s2 = sign * 0.587785252292473129f;
        const float2 a1 = make_float2(v[1].x + v[R - 1].x, v[1].y + v[R - 1].y);
        const float2 b1 = make_float2(v[1].x - v[R - 1].x, v[1].y - v[R - 1].y);
        const float2 a2 = make_float2(v[2].x + v[R - 2].x, v[2].y + v[R - 2].y);
        const float2 b2 = make_float2(v[2].x - v[R - 2].x, v[2].y - v[R - 2].y);
        const float2 t1 = make_float2(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
        const float2 t2 = make_float2(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
        const float2 u1 = make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
        const float2 u2 = make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
        v[0] = make_float2(v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y);
        v[1] = make_float2(t1.x - u1.y, t1.y + u1.x);      // t1 + i u1
        v[2] = make_float2(t2.x - u2.y, t2.y + u2.x);      // t2 + i u2
        v[R - 2] = make_float2(t2.x + u2.y, t2.y - u2.x);  // t2 - i u2
        v[R - 1] = make_float2(t1.x + u1.y, t1.y - u1.x);  // t1 - i u1
    }
}

// One Stockham stage of radix R over Ns already-combined points, for B = 2^bs
// columns: reads x[j + p M/R] (p < R), twiddles it by w^{p k M/(Ns R)} (k = j
// mod Ns), and writes the R-point DFT to y[(j/Ns) Ns R + k + q Ns].
template <int R>
__device__ __forceinline__ void stockham_stage(const float2 *in, float2 *out, const float2 *tw, int M, int Ns,
                                               int bs, int pitch, int sign) {
    const int nb = M / R, step = M / (Ns * R);
    const FastDiv dns((uint32_t)Ns);
    const int total = nb << bs, bmask = (1 << bs) - 1;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int b = e & bmask, j = e >> bs;
        const int g = (int)dns.div((uint32_t)j), k = j - g * Ns;
        const int dst = g * Ns * R + k;
        float2 v[R];
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = in[(j + q * nb) * pitch + b];
        if (k) {
#pragma unroll
            for (int q = 1; q < R; ++q) {
                float2 w = tw[q * k * step];
                if (sign > 0) w.y = -w.y;
                v[q] = cmul(v[q], w);
            }
        }
        dft_small<R>(v, sign);
#pragma unroll
        for (int q = 0; q < R; ++q) out[(dst + q * Ns) * pitch + b] = v[q];
    }
}

// Transform B = 2^bs columns of length M held in x[m*pitch + b]; returns the
// buffer holding the result.  sign = -1: forward (e^{-i}), +1: inverse.
__device__ float2 *fft_columns(float2 *x, float2 *y, const float2 *tw, int M, int bs, int pitch, int sign) {
    int Ns = 1;
    float2 *in = x, *out = y;
    while (Ns < M) {
        const int r = stage_radix(M / Ns);
        switch (r) {
            case 4: stockham_stage<4>(in, out, tw, M, Ns, bs, pitch, sign); break;
            case 2: stockham_stage<2>(in, out, tw, M, Ns, bs, pitch, sign); break;
            case 3: stockham_stage<3>(in, out, tw, M, Ns, bs, pitch, sign); break;
            default: stockham_stage<5>(in, out, tw, M, Ns, bs, pitch, sign); break;
        }
        __syncthreads();
        float2 *t = in;
        in = out;
        out = t;
        Ns *= r;
    }
    return in;
}

__host__ __device__ constexpr int ilog2(int v) {
    int l = 0;
    while ((1 << (l + 1)) <= v) ++l;
    return l;
}

__device__ __forceinline__ void load_twiddles(float2 *tw_s, const float2 *tw, int M) {
    for (int i = threadIdx.x; i < M; i += blockDim.x) tw_s[i] = tw[i];
}

// ------------------------------------------------ register transforms
// Power-of-two meshes M = M1 * M2 (M1, M2 <= 32) take a two-level
// Cooley-Tukey transform with the points in registers: one DFT over M1
// points strided by M2, a twiddle, one shared-memory exchange, one DFT over
// M2 contiguous points.  Each column is handled by max(M1, M2) threads and
// visits shared memory twice instead of once per radix-4 stage.  The
// forward transform leaves X[k] in slot M2 (k mod M1) + k / M1; the inverse
// starts from that layout and ends in natural order, so a forward pass, a
// multiply and an inverse pass (the x pass with the Green's function) need
// no reordering in between.

// cos and sin of 2 pi j / 32, j < 32
__host__ __device__ constexpr float cos32(int j) {
    constexpr float c[32] = {1.0f, 9.807852804e-01f, 9.238795325e-01f, 8.314696123e-01f, 7.071067812e-01f,
                             5.555702330e-01f, 3.826834324e-01f, 1.950903220e-01f, 0.0f, -1.950903220e-01f,
                             -3.826834324e-01f, -5.555702330e-01f, -7.071067812e-01f, -8.314696123e-01f,
                             -9.238795325e-01f, -9.807852804e-01f, -1.0f, -9.807852804e-01f, -9.238795325e-01f,
                             -8.314696123e-01f, -7.071067812e-01f, -5.555702330e-01f, -3.826834324e-01f,
                             -1.950903220e-01f, 0.0f, 1.950903220e-01f, 3.826834324e-01f, 5.555702330e-01f,
                             7.071067812e-01f, 8.314696123e-01f, 9.238795325e-01f, 9.807852804e-01f};
    return c[j & 31];
}
__host__ __device__ constexpr float sin32(int j) { return cos32(j - 8); }

// exp(S 2 pi i m / N) for N dividing 32
template <int N, int S>
__device__ __forceinline__ float2 wconst(int m) {
    const int j = (m * (32 / N)) & 31;
    return make_float2(cos32(j), S * sin32(j));
}

// In-register DFT of N = 2^a <= 32 points, X[k] = sum_n v[n] exp(S 2 pi i n k / N),
// as radix-4 Cooley-Tukey (N = 4 Q: DFTs over n1 of v[Q n1 + n2], twiddle,
// DFTs over n2; X[k1 + 4 k2]).  All indices are compile-time constants.
template <int N, int S>
__device__ __forceinline__ void dft_reg(float2 (&v)[N]) {
    if constexpr (N == 2) {
        const float2 a = v[0], b = v[1];
        v[0] = make_float2(a.x + b.x, a.y + b.y);
        v[1] = make_float2(a.x - b.x, a.y - b.y);
    } else if constexpr (N == 4) {
        dft_small<4>(v, S);
    } else {
        constexpr int Q = N / 4;
        float2 w[N];
#pragma unroll
        for (int n2 = 0; n2 < Q; ++n2) {
            float2 t[4] = {v[n2], v[n2 + Q], v[n2 + 2 * Q], v[n2 + 3 * Q]};
            dft_small<4>(t, S);
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) w[Q * k1 + n2] = (n2 * k1) ? cmul(t[k1], wconst<N, S>(n2 * k1)) : t[k1];
        }
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            float2 u[Q];
#pragma unroll
            for (int j = 0; j < Q; ++j) u[j] = w[Q * k1 + j];
            dft_reg<Q, S>(u);
#pragma unroll
            for (int k2 = 0; k2 < Q; ++k2) v[k1 + 4 * k2] = u[k2];
        }
    }
}

template <int M1, int M2>
struct RegFFT {
    static constexpr int M = M1 * M2, N1 = M1, N2 = M2;
    // a column takes max(M1, M2) threads
    __device__ static int slot(int k) { return M2 * (k & (M1 - 1)) + k / M1; }
    // twiddle exp(S 2 pi i j / M) from the table of exp(-2 pi i j / M)
    template <int S>
    __device__ static float2 tw(const float2 *tw_s, int j) {
        float2 w = tw_s[j];
        if (S > 0) w.y = -w.y;
        return w;
    }
    // the 2^lb columns x[m * pitch + b]: natural order in, slot order out
    template <int S>
    __device__ static void forward(float2 *x, const float2 *tw_s, int pitch, int lb) {
        const int b = threadIdx.x & ((1 << lb) - 1), r = threadIdx.x >> lb;
        if (r < M2) {
            const int n2 = r;
            float2 v[M1];
#pragma unroll
            for (int n1 = 0; n1 < M1; ++n1) v[n1] = x[(M2 * n1 + n2) * pitch + b];
            dft_reg<M1, S>(v);
#pragma unroll
            for (int k1 = 0; k1 < M1; ++k1)
                x[(M2 * k1 + n2) * pitch + b] = k1 ? cmul(v[k1], tw<S>(tw_s, n2 * k1)) : v[k1];
        }
        __syncthreads();
        if (r < M1) {
            const int k1 = r;
            float2 u[M2];
#pragma unroll
            for (int n2 = 0; n2 < M2; ++n2) u[n2] = x[(M2 * k1 + n2) * pitch + b];
            dft_reg<M2, S>(u);
#pragma unroll
            for (int k2 = 0; k2 < M2; ++k2) x[(M2 * k1 + k2) * pitch + b] = u[k2];
        }
        __syncthreads();
    }
    // slot order in, natural order out
    template <int S>
    __device__ static void inverse(float2 *x, const float2 *tw_s, int pitch, int lb) {
        const int b = threadIdx.x & ((1 << lb) - 1), r = threadIdx.x >> lb;
        if (r < M1) {
            const int k1 = r;
            float2 u[M2];
#pragma unroll
            for (int k2 = 0; k2 < M2; ++k2) u[k2] = x[(M2 * k1 + k2) * pitch + b];
            dft_reg<M2, S>(u);
#pragma unroll
            for (int n2 = 0; n2 < M2; ++n2)
                x[(M2 * k1 + n2) * pitch + b] = k1 ? cmul(u[n2], tw<S>(tw_s, n2 * k1)) : u[n2];
        }
        __syncthreads();
        if (r < M2) {
            const int n2 = r;
            float2 v[M1];
#pragma unroll
            for (int k1 = 0; k1 < M1; ++k1) v[k1] = x[(M2 * k1 + n2) * pitch + b];
            dft_reg<M1, S>(v);
#pragma unroll
            for (int n1 = 0; n1 < M1; ++n1) x[(M2 * n1 + n2) * pitch + b] = v[n1];
        }
        __syncthreads();
    }
};

// Whether M takes the register transforms with `cols` columns per CTA (the
// one-box and many-box passes decide alike, so a box's transform is the same
// in both).  512 and 1024 use 32-point register DFTs, which need twice the
// registers: the many-box passes run those boxes in kernels of their own.
__host__ __device__ inline bool reg_fft_ok(int M, int cols) {
    int T;
    switch (M) {
        case 16: T = 4; break;
        case 32: T = 8; break;
        case 64: T = 8; break;
        case 128: T = 16; break;
        case 256: T = 16; break;
        case 512: T = 32; break;
        case 1024: T = 32; break;
        default: return false;
    }
    return T * cols <= kFFTThreads;
}

// The passes below with the register transforms (M = FT::M; one buffer of
// M * pitch points, the twiddle table after it).
template <typename FT>
__device__ __forceinline__ void fft_z_r2c_reg(unsigned long long *__restrict__ rho64, float mscale,
                                              float2 *__restrict__ spec, const float2 *tw, int P, int blk) {
    constexpr int M = FT::M, Mh = M / 2 + 1;
    extern __shared__ float2 sm[];
    const int pitch = P + 1;
    float2 *x = sm, *tw_s = sm + M * pitch;
    const size_t r0 = (size_t)blk * 2 * P;
    load_twiddles(tw_s, tw, M);
    // rows 2pr and 2pr+1 packed as one complex column, one float2 per thread
    // and element (both reads coalesced along the rows); every sum read is
    // cleared for the next deposit
    for (int e0 = threadIdx.x; e0 < P * M; e0 += kLoadBatch * blockDim.x) {
        float2 v[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int e = e0 + u * blockDim.x;
            v[u] = make_float2(0.f, 0.f);
            if (e < P * M) {
                const int pr = e / M, m = e & (M - 1);
                const size_t g = (r0 + 2 * pr) * M + m;
                v[u] = make_float2(__fmul_rn(__ull2float_rn(rho64[g]), mscale),
                                   __fmul_rn(__ull2float_rn(rho64[g + M]), mscale));
            }
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int e = e0 + u * blockDim.x;
            if (e < P * M) {
                const int pr = e / M, m = e & (M - 1);
                const size_t g = (r0 + 2 * pr) * M + m;
                rho64[g] = 0ull;
                rho64[g + M] = 0ull;
                x[m * pitch + pr] = v[u];
            }
        }
    }
    __syncthreads();
    const int ps = ilog2(P);
    FT::template forward<-1>(x, tw_s, pitch, ps);
    // Both rows of a pair from the same two transform values, columns
    // fastest (consecutive banks), into the row-major block y (after the
    // twiddles; 2P (M/2+1) <= M (P+1) points as P <= M/2); then the block
    // goes out whole: the CTA's 2P spectrum rows are contiguous.
    float2 *y = tw_s + M;
    for (int e = threadIdx.x; e < P * Mh; e += blockDim.x) {
        const int pr = e & (P - 1), k = e >> ps;
        const float2 z = x[FT::slot(k) * pitch + pr];
        float2 zc = x[FT::slot((M - k) & (M - 1)) * pitch + pr];
        zc.y = -zc.y;
        y[(2 * pr) * Mh + k] = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y));
        // (z - zc) / (2i)
        y[(2 * pr + 1) * Mh + k] = make_float2(0.5f * (z.y - zc.y), -0.5f * (z.x - zc.x));
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * P * Mh; e += blockDim.x) spec[r0 * Mh + e] = y[e];
}

template <typename FT>
__device__ __forceinline__ void fft_z_c2r_reg(const float2 *__restrict__ spec, float *__restrict__ out,
                                              const float2 *tw, int P, int blk) {
    constexpr int M = FT::M, Mh = M / 2 + 1;
    extern __shared__ float2 sm[];
    const int pitch = P + 1;
    float2 *x = sm, *tw_s = sm + M * pitch;
    const size_t r0 = (size_t)blk * 2 * P;
    load_twiddles(tw_s, tw, M);
    // the CTA's 2P spectrum rows, contiguous, into the row-major block y
    float2 *y = tw_s + M;
    for (int e0 = threadIdx.x; e0 < 2 * P * Mh; e0 += kLoadBatch * blockDim.x) {
        float2 v[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int e = e0 + u * blockDim.x;
            v[u] = e < 2 * P * Mh ? spec[r0 * Mh + e] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int e = e0 + u * blockDim.x;
            if (e < 2 * P * Mh) y[e] = v[u];
        }
    }
    __syncthreads();
    // row pair pr packed as one complex column a + i b (a, b the Hermitian
    // rows 2pr and 2pr+1, imaginary parts at k = 0 and M/2 dropped), placed
    // in the slot order the inverse transform starts from; columns fastest
    const int ps = ilog2(P);
    for (int e = threadIdx.x; e < P * M; e += blockDim.x) {
        const int pr = e & (P - 1), k = e >> ps;
        const int kk = k <= M / 2 ? k : M - k;
        float2 a = y[(2 * pr) * Mh + kk], b = y[(2 * pr + 1) * Mh + kk];
        if (k == 0 || k == M / 2) a.y = b.y = 0.f;
        if (k > M / 2) a.y = -a.y, b.y = -b.y;
        x[FT::slot(k) * pitch + pr] = make_float2(a.x - b.y, a.y + b.x);  // a + i b
    }
    __syncthreads();
    FT::template inverse<+1>(x, tw_s, pitch, ilog2(P));
    // the pair's two real rows from one transform value
    for (int e = threadIdx.x; e < P * M; e += blockDim.x) {
        const int pr = e / M, m = e & (M - 1);
        const float2 z = x[m * pitch + pr];
        out[(r0 + 2 * pr) * M + m] = z.x;
        out[(r0 + 2 * pr + 1) * M + m] = z.y;
    }
}

template <typename FT>
__device__ __forceinline__ void fft_axis_reg(float2 *__restrict__ spec, const float2 *tw,
                                             const float *__restrict__ green1d, int B, int axis, int sign,
                                             int green, int bx, int by) {
    constexpr int M = FT::M, Mh = M / 2 + 1;
    extern __shared__ float2 sm[];
    const int pitch = B;
    float2 *x = sm, *tw_s = sm + M * pitch;
    const int o = by, kz0 = bx * B, bsh = ilog2(B), nb = min(B, Mh - kz0);
    const size_t sm_stride = axis == 1 ? (size_t)Mh : (size_t)M * Mh;
    const size_t base = axis == 1 ? (size_t)o * M * Mh : (size_t)o * Mh;
    // an inverse-only pass starts from the slot order
    const bool to_slots = sign > 0;
    load_twiddles(tw_s, tw, M);
    for (int e0 = threadIdx.x; e0 < M * B; e0 += kLoadBatch * blockDim.x) {
        float2 v[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int e = e0 + u * blockDim.x;
            const int m = e >> bsh, b = e & (B - 1);
            v[u] = (e < M * B && b < nb) ? spec[base + m * sm_stride + kz0 + b] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int e = e0 + u * blockDim.x;
            if (e < M * B) {
                const int m = e >> bsh, b = e & (B - 1);
                x[(to_slots ? FT::slot(m) : m) * pitch + b] = v[u];
            }
        }
    }
    __syncthreads();
    bool natural = true;
    if (sign < 0) {
        FT::template forward<-1>(x, tw_s, pitch, bsh);
        natural = false;
        if (green) {
            // slot s = M2 k1 + k2 holds X[k1 + M1 k2]
            const int ky = o <= M / 2 ? o : M - o;
            const float gy = green1d[ky];
            for (int e = threadIdx.x; e < M * B; e += blockDim.x) {
                const int sl = e >> bsh, b = e & (B - 1);
                const int k1 = sl / FT::N2, k2 = sl - k1 * FT::N2;
                const int m = k1 + FT::N1 * k2;  // the transform index along x
                const int kx = m <= M / 2 ? m : M - m;
                const int kz = kz0 + b;
                const float2 v = x[sl * pitch + b];
                float g = 0.f;
                if (b < nb) {
                    const int k2s = kx * kx + ky * ky + kz * kz;
                    if (k2s > 0) g = -green1d[kx] * gy * green1d[kz] * __frcp_rn((float)k2s);
                }
                x[sl * pitch + b] = make_float2(v.x * g, v.y * g);
            }
            __syncthreads();
            FT::template inverse<+1>(x, tw_s, pitch, bsh);
            natural = true;
        }
    } else {
        FT::template inverse<+1>(x, tw_s, pitch, bsh);
    }
    for (int e = threadIdx.x; e < M * B; e += blockDim.x) {
        const int m = e >> bsh, b = e & (B - 1);
        if (b < nb) spec[base + m * sm_stride + kz0 + b] = x[(natural ? m : FT::slot(m)) * pitch + b];
    }
}

// rows r0 .. r0+2P-1 of the M^3 real grid (row = x*M + y) -> spectrum rows
__device__ __forceinline__ void fft_z_r2c(unsigned long long *__restrict__ rho64, float mscale,
                                          float2 *__restrict__ spec, const float2 *tw, int M, int P, int blk) {
    extern __shared__ float2 sm[];
    const int pitch = P + 1;
    float2 *x = sm, *y = sm + M * pitch, *tw_s = sm + 2 * M * pitch;
    const int Mh = M / 2 + 1;
    const size_t r0 = (size_t)blk * 2 * P;
    const FastDiv dM((uint32_t)M), dMh((uint32_t)Mh);
    const int ps = ilog2(P);  // P is a power of two
    load_twiddles(tw_s, tw, M);
    // kLoadBatch loads in flight per thread before their shared-memory stores
    for (int e0 = threadIdx.x; e0 < 2 * P * M; e0 += kLoadBatch * blockDim.x) {
        float v[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            int e = e0 + u * blockDim.x;
            // the deposit's exact integer sums, rounded once to float
            v[u] = e < 2 * P * M ? __fmul_rn(__ull2float_rn(rho64[r0 * M + e]), mscale) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            int e = e0 + u * blockDim.x;
            if (e < 2 * P * M) {
                rho64[r0 * M + e] = 0ull;  // cleared for the next deposit
                const int row = (int)dM.div((uint32_t)e), m = e - row * M;
                float *slot = reinterpret_cast<float *>(&x[m * pitch + (row >> 1)]);
                slot[row & 1] = v[u];
            }
        }
    }
    __syncthreads();
    float2 *res = fft_columns(x, y, tw_s, M, ps, pitch, -1);
    for (int e = threadIdx.x; e < 2 * P * Mh; e += blockDim.x) {
        const int row = (int)dMh.div((uint32_t)e), k = e - row * Mh, pr = row >> 1;
        float2 z = res[k * pitch + pr];
        float2 zc = res[((M - k) % M) * pitch + pr];
        zc.y = -zc.y;
        float2 o;
        if ((row & 1) == 0)
            o = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y));
        else  // (z - zc) / (2i)
            o = make_float2(0.5f * (z.y - zc.y), -0.5f * (z.x - zc.x));
        spec[(r0 + row) * Mh + k] = o;
    }
}

__device__ __forceinline__ void fft_z_c2r(const float2 *__restrict__ spec, float *__restrict__ out,
                                          const float2 *tw, int M, int P, int blk) {
    extern __shared__ float2 sm[];
    const int pitch = P + 1;
    float2 *x = sm, *y = sm + M * pitch, *tw_s = sm + 2 * M * pitch;
    const int Mh = M / 2 + 1;
    const size_t r0 = (size_t)blk * 2 * P;
    const FastDiv dM((uint32_t)M), dMh((uint32_t)Mh);
    const int ps = ilog2(P);  // P is a power of two
    load_twiddles(tw_s, tw, M);
    // rows into y as h[row*Mh + k]
    for (int e0 = threadIdx.x; e0 < 2 * P * Mh; e0 += kLoadBatch * blockDim.x) {
        float2 v[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            int e = e0 + u * blockDim.x;
            v[u] = e < 2 * P * Mh ? spec[r0 * Mh + e] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            int e = e0 + u * blockDim.x;
            if (e < 2 * P * Mh) {
                const int k = e - (int)dMh.div((uint32_t)e) * Mh;
                if (k == 0 || k == M / 2) v[u].y = 0.f;
                y[e] = v[u];
            }
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < P * M; e += blockDim.x) {
        const int pr = e & (P - 1), k = e >> ps;
        float2 a, b;
        if (k <= M / 2) {
            a = y[(2 * pr) * Mh + k];
            b = y[(2 * pr + 1) * Mh + k];
        } else {
            a = y[(2 * pr) * Mh + (M - k)];
            b = y[(2 * pr + 1) * Mh + (M - k)];
            a.y = -a.y;
            b.y = -b.y;
        }
        x[k * pitch + pr] = make_float2(a.x - b.y, a.y + b.x);  // a + i b
    }
    __syncthreads();
    float2 *res = fft_columns(x, y, tw_s, M, ps, pitch, +1);
    for (int e = threadIdx.x; e < 2 * P * M; e += blockDim.x) {
        const int row = (int)dM.div((uint32_t)e), m = e - row * M;
        float2 z = res[m * pitch + (row >> 1)];
        out[(r0 + row) * M + m] = (row & 1) ? z.y : z.x;
    }
}

// axis 1: y transform for fixed x = by; axis 0: x transform for fixed y = by,
// with the Green's multiply and inverse transform when green != 0; columns
// kz0 = bx * B ...
__device__ __forceinline__ void fft_axis(float2 *__restrict__ spec, const float2 *tw,
                                         const float *__restrict__ green1d, int M, int B, int axis,
                                         int sign, int green, int bx, int by) {
    extern __shared__ float2 sm[];
    const int pitch = B;
    float2 *x = sm, *y = sm + M * pitch, *tw_s = sm + 2 * M * pitch;
    const int Mh = M / 2 + 1;
    const int o = by;
    const int kz0 = bx * B;
    const int bsh = ilog2(B);  // B is a power of two
    const int nb = min(B, Mh - kz0);
    const size_t sm_stride = axis == 1 ? (size_t)Mh : (size_t)M * Mh;
    const size_t base = axis == 1 ? (size_t)o * M * Mh : (size_t)o * Mh;
    load_twiddles(tw_s, tw, M);
    for (int e0 = threadIdx.x; e0 < M * B; e0 += kLoadBatch * blockDim.x) {
        float2 v[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            int e = e0 + u * blockDim.x;
            const int m = e >> bsh, b = e & (B - 1);
            v[u] = (e < M * B && b < nb) ? spec[base + m * sm_stride + kz0 + b] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            int e = e0 + u * blockDim.x;
            if (e < M * B) x[e] = v[u];  // pitch == B
        }
    }
    __syncthreads();
    float2 *res = fft_columns(x, y, tw_s, M, bsh, pitch, sign);
    if (green) {
        // res holds the full forward transform: k index m along x, y index o, kz0+b
        const int ky = o <= M / 2 ? o : M - o;
        const float gy = green1d[ky];
        for (int e = threadIdx.x; e < M * B; e += blockDim.x) {
            const int m = e >> bsh, b = e & (B - 1);
            int kx = m <= M / 2 ? m : M - m;
            int kz = kz0 + b;
            float2 v = res[m * pitch + b];
            float g = 0.f;
            if (b < nb) {
                int k2 = kx * kx + ky * ky + kz * kz;
                if (k2 > 0) g = -green1d[kx] * gy * green1d[kz] * __frcp_rn((float)k2);
            }
            res[m * pitch + b] = make_float2(v.x * g, v.y * g);
        }
        __syncthreads();
        float2 *other = res == x ? y : x;
        res = fft_columns(res, other, tw_s, M, bsh, pitch, +1);
    }
    for (int e = threadIdx.x; e < M * B; e += blockDim.x) {
        const int m = e >> bsh, b = e & (B - 1);
        if (b < nb) spec[base + m * sm_stride + kz0 + b] = res[m * pitch + b];
    }
}

__global__ void __launch_bounds__(kFFTThreads)
    k_fft_z_r2c(unsigned long long *__restrict__ rho64, float mscale, float2 *__restrict__ spec,
                const float2 *tw, int M, int P) {
    fft_z_r2c(rho64, mscale, spec, tw, M, P, blockIdx.x);
}

__global__ void __launch_bounds__(kFFTThreads)
    k_fft_z_c2r(const float2 *__restrict__ spec, float *__restrict__ out, const float2 *tw, int M, int P) {
    fft_z_c2r(spec, out, tw, M, P, blockIdx.x);
}

__global__ void __launch_bounds__(kFFTThreads)
    k_fft_axis(float2 *__restrict__ spec, const float2 *tw, const float *__restrict__ green1d, int M, int B,
               int axis, int sign, int green) {
    fft_axis(spec, tw, green1d, M, B, axis, sign, green, blockIdx.x, blockIdx.y);
}

// fft_axis_reg for one box, with the batch B a compile-time constant
// (B divides the block and M * B is a multiple of it): each thread keeps one
// column b and visits the points m = r0 + j * (threads / B), so the index
// arithmetic of the loads, stores and transforms folds to constants and the
// Green's factor's column terms are computed once.  Same transforms and the
// same operations per point as fft_axis_reg.
template <typename FT, int B>
__device__ __forceinline__ void fft_axis_reg_fixed(float2 *__restrict__ spec, const float2 *tw,
                                                   const float *__restrict__ green1d, int axis, int sign,
                                                   int green, int bx, int by) {
    constexpr int M = FT::M, Mh = M / 2 + 1;
    constexpr int bsh = ilog2(B), rs = kFFTThreads / B, per = M * B / kFFTThreads;
    static_assert(kFFTThreads % B == 0 && (M * B) % kFFTThreads == 0, "batch layout");
    extern __shared__ float2 sm[];
    float2 *x = sm, *tw_s = sm + M * B;
    const int o = by, kz0 = bx * B, nb = min(B, Mh - kz0);
    const int b = threadIdx.x & (B - 1), r0 = threadIdx.x >> bsh;
    const bool valid = b < nb;
    const size_t sm_stride = axis == 1 ? (size_t)Mh : (size_t)M * Mh;
    float2 *col = spec + (axis == 1 ? (size_t)o * M * Mh : (size_t)o * Mh) + kz0 + b;
    // an inverse-only pass starts from the slot order
    const bool to_slots = sign > 0;
    load_twiddles(tw_s, tw, M);
#pragma unroll
    for (int j0 = 0; j0 < per; j0 += kLoadBatch) {
        float2 v[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u)
            if (j0 + u < per) v[u] = valid ? col[(size_t)(r0 + (j0 + u) * rs) * sm_stride] : make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u)
            if (j0 + u < per) {
                const int m = r0 + (j0 + u) * rs;
                x[(to_slots ? FT::slot(m) : m) * B + b] = v[u];
            }
    }
    __syncthreads();
    bool natural = true;
    if (sign < 0) {
        FT::template forward<-1>(x, tw_s, B, bsh);
        natural = false;
        if (green) {
            // slot s = M2 k1 + k2 holds X[k1 + M1 k2]
            const int ky = o <= M / 2 ? o : M - o;
            const float gy = green1d[ky];
            const int kz = kz0 + b;
            const float gz = valid ? green1d[kz] : 0.f;
            const int c = ky * ky + kz * kz;
#pragma unroll 4
            for (int j = 0; j < per; ++j) {
                const int sl = r0 + j * rs;
                const int k1 = sl / FT::N2, k2 = sl - k1 * FT::N2;
                const int m = k1 + FT::N1 * k2;  // the transform index along x
                const int kx = m <= M / 2 ? m : M - m;
                const float2 v = x[sl * B + b];
                float g = 0.f;
                if (valid) {
                    const int k2s = kx * kx + c;
                    if (k2s > 0) g = -green1d[kx] * gy * gz * __frcp_rn((float)k2s);
                }
                x[sl * B + b] = make_float2(v.x * g, v.y * g);
            }
            __syncthreads();
            FT::template inverse<+1>(x, tw_s, B, bsh);
            natural = true;
        }
    } else {
        FT::template inverse<+1>(x, tw_s, B, bsh);
    }
    if (valid) {
#pragma unroll 4
        for (int j = 0; j < per; ++j) {
            const int m = r0 + j * rs;
            col[(size_t)m * sm_stride] = x[(natural ? m : FT::slot(m)) * B + b];
        }
    }
}

// One box, power-of-two mesh M = M1 * M2: the register transforms, one
// instantiation per split (its registers sized for its DFT lengths).
template <int M1, int M2>
__global__ void __launch_bounds__(kFFTThreads, M1 * M2 >= 512 ? 2 : 4)
    k_fft_z_r2c_r(unsigned long long *__restrict__ rho64, float mscale, float2 *__restrict__ spec,
                  const float2 *tw, int P) {
    fft_z_r2c_reg<RegFFT<M1, M2>>(rho64, mscale, spec, tw, P, blockIdx.x);
}

template <int M1, int M2>
__global__ void __launch_bounds__(kFFTThreads, M1 * M2 >= 512 ? 2 : 4)
    k_fft_z_c2r_r(const float2 *__restrict__ spec, float *__restrict__ out, const float2 *tw, int P) {
    fft_z_c2r_reg<RegFFT<M1, M2>>(spec, out, tw, P, blockIdx.x);
}

// the one-box batch of the axis passes, fft_batch_axis(M)
__host__ __device__ constexpr int axis_batch(int M) { return M == 1024 ? 8 : (4096 / M > 16 ? 16 : 4096 / M); }

template <int M1, int M2>
__global__ void __launch_bounds__(kFFTThreads, M1 * M2 >= 512 ? 2 : 4)
    k_fft_axis_r(float2 *__restrict__ spec, const float2 *tw, const float *__restrict__ green1d, int axis,
                 int sign, int green) {
    fft_axis_reg_fixed<RegFFT<M1, M2>, axis_batch(M1 * M2)>(spec, tw, green1d, axis, sign, green, blockIdx.x,
                                                            blockIdx.y);
}

// The five transform passes of one box with the register transforms.
template <int M1, int M2>
cudaError_t fft_passes_reg(const PMPlan &plan, int P, cudaStream_t stream) {
    constexpr int M = M1 * M2, Mh = M / 2 + 1, B = axis_batch(M);
    // z passes: the transform buffer, the twiddles and the block of 2P
    // spectrum rows; axis passes: the buffer and the twiddles
    const size_t smz = sizeof(float2) * ((size_t)M * (P + 1) + M + (size_t)2 * P * Mh),
                 sma = sizeof(float2) * ((size_t)M * B + M);
    static bool attr = [&] {
        cudaFuncSetAttribute(k_fft_z_r2c_r<M1, M2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        cudaFuncSetAttribute(k_fft_z_c2r_r<M1, M2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        cudaFuncSetAttribute(k_fft_axis_r<M1, M2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        return true;
    }();
    (void)attr;
    const unsigned zblocks = (unsigned)((size_t)M * M / (2 * P));
    k_fft_z_r2c_r<M1, M2><<<zblocks, kFFTThreads, smz, stream>>>(plan.rho64, ldexpf(plan.mass, -32), plan.spec,
                                                                 plan.twiddle, P);
    dim3 ag((Mh + B - 1) / B, M);
    k_fft_axis_r<M1, M2><<<ag, kFFTThreads, sma, stream>>>(plan.spec, plan.twiddle, plan.green1d, 1, -1, 0);
    k_fft_axis_r<M1, M2><<<ag, kFFTThreads, sma, stream>>>(plan.spec, plan.twiddle, plan.green1d, 0, -1, 1);
    k_fft_axis_r<M1, M2><<<ag, kFFTThreads, sma, stream>>>(plan.spec, plan.twiddle, plan.green1d, 1, +1, 0);
    k_fft_z_c2r_r<M1, M2><<<zblocks, kFFTThreads, smz, stream>>>(plan.spec, plan.rho, plan.twiddle, P);
    return cudaGetLastError();
}

// Many boxes in one launch: map[blockIdx.x] = (box, the box's own block
// index).  BIG: only the boxes with 32-point register transforms (meshes 512
// and 1024), every other block returns; !BIG: every other box.
__device__ __forceinline__ bool big_box(const PMBoxDesc &d, int cols) {
    return d.M >= 512 && reg_fft_ok(d.M, cols);
}

template <bool BIG>
__global__ void __launch_bounds__(kFFTThreads, BIG ? 2 : 3)
    k_fft_z_r2c_multi(const PMBoxDesc *__restrict__ boxes, const uint2 *__restrict__ map) {
    const uint2 m = map[blockIdx.x];
    const PMBoxDesc &d = boxes[m.x];
    if (big_box(d, d.P) != BIG) return;
    if (BIG) {
        if (d.M == 512)
            fft_z_r2c_reg<RegFFT<16, 32>>(d.rho64, d.mscale, d.spec, d.twiddle, d.P, m.y);
        else
            fft_z_r2c_reg<RegFFT<32, 32>>(d.rho64, d.mscale, d.spec, d.twiddle, d.P, m.y);
    } else if (reg_fft_ok(d.M, d.P)) {
        switch (d.M) {
            case 16: fft_z_r2c_reg<RegFFT<4, 4>>(d.rho64, d.mscale, d.spec, d.twiddle, d.P, m.y); break;
            case 32: fft_z_r2c_reg<RegFFT<4, 8>>(d.rho64, d.mscale, d.spec, d.twiddle, d.P, m.y); break;
            case 64: fft_z_r2c_reg<RegFFT<8, 8>>(d.rho64, d.mscale, d.spec, d.twiddle, d.P, m.y); break;
            case 128: fft_z_r2c_reg<RegFFT<8, 16>>(d.rho64, d.mscale, d.spec, d.twiddle, d.P, m.y); break;
            default: fft_z_r2c_reg<RegFFT<16, 16>>(d.rho64, d.mscale, d.spec, d.twiddle, d.P, m.y); break;
        }
    } else {
        fft_z_r2c(d.rho64, d.mscale, d.spec, d.twiddle, d.M, d.P, m.y);
    }
}

template <bool BIG>
__global__ void __launch_bounds__(kFFTThreads, BIG ? 2 : 3)
    k_fft_z_c2r_multi(const PMBoxDesc *__restrict__ boxes, const uint2 *__restrict__ map) {
    const uint2 m = map[blockIdx.x];
    const PMBoxDesc &d = boxes[m.x];
    if (big_box(d, d.P) != BIG) return;
    if (BIG) {
        if (d.M == 512)
            fft_z_c2r_reg<RegFFT<16, 32>>(d.spec, d.rho, d.twiddle, d.P, m.y);
        else
            fft_z_c2r_reg<RegFFT<32, 32>>(d.spec, d.rho, d.twiddle, d.P, m.y);
    } else if (reg_fft_ok(d.M, d.P)) {
        switch (d.M) {
            case 16: fft_z_c2r_reg<RegFFT<4, 4>>(d.spec, d.rho, d.twiddle, d.P, m.y); break;
            case 32: fft_z_c2r_reg<RegFFT<4, 8>>(d.spec, d.rho, d.twiddle, d.P, m.y); break;
            case 64: fft_z_c2r_reg<RegFFT<8, 8>>(d.spec, d.rho, d.twiddle, d.P, m.y); break;
            case 128: fft_z_c2r_reg<RegFFT<8, 16>>(d.spec, d.rho, d.twiddle, d.P, m.y); break;
            default: fft_z_c2r_reg<RegFFT<16, 16>>(d.spec, d.rho, d.twiddle, d.P, m.y); break;
        }
    } else {
        fft_z_c2r(d.spec, d.rho, d.twiddle, d.M, d.P, m.y);
    }
}

template <bool BIG>
__global__ void __launch_bounds__(kFFTThreads, BIG ? 2 : 3)
    k_fft_axis_multi(const PMBoxDesc *__restrict__ boxes, const uint2 *__restrict__ map, int axis, int sign,
                     int green) {
    const uint2 m = map[blockIdx.x];
    const PMBoxDesc &d = boxes[m.x];
    if (big_box(d, d.B) != BIG) return;
    const int nbx = (d.M / 2 + 1 + d.B - 1) / d.B;
    const int bx = m.y % nbx, by = m.y / nbx;
    if (BIG) {
        if (d.M == 512)
            fft_axis_reg<RegFFT<16, 32>>(d.spec, d.twiddle, d.green1d, d.B, axis, sign, green, bx, by);
        else
            fft_axis_reg<RegFFT<32, 32>>(d.spec, d.twiddle, d.green1d, d.B, axis, sign, green, bx, by);
    } else if (reg_fft_ok(d.M, d.B)) {
        switch (d.M) {
            case 16: fft_axis_reg<RegFFT<4, 4>>(d.spec, d.twiddle, d.green1d, d.B, axis, sign, green, bx, by); break;
            case 32: fft_axis_reg<RegFFT<4, 8>>(d.spec, d.twiddle, d.green1d, d.B, axis, sign, green, bx, by); break;
            case 64: fft_axis_reg<RegFFT<8, 8>>(d.spec, d.twiddle, d.green1d, d.B, axis, sign, green, bx, by); break;
            case 128: fft_axis_reg<RegFFT<8, 16>>(d.spec, d.twiddle, d.green1d, d.B, axis, sign, green, bx, by); break;
            default: fft_axis_reg<RegFFT<16, 16>>(d.spec, d.twiddle, d.green1d, d.B, axis, sign, green, bx, by); break;
        }
    } else {
        fft_axis(d.spec, d.twiddle, d.green1d, d.M, d.B, axis, sign, green, bx, by);
    }
}

__device__ __forceinline__ void cic_axis(float to_slab_fac, float p, int M, int *s, int *ss,
                                         float *d) {
    float t = __fmul_rn(to_slab_fac, p);  // pm_periodic.c:99 in float
    int sl = (int)t;
    if (sl >= M) sl = M - 1;
    if (sl < 0) sl = 0;
    *d = __fsub_rn(t, (float)sl);
    *s = sl;
    *ss = sl + 1 >= M ? sl + 1 - M : sl + 1;
}

// The same for a 32-bit fixed-point coordinate x (units of L / 2^32): the
// mesh coordinate x * M / 2^32 is exact in 32.32 fixed point, so the cell and
// the fraction (rounded once, to float) need no float product.
__device__ __forceinline__ void cic_axis_fixed(uint32_t x, int M, int *s, int *ss, float *d) {
    const uint64_t t = (uint64_t)x * (uint32_t)M;
    const int sl = (int)(t >> 32);  // < M
    *d = (float)(uint32_t)t * 2.3283064365386963e-10f;  // 2^-32
    *s = sl;
    *ss = sl + 1 >= M ? sl + 1 - M : sl + 1;
}

template <bool FIXED>
__device__ __forceinline__ void cic_point(const float4 &p, float to_slab_fac, int M, int s[3][2], float d[3]) {
    if (FIXED) {
        cic_axis_fixed(__float_as_uint(p.x), M, &s[0][0], &s[0][1], &d[0]);
        cic_axis_fixed(__float_as_uint(p.y), M, &s[1][0], &s[1][1], &d[1]);
        cic_axis_fixed(__float_as_uint(p.z), M, &s[2][0], &s[2][1], &d[2]);
    } else {
        cic_axis(to_slab_fac, p.x, M, &s[0][0], &s[0][1], &d[0]);
        cic_axis(to_slab_fac, p.y, M, &s[1][0], &s[1][1], &d[1]);
        cic_axis(to_slab_fac, p.z, M, &s[2][0], &s[2][1], &d[2]);
    }
}

// CIC weights w in [0, 1] are added as the integers w * 2^32 (rounded once):
// integer atomics are associative, so the deposited grid does not depend on
// the order in which particles land, and it is the exact sum of the rounded
// weights.
__device__ __forceinline__ unsigned long long weight_u64(float w) {
    return __float2ull_rn(__fmul_rn(w, 4294967296.0f));
}

// The eight CIC corners of a particle, warp-aggregated: particles of one warp
// in the same mesh cell share all eight corners, so one __match_any_sync on
// the cell finds them; each group adds its members' integer weights with
// shuffles and its lowest lane issues the eight atomics.  When no two active
// lanes share a cell (lattice-ordered particles at high redshift) every lane
// adds its own weights directly.  Integer sums are associative, so the grid
// is the same either way, bit for bit.  Called by every active lane of the
// warp together.
template <bool FIXED>
__device__ __forceinline__ void deposit_one(float4 p, unsigned long long *__restrict__ rho64, int M,
                                            float to_slab_fac) {
    int s[3][2];
    float d[3];
    cic_point<FIXED>(p, to_slab_fac, M, s, d);
    const int sx = s[0][0], sxx = s[0][1], sy = s[1][0], syy = s[1][1], sz = s[2][0], szz = s[2][1];
    const float dx = d[0], dy = d[1], dz = d[2];
    const size_t Mz = M, Myz = (size_t)M * M;
    const float m0 = 1.f - dx, m1 = dx;
    unsigned long long w[8] = {weight_u64(m0 * (1.f - dy) * (1.f - dz)), weight_u64(m0 * dy * (1.f - dz)),
                               weight_u64(m0 * (1.f - dy) * dz),        weight_u64(m0 * dy * dz),
                               weight_u64(m1 * (1.f - dy) * (1.f - dz)), weight_u64(m1 * dy * (1.f - dz)),
                               weight_u64(m1 * (1.f - dy) * dz),        weight_u64(m1 * dy * dz)};
    const unsigned active = __activemask(), lane = threadIdx.x & 31;
    const unsigned cell = ((unsigned)sx * (unsigned)M + (unsigned)sy) * (unsigned)M + (unsigned)sz;
    const unsigned peers = __match_any_sync(active, cell);
    bool lead = true;
    if (!__all_sync(active, peers == (1u << lane))) {
        // sum the group's weights into its lowest lane (every member runs the
        // same number of shuffles, named by the group's own mask)
        const unsigned first = (unsigned)__ffs(peers) - 1;
        lead = lane == first;
        unsigned long long sum[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (unsigned rest = peers; rest; rest &= rest - 1) {
            const int src = __ffs(rest) - 1;
#pragma unroll
            for (int c = 0; c < 8; ++c) sum[c] += __shfl_sync(peers, w[c], src);
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) w[c] = sum[c];
    }
    if (lead) {
        [[maybe_unused]] const uint32_t M3 = (uint32_t)(Myz * Mz);  // the bounds checks' grid size
        atomicAdd(&rho64[CUCO_IDX(sx * Myz + sy * Mz + sz, M3)], w[0]);
        atomicAdd(&rho64[CUCO_IDX(sx * Myz + syy * Mz + sz, M3)], w[1]);
        atomicAdd(&rho64[CUCO_IDX(sx * Myz + sy * Mz + szz, M3)], w[2]);
        atomicAdd(&rho64[CUCO_IDX(sx * Myz + syy * Mz + szz, M3)], w[3]);
        atomicAdd(&rho64[CUCO_IDX(sxx * Myz + sy * Mz + sz, M3)], w[4]);
        atomicAdd(&rho64[CUCO_IDX(sxx * Myz + syy * Mz + sz, M3)], w[5]);
        atomicAdd(&rho64[CUCO_IDX(sxx * Myz + sy * Mz + szz, M3)], w[6]);
        atomicAdd(&rho64[CUCO_IDX(sxx * Myz + syy * Mz + szz, M3)], w[7]);
    }
}

__device__ __forceinline__ int wrapi(int a, int M) { return a < 0 ? a + M : (a >= M ? a - M : a); }

template <bool FIXED>
__device__ __forceinline__ float4 interp_one(float4 p, const float *__restrict__ phi, int M, float to_slab_fac,
                                             float fac) {
    int s[3][2];
    float d[3];
    cic_point<FIXED>(p, to_slab_fac, M, s, d);
    float wx[2] = {1.f - d[0], d[0]}, wy[2] = {1.f - d[1], d[1]}, wz[2] = {1.f - d[2], d[2]};
    // Per dimension the six mesh planes s-2 .. s+3 (periodic), as offsets:
    // the two corners are planes 2 and 3, and along each dimension the two
    // corners' stencils (c-2, c-1, c+1, c+2) share one line of six points,
    // so every potential value loaded is one sum of three offsets.
    int off[3][6];
#pragma unroll
    for (int dim = 0; dim < 3; ++dim) {
        const int scale = dim == 0 ? M * M : (dim == 1 ? M : 1);
#pragma unroll
        for (int q = 0; q < 6; ++q) off[dim][q] = wrapi(s[dim][0] - 2 + q, M) * scale;
    }
    float out[3];
#pragma unroll
    for (int dim = 0; dim < 3; ++dim) {
        // 4 lines x 6 loads instead of 32
        float F[2][2][2];
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int v = 0; v < 2; ++v) {
                // the two other dimensions' corner planes
                const int d1 = (dim + 1) % 3, d2 = (dim + 2) % 3;
                const int base = off[d1][2 + u] + off[d2][2 + v];
                float f[6];
#pragma unroll
                for (int q = 0; q < 6; ++q) f[q] = __ldg(&phi[CUCO_IDX(base + off[dim][q], (uint32_t)M * M * M)]);
                // corner at s0 (f[2]) and at s0 + 1 (f[3])
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float fm1 = f[1 + h], fp1 = f[3 + h], fm2 = f[h], fp2 = f[4 + h];
                    const float Fv = fac * ((4.0f / 3.0f) * (fm1 - fp1) - (1.0f / 6.0f) * (fm2 - fp2));
                    // F indexed by (cx, cy, cz)
                    int idx[3];
                    idx[dim] = h;
                    idx[d1] = u;
                    idx[d2] = v;
                    F[idx[0]][idx[1]][idx[2]] = Fv;
                }
            }
        float a = 0.f;
#pragma unroll
        for (int cx = 0; cx < 2; ++cx)
#pragma unroll
            for (int cy = 0; cy < 2; ++cy)
#pragma unroll
                for (int cz = 0; cz < 2; ++cz) a += F[cx][cy][cz] * wx[cx] * wy[cy] * wz[cz];
        out[dim] = a;
    }
    return make_float4(out[0], out[1], out[2], 0.f);
}

template <bool FIXED>
__global__ void k_deposit(const float4 *__restrict__ pos, uint32_t n, unsigned long long *__restrict__ rho64,
                          int M, float to_slab_fac) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) deposit_one<FIXED>(pos[i], rho64, M, to_slab_fac);
}

template <bool FIXED>
__global__ void k_interp(const float4 *__restrict__ pos, uint32_t n, const float *__restrict__ phi,
                         int M, float to_slab_fac, float fac, float4 *__restrict__ acc) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) acc[i] = interp_one<FIXED>(pos[i], phi, M, to_slab_fac, fac);
}

template <bool FIXED>
__global__ void k_deposit_multi(const float4 *__restrict__ pos, uint32_t n, const PMBoxDesc *__restrict__ boxes,
                                const uint32_t *__restrict__ pbeg, int nbox) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const PMBoxDesc &d = boxes[find_box(pbeg, nbox, i)];
    deposit_one<FIXED>(pos[i], d.rho64, d.M, d.to_slab_fac);
}

template <bool FIXED>
__global__ void k_interp_multi(const float4 *__restrict__ pos, uint32_t n, const PMBoxDesc *__restrict__ boxes,
                               const uint32_t *__restrict__ pbeg, int nbox, float4 *__restrict__ acc) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const PMBoxDesc &d = boxes[find_box(pbeg, nbox, i)];
    acc[i] = interp_one<FIXED>(pos[i], d.rho, d.M, d.to_slab_fac, d.fd_fac);
}

// Batch sizes are powers of two: the transforms split a flat index into
// (row, column) with a shift and a mask.
int fft_batch_z(int M) {
    int P = 4096 / M;
    if (P > 16) P = 16;
    if (P > M / 2) P = M / 2;  // k_fft_z_c2r stages 2P rows of M/2+1 in an M*(P+1) buffer
    if (P < 1) P = 1;
    P = 1 << ilog2(P);
    // P pairs per CTA must divide the M*M/2 row pairs
    while (P > 1 && ((M * M / 2) % P)) P >>= 1;
    return P;
}

int fft_batch_axis(int M) {
    // M = 1024: 8 columns, not 4096 / M = 4.  Its register transform gives a
    // column 32 threads, so 8 columns keep all 256 threads of a CTA busy, and
    // each row of the batch is 64 contiguous bytes (the five passes of one
    // force took 21.2 instead of 26.2 ms)
    if (M == 1024) return 8;
    int B = 4096 / M;
    if (B > 16) B = 16;
    if (B < 1) B = 1;
    return 1 << ilog2(B);
}

}  // namespace

bool pm_big_fft(int M, int P, int B) { return M >= 512 && reg_fft_ok(M, P) && reg_fft_ok(M, B); }

// A power-of-two mesh must take the register transforms in every pass (as one
// box does): its batches may not exceed what they hold.
bool pm_fft_batches_ok(int M, int P, int B) {
    const bool pow2 = M >= 16 && M <= 1024 && (M & (M - 1)) == 0;
    return !pow2 || (reg_fft_ok(M, P) && reg_fft_ok(M, B));
}

int pm_batch_z(int M) { return fft_batch_z(M); }
int pm_batch_axis(int M) { return fft_batch_axis(M); }

void pm_tables(int M, float boxsize, float asmth, float *green1d, float2 *twiddle) {
    const size_t Mh = M / 2 + 1;
    double asmth2 = (2 * M_PI) * (double)asmth / (double)boxsize;
    asmth2 *= asmth2;
    for (size_t k = 0; k < Mh; ++k) {
        double e = exp(-(double)(k * k) * asmth2);
        double f = 1.0;
        if (k) {
            f = (M_PI * (double)k) / M;
            f = sin(f) / f;
        }
        green1d[k] = (float)(e / (f * f * f * f));
    }
    for (int t = 0; t < M; ++t)
        twiddle[t] = make_float2((float)cos(2 * M_PI * t / M), (float)-sin(2 * M_PI * t / M));
}

float pm_fd_fac(int M, float boxsize, double G) {
    double fac = G / (M_PI * (double)boxsize);
    fac *= (double)(1.0f / (2.0f * boxsize / (float)M));
    return (float)fac;
}

size_t pm_smem_z(int M, int P) { return sizeof(float2) * (2 * (size_t)M * (P + 1) + M); }
size_t pm_smem_axis(int M, int B) { return sizeof(float2) * (2 * (size_t)M * B + M); }

cuco_status_t pm_forces_multi(const PMMulti &m, const float4 *pos, uint32_t n, float4 *acc,
                              cudaStream_t stream, int *launches) {
    static bool attr = [] {
        const int mx = 227 * 1024;
        for (bool big : {false, true}) {
            cudaFuncSetAttribute(big ? k_fft_z_r2c_multi<true> : k_fft_z_r2c_multi<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
            cudaFuncSetAttribute(big ? k_fft_z_c2r_multi<true> : k_fft_z_c2r_multi<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
            cudaFuncSetAttribute(big ? k_fft_axis_multi<true> : k_fft_axis_multi<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        }
        return true;
    }();
    (void)attr;
    CUCO_TRY_CUDA(cudaMemsetAsync(m.rho64_all, 0, sizeof(unsigned long long) * m.rho_all_count, stream));
    if (n) {
        if (m.fixed)
            k_deposit_multi<true><<<(n + 255) / 256, 256, 0, stream>>>(pos, n, m.boxes, m.pbeg, m.nbox);
        else
            k_deposit_multi<false><<<(n + 255) / 256, 256, 0, stream>>>(pos, n, m.boxes, m.pbeg, m.nbox);
    }
    // each pass: the boxes of the common kernels, then (when the ensemble has
    // any) the boxes of the large register transforms
    k_fft_z_r2c_multi<false><<<m.nz_blocks, kFFTThreads, m.smz, stream>>>(m.boxes, m.map_z);
    if (m.big) k_fft_z_r2c_multi<true><<<m.nz_blocks, kFFTThreads, m.smz, stream>>>(m.boxes, m.map_z);
    for (int pass = 0; pass < 3; ++pass) {
        const int axis = pass == 1 ? 0 : 1, sign = pass == 2 ? +1 : -1, green = pass == 1;
        k_fft_axis_multi<false><<<m.naxis_blocks, kFFTThreads, m.sma, stream>>>(m.boxes, m.map_axis, axis, sign,
                                                                                green);
        if (m.big)
            k_fft_axis_multi<true><<<m.naxis_blocks, kFFTThreads, m.sma, stream>>>(m.boxes, m.map_axis, axis, sign,
                                                                                   green);
    }
    k_fft_z_c2r_multi<false><<<m.nz_blocks, kFFTThreads, m.smz, stream>>>(m.boxes, m.map_z);
    if (m.big) k_fft_z_c2r_multi<true><<<m.nz_blocks, kFFTThreads, m.smz, stream>>>(m.boxes, m.map_z);
    if (n) {
        if (m.fixed)
            k_interp_multi<true><<<(n + 255) / 256, 256, 0, stream>>>(pos, n, m.boxes, m.pbeg, m.nbox, acc);
        else
            k_interp_multi<false><<<(n + 255) / 256, 256, 0, stream>>>(pos, n, m.boxes, m.pbeg, m.nbox, acc);
    }
    CUCO_TRY_CUDA(cudaGetLastError());
    if (launches) *launches += m.big ? 12 : 7;
    return CUCO_OK;
}

bool pm_mesh_supported(int M) {
    if (M < 8 || M > 1024 || (M & 1)) return false;
    int r = M;
    for (int f : {2, 3, 5})
        while (r % f == 0) r /= f;
    return r == 1;
}

cuco_status_t pm_plan_create(PMPlan *plan, int M, float boxsize, float asmth, float mass,
                             double G, bool fixed) {
    if (!pm_mesh_supported(M)) {
        set_error("PM mesh size must be even, in [8, 1024], with no prime factor above 5");
        return CUCO_ERR_UNSUPPORTED;
    }
    plan->M = M;
    plan->fixed = fixed;
    plan->boxsize = boxsize;
    plan->to_slab_fac = (float)M / boxsize;
    plan->mass = mass;
    double fac = G / (M_PI * (double)boxsize);
    fac *= (double)(1.0f / (2.0f * boxsize / (float)M));
    plan->fd_fac = (float)fac;
    const size_t Mh = M / 2 + 1;
    CUCO_TRY_CUDA(cudaMalloc(&plan->rho, sizeof(float) * (size_t)M * M * M));
    CUCO_TRY_CUDA(cudaMalloc(&plan->rho64, sizeof(unsigned long long) * (size_t)M * M * M));
    plan->rho64_dirty = true;
    CUCO_TRY_CUDA(cudaMalloc(&plan->spec, sizeof(float2) * (size_t)M * M * Mh));
    CUCO_TRY_CUDA(cudaMalloc(&plan->green1d, sizeof(float) * Mh));
    CUCO_TRY_CUDA(cudaMalloc(&plan->twiddle, sizeof(float2) * M));
    std::vector<float> g(Mh);
    double asmth2 = (2 * M_PI) * (double)asmth / (double)boxsize;
    asmth2 *= asmth2;
    for (size_t k = 0; k < Mh; ++k) {
        double e = exp(-(double)(k * k) * asmth2);
        double f = 1.0;
        if (k) {
            f = (M_PI * (double)k) / M;
            f = sin(f) / f;
        }
        g[k] = (float)(e / (f * f * f * f));
    }
    std::vector<float2> tw(M);
    for (int t = 0; t < M; ++t) tw[t] = make_float2((float)cos(2 * M_PI * t / M), (float)-sin(2 * M_PI * t / M));
    CUCO_TRY_CUDA(cudaMemcpy(plan->green1d, g.data(), sizeof(float) * Mh, cudaMemcpyHostToDevice));
    CUCO_TRY_CUDA(cudaMemcpy(plan->twiddle, tw.data(), sizeof(float2) * M, cudaMemcpyHostToDevice));
    // The shared-memory limit is an attribute of the kernel, not of a launch:
    // it is set once to the most a CTA can have, so that boxes of different
    // meshes in one process (a serving loop's) never lower it under each
    // other's launches.
    const int P = fft_batch_z(M), B = fft_batch_axis(M);
    const size_t smz = sizeof(float2) * (2 * (size_t)M * (P + 1) + M);
    const size_t sma = sizeof(float2) * (2 * (size_t)M * B + M);
    constexpr int kMaxSmem = 227 * 1024;
    if (smz > (size_t)kMaxSmem || sma > (size_t)kMaxSmem) {
        set_error("PM: the transform of this mesh needs more shared memory than a CTA has");
        return CUCO_ERR_UNSUPPORTED;
    }
    static const cudaError_t attr = [] {
        cudaError_t e = cudaFuncSetAttribute(k_fft_z_r2c, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_fft_z_c2r, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_fft_axis, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
        return e;
    }();
    CUCO_TRY_CUDA(attr);
    return CUCO_OK;
}

void pm_plan_destroy(PMPlan *plan) {
    cudaFree(plan->rho);
    cudaFree(plan->rho64);
    plan->rho64 = nullptr;
    cudaFree(plan->spec);
    cudaFree(plan->green1d);
    cudaFree(plan->twiddle);
    plan->rho = nullptr;
    plan->spec = nullptr;
}

cuco_status_t pm_forces(PMPlan &plan, const float4 *pos, uint32_t n, float4 *acc,
                        cudaStream_t stream, cudaEvent_t *ev_deposit_done, cudaEvent_t *ev_fft_done,
                        int *launches) {
    const int M = plan.M, Mh = M / 2 + 1;
    // at most 8 row pairs per z-pass CTA: half the shared memory of 16, so
    // more CTAs fit beside the sort's (9 us faster per force at M = 256)
    const int P = std::min(fft_batch_z(M), 8), B = fft_batch_axis(M);
    const size_t smz = sizeof(float2) * (2 * (size_t)M * (P + 1) + M);
    const size_t sma = sizeof(float2) * (2 * (size_t)M * B + M);
    // The z r2c pass clears the sums it reads, so the grid is zero again when
    // the previous call enqueued its passes; otherwise (first call, or a call
    // that stopped at an error) it is cleared here.
    if (plan.rho64_dirty)
        CUCO_TRY_CUDA(cudaMemsetAsync(plan.rho64, 0, sizeof(unsigned long long) * (size_t)M * M * M, stream));
    plan.rho64_dirty = true;
    if (n) {
        if (plan.fixed)
            k_deposit<true><<<(n + 255) / 256, 256, 0, stream>>>(pos, n, plan.rho64, M, plan.to_slab_fac);
        else
            k_deposit<false><<<(n + 255) / 256, 256, 0, stream>>>(pos, n, plan.rho64, M, plan.to_slab_fac);
    }
    CUCO_TRY_CUDA(cudaGetLastError());
    if (ev_deposit_done) CUCO_TRY_CUDA(cudaEventRecord(*ev_deposit_done, stream));
    if (reg_fft_ok(M, P) && reg_fft_ok(M, B)) {
        cudaError_t e;
        switch (M) {
            case 16: e = fft_passes_reg<4, 4>(plan, P, stream); break;
            case 32: e = fft_passes_reg<4, 8>(plan, P, stream); break;
            case 64: e = fft_passes_reg<8, 8>(plan, P, stream); break;
            case 128: e = fft_passes_reg<8, 16>(plan, P, stream); break;
            case 256: e = fft_passes_reg<16, 16>(plan, P, stream); break;
            case 512: e = fft_passes_reg<16, 32>(plan, P, stream); break;
            default: e = fft_passes_reg<32, 32>(plan, P, stream); break;
        }
        CUCO_TRY_CUDA(e);
    } else {
        const unsigned zblocks = (unsigned)((size_t)M * M / (2 * P));
        k_fft_z_r2c<<<zblocks, kFFTThreads, smz, stream>>>(plan.rho64, ldexpf(plan.mass, -32), plan.spec,
                                                           plan.twiddle, M, P);
        dim3 ag((Mh + B - 1) / B, M);
        k_fft_axis<<<ag, kFFTThreads, sma, stream>>>(plan.spec, plan.twiddle, plan.green1d, M, B, 1, -1, 0);
        k_fft_axis<<<ag, kFFTThreads, sma, stream>>>(plan.spec, plan.twiddle, plan.green1d, M, B, 0, -1, 1);
        k_fft_axis<<<ag, kFFTThreads, sma, stream>>>(plan.spec, plan.twiddle, plan.green1d, M, B, 1, +1, 0);
        k_fft_z_c2r<<<zblocks, kFFTThreads, smz, stream>>>(plan.spec, plan.rho, plan.twiddle, M, P);
        CUCO_TRY_CUDA(cudaGetLastError());
    }
    plan.rho64_dirty = false;
    if (ev_fft_done) CUCO_TRY_CUDA(cudaEventRecord(*ev_fft_done, stream));
    if (n) {
        if (plan.fixed)
            k_interp<true><<<(n + 255) / 256, 256, 0, stream>>>(pos, n, plan.rho, M, plan.to_slab_fac, plan.fd_fac, acc);
        else
            k_interp<false><<<(n + 255) / 256, 256, 0, stream>>>(pos, n, plan.rho, M, plan.to_slab_fac, plan.fd_fac, acc);
    }
    CUCO_TRY_CUDA(cudaGetLastError());
    if (launches) *launches += 5 + (n ? 2 : 0);  // five transform passes, deposit and interpolation
    return CUCO_OK;
}

uint32_t bounds_violations_pm() { return bounds_violations_take(); }

}  // namespace cuco
