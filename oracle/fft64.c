/*
 * fft64 — FP64 FFTs for the CPU oracle (test infrastructure only).
 * Conventions: see fft64.h. Algorithm: for power-of-two lengths, iterative
 * radix-2 decimation-in-time Cooley-Tukey on a contiguous copy of each line;
 * for other lengths, recursive mixed-radix decimation in time by the smallest
 * prime factor (a prime length is a direct DFT). Twiddles e^{-2 pi i k/n} from
 * libm cos/sin, cached per length; real transforms of (even) length n use the
 * standard half-length packing (x[2m] + i x[2m+1]) with a split step.
 */
#include "fft64.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double PI = 3.14159265358979323846264338327950288;

static double *g_tw[32];      /* g_tw[l]: n = 2^l, n/2 complex e^{-2 pi i k/n} */
#define NP2_MAX 8192
static double *g_twn[NP2_MAX + 1]; /* other lengths n: n complex e^{-2 pi i k/n} */
static pthread_mutex_t g_tw_lock = PTHREAD_MUTEX_INITIALIZER;
static int g_threads = 0;

static int ilog2(int n) {
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static const double *twiddles_np2(int n) {
    double *t = __atomic_load_n(&g_twn[n], __ATOMIC_ACQUIRE);
    if (t) return t;
    pthread_mutex_lock(&g_tw_lock);
    t = g_twn[n];
    if (!t) {
        t = (double *)malloc(sizeof(double) * 2 * n);
        for (int k = 0; k < n; k++) {
            double ang = 2.0 * PI * (double)k / (double)n;
            t[2 * k] = cos(ang);
            t[2 * k + 1] = -sin(ang);
        }
        __atomic_store_n(&g_twn[n], t, __ATOMIC_RELEASE);
    }
    pthread_mutex_unlock(&g_tw_lock);
    return t;
}

static const double *twiddles(int n) {
    if (!is_pow2(n)) {
        if (n > NP2_MAX) abort();
        return twiddles_np2(n);
    }
    int l = ilog2(n);
    double *t = __atomic_load_n(&g_tw[l], __ATOMIC_ACQUIRE);
    if (t) return t;
    pthread_mutex_lock(&g_tw_lock);
    t = g_tw[l];
    if (!t) {
        int h = n / 2 > 0 ? n / 2 : 1;
        t = (double *)malloc(sizeof(double) * 2 * h);
        for (int k = 0; k < h; k++) {
            double ang = 2.0 * PI * (double)k / (double)n;
            t[2 * k] = cos(ang);
            t[2 * k + 1] = -sin(ang);
        }
        __atomic_store_n(&g_tw[l], t, __ATOMIC_RELEASE);
    }
    pthread_mutex_unlock(&g_tw_lock);
    return t;
}

void fft64_set_threads(int nthreads) { g_threads = nthreads; }

int fft64_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

static int smallest_factor(int n) {
    for (int p = 2; p * p <= n; p++)
        if (n % p == 0) return p;
    return n;
}

/* y[0..n) = DFT of the n complex values x[0], x[xs], ... (any n): p = smallest prime
 * factor of n; the p sub-transforms of length m = n/p of the subsequences x[r xs p^0 ...]
 * go to y[r m ..], then Y[k + q m] = sum_r w^{r (k + q m)} Y_r[k]. tw: the table of length
 * n0 (a multiple of n), used at stride n0/n; sign -1 forward, +1 backward. */
static void dft_mixed(const double *x, ptrdiff_t xs, double *y, int n, int sign, const double *tw, int n0) {
    if (n == 1) {
        y[0] = x[0];
        y[1] = x[1];
        return;
    }
    const int p = smallest_factor(n), m = n / p, ts = n0 / n;
    double *sub = (double *)malloc(sizeof(double) * 2 * n);
    if (m == 1) {
        for (int r = 0; r < p; r++) {
            sub[2 * r] = x[2 * r * xs];
            sub[2 * r + 1] = x[2 * r * xs + 1];
        }
    } else {
        for (int r = 0; r < p; r++) dft_mixed(x + 2 * r * xs, xs * p, sub + 2 * r * m, m, sign, tw, n0);
    }
    for (int k = 0; k < m; k++)
        for (int q = 0; q < p; q++) {
            const int kk = k + q * m;
            double ar = 0.0, ai = 0.0;
            for (int r = 0; r < p; r++) {
                const int e = (int)(((long)r * kk) % n) * ts;
                const double wr = tw[2 * e], wi = (sign < 0 ? 1.0 : -1.0) * tw[2 * e + 1];
                const double vr = sub[2 * (r * m + k)], vi = sub[2 * (r * m + k) + 1];
                ar += vr * wr - vi * wi;
                ai += vr * wi + vi * wr;
            }
            y[2 * kk] = ar;
            y[2 * kk + 1] = ai;
        }
    free(sub);
}

/* contiguous in-place transform of n complex values */
static void fft_contig(double *x, int n, int sign) {
    if (n <= 1) return;
    if (!is_pow2(n)) {
        double *in = (double *)malloc(sizeof(double) * 2 * n);
        memcpy(in, x, sizeof(double) * 2 * n);
        dft_mixed(in, 1, x, n, sign, twiddles(n), n);
        free(in);
        return;
    }
    /* bit reversal */
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = x[2 * i], ti = x[2 * i + 1];
            x[2 * i] = x[2 * j];
            x[2 * i + 1] = x[2 * j + 1];
            x[2 * j] = tr;
            x[2 * j + 1] = ti;
        }
    }
    const double *tw = twiddles(n);
    const double s = (sign < 0) ? 1.0 : -1.0; /* conjugate table for backward */
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int i = 0; i < n; i += len) {
            for (int j = 0; j < half; j++) {
                double wr = tw[2 * j * step], wi = s * tw[2 * j * step + 1];
                double *u = x + 2 * (i + j), *v = x + 2 * (i + j + half);
                double vr = v[0] * wr - v[1] * wi;
                double vi = v[0] * wi + v[1] * wr;
                v[0] = u[0] - vr;
                v[1] = u[1] - vi;
                u[0] += vr;
                u[1] += vi;
            }
        }
    }
}

#define STACK_LINE 4096

void fft64_c2c_line(double *x, int n, ptrdiff_t stride, int sign) {
    if (stride == 1) {
        fft_contig(x, n, sign);
        return;
    }
    double stackbuf[2 * STACK_LINE];
    double *buf = n <= STACK_LINE ? stackbuf : (double *)malloc(sizeof(double) * 2 * n);
    for (int i = 0; i < n; i++) {
        buf[2 * i] = x[2 * i * stride];
        buf[2 * i + 1] = x[2 * i * stride + 1];
    }
    fft_contig(buf, n, sign);
    for (int i = 0; i < n; i++) {
        x[2 * i * stride] = buf[2 * i];
        x[2 * i * stride + 1] = buf[2 * i + 1];
    }
    if (buf != stackbuf) free(buf);
}

void fft64_r2c_line(const double *in, ptrdiff_t istride, double *out, ptrdiff_t ostride, int n) {
    int M = n / 2;
    double stackbuf[2 * STACK_LINE];
    double *z = M <= STACK_LINE ? stackbuf : (double *)malloc(sizeof(double) * 2 * M);
    for (int m = 0; m < M; m++) {
        z[2 * m] = in[(2 * m) * istride];
        z[2 * m + 1] = in[(2 * m + 1) * istride];
    }
    fft_contig(z, M, -1);
    const double *tw = twiddles(n);
    for (int k = 0; k <= M; k++) {
        int k1 = k % M, k2 = (M - k) % M;
        double zr = z[2 * k1], zi = z[2 * k1 + 1];
        double cr = z[2 * k2], ci = -z[2 * k2 + 1];      /* conj(Z[M-k]) */
        double er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci); /* even part */
        double dr = 0.5 * (zr - cr), di = 0.5 * (zi - ci);
        double orr = di, oi = -dr;                         /* (Z - conj)/(2i) */
        double wr, wi;
        if (k < M) { wr = tw[2 * k]; wi = tw[2 * k + 1]; }
        else { wr = -1.0; wi = 0.0; }
        out[2 * k * ostride] = er + (wr * orr - wi * oi);
        out[2 * k * ostride + 1] = ei + (wr * oi + wi * orr);
    }
    if (z != stackbuf) free(z);
}

void fft64_c2r_line(const double *in, ptrdiff_t istride, double *out, ptrdiff_t ostride, int n) {
    int M = n / 2;
    double stackbuf[2 * STACK_LINE];
    double *z = M <= STACK_LINE ? stackbuf : (double *)malloc(sizeof(double) * 2 * M);
    const double *tw = twiddles(n);
    for (int k = 0; k < M; k++) {
        double xr = in[2 * k * istride], xi = in[2 * k * istride + 1];
        double yr = in[2 * (M - k) * istride], yi = -in[2 * (M - k) * istride + 1]; /* conj(X[M-k]) */
        if (k == 0) { xi = 0.0; yi = 0.0; } /* Im of X[0] and X[N/2] ignored */
        double sr = xr + yr, si = xi + yi;
        double dr = xr - yr, di = xi - yi;
        /* omega^k = e^{+2 pi i k/n} = conj(tw[k]) */
        double wr = tw[2 * k], wi = -tw[2 * k + 1];
        double tr = wr * dr - wi * di, ti = wr * di + wi * dr;
        /* i * t */
        z[2 * k] = sr - ti;
        z[2 * k + 1] = si + tr;
    }
    fft_contig(z, M, +1);
    for (int m = 0; m < M; m++) {
        out[(2 * m) * ostride] = z[2 * m];
        out[(2 * m + 1) * ostride] = z[2 * m + 1];
    }
    if (z != stackbuf) free(z);
}

void fft64_r2c_3d(int n0, int n1, int n2, const double *in, double *out) {
    int h = n2 / 2 + 1;
    long lines = (long)n0 * n1;
    int nt = fft64_get_threads();
    (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long l = 0; l < lines; l++)
        fft64_r2c_line(in + l * n2, 1, out + 2 * l * h, 1, n2);
    /* axis 1: for each (i, k) */
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long l = 0; l < (long)n0 * h; l++) {
        long i = l / h, k = l % h;
        fft64_c2c_line(out + 2 * (i * n1 * h + k), n1, h, -1);
    }
    /* axis 0: for each (j, k) */
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long l = 0; l < (long)n1 * h; l++)
        fft64_c2c_line(out + 2 * l, n0, (ptrdiff_t)n1 * h, -1);
}

void fft64_c2r_3d(int n0, int n1, int n2, const double *in, double *out) {
    int h = n2 / 2 + 1;
    size_t total = (size_t)n0 * n1 * h;
    double *work = (double *)malloc(sizeof(double) * 2 * total);
    memcpy(work, in, sizeof(double) * 2 * total);
    int nt = fft64_get_threads();
    (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long l = 0; l < (long)n1 * h; l++)
        fft64_c2c_line(work + 2 * l, n0, (ptrdiff_t)n1 * h, +1);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long l = 0; l < (long)n0 * h; l++) {
        long i = l / h, k = l % h;
        fft64_c2c_line(work + 2 * (i * n1 * h + k), n1, h, +1);
    }
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long l = 0; l < (long)n0 * n1; l++)
        fft64_c2r_line(work + 2 * l * h, 1, out + l * n2, 1, n2);
    free(work);
}
