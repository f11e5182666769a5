/*
 * FFTW3 API shim over oracle/fft64.c (test infrastructure only). A plan records
 * the transform and its buffers; fftw_execute runs it. Plans that the
 * reference never destroys are leaked, as they are under FFTW.
 */
#include "fftw3.h"
#include "../fft64.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { K_R2C_3D, K_C2R_3D, K_R2C_MANY, K_C2R_MANY };

struct psc_shim_plan {
    int kind;
    int n0, n1, n2;
    int howmany, istride, idist, ostride, odist;
    void *in, *out;
};

/* fft64 takes any length up to 8192; its real transforms need an even length */
static void check_len(int n) {
    if (n < 2 || n % 2 != 0 || n > 8192) {
        fprintf(stderr, "fftw shim: length %d is not an even length in [2, 8192]\n", n);
        exit(2);
    }
}

void *fftw_malloc(size_t n) {
    void *p = NULL;
    if (posix_memalign(&p, 64, n ? n : 64) != 0) return NULL;
    return p;
}

fftw_complex *fftw_alloc_complex(size_t n) { return (fftw_complex *)fftw_malloc(n * sizeof(fftw_complex)); }
void fftw_free(void *p) { free(p); }
int fftw_init_threads(void) { return 1; }

void fftw_plan_with_nthreads(int nthreads) {
    /* PSC_ORACLE_THREADS overrides the compiled-in n_threads so the CPU
     * baseline can use every host core. */
    const char *env = getenv("PSC_ORACLE_THREADS");
    fft64_set_threads(env ? atoi(env) : nthreads);
}

static fftw_plan mk(int kind) {
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    p->kind = kind;
    return p;
}

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out, unsigned flags) {
    (void)flags;
    check_len(n0); check_len(n1); check_len(n2);
    fftw_plan p = mk(K_R2C_3D);
    p->n0 = n0; p->n1 = n1; p->n2 = n2; p->in = in; p->out = out;
    return p;
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out, unsigned flags) {
    (void)flags;
    check_len(n0); check_len(n1); check_len(n2);
    fftw_plan p = mk(K_C2R_3D);
    p->n0 = n0; p->n1 = n1; p->n2 = n2; p->in = in; p->out = out;
    return p;
}

static fftw_plan many(int kind, int rank, const int *n, int howmany, void *in, const int *inembed, int istride,
                      int idist, void *out, const int *onembed, int ostride, int odist) {
    if (rank != 1 || inembed || onembed) {
        fprintf(stderr, "fftw shim: only rank-1 plans without embeds are supported\n");
        exit(2);
    }
    check_len(n[0]);
    fftw_plan p = mk(kind);
    p->n0 = n[0]; p->howmany = howmany;
    p->istride = istride; p->idist = idist; p->ostride = ostride; p->odist = odist;
    p->in = in; p->out = out;
    return p;
}

fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany, double *in, const int *inembed, int istride,
                                 int idist, fftw_complex *out, const int *onembed, int ostride, int odist,
                                 unsigned flags) {
    (void)flags;
    return many(K_R2C_MANY, rank, n, howmany, in, inembed, istride, idist, out, onembed, ostride, odist);
}

fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed,
                                 int istride, int idist, double *out, const int *onembed, int ostride, int odist,
                                 unsigned flags) {
    (void)flags;
    return many(K_C2R_MANY, rank, n, howmany, in, inembed, istride, idist, out, onembed, ostride, odist);
}

void fftw_execute(const fftw_plan p) {
    switch (p->kind) {
    case K_R2C_3D:
        fft64_r2c_3d(p->n0, p->n1, p->n2, (const double *)p->in, (double *)p->out);
        break;
    case K_C2R_3D:
        fft64_c2r_3d(p->n0, p->n1, p->n2, (const double *)p->in, (double *)p->out);
        break;
    case K_R2C_MANY: {
        const double *in = (const double *)p->in;
        double *out = (double *)p->out;
        int nt = fft64_get_threads();
        (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int t = 0; t < p->howmany; t++)
            fft64_r2c_line(in + (ptrdiff_t)t * p->idist, p->istride, out + 2 * (ptrdiff_t)t * p->odist, p->ostride,
                           p->n0);
        break;
    }
    case K_C2R_MANY: {
        const double *in = (const double *)p->in;
        double *out = (double *)p->out;
        int nt = fft64_get_threads();
        (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int t = 0; t < p->howmany; t++)
            fft64_c2r_line(in + 2 * (ptrdiff_t)t * p->idist, p->istride, out + (ptrdiff_t)t * p->odist, p->ostride,
                           p->n0);
        break;
    }
    }
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
