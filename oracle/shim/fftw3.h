/*
 * FFTW3 API shim for building the reference's own sources as the CPU oracle
 * (test infrastructure only; never linked into the product).
 *
 * FFTW is not installed on this machine, so the reference's calls to it are
 * served by oracle/fft64.c. Only the entry points the reference uses are
 * declared, with FFTW's public signatures (the reference's call sites must
 * compile unchanged): fftw_malloc / fftw_alloc_complex / fftw_free,
 * fftw_init_threads / fftw_plan_with_nthreads, fftw_plan_dft_{r2c,c2r}_3d,
 * fftw_plan_many_dft_{r2c,c2r} (rank 1, strided) and fftw_execute /
 * fftw_destroy_plan. Transforms are unnormalised, as FFTW's are.
 *
 * The reference's header uses std::array without including <array>; this shim
 * includes it so the unmodified header compiles.
 */
#ifndef PSC_SHIM_FFTW3_H
#define PSC_SHIM_FFTW3_H

#include <stddef.h>
#ifdef __cplusplus
#include <array>
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct psc_shim_plan *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
fftw_complex *fftw_alloc_complex(size_t n);
void fftw_free(void *p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out, unsigned flags);
fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany, double *in, const int *inembed,
                                 int istride, int idist, fftw_complex *out, const int *onembed, int ostride,
                                 int odist, unsigned flags);
fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed,
                                 int istride, int idist, double *out, const int *onembed, int ostride,
                                 int odist, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
