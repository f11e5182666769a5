/*
 * fft64 — FP64 power-of-two FFTs for the CPU oracle (test infrastructure only).
 *
 * This is the checker's transform library: it backs the FFTW-API shim that the
 * reference's own sources are compiled against (oracle/shim/fftw3.h), and the C
 * restatement of the evolution path (oracle/port/psc_oracle.c). Nothing in the
 * product links it.
 *
 * Conventions follow FFTW's, which the reference calls (evolution.cpp:1145-1150,
 * 1112-1113, 484-562): transforms are unnormalised; the forward transform uses
 * e^{-2 pi i k n / N}; a real transform of length N stores N/2+1 complex values;
 * a complex-to-real transform reads only X[0..N/2] and ignores the imaginary
 * parts of X[0] and X[N/2]; a 3-D real transform of a row-major [n0][n1][n2]
 * array produces [n0][n1][n2/2+1] with the last index fastest.
 *
 * Any length >= 2 (power-of-two lengths by radix-2, others mixed-radix up to
 * 8192); real transforms need an even length. Multi-line transforms run on all
 * host threads with OpenMP when it is enabled at compile time.
 */
#ifndef PSC_ORACLE_FFT64_H
#define PSC_ORACLE_FFT64_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* In-place complex transform of one line of n points, element stride `stride`
 * (in complex elements). sign = -1 forward, +1 backward (unnormalised). */
void fft64_c2c_line(double *x, int n, ptrdiff_t stride, int sign);

/* One real line -> n/2+1 complex, and back. Strides in elements (doubles for
 * real data, complex pairs for complex data). The c2r input is not modified. */
void fft64_r2c_line(const double *in, ptrdiff_t istride, double *out, ptrdiff_t ostride, int n);
void fft64_c2r_line(const double *in, ptrdiff_t istride, double *out, ptrdiff_t ostride, int n);

/* 3-D transforms of a row-major [n0][n1][n2] real array <-> [n0][n1][n2/2+1]
 * complex array (interleaved re,im). The c2r input is not modified. */
void fft64_r2c_3d(int n0, int n1, int n2, const double *in, double *out);
void fft64_c2r_3d(int n0, int n1, int n2, const double *in, double *out);

/* Number of host threads used by the multi-line transforms (default: all). */
void fft64_set_threads(int nthreads);
int fft64_get_threads(void);

#ifdef __cplusplus
}
#endif

#endif
