/*
 * psc_oracle — FP64 CPU restatement of the reference's evolution path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the CPU baseline of
 * bench.py. It follows the reference's algorithm routine by routine (file:line
 * citations in psc_oracle.c) with our own FFT (oracle/fft64.c), and is pinned
 * against the golden fixtures that the reference's own sources produce
 * (tests/golden/). The product never links or calls it.
 */
#ifndef PSC_ORACLE_H
#define PSC_ORACLE_H

#include "../../include/psc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_state orc_state;

orc_state *orc_create(const psc_params *p);
void orc_destroy(orc_state *s);
void orc_set_threads(int n);

/* initialize() (+ initialize_GW()); returns the printed ("pre-lattice") a'' */
double orc_init_ic(orc_state *s);
double orc_hubble_init(orc_state *s);

/* one step: evolve_VV_k_nopad (spectral) or evolve_VV (real space) */
void orc_step(orc_state *s, double dt);
/* the first nstages Yoshida stages of one step (a bounded CPU timing sample; the
 * state afterwards is not a step boundary) */
void orc_step_stages(orc_state *s, double dt, int nstages);
int orc_stages(orc_state *s);

/* background */
void orc_get_bg(orc_state *s, double *t, double *a, double *ad, double *add);
void orc_set_bg(orc_state *s, double t, double a, double ad, double add);

/* k-space state, same layout as psc_get_state (r2c of the real-space state on
 * the real-space path). u_k / pi_u_k: 6 symmetric components. */
void orc_get_state_k(orc_state *s, double *f_k, double *pi_k, double *u_k, double *pi_u_k);
/* set k-space state (spectral path), or the real-space state derived from it
 * by c2r (real-space path, as initialize() does) */
void orc_set_state_k(orc_state *s, const double *f_k, const double *pi_k, const double *u_k, const double *pi_u_k);
/* real-space f, pi_f [nflds][N^3] (c2r of the spectral state, as meansvars does) */
void orc_get_fields_real(orc_state *s, double *f, double *pi_f);
/* real-space GW tensors, 6 components (real-space path only) */
void orc_get_gw_real(orc_state *s, double *u, double *pi_u);

/* recompute a'' from the current state as kernel_a_k_nopad / kernel_a do */
double orc_kernel_a(orc_state *s);

int orc_maxnumbins(int N);
/* same outputs as psc_spectra */
void orc_spectra(orc_state *s, int *numpoints, double *f2, double *pi2, double *n2, int *gw_numpoints,
                 double *h2, double *hdot2, double *hdot2_zero);
/* same outputs as psc_energies */
void orc_energies(orc_state *s, double *K, double *G, double *V, double *total, double *fviol, double *rho_gw);
/* same output as psc_means */
void orc_means(orc_state *s, double *out);

/* Park-Miller stream of rand_uniform (initialize.cpp:13-28), for tests */
void orc_rand_stream(int seed, int count, double *out);

#ifdef __cplusplus
}
#endif
#endif
