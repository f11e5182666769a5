/*
 * psc.h — C ABI of the GB300 pseudo-spectral lattice evolution (libpsc.so).
 *
 * The reference (PSpectCosmo) has no library interface: its path is a set of free
 * functions on global arrays, configured at compile time. This header is the
 * drop-in boundary for that path. Each entry point says which reference routine
 * it replaces (file:line inside the reference project).
 *
 *   compile-time parameters.h / model.h   -> psc_params (run-time values, same names)
 *   initialize() + initialize_GW()        -> psc_init_ic
 *   evolve_VV_k_nopad(dt) / evolve_VV(dt) -> psc_step
 *   spectra(), energy(), meansvars(), scale() -> psc_spectra, psc_energies, psc_means
 *   global arrays f_k, pi_k, u_k, pi_u_k, a, ad, add -> psc_get_state / psc_set_state
 *   histograms(), histograms_2d(), slices()   -> psc_histograms, psc_histograms_2d, psc_slices
 *   save_Snap() / the HDF5 snapshot files     -> psc_snapshot_arrays, psc_write_snapshot, psc_h5_*
 *   evolve_VV_k_pad(dt) (N_PAD != N)          -> psc_step on a handle created with N_pad
 *   ANALYTIC_EVOLUTION phase                  -> psc_analytic_begin / _step / _to_lattice
 *   (no reference counterpart) checkpoint/resume, ensembles, adjoint gradients
 *                                             -> psc_checkpoint_*, psc_batch_*, psc_adjoint*
 *
 * Conventions: every call returns PSC_OK (0) or a negative PSC_ERR_* code and
 * never throws or exits; psc_strerror names the code and psc_last_error gives the
 * message of the last failure on the calling thread. A handle owns its device
 * memory and one CUDA stream; calls on one handle must not run concurrently.
 * Complex arrays are interleaved (re, im) doubles in the reference's FFTW layout:
 * [N][N][N/2+1] with the last index fastest, one block of N*N*(N/2+1) complex per
 * field or tensor component. Real arrays are [N][N][N] doubles. Host buffers are
 * always FP64, whatever precision the device evolves in.
 */
#ifndef PSC_H
#define PSC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PSC_OK 0
#define PSC_ERR_CONFIG (-1)     /* unsupported parameter (N outside the sizes below, ...) */
#define PSC_ERR_ARG (-2)        /* null pointer / bad argument */
#define PSC_ERR_CUDA (-3)       /* a CUDA runtime call failed */
#define PSC_ERR_NONFINITE (-4)  /* the on-device finite check tripped (NaN/Inf in the background) */
#define PSC_ERR_TIMEOUT (-5)    /* a bounded device-side wait gave up */
#define PSC_ERR_STATE (-6)      /* call out of order (e.g. step before state is set) */
#define PSC_ERR_NOMEM (-7)      /* device allocation failed */
#define PSC_ERR_IO (-8)         /* a file could not be written */
#define PSC_ERR_DEVICE (-9)     /* a bounded wait ran out and the copies it waited for never completed:
                                   the CUDA context can no longer be trusted (destroy the handle and
                                   do no further GPU work in this process) */

#define PSC_MODEL_PHI2 0      /* V = phi^2/2 (reference model.h:35-99), built in */
#define PSC_MODEL_PHI2CHI2 1  /* V = phi^2/2 + gsq phi^2 chi^2 / 2 (two-field preheating), built in */
/* Model ids PSC_MODEL_USER + i: the model.h files compiled into the library (file i of the
 * PSC_MODEL_H list at build time, by default every .h file in pspectcosmo_gb300/models/),
 * each written in the reference's model interface (model.h:10-104) and evaluated on the
 * device in the lattice's precision; psc_model_find gives the id of a file stem. */
#define PSC_MODEL_USER 16
#define PSC_MAX_FIELDS 4      /* nflds <= 4 (built-in models: 1 and 2) */
#define PSC_MAX_TERMS 4       /* num_potential_terms <= 4 */

/*
 * Run configuration: the reference's compile-time parameters.h / model.h surface as
 * run-time values. Field names follow parameters.h.
 */
typedef struct psc_params {
    int N;                  /* parameters.h:22   points per lattice edge: a power of two in 8..1024 (the
                               register FFT engine from 32 on), or an even size in 8..512 whose prime
                               factors are 2, 3, 5, 7 (e.g. 24, 40, 56, 96; the generic engine) */
    int nflds;              /* parameters.h:20   number of scalar fields: 1 .. PSC_MAX_FIELDS (GWs with more
                               than two fields: N <= 512) */
    int vv;                 /* parameters.h:10   integrator: 2 (velocity Verlet), 4, 6, 8, 10 (Yoshida) */
    int alpha;              /* parameters.h:120  time variable exponent (0 = cosmic time) */
    int expansion;          /* parameters.h:67   must be 2 (self-consistent Friedmann) for evolution */
    int simulate_inflation; /* parameters.h:17   fixed-amplitude ICs + R_Q2C mask in K, G */
    int spectral;           /* parameters.h:12   1: evolve_VV_k_nopad semantics, 0: evolve_VV (real space) */
    int with_gw;            /* parameters.h:15   tensor perturbations u_ij: evolved on the real-space path
                               (spectral = 0); on the spectral path they keep their initial values
                               and appear in the GW spectra, as the reference does */
    int precision;          /* 64: FP64 state (the plain method) or 32: FP32 state, FP64 background */
    int model;              /* model.h: PSC_MODEL_PHI2, PSC_MODEL_PHI2CHI2 or PSC_MODEL_USER + i */
    int seed;               /* parameters.h:65   Park-Miller seed (rand_uniform, initialize.cpp:13) */
    int N_pad;              /* parameters.h:13,23 PAD_FLAG / N_pad: 0 = off, else the padded grid of the
                               dealiased spectral step evolve_VV_k_pad (N < N_pad, a size N may take,
                               spectral = 1, no GWs) */
    double kIR;             /* parameters.h:27   smallest lattice wavenumber (program units) */
    double a0;              /* parameters.h:29   initial scale factor */
    double MPl;             /* parameters.h:121  Planck mass */
    double m_in_MPl;        /* parameters.h:110  mass in Planck units (omegaStar = m_in_MPl * fStar) */
    double fStar;           /* parameters.h:127  field unit (0 => MPl) */
    double epsilon;         /* parameters.h:39   R_Q2C threshold of the K, G mask */
    double gsq;             /* coupling g^2 of PSC_MODEL_PHI2CHI2 in program units (a user model
                               holds its own couplings, as a model.h does) */
    double initfield[PSC_MAX_FIELDS];    /* parameters.h:123  initial homogeneous fields */
    double initderivs[PSC_MAX_FIELDS];   /* parameters.h:124  initial homogeneous field derivatives */
    double kcutoff;         /* parameters.h:30   initial low-pass cut (0 = none) */
} psc_params;

typedef struct psc_handle psc_handle;

/* ---- the model surface (model.h). The reference compiles one model.h into its binary;
 * this library compiles a list of them (see PSC_MODEL_USER) next to its two built-in
 * models. psc_model_count: number of user models; psc_model_name: the name of a model id,
 * the file stem for a user model and "builtin:phi2", "builtin:phi2chi2" for the built-ins
 * (NULL for an unknown id); psc_model_find: the id of such a name (PSC_ERR_CONFIG when
 * unknown); psc_model_nterms: num_potential_terms of a model id (0 when unknown). */
int psc_model_count(void);
const char *psc_model_name(int model);
int psc_model_find(const char *name, int *model);
int psc_model_nterms(int model);

/* Evaluates the model of p (p->model, p->nflds, p->gsq, p->precision) at n field points
 * (fields [n][nflds], FP64) the way the lattice does: dvdf [n][nflds] = dvdf(fld, f) (model.h
 * dvdf, in the arithmetic of the lattice path of p->precision), terms [n][nterms] =
 * potential_energy(term, f) (same arithmetic), mass_sq [n][nflds] = effective_mass(f) (FP64,
 * as the initial conditions and spectra use it); any output may be NULL. on_device = 1
 * evaluates on the current GPU (the device code the passes call), 0 on the host (the same
 * model code compiled for the host). The reference's counterpart is a direct call of
 * model.h's functions (evolution.cpp:1077-1109, initialize.cpp:644). */
int psc_model_eval(const psc_params *p, int on_device, long long n, const double *fields, double *dvdf,
                   double *terms, double *mass_sq);

/* Fill *p with the reference's shipped parameters.h / model.h values (N = 64,
 * one field, VV = 2, kIR = 25, phi0 = 11, spectral path, FP64). */
void psc_default_params(psc_params *p);

/* Allocate device state for one lattice (replaces the allocation block of the
 * reference main, pspectcosmo.cpp:253-282). Validates the configuration. */
int psc_create(const psc_params *p, psc_handle **out);
void psc_destroy(psc_handle *h);

/* Initial conditions with the reference's RNG stream and mode order
 * (initialize.cpp:562-810 and, with GWs, initialize_GW initialize.cpp:341-470).
 * Generated on the device, one thread per mode, each thread reaching its draws of the
 * Park-Miller stream by skip-ahead (the integer draws are the reference's exactly);
 * seed < 1 (constant draws) and an initial low-pass cut (kcutoff) use the FP64 host
 * generator of psc_generate_ic and upload. Then a'' as kernel_a_k_nopad / kernel_a
 * (evolution.cpp:1061, 421). */
int psc_init_ic(psc_handle *h);

/* Host-only initial conditions: fills f_k, pi_k (nflds blocks) and, with GWs,
 * u_k, pi_u_k (6 blocks) exactly as initialize() / initialize_GW() do
 * (initialize.cpp:562-810, 341-470), without touching a GPU. info (may be NULL)
 * receives {hubble_init, a, ad, printed a'', kinetic, potential}
 * (initialize.cpp:649-670). Buffers are overwritten entirely. */
int psc_generate_ic(const psc_params *p, double *f_k, double *pi_k, double *u_k, double *pi_u_k, double *info);

/* Replace the state. f_k, pi_k: nflds blocks; u_k, pi_u_k: 6 blocks (components
 * 00,01,02,11,12,22) or NULL when GWs are off. add < 0 is not special: the value
 * is taken as given. Equivalent to writing the reference's globals. */
int psc_set_state(psc_handle *h, const double *f_k, const double *pi_k, double a, double ad, double add,
                  const double *u_k, const double *pi_u_k);
int psc_get_state(psc_handle *h, double *f_k, double *pi_k, double *a, double *ad, double *add,
                  double *u_k, double *pi_u_k);
int psc_get_time(psc_handle *h, double *t);
int psc_set_time(psc_handle *h, double t);

/* Advance nsteps steps of size dt: evolve_VV_k_nopad (evolution.cpp:1131-1198)
 * when spectral = 1, evolve_VV (evolution.cpp:607-694) when spectral = 0. The
 * step sequence is captured in a CUDA graph. Returns PSC_ERR_NONFINITE if the
 * background became non-finite (the reference aborts in meansvars/scale,
 * output.cpp:450-454, 480-483). */
int psc_step(psc_handle *h, double dt, int nsteps);

/* Real-space fields f, pi_f ([nflds][N^3], what meansvars() reads after its c2r,
 * output.cpp:396-424). Either pointer may be NULL. */
int psc_get_fields_real(psc_handle *h, double *f, double *pi_f);

/* Radial-bin spectra of spectra() (output.cpp:490-705, 780-1062). Arrays have
 * maxnumbins = (int)(sqrt(3) N/2) + 2 entries (parameters.h:25); pass NULL for
 * any output not needed. numpoints[l] counts modes in bin l (bit-exact integer);
 * f2/pi2/n2 are the per-bin MEANS the reference computes before printing,
 * [nflds][maxnumbins]; h2/hdot2 are the GW per-bin means ([maxnumbins]); gw_numpoints
 * the GW bin counts. */
int psc_maxnumbins(int N);
int psc_spectra(psc_handle *h, int32_t *numpoints, double *f2, double *pi2, double *n2, int32_t *gw_numpoints,
                double *h2, double *hdot2, double *hdot2_zero);

/* Energy components of energy_density() (output.cpp:57-115): per field K and G
 * ([nflds] each, masked by R_Q2C on the spectral path), per potential term V
 * ([num_potential_terms]), their total, the Friedmann-constraint violation of
 * energy() (output.cpp:1178-1185) and the GW energy density rho_GW of spectra()
 * (output.cpp:1030-1060; 0 without GWs). Any pointer may be NULL. */
int psc_energies(psc_handle *h, double *K, double *G, double *V, double *total, double *friedmann_violation,
                 double *rho_gw);

/* meansvars() (output.cpp:380-461): per field <f>, a^(alpha-3)<pi>, <f^2>,
 * a^(2(alpha-3))<pi^2>, rms(f), a^(alpha-3) rms(pi); out has 6*nflds doubles. */
int psc_means(psc_handle *h, double *out);

/* <effective_mass(f(x))> over the lattice, the mass_sq_av of spectra() (output.cpp:566-580)
 * that its occupation numbers n_k use; out has nflds doubles. */
int psc_mass_sq_av(psc_handle *h, double *out);

/* histograms() (output.cpp:1193-1297): for each field, the nbins frequencies of its
 * real-space values ([nflds][nbins], each count divided by the number of points
 * binned), the lower edge of the first bin and the bin width ([nflds] each). With
 * hmin == hmax (the reference's histogram_min == histogram_max) the bins span the
 * field's current minimum and maximum; otherwise [hmin, hmax]. Bin index
 * (int)((f - bmin) / df) in FP64, the maximum in the last bin, as the reference. */
int psc_histograms(psc_handle *h, int nbins, double hmin, double hmax, double *binfreq, double *bmin, double *df);

/* histograms_2d() (output.cpp:1300-1413) of the field pair (fld1, fld2): binfreq
 * [nbins0][nbins1] = counts / N^3 (the reference's normalisation), bmin[2], df[2]; limits
 * as psc_histograms (hmin == hmax: the fields' own minima and maxima). */
int psc_histograms_2d(psc_handle *h, int fld1, int fld2, int nbins0, int nbins1, double hmin, double hmax,
                      double *binfreq, double *bmin, double *df);

/* slices() (output.cpp:1415-1539): per field the values of a slicedim-dimensional slice
 * through the origin (a z line at x = y = 0, the x = 0 plane, or the lattice), every
 * sliceskip-th site up to slicelength * sliceskip (at most N), each the mean of its
 * sliceskip block when sliceaverage. out = [nflds][*count] in the reference's output
 * order (NULL: only *count). */
int psc_slices(psc_handle *h, int slicedim, int slicelength, int sliceskip, int sliceaverage, double *out,
               long long *count);

/* The datasets of snapshots() (output.cpp:1541-1648), N^3 doubles each, [x][y][z];
 * any pointer may be NULL: f = the real-space fields [nflds][N^3]; pot, kin, grad,
 * tot = the lattice energy densities of SNAPSHOTS_ENERGY at the current scale factor
 * (kinetic_energy_lattice and gradient_energy_lattice, evolution.cpp:7-138; the
 * potential and their sum, output.cpp:1614-1627). */
int psc_snapshot_arrays(psc_handle *h, double *f, double *pot, double *kin, double *grad, double *tot);

/* Writes the reference's snapshot file (output.cpp:1541-1648; the reference names it
 * <dir>/Snapshots/data_<step>_snapshot.h5) at `path`: HDF5 with the N x N x N
 * IEEE F64LE datasets /ScalarField_<fld> and, when with_energy (SNAPSHOTS_ENERGY),
 * /PotentialEnergy, /KineticEnergy, /GradientEnergy and /TotalEnergy. The file is
 * written by the library's own HDF5 writer (no libhdf5 needed). PSC_ERR_IO when
 * the file cannot be written. */
int psc_write_snapshot(psc_handle *h, const char *path, int with_energy);

/* Checkpoint / resume in a fixed format (the reference's own checkpoint, output.cpp:1652-1705,
 * stores only real-space fields and cannot resume a k-space run, initialize.cpp:590-620).
 * An HDF5 file (the library's writer) with the full state in the layout of psc_get_state:
 * /f_k, /pi_k [nflds][N*N*(N/2+1)][2] and with GWs /u_k, /pi_u_k [6][...][2], FP64;
 * /background = {t, a, a', a''}; /lattice = {N, nflds, with_gw, spectral, N_pad, vv,
 * model, precision}. psc_checkpoint_read restores state, background and t into a handle
 * of the same N, nflds and with_gw (PSC_ERR_CONFIG otherwise); a run continued from it
 * repeats the uninterrupted run bit for bit. */
int psc_checkpoint_write(psc_handle *h, const char *path);
int psc_checkpoint_read(psc_handle *h, const char *path);

/* The HDF5 writer alone (host only): n datasets names[i] of shape dims[0..rank) from
 * the host FP64 arrays data[i], in the layout psc_write_snapshot uses. */
int psc_h5_write_f64(const char *path, int n, const char *const *names, const double *const *data, int rank,
                     const uint64_t *dims);
/* Reading back a file in that layout (host only; other HDF5 layouts are refused with
 * PSC_ERR_IO): the shape of dataset `name` (rank, dims[0..min(rank, maxrank))) and its
 * count FP64 values. */
int psc_h5_dataset_shape(const char *path, const char *name, uint64_t *dims, int maxrank, int *rank);
int psc_h5_read_f64(const char *path, const char *name, double *out, uint64_t count);

/* Device-time of the last psc_step call (CUDA events on the handle's stream), ms. */
int psc_last_step_ms(psc_handle *h, float *ms);

/* Per-pass device times of one stage (no reference counterpart; the measurement
 * hook of the benchmark): runs `reps` force evaluations of the current state with
 * CUDA events between the kernels on the handle's stream and writes the average
 * milliseconds of [X inverse pass, Y inverse pass, fused Z pass, Y forward pass,
 * X forward pass + kick, background update] to ms[0..5]. The state is left as
 * it was (the evaluations apply zero-length kicks). */
#define PSC_NPASS 6
int psc_time_passes(psc_handle *h, int reps, float *ms);

/* Sets the state from a coarser Nsrc lattice (Nsrc < N, power of two; arrays in the
 * layout of psc_set_state at Nsrc): every mode is placed at its image in this N lattice
 * by the zero-padding of padding() (evolution.cpp:1271-1443: zero outside the Nsrc band,
 * each Nyquist index split over its +-Nsrc/2 images with 1/2 per Nyquist axis) with the
 * amplitudes times (N/Nsrc)^3 for the unnormalised transforms, so the real-space fields
 * are the spectral interpolation of the coarse ones. u_k, pi_u_k as in psc_set_state. */
int psc_set_state_padded(psc_handle *h, int Nsrc, const double *f_k, const double *pi_k, double a, double ad,
                         double add, const double *u_k, const double *pi_u_k);

/* ANALYTIC_EVOLUTION, the analytic pre-lattice phase (single-lattice handles):
 *   psc_analytic_begin      k_square_initialize + initialize_analytic_perturbation
 *                           (initialize.cpp:815-958, 1124-1138): the background and, for every
 *                           distinct k^2 of the lattice, the left and right Bunch-Davies mode
 *                           functions of every field, at t = 0;
 *   psc_analytic_step       evolve_VV_analytic_perturbation(dt) (evolution.cpp:167-336): the
 *                           background on the host, every mode on the device;
 *   psc_analytic_background t, a, a', a'' and the homogeneous fields / momenta ([nflds]);
 *   psc_analytic_modes      the number of distinct k^2, their values (sorted) and the modes
 *                           [4][nflds][nk] complex (f_left, pi_left, f_right, pi_right; index 0
 *                           holds the background as the reference stores it: (f, 0) and
 *                           (pi, pi at the last half step)), any pointer may be NULL;
 *   psc_analytic_to_lattice initialize_lattice() (initialize.cpp:961-1097): the lattice state
 *                           from the modes with the reference's random phases and amplitudes,
 *                           a, a', a'' and t of the phase (no GW modes). */
int psc_analytic_begin(psc_handle *h);
int psc_analytic_step(psc_handle *h, double dt);
int psc_analytic_background(psc_handle *h, double *t, double *a, double *ad, double *add, double *f_bg,
                            double *pi_bg);
int psc_analytic_modes(psc_handle *h, int *nk, int32_t *k2, double *modes);
int psc_analytic_to_lattice(psc_handle *h);

/* Device time of one c2r of the nflds field arrays f_k to real space (X, Y inverse
 * passes and the Z c2r pass, the transform of the reference's isChanged block,
 * output.cpp:1555-1578), averaged over `reps` launches on the handle's stream, ms.
 * The yardstick against a library 3-D c2r of the same size; the result is left in
 * the real-space buffer that psc_get_fields_real reads. */
int psc_time_c2r(psc_handle *h, int reps, float *ms);

/* FFT tile and grid shapes picked by measurement (no reference counterpart: the reference
 * plans its FFTW transforms with FFTW_ESTIMATE). Times, on the handle's current state, every
 * candidate shape of the register-engine passes (N >= 32): lines per tile of the X and Y passes
 * (the default and two narrower tiles), and lines per tile x resident blocks per SM of the Z
 * pass; each candidate runs reps + 1 stage evaluations with zero drift and kick coefficients
 * (the state is left as it was). The fastest shapes stay in use for the handle (the step graph
 * is captured again) and are cached per configuration (N, nflds, GWs, precision, batch size,
 * user model, SM count) for the process and, when the environment variable PSC_TUNE_CACHE
 * names a file, across processes; a cached configuration is applied without timing
 * (*from_cache = 1). shape (may be NULL) receives {log2 X/Y lines per tile, log2 Z lines per
 * tile, Z blocks per SM}, -1 where the handle has nothing to tune (N < 32, padded step).
 * The shapes set the order of the K, G and <V> partial sums, so results differ from another
 * shape's at the rounding of those reductions; a run with given shapes is reproducible. */
int psc_autotune(psc_handle *h, int reps, int *shape, int *from_cache);
/* The shapes in use ({-1, -1, -1} where nothing is tunable), and a given set of shapes (as
 * psc_autotune reports them; each is clamped to its limits, -1 / 0 = the default), e.g. a
 * choice recorded by an earlier run. */
int psc_get_shapes(psc_handle *h, int *shape);
int psc_set_shapes(psc_handle *h, const int *shape);

/* Tile staging by tensor maps (TMA; no reference counterpart). The register-engine passes
 * stage their tiles in shared memory with tiled tensor copies: PSC_TMAP_X, the X inverse (FP32)
 * and the X forward + kick pass (input and operand tiles, every N >= 32); PSC_TMAP_Y, the FP32 Y
 * forward pass at N = 128 .. 1024 (where a tile's lines divide N/2; persistent, the next tile's
 * copies in flight during the current transform) and, at N = 1024, the FP32 GW Y inverse pass in
 * the same pipelined form (it measured slower at 256); PSC_TMAP_YINV (with PSC_TMAP_Y) takes that
 * form at every size from 128 on (tests, timing). Without them each thread loads its own
 * elements. Both forms give bit-identical results. psc_set_tensor_maps allows the groups in mask
 * (both by default; a group also needs a fitting shape); psc_get_tensor_maps reports the groups
 * in use. */
#define PSC_TMAP_X 1
#define PSC_TMAP_Y 2
#define PSC_TMAP_YINV 4
int psc_set_tensor_maps(psc_handle *h, int mask);
int psc_get_tensor_maps(psc_handle *h, int *mask);

/* Compulsory HBM bytes each of the PSC_NPASS passes moves per launch (the bytes
 * of the arrays it must read and write once), for roofline accounting. */
int psc_pass_bytes(psc_handle *h, double *bytes);

/* Failure detection of the device-side waits (no reference counterpart). The GW Z pass
 * waits for its bulk copies (TMA) on an mbarrier for at most one second of wall time. When
 * a wait runs out, the block records PSC_ERR_TIMEOUT and waits once more (bounded) for the
 * copies still in flight, so that it never leaves while a copy can write into its shared
 * memory. If they land, psc_step returns PSC_ERR_TIMEOUT and the context stays usable
 * (psc_set_state / psc_init_ic / psc_checkpoint_read clear the handle's error). If they
 * never land, psc_step returns PSC_ERR_DEVICE: the context can no longer be trusted. After
 * a failure the rest of the step call does no work (no further waits).
 * This self-test runs that bounded wait on an mbarrier whose transactions never arrive, for
 * limit_ms milliseconds (0 < limit_ms <= 10000), and stores the kernel's status in *status:
 * PSC_ERR_TIMEOUT when the wait ran out as designed. */
int psc_selftest_bulk_wait(double limit_ms, int *status);

/* Test hook of the same waits on the real path. Sets the handle's wait limit to limit_ms
 * (0 < limit_ms <= 10000; 1000 by default) and, with plant_bytes > 0 (at most 4096), makes
 * every tile of the GW Z pass expect plant_bytes more than its copies deliver: the copies
 * land, the wait runs out, the timeout path counts the planted bytes itself and the block
 * leaves, so psc_step returns PSC_ERR_TIMEOUT. plant_bytes = 0 restores normal waits.
 * PSC_ERR_CONFIG when plant_bytes > 0 and the handle's GW Z pass does not stage its tiles by
 * bulk copies (FP32 GW runs with an even number of lines per tile do). */
int psc_test_wait_hook(psc_handle *h, double limit_ms, int plant_bytes);
/* The same hook on the tensor-map waits of another pass (PSC_NPASS order: 0 X inverse, 1 Y
 * inverse, 2 the GW Z pass as above, 3 Y forward, 4 X forward + kick): every tile that pass
 * stages by tensor copies expects plant_bytes more than its copies deliver, waits out the limit,
 * counts the planted bytes itself and leaves; psc_step returns PSC_ERR_TIMEOUT. PSC_ERR_CONFIG
 * when plant_bytes > 0 and the handle's pass does not stage its tiles that way
 * (psc_get_tensor_maps; the X inverse stages by tensor maps in FP32 only, the Y inverse with GWs
 * in FP32 only). */
int psc_test_wait_hook_pass(psc_handle *h, double limit_ms, int plant_bytes, int pass);

/* ---------------------------------------------------------------- batches
 * Ensembles of independent realizations (the batched-ensemble workload). The
 * reference runs one lattice per process; these entry points have no single
 * counterpart and compose the ones above. psc_batch_create groups the n
 * realizations by configuration (all psc_params fields except seed, initfield,
 * initderivs, a0 and kcutoff must agree within a group; sizes may differ between
 * groups). One CUDA graph holds a whole step of every group (see psc_batch_launch_mode for
 * how the groups' passes are launched). Realizations are addressed by
 * their index in the array given to psc_batch_create. */
typedef struct psc_batch psc_batch;
int psc_batch_create(const psc_params *per_realization, int n, psc_batch **out);
void psc_batch_destroy(psc_batch *b);
int psc_batch_size(psc_batch *b);
int psc_batch_groups(psc_batch *b);
int psc_batch_init_ic(psc_batch *b);                      /* initialize() for every realization */
int psc_batch_step(psc_batch *b, double dt, int nsteps);  /* nsteps steps of every realization */
int psc_batch_last_step_ms(psc_batch *b, float *ms);
int psc_batch_autotune(psc_batch *b, int reps);         /* psc_autotune for every group */
/* How the groups' passes are launched. By default every group's passes run on its own
 * stream, the streams forked and joined inside the step graph. per_group = 0 asks for ONE
 * launch per pass for all groups instead: persistent kernels over a work list of (group,
 * realization, array, tile), and one background launch per stage; it applies when every
 * group runs the register engine at N <= 256 with 256-thread blocks, a built-in model, and
 * one precision, GW setting and integrator (at most four groups). per_group = 1 restores the
 * default, -1 leaves the choice; *one_launch_per_pass (may be NULL) receives 1 when the
 * batched launches are in use. Both give each realization the results it has alone, bit for
 * bit. (On the mixed 32^3 / 64^3 / 128^3 ensemble the per-group launches are the faster:
 * their streams fill each other's kernel tails.) */
int psc_batch_launch_mode(psc_batch *b, int per_group, int *one_launch_per_pass);
int psc_batch_set_state(psc_batch *b, int idx, const double *f_k, const double *pi_k, double a, double ad, double add,
                        const double *u_k, const double *pi_u_k);
int psc_batch_get_state(psc_batch *b, int idx, double *f_k, double *pi_k, double *a, double *ad, double *add,
                        double *u_k, double *pi_u_k);
int psc_batch_spectra(psc_batch *b, int idx, int32_t *numpoints, double *f2, double *pi2, double *n2,
                      int32_t *gw_numpoints, double *h2, double *hdot2, double *hdot2_zero);
int psc_batch_energies(psc_batch *b, int idx, double *K, double *G, double *V, double *total,
                       double *friedmann_violation, double *rho_gw);
int psc_batch_means(psc_batch *b, int idx, double *out);
int psc_batch_histograms(psc_batch *b, int idx, int nbins, double hmin, double hmax, double *binfreq, double *bmin,
                         double *df);
int psc_batch_write_snapshot(psc_batch *b, int idx, const char *path, int with_energy);

/* Scalar power spectrum without any device allocation. It has no counterpart in
 * the reference; it is the bin-summing step of spectra() (output.cpp:626-690) for
 * callers that cannot call cudaMalloc: applications whose own memory pool owns all
 * device memory, or code that must not allocate once it is running (an allocation
 * synchronises the device and can fail late). Instead of a handle it takes the
 * caller's device arrays: f_k, pi_k ([nflds][N][N][N/2+1] complex of p->precision,
 * as psc_get_state lays them out) and the outputs numpoints, f2, pi2, n2
 * ([nflds][maxnumbins], any may be NULL), filled as psc_spectra fills them; a and
 * ad are the background. Only p->N, p->nflds, p->precision and p->alpha are read.
 * Limit: N <= PSC_NOALLOC_MAX_N and nflds <= 2, otherwise PSC_ERR_CONFIG. The bin
 * accumulators live in one fixed array of device memory inside the library (about
 * 50 KB, held by every GPU that loads the library until the process exits),
 * shared by all calls on a device: each call clears it first, so calls whose work
 * overlaps on the GPU (different streams or threads) race and must be serialised
 * by the caller. Every call looks up that array's address on the current device
 * (cudaGetSymbolAddress, which allocates nothing); the first call in a CUDA context also
 * loads the library's device code there, so make it before any stream capture. Work is
 * queued on `stream` (a cudaStream_t; NULL = default stream), which must belong to the
 * current device (PSC_ERR_ARG otherwise), and is complete when the stream is. Calls no
 * cudaMalloc or cudaFree. */
#define PSC_NOALLOC_MAX_N 1024
int psc_spectra_noalloc(const psc_params *p, double a, double ad, const void *f_k, const void *pi_k,
                        int32_t *numpoints, double *f2, double *pi2, double *n2, void *stream);

/* ---- discrete adjoint (no reference counterpart: the reference has no adjoint).
 * Differentiates the step of evolve_VV (evolution.cpp:607-694) for the scalar fields and
 * the self-consistent background (a'' through K, G, V: evolution.cpp:421-439), for the
 * observable O = <chi^2> (the last field's lattice mean of its square) after `nsteps`
 * steps of `dt` from the handle's current state, with a''(0) recomputed from that state.
 * Needs a single-lattice handle, N >= 32, expansion = 2 and the unmasked step
 * (spectral = 0, or simulate_inflation = 0); with GWs N <= 512. Checkpoints are taken every `every` steps
 * (every <= 0: one segment); each segment is recomputed once in the reverse sweep.
 * Outputs (any pointer but O may be NULL):
 *   grad_f_k, grad_pi_k  [nflds][N][N][N/2+1] complex as interleaved doubles:
 *                        dO/dRe + i dO/dIm of each stored half-spectrum mode;
 *   grad_ad0             dO/da'(0) at fixed a(0);
 *   grad_theta[2]        dO/d(gsq) and dO/d(mu), mu the coefficient of phi^2/2 in V (mu = 1).
 * On return the handle holds the final state, as after psc_step(h, dt, nsteps), and
 * psc_last_step_ms reports the device time of the whole computation (evaluation,
 * forward passes and reverse sweep; not the download of the gradients). */
int psc_adjoint_chi2(psc_handle *h, double dt, int nsteps, int every, double *O, double *grad_f_k,
                     double *grad_pi_k, double *grad_ad0, double *grad_theta);
/* The adjoint's forward map alone (the product step from a''(0) = A(state(0))): O after nsteps. */
int psc_adjoint_forward_chi2(psc_handle *h, double dt, int nsteps, double *O);

/* The same adjoint for a chosen observable (no reference counterpart):
 *   PSC_OBS_CHI2    O = <chi^2>, as psc_adjoint_chi2;
 *   PSC_OBS_RHO_GW  O = rho_GW, the GW energy density of energy() (output.cpp:1030-1060):
 *                   (fStar/MPl)^2 / (4 N^6 a^6) [sum over spectra()'s GW walk of the P-projected
 *                   |pi_u_k|^2 (output.cpp:18-53, 780-1062) + the k = 0 term]; needs with_gw = 1
 *                   and N <= 512 (spectral = 0, the GW path).
 * grad_u_k, grad_pi_u_k ([6][N][N][N/2+1] interleaved, may be NULL) receive dO/d(u_k(0), pi_u_k(0))
 * on a GW handle (zero for PSC_OBS_CHI2); the other outputs as psc_adjoint_chi2. */
#define PSC_OBS_CHI2 0
#define PSC_OBS_RHO_GW 1
int psc_adjoint(psc_handle *h, int observable, double dt, int nsteps, int every, double *O, double *grad_f_k,
                double *grad_pi_k, double *grad_u_k, double *grad_pi_u_k, double *grad_ad0, double *grad_theta);
int psc_adjoint_forward(psc_handle *h, int observable, double dt, int nsteps, double *O);

const char *psc_strerror(int code);
const char *psc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
