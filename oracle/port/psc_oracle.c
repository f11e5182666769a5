/*
 * psc_oracle — FP64 CPU restatement of the reference's evolution path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the CUDA path and the CPU baseline of
 * bench.py; the product never links it). Each routine restates the reference
 * routine cited beside it, in the same order of operations, with oracle/fft64.c
 * standing in for FFTW. All citations are file:line in the reference project.
 */
#include "psc_oracle.h"
#include "../fft64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_D 3.14159265358979323846 /* pspectcosmo.h:27: 2*asin(1) */

static inline double pw2(double x) { return x * x; }

/* Yoshida composition weights (pspectcosmo.h:283-297); published coefficient
 * tables kept digit for digit so the stages match the reference's. */
static const double W4[3] = {1.351207191959657771818, -1.702414403875838200264, 1.351207191959657771818};
static const double W6[7] = {0.78451361047755726382, 0.23557321335935813368, -1.1776799841788710069,
                             1.3151863206839112189, -1.1776799841788710069, 0.23557321335935813368,
                             0.78451361047755726382};
static const double W8[15] = {0.74167036435061295345, -0.40910082580003159400, 0.19075471029623837995,
                              -0.57386247111608226666, 0.29906418130365592384, 0.33462491824529818378,
                              0.31529309239676659663, -0.79688793935291635402, 0.31529309239676659663,
                              0.33462491824529818378, 0.29906418130365592384, -0.57386247111608226666,
                              0.19075471029623837995, -0.40910082580003159400, 0.74167036435061295345};
static const double W10[31] = {
    -0.48159895600253002870, 0.0036303931544595926879, 0.50180317558723140279, 0.28298402624506254868,
    0.80702967895372223806,  -0.026090580538592205447, -0.87286590146318071547, -0.52373568062510581643,
    0.44521844299952789252,  0.18612289547097907887,   0.23137327866438360633, -0.52191036590418628905,
    0.74866113714499296793,  0.066736511890604057532,  -0.80360324375670830316, 0.91249037635867994571,
    -0.80360324375670830316, 0.066736511890604057532,  0.74866113714499296793, -0.52191036590418628905,
    0.23137327866438360633,  0.18612289547097907887,   0.44521844299952789252, -0.52373568062510581643,
    -0.87286590146318071547, -0.026090580538592205447, 0.80702967895372223806, 0.28298402624506254868,
    0.50180317558723140279,  0.0036303931544595926879, -0.48159895600253002870};

/* symmetric tensor component c <-> (i, j) */
static const int SYM_I[6] = {0, 0, 0, 1, 1, 2};
static const int SYM_J[6] = {0, 1, 2, 1, 2, 2};
static int sym_index(int i, int j) {
    if (i > j) { int t = i; i = j; j = t; }
    static const int tab[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    return tab[i][j];
}

struct orc_state {
    psc_params p;
    int N, H, nf, gw, spectral, alpha, nterms, s;
    long modes, sites;
    double kIR, L, dx, fStar, MPl, omegaStar, DFDP;
    const double *w;
    double t, a, ad, add, hubble_init;
    double *f_k, *pi_k, *f, *pi_f;
    /* spectral path */
    double *pi_k_half, *Vp, *Vp_k, *kern_k, *RQ2C, *cache;
    /* real-space path */
    double *pi_half, *lapl_buf, *kern_r, *work_k;
    double *u, *pi_u, *pi_u_half, *u_k, *pi_u_k, *fder;
    int der_valid;
    int rng_i, rng_next;
};

/* ---------------------------------------------------------------- model */
/* model.h:35-99 (phi^2) and the two-field phi^2 chi^2 model in the same API */
static double potential_term(const orc_state *s, int term, const double *v) {
    if (s->p.model == PSC_MODEL_PHI2) return 0.5 * pw2(v[0]);
    if (term == 0) return 0.5 * pw2(v[0]);
    return 0.5 * s->p.gsq * pw2(v[0]) * pw2(v[1]);
}
static double dvdf(const orc_state *s, int fld, const double *v) {
    if (s->p.model == PSC_MODEL_PHI2) return v[0];
    if (fld == 0) return v[0] + s->p.gsq * v[0] * pw2(v[1]);
    return s->p.gsq * pw2(v[0]) * v[1];
}
static void effective_mass(const orc_state *s, double *m2, const double *v) {
    if (s->p.model == PSC_MODEL_PHI2) { m2[0] = 1.; return; }
    m2[0] = 1. + s->p.gsq * pw2(v[1]);
    m2[1] = s->p.gsq * pw2(v[0]);
}

/* ---------------------------------------------------------------- RNG */
/* rand_uniform, initialize.cpp:13-28: Park-Miller minimal standard with Schrage's
 * factorisation; the first call discards 99 draws. */
static double rand_uniform(orc_state *s) {
    if (s->p.seed < 1) return 0.33;
    if (!(s->rng_next > 0)) s->rng_next = 1;
    if (s->rng_i == 0)
        for (s->rng_i = 1; s->rng_i < 100; s->rng_i++) rand_uniform(s);
    s->rng_next = 16807 * (s->rng_next % 127773) - 2836 * (s->rng_next / 127773);
    if (s->rng_next < 0) s->rng_next += 2147483647;
    return (double)s->rng_next / (double)2147483647;
}

void orc_rand_stream(int seed, int count, double *out) {
    orc_state tmp;
    memset(&tmp, 0, sizeof tmp);
    tmp.p.seed = seed;
    tmp.rng_next = seed;
    for (int i = 0; i < count; i++) out[i] = rand_uniform(&tmp);
}

/* ---------------------------------------------------------------- setup */
void orc_set_threads(int n) { fft64_set_threads(n); }

static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

orc_state *orc_create(const psc_params *p) {
    orc_state *s = (orc_state *)calloc(1, sizeof *s);
    s->p = *p;
    s->N = p->N;
    s->H = p->N / 2 + 1;
    s->nf = p->nflds;
    s->gw = p->with_gw;
    s->spectral = p->spectral;
    s->alpha = p->alpha;
    s->nterms = p->model == PSC_MODEL_PHI2 ? 1 : 2;
    s->modes = (long)s->N * s->N * s->H;
    s->sites = (long)s->N * s->N * s->N;
    s->kIR = p->kIR;
    s->MPl = p->MPl;
    s->fStar = p->fStar > 0 ? p->fStar : p->MPl;
    s->omegaStar = p->m_in_MPl * s->fStar;
    s->L = 2 * PI_D / s->kIR;          /* parameters.h:31 */
    s->dx = s->L / (double)s->N;       /* parameters.h:32 */
    s->DFDP = pow(s->omegaStar / s->fStar, 2) * (s->N / s->dx) / 2.; /* parameters.h:132 */
    switch (p->vv) {
    case 4: s->s = 3; s->w = W4; break;
    case 6: s->s = 7; s->w = W6; break;
    case 8: s->s = 15; s->w = W8; break;
    case 10: s->s = 31; s->w = W10; break;
    default: { static const double W2[1] = {1.}; s->s = 1; s->w = W2; }
    }
    s->rng_next = p->seed;
    s->a = p->a0;
    long m2 = 2 * s->modes;
    s->f_k = zalloc(m2 * s->nf);
    s->pi_k = zalloc(m2 * s->nf);
    s->f = zalloc(s->sites * s->nf);
    s->pi_f = zalloc(s->sites * s->nf);
    s->cache = zalloc(m2);
    s->RQ2C = zalloc(s->modes * s->nf);
    if (s->spectral) {
        s->pi_k_half = zalloc(m2 * s->nf);
        s->Vp = zalloc(s->sites * s->nf);
        s->Vp_k = zalloc(m2 * s->nf);
        s->kern_k = zalloc(m2 * s->nf);
    } else {
        s->pi_half = zalloc(s->sites * s->nf);
        s->lapl_buf = zalloc(s->sites);
        s->kern_r = zalloc(s->sites * s->nf);
        s->work_k = zalloc(m2);
    }
    if (s->gw) {
        s->u = zalloc(s->sites * 6);
        s->pi_u = zalloc(s->sites * 6);
        s->pi_u_half = zalloc(s->sites * 6);
        s->u_k = zalloc(m2 * 6);
        s->pi_u_k = zalloc(m2 * 6);
        s->fder = zalloc(s->sites * 3 * s->nf);
    }
    return s;
}

void orc_destroy(orc_state *s) {
    if (!s) return;
    double *bufs[] = {s->f_k, s->pi_k, s->f, s->pi_f, s->cache, s->RQ2C, s->pi_k_half, s->Vp, s->Vp_k,
                      s->kern_k, s->pi_half, s->lapl_buf, s->kern_r, s->work_k, s->u, s->pi_u,
                      s->pi_u_half, s->u_k, s->pi_u_k, s->fder};
    for (size_t i = 0; i < sizeof bufs / sizeof bufs[0]; i++) free(bufs[i]);
    free(s);
}

static inline int pcoord(int i, int N) { return i <= N / 2 ? i : i - N; }

/* c2r_3d followed by /N3, as every reference call site does */
static void c2r_norm(orc_state *s, const double *in_k, double *out) {
    fft64_c2r_3d(s->N, s->N, s->N, in_k, out);
    const double n3 = (double)s->sites;
#pragma omp parallel for schedule(static)
    for (long x = 0; x < s->sites; x++) out[x] /= n3;
}

/* ---------------------------------------------------------------- energies */
/* Caluculate_R_Q2C, evolution.cpp:1038-1056 (uses the current global a and ad) */
static void calc_RQ2C(orc_state *s) {
    const double a = s->a, ad = s->ad;
    for (int fld = 0; fld < s->nf; fld++) {
        const double *fk = s->f_k + 2 * s->modes * fld, *pk = s->pi_k + 2 * s->modes * fld;
        double *R = s->RQ2C + s->modes * fld;
#pragma omp parallel for schedule(static)
        for (long m = 1; m < s->modes; m++) {
            R[m] = s->DFDP / (sqrt(pw2(fk[2 * m]) + pw2(fk[2 * m + 1])) * pow(a, 3 - s->alpha) *
                              sqrt(pw2(ad / a * fk[2 * m] + pow(a, s->alpha - 3) * pk[2 * m]) +
                                   pw2(ad / a * fk[2 * m + 1] + pow(a, s->alpha - 3) * pk[2 * m + 1])));
        }
        R[0] = 0.;
    }
}

/* kinetic_energy_k / gradient_energy_k, evolution.cpp:923-1035: sums over the
 * half spectrum with weight 2 for 1 <= kz < N/2, masked by R_Q2C < epsilon when
 * simulating inflation */
static void kg_k(orc_state *s, int fld, double *K, double *G) {
    const int N = s->N, H = s->H;
    const int mask = s->p.simulate_inflation;
    const double *fk = s->f_k + 2 * s->modes * fld, *pk = s->pi_k + 2 * s->modes * fld;
    const double *R = s->RQ2C + s->modes * fld;
    double kin_in = 0, kin_pl = 0, gr_in = 0, gr_pl = 0;
#pragma omp parallel for schedule(static) reduction(+ : kin_in, kin_pl, gr_in, gr_pl)
    for (long ij = 0; ij < (long)N * N; ij++) {
        int i = (int)(ij / N), j = (int)(ij % N);
        int px = pcoord(i, N), py = pcoord(j, N);
        for (int k = 0; k < H; k++) {
            long m = ij * H + k;
            if (mask && !(R[m] < s->p.epsilon)) continue;
            double kin = pw2(pk[2 * m]) + pw2(pk[2 * m + 1]);
            double gr = pow(s->kIR, 2) * (px * px + py * py + k * k) * (pow(fk[2 * m], 2) + pow(fk[2 * m + 1], 2));
            if (k == 0 || k == N / 2) { kin_pl += kin; gr_pl += gr; }
            else { kin_in += kin; gr_in += gr; }
        }
    }
    double kinetic = kin_in * 2. + kin_pl;
    double grad = gr_in * 2. + gr_pl;
    *K = .5 * kinetic / pow(s->a, 6) / pw2((double)s->sites);
    grad /= (double)s->sites;
    grad /= 2.;
    *G = grad / pw2(s->a) / (double)s->sites;
}

/* kinetic_energy / gradient_energy (real-space path), evolution.cpp:375-418 */
static void kg_real(orc_state *s, int fld, double *K, double *G) {
    const double *pf = s->pi_f + s->sites * fld;
    double kin = 0;
#pragma omp parallel for schedule(static) reduction(+ : kin)
    for (long x = 0; x < s->sites; x++) kin += pw2(pf[x]);
    *K = .5 * kin / pow(s->a, 6) / (double)s->sites;
    /* gradient_energy: r2c of f into f_k, then the same k-space sum */
    double *fk = s->f_k + 2 * s->modes * fld;
    fft64_r2c_3d(s->N, s->N, s->N, s->f + s->sites * fld, fk);
    const int N = s->N, H = s->H;
    double gr_in = 0, gr_pl = 0;
#pragma omp parallel for schedule(static) reduction(+ : gr_in, gr_pl)
    for (long ij = 0; ij < (long)N * N; ij++) {
        int px = pcoord((int)(ij / N), N), py = pcoord((int)(ij % N), N);
        for (int k = 0; k < H; k++) {
            long m = ij * H + k;
            double gr = pow(s->kIR, 2) * (px * px + py * py + k * k) * (pow(fk[2 * m], 2) + pow(fk[2 * m + 1], 2));
            if (k == 0 || k == N / 2) gr_pl += gr; else gr_in += gr;
        }
    }
    double grad = gr_in * 2. + gr_pl;
    grad /= (double)s->sites;
    grad /= 2.;
    *G = grad / pw2(s->a) / (double)s->sites;
}

/* potential_energy(term, NULL): lattice average of one term (model.h:37-60) */
static double pot_avg(orc_state *s, int term) {
    double sum = 0;
    const long n = s->sites;
#pragma omp parallel for schedule(static) reduction(+ : sum)
    for (long x = 0; x < n; x++) {
        double v[2] = {s->f[x], s->nf > 1 ? s->f[n + x] : 0.};
        sum += potential_term(s, term, v);
    }
    return sum / (double)n;
}

/* V_E of kernel_a_k_nopad, evolution.cpp:1077-1085: per-site sum over terms */
static double pot_sites(orc_state *s) {
    double sum = 0;
    const long n = s->sites;
#pragma omp parallel for schedule(static) reduction(+ : sum)
    for (long x = 0; x < n; x++) {
        double v[2] = {s->f[x], s->nf > 1 ? s->f[n + x] : 0.};
        for (int term = 0; term < s->nterms; term++) sum += potential_term(s, term, v);
    }
    return sum / (double)n;
}

static double friedmann_add(const orc_state *s, double K, double G, double V) {
    const int al = s->alpha;
    return 1. / 3. * pw2(s->fStar / s->MPl) * pow(s->a, 1 + 2 * al) * ((al - 2) * K + al * G + (al + 1) * V);
}

/* kernel_a_k_nopad (evolution.cpp:1061-1090) / kernel_a (evolution.cpp:421-439) */
double orc_kernel_a(orc_state *s) {
    double K = 0, G = 0, V = 0;
    if (s->spectral) {
        if (s->p.simulate_inflation) calc_RQ2C(s);
        for (int fld = 0; fld < s->nf; fld++) {
            double k, g;
            kg_k(s, fld, &k, &g);
            K += k;
            G += g;
        }
        V = pot_sites(s);
    } else {
        for (int fld = 0; fld < s->nf; fld++) {
            double k, g;
            kg_real(s, fld, &k, &g);
            K += k;
            G += g;
        }
        for (int term = 0; term < s->nterms; term++) V += pot_avg(s, term);
    }
    return friedmann_add(s, K, G, V);
}

/* ---------------------------------------------------------------- ICs */
/* set_mode, initialize.cpp:128-220 */
static void set_mode(orc_state *s, double p2, double m2, double *fk, double *pk, int isReal) {
    const double a = s->a, H0 = s->hubble_init;
    double norm = sqrt(s->DFDP);
    double kc = s->p.kcutoff;
    double k2cutoff = (kc < 2. * PI_D * (double)s->N / s->L ? pw2(kc) : 0.);
    if (k2cutoff > 0. && p2 > k2cutoff) {
        fk[0] = fk[1] = pk[0] = pk[1] = 0.;
        return;
    }
    double omega = (p2 + m2 > 0.) ? sqrt(p2 + pw2(a) * m2) : sqrt(p2);
    double rms = omega > 0. ? norm / sqrt(omega) : 0.;
    if (s->p.simulate_inflation) {
        double amp = rms / a;
        double phase = 2. * PI_D * rand_uniform(s);
        double re = amp * cos(phase), im = amp * sin(phase);
        fk[0] = re;
        fk[1] = im;
        pk[0] = pow(a, s->alpha - 3) * (-omega * im - H0 * fk[0]);
        pk[1] = pow(a, s->alpha - 3) * (omega * re - H0 * fk[1]);
        if (isReal) {
            fk[0] = sqrt(pw2(fk[0]) + pw2(fk[1]));
            fk[1] = 0;
            pk[0] = sqrt(pw2(pk[0]) + pw2(pk[1]));
            pk[1] = 0.;
        }
    } else {
        double al = rms / sqrt(2.) * sqrt(log(1. / rand_uniform(s))) / a;
        double ar = rms / sqrt(2.) * sqrt(log(1. / rand_uniform(s))) / a;
        double ph = 2. * PI_D * rand_uniform(s);
        double rel = al * cos(ph), iml = al * sin(ph);
        ph = 2. * PI_D * rand_uniform(s);
        double rer = ar * cos(ph), imr = ar * sin(ph);
        fk[0] = rel + rer;
        fk[1] = iml + imr;
        pk[0] = pow(a, s->alpha - 3) * (-omega * (iml - imr) - H0 * fk[0]);
        pk[1] = pow(a, s->alpha - 3) * (omega * (rel - rer) - H0 * fk[1]);
        if (isReal) { fk[1] = 0.; pk[1] = 0.; }
    }
}

static void set_conj(double *arr, long conj, long idx) {
    arr[2 * conj] = arr[2 * idx];
    arr[2 * conj + 1] = -arr[2 * idx + 1];
}

/* orthogonal_unit_vectors + TT_tensors, initialize.cpp:66-122 */
static void tt_tensor(const double k[3], double e[3][3]) {
    double kn = sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
    double kh[3] = {k[0] / kn, k[1] / kn, k[2] / kn};
    double tmp[3] = {0, 0, 1};
    if (fabs(kh[0] - 0) < 1e-9 && fabs(kh[1] - 0) < 1e-9 && fabs(kh[2] - 1) < 1e-9) { tmp[1] = 1; tmp[2] = 0; }
    double u[3] = {kh[1] * tmp[2] - kh[2] * tmp[1], kh[2] * tmp[0] - kh[0] * tmp[2], kh[0] * tmp[1] - kh[1] * tmp[0]};
    double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    u[0] /= un; u[1] /= un; u[2] /= un;
    double v[3] = {kh[1] * u[2] - kh[2] * u[1], kh[2] * u[0] - kh[0] * u[2], kh[0] * u[1] - kh[1] * u[0]};
    double vn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= vn; v[1] /= vn; v[2] /= vn;
    for (int i = 0; i < 3; i++)
        if (u[i] < 0) { u[0] = -u[0]; u[1] = -u[1]; u[2] = -u[2]; break; }
    for (int i = 0; i < 3; i++)
        if (v[i] < 0) { v[0] = -v[0]; v[1] = -v[1]; v[2] = -v[2]; break; }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) e[i][j] = u[i] * u[j] - v[i] * v[j] + u[i] * v[j] + v[i] * u[j];
}

/* set_mode_GW, initialize.cpp:273-326, into the six symmetric components */
static void set_mode_gw(orc_state *s, const double kv[3], double k2, long idx, int isReal) {
    const double a = s->a, H0 = s->hubble_init;
    double e[3][3];
    tt_tensor(kv, e);
    double norm = s->MPl * s->omegaStar / pw2(s->fStar) * pow(s->N / s->dx, 1.5);
    double kc = s->p.kcutoff;
    double k2cutoff = (kc < 2. * PI_D * (double)s->N / s->L ? pw2(kc) : 0.);
    if (k2cutoff > 0. && k2 > k2cutoff) {
        for (int c = 0; c < 6; c++) {
            double *uk = s->u_k + 2 * s->modes * c, *pu = s->pi_u_k + 2 * s->modes * c;
            uk[2 * idx] = uk[2 * idx + 1] = pu[2 * idx] = pu[2 * idx + 1] = 0.;
        }
        return;
    }
    double k = sqrt(k2);
    double rms = norm / sqrt(k);
    double al = rms / sqrt(2.) * sqrt(log(1. / rand_uniform(s))) / a;
    double ar = rms / sqrt(2.) * sqrt(log(1. / rand_uniform(s))) / a;
    double ph = 2. * PI_D * rand_uniform(s);
    double rel = al * cos(ph), iml = al * sin(ph);
    ph = 2. * PI_D * rand_uniform(s);
    double rer = ar * cos(ph), imr = ar * sin(ph);
    for (int c = 0; c < 6; c++) {
        double ec = e[SYM_I[c]][SYM_J[c]];
        double *uk = s->u_k + 2 * s->modes * c, *pu = s->pi_u_k + 2 * s->modes * c;
        uk[2 * idx] = ec * (rel + rer);
        uk[2 * idx + 1] = ec * (iml + imr);
        pu[2 * idx] = pow(a, s->alpha - 3) * (ec * (-k * (iml - imr) - H0 * uk[2 * idx]));
        pu[2 * idx + 1] = pow(a, s->alpha - 3) * (ec * (k * (rel - rer) - H0 * uk[2 * idx + 1]));
        if (isReal) { uk[2 * idx + 1] = 0.; pu[2 * idx + 1] = 0.; }
    }
}

/* initialize_GW, initialize.cpp:341-470 */
static void init_gw(orc_state *s) {
    const int N = s->N, H = s->H;
    const double kIR = s->kIR, dp2 = pw2(kIR);
    for (int k = 0; k <= N / 2; k += N / 2) {
        for (int i = 0; i <= N / 2; i += N / 2)
            for (int j = 1; j < N / 2; j++) {
                double kv[3] = {i * kIR, j * kIR, k * kIR};
                long idx = ((long)i * N + j) * H + k, cj = ((long)i * N + (N - j)) * H + k;
                set_mode_gw(s, kv, dp2 * (pw2(i) + pw2(j) + pw2(k)), idx, 0);
                for (int c = 0; c < 6; c++) { set_conj(s->u_k + 2 * s->modes * c, cj, idx); set_conj(s->pi_u_k + 2 * s->modes * c, cj, idx); }
            }
        for (int j = 0; j <= N / 2; j += N / 2)
            for (int i = 1; i < N / 2; i++) {
                double kv[3] = {i * kIR, j * kIR, k * kIR};
                long idx = ((long)i * N + j) * H + k, cj = ((long)(N - i) * N + j) * H + k;
                set_mode_gw(s, kv, dp2 * (pw2(i) + pw2(j) + pw2(k)), idx, 0);
                for (int c = 0; c < 6; c++) { set_conj(s->u_k + 2 * s->modes * c, cj, idx); set_conj(s->pi_u_k + 2 * s->modes * c, cj, idx); }
            }
        for (int i = 1; i < N / 2; i++) {
            for (int j = 1; j < N / 2; j++) {
                double kv[3] = {i * kIR, j * kIR, k * kIR};
                long idx = ((long)i * N + j) * H + k, cj = ((long)(N - i) * N + (N - j)) * H + k;
                set_mode_gw(s, kv, dp2 * (pw2(i) + pw2(j) + pw2(k)), idx, 0);
                for (int c = 0; c < 6; c++) { set_conj(s->u_k + 2 * s->modes * c, cj, idx); set_conj(s->pi_u_k + 2 * s->modes * c, cj, idx); }
            }
            for (int j = N / 2 + 1; j < N; j++) {
                double kv[3] = {i * kIR, (j - N) * kIR, k * kIR};
                long idx = ((long)i * N + j) * H + k, cj = ((long)(N - i) * N + (N - j)) * H + k;
                set_mode_gw(s, kv, dp2 * (pw2(i) + pw2(j - N) + pw2(k)), idx, 0);
                for (int c = 0; c < 6; c++) { set_conj(s->u_k + 2 * s->modes * c, cj, idx); set_conj(s->pi_u_k + 2 * s->modes * c, cj, idx); }
            }
        }
    }
    for (int k = 1; k < N / 2; k++)
        for (int i = 0; i < N; i++) {
            int px = pcoord(i, N);
            for (int j = 0; j < N; j++) {
                int py = pcoord(j, N);
                double kv[3] = {px * kIR, py * kIR, k * kIR};
                set_mode_gw(s, kv, dp2 * (pw2(px) + pw2(py) + pw2(k)), ((long)i * N + j) * H + k, 0);
            }
        }
    for (int k = 0; k <= N / 2; k += N / 2)
        for (int i = 0; i <= N / 2; i += N / 2)
            for (int j = 0; j <= N / 2; j += N / 2) {
                if (i == 0 && j == 0 && k == 0) {
                    for (int c = 0; c < 6; c++) {
                        s->u_k[2 * s->modes * c] = s->u_k[2 * s->modes * c + 1] = 0.;
                        s->pi_u_k[2 * s->modes * c] = s->pi_u_k[2 * s->modes * c + 1] = 0.;
                    }
                    continue;
                }
                double kv[3] = {i * kIR, j * kIR, k * kIR};
                set_mode_gw(s, kv, dp2 * (pw2(i) + pw2(j) + pw2(k)), ((long)i * N + j) * H + k, 1);
            }
    if (s->p.seed >= 0)
        for (int c = 0; c < 6; c++) {
            c2r_norm(s, s->u_k + 2 * s->modes * c, s->u + s->sites * c);
            c2r_norm(s, s->pi_u_k + 2 * s->modes * c, s->pi_u + s->sites * c);
        }
}

/* initialize, initialize.cpp:562-810 (fresh run, no checkpoint) */
double orc_init_ic(orc_state *s) {
    const int N = s->N, H = s->H, nf = s->nf;
    const double dp2 = pw2(s->kIR);
    double initial_f[2] = {0, 0}, initial_fd[2] = {0, 0}, mass_sq[2] = {0, 0};
    s->t = 0.;
    s->rng_i = 0;
    s->rng_next = s->p.seed;
    for (int fld = 0; fld < nf; fld++) {
        initial_f[fld] = s->p.initfield[fld] / s->fStar;
        initial_fd[fld] = s->p.initderivs[fld] / s->fStar / s->omegaStar;
    }
    effective_mass(s, mass_sq, initial_f);
    double add_printed = 0.;
    s->a = s->p.a0;
    if (s->p.expansion > 0) {
        double fdsq = 0., pot = 0.;
        for (int fld = 0; fld < nf; fld++) fdsq += pw2(initial_fd[fld]);
        for (int term = 0; term < s->nterms; term++) pot += potential_term(s, term, initial_f);
        double h = fdsq / 2.;
        h += pot;
        h *= pw2(s->fStar / s->MPl) / 3.;
        s->hubble_init = sqrt(h);
        s->a = s->p.a0;
        s->ad = s->hubble_init * s->a;
        s->add = pw2(s->fStar / s->MPl) / 3. * ((s->alpha - 2) * fdsq + (s->alpha + 1) * pot) * s->a;
        add_printed = s->add;
    }
    for (int fld = 0; fld < nf; fld++) {
        double *fk = s->f_k + 2 * s->modes * fld, *pk = s->pi_k + 2 * s->modes * fld;
        const double m2 = mass_sq[fld];
#define SETM(ii, jj, kk, p2v, conjidx, real)                                                 \
    do {                                                                                     \
        long idx_ = ((long)(ii) * N + (jj)) * H + (kk);                                      \
        set_mode(s, (p2v), m2, fk + 2 * idx_, pk + 2 * idx_, (real));                        \
        if ((conjidx) >= 0) { set_conj(fk, (conjidx), idx_); set_conj(pk, (conjidx), idx_); } \
    } while (0)
        for (int k = 0; k <= N / 2; k += N / 2) {
            for (int i = 0; i <= N / 2; i += N / 2)
                for (int j = 1; j < N / 2; j++)
                    SETM(i, j, k, dp2 * (pw2(i) + pw2(j) + pw2(k)), ((long)i * N + (N - j)) * H + k, 0);
            for (int j = 0; j <= N / 2; j += N / 2)
                for (int i = 1; i < N / 2; i++)
                    SETM(i, j, k, dp2 * (pw2(i) + pw2(j) + pw2(k)), ((long)(N - i) * N + j) * H + k, 0);
            for (int i = 1; i < N / 2; i++) {
                for (int j = 1; j < N / 2; j++)
                    SETM(i, j, k, dp2 * (pw2(i) + pw2(j) + pw2(k)), ((long)(N - i) * N + (N - j)) * H + k, 0);
                for (int j = N / 2 + 1; j < N; j++)
                    SETM(i, j, k, dp2 * (pw2(i) + pw2(j - N) + pw2(k)), ((long)(N - i) * N + (N - j)) * H + k, 0);
            }
        }
        for (int k = 1; k < N / 2; k++)
            for (int i = 0; i < N; i++) {
                int px = pcoord(i, N);
                for (int j = 0; j < N; j++) {
                    int py = pcoord(j, N);
                    SETM(i, j, k, dp2 * (pw2(px) + pw2(py) + pw2(k)), -1L, 0);
                }
            }
        for (int k = 0; k <= N / 2; k += N / 2)
            for (int i = 0; i <= N / 2; i += N / 2)
                for (int j = 0; j <= N / 2; j += N / 2) SETM(i, j, k, dp2 * (pw2(i) + pw2(j) + pw2(k)), -1L, 1);
#undef SETM
        fk[0] = initial_f[fld] * (double)s->sites;
        fk[1] = 0.;
        pk[0] = pow(s->a, s->alpha - 3) * initial_fd[fld] * (double)s->sites;
        pk[1] = 0.;
        if (s->p.seed >= 0) {
            c2r_norm(s, fk, s->f + s->sites * fld);
            c2r_norm(s, pk, s->pi_f + s->sites * fld);
        }
    }
    s->add = orc_kernel_a(s);
    s->der_valid = 0;
    if (s->gw) init_gw(s);
    return add_printed;
}

double orc_hubble_init(orc_state *s) { return s->hubble_init; }

/* ---------------------------------------------------------------- spectral step */
/* kernel_field_k_nopad, evolution.cpp:1092-1129 */
static void kernel_field_k(orc_state *s) {
    const int N = s->N, H = s->H, nf = s->nf;
    const double norm1 = pow(s->a, 1 + s->alpha), norm2 = pow(s->a, 3 + s->alpha);
    const long n = s->sites;
#pragma omp parallel for schedule(static)
    for (long x = 0; x < n; x++) {
        double v[2] = {s->f[x], nf > 1 ? s->f[n + x] : 0.};
        for (int fld = 0; fld < nf; fld++) s->Vp[n * fld + x] = dvdf(s, fld, v);
    }
    for (int fld = 0; fld < nf; fld++) {
        double *vk = s->Vp_k + 2 * s->modes * fld, *kf = s->kern_k + 2 * s->modes * fld;
        const double *fk = s->f_k + 2 * s->modes * fld;
        fft64_r2c_3d(N, N, N, s->Vp + n * fld, vk);
#pragma omp parallel for schedule(static)
        for (long ij = 0; ij < (long)N * N; ij++) {
            int px = pcoord((int)(ij / N), N), py = pcoord((int)(ij % N), N);
            for (int k = 0; k < H; k++) {
                long m = ij * H + k;
                int k2 = px * px + py * py + k * k;
                kf[2 * m] = -norm1 * pw2(s->kIR) * k2 * fk[2 * m] - norm2 * vk[2 * m];
                kf[2 * m + 1] = -norm1 * pw2(s->kIR) * k2 * fk[2 * m + 1] - norm2 * vk[2 * m + 1];
            }
        }
    }
}

/* evolve_VV_k_nopad, evolution.cpp:1131-1198 */
static void step_spectral(orc_state *s, double dt, int nst) {
    const int nf = s->nf;
    const long m2 = 2 * s->modes;
    double b = s->ad, b_half, a_half, norm;
    for (int p = 0; p < nst; p++) {
        const double w = s->w[p];
        b_half = b + w * dt / 2. * s->add;
        for (int fld = 0; fld < nf; fld++) c2r_norm(s, s->f_k + m2 * fld, s->f + s->sites * fld);
        kernel_field_k(s);
#pragma omp parallel for schedule(static)
        for (long m = 0; m < m2 * nf; m++) s->pi_k_half[m] = s->pi_k[m] + w * dt / 2 * s->kern_k[m];
        a_half = s->a + b_half * w * dt / 2.;
        norm = pow(a_half, s->alpha - 3);
        for (int fld = 0; fld < nf; fld++) {
#pragma omp parallel for schedule(static)
            for (long m = m2 * fld; m < m2 * (fld + 1); m++) s->f_k[m] += w * dt * norm * s->pi_k_half[m];
            c2r_norm(s, s->f_k + m2 * fld, s->f + s->sites * fld);
        }
        s->a = a_half + b_half * w * dt / 2.;
        kernel_field_k(s);
#pragma omp parallel for schedule(static)
        for (long m = 0; m < m2 * nf; m++) s->pi_k[m] = s->pi_k_half[m] + w * dt / 2 * s->kern_k[m];
        s->add = orc_kernel_a(s);
        b = b_half + w * dt / 2. * s->add;
    }
    s->ad = b;
    s->t += dt;
}

/* ---------------------------------------------------------------- real-space step */
/* lapl, evolution.cpp:343-372 */
static void lapl(orc_state *s, const double *in, double *out) {
    const int N = s->N, H = s->H;
    double *fr = s->work_k;
    fft64_r2c_3d(N, N, N, in, fr);
    const double kIR = s->kIR;
#pragma omp parallel for schedule(static)
    for (long ij = 0; ij < (long)N * N; ij++) {
        int px = pcoord((int)(ij / N), N), py = pcoord((int)(ij % N), N);
        for (int k = 0; k < H; k++) {
            long m = ij * H + k;
            double mult = (-pw2(kIR * px) - pw2(kIR * py) - pw2(kIR * k));
            fr[2 * m] *= mult;
            fr[2 * m + 1] *= mult;
        }
    }
    c2r_norm(s, fr, out);
}

/* kernel_field, evolution.cpp:441-461 */
static void kernel_field_real(orc_state *s, int fld, double *kern) {
    const double norm1 = pow(s->a, 1 + s->alpha), norm2 = pow(s->a, 3 + s->alpha);
    lapl(s, s->f + s->sites * fld, s->lapl_buf);
    const long n = s->sites;
#pragma omp parallel for schedule(static)
    for (long x = 0; x < n; x++) {
        double v[2] = {s->f[x], s->nf > 1 ? s->f[n + x] : 0.};
        kern[x] = norm1 * s->lapl_buf[x] - norm2 * dvdf(s, fld, v);
    }
}

/* field_1st_derivative, evolution.cpp:466-578: 1-D spectral derivative along
 * each axis, Nyquist zeroed, /N */
static void field_derivs(orc_state *s) {
    const int N = s->N, H = s->H;
    const long n = s->sites;
    for (int fld = 0; fld < s->nf; fld++) {
        const double *f = s->f + n * fld;
        for (int ax = 0; ax < 3; ax++) {
            double *out = s->fder + n * (3 * fld + ax);
            long stride = ax == 0 ? (long)N * N : (ax == 1 ? N : 1);
#pragma omp parallel for schedule(static)
            for (long l = 0; l < (long)N * N; l++) {
                long base;
                if (ax == 0) base = l;                                     /* (j, k) */
                else if (ax == 1) base = (l / N) * (long)N * N + (l % N); /* (i, k) */
                else base = l * N;                                         /* (i, j) */
                double line[2 * 1024 + 4];
                fft64_r2c_line(f + base, stride, line, 1, N);
                for (int k = 0; k < N / 2; k++) {
                    double temp = line[2 * k];
                    line[2 * k] = -s->kIR * k * line[2 * k + 1];
                    line[2 * k + 1] = s->kIR * k * temp;
                }
                line[2 * (N / 2)] = 0.;
                line[2 * (N / 2) + 1] = 0.;
                fft64_c2r_line(line, 1, out + base, stride, N);
                for (int m = 0; m < N; m++) out[base + m * stride] /= N;
            }
            (void)H;
        }
    }
    s->der_valid = 1;
}

/* kernel_GW, evolution.cpp:581-601 */
static void kernel_gw(orc_state *s, int c, double *kern) {
    lapl(s, s->u + s->sites * c, s->lapl_buf);
    if (!s->der_valid) field_derivs(s);
    const double norm = pow(s->a, 1 + s->alpha);
    const long n = s->sites;
    const int i = SYM_I[c], j = SYM_J[c];
#pragma omp parallel for schedule(static)
    for (long x = 0; x < n; x++) {
        double v = s->lapl_buf[x];
        for (int fld = 0; fld < s->nf; fld++)
            v += 2 * s->fder[n * (3 * fld + i) + x] * s->fder[n * (3 * fld + j) + x];
        kern[x] = v * norm;
    }
}

/* evolve_VV, evolution.cpp:607-694 */
static void step_real(orc_state *s, double dt, int nst) {
    const int nf = s->nf;
    const long n = s->sites;
    double b = s->ad, b_half, a_half, a_of_pi;
    for (int p = 0; p < nst; p++) {
        const double w = s->w[p];
        b_half = b + w * dt / 2. * s->add;
        for (int fld = 0; fld < nf; fld++) {
            kernel_field_real(s, fld, s->kern_r);
#pragma omp parallel for schedule(static)
            for (long x = 0; x < n; x++) s->pi_half[n * fld + x] = s->pi_f[n * fld + x] + w * dt / 2. * s->kern_r[x];
        }
        if (s->gw)
            for (int c = 0; c < 6; c++) {
                kernel_gw(s, c, s->kern_r);
#pragma omp parallel for schedule(static)
                for (long x = 0; x < n; x++) s->pi_u_half[n * c + x] = s->pi_u[n * c + x] + w * dt / 2 * s->kern_r[x];
            }
        a_half = s->a + b_half * w * dt / 2.;
        a_of_pi = pow(a_half, s->alpha - 3);
#pragma omp parallel for schedule(static)
        for (long x = 0; x < n * nf; x++) s->f[x] += w * dt * a_of_pi * s->pi_half[x];
        if (s->gw) {
            s->der_valid = 0;
#pragma omp parallel for schedule(static)
            for (long x = 0; x < n * 6; x++) s->u[x] += w * dt * a_of_pi * s->pi_u_half[x];
        }
        s->a = a_half + b_half * w * dt / 2.;
        for (int fld = 0; fld < nf; fld++) {
            kernel_field_real(s, fld, s->kern_r);
#pragma omp parallel for schedule(static)
            for (long x = 0; x < n; x++) s->pi_f[n * fld + x] = s->pi_half[n * fld + x] + w * dt / 2 * s->kern_r[x];
        }
        if (s->gw)
            for (int c = 0; c < 6; c++) {
                kernel_gw(s, c, s->kern_r);
#pragma omp parallel for schedule(static)
                for (long x = 0; x < n; x++) s->pi_u[n * c + x] = s->pi_u_half[n * c + x] + w * dt / 2 * s->kern_r[x];
            }
        s->add = orc_kernel_a(s);
        b = b_half + w * dt / 2. * s->add;
    }
    s->ad = b;
    s->t += dt;
}

void orc_step(orc_state *s, double dt) {
    if (s->spectral) step_spectral(s, dt, s->s);
    else step_real(s, dt, s->s);
}

void orc_step_stages(orc_state *s, double dt, int nstages) {
    if (nstages > s->s) nstages = s->s;
    if (s->spectral) step_spectral(s, dt, nstages);
    else step_real(s, dt, nstages);
}

int orc_stages(orc_state *s) { return s->s; }

/* ---------------------------------------------------------------- state access */
void orc_get_bg(orc_state *s, double *t, double *a, double *ad, double *add) {
    if (t) *t = s->t;
    if (a) *a = s->a;
    if (ad) *ad = s->ad;
    if (add) *add = s->add;
}

void orc_set_bg(orc_state *s, double t, double a, double ad, double add) {
    s->t = t; s->a = a; s->ad = ad; s->add = add;
}

/* the k-space view: the spectral state itself, or r2c of the real-space state
 * (what spectra() computes, output.cpp:585-618) */
static void refresh_k(orc_state *s) {
    if (s->spectral) return;
    const int N = s->N;
    for (int fld = 0; fld < s->nf; fld++) {
        fft64_r2c_3d(N, N, N, s->f + s->sites * fld, s->f_k + 2 * s->modes * fld);
        fft64_r2c_3d(N, N, N, s->pi_f + s->sites * fld, s->pi_k + 2 * s->modes * fld);
    }
    if (s->gw)
        for (int c = 0; c < 6; c++) {
            fft64_r2c_3d(N, N, N, s->u + s->sites * c, s->u_k + 2 * s->modes * c);
            fft64_r2c_3d(N, N, N, s->pi_u + s->sites * c, s->pi_u_k + 2 * s->modes * c);
        }
}

void orc_get_state_k(orc_state *s, double *f_k, double *pi_k, double *u_k, double *pi_u_k) {
    refresh_k(s);
    size_t fb = sizeof(double) * 2 * s->modes * s->nf;
    if (f_k) memcpy(f_k, s->f_k, fb);
    if (pi_k) memcpy(pi_k, s->pi_k, fb);
    if (s->gw) {
        size_t gb = sizeof(double) * 2 * s->modes * 6;
        if (u_k) memcpy(u_k, s->u_k, gb);
        if (pi_u_k) memcpy(pi_u_k, s->pi_u_k, gb);
    }
}

void orc_set_state_k(orc_state *s, const double *f_k, const double *pi_k, const double *u_k, const double *pi_u_k) {
    size_t fb = sizeof(double) * 2 * s->modes * s->nf;
    memcpy(s->f_k, f_k, fb);
    memcpy(s->pi_k, pi_k, fb);
    for (int fld = 0; fld < s->nf; fld++) {
        c2r_norm(s, s->f_k + 2 * s->modes * fld, s->f + s->sites * fld);
        c2r_norm(s, s->pi_k + 2 * s->modes * fld, s->pi_f + s->sites * fld);
    }
    if (s->gw && u_k && pi_u_k) {
        size_t gb = sizeof(double) * 2 * s->modes * 6;
        memcpy(s->u_k, u_k, gb);
        memcpy(s->pi_u_k, pi_u_k, gb);
        for (int c = 0; c < 6; c++) {
            c2r_norm(s, s->u_k + 2 * s->modes * c, s->u + s->sites * c);
            c2r_norm(s, s->pi_u_k + 2 * s->modes * c, s->pi_u + s->sites * c);
        }
    }
    s->der_valid = 0;
}

void orc_get_fields_real(orc_state *s, double *f, double *pi_f) {
    if (s->spectral)
        for (int fld = 0; fld < s->nf; fld++) {
            c2r_norm(s, s->f_k + 2 * s->modes * fld, s->f + s->sites * fld);
            c2r_norm(s, s->pi_k + 2 * s->modes * fld, s->pi_f + s->sites * fld);
        }
    size_t b = sizeof(double) * s->sites * s->nf;
    if (f) memcpy(f, s->f, b);
    if (pi_f) memcpy(pi_f, s->pi_f, b);
}

void orc_get_gw_real(orc_state *s, double *u, double *pi_u) {
    if (!s->gw) return;
    size_t b = sizeof(double) * s->sites * 6;
    if (u) memcpy(u, s->u, b);
    if (pi_u) memcpy(pi_u, s->pi_u, b);
}

/* ---------------------------------------------------------------- outputs */
int orc_maxnumbins(int N) { return (int)(sqrt(3.0) * (N / 2)) + 2; } /* parameters.h:25 */

static int bin_of(int px, int py, int pz) { return (int)floor(sqrt(pw2(px) + pw2(py) + pw2(pz)) + 0.5); }

/* v = P u with P = delta - khat khat (projection_operator / P_projection,
 * output.cpp:18-53); returns sum_ij |v_ij|^2 - |tr v|^2 / 2 */
static double gw_proj_norm(const double kv[3], const double *comp_re, const double *comp_im) {
    double kn = sqrt(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
    double kh[3] = {kv[0] / kn, kv[1] / kn, kv[2] / kn};
    double P[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) P[i][j] = (i == j ? 1. : 0.) - kh[i] * kh[j];
    double vr[3][3], vi[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double r = 0, im = 0;
            for (int k = 0; k < 3; k++) {
                int c = sym_index(k, j);
                r += P[i][k] * comp_re[c];
                im += P[i][k] * comp_im[c];
            }
            vr[i][j] = r;
            vi[i][j] = im;
        }
#define NRM(i, j) (vr[i][j] * vr[i][j] + vi[i][j] * vi[i][j])
    double tr_r = vr[0][0] + vr[1][1] + vr[2][2], tr_i = vi[0][0] + vi[1][1] + vi[2][2];
    return NRM(0, 0) + NRM(1, 1) + NRM(2, 2) + NRM(0, 1) + NRM(1, 0) + NRM(0, 2) + NRM(2, 0) + NRM(1, 2) + NRM(2, 1) -
           (tr_r * tr_r + tr_i * tr_i) / 2.;
#undef NRM
}

/* GW block of spectra(), output.cpp:780-1062: bin SUMS over the "+" half of the
 * kz = 0, N/2 planes (weight 2), the interior (weight 2) and the seven non-zero
 * corners (weight 1); *hz = |pi_u_k(0)|^2 summed over the nine components */
static void gw_bins(orc_state *s, int *cnt, double *Hs, double *Hd, double *hz) {
    const int N = s->N, H = s->H;
    const double kIR = s->kIR;
#define GWACC(ii, jj, kk, pxv, pyv, wgt)                                                     \
    do {                                                                                     \
        long m_ = ((long)(ii) * N + (jj)) * H + (kk);                                        \
        double kv_[3] = {(pxv) * kIR, (pyv) * kIR, (kk) * kIR};                              \
        double ur_[6], ui_[6], pr_[6], pim_[6];                                              \
        for (int c = 0; c < 6; c++) {                                                        \
            ur_[c] = s->u_k[2 * s->modes * c + 2 * m_];                                      \
            ui_[c] = s->u_k[2 * s->modes * c + 2 * m_ + 1];                                  \
            pr_[c] = s->pi_u_k[2 * s->modes * c + 2 * m_];                                   \
            pim_[c] = s->pi_u_k[2 * s->modes * c + 2 * m_ + 1];                              \
        }                                                                                    \
        int l_ = bin_of((pxv), (pyv), (kk));                                                 \
        cnt[l_] += (wgt);                                                                    \
        Hs[l_] += (wgt) * gw_proj_norm(kv_, ur_, ui_);                                       \
        Hd[l_] += (wgt) * gw_proj_norm(kv_, pr_, pim_);                                      \
    } while (0)
    for (int k = 0; k <= N / 2; k += N / 2) {
        for (int i = 0; i <= N / 2; i += N / 2)
            for (int j = 1; j < N / 2; j++) GWACC(i, j, k, i, j, 2);
        for (int j = 0; j <= N / 2; j += N / 2)
            for (int i = 1; i < N / 2; i++) GWACC(i, j, k, i, j, 2);
        for (int i = 1; i < N / 2; i++) {
            for (int j = 1; j < N / 2; j++) GWACC(i, j, k, i, j, 2);
            for (int j = N / 2 + 1; j < N; j++) GWACC(i, j, k, i, j - N, 2);
        }
    }
    for (int k = 1; k < N / 2; k++)
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++) GWACC(i, j, k, pcoord(i, N), pcoord(j, N), 2);
    for (int k = 0; k <= N / 2; k += N / 2)
        for (int i = 0; i <= N / 2; i += N / 2)
            for (int j = 0; j <= N / 2; j += N / 2) {
                if (i == 0 && j == 0 && k == 0) continue;
                GWACC(i, j, k, i, j, 1);
            }
#undef GWACC
    double z = 0.;
    for (int c = 0; c < 6; c++) {
        double mult = (SYM_I[c] == SYM_J[c]) ? 1. : 2.;
        z += mult * (pw2(s->pi_u_k[2 * s->modes * c]) + pw2(s->pi_u_k[2 * s->modes * c + 1]));
    }
    *hz = z;
}

void orc_spectra(orc_state *s, int *numpoints, double *f2, double *pi2, double *n2, int *gw_numpoints, double *h2,
                 double *hdot2, double *hdot2_zero) {
    const int N = s->N, H = s->H, nb = orc_maxnumbins(N);
    refresh_k(s);
    const double a_of_pi = pow(s->a, s->alpha - 3), hub = s->ad / s->a;
    for (int fld = 0; fld < s->nf; fld++) {
        const double *fk = s->f_k + 2 * s->modes * fld, *pk = s->pi_k + 2 * s->modes * fld;
        int *np = numpoints ? numpoints + (long)nb * fld : NULL;
        double *F = (double *)calloc(nb, sizeof(double)), *P = (double *)calloc(nb, sizeof(double)),
               *Nn = (double *)calloc(nb, sizeof(double));
        int *cnt = (int *)calloc(nb, sizeof(int));
        /* output.cpp:626-669 */
        for (int i = 0; i < N; i++) {
            int px = pcoord(i, N);
            for (int j = 0; j < N; j++) {
                int py = pcoord(j, N);
                for (int k = 0; k < H; k++) {
                    long m = ((long)i * N + j) * H + k;
                    int l = bin_of(px, py, k);
                    double fp2 = pw2(fk[2 * m]) + pw2(fk[2 * m + 1]);
                    double pp2 = pw2(pk[2 * m]) + pw2(pk[2 * m + 1]);
                    double np2 = pw2(a_of_pi * pk[2 * m] + hub * fk[2 * m]) + pw2(a_of_pi * pk[2 * m + 1] + hub * fk[2 * m + 1]);
                    if (k == 0 || k == N / 2) { cnt[l]++; F[l] += fp2; P[l] += pp2; Nn[l] += np2; }
                    else { cnt[l] += 2; F[l] += 2. * fp2; P[l] += 2. * pp2; Nn[l] += 2. * np2; }
                }
            }
        }
        for (int l = 0; l < nb; l++) {
            if (cnt[l] > 0) { F[l] /= cnt[l]; P[l] /= cnt[l]; Nn[l] /= cnt[l]; }
            if (np) np[l] = cnt[l];
            if (f2) f2[(long)nb * fld + l] = F[l];
            if (pi2) pi2[(long)nb * fld + l] = P[l];
            if (n2) n2[(long)nb * fld + l] = Nn[l];
        }
        free(F); free(P); free(Nn); free(cnt);
    }
    if (!s->gw) return;
    double *Hs = (double *)calloc(nb, sizeof(double)), *Hd = (double *)calloc(nb, sizeof(double)), hz = 0.;
    int *cnt = (int *)calloc(nb, sizeof(int));
    gw_bins(s, cnt, Hs, Hd, &hz);
    if (hdot2_zero) *hdot2_zero = hz;
    for (int l = 0; l < nb; l++) {
        double hsum = Hs[l], dsum = Hd[l];
        if (cnt[l] > 0 && l >= 1) { hsum /= cnt[l]; dsum /= cnt[l]; }
        if (gw_numpoints) gw_numpoints[l] = cnt[l];
        if (h2) h2[l] = hsum;
        if (hdot2) hdot2[l] = dsum;
    }
    free(Hs); free(Hd); free(cnt);
}

void orc_energies(orc_state *s, double *K, double *G, double *V, double *total, double *fviol, double *rho_gw) {
    double tot = 0.;
    if (s->spectral) {
        /* energy_density (output.cpp:57-115) after its c2r; K and G use the R_Q2C
         * array of the last kernel_a_k_nopad call */
        for (int fld = 0; fld < s->nf; fld++)
            c2r_norm(s, s->f_k + 2 * s->modes * fld, s->f + s->sites * fld);
    }
    for (int fld = 0; fld < s->nf; fld++) {
        double k, g;
        if (s->spectral) kg_k(s, fld, &k, &g);
        else kg_real(s, fld, &k, &g);
        if (K) K[fld] = k;
        if (G) G[fld] = g;
        tot += k;
        tot += g;
    }
    for (int term = 0; term < s->nterms; term++) {
        double v = pot_avg(s, term);
        if (V) V[term] = v;
        tot += v;
    }
    if (total) *total = tot;
    /* energy(), output.cpp:1178-1185 */
    double LHS = pw2(s->ad);
    double RHS = pw2(s->fStar / s->MPl) * pow(s->a, 2 * (s->alpha + 1)) * tot / 3.;
    if (fviol) *fviol = fabs(LHS - RHS) / fabs(LHS + RHS);
    if (rho_gw) {
        *rho_gw = 0.;
        if (s->gw) {
            const int nb = orc_maxnumbins(s->N);
            int *cnt = (int *)calloc(nb, sizeof(int));
            double *hs = (double *)calloc(nb, sizeof(double)), *hd = (double *)calloc(nb, sizeof(double)), hz = 0;
            refresh_k(s);
            gw_bins(s, cnt, hs, hd, &hz);
            /* output.cpp:1030-1060: rho_GW sums the un-normalised bins */
            double r = hz;
            for (int l = 1; l < nb; l++) r += hd[l];
            r *= pw2(s->omegaStar) * pow(s->fStar, 4) / pw2(s->MPl) / 4. / pw2((double)s->sites) / pow(s->a, 6);
            r /= pw2(s->fStar * s->omegaStar);
            *rho_gw = r;
            free(cnt);
            free(hs);
            free(hd);
        }
    }
}

void orc_means(orc_state *s, double *out) {
    if (s->spectral)
        for (int fld = 0; fld < s->nf; fld++) {
            c2r_norm(s, s->f_k + 2 * s->modes * fld, s->f + s->sites * fld);
            c2r_norm(s, s->pi_k + 2 * s->modes * fld, s->pi_f + s->sites * fld);
        }
    const double a_of_pi = pow(s->a, s->alpha - 3);
    const long n = s->sites;
    for (int fld = 0; fld < s->nf; fld++) {
        double fa = 0, f2 = 0, pa = 0, p2 = 0;
        const double *f = s->f + n * fld, *pf = s->pi_f + n * fld;
#pragma omp parallel for schedule(static) reduction(+ : fa, f2, pa, p2)
        for (long x = 0; x < n; x++) {
            fa += f[x];
            f2 += pw2(f[x]);
            pa += pf[x];
            p2 += pw2(pf[x]);
        }
        fa /= n; f2 /= n; pa /= n; p2 /= n;
        double var_f = (f2 - pw2(fa) > 0 ? sqrt(f2 - pw2(fa)) : 0);
        double var_fd = (p2 - pw2(pa) > 0 ? a_of_pi * sqrt(p2 - pw2(pa)) : 0);
        double *o = out + 6 * fld;
        o[0] = fa;
        o[1] = a_of_pi * pa;
        o[2] = f2;
        o[3] = pw2(a_of_pi) * p2;
        o[4] = var_f;
        o[5] = var_fd;
    }
}
