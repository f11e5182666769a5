// psc_analytic.cu — the analytic pre-lattice phase (ANALYTIC_EVOLUTION).
//
// Before the lattice exists the reference evolves the homogeneous background and, for
// every distinct |k|^2 of the lattice, two linear mode functions per field (a "left" and
// a "right" moving solution of the Bunch-Davies vacuum) coupled through V''(phi_bg):
//   k_square_initialize()               initialize.cpp:1124-1138  the sorted distinct k^2
//   initialize_analytic_perturbation()  initialize.cpp:815-958    background, H, modes
//   evolve_VV_analytic_perturbation(dt) evolution.cpp:167-336     Yoshida stages
//   initialize_lattice()                initialize.cpp:961-1097   lattice modes from them
// The background is a handful of FP64 numbers and runs on the host with the reference's
// own arithmetic; it also yields every stage's coefficients (V''(phi_bg), a powers, the
// kick and drift weights). All distinct k^2 (up to ~5e4 at 256^3, each with 2 solutions
// x nflds fields) then advance on the device, one launch per step for all stages.
// initialize_lattice() draws 4 random numbers per visited mode in its own traversal
// order on the host (the stream of initialize.cpp:13-28) and uploads the lattice.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "psc_handle.h"
#include "psc_model.h"

namespace psc {
namespace {

constexpr double kPi = 3.14159265358979323846;   // 2 asin(1), pspectcosmo.h:27
inline double pw2(double x) { return x * x; }

// model.h (shipped phi^2) and the two-field phi^2 chi^2 model, host side
double potential_term(const psc_params &p, int term, const double *v) {
    if (p.model == PSC_MODEL_PHI2 || term == 0) return 0.5 * pw2(v[0]);
    return 0.5 * p.gsq * pw2(v[0]) * pw2(v[1]);
}
double dvdf(const psc_params &p, int fld, const double *v) {
    if (p.model == PSC_MODEL_PHI2) return v[0];
    return fld == 0 ? v[0] + p.gsq * v[0] * pw2(v[1]) : p.gsq * pw2(v[0]) * v[1];
}
double d2vdf2(const psc_params &p, int term, const double *v) {
    if (p.model == PSC_MODEL_PHI2) return 1.;
    if (term == 0) return 1. + p.gsq * pw2(v[1]);
    if (term == 1) return 2. * p.gsq * v[0] * v[1];
    return p.gsq * pw2(v[0]);
}
void effective_mass(const psc_params &p, double *m2, const double *v) {
    if (p.model == PSC_MODEL_PHI2) {
        m2[0] = 1.;
        return;
    }
    m2[0] = 1. + p.gsq * pw2(v[1]);
    m2[1] = p.gsq * pw2(v[0]);
}

// rand_uniform (initialize.cpp:13-28): Park-Miller with Schrage's factorisation, the
// first call discarding 99 values
class ParkMiller {
  public:
    explicit ParkMiller(int seed) : seed_(seed), next_(seed) {}
    double operator()() {
        if (seed_ < 1) return 0.33;
        if (!(next_ > 0)) next_ = 1;
        if (!warmed_) {
            warmed_ = true;
            for (int i = 1; i < 100; ++i) advance();
        }
        advance();
        return (double)next_ / (double)2147483647;
    }

  private:
    void advance() {
        next_ = 16807 * (next_ % 127773) - 2836 * (next_ / 127773);
        if (next_ < 0) next_ += 2147483647;
    }
    int seed_, next_;
    bool warmed_ = false;
};

// coefficients of one Yoshida stage for the modes: first kick (V'' at the background
// before the drift, a powers at the old a), drift, second kick (after)
struct StageCoef {
    double d2a[3], n1a, n2a;
    double hdt, wdn3;
    double d2b[3], n1b, n2b;
};
struct StepCoef {
    StageCoef c[kMaxStages];
    int s, nf;
    double kIR2;
};

// one kick of mode field fl (evolution.cpp:222-244, 299-319)
__device__ __forceinline__ double2 kick(const double2 *f, double2 base, const double *d2, double n1, double n2,
                                        double hdt, double ksq, int fl, int nf) {
    double2 x = make_double2(0., 0.);
    for (int f2 = 0; f2 < nf; ++f2) {
        x.x = __dadd_rn(x.x, __dmul_rn(d2[fl + f2], f[f2].x));
        x.y = __dadd_rn(x.y, __dmul_rn(d2[fl + f2], f[f2].y));
    }
    x.x = __dmul_rn(x.x, -n2);
    x.y = __dmul_rn(x.y, -n2);
    const double nk = __dmul_rn(n1, ksq);
    x.x = __dadd_rn(x.x, -__dmul_rn(nk, f[fl].x));
    x.y = __dadd_rn(x.y, -__dmul_rn(nk, f[fl].y));
    x.x = __dmul_rn(x.x, hdt);
    x.y = __dmul_rn(x.y, hdt);
    x.x = __dadd_rn(x.x, base.x);
    x.y = __dadd_rn(x.y, base.y);
    return x;
}

// modes [4][nf][na] (f_left, pi_left, f_right, pi_right), complex FP64; index 0 (k^2 = 0)
// is the background and is not touched here
__global__ void __launch_bounds__(256) k_analytic_step(double2 *__restrict__ modes, const int *__restrict__ k2,
                                                       int na, const __grid_constant__ StepCoef sc) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (k >= na) return;
    const int nf = sc.nf;
    const double ksq = __dmul_rn((double)k2[k], sc.kIR2);
    for (int sol = 0; sol < 2; ++sol) {
        double2 *fk = modes + (size_t)(2 * sol) * nf * na;
        double2 *pk = modes + (size_t)(2 * sol + 1) * nf * na;
        double2 f[kMaxFields], p[kMaxFields], ph[kMaxFields];
        for (int fl = 0; fl < nf; ++fl) {
            f[fl] = fk[(size_t)fl * na + k];
            p[fl] = pk[(size_t)fl * na + k];
        }
        // every product and sum rounded on its own (__dmul_rn / __dadd_rn: no fused
        // multiply-add), in the reference's order of operations
        for (int st = 0; st < sc.s; ++st) {
            const StageCoef &c = sc.c[st];
            // pi_half = ((sum V''(fl+f2) f_f2) (-n2) - (n1 k^2) f) (w dt / 2) + pi
            for (int fl = 0; fl < nf; ++fl)
                ph[fl] = kick(f, p[fl], c.d2a, c.n1a, c.n2a, c.hdt, ksq, fl, nf);
            for (int fl = 0; fl < nf; ++fl) {
                f[fl].x = __dadd_rn(f[fl].x, __dmul_rn(c.wdn3, ph[fl].x));
                f[fl].y = __dadd_rn(f[fl].y, __dmul_rn(c.wdn3, ph[fl].y));
            }
            for (int fl = 0; fl < nf; ++fl) p[fl] = kick(f, ph[fl], c.d2b, c.n1b, c.n2b, c.hdt, ksq, fl, nf);
        }
        for (int fl = 0; fl < nf; ++fl) {
            fk[(size_t)fl * na + k] = f[fl];
            pk[(size_t)fl * na + k] = p[fl];
        }
    }
}

struct Analytic {
    int nf = 1, na = 0;
    std::vector<int> k2;
    double t = 0, a = 1, ad = 0, add = 0, hubble = 0;
    double f0[kMaxFields] = {0, 0}, p0[kMaxFields] = {0, 0};   // fk_left[f][0].real(), pi_k_left[f][0].real()
    double p0h[kMaxFields] = {0, 0};   // pi_k_left[f][0].imag(): the reference parks the half-step pi there
    double2 *modes = nullptr;
    int *dk2 = nullptr;
};

void free_analytic(void *x) {
    Analytic *an = static_cast<Analytic *>(x);
    if (!an) return;
    if (an->modes) cudaFree(an->modes);
    if (an->dk2) cudaFree(an->dk2);
    delete an;
}

// kernel_a_only_backgroud (evolution.cpp:140-156): a'' from the homogeneous fields
double kernel_a_only(const psc_params &p, double a, const double *f, const double *pi) {
    const int al = p.alpha, nt = p.model == PSC_MODEL_PHI2 ? 1 : 2;
    const double fStar = p.fStar > 0 ? p.fStar : p.MPl;
    double K = 0, G = 0, V = 0;
    for (int fld = 0; fld < p.nflds; fld++) K += pw2(pi[fld]);
    K /= 2. * std::pow(a, 6);
    for (int term = 0; term < nt; term++) V += potential_term(p, term, f);
    return std::pow(a, 1 + 2 * al) / 3. * pw2(fStar / p.MPl) * ((al - 2) * K + al * G + (al + 1) * V);
}

Analytic *get(psc_handle *h) { return h->ana ? static_cast<Analytic *>(h->ana) : nullptr; }

}  // namespace

namespace hapi {

#define CU(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return fail(e_ == cudaErrorMemoryAllocation ? PSC_ERR_NOMEM : PSC_ERR_CUDA,                  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                             \
    } while (0)

// k_square_initialize + initialize_analytic_perturbation
int analytic_begin(psc_handle *h) {
    if (h->R != 1) return fail(PSC_ERR_CONFIG, "the analytic phase runs on single-lattice handles");
    const psc_params &p = h->p0();
    if (p.expansion != 2) return fail(PSC_ERR_CONFIG, "the analytic phase needs expansion = 2");
    // the linear mode equations use d2Vdf2(fld + fld2) (evolution.cpp:229), whose index names a
    // field pair uniquely for the built-in models only
    if (psc::model_is_user(p.model))
        return fail(PSC_ERR_CONFIG, "the analytic phase runs the built-in models (PSC_MODEL_PHI2, PSC_MODEL_PHI2CHI2)");
    if (h->ana && h->ana_free) h->ana_free(h->ana);
    Analytic *an = new Analytic();
    h->ana = an;
    h->ana_free = free_analytic;
    const int N = p.N, nf = p.nflds, H = N / 2 + 1;
    // the distinct i^2 + j^2 + k^2 (i, j, k <= N/2) and every l^2 with l < maxnumbins
    std::set<int> ks;
    for (int i = 0; i < H; ++i)
        for (int j = 0; j < H; ++j)
            for (int k = 0; k < H; ++k) ks.insert(i * i + j * j + k * k);
    for (int l = 0; l < psc_maxnumbins(N); ++l) ks.insert(l * l);
    an->k2.assign(ks.begin(), ks.end());
    an->na = (int)an->k2.size();
    an->nf = nf;
    const int na = an->na;
    const double fStar = p.fStar > 0 ? p.fStar : p.MPl, omegaStar = p.m_in_MPl * fStar;
    const double norm = omegaStar / fStar;
    const int al = p.alpha;
    an->t = 0.0;   // t = t0
    an->a = p.a0;
    double f0[kMaxFields] = {0, 0}, pi0[kMaxFields] = {0, 0};
    for (int fld = 0; fld < nf; fld++) {
        f0[fld] = p.initfield[fld] / fStar;
        pi0[fld] = std::pow(an->a, 3) * p.initderivs[fld] / fStar / omegaStar;
    }
    const int nt = p.model == PSC_MODEL_PHI2 ? 1 : 2;
    double fdsq = 0., pot = 0.;
    for (int fld = 0; fld < nf; fld++) fdsq += pw2(pi0[fld]);
    for (int term = 0; term < nt; term++) pot += potential_term(p, term, f0);
    fdsq /= 2. * std::pow(an->a, 6);
    double hub = fdsq;
    hub += pot;
    hub *= std::pow(an->a, 2 * al) / 3. * pw2(fStar / p.MPl);
    hub = std::sqrt(hub);
    if (!(hub >= 0.)) return fail(PSC_ERR_NONFINITE, "initial Hubble rate is not a real number");
    an->hubble = hub;
    an->ad = hub * an->a;
    an->add = kernel_a_only(p, an->a, f0, pi0);
    double m2[kMaxFields];
    effective_mass(p, m2, f0);
    // Bunch-Davies modes of every k^2 > 0 (initialize.cpp:920-936)
    std::vector<double2> host((size_t)4 * nf * na);
    auto at = [&](int which, int fld, int k) -> double2 & { return host[((size_t)which * nf + fld) * na + k]; };
    const double t0 = 0.0, a = an->a;
    for (int k = 1; k < na; k++) {
        const double p2 = an->k2[k] * pw2(p.kIR);
        for (int fld = 0; fld < nf; fld++) {
            const double om = std::sqrt(p2 + pw2(a) * m2[fld]);
            const double re = std::cos(om * t0) / std::sqrt(2 * om) / a;
            const double im = std::sin(om * t0) / std::sqrt(2 * om) / a;
            const double c = std::pow(a, 3 - al) * norm, pa = std::pow(a, al - 1);
            at(0, fld, k) = make_double2(norm * re, norm * im);
            at(1, fld, k) = make_double2(c * (-im * om * pa - hub * re), c * (re * om * pa - hub * im));
            at(2, fld, k) = make_double2(norm * re, norm * im);
            at(3, fld, k) = make_double2(c * (im * om * pa - hub * re), c * (-re * om * pa - hub * im));
        }
    }
    for (int fld = 0; fld < nf; fld++) {
        an->f0[fld] = f0[fld];
        an->p0[fld] = pi0[fld];
        at(0, fld, 0) = make_double2(f0[fld], 0.);
        at(1, fld, 0) = make_double2(pi0[fld], 0.);
        at(2, fld, 0) = make_double2(f0[fld], 0.);
        at(3, fld, 0) = make_double2(pi0[fld], 0.);
    }
    CU(cudaMalloc(&an->modes, host.size() * sizeof(double2)));
    CU(cudaMalloc(&an->dk2, (size_t)na * sizeof(int)));
    CU(cudaMemcpyAsync(an->modes, host.data(), host.size() * sizeof(double2), cudaMemcpyHostToDevice, h->st));
    CU(cudaMemcpyAsync(an->dk2, an->k2.data(), (size_t)na * sizeof(int), cudaMemcpyHostToDevice, h->st));
    CU(cudaStreamSynchronize(h->st));
    return PSC_OK;
}

// evolve_VV_analytic_perturbation(dt): the background stages on the host (their
// coefficients for the modes as a by-product), then all modes on the device
int analytic_step(psc_handle *h, double dt) {
    Analytic *an = get(h);
    if (!an) return fail(PSC_ERR_STATE, "call psc_analytic_begin first");
    if (!(dt > 0) || !std::isfinite(dt)) return fail(PSC_ERR_ARG, "need dt > 0");
    const psc_params &p = h->p0();
    const int nf = an->nf, al = p.alpha, s = h->s;
    const double *w = h->w;
    StepCoef sc;
    std::memset(&sc, 0, sizeof sc);
    sc.s = s;
    sc.nf = nf;
    sc.kIR2 = pw2(p.kIR);
    double b = an->ad;
    double a = an->a, add = an->add;
    double fbg[kMaxFields], pih[kMaxFields], kf[kMaxFields];
    for (int pst = 0; pst < s; pst++) {
        StageCoef &c = sc.c[pst];
        const double b_half = b + w[pst] * dt / 2. * add;
        for (int fld = 0; fld < nf; fld++) fbg[fld] = an->f0[fld];
        // kernel_field_background: -a^(3+alpha) dV/dphi of the background
        double n2 = std::pow(a, 3 + al);
        for (int fld = 0; fld < nf; fld++) kf[fld] = -n2 * dvdf(p, fld, fbg);
        for (int fld = 0; fld < nf; fld++) pih[fld] = an->p0[fld] + w[pst] * dt / 2 * kf[fld];
        c.n1a = std::pow(a, 1 + al);
        c.n2a = std::pow(a, 3 + al);
        for (int term = 0; term < 2 * nf - 1; term++) c.d2a[term] = d2vdf2(p, term, fbg);
        c.hdt = w[pst] * dt / 2.;
        const double a_half = a + b_half * w[pst] * dt / 2.;
        const double n3 = std::pow(a_half, al - 3);
        for (int fld = 0; fld < nf; fld++) {
            an->f0[fld] = an->f0[fld] + w[pst] * dt * n3 * pih[fld];
            fbg[fld] = an->f0[fld];
        }
        c.wdn3 = w[pst] * dt * n3;
        a = a_half + b_half * w[pst] * dt / 2.;
        n2 = std::pow(a, 3 + al);
        for (int fld = 0; fld < nf; fld++) kf[fld] = -n2 * dvdf(p, fld, fbg);
        for (int fld = 0; fld < nf; fld++) {
            an->p0h[fld] = pih[fld];
            an->p0[fld] = pih[fld] + w[pst] * dt / 2 * kf[fld];
        }
        c.n1b = std::pow(a, 1 + al);
        c.n2b = std::pow(a, 3 + al);
        for (int term = 0; term < 2 * nf - 1; term++) c.d2b[term] = d2vdf2(p, term, fbg);
        add = kernel_a_only(p, a, fbg, an->p0);
        b = b_half + w[pst] * dt / 2. * add;
    }
    an->ad = b;
    an->a = a;
    an->add = add;
    an->t += dt;
    if (!std::isfinite(an->a) || !std::isfinite(an->ad) || !std::isfinite(an->add))
        return fail(PSC_ERR_NONFINITE, "non-finite background in the analytic phase");
    if (an->na > 1) {
        const int blocks = (an->na - 1 + 255) / 256;
        k_analytic_step<<<blocks, 256, 0, h->st>>>(an->modes, an->dk2, an->na, sc);
        CU(cudaGetLastError());
    }
    return PSC_OK;
}

int analytic_background(psc_handle *h, double *t, double *a, double *ad, double *add, double *f_bg, double *pi_bg) {
    Analytic *an = get(h);
    if (!an) return fail(PSC_ERR_STATE, "call psc_analytic_begin first");
    if (t) *t = an->t;
    if (a) *a = an->a;
    if (ad) *ad = an->ad;
    if (add) *add = an->add;
    for (int fld = 0; fld < an->nf; fld++) {
        if (f_bg) f_bg[fld] = an->f0[fld];
        if (pi_bg) pi_bg[fld] = an->p0[fld];
    }
    return PSC_OK;
}

int analytic_modes(psc_handle *h, int *nk, int32_t *k2, double *modes) {
    Analytic *an = get(h);
    if (!an) return fail(PSC_ERR_STATE, "call psc_analytic_begin first");
    if (nk) *nk = an->na;
    if (k2) std::copy(an->k2.begin(), an->k2.end(), k2);
    if (modes) {
        CU(cudaMemcpyAsync(modes, an->modes, (size_t)4 * an->nf * an->na * sizeof(double2), cudaMemcpyDeviceToHost,
                           h->st));
        CU(cudaStreamSynchronize(h->st));
        // the background entries live on the host during the phase
        for (int fld = 0; fld < an->nf; fld++)
            for (int which = 0; which < 4; which++) {
                double *e = modes + 2 * (((size_t)which * an->nf + fld) * an->na);
                e[0] = (which % 2 == 0) ? an->f0[fld] : an->p0[fld];
                e[1] = (which % 2 == 0) ? 0.0 : an->p0h[fld];
            }
    }
    return PSC_OK;
}

// initialize_lattice (initialize.cpp:961-1097): every stored lattice mode from the mode
// functions of its k^2, with a random phase and a Rayleigh amplitude for each of the two
// solutions (4 draws per mode, in the reference's traversal order), then a, a', a'' and t
// of the phase
int analytic_to_lattice(psc_handle *h) {
    Analytic *an = get(h);
    if (!an) return fail(PSC_ERR_STATE, "call psc_analytic_begin first");
    const psc_params &p = h->p0();
    const Geo &g = h->cfg.g;
    const int N = g.N, H = g.H, nf = an->nf, na = an->na;
    std::vector<double2> m((size_t)4 * nf * na);
    CU(cudaMemcpyAsync(m.data(), an->modes, m.size() * sizeof(double2), cudaMemcpyDeviceToHost, h->st));
    CU(cudaStreamSynchronize(h->st));
    auto md = [&](int which, int fld, int k) { return m[((size_t)which * nf + fld) * na + k]; };
    const double n3 = (double)N * N * N, L = 2 * kPi / p.kIR, l15 = std::pow(L, 1.5);
    ParkMiller rng(p.seed);
    std::vector<double> fk((size_t)2 * g.modes * nf, 0.0), pk((size_t)2 * g.modes * nf, 0.0);
    auto pos = [&](int k2) {
        return (int)(std::lower_bound(an->k2.begin(), an->k2.end(), k2) - an->k2.begin());
    };
    for (int fld = 0; fld < nf; fld++) {
        double *F = fk.data() + (size_t)2 * g.modes * fld, *P = pk.data() + (size_t)2 * g.modes * fld;
        auto idx = [&](int i, int j, int k) { return ((long long)i * N + j) * H + k; };
        auto set = [&](int k2, long long at, bool isReal) {
            const int q = pos(k2);
            const double2 fl = md(0, fld, q), pl = md(1, fld, q), fr = md(2, fld, q), pr = md(3, fld, q);
            double ph = 2. * kPi * rng();
            const double al = std::sqrt(std::log(1. / rng()));
            const double cl = std::cos(ph), sl = std::sin(ph);
            const double ref = (fl.x * cl - fl.y * sl) / std::sqrt(2) * al, imf = (fl.y * cl + fl.x * sl) / std::sqrt(2) * al;
            const double rep = (pl.x * cl - pl.y * sl) / std::sqrt(2) * al, imp = (pl.y * cl + pl.x * sl) / std::sqrt(2) * al;
            ph = 2. * kPi * rng();
            const double ar = std::sqrt(std::log(1. / rng()));
            const double cr = std::cos(ph), sr = std::sin(ph);
            const double rfr = (fr.x * cr - fr.y * sr) / std::sqrt(2) * ar, ifr = (fr.y * cr + fr.x * sr) / std::sqrt(2) * ar;
            const double rpr = (pr.x * cr - pr.y * sr) / std::sqrt(2) * ar, ipr = (pr.y * cr + pr.x * sr) / std::sqrt(2) * ar;
            F[2 * at] = (ref + rfr) * n3 / l15;
            F[2 * at + 1] = (imf + ifr) * n3 / l15;
            P[2 * at] = (rep + rpr) * n3 / l15;
            P[2 * at + 1] = (imp + ipr) * n3 / l15;
            if (isReal) {
                F[2 * at + 1] = 0.;
                P[2 * at + 1] = 0.;
            }
        };
        auto conj = [&](long long to, long long from) {
            F[2 * to] = F[2 * from];
            F[2 * to + 1] = -F[2 * from + 1];
            P[2 * to] = P[2 * from];
            P[2 * to + 1] = -P[2 * from + 1];
        };
        for (int k = 0; k <= N / 2; k += N / 2) {   // the k = 0, N/2 planes: half set, half conjugate
            for (int i = 0; i <= N / 2; i += N / 2)
                for (int j = 1; j < N / 2; j++) {
                    set(i * i + j * j + k * k, idx(i, j, k), false);
                    conj(idx(i, N - j, k), idx(i, j, k));
                }
            for (int j = 0; j <= N / 2; j += N / 2)
                for (int i = 1; i < N / 2; i++) {
                    set(i * i + j * j + k * k, idx(i, j, k), false);
                    conj(idx(N - i, j, k), idx(i, j, k));
                }
            for (int i = 1; i < N / 2; i++) {
                for (int j = 1; j < N / 2; j++) {
                    set(i * i + j * j + k * k, idx(i, j, k), false);
                    conj(idx(N - i, N - j, k), idx(i, j, k));
                }
                for (int j = N / 2 + 1; j < N; j++) {
                    set(i * i + (j - N) * (j - N) + k * k, idx(i, j, k), false);
                    conj(idx(N - i, N - j, k), idx(i, j, k));
                }
            }
        }
        for (int k = 1; k < N / 2; k++)   // every other plane, no conjugates
            for (int i = 0; i < N; i++) {
                const int px = i <= N / 2 ? i : i - N;
                for (int j = 0; j < N; j++) {
                    const int py = j <= N / 2 ? j : j - N;
                    set(px * px + py * py + k * k, idx(i, j, k), false);
                }
            }
        for (int k = 0; k <= N / 2; k += N / 2)   // the 8 real "corners"
            for (int i = 0; i <= N / 2; i += N / 2)
                for (int j = 0; j <= N / 2; j += N / 2) set(i * i + j * j + k * k, idx(i, j, k), true);
        F[0] = an->f0[fld] * n3;
        F[1] = 0.;
        P[0] = an->p0[fld] * n3;
        P[1] = 0.;
    }
    std::vector<double> zeros;
    if (g.gw) zeros.assign((size_t)2 * g.modes * 6, 0.0);   // the analytic path sets no GW modes
    int rc = set_state(h, 0, fk.data(), pk.data(), an->a, an->ad, an->add, g.gw ? zeros.data() : nullptr,
                       g.gw ? zeros.data() : nullptr);
    if (rc) return rc;
    DevBG bg;
    if ((rc = read_bg(h, 0, &bg))) return rc;
    bg.t = an->t;
    return write_bg(h, 0, bg);
}

}  // namespace hapi
}  // namespace psc

using namespace psc::hapi;

extern "C" {

int psc_analytic_begin(psc_handle *h) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return analytic_begin(h);
}

int psc_analytic_step(psc_handle *h, double dt) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return analytic_step(h, dt);
}

int psc_analytic_background(psc_handle *h, double *t, double *a, double *ad, double *add, double *f_bg,
                            double *pi_bg) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return analytic_background(h, t, a, ad, add, f_bg, pi_bg);
}

int psc_analytic_modes(psc_handle *h, int *nk, int32_t *k2, double *modes) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return analytic_modes(h, nk, k2, modes);
}

int psc_analytic_to_lattice(psc_handle *h) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return analytic_to_lattice(h);
}

}  // extern "C"
