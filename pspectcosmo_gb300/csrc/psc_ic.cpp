// psc_ic.cpp — initial conditions with the reference's random stream.
//
// The draws must come in the reference's order to reproduce its lattices, and
// that order is one sequential Park-Miller stream, so this runs on the host in
// FP64 (O(modes), once per run) and the result is uploaded.
//   rand_uniform          initialize.cpp:13-28
//   set_mode              initialize.cpp:128-220
//   initialize            initialize.cpp:562-810 (fresh run)
//   orthogonal_unit_vectors / TT_tensors   initialize.cpp:66-122
//   set_mode_GW / initialize_GW            initialize.cpp:273-470
#include <cmath>
#include <cstring>
#include <vector>

#include "psc_ic.h"
#include "psc_model.h"

namespace psc {
namespace {

constexpr double kPi = 3.14159265358979323846;  // 2 asin(1), pspectcosmo.h:27

inline double pw2(double x) { return x * x; }
inline int pcoord(int i, int N) { return i <= N / 2 ? i : i - N; }

// Park-Miller "minimal standard" generator with Schrage's factorisation; the
// first call discards 99 values.
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

struct Ctx {
    const psc_params &p;
    int N, H;
    long long modes;
    double fStar, omegaStar, L, dx, DFDP, a, hubble;
    ParkMiller rng;
    Ctx(const psc_params &pp)
        : p(pp), N(pp.N), H(pp.N / 2 + 1), modes((long long)pp.N * pp.N * (pp.N / 2 + 1)),
          fStar(pp.fStar > 0 ? pp.fStar : pp.MPl), omegaStar(pp.m_in_MPl * (pp.fStar > 0 ? pp.fStar : pp.MPl)),
          L(2 * kPi / pp.kIR), dx(2 * kPi / pp.kIR / (double)pp.N), DFDP(0), a(pp.a0), hubble(0), rng(pp.seed) {
        DFDP = std::pow(omegaStar / fStar, 2) * (N / dx) / 2.;  // parameters.h:132
    }
    long long idx(int i, int j, int k) const { return ((long long)i * N + j) * H + k; }
    double k2cutoff() const {
        const double kc = p.kcutoff;
        return kc < 2. * kPi * (double)N / L ? pw2(kc) : 0.;
    }
};

// potential_energy / effective_mass of the run's model (model.h:36-100), FP64
double potential_term(const psc_params &p, int term, const double *v) {
    return model_potential_term(p.model, p.gsq, term, v);
}

void effective_mass(const psc_params &p, double *m2, const double *v) { model_effective_mass(p.model, p.gsq, m2, v); }

// one mode of one field (set_mode)
void set_mode(Ctx &c, double p2, double m2, double *fk, double *pk, bool isReal) {
    const double k2c = c.k2cutoff();
    if (k2c > 0. && p2 > k2c) {
        fk[0] = fk[1] = pk[0] = pk[1] = 0.;
        return;
    }
    const double a = c.a, H0 = c.hubble;
    const double norm = std::sqrt(c.DFDP);
    const double omega = (p2 + m2 > 0.) ? std::sqrt(p2 + pw2(a) * m2) : std::sqrt(p2);
    const double rms = omega > 0. ? norm / std::sqrt(omega) : 0.;
    const double aop = std::pow(a, c.p.alpha - 3);
    if (c.p.simulate_inflation) {
        const double amp = rms / a;
        const double phase = 2. * kPi * c.rng();
        const double re = amp * std::cos(phase), im = amp * std::sin(phase);
        fk[0] = re;
        fk[1] = im;
        pk[0] = aop * (-omega * im - H0 * fk[0]);
        pk[1] = aop * (omega * re - H0 * fk[1]);
        if (isReal) {
            fk[0] = std::sqrt(pw2(fk[0]) + pw2(fk[1]));
            fk[1] = 0;
            pk[0] = std::sqrt(pw2(pk[0]) + pw2(pk[1]));
            pk[1] = 0.;
        }
    } else {
        const double al = rms / std::sqrt(2.) * std::sqrt(std::log(1. / c.rng())) / a;
        const double ar = rms / std::sqrt(2.) * std::sqrt(std::log(1. / c.rng())) / a;
        double ph = 2. * kPi * c.rng();
        const double rel = al * std::cos(ph), iml = al * std::sin(ph);
        ph = 2. * kPi * c.rng();
        const double rer = ar * std::cos(ph), imr = ar * std::sin(ph);
        fk[0] = rel + rer;
        fk[1] = iml + imr;
        pk[0] = aop * (-omega * (iml - imr) - H0 * fk[0]);
        pk[1] = aop * (omega * (rel - rer) - H0 * fk[1]);
        if (isReal) fk[1] = pk[1] = 0.;
    }
}

inline void conj_copy(double *arr, long long to, long long from) {
    arr[2 * to] = arr[2 * from];
    arr[2 * to + 1] = -arr[2 * from + 1];
}

// The reference's mode traversal (initialize.cpp:686-749 and 356-444): the
// kz = 0, N/2 planes with explicit conjugates, the interior planes, the eight
// real corners. `visit(i, j, k, px, py, conj_index_or_-1, isReal)`.
template <typename F>
void traverse(int N, int H, bool skip_origin_corner, F visit) {
    auto id = [&](int i, int j, int k) { return ((long long)i * N + j) * H + k; };
    for (int k = 0; k <= N / 2; k += N / 2) {
        for (int i = 0; i <= N / 2; i += N / 2)
            for (int j = 1; j < N / 2; j++) visit(i, j, k, i, j, id(i, N - j, k), false);
        for (int j = 0; j <= N / 2; j += N / 2)
            for (int i = 1; i < N / 2; i++) visit(i, j, k, i, j, id(N - i, j, k), false);
        for (int i = 1; i < N / 2; i++) {
            for (int j = 1; j < N / 2; j++) visit(i, j, k, i, j, id(N - i, N - j, k), false);
            for (int j = N / 2 + 1; j < N; j++) visit(i, j, k, i, j - N, id(N - i, N - j, k), false);
        }
    }
    for (int k = 1; k < N / 2; k++)
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++) visit(i, j, k, pcoord(i, N), pcoord(j, N), -1LL, false);
    for (int k = 0; k <= N / 2; k += N / 2)
        for (int i = 0; i <= N / 2; i += N / 2)
            for (int j = 0; j <= N / 2; j += N / 2) {
                if (skip_origin_corner && i == 0 && j == 0 && k == 0) continue;
                visit(i, j, k, i, j, -1LL, true);
            }
}

void tt_tensor(const double k[3], double e[3][3]) {
    const double kn = std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
    const double kh[3] = {k[0] / kn, k[1] / kn, k[2] / kn};
    double tmp[3] = {0, 0, 1};
    if (std::fabs(kh[0]) < 1e-9 && std::fabs(kh[1]) < 1e-9 && std::fabs(kh[2] - 1) < 1e-9) {
        tmp[1] = 1;
        tmp[2] = 0;
    }
    double u[3] = {kh[1] * tmp[2] - kh[2] * tmp[1], kh[2] * tmp[0] - kh[0] * tmp[2], kh[0] * tmp[1] - kh[1] * tmp[0]};
    const double un = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (double &x : u) x /= un;
    double v[3] = {kh[1] * u[2] - kh[2] * u[1], kh[2] * u[0] - kh[0] * u[2], kh[0] * u[1] - kh[1] * u[0]};
    const double vn = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (double &x : v) x /= vn;
    for (int i = 0; i < 3; i++)
        if (u[i] < 0) {
            for (double &x : u) x = -x;
            break;
        }
    for (int i = 0; i < 3; i++)
        if (v[i] < 0) {
            for (double &x : v) x = -x;
            break;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) e[i][j] = u[i] * u[j] - v[i] * v[j] + u[i] * v[j] + v[i] * u[j];
}

const int kSymI[6] = {0, 0, 0, 1, 1, 2};
const int kSymJ[6] = {0, 1, 2, 1, 2, 2};

void set_mode_gw(Ctx &c, const double kv[3], double k2, long long m, bool isReal, double *u_k, double *pu_k) {
    const long long M2 = 2 * c.modes;
    const double k2c = c.k2cutoff();
    if (k2c > 0. && k2 > k2c) {
        for (int q = 0; q < 6; q++) {
            u_k[q * M2 + 2 * m] = u_k[q * M2 + 2 * m + 1] = 0.;
            pu_k[q * M2 + 2 * m] = pu_k[q * M2 + 2 * m + 1] = 0.;
        }
        return;
    }
    double e[3][3];
    tt_tensor(kv, e);
    const double a = c.a, H0 = c.hubble;
    const double norm = c.p.MPl * c.omegaStar / pw2(c.fStar) * std::pow(c.N / c.dx, 1.5);
    const double k = std::sqrt(k2);
    const double rms = norm / std::sqrt(k);
    const double al = rms / std::sqrt(2.) * std::sqrt(std::log(1. / c.rng())) / a;
    const double ar = rms / std::sqrt(2.) * std::sqrt(std::log(1. / c.rng())) / a;
    double ph = 2. * kPi * c.rng();
    const double rel = al * std::cos(ph), iml = al * std::sin(ph);
    ph = 2. * kPi * c.rng();
    const double rer = ar * std::cos(ph), imr = ar * std::sin(ph);
    const double aop = std::pow(a, c.p.alpha - 3);
    for (int q = 0; q < 6; q++) {
        const double ec = e[kSymI[q]][kSymJ[q]];
        double *u = u_k + q * M2 + 2 * m, *pu = pu_k + q * M2 + 2 * m;
        u[0] = ec * (rel + rer);
        u[1] = ec * (iml + imr);
        pu[0] = aop * (ec * (-k * (iml - imr) - H0 * u[0]));
        pu[1] = aop * (ec * (k * (rel - rer) - H0 * u[1]));
        if (isReal) u[1] = pu[1] = 0.;
    }
}

}  // namespace

ICSetup ic_setup(const psc_params &p) {
    Ctx c(p);
    ICSetup s{};
    const int N = c.N, nf = p.nflds;
    s.N = N;
    s.H = c.H;
    s.nf = nf;
    s.model = p.model;
    s.alpha = p.alpha;
    s.simulate_inflation = p.simulate_inflation;
    s.gw = p.with_gw;
    s.fStar = c.fStar;
    s.omegaStar = c.omegaStar;
    s.dx = c.dx;
    s.DFDP = c.DFDP;
    s.kIR = p.kIR;
    s.gsq = p.gsq;
    s.dp2 = pw2(p.kIR);
    s.k2c = c.k2cutoff();
    for (int fld = 0; fld < nf; fld++) {
        s.f0[fld] = p.initfield[fld] / c.fStar;
        s.fd0[fld] = p.initderivs[fld] / c.fStar / c.omegaStar;
    }
    effective_mass(p, s.m2, s.f0);
    s.a = p.a0;
    s.info.a = s.a;
    if (p.expansion > 0) {
        double fdsq = 0., pot = 0.;
        for (int fld = 0; fld < nf; fld++) fdsq += pw2(s.fd0[fld]);
        const int nterms = model_nterms(p.model);
        for (int t = 0; t < nterms; t++) pot += potential_term(p, t, s.f0);
        double h = fdsq / 2.;
        h += pot;
        h *= pw2(c.fStar / p.MPl) / 3.;
        s.hubble = std::sqrt(h);
        s.info.ad = s.hubble * s.a;
        s.info.add_printed = pw2(c.fStar / p.MPl) / 3. * ((p.alpha - 2) * fdsq + (p.alpha + 1) * pot) * s.a;
        s.info.kinetic = fdsq / 2.;
        s.info.potential = pot;
    }
    s.info.hubble_init = s.hubble;
    s.aop = std::pow(s.a, p.alpha - 3);
    s.norm_s = std::sqrt(c.DFDP);
    s.norm_gw = p.MPl * c.omegaStar / pw2(c.fStar) * std::pow(c.N / c.dx, 1.5);
    s.n3 = (double)N * N * N;
    s.seed = p.seed;
    const long long h2 = N / 2 - 1;
    s.visits = 2 * h2 * (N + 2) + h2 * (long long)N * N + 8;
    s.dpm = p.simulate_inflation ? 1 : 4;
    return s;
}

ICInfo generate_ic(const psc_params &p, double *f_k, double *pi_k, double *u_k, double *pi_u_k) {
    Ctx c(p);
    const int N = c.N, H = c.H, nf = p.nflds;
    const double dp2 = pw2(p.kIR);
    const long long M2 = 2 * c.modes;
    double initial_f[PSC_MAX_FIELDS] = {}, initial_fd[PSC_MAX_FIELDS] = {}, mass_sq[PSC_MAX_FIELDS] = {};
    for (int fld = 0; fld < nf; fld++) {
        initial_f[fld] = p.initfield[fld] / c.fStar;
        initial_fd[fld] = p.initderivs[fld] / c.fStar / c.omegaStar;
    }
    effective_mass(p, mass_sq, initial_f);
    ICInfo info{};
    c.a = p.a0;
    info.a = c.a;
    if (p.expansion > 0) {
        double fdsq = 0., pot = 0.;
        for (int fld = 0; fld < nf; fld++) fdsq += pw2(initial_fd[fld]);
        const int nterms = model_nterms(p.model);
        for (int t = 0; t < nterms; t++) pot += potential_term(p, t, initial_f);
        double h = fdsq / 2.;
        h += pot;
        h *= pw2(c.fStar / p.MPl) / 3.;
        c.hubble = std::sqrt(h);
        info.ad = c.hubble * c.a;
        info.add_printed = pw2(c.fStar / p.MPl) / 3. * ((p.alpha - 2) * fdsq + (p.alpha + 1) * pot) * c.a;
        info.kinetic = fdsq / 2.;
        info.potential = pot;
    }
    info.hubble_init = c.hubble;
    const double n3 = (double)N * N * N;
    for (int fld = 0; fld < nf; fld++) {
        double *fk = f_k + fld * M2, *pk = pi_k + fld * M2;
        const double m2 = mass_sq[fld];
        traverse(N, H, false, [&](int i, int j, int k, int px, int py, long long conj, bool real) {
            const long long m = c.idx(i, j, k);
            set_mode(c, dp2 * (pw2(px) + pw2(py) + pw2(k)), m2, fk + 2 * m, pk + 2 * m, real);
            if (conj >= 0) {
                conj_copy(fk, conj, m);
                conj_copy(pk, conj, m);
            }
        });
        fk[0] = initial_f[fld] * n3;
        fk[1] = 0.;
        pk[0] = std::pow(c.a, p.alpha - 3) * initial_fd[fld] * n3;
        pk[1] = 0.;
    }
    if (p.with_gw && u_k && pi_u_k) {
        traverse(N, H, true, [&](int i, int j, int k, int px, int py, long long conj, bool real) {
            const long long m = c.idx(i, j, k);
            const double kv[3] = {px * p.kIR, py * p.kIR, k * p.kIR};
            set_mode_gw(c, kv, dp2 * (pw2(px) + pw2(py) + pw2(k)), m, real, u_k, pi_u_k);
            if (conj >= 0)
                for (int q = 0; q < 6; q++) {
                    conj_copy(u_k + q * M2, conj, m);
                    conj_copy(pi_u_k + q * M2, conj, m);
                }
        });
        for (int q = 0; q < 6; q++) {
            u_k[q * M2] = u_k[q * M2 + 1] = 0.;
            pi_u_k[q * M2] = pi_u_k[q * M2 + 1] = 0.;
        }
    }
    return info;
}

}  // namespace psc
