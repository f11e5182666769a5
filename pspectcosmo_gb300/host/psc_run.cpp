// psc_run.cpp — C++ host of the lattice evolution: drives libpsc.so through its C ABI
// (include/psc.h) the way the reference's main() drives its evolution functions.
//
// Two modes:
//   * the run loop (default) — pspectcosmo.cpp:600-697: initialize(), save(), then
//       dt = calculate_dt(kIR N sqrt(3)/2, a)           (pspectcosmo.cpp:213-233: 0.2 a / k)
//       dt = min(dt, tOutputFreq), clipped to the next frequent / infrequent output time
//       evolve(dt); save_Freq() / save_Infreq() at the output times (|t - next| < 1e-10)
//     writing the reference's text files into `out`: average_scalar_<f>, average_scale_factor,
//     average_energies, average_energy_conservation (save_Freq, output.cpp:1831-1840) and
//     spectra_scalar_<f>, average_spectra_times, spectra_gws, energy_gws (spectra(),
//     output.cpp:490-1062), with the reference's 6-digit formatting;
//   * a fixed step (nsteps=K dt=D): initialize(), then K steps of D in one psc_step call, and
//     the final state written to `state` (binary: int32 {0x53435350, N, nflds, with_gw},
//     double {t, a, a', a''}, then f_k, pi_k [, u_k, pi_u_k] as interleaved FP64 complex in
//     the reference's FFTW layout).
//
// Arguments are key=value pairs: preset=reference|preheating (the shipped parameters.h /
// model.h, or two-field preheating), any psc_params field by its parameters.h name
// (N, nflds, vv, spectral, with_gw, precision, model, seed, kIR, gsq, m_in_MPl, initfield0,
// initderivs0, ... initfield3, initderivs3), model_name (a model.h compiled into the library,
// by file stem), and tf, tOutputFreq, tOutputInfreq, nsteps, dt, out, state.
//
// Build (one line): g++ -O2 -std=c++17 -I include pspectcosmo_gb300/host/psc_run.cpp
//   -L pspectcosmo_gb300 -lpsc -Wl,-rpath,<dir of libpsc.so> -o psc_run
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <sys/stat.h>
#include <vector>

#include "psc.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

void check(int rc, const char *where) {
    if (rc != PSC_OK) {
        std::fprintf(stderr, "%s: %s (%d): %s\n", where, psc_strerror(rc), rc, psc_last_error());
        std::exit(1);
    }
}

struct Run {
    psc_params p{};
    double tf = 0.02, tOutputFreq = 0.001, tOutputInfreq = 0.005, dt = 0.0;
    int nsteps = 0;
    std::string out = "output", state;
};

void preheating(psc_params &p) {
    psc_default_params(&p);
    p.nflds = 2;
    p.model = PSC_MODEL_PHI2CHI2;
    p.gsq = 2.5e5;
    p.kIR = 1.0;
    p.vv = 4;
    p.initfield[0] = 0.193 * p.MPl;
    p.initfield[1] = 0.0;
    p.initderivs[0] = -0.142e-6 * p.MPl * p.MPl;
    p.initderivs[1] = 0.0;
}

bool set_param(Run &r, const std::string &k, const std::string &v) {
    psc_params &p = r.p;
    const double d = std::atof(v.c_str());
    const int i = std::atoi(v.c_str());
    struct IntField { const char *name; int *dst; };
    struct DblField { const char *name; double *dst; };
    const IntField ints[] = {{"N", &p.N},           {"nflds", &p.nflds},       {"vv", &p.vv},
                             {"alpha", &p.alpha},   {"expansion", &p.expansion}, {"simulate_inflation", &p.simulate_inflation},
                             {"spectral", &p.spectral}, {"with_gw", &p.with_gw}, {"precision", &p.precision},
                             {"model", &p.model},   {"seed", &p.seed},         {"N_pad", &p.N_pad},
                             {"nsteps", &r.nsteps}};
    const DblField dbls[] = {{"kIR", &p.kIR},         {"a0", &p.a0},       {"MPl", &p.MPl},
                             {"m_in_MPl", &p.m_in_MPl}, {"fStar", &p.fStar}, {"epsilon", &p.epsilon},
                             {"gsq", &p.gsq},         {"kcutoff", &p.kcutoff}, {"initfield0", &p.initfield[0]},
                             {"initfield1", &p.initfield[1]}, {"initfield2", &p.initfield[2]},
                             {"initfield3", &p.initfield[3]}, {"initderivs0", &p.initderivs[0]},
                             {"initderivs1", &p.initderivs[1]}, {"initderivs2", &p.initderivs[2]},
                             {"initderivs3", &p.initderivs[3]}, {"tf", &r.tf}, {"tOutputFreq", &r.tOutputFreq},
                             {"tOutputInfreq", &r.tOutputInfreq}, {"dt", &r.dt}};
    for (const IntField &f : ints)
        if (k == f.name) return *f.dst = i, true;
    for (const DblField &f : dbls)
        if (k == f.name) return *f.dst = d, true;
    if (k == "model_name") return psc_model_find(v.c_str(), &p.model) == PSC_OK;   // a compiled model.h by file stem
    if (k == "out") return r.out = v, true;
    if (k == "state") return r.state = v, true;
    return false;
}

// The reference's text outputs (output.cpp) from the library's reductions.
class Writer {
  public:
    Writer(const psc_params &p, std::string dir) : p_(p), dir_(std::move(dir)), nb_(psc_maxnumbins(p.N)) {
        ::mkdir(dir_.c_str(), 0755);
    }

    // save_Freq() (output.cpp:1831-1840): meansvars, scale, energy
    void save_freq(psc_handle *h) {
        const Bg b = bg(h);
        std::vector<double> m(6 * p_.nflds);
        check(psc_means(h, m.data()), "psc_means");
        for (int f = 0; f < p_.nflds; ++f) {
            FILE *fh = open("average_scalar_" + std::to_string(f));
            std::fprintf(fh, "%.3f", b.t);
            for (int c = 0; c < 6; ++c) std::fprintf(fh, "%15.6e", m[6 * f + c]);
            std::fprintf(fh, "\n");
            std::fclose(fh);
        }
        const int al = p_.alpha;
        if (p_.expansion == 2) {   // scale() (output.cpp:467-486)
            FILE *fh = open("average_scale_factor");
            std::fprintf(fh, "%.6f %.6f %.6f %.6f %.6f %15.6e %.6f\n", b.t, b.a, b.ad, b.ad / b.a, b.add,
                         1.0 / (std::pow(b.a, -al) * b.ad), 1.0 + al - b.a * b.add / (b.ad * b.ad));
            std::fclose(fh);
        }
        const En e = energies(h);
        FILE *fh = open("average_energies");   // energy() (output.cpp:1163-1168)
        std::fprintf(fh, "%.3f", b.t);
        for (int f = 0; f < p_.nflds; ++f) std::fprintf(fh, " %.6e %.6e", e.K[f], e.G[f]);
        for (double v : e.V) std::fprintf(fh, " %.6e", v);
        std::fprintf(fh, " %.6e\n", e.total);
        std::fclose(fh);
        if (p_.expansion != 1) {   // output.cpp:1171-1185
            const double fs = p_.fStar > 0 ? p_.fStar : p_.MPl;
            const double lhs = b.ad * b.ad;
            const double rhs = (fs / p_.MPl) * (fs / p_.MPl) * std::pow(b.a, 2 * (al + 1)) * e.total / 3.0;
            FILE *fc = open("average_energy_conservation");
            std::fprintf(fc, "%.3f %.8e %.6f %.6f\n", b.t, e.fviol, lhs, rhs);
            std::fclose(fc);
        }
    }

    // spectra() (output.cpp:490-1062): the columns of output.cpp:671-690 and 1041-1060
    void spectra(psc_handle *h) {
        const Bg b = bg(h);
        const En e = energies(h);
        const int nf = p_.nflds, nb = nb_, al = p_.alpha;
        std::vector<int32_t> np(nf * nb), gnp(nb);
        std::vector<double> f2(nf * nb), pi2(nf * nb), n2(nf * nb), h2(nb), hd2(nb), m(6 * nf);
        double hd0 = 0.0;
        check(psc_spectra(h, np.data(), f2.data(), pi2.data(), n2.data(), gnp.data(), h2.data(), hd2.data(), &hd0),
              "psc_spectra");
        check(psc_means(h, m.data()), "psc_means");
        const double n3 = std::pow((double)p_.N, 3), fs = p_.fStar > 0 ? p_.fStar : p_.MPl;
        const double omega = p_.m_in_MPl * fs, L = 2 * kPi / p_.kIR;
        // <effective_mass(f(x))> (output.cpp:571-580): the built-in models' masses are linear in
        // f^2; a model.h compiled in is evaluated at every site by the library
        double m2[PSC_MAX_FIELDS] = {1.0, 0.0, 0.0, 0.0};
        if (p_.model == PSC_MODEL_PHI2CHI2) {
            m2[0] = 1.0 + p_.gsq * m[6 + 2];
            m2[1] = p_.gsq * m[2];
        } else if (p_.model != PSC_MODEL_PHI2) {
            check(psc_mass_sq_av(h, m2), "psc_mass_sq_av");
        }
        const double aop = std::pow(b.a, al - 3);
        for (int f = 0; f < nf; ++f) {
            FILE *fh = open("spectra_scalar_" + std::to_string(f));
            for (int i = 1; i < nb; ++i) {
                const double pk = p_.kIR * i;
                const int c = np[f * nb + i];
                double nd = 0.0;
                const double om2 = std::fabs(pk * pk + b.a * b.a * m2[f]);
                if (om2 > 0) {
                    const double om = std::sqrt(om2);
                    nd = b.a * b.a * L * L * L / 2.0 / (n3 * n3) * (fs / omega) * (fs / omega) *
                         (om * f2[f * nb + i] + std::pow(b.a, 2 * (1 - al)) / om * n2[f * nb + i]);
                }
                std::fprintf(fh, "%.1f %15.6e %15.6e %15.6e %d\n", pk, i / (n3 * n3) * c * f2[f * nb + i],
                             i / (n3 * n3) * c * aop * aop * pi2[f * nb + i], nd, c);
            }
            std::fprintf(fh, "\n");
            std::fclose(fh);
        }
        FILE *ft = open("average_spectra_times");
        std::fprintf(ft, "%.2f\n", b.t);
        std::fclose(ft);
        if (!p_.with_gw) return;
        FILE *fg = open("spectra_gws");
        for (int i = 1; i < nb; ++i) {
            const int c = gnp[i];
            std::fprintf(fg, "%.1f %15.6e %15.6e %15.6e %d\n", p_.kIR * i, i / (n3 * n3) * c * h2[i],
                         i / (n3 * n3) / 4.0 / std::pow(b.a, 6) * (fs / p_.MPl) * (fs / p_.MPl) / e.total * c * hd2[i],
                         (p_.MPl * omega) * (p_.MPl * omega) / std::pow(fs, 4) * 2 / (kPi * kPi) * b.ad * b.ad /
                             std::pow(b.a, 2 * al + 2),
                         c);
        }
        std::fprintf(fg, "\n");
        std::fclose(fg);
        FILE *fe = open("energy_gws");
        std::fprintf(fe, "%.2f %.6e %.6e\n", b.t, e.rho / e.total, e.rho);
        std::fclose(fe);
    }

  private:
    struct Bg { double t, a, ad, add; };
    struct En {
        std::vector<double> K, G, V;
        double total, fviol, rho;
    };
    Bg bg(psc_handle *h) const {
        Bg b{};
        check(psc_get_time(h, &b.t), "psc_get_time");
        check(psc_get_state(h, nullptr, nullptr, &b.a, &b.ad, &b.add, nullptr, nullptr), "psc_get_state");
        return b;
    }
    En energies(psc_handle *h) const {
        En e;
        e.K.resize(p_.nflds);
        e.G.resize(p_.nflds);
        e.V.resize(p_.model == PSC_MODEL_PHI2 ? 1 : 2);
        check(psc_energies(h, e.K.data(), e.G.data(), e.V.data(), &e.total, &e.fviol, &e.rho), "psc_energies");
        return e;
    }
    FILE *open(const std::string &name) const {
        FILE *fh = std::fopen((dir_ + "/" + name + ".txt").c_str(), "a");
        if (!fh) {
            std::perror(name.c_str());
            std::exit(1);
        }
        return fh;
    }
    psc_params p_;
    std::string dir_;
    int nb_;
};

void write_state(psc_handle *h, const psc_params &p, const std::string &path) {
    const size_t modes = (size_t)p.N * p.N * (p.N / 2 + 1);
    std::vector<double> f(2 * modes * p.nflds), pi(f.size()), u, pu;
    if (p.with_gw) {
        u.resize(2 * modes * 6);
        pu.resize(u.size());
    }
    double bg[4];
    check(psc_get_time(h, &bg[0]), "psc_get_time");
    check(psc_get_state(h, f.data(), pi.data(), &bg[1], &bg[2], &bg[3], p.with_gw ? u.data() : nullptr,
                        p.with_gw ? pu.data() : nullptr),
          "psc_get_state");
    FILE *fh = std::fopen(path.c_str(), "wb");
    if (!fh) {
        std::perror(path.c_str());
        std::exit(1);
    }
    const int32_t hdr[4] = {0x53435350, p.N, p.nflds, p.with_gw};
    std::fwrite(hdr, sizeof hdr, 1, fh);
    std::fwrite(bg, sizeof bg, 1, fh);
    std::fwrite(f.data(), sizeof(double), f.size(), fh);
    std::fwrite(pi.data(), sizeof(double), pi.size(), fh);
    if (p.with_gw) {
        std::fwrite(u.data(), sizeof(double), u.size(), fh);
        std::fwrite(pu.data(), sizeof(double), pu.size(), fh);
    }
    std::fclose(fh);
}

}  // namespace

int main(int argc, char **argv) {
    Run r;
    psc_default_params(&r.p);
    for (int i = 1; i < argc; ++i) {   // a preset first, so that later keys override it
        if (std::strcmp(argv[i], "preset=preheating") == 0) preheating(r.p);
    }
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        const size_t eq = a.find('=');
        if (eq == std::string::npos) {
            std::fprintf(stderr, "argument %s is not key=value\n", argv[i]);
            return 2;
        }
        const std::string k = a.substr(0, eq), v = a.substr(eq + 1);
        if (k == "preset") continue;
        if (!set_param(r, k, v)) {
            std::fprintf(stderr, "unknown key %s\n", k.c_str());
            return 2;
        }
    }
    psc_handle *h = nullptr;
    check(psc_create(&r.p, &h), "psc_create");
    check(psc_init_ic(h), "psc_init_ic");   // initialize() [+ initialize_GW()]

    if (r.nsteps > 0) {   // a fixed step
        if (!(r.dt > 0)) {
            std::fprintf(stderr, "nsteps needs dt > 0\n");
            return 2;
        }
        check(psc_step(h, r.dt, r.nsteps), "psc_step");
        if (!r.state.empty()) write_state(h, r.p, r.state);
        psc_destroy(h);
        return 0;
    }

    // the run loop (pspectcosmo.cpp:600-697)
    Writer w(r.p, r.out);
    w.save_freq(h);   // save() (output.cpp:1796-1829) without histograms
    w.spectra(h);
    const double kmax = r.p.kIR * r.p.N * std::sqrt(3.0) / 2.0;
    double next_freq = r.tOutputFreq, next_infreq = r.tOutputInfreq, t = 0.0;
    check(psc_get_time(h, &t), "psc_get_time");
    while (t < r.tf) {
        double a = 0.0;
        check(psc_get_state(h, nullptr, nullptr, &a, nullptr, nullptr, nullptr, nullptr), "psc_get_state");
        double dt = 2.0 / (kmax / a) / 10;   // calculate_dt (pspectcosmo.cpp:213-233)
        dt = std::min(dt, r.tOutputFreq);
        if (t + dt > next_freq || t + dt > next_infreq) dt = std::min(next_freq - t, next_infreq - t);
        const int rc = psc_step(h, dt, 1);   // evolve_VV_k_nopad(dt) / evolve_VV(dt)
        if (rc == PSC_ERR_NONFINITE) {   // the reference's "Unstable solution" exit (output.cpp:450-454)
            std::fprintf(stderr, "Unstable solution at t = %g: %s\n", t, psc_last_error());
            psc_destroy(h);
            return 1;
        }
        check(rc, "psc_step");
        check(psc_get_time(h, &t), "psc_get_time");
        if (std::fabs(t - next_freq) < 1e-10) {
            next_freq += r.tOutputFreq;
            w.save_freq(h);
        }
        if (std::fabs(t - next_infreq) < 1e-10) {
            next_infreq += r.tOutputInfreq;
            w.spectra(h);   // save_Infreq() without histograms
        }
    }
    psc_destroy(h);
    return 0;
}
