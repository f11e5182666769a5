/*
 * Harness main for the oracle build of the reference's own sources
 * (test infrastructure only; compiled by oracle/build_ref.py into oracle/_ref/).
 *
 * It replaces the reference's main() (pspectcosmo.cpp:236-742, compiled here as
 * reference_main and never called) with a fixed-dt driver:
 *   - replicates the allocation block (pspectcosmo.cpp:253-282) and a = a0, t = 0
 *     (pspectcosmo.cpp:295-300);
 *   - calls initialize() (initialize.cpp:562) and, with GWs, initialize_GW()
 *     (initialize.cpp:341), then save() (output.cpp:1796) as main does
 *     (pspectcosmo.cpp:489-545);
 *   - steps evolve_VV_k_nopad(dt) (evolution.cpp:1131), evolve_VV_k_pad(dt) with
 *     PAD_FLAG (evolution.cpp:1688) or evolve_VV(dt) (evolution.cpp:607) with the FIXED dt given on the command line instead of
 *     the adaptive calculate_dt (pspectcosmo.cpp:213-233);
 *   - every `every` steps calls save_Freq(), save_Infreq() and save_Snap(step)
 *     (output.cpp:1831, 1842, 1850) and dumps the raw state.
 * Everything runs on a thread with a 2 GiB stack, because the real-space path
 * keeps N^3 arrays on the stack (evolution.cpp:612, 441, 581).
 *
 * usage: harness NSTEPS DT EVERY      (run inside the output directory)
 *        harness main                 (the reference's own main(): its adaptive-dt driver loop)
 *        harness analytic NA DTA EVERYA NSTEPS DT EVERY   (ANALYTIC_EVOLUTION builds: NA analytic
 *                                     steps of DTA, initialize_lattice(), NSTEPS lattice steps)
 * writes: output/*.txt (reference writers, 17 digits), state_<step>.bin, bg.txt,
 *         ic_info.txt, and with ssnapshot output/Snapshots/data_<step>_snapshot.h5.*.bin
 *         (the raw datasets, through the HDF5 shim)
 */
#include "pspectcosmo.h"

#include <omp.h>
#include <pthread.h>
#include <chrono>
#include <algorithm>
#include <complex>
#include <vector>
#include <cstdio>
#include <cstdlib>
#include <string>

static long g_nsteps = 0, g_every = 1;
static double g_dt = 0.0;

static void dump_state(long step) {
    char name[64];
    std::snprintf(name, sizeof name, "state_%06ld.bin", step);
    std::FILE *fp = std::fopen(name, "wb");
    if (!fp) { std::perror(name); std::exit(3); }
    int hdr[6] = {0x44435350 /* 'PSCD' */, 1, N, nflds, (int)SPECTRAL_FLAG, (int)WITH_GW};
    std::fwrite(hdr, sizeof(int), 6, fp);
    double bg[4] = {t, a, ad, add};
    std::fwrite(bg, sizeof(double), 4, fp);
    const size_t modes = (size_t)N * N * (N / 2 + 1);
    const size_t sites = (size_t)N * N * N;
    for (int fld = 0; fld < nflds; fld++) std::fwrite(f_k[fld], sizeof(fftw_complex), modes, fp);
    for (int fld = 0; fld < nflds; fld++) std::fwrite(pi_k[fld], sizeof(fftw_complex), modes, fp);
    std::fwrite(&f[0][0][0][0], sizeof(double), sites * nflds, fp);
    std::fwrite(&pi_f[0][0][0][0], sizeof(double), sites * nflds, fp);
#if WITH_GW
    std::fwrite(&u[0][0][0][0][0], sizeof(double), sites * 9, fp);
    std::fwrite(&pi_u[0][0][0][0][0], sizeof(double), sites * 9, fp);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) std::fwrite(u_k[i][j], sizeof(fftw_complex), modes, fp);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) std::fwrite(pi_u_k[i][j], sizeof(fftw_complex), modes, fp);
#endif
    std::fclose(fp);
}

#if ANALYTIC_EVOLUTION
// the analytic perturbation state (initialize.cpp:814-958, evolution.cpp:174-336)
static void dump_analytic(long step) {
    char name[64];
    std::snprintf(name, sizeof name, "analytic_%06ld.bin", step);
    std::FILE *fp = std::fopen(name, "wb");
    if (!fp) { std::perror(name); std::exit(3); }
    int hdr[4] = {0x41435350 /* 'PSCA' */, (int)num_k_values, nflds, 0};
    std::fwrite(hdr, sizeof(int), 4, fp);
    double bg[4] = {t, a_k, ad_k, add_k};
    std::fwrite(bg, sizeof(double), 4, fp);
    std::vector<int> k2(k_square_vec.begin(), k_square_vec.end());
    std::fwrite(k2.data(), sizeof(int), k2.size(), fp);
    for (const auto *v : {&fk_left, &pi_k_left, &fk_right, &pi_k_right})
        for (int fld = 0; fld < nflds; fld++) std::fwrite((*v)[fld].data(), sizeof(std::complex<double>), num_k_values, fp);
    std::fclose(fp);
}
#endif

static void step_once(double dt_) {
#if SPECTRAL_FLAG && PAD_FLAG
    evolve_VV_k_pad(dt_);
#elif SPECTRAL_FLAG
    evolve_VV_k_nopad(dt_);
#else
    evolve_VV(dt_);
#endif
}

static void *run(void *) {
    checkdirectory();
    fftw_init_threads();
    fftw_plan_with_nthreads(n_threads);

    const size_t modes = (size_t)N * N * (N / 2 + 1);
    Cache_Data_k = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
    R_k = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
    for (int fld = 0; fld < nflds; fld++) {
        f_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        pi_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
#if SPECTRAL_FLAG
        pi_k_half[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        V_prime_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        kernel_f_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
#endif
    }
#if SPECTRAL_FLAG && PAD_FLAG
    // the padded step's buffers (pspectcosmo.cpp:254-271)
    {
        const size_t modes_pad = (size_t)N_pad * N_pad * (N_pad / 2 + 1);
        Cache_Data_k_pad = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes_pad);
        for (int fld = 0; fld < nflds; fld++) {
            f_k_pad[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes_pad);
            V_prime_k_pad[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes_pad);
        }
    }
#endif
#if WITH_GW
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            u_k[i][j] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
            pi_u_k[i][j] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        }
#endif
    dt = g_dt;
    t0 = 0.;
    t = t0;
    a = a0;

    initialize();
    {
        std::FILE *fp = std::fopen("ic_info.txt", "w");
        std::fprintf(fp, "hubble_init %.17g\na %.17g\nad %.17g\nadd %.17g\n", hubble_init, a, ad, add);
        std::fclose(fp);
    }
#if WITH_GW
    initialize_GW();
#endif
    dump_state(0);
    save();

    std::FILE *bgf = std::fopen("bg.txt", "w");
    std::fprintf(bgf, "%ld %.17g %.17g %.17g %.17g\n", 0L, t, a, ad, add);
    for (long s = 1; s <= g_nsteps; s++) {
        step_once(g_dt);
        std::fprintf(bgf, "%ld %.17g %.17g %.17g %.17g\n", s, t, a, ad, add);
        if (s % g_every == 0) {
            save_Freq();
            save_Infreq();
            save_Snap((double)s);   // snapshots() when ssnapshot is on (output.cpp:1850-1853)
            dump_state(s);
        }
    }
    std::fclose(bgf);
    return nullptr;
}

// timing mode: initialize() [+ initialize_GW()], then g_nsteps steps of g_dt timed on the
// wall clock, with no output; prints the seconds per step. The FFTs (the reference's only
// threaded part, pspectcosmo.cpp:251) use every host core.
static void *run_timing(void *) {
    fftw_init_threads();
    fftw_plan_with_nthreads(std::max(1, omp_get_max_threads()));
    const size_t modes = (size_t)N * N * (N / 2 + 1);
    Cache_Data_k = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
    R_k = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
    for (int fld = 0; fld < nflds; fld++) {
        f_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        pi_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
#if SPECTRAL_FLAG
        pi_k_half[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        V_prime_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        kernel_f_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
#endif
    }
#if WITH_GW
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            u_k[i][j] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
            pi_u_k[i][j] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        }
#endif
    dt = g_dt;
    t0 = 0.;
    t = t0;
    a = a0;
    initialize();
#if WITH_GW
    initialize_GW();
#endif
    const auto t_start = std::chrono::steady_clock::now();
    for (long s = 1; s <= g_nsteps; s++) step_once(g_dt);
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    std::printf("steps %ld seconds %.6f seconds_per_step %.6f threads %d a %.17g\n", g_nsteps, el,
                el / (double)g_nsteps, omp_get_max_threads(), a);
    return nullptr;
}

int reference_main();   // the reference's own main() (pspectcosmo.cpp:236), renamed at compile time

static void *run_reference_main(void *) {
    reference_main();
    return nullptr;
}

#if ANALYTIC_EVOLUTION
static long g_na = 0, g_everya = 1;
static double g_dta = 0.0;

// the reference's analytic phase with a fixed step (pspectcosmo.cpp:370-447 with its
// adaptive dt replaced), initialize_lattice(), then fixed-dt lattice steps
static void *run_analytic(void *) {
    checkdirectory();
    fftw_init_threads();
    fftw_plan_with_nthreads(n_threads);
    const size_t modes = (size_t)N * N * (N / 2 + 1);
    Cache_Data_k = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
    R_k = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
    for (int fld = 0; fld < nflds; fld++) {
        f_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        pi_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
#if SPECTRAL_FLAG
        pi_k_half[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        V_prime_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
        kernel_f_k[fld] = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * modes);
#endif
    }
    t0 = 0.;
    t = t0;
    a = a0;
    k_square_initialize();
    initialize_analytic_perturbation();
    dump_analytic(0);
    for (long s = 1; s <= g_na; s++) {
        evolve_VV_analytic_perturbation(g_dta);
        if (s % g_everya == 0) {
            save_Freq_analytic();
            save_Infreq_analytic();
            dump_analytic(s);
        }
    }
    initialize_lattice();
    dump_state(0);
    for (long s = 1; s <= g_nsteps; s++) {
        step_once(g_dt);
        if (s % g_every == 0) dump_state(s);
    }
    return nullptr;
}
#endif

int main(int argc, char **argv) {
#if ANALYTIC_EVOLUTION
    if (argc == 8 && std::string(argv[1]) == "analytic") {
        g_na = std::atol(argv[2]);
        g_dta = std::atof(argv[3]);
        g_everya = std::max(1L, std::atol(argv[4]));
        g_nsteps = std::atol(argv[5]);
        g_dt = std::atof(argv[6]);
        g_every = std::max(1L, std::atol(argv[7]));
        pthread_attr_t attr;
        pthread_attr_init(&attr);
        pthread_attr_setstacksize(&attr, (size_t)2 << 30);
        pthread_t th;
        if (pthread_create(&th, &attr, run_analytic, nullptr) != 0) return 3;
        pthread_join(th, nullptr);
        return 0;
    }
#endif
    // the worker thread's stack: the real-space path keeps N^3 arrays on the stack
    // (evolution.cpp:612, 441, 581); PSC_HARNESS_STACK_GB raises it for large lattices
    const char *sgb = std::getenv("PSC_HARNESS_STACK_GB");
    const size_t stack = (size_t)(sgb ? std::max(1, std::atoi(sgb)) : 2) << 30;
    if (argc == 4 && std::string(argv[1]) == "time") {
        g_nsteps = std::max(1L, std::atol(argv[2]));
        g_dt = std::atof(argv[3]);
        pthread_attr_t attr;
        pthread_attr_init(&attr);
        pthread_attr_setstacksize(&attr, stack);
        pthread_t th;
        if (pthread_create(&th, &attr, run_timing, nullptr) != 0) return 3;
        pthread_join(th, nullptr);
        return 0;
    }
    if (argc == 2 && std::string(argv[1]) == "main") {
        // the reference's own driver: adaptive dt, output cadence (pspectcosmo.cpp:600-697)
        pthread_attr_t attr;
        pthread_attr_init(&attr);
        pthread_attr_setstacksize(&attr, (size_t)2 << 30);
        pthread_t th;
        if (pthread_create(&th, &attr, run_reference_main, nullptr) != 0) return 3;
        pthread_join(th, nullptr);
        return 0;
    }
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s NSTEPS DT EVERY | %s main\n", argv[0], argv[0]);
        return 2;
    }
    g_nsteps = std::atol(argv[1]);
    g_dt = std::atof(argv[2]);
    g_every = std::atol(argv[3]);
    if (g_every < 1) g_every = 1;
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, stack);
    pthread_t th;
    if (pthread_create(&th, &attr, run, nullptr) != 0) {
        std::fprintf(stderr, "cannot start worker thread\n");
        return 3;
    }
    pthread_join(th, nullptr);
    return 0;
}
