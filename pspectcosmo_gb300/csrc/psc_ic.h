// psc_ic.h — host-side initial-condition generator (see psc_ic.cpp).
#pragma once

#include "../../include/psc.h"

namespace psc {

struct ICInfo {
    double hubble_init;   // initial Hubble rate (initialize.cpp:656-660)
    double a, ad;         // a0 and hubble_init * a0
    double add_printed;   // the pre-lattice a'' printed by initialize() (initialize.cpp:667)
    double kinetic;       // sum of field derivatives squared / 2 (initialize.cpp:653)
    double potential;     // potential of the homogeneous fields (initialize.cpp:654)
};

// The constants of a run's initial conditions, shared by the host generator and the
// device generator (psc_ic_gpu.cu): the homogeneous background (initialize.cpp:636-670),
// the mode normalisations (parameters.h:132, initialize.cpp:128-220, 273-340) and the
// layout of the reference's random stream over the mode traversal.
struct ICSetup {
    ICInfo info;
    int N, H, nf, model, alpha, simulate_inflation, gw;
    double fStar, omegaStar, dx, DFDP, a, hubble, aop, k2c, dp2, kIR, gsq;
    double norm_s;       // sqrt(DFDP): scalar mode amplitude factor
    double norm_gw;      // MPl omegaStar / fStar^2 (N/dx)^1.5: GW mode amplitude factor
    double n3;
    double m2[PSC_MAX_FIELDS], f0[PSC_MAX_FIELDS], fd0[PSC_MAX_FIELDS];
    int seed;
    long long visits;    // modes visited per scalar field (initialize.cpp:686-749)
    int dpm;             // draws per scalar mode: 1 (fixed amplitude) or 4 (Rayleigh)
};
ICSetup ic_setup(const psc_params &p);

// The same initial conditions generated on the device into realization r of a handle
// (psc_ic_gpu.cu): one thread per mode, draws by skip-ahead in the reference's stream.
// Needs seed >= 1 and no initial low-pass cut (kcutoff, which changes how many draws
// a mode takes).
int ic_device(psc_handle *h, int r, ICInfo *info);

// Fill f_k, pi_k ([nflds][N][N][N/2+1] interleaved complex, FP64) and, when
// p.with_gw, u_k, pi_u_k (6 symmetric components) exactly as the reference's
// initialize() and initialize_GW() do. The buffers must be zero-initialised
// by the caller (modes the reference never writes stay zero).
ICInfo generate_ic(const psc_params &p, double *f_k, double *pi_k, double *u_k, double *pi_u_k);

}  // namespace psc
