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

// Fill f_k, pi_k ([nflds][N][N][N/2+1] interleaved complex, FP64) and, when
// p.with_gw, u_k, pi_u_k (6 symmetric components) exactly as the reference's
// initialize() and initialize_GW() do. The buffers must be zero-initialised
// by the caller (modes the reference never writes stay zero).
ICInfo generate_ic(const psc_params &p, double *f_k, double *pi_k, double *u_k, double *pi_u_k);

}  // namespace psc
