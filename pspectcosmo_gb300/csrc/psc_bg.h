// psc_bg.h — the FP64 background record shared by host and device code.
#pragma once

namespace psc {

constexpr int kMaxStages = 31;   // Yoshida-10 (pspectcosmo.h:295-297)
constexpr int kMaxFields = 4;   // PSC_MAX_FIELDS
constexpr int kMaxTerms = 4;    // PSC_MAX_TERMS

// FP64 background and per-stage coefficients, resident in device memory so a
// captured step graph needs no host values. Mirrors the reference globals
// a, ad, add, t (pspectcosmo.cpp:155-156) and the locals b, b_half, a_half of
// evolve_VV_k_nopad (evolution.cpp:1131-1198).
struct DevBG {
    double a, ad, add, t;           // state at step boundaries
    double b, b_half;               // within a step (b = a' during the stages)
    double ad_stale;                // ad at the start of the step: the R_Q2C mask reads the stale global ad
    double dt;
    double c_drift;                 // w dt a_half^(alpha-3)            (evolution.cpp:1164-1168)
    double c_close, c_open;         // closing / next opening half kick  (evolution.cpp:1153-1158, 1184-1189)
    double norm1, norm2;            // a^(1+alpha), a^(3+alpha)          (evolution.cpp:1099-1100)
    double hub, apow, a3;           // ad_stale/a, a^(alpha-3), a^(3-alpha) for R_Q2C (evolution.cpp:1047)
    double K[kMaxFields], G[kMaxFields], V[kMaxTerms];   // last reductions (kinetic, gradient, potential)
    double w[kMaxStages];
    // run constants
    double kIR, kIR2, DFDP, eps, fs_over_mpl2, gsq, inv_n3, inv_n3sq;
    double inv_nv;                  // 1 / (sites the <V> partials sum over): N^3, or N_pad^3 when padded
    int s, alpha, nf, nterms, mask, model, nbx, nbz;   // nbz: blocks of the <V> partials
    int stage, steps_left, err, pad;
    // bounded device-side waits: the limit of one wait (1 s unless a test sets it), and a
    // test hook: bytes every staged tile of pass wait_plant_pass (PSC_NPASS order: 0 X
    // inverse, 1 Y inverse, 2 Z, 3 Y forward, 4 X forward) is told to expect that no copy
    // delivers, so its wait runs out after the real copies have landed (0 = off)
    unsigned long long wait_ns;
    int wait_plant, fp32;           // fp32: the handle's arrays hold FP32 values
    int wait_plant_pass, pad2;
    // FP64 shadow of each field's homogeneous mode f_k(0), pi_k(0) (re, im). The background
    // kernel evolves it (drift when a stage begins, the kicks after the kick pass) and writes
    // its rounding into the arrays, which every other kernel reads as before. Stored in FP32
    // and re-rounded by each kick, the homogeneous mode random-walks: at 256^3 two-field
    // preheating a(t) drifted 7.6e-7 from FP64 over 4000 steps and shifted the phases of the
    // highest GW modes (3e-4 in hdot^2); with the mode pinned to FP64, 4e-8 and 3e-5.
    double z0f[kMaxFields][2], z0p[kMaxFields][2];
    double z0q[kMaxFields][2];      // the zero mode of V'_k as the last kick pass read it
    double z0F[kMaxFields][2];      // the zero mode's force at the last synchronising kick
    int zero64;                     // 1 when the shadow holds the state (set with the state)
    int z0pending;                  // 1 after a kick pass, until the background kernel kicks
};

// Scalar state of the discrete adjoint (psc_adjoint.cu), resident in device memory
// so the reverse sweep needs no host round trip: the adjoints of a, b = a', a''
// and of the couplings, and the coefficients the array kernels of the current
// lattice point (point) or stage (stage) read.
struct DevAdj {
    double la, lb, ladd, lbh, lat;
    double gth[2];
    // point: M = alpha1 Lp + alpha2 p; Lp += beta p;
    //        Lf += J^T-part (eta1 k^2 M, eta2 V''(f) m) + gamma V'(f) + delta k^2 f
    double alpha1, alpha2, beta, gamma, delta, eta1, eta2;
    // stage: ph = p + kc (-kn1 k^2 f - kn2 Vp); Lp += c2 Lf
    double c2, kc, kn1, kn2;
    // GW: transposed source factor -a^(1+alpha) (point), pi_u_half = pi_u + kfu Fu (stage)
    double etaS, kfu;
    double O;
};

}  // namespace psc
