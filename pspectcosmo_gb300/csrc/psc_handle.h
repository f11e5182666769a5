// psc_handle.h — the lattice handle shared by the C-ABI layer (psc_api.cu) and
// the adjoint (psc_adjoint.cu) and the output quantities (psc_outputs.cu).
// Private to the library.
#pragma once

#include <string>
#include <vector>

#include "../../include/psc.h"
#include "psc_bg.h"
#include "psc_launch.h"

struct psc_handle {
    std::vector<psc_params> p;   // per realization (identical except seed / initial values)
    int R = 1;
    psc::LaunchCfg cfg{};
    psc::Buffers b{};
    size_t csize = 0;            // bytes of one complex element on the device
    int s = 1;
    const double *w = nullptr;   // Yoshida weights
    int nb = 0;                  // maxnumbins
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t gexec = nullptr;
    bool have_state = false;
    // the kept force (b.Fk, b.Fu) is that of the current state: the last call was a step
    // call that ended with a synchronising kick and nothing has changed the state since
    bool force_valid = false;
    bool diag_valid = false;
    float last_ms = 0.f;
    void *stage_buf = nullptr;   // pinned staging for precision conversion
    size_t stage_bytes = 0;
    double *xfer = nullptr;      // device FP64 scratch of the FP32 upload (one chunk)
    size_t xfer_elems = 0;
    std::vector<void *> allocs;
    size_t partKG_cap = 0, partV_cap = 0;   // doubles held by b.partKG, b.partV (the autotuner may grow them)
    psc::XTma xtma{};            // tensor maps of the X forward + kick operands (b.xtma points here when on)
    psc::YTma ytma{};            // tensor maps of the Y forward tiles (b.ytma points here when on)
    psc::YTma ytma_i{};          // tensor maps of the GW Y inverse tiles (b.ytma_i)
    int tmap_mask = PSC_TMAP_X | PSC_TMAP_Y;   // passes allowed to stage their tiles by tensor maps
    void *adj = nullptr;         // adjoint workspace (psc_adjoint.cu), owned by the handle
    void (*adj_free)(void *) = nullptr;
    void *ana = nullptr;         // analytic pre-lattice phase (psc_analytic.cu), owned by the handle
    void (*ana_free)(void *) = nullptr;
    // padded step (N_pad > 0): the launch configuration and buffers of the N_pad grid
    // (fk = padded spectra, TA, QV = transform intermediates, tw = N_pad twiddles)
    bool padded = false;
    psc::LaunchCfg cfgp{};
    psc::Buffers bp{};
    const psc_params &p0() const { return p[0]; }
};

namespace psc {
namespace hapi {
int fail(int code, const std::string &msg);
void encode_xtma(psc_handle *h);
int dalloc(psc_handle *h, void **out, size_t bytes);
int upload(psc_handle *h, void *dst, const double *src, size_t ncplx);
int download_real(psc_handle *h, double *dst, const void *src, size_t count);
int read_bg(psc_handle *h, int r, DevBG *out);
int write_bg(psc_handle *h, int r, const DevBG &in);
int step(psc_handle *h, double dt, int nsteps);
int evaluate(psc_handle *h, int keep_add);
Buffers buffers_of(psc_handle *h, int r);
int set_state(psc_handle *h, int r, const double *f_k, const double *pi_k, double a, double ad, double add,
              const double *u_k, const double *pi_u_k);
int get_state(psc_handle *h, int r, double *f_k, double *pi_k, double *a, double *ad, double *add, double *u_k,
              double *pi_u_k);
LaunchCfg single_cfg(psc_handle *h);
// psc_outputs.cu: histograms and snapshot datasets of realization r
int histograms(psc_handle *h, int r, int nbins, double hmin, double hmax, double *binfreq, double *bmin, double *df);
int snapshot_arrays(psc_handle *h, int r, double *f, double *pot, double *kin, double *grad, double *tot);
int write_snapshot(psc_handle *h, int r, const char *path, int with_energy);
}  // namespace hapi
}  // namespace psc
