// psc_api.cu — the C ABI (include/psc.h): one handle per lattice, device
// buffers, the captured step graph, host<->device state transfer and outputs.
// Host code only; the kernels live in psc_kernels.cu.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/psc.h"
#include "psc_bg.h"
#include "psc_ic.h"
#include "psc_launch.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define CU(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return fail(e_ == cudaErrorMemoryAllocation ? PSC_ERR_NOMEM : PSC_ERR_CUDA,                  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                             \
    } while (0)

// Yoshida composition weights (pspectcosmo.h:283-297): published coefficient
// tables, kept digit for digit so the stages equal the reference's.
const double kW2[1] = {1.};
const double kW4[3] = {1.351207191959657771818, -1.702414403875838200264, 1.351207191959657771818};
const double kW6[7] = {0.78451361047755726382, 0.23557321335935813368, -1.1776799841788710069, 1.3151863206839112189,
                       -1.1776799841788710069, 0.23557321335935813368, 0.78451361047755726382};
const double kW8[15] = {0.74167036435061295345, -0.40910082580003159400, 0.19075471029623837995,
                        -0.57386247111608226666, 0.29906418130365592384, 0.33462491824529818378,
                        0.31529309239676659663, -0.79688793935291635402, 0.31529309239676659663,
                        0.33462491824529818378, 0.29906418130365592384, -0.57386247111608226666,
                        0.19075471029623837995, -0.40910082580003159400, 0.74167036435061295345};
const double kW10[31] = {
    -0.48159895600253002870, 0.0036303931544595926879, 0.50180317558723140279, 0.28298402624506254868,
    0.80702967895372223806,  -0.026090580538592205447, -0.87286590146318071547, -0.52373568062510581643,
    0.44521844299952789252,  0.18612289547097907887,   0.23137327866438360633, -0.52191036590418628905,
    0.74866113714499296793,  0.066736511890604057532,  -0.80360324375670830316, 0.91249037635867994571,
    -0.80360324375670830316, 0.066736511890604057532,  0.74866113714499296793, -0.52191036590418628905,
    0.23137327866438360633,  0.18612289547097907887,   0.44521844299952789252, -0.52373568062510581643,
    -0.87286590146318071547, -0.026090580538592205447, 0.80702967895372223806, 0.28298402624506254868,
    0.50180317558723140279,  0.0036303931544595926879, -0.48159895600253002870};

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

}  // namespace

void psc::set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }

struct psc_handle {
    psc_params p{};
    psc::LaunchCfg cfg{};
    psc::Buffers b{};
    size_t csize = 0;   // bytes of one complex element on the device
    int s = 1;
    const double *w = kW2;
    int nb = 0;         // maxnumbins
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t gexec = nullptr;
    bool have_state = false;
    bool diag_valid = false;
    float last_ms = 0.f;
    void *stage_buf = nullptr;    // pinned staging for precision conversion
    size_t stage_bytes = 0;
    std::vector<void *> allocs;
};

namespace {

void free_all(psc_handle *h) {
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    for (void *q : h->allocs) cudaFree(q);
    h->allocs.clear();
    if (h->stage_buf) cudaFreeHost(h->stage_buf);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->st) cudaStreamDestroy(h->st);
}

int dalloc(psc_handle *h, void **out, size_t bytes) {
    *out = nullptr;
    if (bytes == 0) return PSC_OK;
    CU(cudaMalloc(out, bytes));
    h->allocs.push_back(*out);
    return PSC_OK;
}

int validate(const psc_params *p) {
    if (!p) return fail(PSC_ERR_ARG, "null parameters");
    if (!pow2(p->N) || p->N < 8 || p->N > 1024) return fail(PSC_ERR_CONFIG, "N must be a power of two in [8, 1024]");
    if (p->nflds < 1 || p->nflds > 2) return fail(PSC_ERR_CONFIG, "nflds must be 1 or 2");
    if (p->model == PSC_MODEL_PHI2 && p->nflds != 1) return fail(PSC_ERR_CONFIG, "the phi^2 model has one field");
    if (p->model == PSC_MODEL_PHI2CHI2 && p->nflds != 2) return fail(PSC_ERR_CONFIG, "the phi^2 chi^2 model has two fields");
    if (p->model != PSC_MODEL_PHI2 && p->model != PSC_MODEL_PHI2CHI2) return fail(PSC_ERR_CONFIG, "unknown model");
    if (p->vv != 2 && p->vv != 4 && p->vv != 6 && p->vv != 8 && p->vv != 10)
        return fail(PSC_ERR_CONFIG, "vv must be 2, 4, 6, 8 or 10");
    if (p->precision != 32 && p->precision != 64) return fail(PSC_ERR_CONFIG, "precision must be 32 or 64");
    if (p->with_gw && p->spectral)
        return fail(PSC_ERR_CONFIG, "GWs are evolved on the real-space path only (spectral = 0), as in the reference");
    if (p->expansion < 0 || p->expansion > 2) return fail(PSC_ERR_CONFIG, "expansion must be 0, 1 or 2");
    if (!(p->kIR > 0) || !(p->MPl > 0) || !(p->m_in_MPl > 0) || !(p->a0 > 0))
        return fail(PSC_ERR_CONFIG, "kIR, MPl, m_in_MPl and a0 must be positive");
    return PSC_OK;
}

int ensure_staging(psc_handle *h, size_t bytes) {
    if (h->stage_bytes >= bytes) return PSC_OK;
    if (h->stage_buf) cudaFreeHost(h->stage_buf);
    h->stage_buf = nullptr;
    h->stage_bytes = 0;
    CU(cudaMallocHost(&h->stage_buf, bytes));
    h->stage_bytes = bytes;
    return PSC_OK;
}

// host FP64 complex -> device array of the handle's precision
int upload(psc_handle *h, void *dst, const double *src, size_t ncplx) {
    if (h->p.precision == 64) {
        CU(cudaMemcpyAsync(dst, src, ncplx * 16, cudaMemcpyHostToDevice, h->st));
        CU(cudaStreamSynchronize(h->st));
        return PSC_OK;
    }
    int rc = ensure_staging(h, ncplx * 8);
    if (rc) return rc;
    float *f = static_cast<float *>(h->stage_buf);
    for (size_t i = 0; i < 2 * ncplx; ++i) f[i] = (float)src[i];
    CU(cudaMemcpyAsync(dst, f, ncplx * 8, cudaMemcpyHostToDevice, h->st));
    CU(cudaStreamSynchronize(h->st));
    return PSC_OK;
}

// device array of the handle's precision -> host FP64 (count scalars)
int download_real(psc_handle *h, double *dst, const void *src, size_t count) {
    if (h->p.precision == 64) {
        CU(cudaMemcpyAsync(dst, src, count * 8, cudaMemcpyDeviceToHost, h->st));
        CU(cudaStreamSynchronize(h->st));
        return PSC_OK;
    }
    int rc = ensure_staging(h, count * 4);
    if (rc) return rc;
    CU(cudaMemcpyAsync(h->stage_buf, src, count * 4, cudaMemcpyDeviceToHost, h->st));
    CU(cudaStreamSynchronize(h->st));
    const float *f = static_cast<const float *>(h->stage_buf);
    for (size_t i = 0; i < count; ++i) dst[i] = (double)f[i];
    return PSC_OK;
}

int read_bg(psc_handle *h, psc::DevBG *out) {
    CU(cudaMemcpyAsync(out, h->b.bg, sizeof(psc::DevBG), cudaMemcpyDeviceToHost, h->st));
    CU(cudaStreamSynchronize(h->st));
    return PSC_OK;
}

int write_bg(psc_handle *h, const psc::DevBG &in) {
    CU(cudaMemcpyAsync(h->b.bg, &in, sizeof(psc::DevBG), cudaMemcpyHostToDevice, h->st));
    CU(cudaStreamSynchronize(h->st));
    return PSC_OK;
}

// pure evaluation of the force pipeline: K, G, V and (keep_add = 0) a''
int evaluate(psc_handle *h, int keep_add) {
    CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_EVAL, 0, h->st));
    CU(psc::launch_stage(h->cfg, h->b, h->p.precision, 0, h->st));
    CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_EVAL_END, keep_add, h->st));
    CU(cudaStreamSynchronize(h->st));
    h->diag_valid = true;
    return PSC_OK;
}

int build_graph(psc_handle *h) {
    if (h->gexec) return PSC_OK;
    cudaGraph_t graph = nullptr;
    CU(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    for (int p = 0; p < h->s && err == cudaSuccess; ++p) {
        err = psc::launch_stage(h->cfg, h->b, h->p.precision, 1, h->st);
        if (err == cudaSuccess) err = psc::launch_scalar(h->cfg, h->b, psc::SCALAR_END, p, h->st);
    }
    cudaError_t e2 = cudaStreamEndCapture(h->st, &graph);
    if (err != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(PSC_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(err));
    }
    if (e2 != cudaSuccess) return fail(PSC_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(e2));
    cudaError_t e3 = cudaGraphInstantiate(&h->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e3 != cudaSuccess) {
        h->gexec = nullptr;
        return fail(PSC_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
    }
    return PSC_OK;
}

}  // namespace

extern "C" {

void psc_default_params(psc_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->N = 64;
    p->nflds = 1;
    p->vv = 2;
    p->alpha = 0;
    p->expansion = 2;
    p->simulate_inflation = 1;
    p->spectral = 1;
    p->with_gw = 0;
    p->precision = 64;
    p->model = PSC_MODEL_PHI2;
    p->seed = 1;
    p->kIR = 25.;
    p->a0 = 1.;
    p->MPl = 1.;
    p->m_in_MPl = 1.e-6;
    p->fStar = 1.;
    p->epsilon = 1.e-3;
    p->gsq = 0.;
    p->initfield[0] = 11. * p->MPl;
    p->initderivs[0] = -0.815284e-6 * p->MPl * p->MPl;
    p->kcutoff = 0.;
}

int psc_maxnumbins(int N) { return (int)(std::sqrt(3.0) * (N / 2)) + 2; }

int psc_create(const psc_params *p, psc_handle **out) {
    if (!out) return fail(PSC_ERR_ARG, "null output handle");
    *out = nullptr;
    int rc = validate(p);
    if (rc) return rc;
    psc_handle *h = new (std::nothrow) psc_handle();
    if (!h) return fail(PSC_ERR_NOMEM, "host allocation failed");
    h->p = *p;
    if (h->p.fStar <= 0) h->p.fStar = h->p.MPl;
    switch (p->vv) {
    case 4: h->s = 3; h->w = kW4; break;
    case 6: h->s = 7; h->w = kW6; break;
    case 8: h->s = 15; h->w = kW8; break;
    case 10: h->s = 31; h->w = kW10; break;
    default: h->s = 1; h->w = kW2;
    }
    h->csize = p->precision == 32 ? 8 : 16;
    h->nb = psc_maxnumbins(p->N);
    psc::plan(h->p, &h->cfg);
    const psc::Geo &g = h->cfg.g;
    auto bail = [&](int code) {
        free_all(h);
        delete h;
        return code;
    };
#define CUB(call)                                                                                      \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return bail(fail(e_ == cudaErrorMemoryAllocation ? PSC_ERR_NOMEM : PSC_ERR_CUDA,           \
                             std::string(#call) + ": " + cudaGetErrorString(e_)));                     \
    } while (0)
    CUB(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    CUB(cudaEventCreate(&h->ev0));
    CUB(cudaEventCreate(&h->ev1));
    CUB(psc::configure(h->cfg, p->precision));
    const size_t arr = (size_t)g.modes * h->csize;
    const int nf = g.nf;
    psc::Buffers &b = h->b;
    if ((rc = dalloc(h, &b.fk, nf * arr)) || (rc = dalloc(h, &b.pk, nf * arr)) || (rc = dalloc(h, &b.TA, nf * arr)) ||
        (rc = dalloc(h, &b.QV, nf * arr)))
        return bail(rc);
    if (g.gw) {
        if ((rc = dalloc(h, &b.uk, 6 * arr)) || (rc = dalloc(h, &b.puk, 6 * arr)) || (rc = dalloc(h, &b.TB, nf * arr)) ||
            (rc = dalloc(h, &b.TC, nf * arr)) || (rc = dalloc(h, &b.QS, 6 * arr)))
            return bail(rc);
    }
    void *tmp = nullptr;
    if ((rc = dalloc(h, &b.tw, (size_t)g.N * h->csize))) return bail(rc);
    if ((rc = dalloc(h, &tmp, sizeof(double) * 2 * psc::kMaxFields * h->cfg.nbx))) return bail(rc);
    b.partKG = static_cast<double *>(tmp);
    if ((rc = dalloc(h, &tmp, sizeof(double) * psc::kMaxTerms * h->cfg.nbz))) return bail(rc);
    b.partV = static_cast<double *>(tmp);
    if ((rc = dalloc(h, &tmp, sizeof(double) * (nf * 3 + 2) * h->nb))) return bail(rc);
    b.spec = static_cast<double *>(tmp);
    if ((rc = dalloc(h, &tmp, sizeof(int) * (nf + 1) * h->nb))) return bail(rc);
    b.spec_cnt = static_cast<int *>(tmp);
    if ((rc = dalloc(h, &tmp, sizeof(psc::DevBG)))) return bail(rc);
    b.bg = static_cast<psc::DevBG *>(tmp);
    CUB(cudaMemsetAsync(b.fk, 0, nf * arr, h->st));
    CUB(cudaMemsetAsync(b.pk, 0, nf * arr, h->st));
    if (g.gw) {
        CUB(cudaMemsetAsync(b.uk, 0, 6 * arr, h->st));
        CUB(cudaMemsetAsync(b.puk, 0, 6 * arr, h->st));
    }
    // twiddles e^{-2 pi i q/N} from FP64 sin/cos
    {
        std::vector<double> tw(2 * g.N);
        for (int q = 0; q < g.N; ++q) {
            const double ang = 2.0 * 3.14159265358979323846 * (double)q / (double)g.N;
            tw[2 * q] = std::cos(ang);
            tw[2 * q + 1] = -std::sin(ang);
        }
        if ((rc = upload(h, b.tw, tw.data(), g.N))) return bail(rc);
    }
    psc::DevBG bg{};
    bg.a = h->p.a0;
    bg.s = h->s;
    for (int i = 0; i < h->s; ++i) bg.w[i] = h->w[i];
    bg.alpha = p->alpha;
    bg.nf = nf;
    bg.nterms = g.nterms;
    bg.mask = g.mask;
    bg.model = p->model;
    bg.nbx = h->cfg.nbx;
    bg.nbz = h->cfg.nbz;
    bg.kIR = p->kIR;
    bg.kIR2 = p->kIR * p->kIR;
    {
        const double fStar = h->p.fStar, omegaStar = p->m_in_MPl * fStar;
        const double L = 2 * 3.14159265358979323846 / p->kIR, dx = L / (double)p->N;
        bg.DFDP = std::pow(omegaStar / fStar, 2) * (p->N / dx) / 2.;   // parameters.h:132
        bg.fs_over_mpl2 = (fStar / p->MPl) * (fStar / p->MPl);
    }
    bg.eps = p->epsilon;
    bg.gsq = p->gsq;
    bg.inv_n3 = 1.0 / (double)g.sites;
    bg.inv_n3sq = bg.inv_n3 * bg.inv_n3;
    if ((rc = write_bg(h, bg))) return bail(rc);
#undef CUB
    *out = h;
    return PSC_OK;
}

void psc_destroy(psc_handle *h) {
    if (!h) return;
    cudaStreamSynchronize(h->st);
    free_all(h);
    delete h;
}

int psc_init_ic(psc_handle *h) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    const psc::Geo &g = h->cfg.g;
    const size_t n = (size_t)g.modes;
    std::vector<double> fk(2 * n * g.nf, 0.0), pk(2 * n * g.nf, 0.0), uk, puk;
    if (g.gw) {
        uk.assign(2 * n * 6, 0.0);
        puk.assign(2 * n * 6, 0.0);
    }
    psc::ICInfo info = psc::generate_ic(h->p, fk.data(), pk.data(), g.gw ? uk.data() : nullptr,
                                        g.gw ? puk.data() : nullptr);
    int rc;
    if ((rc = upload(h, h->b.fk, fk.data(), n * g.nf)) || (rc = upload(h, h->b.pk, pk.data(), n * g.nf))) return rc;
    if (g.gw && ((rc = upload(h, h->b.uk, uk.data(), n * 6)) || (rc = upload(h, h->b.puk, puk.data(), n * 6))))
        return rc;
    psc::DevBG bg;
    if ((rc = read_bg(h, &bg))) return rc;
    bg.a = info.a;
    bg.ad = info.ad;
    bg.add = info.add_printed;
    bg.t = 0.0;
    bg.err = 0;
    if ((rc = write_bg(h, bg))) return rc;
    h->have_state = true;
    // initialize() ends with add = kernel_a_k_nopad() / kernel_a() (initialize.cpp:786-797)
    return evaluate(h, 0);
}

int psc_generate_ic(const psc_params *p, double *f_k, double *pi_k, double *u_k, double *pi_u_k, double *info) {
    int rc = validate(p);
    if (rc) return rc;
    if (!f_k || !pi_k || (p->with_gw && (!u_k || !pi_u_k))) return fail(PSC_ERR_ARG, "null output buffer");
    psc_params q = *p;
    if (q.fStar <= 0) q.fStar = q.MPl;
    const size_t n = (size_t)q.N * q.N * (q.N / 2 + 1);
    std::memset(f_k, 0, sizeof(double) * 2 * n * q.nflds);
    std::memset(pi_k, 0, sizeof(double) * 2 * n * q.nflds);
    if (q.with_gw) {
        std::memset(u_k, 0, sizeof(double) * 2 * n * 6);
        std::memset(pi_u_k, 0, sizeof(double) * 2 * n * 6);
    }
    psc::ICInfo ii = psc::generate_ic(q, f_k, pi_k, q.with_gw ? u_k : nullptr, q.with_gw ? pi_u_k : nullptr);
    if (info) {
        info[0] = ii.hubble_init;
        info[1] = ii.a;
        info[2] = ii.ad;
        info[3] = ii.add_printed;
        info[4] = ii.kinetic;
        info[5] = ii.potential;
    }
    return PSC_OK;
}

int psc_set_state(psc_handle *h, const double *f_k, const double *pi_k, double a, double ad, double add,
                  const double *u_k, const double *pi_u_k) {
    if (!h || !f_k || !pi_k) return fail(PSC_ERR_ARG, "null argument");
    const psc::Geo &g = h->cfg.g;
    if (g.gw && (!u_k || !pi_u_k)) return fail(PSC_ERR_ARG, "GW run needs u_k and pi_u_k");
    const size_t n = (size_t)g.modes;
    int rc;
    if ((rc = upload(h, h->b.fk, f_k, n * g.nf)) || (rc = upload(h, h->b.pk, pi_k, n * g.nf))) return rc;
    if (g.gw && ((rc = upload(h, h->b.uk, u_k, n * 6)) || (rc = upload(h, h->b.puk, pi_u_k, n * 6)))) return rc;
    psc::DevBG bg;
    if ((rc = read_bg(h, &bg))) return rc;
    bg.a = a;
    bg.ad = ad;
    bg.add = add;
    bg.err = 0;
    if ((rc = write_bg(h, bg))) return rc;
    h->have_state = true;
    h->diag_valid = false;
    return PSC_OK;
}

int psc_get_state(psc_handle *h, double *f_k, double *pi_k, double *a, double *ad, double *add, double *u_k,
                  double *pi_u_k) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    const psc::Geo &g = h->cfg.g;
    const size_t n = (size_t)g.modes;
    int rc;
    if (f_k && (rc = download_real(h, f_k, h->b.fk, 2 * n * g.nf))) return rc;
    if (pi_k && (rc = download_real(h, pi_k, h->b.pk, 2 * n * g.nf))) return rc;
    if (g.gw) {
        if (u_k && (rc = download_real(h, u_k, h->b.uk, 2 * n * 6))) return rc;
        if (pi_u_k && (rc = download_real(h, pi_u_k, h->b.puk, 2 * n * 6))) return rc;
    }
    psc::DevBG bg;
    if ((rc = read_bg(h, &bg))) return rc;
    if (a) *a = bg.a;
    if (ad) *ad = bg.ad;
    if (add) *add = bg.add;
    return PSC_OK;
}

int psc_get_time(psc_handle *h, double *t) {
    if (!h || !t) return fail(PSC_ERR_ARG, "null argument");
    psc::DevBG bg;
    int rc = read_bg(h, &bg);
    if (rc) return rc;
    *t = bg.t;
    return PSC_OK;
}

int psc_set_time(psc_handle *h, double t) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    psc::DevBG bg;
    int rc = read_bg(h, &bg);
    if (rc) return rc;
    bg.t = t;
    return write_bg(h, bg);
}

int psc_step(psc_handle *h, double dt, int nsteps) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state: call psc_init_ic or psc_set_state first");
    if (nsteps < 0 || !(dt > 0) || !std::isfinite(dt)) return fail(PSC_ERR_ARG, "need dt > 0 and nsteps >= 0");
    if (nsteps == 0) return PSC_OK;
    int rc = build_graph(h);
    if (rc) return rc;
    CU(cudaEventRecord(h->ev0, h->st));
    CU(psc::launch_set_run(h->b.bg, dt, nsteps, h->st));
    // opening half kick: pi_half = pi + w0 dt/2 F(f, a)  (evolution.cpp:1144-1158, stage 0)
    CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_PRIME, 0, h->st));
    CU(psc::launch_stage(h->cfg, h->b, h->p.precision, 0, h->st));
    CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_BEGIN, 0, h->st));
    for (int i = 0; i < nsteps; ++i) CU(cudaGraphLaunch(h->gexec, h->st));
    CU(cudaEventRecord(h->ev1, h->st));
    int err = 0;
    CU(cudaMemcpyAsync(&err, &h->b.bg->err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CU(cudaStreamSynchronize(h->st));
    CU(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
    h->diag_valid = true;
    if (err) return fail(err, "non-finite background (NaN/Inf in a, a' or a'') during the step");
    return PSC_OK;
}

int psc_last_step_ms(psc_handle *h, float *ms) {
    if (!h || !ms) return fail(PSC_ERR_ARG, "null argument");
    *ms = h->last_ms;
    return PSC_OK;
}

int psc_time_passes(psc_handle *h, int reps, float *ms) {
    if (!h || !ms || reps < 1) return fail(PSC_ERR_ARG, "bad argument");
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state");
    cudaEvent_t ev[7];
    for (int i = 0; i < 7; ++i) CU(cudaEventCreate(&ev[i]));
    double acc[PSC_NPASS] = {0, 0, 0, 0, 0, 0};
    // zero-length kicks: the state is unchanged; a'' is kept (diagnostics mode)
    for (int r = 0; r < reps; ++r) {
        CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_EVAL, 0, h->st));
        CU(psc::launch_stage_timed(h->cfg, h->b, h->p.precision, 0, psc::SCALAR_EVAL_END, ev, h->st));
        CU(cudaEventSynchronize(ev[6]));
        for (int i = 0; i < PSC_NPASS; ++i) {
            float t = 0.f;
            CU(cudaEventElapsedTime(&t, ev[i], ev[i + 1]));
            acc[i] += t;
        }
    }
    for (int i = 0; i < 7; ++i) cudaEventDestroy(ev[i]);
    for (int i = 0; i < PSC_NPASS; ++i) ms[i] = (float)(acc[i] / reps);
    h->diag_valid = true;
    return PSC_OK;
}

int psc_pass_bytes(psc_handle *h, double *bytes) {
    if (!h || !bytes) return fail(PSC_ERR_ARG, "bad argument");
    const psc::Geo &g = h->cfg.g;
    const double C = (double)g.modes * h->csize, R = (double)g.sites * (h->csize / 2);
    const int nf = g.nf, gw = g.gw;
    (void)R;
    // X inverse: read f_k, pi_half; write f_k, TA [, TB]
    bytes[0] = nf * (4 + gw) * C;
    // Y inverse: read TA [, TB]; write TA [, TB, TC]
    bytes[1] = nf * (gw ? 5 : 2) * C;
    // fused Z: read TA [, TB, TC]; write QV [, QS]
    bytes[2] = (nf * (gw ? 3 : 1) + nf + (gw ? 6 : 0)) * C;
    // Y forward: in place over QV [, QS]
    bytes[3] = 2.0 * (nf + (gw ? 6 : 0)) * C;
    // X forward + kick: read QV, f_k, pi; write pi [; read QS, u, pi_u; write u, pi_u]
    bytes[4] = (4.0 * nf + (gw ? 6 * 5 : 0)) * C;
    bytes[5] = 0.0;
    return PSC_OK;
}

int psc_get_fields_real(psc_handle *h, double *f, double *pi_f) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    const psc::Geo &g = h->cfg.g;
    const size_t rsize = h->csize / 2;
    int rc;
    if (!h->b.real && (rc = dalloc(h, &h->b.real, (size_t)g.sites * g.nf * rsize))) return rc;
    if (f) {
        CU(psc::launch_c2r_real(h->cfg, h->b, h->p.precision, h->b.fk, g.nf, h->st));
        if ((rc = download_real(h, f, h->b.real, (size_t)g.sites * g.nf))) return rc;
    }
    if (pi_f) {
        CU(psc::launch_c2r_real(h->cfg, h->b, h->p.precision, h->b.pk, g.nf, h->st));
        if ((rc = download_real(h, pi_f, h->b.real, (size_t)g.sites * g.nf))) return rc;
    }
    return PSC_OK;
}

int psc_spectra(psc_handle *h, int32_t *numpoints, double *f2, double *pi2, double *n2, int32_t *gw_numpoints,
                double *h2, double *hdot2, double *hdot2_zero) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    const psc::Geo &g = h->cfg.g;
    const int nb = h->nb, nf = g.nf;
    CU(psc::launch_spectra(h->cfg, h->b, h->p.precision, nb, h->st));
    std::vector<double> acc((size_t)(nf * 3 + 2) * nb);
    std::vector<int> cnt((size_t)(nf + 1) * nb);
    CU(cudaMemcpyAsync(acc.data(), h->b.spec, acc.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CU(cudaMemcpyAsync(cnt.data(), h->b.spec_cnt, cnt.size() * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CU(cudaStreamSynchronize(h->st));
    for (int f = 0; f < nf; ++f)
        for (int l = 0; l < nb; ++l) {
            const int c = cnt[(size_t)f * nb + l];
            const double d = c > 0 ? (double)c : 1.0;
            if (numpoints) numpoints[(size_t)f * nb + l] = c;
            if (f2) f2[(size_t)f * nb + l] = acc[(size_t)f * 3 * nb + l] / d;
            if (pi2) pi2[(size_t)f * nb + l] = acc[(size_t)f * 3 * nb + nb + l] / d;
            if (n2) n2[(size_t)f * nb + l] = acc[(size_t)f * 3 * nb + 2 * nb + l] / d;
        }
    if (g.gw) {
        const double *H = acc.data() + (size_t)nf * 3 * nb, *D = H + nb;
        const int *C = cnt.data() + (size_t)nf * nb;
        for (int l = 0; l < nb; ++l) {
            const double d = (C[l] > 0 && l >= 1) ? (double)C[l] : 1.0;
            if (gw_numpoints) gw_numpoints[l] = C[l];
            if (h2) h2[l] = H[l] / d;
            if (hdot2) hdot2[l] = D[l] / d;
        }
        if (hdot2_zero) {
            // |pi_u_k(0)|^2 over the nine components (output.cpp:1033-1039)
            double z = 0.0;
            for (int c = 0; c < 6; ++c) {
                double v[2];
                const char *base = static_cast<const char *>(h->b.puk) + (size_t)c * g.modes * h->csize;
                if (h->p.precision == 64) {
                    CU(cudaMemcpy(v, base, 16, cudaMemcpyDeviceToHost));
                } else {
                    float fv[2];
                    CU(cudaMemcpy(fv, base, 8, cudaMemcpyDeviceToHost));
                    v[0] = fv[0];
                    v[1] = fv[1];
                }
                const double mult = (c == 0 || c == 3 || c == 5) ? 1.0 : 2.0;
                z += mult * (v[0] * v[0] + v[1] * v[1]);
            }
            *hdot2_zero = z;
        }
    } else {
        if (hdot2_zero) *hdot2_zero = 0.0;
    }
    return PSC_OK;
}

int psc_energies(psc_handle *h, double *K, double *G, double *V, double *total, double *friedmann_violation,
                 double *rho_gw) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    int rc;
    if (!h->diag_valid && (rc = evaluate(h, 1))) return rc;
    psc::DevBG bg;
    if ((rc = read_bg(h, &bg))) return rc;
    const psc::Geo &g = h->cfg.g;
    double tot = 0.0;
    for (int f = 0; f < g.nf; ++f) {
        if (K) K[f] = bg.K[f];
        if (G) G[f] = bg.G[f];
        tot += bg.K[f];
        tot += bg.G[f];
    }
    for (int t = 0; t < g.nterms; ++t) {
        if (V) V[t] = bg.V[t];
        tot += bg.V[t];
    }
    if (total) *total = tot;
    // energy(), output.cpp:1178-1185
    const double LHS = bg.ad * bg.ad;
    const double RHS = bg.fs_over_mpl2 * std::pow(bg.a, 2 * (h->p.alpha + 1)) * tot / 3.;
    if (friedmann_violation) *friedmann_violation = std::fabs(LHS - RHS) / std::fabs(LHS + RHS);
    if (rho_gw) {
        *rho_gw = 0.0;
        if (g.gw) {
            // output.cpp:1030-1060: zero mode plus the un-normalised bins
            const int nb = h->nb;
            std::vector<int> cnt(nb);
            std::vector<double> hd(nb);
            double hz = 0.0;
            if ((rc = psc_spectra(h, nullptr, nullptr, nullptr, nullptr, cnt.data(), nullptr, hd.data(), &hz)))
                return rc;
            double r = hz;
            for (int l = 1; l < nb; ++l) r += hd[l] * (cnt[l] > 0 ? cnt[l] : 1);
            const double fStar = h->p.fStar, omegaStar = h->p.m_in_MPl * fStar, MPl = h->p.MPl;
            r *= omegaStar * omegaStar * std::pow(fStar, 4) / (MPl * MPl) / 4. * bg.inv_n3sq / std::pow(bg.a, 6);
            r /= (fStar * omegaStar) * (fStar * omegaStar);
            *rho_gw = r;
        }
    }
    return PSC_OK;
}

int psc_means(psc_handle *h, double *out) {
    if (!h || !out) return fail(PSC_ERR_ARG, "null argument");
    const psc::Geo &g = h->cfg.g;
    std::vector<double> f((size_t)g.sites * g.nf), pf((size_t)g.sites * g.nf);
    int rc = psc_get_fields_real(h, f.data(), pf.data());
    if (rc) return rc;
    psc::DevBG bg;
    if ((rc = read_bg(h, &bg))) return rc;
    const double aop = std::pow(bg.a, h->p.alpha - 3);
    const double n = (double)g.sites;
    for (int fl = 0; fl < g.nf; ++fl) {
        double fa = 0, f2 = 0, pa = 0, p2 = 0;
        const double *x = f.data() + (size_t)fl * g.sites, *y = pf.data() + (size_t)fl * g.sites;
        for (long long i = 0; i < g.sites; ++i) {
            fa += x[i];
            f2 += x[i] * x[i];
            pa += y[i];
            p2 += y[i] * y[i];
        }
        fa /= n; f2 /= n; pa /= n; p2 /= n;
        double *o = out + 6 * fl;
        o[0] = fa;
        o[1] = aop * pa;
        o[2] = f2;
        o[3] = aop * aop * p2;
        o[4] = (f2 - fa * fa > 0) ? std::sqrt(f2 - fa * fa) : 0;
        o[5] = (p2 - pa * pa > 0) ? aop * std::sqrt(p2 - pa * pa) : 0;
    }
    return PSC_OK;
}

const char *psc_strerror(int code) {
    switch (code) {
    case PSC_OK: return "ok";
    case PSC_ERR_CONFIG: return "unsupported configuration";
    case PSC_ERR_ARG: return "bad argument";
    case PSC_ERR_CUDA: return "CUDA runtime error";
    case PSC_ERR_NONFINITE: return "non-finite background";
    case PSC_ERR_TIMEOUT: return "device-side wait timed out";
    case PSC_ERR_STATE: return "call out of order";
    case PSC_ERR_NOMEM: return "out of device memory";
    default: return "unknown error";
    }
}

const char *psc_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"
