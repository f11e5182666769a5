// psc_api.cu — the C ABI (include/psc.h): handles, device buffers, the captured
// step graph, host<->device state transfer, outputs, and batches of lattices.
// Host code only; the kernels live in psc_kernels.cu and psc_reg_*.cu.
//
// A handle holds R >= 1 lattices of one configuration ("realizations") laid
// out back to back in every device array; the pass kernels advance all R with
// one launch each (realization = blockIdx.z). psc_create makes R = 1; a batch
// groups its realizations by configuration into such handles and captures all
// of them in one CUDA graph per step.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <thread>
#include <vector>

#ifdef __linux__
#include <sched.h>
#endif

#include <cudaTypedefs.h>

#include "../../include/psc.h"
#include "psc_bg.h"
#include "psc_dev.cuh"
#include "psc_ic.h"
#include "psc_launch.h"

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace psc {
namespace hapi {
int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
}  // namespace hapi
}  // namespace psc
using psc::hapi::fail;

namespace {

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
// n has no prime factor above 7 (the generic engine's radices 2, 3, 5, 7)
bool smooth7(int n) {
    if (n < 1) return false;
    for (int p : {2, 3, 5, 7})
        while (n % p == 0) n /= p;
    return n == 1;
}

constexpr double kPi = 3.14159265358979323846;

}  // namespace

void psc::set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }

#include "psc_handle.h"

namespace psc {
namespace hapi {

void free_all(psc_handle *h) {
    if (h->adj && h->adj_free) h->adj_free(h->adj);
    h->adj = nullptr;
    if (h->ana && h->ana_free) h->ana_free(h->ana);
    h->ana = nullptr;
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    for (void *q : h->allocs) cudaFree(q);
    h->allocs.clear();
    if (h->stage_buf) cudaFreeHost(h->stage_buf);
    if (h->xfer) cudaFree(h->xfer);
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
    // powers of two up to 1024 (the register engine from 32 on); other even sizes up to 512 with
    // prime factors 2, 3, 5, 7 on the generic engine (FFTW, which the reference uses, takes any N)
    if (p->N < 8 || !(pow2(p->N) ? p->N <= 1024 : (p->N % 2 == 0 && smooth7(p->N) && p->N <= 512)))
        return fail(PSC_ERR_CONFIG,
                    "N must be a power of two in [8, 1024] or an even size in [8, 512] with prime factors 2, 3, 5, 7");
    if (p->nflds < 1 || p->nflds > PSC_MAX_FIELDS) return fail(PSC_ERR_CONFIG, "nflds must be 1 .. PSC_MAX_FIELDS (4)");
    if (p->model == PSC_MODEL_PHI2 && p->nflds != 1) return fail(PSC_ERR_CONFIG, "the phi^2 model has one field");
    if (p->model == PSC_MODEL_PHI2CHI2 && p->nflds != 2) return fail(PSC_ERR_CONFIG, "the phi^2 chi^2 model has two fields");
    if (!psc::model_known(p->model)) return fail(PSC_ERR_CONFIG, "unknown model (not built in and not a compiled model.h)");
    // the GW Z pass carries 2 nflds input line pairs of N/16 threads in a 256-thread block
    if (p->with_gw && !p->spectral && p->N >= 32 && p->nflds * p->N > 2048)
        return fail(PSC_ERR_CONFIG, "GWs with more than two fields need N <= 512 (three or four fields)");
    if (p->vv != 2 && p->vv != 4 && p->vv != 6 && p->vv != 8 && p->vv != 10)
        return fail(PSC_ERR_CONFIG, "vv must be 2, 4, 6, 8 or 10");
    if (p->precision != 32 && p->precision != 64) return fail(PSC_ERR_CONFIG, "precision must be 32 or 64");
    if (p->N_pad != 0) {
        if (!p->spectral || p->with_gw)
            return fail(PSC_ERR_CONFIG, "the padded step (N_pad) is the spectral step without GWs, as in the reference");
        // N_pad: a size psc_create takes for N, above N (the register engine at N_pad when it is a
        // power of two >= 32, the generic engine otherwise)
        if (p->N_pad <= p->N ||
            !(pow2(p->N_pad) ? p->N_pad <= 1024 : (p->N_pad % 2 == 0 && smooth7(p->N_pad) && p->N_pad <= 512)))
            return fail(PSC_ERR_CONFIG, "N_pad must be above N and a lattice size psc_create takes for N");
    }
    if (p->expansion < 0 || p->expansion > 2) return fail(PSC_ERR_CONFIG, "expansion must be 0, 1 or 2");
    if (!(p->kIR > 0) || !(p->MPl > 0) || !(p->m_in_MPl > 0) || !(p->a0 > 0))
        return fail(PSC_ERR_CONFIG, "kIR, MPl, m_in_MPl and a0 must be positive");
    return PSC_OK;
}

// the fields two realizations must share to be advanced by the same launches
std::tuple<int, int, int, int, int, int, int, int, int, int, double, double, double, double, double, double>
config_key(const psc_params &p) {
    return std::make_tuple(p.N, p.nflds, p.vv, p.alpha, p.expansion, p.simulate_inflation, p.spectral, p.with_gw,
                           p.precision, p.model, p.gsq, p.kIR, p.MPl, p.m_in_MPl, p.fStar > 0 ? p.fStar : p.MPl,
                           p.epsilon);
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

// host threads of the download's FP32 -> FP64 widening (memory-bound; one thread
// converts ~1-2 GB/s): the CPUs this process may run on, at most 32
unsigned host_threads() {
    unsigned nt = 0;
#ifdef __linux__
    cpu_set_t set;
    if (sched_getaffinity(0, sizeof(set), &set) == 0) nt = (unsigned)CPU_COUNT(&set);
#endif
    if (nt == 0) nt = std::thread::hardware_concurrency();
    if (nt == 0) nt = 1;
    return nt > 32 ? 32 : nt;
}

// out[i] = (float)in[i], round to nearest even: the host cast's rounding
__global__ void k_round_f32(const double *__restrict__ in, float *__restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __double2float_rn(in[i]);
}

// host FP64 complex -> device array of the handle's precision. An FP32 handle copies
// the caller's FP64 data chunk by chunk into a device scratch and rounds it there: the
// copy engine reads the caller's memory at C2C speed, while rounding on the host
// cores moved 1.5x the bytes through host memory (256^3 + GW state: 12 ms vs 21 ms).
// the device FP64 scratch of the FP32 state exchange: one chunk of up to 16 Mi doubles
// (128 MB), enough for n doubles or one chunk of them
int ensure_xfer(psc_handle *h, size_t n) {
    const size_t kChunk = (size_t)16 << 20;
    const size_t want = n < kChunk ? n : kChunk;
    if (h->xfer_elems >= want) return PSC_OK;
    if (h->xfer) cudaFree(h->xfer);
    h->xfer = nullptr;
    h->xfer_elems = 0;
    if (cudaMalloc(&h->xfer, want * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return fail(PSC_ERR_NOMEM, "state exchange scratch");
    }
    h->xfer_elems = want;
    return PSC_OK;
}

// out[i] = in[i] widened to FP64
__global__ void k_widen_f64(const float *__restrict__ in, double *__restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

// true when p is page-locked host memory the copy engine can address directly
bool pinned_host(const void *p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// the device's address of page-locked host memory mapped into its address space (the memory
// of cudaHostAlloc / torch's pin_memory), or null
void *mapped_host(const void *p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// out[i] = (float2)in[i] (round to nearest even), in read by the device straight from mapped
// host memory: one pass over the chip-to-chip link, no staging copy
__global__ void __launch_bounds__(256) k_round_f32_mapped(const double2 *__restrict__ in, float2 *__restrict__ out,
                                                          size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double2 v = in[i];
        out[i] = make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
    }
}

// out[i] = (double2)in[i], written by the device straight into mapped host memory
__global__ void __launch_bounds__(256) k_widen_f64_mapped(const float2 *__restrict__ in, double2 *__restrict__ out,
                                                          size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = in[i];
        out[i] = make_double2((double)v.x, (double)v.y);
    }
}

unsigned mapped_grid(size_t n) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        sms = 152;
    const size_t want = (n + 255) / 256, most = (size_t)sms * 8;
    return (unsigned)(want < most ? want : most);
}

int upload(psc_handle *h, void *dst, const double *src, size_t ncplx) {
    if (h->p0().precision == 64) {
        CU(cudaMemcpyAsync(dst, src, ncplx * 16, cudaMemcpyHostToDevice, h->st));
        CU(cudaStreamSynchronize(h->st));
        return PSC_OK;
    }
    if (const void *dsrc = ((uintptr_t)src % 16 == 0) ? mapped_host(src) : nullptr) {
        // page-locked and mapped: the rounding kernel reads the caller's FP64 values directly
        k_round_f32_mapped<<<mapped_grid(ncplx), 256, 0, h->st>>>(static_cast<const double2 *>(dsrc),
                                                                  static_cast<float2 *>(dst), ncplx);
        CU(cudaGetLastError());
        CU(cudaStreamSynchronize(h->st));
        return PSC_OK;
    }
    const size_t n = 2 * ncplx;
    if (int rc = ensure_xfer(h, n)) return rc;
    float *out = static_cast<float *>(dst);
    for (size_t off = 0; off < n; off += h->xfer_elems) {
        const size_t c = n - off < h->xfer_elems ? n - off : h->xfer_elems;
        CU(cudaMemcpyAsync(h->xfer, src + off, c * sizeof(double), cudaMemcpyHostToDevice, h->st));
        const size_t blocks = (c + 255) / 256;
        k_round_f32<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, h->st>>>(h->xfer, out + off, c);
        CU(cudaGetLastError());
    }
    CU(cudaStreamSynchronize(h->st));
    return PSC_OK;
}

// device array of the handle's precision -> host FP64 (count scalars)
int download_real(psc_handle *h, double *dst, const void *src, size_t count) {
    if (h->p0().precision == 64) {
        CU(cudaMemcpyAsync(dst, src, count * 8, cudaMemcpyDeviceToHost, h->st));
        CU(cudaStreamSynchronize(h->st));
        return PSC_OK;
    }
    if (void *ddst = (count % 2 == 0 && (uintptr_t)dst % 16 == 0 && (uintptr_t)src % 8 == 0) ? mapped_host(dst)
                                                                                           : nullptr) {
        // a page-locked destination mapped into the device: the widening kernel writes the FP64
        // values straight into it (one pass over the chip-to-chip link)
        k_widen_f64_mapped<<<mapped_grid(count / 2), 256, 0, h->st>>>(static_cast<const float2 *>(src),
                                                                      static_cast<double2 *>(ddst), count / 2);
        CU(cudaGetLastError());
        CU(cudaStreamSynchronize(h->st));
        return PSC_OK;
    }
    if (pinned_host(dst)) {
        // a page-locked destination: widen on the device chunk by chunk and copy the FP64
        // values straight into it (no host-core work)
        if (int rc = ensure_xfer(h, count)) return rc;
        const float *sf = static_cast<const float *>(src);
        for (size_t off = 0; off < count; off += h->xfer_elems) {
            const size_t c = count - off < h->xfer_elems ? count - off : h->xfer_elems;
            const size_t blocks = (c + 255) / 256;
            k_widen_f64<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, h->st>>>(sf + off, h->xfer, c);
            CU(cudaGetLastError());
            CU(cudaMemcpyAsync(dst + off, h->xfer, c * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        }
        CU(cudaStreamSynchronize(h->st));
        return PSC_OK;
    }
    int rc = ensure_staging(h, count * 4);
    if (rc) return rc;
    const float *s = static_cast<const float *>(src);
    float *stg = static_cast<float *>(h->stage_buf);
    // K chunks copied back-to-back into the pinned staging, an event after each; the host
    // threads widen chunk k as soon as its event has completed, while the copy engine
    // moves chunk k+1 (no staging slot is reused, so no copy waits for a conversion)
    const size_t kMinChunk = (size_t)4 << 20;
    int K = (int)(count / kMinChunk);
    if (K > 16) K = 16;
    if (K < 1) K = 1;
    const size_t clen = (count + K - 1) / K;
    cudaEvent_t ev[16];
    int made = 0;
    for (int k = 0; k < K; ++k) {
        const size_t b = (size_t)k * clen, e = std::min(count, b + clen);
        cudaError_t err = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
        if (err == cudaSuccess) {
            ++made;
            if (b < e) err = cudaMemcpyAsync(stg + b, s + b, (e - b) * 4, cudaMemcpyDeviceToHost, h->st);
        }
        if (err == cudaSuccess) err = cudaEventRecord(ev[k], h->st);
        if (err != cudaSuccess) {
            cudaStreamSynchronize(h->st);
            for (int i = 0; i < made; ++i) cudaEventDestroy(ev[i]);
            return fail(PSC_ERR_CUDA, std::string("download: ") + cudaGetErrorString(err));
        }
    }
    unsigned nt = host_threads();
    if (count < ((size_t)2 << 20)) nt = 1;
    std::atomic<int> bad{0};
    int dev = 0;
    cudaGetDevice(&dev);
    auto work = [&](unsigned w) {
        if (w && cudaSetDevice(dev) != cudaSuccess) {
            bad.store(1);
            return;
        }
        for (int k = 0; k < K; ++k) {
            if (cudaEventSynchronize(ev[k]) != cudaSuccess) {
                bad.store(1);
                return;
            }
            const size_t b = (size_t)k * clen, e = std::min(count, b + clen);
            const size_t per = (e - b + nt - 1) / nt;
            const size_t lo = std::min(e, b + w * per), hi = std::min(e, lo + per);
            for (size_t i = lo; i < hi; ++i) dst[i] = (double)stg[i];
        }
    };
    std::vector<std::thread> th;
    for (unsigned w = 1; w < nt; ++w) th.emplace_back(work, w);
    work(0);
    for (auto &x : th) x.join();
    for (int k = 0; k < K; ++k) cudaEventDestroy(ev[k]);
    if (bad.load()) return fail(PSC_ERR_CUDA, "download: copy failed");
    return PSC_OK;
}

int read_bg(psc_handle *h, int r, psc::DevBG *out) {
    CU(cudaMemcpyAsync(out, h->b.bg + r, sizeof(psc::DevBG), cudaMemcpyDeviceToHost, h->st));
    CU(cudaStreamSynchronize(h->st));
    return PSC_OK;
}

int write_bg(psc_handle *h, int r, const psc::DevBG &in) {
    CU(cudaMemcpyAsync(h->b.bg + r, &in, sizeof(psc::DevBG), cudaMemcpyHostToDevice, h->st));
    CU(cudaStreamSynchronize(h->st));
    return PSC_OK;
}

// element offsets of realization r
void *foff(psc_handle *h, void *base, int r) {
    return static_cast<char *>(base) + (size_t)r * h->cfg.g.fstride * h->csize;
}
void *goff(psc_handle *h, void *base, int r) {
    return static_cast<char *>(base) + (size_t)r * h->cfg.g.gstride * h->csize;
}

// the buffers of realization r seen as a single lattice
psc::Buffers buffers_of(psc_handle *h, int r) {
    psc::Buffers b = h->b;
    b.fk = foff(h, h->b.fk, r);
    b.pk = foff(h, h->b.pk, r);
    b.TA = foff(h, h->b.TA, r);
    b.QV = foff(h, h->b.QV, r);
    if (h->b.Fk) b.Fk = foff(h, h->b.Fk, r);
    if (h->b.Fu) b.Fu = goff(h, h->b.Fu, r);
    if (h->cfg.g.gw) {
        b.uk = goff(h, h->b.uk, r);
        b.puk = goff(h, h->b.puk, r);
        b.TB = foff(h, h->b.TB, r);
        b.TC = foff(h, h->b.TC, r);
        b.QS = goff(h, h->b.QS, r);
    }
    b.bg = h->b.bg + r;
    // the tensor maps describe all R realizations at once: a single-lattice view has none
    b.xtma = nullptr;
    b.ytma = b.ytma_i = nullptr;
    return b;
}

psc::LaunchCfg single_cfg(psc_handle *h) {
    psc::LaunchCfg c = h->cfg;
    c.R = 1;
    return c;
}

// one force evaluation (with the drift when drift != 0): the padded step's on a padded
// handle (psc_pad.cu), the fused passes otherwise
cudaError_t stage_of(psc_handle *h, int drift, cudaStream_t st) {
    if (h->padded) return psc::launch_pad_stage(h->cfg, h->cfgp, h->b, h->bp, h->p0().precision, drift, st);
    return psc::launch_stage(h->cfg, h->b, h->p0().precision, drift, st);
}

// pure evaluation of the force pipeline for all realizations: K, G, V and
// (keep_add = 0) a''
int evaluate(psc_handle *h, int keep_add) {
    CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_EVAL, 0, h->st));
    CU(stage_of(h, 0, h->st));
    CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_EVAL_END, keep_add, h->st));
    CU(cudaStreamSynchronize(h->st));
    h->diag_valid = true;
    return PSC_OK;
}

// the kernels of one step (all stages) on stream st
cudaError_t enqueue_step(psc_handle *h, cudaStream_t st) {
    cudaError_t err = cudaSuccess;
    for (int p = 0; p < h->s && err == cudaSuccess; ++p) {
        err = stage_of(h, 1, st);
        if (err == cudaSuccess) err = psc::launch_scalar(h->cfg, h->b, psc::SCALAR_END, p, st);
    }
    return err;
}

// the opening half kick of a call and the start of its first step
cudaError_t enqueue_prologue(psc_handle *h, double dt, int nsteps, cudaStream_t st) {
    cudaError_t e = psc::launch_set_run(h->b.bg, h->R, dt, nsteps, st);
    if (e == cudaSuccess) e = psc::launch_scalar(h->cfg, h->b, psc::SCALAR_PRIME, h->force_valid ? 1 : 0, st);
    // the force at the current (f, a) is the one the previous call's last kick kept: the
    // opening half kick needs no force evaluation then (same arithmetic, same bits)
    if (e == cudaSuccess)
        e = h->force_valid ? psc::launch_open_kick(h->cfg, h->b, h->p0().precision, st) : stage_of(h, 0, st);
    if (e == cudaSuccess) e = psc::launch_scalar(h->cfg, h->b, psc::SCALAR_BEGIN, 0, st);
    return e;
}

int instantiate(cudaStream_t st, cudaError_t err, cudaGraphExec_t *out) {
    cudaGraph_t graph = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    if (err != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(PSC_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(err));
    }
    if (e2 != cudaSuccess) return fail(PSC_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(e2));
    cudaError_t e3 = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e3 != cudaSuccess) {
        *out = nullptr;
        return fail(PSC_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
    }
    return PSC_OK;
}

int build_graph(psc_handle *h) {
    if (h->gexec) return PSC_OK;
    CU(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    return instantiate(h->st, enqueue_step(h, h->st), &h->gexec);
}

// the error word of the handle's realizations: PSC_ERR_DEVICE before any other code
int read_err(psc_handle *h) {
    std::vector<psc::DevBG> bgs(h->R);
    CU(cudaMemcpyAsync(bgs.data(), h->b.bg, sizeof(psc::DevBG) * h->R, cudaMemcpyDeviceToHost, h->st));
    CU(cudaStreamSynchronize(h->st));
    int err = 0;
    for (int r = 0; r < h->R; ++r)
        if (bgs[r].err && (!err || bgs[r].err == PSC_ERR_DEVICE)) err = bgs[r].err;
    return err;
}

const char *step_err_msg(int err) {
    switch (err) {
    case PSC_ERR_TIMEOUT: return "a bulk copy's bounded wait ran out during the step (the copies then landed)";
    case PSC_ERR_DEVICE:
        return "a bulk copy's bounded wait ran out and the copies never completed: the CUDA context can no "
               "longer be trusted";
    default: return "non-finite background (NaN/Inf in a, a' or a'') during the step";
    }
}

int create_handle(const psc_params *ps, int R, psc_handle **out) {
    *out = nullptr;
    int rc;
    for (int r = 0; r < R; ++r)
        if ((rc = validate(ps + r))) return rc;
    psc_handle *h = new (std::nothrow) psc_handle();
    if (!h) return fail(PSC_ERR_NOMEM, "host allocation failed");
    h->p.assign(ps, ps + R);
    for (auto &q : h->p)
        if (q.fStar <= 0) q.fStar = q.MPl;
    h->R = R;
    h->w = kW2;
    const psc_params &p = h->p0();
    switch (p.vv) {
    case 4: h->s = 3; h->w = kW4; break;
    case 6: h->s = 7; h->w = kW6; break;
    case 8: h->s = 15; h->w = kW8; break;
    case 10: h->s = 31; h->w = kW10; break;
    default: h->s = 1; h->w = kW2;
    }
    h->csize = p.precision == 32 ? 8 : 16;
    h->nb = psc_maxnumbins(p.N);
    psc::plan(p, R, &h->cfg);
    h->padded = p.N_pad > 0;
    if (h->padded) {
        if (R != 1) {
            delete h;
            return fail(PSC_ERR_CONFIG, "padded lattices run one per handle (no batches)");
        }
        // the padded step never fills the R_Q2C mask (evolution.cpp:1611-1637): K, G over all modes
        h->cfg.g.mask = 0;
        psc_params q = p;
        q.N = p.N_pad;
        psc::plan(q, 1, &h->cfgp);
    }
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
    CUB(psc::configure(h->cfg, p.precision));
    if (h->padded) CUB(psc::configure(h->cfgp, p.precision));
    const size_t farr = (size_t)R * g.fstride * h->csize;   // nf arrays per realization
    const size_t garr = (size_t)R * g.gstride * h->csize;   // 6 arrays per realization (GW)
    psc::Buffers &b = h->b;
    if ((rc = dalloc(h, &b.fk, farr)) || (rc = dalloc(h, &b.pk, farr)) || (rc = dalloc(h, &b.TA, farr)) ||
        (rc = dalloc(h, &b.QV, farr)))
        return bail(rc);
    if (g.gw) {
        if ((rc = dalloc(h, &b.uk, garr)) || (rc = dalloc(h, &b.puk, garr)) || (rc = dalloc(h, &b.TB, farr)) ||
            (rc = dalloc(h, &b.TC, farr)) || (rc = dalloc(h, &b.QS, garr)))
            return bail(rc);
    }
    void *tmp = nullptr;
    if ((rc = dalloc(h, &b.tw, (size_t)g.N * h->csize))) return bail(rc);
    if ((rc = dalloc(h, &tmp, sizeof(double) * (size_t)R * g.pkg_stride))) return bail(rc);
    b.partKG = static_cast<double *>(tmp);
    h->partKG_cap = (size_t)R * g.pkg_stride;
    const size_t pv = h->padded ? std::max(g.pv_stride, h->cfgp.g.pv_stride) : g.pv_stride;
    if ((rc = dalloc(h, &tmp, sizeof(double) * (size_t)R * pv))) return bail(rc);
    b.partV = static_cast<double *>(tmp);
    h->partV_cap = (size_t)R * pv;
    if ((rc = dalloc(h, &tmp, sizeof(double) * (g.nf * 3 + 2) * h->nb))) return bail(rc);
    b.spec = static_cast<double *>(tmp);
    if ((rc = dalloc(h, &tmp, sizeof(int) * (g.nf + 1) * h->nb))) return bail(rc);
    b.spec_cnt = static_cast<int *>(tmp);
    if ((rc = dalloc(h, &tmp, sizeof(psc::DevBG) * R))) return bail(rc);
    b.bg = static_cast<psc::DevBG *>(tmp);
    // the kept force (register-engine and padded steps; the small-N generic engine
    // evaluates the opening force every call)
    if (g.reg || h->padded) {
        if ((rc = dalloc(h, &b.Fk, farr))) return bail(rc);
        if (g.gwev && (rc = dalloc(h, &b.Fu, garr))) return bail(rc);
    }
    if (h->padded) {
        // N_pad-grid arrays: padded spectra (zero outside the band, written in-band each
        // stage), the transform intermediates and the N_pad twiddles
        const psc::Geo &gp = h->cfgp.g;
        const size_t parr = (size_t)gp.fstride * h->csize;
        psc::Buffers &bp = h->bp;
        bp = b;   // partKG, partV, bg shared with the lattice grid
        if ((rc = dalloc(h, &bp.fk, parr)) || (rc = dalloc(h, &bp.TA, parr)) || (rc = dalloc(h, &bp.QV, parr)) ||
            (rc = dalloc(h, &bp.tw, (size_t)gp.N * h->csize)))
            return bail(rc);
        bp.pk = bp.uk = bp.puk = bp.TB = bp.TC = bp.QS = nullptr;
        bp.Fk = bp.Fu = nullptr;
        bp.tape_f = bp.tape_p = bp.tape_vp = bp.tape_fx = bp.tape_pu = bp.tape_fu = nullptr;
        CUB(cudaMemsetAsync(bp.fk, 0, parr, h->st));
    }
    CUB(cudaMemsetAsync(b.fk, 0, farr, h->st));
    CUB(cudaMemsetAsync(b.pk, 0, farr, h->st));
    if (g.gw) {
        CUB(cudaMemsetAsync(b.uk, 0, garr, h->st));
        CUB(cudaMemsetAsync(b.puk, 0, garr, h->st));
    }
    // twiddles e^{-2 pi i q/N} from FP64 sin/cos
    {
        std::vector<double> tw(2 * g.N);
        for (int q = 0; q < g.N; ++q) {
            const double ang = 2.0 * kPi * (double)q / (double)g.N;
            tw[2 * q] = std::cos(ang);
            tw[2 * q + 1] = -std::sin(ang);
        }
        if ((rc = upload(h, b.tw, tw.data(), g.N))) return bail(rc);
        if (h->padded) {
            const int Np = h->cfgp.g.N;
            tw.assign(2 * Np, 0.0);
            for (int q = 0; q < Np; ++q) {
                const double ang = 2.0 * kPi * (double)q / (double)Np;
                tw[2 * q] = std::cos(ang);
                tw[2 * q + 1] = -std::sin(ang);
            }
            if ((rc = upload(h, h->bp.tw, tw.data(), Np))) return bail(rc);
        }
    }
    for (int r = 0; r < R; ++r) {
        const psc_params &q = h->p[r];
        psc::DevBG bg{};
        bg.a = q.a0;
        bg.s = h->s;
        for (int i = 0; i < h->s; ++i) bg.w[i] = h->w[i];
        bg.alpha = q.alpha;
        bg.nf = g.nf;
        bg.nterms = g.nterms;
        bg.mask = g.mask;
        bg.model = q.model;
        bg.nbx = h->cfg.nbx;
        bg.nbz = h->cfg.nbz;
        bg.kIR = q.kIR;
        bg.kIR2 = q.kIR * q.kIR;
        const double fStar = q.fStar, omegaStar = q.m_in_MPl * fStar;
        const double L = 2 * kPi / q.kIR, dx = L / (double)q.N;
        bg.DFDP = std::pow(omegaStar / fStar, 2) * (q.N / dx) / 2.;   // parameters.h:132
        bg.fs_over_mpl2 = (fStar / q.MPl) * (fStar / q.MPl);
        bg.eps = q.epsilon;
        bg.gsq = q.gsq;
        bg.inv_n3 = 1.0 / (double)g.sites;
        bg.inv_n3sq = bg.inv_n3 * bg.inv_n3;
        bg.inv_nv = bg.inv_n3;
        bg.wait_ns = psc::kBulkWaitNs;
        bg.fp32 = q.precision == 32 ? 1 : 0;
        if (h->padded) {
            // <V> over the padded sites (kernel_a_k_pad, evolution.cpp:1624-1631)
            bg.nbz = h->cfgp.nbz;
            bg.inv_nv = 1.0 / (double)h->cfgp.g.sites;
        }
        if ((rc = write_bg(h, r, bg))) return bail(rc);
    }
#undef CUB
    encode_xtma(h);
    *out = h;
    return PSC_OK;
}

// the host generator (initialize.cpp:562-810) for realization r, uploaded
int init_ic_host(psc_handle *h, int r, std::vector<double> &fk, std::vector<double> &pk, std::vector<double> &uk,
                 std::vector<double> &puk, psc::ICInfo *info) {
    const psc::Geo &g = h->cfg.g;
    const size_t n = (size_t)g.modes;
    int rc;
    std::fill(fk.begin(), fk.end(), 0.0);
    std::fill(pk.begin(), pk.end(), 0.0);
    if (g.gw) {
        std::fill(uk.begin(), uk.end(), 0.0);
        std::fill(puk.begin(), puk.end(), 0.0);
    }
    *info = psc::generate_ic(h->p[r], fk.data(), pk.data(), g.gw ? uk.data() : nullptr, g.gw ? puk.data() : nullptr);
    if ((rc = upload(h, foff(h, h->b.fk, r), fk.data(), n * g.nf)) ||
        (rc = upload(h, foff(h, h->b.pk, r), pk.data(), n * g.nf)))
        return rc;
    if (g.gw && ((rc = upload(h, goff(h, h->b.uk, r), uk.data(), n * 6)) ||
                 (rc = upload(h, goff(h, h->b.puk, r), puk.data(), n * 6))))
        return rc;
    return PSC_OK;
}

// the homogeneous modes' FP64 shadow from FP64 host arrays ([nf][modes] interleaved complex)
void shadow_from(psc::DevBG &bg, const double *f_k, const double *pi_k, int nf, long long modes) {
    for (int f = 0; f < nf; ++f)
        for (int c = 0; c < 2; ++c) {
            bg.z0f[f][c] = f_k[2 * (size_t)f * modes + c];
            bg.z0p[f][c] = pi_k[2 * (size_t)f * modes + c];
        }
    bg.zero64 = 1;
    bg.z0pending = 0;
}

int init_ic(psc_handle *h) {
    const psc::Geo &g = h->cfg.g;
    const size_t n = (size_t)g.modes;
    std::vector<double> fk, pk, uk, puk;
    int rc;
    for (int r = 0; r < h->R; ++r) {
        psc::ICInfo info;
        const bool on_device = h->p[r].seed >= 1 && !(psc::ic_setup(h->p[r]).k2c > 0.);
        if (on_device) {
            // on the device: one thread per mode (initialize.cpp:686-749 by skip-ahead)
            if ((rc = psc::ic_device(h, r, &info))) return rc;
        } else {
            // seed < 1 (constant draws) or an initial low-pass cut: the host generator
            if (fk.empty()) {
                fk.resize(2 * n * g.nf);
                pk.resize(2 * n * g.nf);
                if (g.gw) {
                    uk.resize(2 * n * 6);
                    puk.resize(2 * n * 6);
                }
            }
            if ((rc = init_ic_host(h, r, fk, pk, uk, puk, &info))) return rc;
        }
        psc::DevBG bg;
        if ((rc = read_bg(h, r, &bg))) return rc;
        bg.a = info.a;
        bg.ad = info.ad;
        bg.add = info.add_printed;
        bg.t = 0.0;
        bg.err = 0;
        if (on_device) {
            // the homogeneous modes as the device generator computes them in FP64
            // (initialize.cpp:760-765), before their rounding to the array precision
            const psc::ICSetup s = psc::ic_setup(h->p[r]);
            for (int f = 0; f < g.nf; ++f) {
                bg.z0f[f][0] = s.f0[f] * s.n3;
                bg.z0p[f][0] = s.aop * s.fd0[f] * s.n3;
                bg.z0f[f][1] = bg.z0p[f][1] = 0.0;
            }
            bg.zero64 = 1;
            bg.z0pending = 0;
        } else {
            shadow_from(bg, fk.data(), pk.data(), g.nf, g.modes);
        }
        if ((rc = write_bg(h, r, bg))) return rc;
    }
    h->have_state = true;
    h->force_valid = false;
    // initialize() ends with add = kernel_a_k_nopad() / kernel_a() (initialize.cpp:786-797)
    return evaluate(h, 0);
}

int set_state(psc_handle *h, int r, const double *f_k, const double *pi_k, double a, double ad, double add,
              const double *u_k, const double *pi_u_k) {
    if (!f_k || !pi_k) return fail(PSC_ERR_ARG, "null argument");
    const psc::Geo &g = h->cfg.g;
    if (g.gw && (!u_k || !pi_u_k)) return fail(PSC_ERR_ARG, "GW run needs u_k and pi_u_k");
    const size_t n = (size_t)g.modes;
    int rc;
    if ((rc = upload(h, foff(h, h->b.fk, r), f_k, n * g.nf)) || (rc = upload(h, foff(h, h->b.pk, r), pi_k, n * g.nf)))
        return rc;
    if (g.gw && ((rc = upload(h, goff(h, h->b.uk, r), u_k, n * 6)) ||
                 (rc = upload(h, goff(h, h->b.puk, r), pi_u_k, n * 6))))
        return rc;
    psc::DevBG bg;
    if ((rc = read_bg(h, r, &bg))) return rc;
    bg.a = a;
    bg.ad = ad;
    bg.add = add;
    bg.err = 0;
    shadow_from(bg, f_k, pi_k, g.nf, g.modes);
    if ((rc = write_bg(h, r, bg))) return rc;
    h->have_state = true;
    h->diag_valid = false;
    h->force_valid = false;
    return PSC_OK;
}

int get_state(psc_handle *h, int r, double *f_k, double *pi_k, double *a, double *ad, double *add, double *u_k,
              double *pi_u_k) {
    const psc::Geo &g = h->cfg.g;
    const size_t n = (size_t)g.modes;
    int rc;
    if (f_k && (rc = download_real(h, f_k, foff(h, h->b.fk, r), 2 * n * g.nf))) return rc;
    if (pi_k && (rc = download_real(h, pi_k, foff(h, h->b.pk, r), 2 * n * g.nf))) return rc;
    if (g.gw) {
        if (u_k && (rc = download_real(h, u_k, goff(h, h->b.uk, r), 2 * n * 6))) return rc;
        if (pi_u_k && (rc = download_real(h, pi_u_k, goff(h, h->b.puk, r), 2 * n * 6))) return rc;
    }
    psc::DevBG bg;
    if ((rc = read_bg(h, r, &bg))) return rc;
    if (bg.zero64)   // the homogeneous modes at the precision the device evolves them in
        for (int f = 0; f < g.nf; ++f)
            for (int c = 0; c < 2; ++c) {
                if (f_k) f_k[2 * (size_t)f * n + c] = bg.z0f[f][c];
                if (pi_k) pi_k[2 * (size_t)f * n + c] = bg.z0p[f][c];
            }
    if (a) *a = bg.a;
    if (ad) *ad = bg.ad;
    if (add) *add = bg.add;
    return PSC_OK;
}

int step(psc_handle *h, double dt, int nsteps) {
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state: call psc_init_ic or psc_set_state first");
    if (nsteps < 0 || !(dt > 0) || !std::isfinite(dt)) return fail(PSC_ERR_ARG, "need dt > 0 and nsteps >= 0");
    if (nsteps == 0) return PSC_OK;
    int rc = build_graph(h);
    if (rc) return rc;
    const bool kept = h->force_valid;
    h->force_valid = false;
    CU(cudaEventRecord(h->ev0, h->st));
    // opening half kick: pi_half = pi + w0 dt/2 F(f, a)  (evolution.cpp:1144-1158, stage 0)
    h->force_valid = kept;
    const cudaError_t pe = enqueue_prologue(h, dt, nsteps, h->st);
    h->force_valid = false;
    CU(pe);
    for (int i = 0; i < nsteps; ++i) CU(cudaGraphLaunch(h->gexec, h->st));
    CU(cudaEventRecord(h->ev1, h->st));
    const int err = read_err(h);
    CU(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
    h->diag_valid = true;
    h->force_valid = false;
    if (err) return fail(err, step_err_msg(err));
    h->force_valid = h->b.Fk != nullptr;
    return PSC_OK;
}

int fields_real(psc_handle *h, int r, double *f, double *pi_f) {
    const psc::Geo &g = h->cfg.g;
    const size_t rsize = h->csize / 2;
    int rc;
    if (!h->b.real && (rc = dalloc(h, &h->b.real, (size_t)g.sites * g.nf * rsize))) return rc;
    const psc::LaunchCfg c1 = single_cfg(h);
    const psc::Buffers b1 = buffers_of(h, r);
    if (f) {
        CU(psc::launch_c2r_real(c1, b1, h->p0().precision, b1.fk, g.nf, h->st));
        if ((rc = download_real(h, f, h->b.real, (size_t)g.sites * g.nf))) return rc;
    }
    if (pi_f) {
        CU(psc::launch_c2r_real(c1, b1, h->p0().precision, b1.pk, g.nf, h->st));
        if ((rc = download_real(h, pi_f, h->b.real, (size_t)g.sites * g.nf))) return rc;
    }
    return PSC_OK;
}

int spectra(psc_handle *h, int r, int32_t *numpoints, double *f2, double *pi2, double *n2, int32_t *gw_numpoints,
            double *h2, double *hdot2, double *hdot2_zero) {
    const psc::Geo &g = h->cfg.g;
    const int nb = h->nb, nf = g.nf;
    const psc::Buffers b1 = buffers_of(h, r);
    CU(psc::launch_spectra(single_cfg(h), b1, h->p0().precision, nb, h->st));
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
    if (hdot2_zero) *hdot2_zero = 0.0;
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
                const char *base = static_cast<const char *>(b1.puk) + (size_t)c * g.modes * h->csize;
                if (h->p0().precision == 64) {
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
    }
    return PSC_OK;
}

int energies(psc_handle *h, int r, double *K, double *G, double *V, double *total, double *friedmann_violation,
             double *rho_gw) {
    int rc;
    if (!h->diag_valid && (rc = evaluate(h, 1))) return rc;
    psc::DevBG bg;
    if ((rc = read_bg(h, r, &bg))) return rc;
    const psc::Geo &g = h->cfg.g;
    const psc_params &q = h->p[r];
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
    const double RHS = bg.fs_over_mpl2 * std::pow(bg.a, 2 * (q.alpha + 1)) * tot / 3.;
    if (friedmann_violation) *friedmann_violation = std::fabs(LHS - RHS) / std::fabs(LHS + RHS);
    if (rho_gw) {
        *rho_gw = 0.0;
        if (g.gw) {
            // output.cpp:1030-1060: zero mode plus the un-normalised bins
            const int nb = h->nb;
            std::vector<int> cnt(nb);
            std::vector<double> hd(nb);
            double hz = 0.0;
            if ((rc = spectra(h, r, nullptr, nullptr, nullptr, nullptr, cnt.data(), nullptr, hd.data(), &hz)))
                return rc;
            double s = hz;
            for (int l = 1; l < nb; ++l) s += hd[l] * (cnt[l] > 0 ? cnt[l] : 1);
            const double fStar = q.fStar, omegaStar = q.m_in_MPl * fStar, MPl = q.MPl;
            s *= omegaStar * omegaStar * std::pow(fStar, 4) / (MPl * MPl) / 4. * bg.inv_n3sq / std::pow(bg.a, 6);
            s /= (fStar * omegaStar) * (fStar * omegaStar);
            *rho_gw = s;
        }
    }
    return PSC_OK;
}

int means(psc_handle *h, int r, double *out) {
    const psc::Geo &g = h->cfg.g;
    std::vector<double> f((size_t)g.sites * g.nf), pf((size_t)g.sites * g.nf);
    int rc = fields_real(h, r, f.data(), pf.data());
    if (rc) return rc;
    psc::DevBG bg;
    if ((rc = read_bg(h, r, &bg))) return rc;
    const double aop = std::pow(bg.a, h->p[r].alpha - 3);
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
        fa /= n;
        f2 /= n;
        pa /= n;
        p2 /= n;
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

// ------------------------------------------------------------------ tensor maps (TMA)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// The tensor maps of the handle's passes (TMA staging), re-encoded whenever the tile shape
// changes. Register engine, single-lattice or batch handles alike (the realization is a map
// dimension); otherwise, or when the handle's mask (psc_set_tensor_maps) leaves a group out,
// that group is off and its passes load directly.
// X passes: an array group (na arrays of `modes` complex, realization stride rstride) as
// {lines_x, N, na, R} in 8-byte elements (an FP64 complex is two), box {lines per tile,
// min(N, 256), 1, 1} (a box edge is at most 256: a tile of N > 256 points is N/256 boxes).
// Y forward pass (FP32): V' and S_ab as {2 H, N N/2, na, R} (rows of two y; YTma,
// psc_launch.h), boxes {TL, min(N/2, 256), 1, 1} (even rows) and {TL + 2, min(N/2, 256), 1, 1}
// (odd rows); on for the sizes with the tensor-map instantiation (N = 128 .. 1024) when TL
// divides N/2 and a box row is a multiple of 16 bytes.
void encode_xtma(psc_handle *h) {
    h->xtma = psc::XTma{};
    h->ytma = h->ytma_i = psc::YTma{};
    h->b.xtma = nullptr;
    h->b.ytma = h->b.ytma_i = nullptr;
    const psc::Geo &g = h->cfg.g;
    auto enc = tensor_map_encoder();
    if (!enc || !g.reg || h->padded) return;
    const cuuint64_t w = h->csize / 8, TL = 1u << g.tlx_shift;
    auto map4 = [&](CUtensorMap *m, void *base, const cuuint64_t (&dims)[4], const cuuint64_t (&strides)[3],
                    cuuint32_t box0, cuuint32_t box1) -> bool {
        const cuuint32_t box[4] = {box0, box1, 1, 1};
        const cuuint32_t es[4] = {1, 1, 1, 1};
        return enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    };
    auto rs = [&](long long rstride, int na) {
        return (cuuint64_t)(rstride > 0 ? rstride : g.modes * na) * h->csize;
    };
    if (h->tmap_mask & PSC_TMAP_X) {
        auto make = [&](CUtensorMap *m, void *base, int na, long long rstride) -> bool {
            const cuuint64_t dims[4] = {(cuuint64_t)g.lines_x * w, (cuuint64_t)g.N, (cuuint64_t)na, (cuuint64_t)h->R};
            const cuuint64_t strides[3] = {(cuuint64_t)g.lines_x * h->csize, (cuuint64_t)g.modes * h->csize,
                                           rs(rstride, na)};
            return map4(m, base, dims, strides, (cuuint32_t)(TL * w), (cuuint32_t)std::min(g.N, 256));
        };
        bool ok = make(&h->xtma.fk, h->b.fk, g.nf, g.fstride) && make(&h->xtma.pk, h->b.pk, g.nf, g.fstride) &&
                  make(&h->xtma.qv, h->b.QV, g.nf, g.fstride);
        if (ok && g.gwev)
            ok = make(&h->xtma.uk, h->b.uk, 6, g.gstride) && make(&h->xtma.puk, h->b.puk, 6, g.gstride) &&
                 make(&h->xtma.qs, h->b.QS, 6, g.gstride);
        if (ok) {
            h->xtma.on = 1;
            h->xtma.xi = h->csize == 8 ? 1 : 0;   // FP64: three 64 KB tiles would leave one block per SM
            h->b.xtma = &h->xtma;
        } else {
            h->xtma = psc::XTma{};
        }
    }
    const cuuint64_t ox = w == 1 ? 1 : 0;   // FP32: the odd rows' box starts one element early
    const bool yfits = w == 1 && psc::y_pipe_size(g.N) && TL <= (cuuint64_t)g.M && (TL * w * 8) % 16 == 0 &&
                       (TL + 2 * ox) * w <= 256;
    if ((h->tmap_mask & PSC_TMAP_Y) && yfits) {
        auto make = [&](CUtensorMap *me, CUtensorMap *mo, void *base, int na, long long rstride) -> bool {
            const cuuint64_t dims[4] = {(cuuint64_t)(2 * g.H) * w, (cuuint64_t)g.N * g.M, (cuuint64_t)na,
                                        (cuuint64_t)h->R};
            const cuuint64_t strides[3] = {(cuuint64_t)(2 * g.H) * h->csize, (cuuint64_t)g.modes * h->csize,
                                           rs(rstride, na)};
            const cuuint32_t yb = (cuuint32_t)std::min(g.M, 256);   // pairs per box
            return map4(me, base, dims, strides, (cuuint32_t)(TL * w), yb) &&
                   map4(mo, base, dims, strides, (cuuint32_t)((TL + 2 * ox) * w), yb);
        };
        psc::YTma &y = h->ytma;
        bool ok = make(&y.ae, &y.ao, h->b.QV, g.nf, g.fstride);
        if (ok && g.gwev) ok = make(&y.be, &y.bo, h->b.QS, 6, g.gstride);
        if (ok) {
            y.na = g.nf;
            y.on = 1;
            h->b.ytma = &h->ytma;
        } else {
            h->ytma = psc::YTma{};
        }
        // the GW Y inverse pass (pipelined): TA and TB of each field; by default at N = 1024 only
        // (0.212 against 0.203 ms for the direct form at 256^3; 15.4 against 19.5 ms at 1024^3)
        psc::YTma &yi = h->ytma_i;
        const bool yinv = g.N >= 1024 || (h->tmap_mask & PSC_TMAP_YINV);
        if (g.gwev && yinv && make(&yi.ae, &yi.ao, h->b.TA, g.nf, g.fstride) &&
            make(&yi.be, &yi.bo, h->b.TB, g.nf, g.fstride)) {
            yi.na = g.nf;
            yi.on = 1;
            h->b.ytma_i = &h->ytma_i;
        } else {
            h->ytma_i = psc::YTma{};
        }
    }
}

// ------------------------------------------------------------------ autotuner
// Tile and grid shapes of the register-engine passes chosen by timing the candidates on the
// handle's own buffers. Choices are cached per configuration in the process and, when
// PSC_TUNE_CACHE names a file, across processes (one line per configuration).
using TuneKey = std::tuple<int, int, int, int, int, int, int>;   // N, nflds, GW evolved, precision, R, user, SMs

TuneKey tune_key(psc_handle *h) {
    const psc::Geo &g = h->cfg.g;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return TuneKey(g.N, g.nf, g.gwev, h->p0().precision, h->R, psc::model_is_user(h->p0().model) ? 1 : 0, sms);
}

std::map<TuneKey, psc::TileChoice> &tune_cache() {
    static std::map<TuneKey, psc::TileChoice> m;
    return m;
}
std::mutex &tune_mutex() {
    static std::mutex m;
    return m;
}

void tune_cache_load() {
    static bool loaded = false;
    if (loaded) return;
    loaded = true;
    const char *path = std::getenv("PSC_TUNE_CACHE");
    if (!path || !*path) return;
    FILE *fh = std::fopen(path, "r");
    if (!fh) return;
    int k[7], c[3];
    while (std::fscanf(fh, "%d %d %d %d %d %d %d %d %d %d", &k[0], &k[1], &k[2], &k[3], &k[4], &k[5], &k[6], &c[0],
                       &c[1], &c[2]) == 10) {
        psc::TileChoice tc;
        tc.xy_shift = c[0];
        tc.z_shift = c[1];
        tc.z_per_sm = c[2];
        tune_cache()[TuneKey(k[0], k[1], k[2], k[3], k[4], k[5], k[6])] = tc;
    }
    std::fclose(fh);
}

void tune_cache_store(const TuneKey &k, const psc::TileChoice &tc) {
    tune_cache()[k] = tc;
    const char *path = std::getenv("PSC_TUNE_CACHE");
    if (!path || !*path) return;
    FILE *fh = std::fopen(path, "a");
    if (!fh) return;
    std::fprintf(fh, "%d %d %d %d %d %d %d %d %d %d\n", std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k),
                 std::get<4>(k), std::get<5>(k), std::get<6>(k), tc.xy_shift, tc.z_shift, tc.z_per_sm);
    std::fclose(fh);
}

// Re-plan the handle with shapes tc: launch configuration, kernel attributes, partial-sum
// buffers large enough for the new block counts, the block counts in the background records,
// and a fresh step graph at the next step call.
int apply_shapes(psc_handle *h, const psc::TileChoice &tc) {
    psc::LaunchCfg c;
    psc::plan(h->p0(), h->R, &c, &tc);
    CU(psc::configure(c, h->p0().precision));
    const size_t kg = (size_t)h->R * c.g.pkg_stride, pv = (size_t)h->R * c.g.pv_stride;
    void *tmp = nullptr;
    int rc;
    if (kg > h->partKG_cap) {
        if ((rc = dalloc(h, &tmp, sizeof(double) * kg))) return rc;
        h->b.partKG = static_cast<double *>(tmp);
        h->partKG_cap = kg;
    }
    if (pv > h->partV_cap) {
        if ((rc = dalloc(h, &tmp, sizeof(double) * pv))) return rc;
        h->b.partV = static_cast<double *>(tmp);
        h->partV_cap = pv;
    }
    h->cfg = c;
    encode_xtma(h);   // the operand tiles follow the tile shape
    for (int r = 0; r < h->R; ++r) {
        psc::DevBG bg;
        if ((rc = read_bg(h, r, &bg))) return rc;
        bg.nbx = c.nbx;
        bg.nbz = c.nbz;
        if ((rc = write_bg(h, r, bg))) return rc;
    }
    if (h->gexec) {
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
    }
    return PSC_OK;
}

// Device time of each pass of `reps` stage evaluations (zero drift and kick coefficients:
// the state is unchanged) with the current shapes.
int time_stage(psc_handle *h, int reps, double *ms) {
    cudaEvent_t ev[7];
    for (int i = 0; i < 7; ++i) CU(cudaEventCreate(&ev[i]));
    for (int i = 0; i < PSC_NPASS; ++i) ms[i] = 0;
    psc::Buffers bt = h->b;
    bt.Fk = bt.Fu = nullptr;
    int rc = PSC_OK;
    for (int r = 0; r < reps + 1 && rc == PSC_OK; ++r) {   // the first evaluation warms up
        cudaError_t e = psc::launch_scalar(h->cfg, bt, psc::SCALAR_EVAL, 0, h->st);
        if (e == cudaSuccess) e = psc::launch_stage_timed(h->cfg, bt, h->p0().precision, 1, psc::SCALAR_EVAL_END, ev, h->st);
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[6]);
        for (int i = 0; i < PSC_NPASS && e == cudaSuccess && r > 0; ++i) {
            float t = 0.f;
            e = cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
            ms[i] += t / reps;
        }
        if (e != cudaSuccess) rc = fail(PSC_ERR_CUDA, cudaGetErrorString(e));
    }
    for (int i = 0; i < 7; ++i) cudaEventDestroy(ev[i]);
    h->diag_valid = true;
    return rc;
}

int autotune(psc_handle *h, int reps, int *shape, int *from_cache) {
    const psc::Geo &g = h->cfg.g;
    if (from_cache) *from_cache = 0;
    if (!g.reg || h->padded) {   // the generic engine (N < 32) and the padded step keep their shapes
        if (shape) shape[0] = shape[1] = shape[2] = -1;
        return PSC_OK;
    }
    std::lock_guard<std::mutex> lock(tune_mutex());
    tune_cache_load();
    const TuneKey key = tune_key(h);
    auto it = tune_cache().find(key);
    psc::TileChoice best;
    int rc;
    if (it != tune_cache().end()) {
        best = it->second;
        if (from_cache) *from_cache = 1;
    } else {
        if (!h->have_state) return fail(PSC_ERR_STATE, "no state: the candidates are timed on the lattice's state");
        psc::LaunchCfg def;
        psc::plan(h->p0(), h->R, &def);
        const psc::TileChoice d0 = def.tc;
        double ms[PSC_NPASS];
        // X and Y passes (one tile shape for all four): the default and two narrower tiles of at
        // least four lines (32 contiguous bytes of an FP32 row)
        double best_xy = 1e30;
        for (int s = d0.xy_shift; s >= 2 && s >= d0.xy_shift - 2; --s) {
            psc::TileChoice tc = d0;
            tc.xy_shift = s;
            if ((rc = apply_shapes(h, tc)) || (rc = time_stage(h, reps, ms))) return rc;
            const double t = ms[0] + ms[1] + ms[3] + ms[4];
            if (t < best_xy) {
                best_xy = t;
                best.xy_shift = s;
            }
        }
        // Z pass: lines per tile x resident blocks per SM of the persistent forms
        double best_z = 1e30;
        for (int s = d0.z_shift; s >= 0 && s >= d0.z_shift - 2; --s)
            for (int k = d0.z_per_sm; k >= 1; --k) {
                psc::TileChoice tc = d0;
                tc.z_shift = s;
                tc.z_per_sm = k;
                if ((rc = apply_shapes(h, tc)) || (rc = time_stage(h, reps, ms))) return rc;
                if (ms[2] < best_z) {
                    best_z = ms[2];
                    best.z_shift = s;
                    best.z_per_sm = k;
                }
            }
        tune_cache_store(key, best);
    }
    if ((rc = apply_shapes(h, best))) return rc;
    if (shape) {
        shape[0] = h->cfg.tc.xy_shift;
        shape[1] = h->cfg.tc.z_shift;
        shape[2] = h->cfg.tc.z_per_sm;
    }
    return PSC_OK;
}

// mass_sq_av of spectra() (output.cpp:566-580): effective_mass at every site of the real-space
// fields, summed in the reference's site order in FP64, over N^3
int mass_sq_av(psc_handle *h, int r, double *out) {
    const psc::Geo &g = h->cfg.g;
    std::vector<double> f((size_t)g.sites * g.nf);
    int rc = fields_real(h, r, f.data(), nullptr);
    if (rc) return rc;
    const psc_params &p = h->p[r];
    double acc[PSC_MAX_FIELDS] = {}, pt[PSC_MAX_FIELDS] = {}, m2[PSC_MAX_FIELDS] = {};
    for (long long i = 0; i < g.sites; ++i) {
        for (int q = 0; q < g.nf; ++q) pt[q] = f[(size_t)q * g.sites + i];
        model_effective_mass(p.model, p.gsq, m2, pt);
        for (int q = 0; q < g.nf; ++q) acc[q] += m2[q];
    }
    for (int q = 0; q < g.nf; ++q) out[q] = acc[q] / (double)g.sites;
    return PSC_OK;
}

}  // namespace hapi
}  // namespace psc
using namespace psc::hapi;

// ------------------------------------------------------------------ batches
struct psc_batch {
    std::vector<psc_handle *> groups;
    std::vector<std::pair<int, int>> where;   // realization index -> (group, slot)
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
    cudaGraphExec_t gexec = nullptr;
    float last_ms = 0.f;
    // one launch per pass for all groups (psc_batch.cuh): the work lists, and per pass the grid
    // and dynamic shared memory of the batched kernel; `multi` when the caller asked for it
    // (per_group = false) and the batch qualifies. Per-group launches are the default: on the
    // mixed 32^3 / 64^3 / 128^3 ensemble they measured 2.53 ms per step against 2.89 ms
    bool multi = false, per_group = true;
    psc::BatchTable bt{};
    int grid[psc::kBatchPasses] = {};
    size_t smem[psc::kBatchPasses] = {};
};

namespace {

// The batched passes of psc_batch.cuh cover the register engine's line lengths 32 .. 256 with
// 256-thread blocks, the built-in models and one precision, GW setting and integrator for all
// groups; other batches launch every group's passes on its own stream.
int batch_multi_setup(psc_batch *b) {
    b->multi = false;
    if (b->per_group || b->groups.empty() || (int)b->groups.size() > psc::kMaxBatchGroups) return PSC_OK;
    const psc_handle *h0 = b->groups[0];
    for (const psc_handle *h : b->groups) {
        const psc::Geo &g = h->cfg.g;
        if (!g.reg || g.N > 256 || h->padded || psc::model_is_user(h->p0().model) || h->cfg.thr_xy != 256 ||
            h->cfg.thr_z != 256 || h->p0().precision != h0->p0().precision || g.gwev != h0->cfg.g.gwev || h->s != h0->s)
            return PSC_OK;
    }
    psc::BatchTable &bt = b->bt;
    bt = psc::BatchTable{};
    bt.ngroups = (int)b->groups.size();
    size_t smem[psc::kBatchPasses] = {0, 0, 0, 0, 0};
    for (int gi = 0; gi < bt.ngroups; ++gi) {
        const psc_handle *h = b->groups[gi];
        const psc::LaunchCfg &c = h->cfg;
        const psc::Geo &g = c.g;
        psc::BatchGroup &G = bt.grp[gi];
        G.g = g;
        G.L = g.N;
        G.nbx = c.nbx;
        G.nbz = c.nbz;
        G.R = h->R;
        G.nj = g.nf + (g.gwev ? 6 : 0);
        const psc::Buffers &B = h->b;
        G.fk = B.fk; G.pk = B.pk; G.uk = B.uk; G.puk = B.puk;
        G.TA = B.TA; G.TB = B.TB; G.TC = B.TC; G.QV = B.QV; G.QS = B.QS; G.tw = B.tw;
        G.Fk = B.Fk; G.Fu = B.Fu; G.partKG = B.partKG; G.partV = B.partV; G.bg = B.bg;
        int nj = 0;
        for (int f = 0; f < g.nf; ++f) {
            G.fwd.rs[nj] = g.fstride;
            G.fwd.p[nj++] = static_cast<char *>(B.QV) + (size_t)f * g.modes * h->csize;
        }
        if (g.gwev)
            for (int q = 0; q < 6; ++q) {
                G.fwd.rs[nj] = g.gstride;
                G.fwd.p[nj++] = static_cast<char *>(B.QS) + (size_t)q * g.modes * h->csize;
            }
        const int count[psc::kBatchPasses] = {c.nbx * g.nf * h->R, c.nbx * g.nf * h->R, c.nbz * h->R,
                                              c.nbx * G.nj * h->R, c.nbx * G.nj * h->R};
        for (int k = 0; k < psc::kBatchPasses; ++k) {
            G.start[k] = bt.total[k];
            bt.total[k] += count[k];
        }
        const size_t need[psc::kBatchPasses] = {c.smem_xy, g.gwev ? 3 * c.smem_xy : c.smem_xy, c.smem_z, c.smem_xy,
                                                c.smem_xf};
        for (int k = 0; k < psc::kBatchPasses; ++k) smem[k] = std::max(smem[k], need[k]);
    }
    int dev = 0, sms = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const bool f32 = h0->p0().precision == 32;
    for (int k = 0; k < psc::kBatchPasses; ++k) {
        int per_sm = 0;
        for (int drift = 0; drift < (k == 0 ? 2 : 1); ++drift) {
            const void *kern = f32 ? psc::reg_batch_kernel_f32(k, drift) : psc::reg_batch_kernel_f64(k, drift);
            CU(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem[k]));
            CU(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    cudaSharedmemCarveoutMaxShared));
            CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem[k]));
        }
        if (per_sm < 1) return PSC_OK;   // does not fit: per-group launches
        b->smem[k] = smem[k];
        b->grid[k] = std::min(bt.total[k], per_sm * sms);
    }
    b->multi = true;
    return PSC_OK;
}

// the kernels of one step of every group: one launch per pass and one background launch per
// stage for all groups
cudaError_t enqueue_batch_step(psc_batch *b, cudaStream_t st) {
    const bool f32 = b->groups[0]->p0().precision == 32;
    cudaError_t e = cudaSuccess;
    for (int p = 0; p < b->groups[0]->s && e == cudaSuccess; ++p) {
        for (int k = 0; k < psc::kBatchPasses && e == cudaSuccess; ++k)
            e = f32 ? psc::reg_batch_pass_f32(b->bt, k, k == 0, b->grid[k], b->smem[k], st)
                    : psc::reg_batch_pass_f64(b->bt, k, k == 0, b->grid[k], b->smem[k], st);
        if (e == cudaSuccess) e = psc::launch_scalar_batch(b->bt, p, st);
    }
    return e;
}

}  // namespace

// ------------------------------------------------------------------ model evaluation
namespace {

// dvdf, the potential terms (arithmetic T, the lattice path's) and the effective masses
// (FP64) of one field point
template <typename T>
__host__ __device__ void model_point(int model, double gsq, int nf, const double *fv, double *dvdf, double *terms,
                                     double *mass_sq) {
    T v[psc::kMaxFields] = {}, out[psc::kMaxFields] = {}, t[psc::kMaxTerms] = {};
    double vd[psc::kMaxFields] = {};
    for (int q = 0; q < nf; ++q) {
        v[q] = (T)fv[q];
        vd[q] = fv[q];
    }
    const psc::ModelG<T> m{model, (T)gsq};
    const int nt = psc::model_nterms(model);
    if (dvdf) {
        psc::model_dvdf<T, T, true>(m, v, out, nf);
        for (int q = 0; q < nf; ++q) dvdf[q] = (double)out[q];
    }
    if (terms) {
        psc::model_potential<T, T, T, true>(m, v, t);
        for (int q = 0; q < nt; ++q) terms[q] = (double)t[q];
    }
    if (mass_sq) {
        double m2[psc::kMaxFields] = {};
        psc::model_effective_mass(model, gsq, m2, vd);
        for (int q = 0; q < nf; ++q) mass_sq[q] = m2[q];
    }
}

template <typename T>
__global__ void k_model_eval(int model, double gsq, int nf, long long n, const double *fields, double *dvdf,
                             double *terms, double *mass_sq) {
    const int nt = psc::model_nterms(model);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        model_point<T>(model, gsq, nf, fields + i * nf, dvdf ? dvdf + i * nf : nullptr, terms ? terms + i * nt : nullptr,
                       mass_sq ? mass_sq + i * nf : nullptr);
}

}  // namespace

extern "C" {

int psc_model_count(void) { return psc::kUserModels; }

const char *psc_model_name(int model) {
    if (model == PSC_MODEL_PHI2) return "builtin:phi2";
    if (model == PSC_MODEL_PHI2CHI2) return "builtin:phi2chi2";
    if (psc::model_is_user(model)) return psc::kUserModelNames[model - PSC_MODEL_USER];
    return nullptr;
}

int psc_model_find(const char *name, int *model) {
    if (!name || !model) return fail(PSC_ERR_ARG, "null argument");
    for (int id : {PSC_MODEL_PHI2, PSC_MODEL_PHI2CHI2})
        if (std::strcmp(name, psc_model_name(id)) == 0) {
            *model = id;
            return PSC_OK;
        }
    for (int i = 0; i < psc::kUserModels; ++i)
        if (std::strcmp(name, psc::kUserModelNames[i]) == 0) {
            *model = PSC_MODEL_USER + i;
            return PSC_OK;
        }
    return fail(PSC_ERR_CONFIG, (std::string("no model named ") + name + " in this build").c_str());
}

int psc_model_nterms(int model) { return psc::model_known(model) ? psc::model_nterms(model) : 0; }

int psc_model_eval(const psc_params *p, int on_device, long long n, const double *fields, double *dvdf,
                   double *terms, double *mass_sq) {
    if (!p || !fields || n < 0) return fail(PSC_ERR_ARG, "bad argument");
    if (!psc::model_known(p->model)) return fail(PSC_ERR_CONFIG, "unknown model");
    if (p->nflds < 1 || p->nflds > PSC_MAX_FIELDS) return fail(PSC_ERR_CONFIG, "nflds must be 1 .. PSC_MAX_FIELDS");
    if (p->precision != 32 && p->precision != 64) return fail(PSC_ERR_CONFIG, "precision must be 32 or 64");
    const int nf = p->nflds, nt = psc::model_nterms(p->model);
    if (n == 0) return PSC_OK;
    if (!on_device) {
        for (long long i = 0; i < n; ++i) {
            double *d = dvdf ? dvdf + i * nf : nullptr, *t = terms ? terms + i * nt : nullptr;
            double *m = mass_sq ? mass_sq + i * nf : nullptr;
            if (p->precision == 32) model_point<float>(p->model, p->gsq, nf, fields + i * nf, d, t, m);
            else model_point<double>(p->model, p->gsq, nf, fields + i * nf, d, t, m);
        }
        return PSC_OK;
    }
    const size_t fb = sizeof(double) * (size_t)n * nf, tb = sizeof(double) * (size_t)n * nt;
    double *dev = nullptr;
    CU(cudaMalloc(&dev, 3 * fb + tb));
    double *df = dev, *dd = dev + (size_t)n * nf, *dm = dd + (size_t)n * nf, *dt = dm + (size_t)n * nf;
    int rc = PSC_OK;
    cudaError_t e = cudaMemcpy(df, fields, fb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
        if (p->precision == 32)
            k_model_eval<float><<<blocks, 256>>>(p->model, p->gsq, nf, n, df, dd, dt, dm);
        else
            k_model_eval<double><<<blocks, 256>>>(p->model, p->gsq, nf, n, df, dd, dt, dm);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess && dvdf) e = cudaMemcpy(dvdf, dd, fb, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && terms) e = cudaMemcpy(terms, dt, tb, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && mass_sq) e = cudaMemcpy(mass_sq, dm, fb, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = fail(PSC_ERR_CUDA, cudaGetErrorString(e));
    cudaFree(dev);
    return rc;
}


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
    if (!p) return fail(PSC_ERR_ARG, "null parameters");
    return create_handle(p, 1, out);
}

void psc_destroy(psc_handle *h) {
    if (!h) return;
    cudaStreamSynchronize(h->st);
    free_all(h);
    delete h;
}

int psc_init_ic(psc_handle *h) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return init_ic(h);
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
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return set_state(h, 0, f_k, pi_k, a, ad, add, u_k, pi_u_k);
}

int psc_set_state_padded(psc_handle *h, int Nsrc, const double *f_k, const double *pi_k, double a, double ad,
                         double add, const double *u_k, const double *pi_u_k) {
    if (!h || !f_k || !pi_k) return fail(PSC_ERR_ARG, "null argument");
    if (h->R != 1) return fail(PSC_ERR_CONFIG, "single-lattice handles only");
    const psc::Geo &g = h->cfg.g;
    if (!pow2(Nsrc) || Nsrc < 2 || Nsrc >= g.N) return fail(PSC_ERR_ARG, "Nsrc must be a power of two below N");
    if (g.gw && (!u_k || !pi_u_k)) return fail(PSC_ERR_ARG, "GW run needs u_k and pi_u_k");
    const size_t ms = (size_t)Nsrc * Nsrc * (Nsrc / 2 + 1);
    const int prec = h->p0().precision;
    void *src = nullptr;
    CU(cudaMallocAsync(&src, ms * 6 * h->csize, h->st));
    struct Arr { const double *host; void *dev; int count; };
    std::vector<Arr> arrs = {{f_k, h->b.fk, g.nf}, {pi_k, h->b.pk, g.nf}};
    if (g.gw) {
        arrs.push_back({u_k, h->b.uk, 6});
        arrs.push_back({pi_u_k, h->b.puk, 6});
    }
    int rc = PSC_OK;
    for (const Arr &x : arrs) {
        if ((rc = upload(h, src, x.host, ms * x.count))) break;
        const cudaError_t e = psc::launch_prolong(src, x.dev, x.count, Nsrc, g.N, prec, h->st);
        if (e != cudaSuccess) {
            rc = fail(PSC_ERR_CUDA, std::string("prolongation: ") + cudaGetErrorString(e));
            break;
        }
    }
    cudaFreeAsync(src, h->st);
    if (rc) return rc;
    CU(psc::launch_zero_sync(h->cfg, h->b, h->st));
    CU(cudaStreamSynchronize(h->st));
    psc::DevBG bg;
    if ((rc = read_bg(h, 0, &bg))) return rc;
    bg.a = a;
    bg.ad = ad;
    bg.add = add;
    bg.err = 0;
    if ((rc = write_bg(h, 0, bg))) return rc;
    h->have_state = true;
    h->diag_valid = false;
    h->force_valid = false;
    return PSC_OK;
}

int psc_get_state(psc_handle *h, double *f_k, double *pi_k, double *a, double *ad, double *add, double *u_k,
                  double *pi_u_k) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return get_state(h, 0, f_k, pi_k, a, ad, add, u_k, pi_u_k);
}

int psc_get_time(psc_handle *h, double *t) {
    if (!h || !t) return fail(PSC_ERR_ARG, "null argument");
    psc::DevBG bg;
    int rc = read_bg(h, 0, &bg);
    if (rc) return rc;
    *t = bg.t;
    return PSC_OK;
}

int psc_set_time(psc_handle *h, double t) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    psc::DevBG bg;
    int rc = read_bg(h, 0, &bg);
    if (rc) return rc;
    bg.t = t;
    return write_bg(h, 0, bg);
}

int psc_step(psc_handle *h, double dt, int nsteps) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return step(h, dt, nsteps);
}

int psc_last_step_ms(psc_handle *h, float *ms) {
    if (!h || !ms) return fail(PSC_ERR_ARG, "null argument");
    *ms = h->last_ms;
    return PSC_OK;
}

int psc_time_passes(psc_handle *h, int reps, float *ms) {
    if (!h || !ms || reps < 1) return fail(PSC_ERR_ARG, "bad argument");
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state");
    if (h->padded) return fail(PSC_ERR_CONFIG, "per-pass times are those of the unpadded step (N_pad = 0)");
    cudaEvent_t ev[7];
    for (int i = 0; i < 7; ++i) CU(cudaEventCreate(&ev[i]));
    double acc[PSC_NPASS] = {0, 0, 0, 0, 0, 0};
    // the passes of a stage with the drift on and zero drift and kick coefficients
    // (SCALAR_EVAL): the full memory traffic of a step's stage, the state unchanged
    // (f + 0 pi = f exactly); a'' is kept (diagnostics mode). The kick does not keep its
    // force (no Fk, Fu): like every stage of a step call but the call's last one.
    psc::Buffers bt = h->b;
    bt.Fk = bt.Fu = nullptr;
    for (int r = 0; r < reps; ++r) {
        CU(psc::launch_scalar(h->cfg, bt, psc::SCALAR_EVAL, 0, h->st));
        CU(psc::launch_stage_timed(h->cfg, bt, h->p0().precision, 1, psc::SCALAR_EVAL_END, ev, h->st));
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

int psc_autotune(psc_handle *h, int reps, int *shape, int *from_cache) {
    if (!h || reps < 1) return fail(PSC_ERR_ARG, "bad argument");
    return autotune(h, reps, shape, from_cache);
}

int psc_set_shapes(psc_handle *h, const int *shape) {
    if (!h || !shape) return fail(PSC_ERR_ARG, "null argument");
    if (!h->cfg.g.reg || h->padded) return PSC_OK;
    psc::TileChoice tc;
    tc.xy_shift = shape[0];
    tc.z_shift = shape[1];
    tc.z_per_sm = shape[2];
    return apply_shapes(h, tc);
}

int psc_set_tensor_maps(psc_handle *h, int mask) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    if (mask & ~(PSC_TMAP_X | PSC_TMAP_Y | PSC_TMAP_YINV)) return fail(PSC_ERR_ARG, "unknown tensor-map group");
    h->tmap_mask = mask;
    encode_xtma(h);
    if (h->gexec) {   // the step graph holds the maps of its launches
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
    }
    return PSC_OK;
}

int psc_get_tensor_maps(psc_handle *h, int *mask) {
    if (!h || !mask) return fail(PSC_ERR_ARG, "null argument");
    *mask = (h->b.xtma ? PSC_TMAP_X : 0) | (h->b.ytma ? PSC_TMAP_Y : 0) | (h->b.ytma_i ? PSC_TMAP_YINV : 0);
    return PSC_OK;
}

int psc_get_shapes(psc_handle *h, int *shape) {
    if (!h || !shape) return fail(PSC_ERR_ARG, "null argument");
    const bool tunable = h->cfg.g.reg && !h->padded;
    shape[0] = tunable ? h->cfg.tc.xy_shift : -1;
    shape[1] = tunable ? h->cfg.tc.z_shift : -1;
    shape[2] = tunable ? h->cfg.tc.z_per_sm : -1;
    return PSC_OK;
}

// the bounded wait of the bulk-copy staging on an mbarrier whose transactions never
// arrive: thread 0 expects 16 bytes that no copy delivers
__global__ void k_bulk_wait_selftest(int *out, unsigned long long limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        psc::mbar_init(&bar, 1);
        psc::mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) psc::mbar_arrive_expect_tx(&bar, 16);
    const bool ok = psc::mbar_wait_bounded(&bar, 0, limit_ns);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) out[0] = PSC_ERR_TIMEOUT;
        return;
    }
    if (threadIdx.x == 0) out[0] = PSC_OK;
}

int psc_selftest_bulk_wait(double limit_ms, int *status) {
    if (!status || !(limit_ms > 0.0) || limit_ms > 10000.0) return fail(PSC_ERR_ARG, "bad argument");
    int *d = nullptr;
    CU(cudaMalloc(&d, sizeof(int)));
    int v = PSC_ERR_STATE;
    cudaError_t e = cudaMemcpy(d, &v, sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_bulk_wait_selftest<<<1, 64>>>(d, (unsigned long long)(limit_ms * 1e6));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&v, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(PSC_ERR_CUDA, std::string("wait self-test: ") + cudaGetErrorString(e));
    *status = v;
    return PSC_OK;
}

int psc_test_wait_hook_pass(psc_handle *h, double limit_ms, int plant_bytes, int pass) {
    if (!h || !(limit_ms > 0.0) || limit_ms > 10000.0 || plant_bytes < 0 || plant_bytes > 4096 || pass < 0 ||
        pass > 4)
        return fail(PSC_ERR_ARG, "bad argument");
    const psc::Geo &g = h->cfg.g;
    bool staged = false;
    switch (pass) {
    case 0: staged = h->b.xtma && h->xtma.xi; break;                 // X inverse (FP32 tensor maps)
    case 1: staged = h->b.ytma_i != nullptr; break;                  // GW Y inverse (tensor maps)
    case 3: staged = h->b.ytma != nullptr; break;                    // Y forward (tensor maps)
    case 2:                                                          // GW Z pass (bulk copies)
        staged = g.gwev && g.reg && h->p0().precision == 32 &&
                 ((size_t(1) << g.tlz_shift) * (size_t)g.H * h->csize) % 16 == 0;
        break;
    default: staged = h->b.xtma != nullptr; break;                   // X forward + kick (tensor maps)
    }
    if (plant_bytes && !staged) return fail(PSC_ERR_CONFIG, "the handle's pass does not stage its tiles by bulk copies");
    for (int r = 0; r < h->R; ++r) {
        psc::DevBG bg;
        int rc;
        if ((rc = read_bg(h, r, &bg))) return rc;
        bg.wait_ns = (unsigned long long)(limit_ms * 1e6);
        bg.wait_plant = plant_bytes;
        bg.wait_plant_pass = pass;
        if ((rc = write_bg(h, r, bg))) return rc;
    }
    return PSC_OK;
}

int psc_test_wait_hook(psc_handle *h, double limit_ms, int plant_bytes) {
    return psc_test_wait_hook_pass(h, limit_ms, plant_bytes, 2);
}

int psc_pass_bytes(psc_handle *h, double *bytes) {
    if (!h || !bytes) return fail(PSC_ERR_ARG, "bad argument");
    const psc::Geo &g = h->cfg.g;
    const double C = (double)g.modes * h->csize * h->R;
    const int nf = g.nf, gw = g.gwev;
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
    return fields_real(h, 0, f, pi_f);
}

int psc_spectra(psc_handle *h, int32_t *numpoints, double *f2, double *pi2, double *n2, int32_t *gw_numpoints,
                double *h2, double *hdot2, double *hdot2_zero) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return spectra(h, 0, numpoints, f2, pi2, n2, gw_numpoints, h2, hdot2, hdot2_zero);
}

int psc_energies(psc_handle *h, double *K, double *G, double *V, double *total, double *friedmann_violation,
                 double *rho_gw) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return energies(h, 0, K, G, V, total, friedmann_violation, rho_gw);
}

int psc_means(psc_handle *h, double *out) {
    if (!h || !out) return fail(PSC_ERR_ARG, "null argument");
    return means(h, 0, out);
}

int psc_mass_sq_av(psc_handle *h, double *out) {
    if (!h || !out) return fail(PSC_ERR_ARG, "null argument");
    return mass_sq_av(h, 0, out);
}

// ------------------------------------------------------------------ batches
int psc_batch_create(const psc_params *per_realization, int n, psc_batch **out) {
    if (!out || !per_realization || n < 1) return fail(PSC_ERR_ARG, "bad argument");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        int rc = validate(per_realization + i);
        if (rc) return rc;
        if (per_realization[i].N_pad) return fail(PSC_ERR_CONFIG, "padded lattices run one per handle (no batches)");
    }
    // group realizations that can share launches, in order of first appearance
    std::map<decltype(config_key(per_realization[0])), int> gid;
    std::vector<std::vector<int>> members;
    for (int i = 0; i < n; ++i) {
        auto key = config_key(per_realization[i]);
        auto it = gid.find(key);
        if (it == gid.end()) {
            it = gid.emplace(key, (int)members.size()).first;
            members.emplace_back();
        }
        members[it->second].push_back(i);
    }
    psc_batch *b = new (std::nothrow) psc_batch();
    if (!b) return fail(PSC_ERR_NOMEM, "host allocation failed");
    b->where.resize(n);
    auto bail = [&](int code) {
        psc_batch_destroy(b);
        return code;
    };
    for (size_t g = 0; g < members.size(); ++g) {
        std::vector<psc_params> ps;
        for (size_t k = 0; k < members[g].size(); ++k) {
            ps.push_back(per_realization[members[g][k]]);
            b->where[members[g][k]] = {(int)g, (int)k};
        }
        psc_handle *h = nullptr;
        int rc = create_handle(ps.data(), (int)ps.size(), &h);
        if (rc) return bail(rc);
        b->groups.push_back(h);
    }
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(PSC_ERR_CUDA, "batch stream/event creation failed"));
    b->join.resize(b->groups.size());
    for (auto &e : b->join)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(PSC_ERR_CUDA, "batch event creation failed"));
    if (int rc = batch_multi_setup(b)) return bail(rc);
    *out = b;
    return PSC_OK;
}

int psc_batch_launch_mode(psc_batch *b, int per_group, int *one_launch_per_pass) {
    if (!b) return fail(PSC_ERR_ARG, "null batch");
    if (per_group >= 0) {
        b->per_group = per_group != 0;
        if (int rc = batch_multi_setup(b)) return rc;
        if (b->gexec) {
            cudaGraphExecDestroy(b->gexec);
            b->gexec = nullptr;
        }
    }
    if (one_launch_per_pass) *one_launch_per_pass = b->multi ? 1 : 0;
    return PSC_OK;
}

void psc_batch_destroy(psc_batch *b) {
    if (!b) return;
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (psc_handle *h : b->groups) psc_destroy(h);
    for (cudaEvent_t e : b->join)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

int psc_batch_size(psc_batch *b) { return b ? (int)b->where.size() : 0; }

int psc_batch_groups(psc_batch *b) { return b ? (int)b->groups.size() : 0; }

int psc_batch_init_ic(psc_batch *b) {
    if (!b) return fail(PSC_ERR_ARG, "null batch");
    for (psc_handle *h : b->groups) {
        int rc = init_ic(h);
        if (rc) return rc;
    }
    return PSC_OK;
}

int psc_batch_step(psc_batch *b, double dt, int nsteps) {
    if (!b) return fail(PSC_ERR_ARG, "null batch");
    for (psc_handle *h : b->groups)
        if (!h->have_state) return fail(PSC_ERR_STATE, "no state: call psc_batch_init_ic first");
    if (nsteps < 0 || !(dt > 0) || !std::isfinite(dt)) return fail(PSC_ERR_ARG, "need dt > 0 and nsteps >= 0");
    if (nsteps == 0) return PSC_OK;
    // one graph per step for every group: fork to the groups' streams, join back
    auto fork_join = [&](auto &&body) -> cudaError_t {
        cudaError_t e = cudaEventRecord(b->fork, b->st);
        for (size_t g = 0; g < b->groups.size() && e == cudaSuccess; ++g) {
            psc_handle *h = b->groups[g];
            e = cudaStreamWaitEvent(h->st, b->fork, 0);
            if (e == cudaSuccess) e = body(h);
            if (e == cudaSuccess) e = cudaEventRecord(b->join[g], h->st);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->join[g], 0);
        }
        return e;
    };
    if (!b->gexec) {
        CU(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        const cudaError_t err = b->multi ? enqueue_batch_step(b, b->st)
                                         : fork_join([&](psc_handle *h) { return enqueue_step(h, h->st); });
        int rc = instantiate(b->st, err, &b->gexec);
        if (rc) return rc;
    }
    CU(cudaEventRecord(b->ev0, b->st));
    CU(fork_join([&](psc_handle *h) { return enqueue_prologue(h, dt, nsteps, h->st); }));
    for (int i = 0; i < nsteps; ++i) CU(cudaGraphLaunch(b->gexec, b->st));
    CU(cudaEventRecord(b->ev1, b->st));
    CU(cudaStreamSynchronize(b->st));
    CU(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1));
    for (psc_handle *h : b->groups) {
        h->diag_valid = true;
        const int err = read_err(h);
        if (err) return fail(err, step_err_msg(err));
    }
    return PSC_OK;
}

int psc_batch_autotune(psc_batch *b, int reps) {
    if (!b || reps < 1) return fail(PSC_ERR_ARG, "bad argument");
    for (psc_handle *h : b->groups) {
        int rc = autotune(h, reps, nullptr, nullptr);
        if (rc) return rc;
    }
    if (int rc = batch_multi_setup(b)) return rc;   // the groups' shapes may have changed
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    return PSC_OK;
}

int psc_batch_last_step_ms(psc_batch *b, float *ms) {
    if (!b || !ms) return fail(PSC_ERR_ARG, "null argument");
    *ms = b->last_ms;
    return PSC_OK;
}

#define PSC_BATCH_AT(b, idx, h, r)                                                                              \
    if (!(b) || (idx) < 0 || (idx) >= (int)(b)->where.size()) return fail(PSC_ERR_ARG, "bad realization index"); \
    psc_handle *h = (b)->groups[(b)->where[idx].first];                                                         \
    const int r = (b)->where[idx].second

int psc_batch_set_state(psc_batch *b, int idx, const double *f_k, const double *pi_k, double a, double ad, double add,
                        const double *u_k, const double *pi_u_k) {
    PSC_BATCH_AT(b, idx, h, r);
    return set_state(h, r, f_k, pi_k, a, ad, add, u_k, pi_u_k);
}

int psc_batch_get_state(psc_batch *b, int idx, double *f_k, double *pi_k, double *a, double *ad, double *add,
                        double *u_k, double *pi_u_k) {
    PSC_BATCH_AT(b, idx, h, r);
    return get_state(h, r, f_k, pi_k, a, ad, add, u_k, pi_u_k);
}

int psc_batch_spectra(psc_batch *b, int idx, int32_t *numpoints, double *f2, double *pi2, double *n2,
                      int32_t *gw_numpoints, double *h2, double *hdot2, double *hdot2_zero) {
    PSC_BATCH_AT(b, idx, h, r);
    return spectra(h, r, numpoints, f2, pi2, n2, gw_numpoints, h2, hdot2, hdot2_zero);
}

int psc_batch_energies(psc_batch *b, int idx, double *K, double *G, double *V, double *total,
                       double *friedmann_violation, double *rho_gw) {
    PSC_BATCH_AT(b, idx, h, r);
    return energies(h, r, K, G, V, total, friedmann_violation, rho_gw);
}

int psc_batch_means(psc_batch *b, int idx, double *out) {
    PSC_BATCH_AT(b, idx, h, r);
    if (!out) return fail(PSC_ERR_ARG, "null argument");
    return means(h, r, out);
}

int psc_batch_histograms(psc_batch *b, int idx, int nbins, double hmin, double hmax, double *binfreq, double *bmin,
                         double *df) {
    PSC_BATCH_AT(b, idx, h, r);
    return histograms(h, r, nbins, hmin, hmax, binfreq, bmin, df);
}

int psc_batch_write_snapshot(psc_batch *b, int idx, const char *path, int with_energy) {
    PSC_BATCH_AT(b, idx, h, r);
    return write_snapshot(h, r, path, with_energy);
}

#undef PSC_BATCH_AT

const char *psc_strerror(int code) {
    switch (code) {
    case PSC_OK: return "ok";
    case PSC_ERR_CONFIG: return "unsupported configuration";
    case PSC_ERR_ARG: return "bad argument";
    case PSC_ERR_CUDA: return "CUDA runtime error";
    case PSC_ERR_NONFINITE: return "non-finite background";
    case PSC_ERR_TIMEOUT: return "device-side wait timed out";
    case PSC_ERR_DEVICE: return "device-side wait timed out with copies still outstanding (context unusable)";
    case PSC_ERR_STATE: return "call out of order";
    case PSC_ERR_NOMEM: return "out of device memory";
    case PSC_ERR_IO: return "file could not be written";
    default: return "unknown error";
    }
}

const char *psc_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"
