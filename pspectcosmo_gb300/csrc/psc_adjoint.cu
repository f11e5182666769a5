// psc_adjoint.cu — hand-written discrete adjoint of the evolution step.
//
// The reference has no adjoint. This differentiates the step of evolve_VV
// (evolution.cpp:607-694; evolve_VV_k_nopad without the R_Q2C mask is the same
// map) for the scalar fields and the self-consistent background, including the
// coupling of every mode to a'' through K, G and V (evolution.cpp:421-439,
// 1087) and of the drift coefficient to a_half (evolution.cpp:1161-1165). The GW
// tensors do not act back on the fields or a(t), so they drop out of a
// scalar-field observable.
//
// Observable: O = <chi^2> (the last field) over the lattice at the final time.
// Gradients: with respect to the initial half-spectrum state f_k(0), pi_k(0)
// (as dO/dRe + i dO/dIm per stored mode), a'(0), and the model couplings
// (gsq and the phi mass coefficient mu, V = mu phi^2/2 + gsq phi^2 chi^2/2 at
// mu = 1), at a''(0) consistent with the initial state.
//
// Per stage, forward (stage inputs f, pi, a, b = a', add = a''; c1 = w dt/2):
//   bh = b + c1 add;  ph = pi + c1 F(f, a);  ah = a + c1 bh;  f1 = f + w dt ah^(al-3) ph
//   a1 = ah + c1 bh;  p1 = ph + c1 F(f1, a1);  add1 = A(f1, p1, a1);  b1 = bh + c1 add1
// with F(f, a) = -a^(1+al) kIR^2 k^2 f_k - a^(3+al) r2c(V'(f(x))) and
// A = (fStar/MPl)^2/3 a^(1+2al) ((al-2) K + al G + (al+1) V). The reverse sweep
// transposes these lines in opposite order; (dF/df)^T = F's Laplacian part plus
// -a^(3+al) r2c(V''(f(x)) lambda(x)) (the Hessian is symmetric). Adjoint arrays
// are kept as Lambda = r2c(lambda(x)); <lambda, y> = (1/N^3) sum' w Re(conj Lambda Y).
//
// Memory: checkpoints of the state every `every` steps; each segment is
// recomputed from its checkpoint with every stage input kept, then reversed.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "psc_dev.cuh"
#include "psc_handle.h"

using psc::hapi::fail;

namespace {

#define CU(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return fail(e_ == cudaErrorMemoryAllocation ? PSC_ERR_NOMEM : PSC_ERR_CUDA,                  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                             \
    } while (0)

constexpr int kThreads = 256;

__device__ __forceinline__ double wk_of(long long m, int H, int M) {
    const int kz = (int)(m % H);
    return (kz == 0 || kz == M) ? 1.0 : 2.0;
}

__device__ __forceinline__ double k2_of(long long m, int N, int H) {
    const int kz = (int)(m % H);
    const long long xy = m / H;
    const int y = (int)(xy % N), x = (int)(xy / N);
    const int px = psc::pcoord(x, N), py = psc::pcoord(y, N);
    return (double)(px * px + py * py + kz * kz);
}

template <int NV>
__device__ __forceinline__ void block_atomic_add(double (&v)[NV], double *acc) {
    __shared__ double red[32][NV];
#pragma unroll
    for (int i = 0; i < NV; ++i)
        for (int off = 16; off > 0; off >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) red[warp][i] = v[i];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double x = lane < nw ? red[lane][i] : 0.0;
            for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
            if (lane == 0) atomicAdd(&acc[i], x);
        }
    }
}

// y += (c0 + ck2 k^2) x over n complex elements (n = arrays * modes)
template <typename T>
__global__ void ka_lin(long long n, long long modes, int N, int H, psc::cplx<T> *y, const psc::cplx<T> *x, double c0,
                       double ck2) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double c = c0 + ck2 * k2_of(i % modes, N, H);
        psc::cplx<T> a = y[i];
        const psc::cplx<T> b = x[i];
        a.x += (T)(c * (double)b.x);
        a.y += (T)(c * (double)b.y);
        y[i] = a;
    }
}

// acc[0] += sum' w Re(conj X Y1) k^2 ; acc[1] += sum' w Re(conj X Y2)  (Y1 or Y2 may be null)
template <typename T>
__global__ void ka_dot2(long long n, long long modes, int N, int H, const psc::cplx<T> *X, const psc::cplx<T> *Y1,
                        const psc::cplx<T> *Y2, double *acc) {
    double v[2] = {0.0, 0.0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long m = i % modes;
        const double w = wk_of(m, H, N / 2);
        const psc::cplx<T> a = X[i];
        if (Y1) {
            const psc::cplx<T> b = Y1[i];
            v[0] += w * k2_of(m, N, H) * ((double)a.x * b.x + (double)a.y * b.y);
        }
        if (Y2) {
            const psc::cplx<T> b = Y2[i];
            v[1] += w * ((double)a.x * b.x + (double)a.y * b.y);
        }
    }
    block_atomic_add<2>(v, acc);
}

// acc[0] += sum' w |p|^2 ; acc[1] += sum' w k^2 |f|^2
template <typename T>
__global__ void ka_kg(long long n, long long modes, int N, int H, const psc::cplx<T> *f, const psc::cplx<T> *p,
                      double *acc) {
    double v[2] = {0.0, 0.0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long m = i % modes;
        const double w = wk_of(m, H, N / 2);
        const psc::cplx<T> a = p[i], b = f[i];
        v[0] += w * ((double)a.x * a.x + (double)a.y * a.y);
        v[1] += w * k2_of(m, N, H) * ((double)b.x * b.x + (double)b.y * b.y);
    }
    block_atomic_add<2>(v, acc);
}

// Real-space pointwise model work. mode 0: out = V'(f), acc += {V, dV/dgsq, dV/dmu};
// mode 1: out = V''(f) lambda, acc += {lambda . dV'/dgsq, lambda . dV'/dmu}.
template <typename T>
__global__ void kr_model(int mode, long long sites, int nf, int model, double gsq, const T *fx, const T *lam, T *out,
                         double *acc) {
    double v[3] = {0.0, 0.0, 0.0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < sites;
         i += (long long)gridDim.x * blockDim.x) {
        const double p = fx[i], c = (nf > 1) ? (double)fx[sites + i] : 0.0;
        const bool two = (model == PSC_MODEL_PHI2CHI2);
        if (mode == 0) {
            out[i] = (T)(two ? p + gsq * p * c * c : p);
            if (two) out[sites + i] = (T)(gsq * p * p * c);
            v[0] += 0.5 * p * p + (two ? 0.5 * gsq * p * p * c * c : 0.0);
            v[1] += two ? 0.5 * p * p * c * c : 0.0;
            v[2] += 0.5 * p * p;
        } else {
            const double l0 = lam[i], l1 = (nf > 1) ? (double)lam[sites + i] : 0.0;
            if (two) {
                const double h00 = 1.0 + gsq * c * c, h01 = 2.0 * gsq * p * c, h11 = gsq * p * p;
                out[i] = (T)(h00 * l0 + h01 * l1);
                out[sites + i] = (T)(h01 * l0 + h11 * l1);
                v[0] += l0 * p * c * c + l1 * p * p * c;
                v[1] += l0 * p;
            } else {
                out[i] = (T)l0;
                v[1] += l0 * p;
            }
        }
    }
    block_atomic_add<3>(v, acc);
}

struct BG3 {
    double a, b, add;
};

struct AdjWS {
    size_t carr = 0, rarr = 0;   // bytes of nf complex / real arrays
    void *ph = nullptr, *f1 = nullptr, *p1 = nullptr, *F0 = nullptr, *Vp0 = nullptr, *F1 = nullptr, *Vp1 = nullptr,
         *Lf = nullptr, *Lp = nullptr, *tmp = nullptr;
    void *fx0 = nullptr, *fx1 = nullptr, *lam = nullptr, *hout = nullptr;
    double *acc = nullptr;
    std::vector<void *> ckpt_f, ckpt_p;   // checkpoints (device)
    std::vector<BG3> ckpt_bg;
    std::vector<void *> tape_f, tape_p;   // stage inputs of one segment (device)
    std::vector<BG3> tape_bg;
    std::vector<void *> owned;
};

void ws_free(void *p) {
    AdjWS *ws = static_cast<AdjWS *>(p);
    for (void *q : ws->owned) cudaFree(q);
    delete ws;
}

int ws_alloc(AdjWS *ws, void **out, size_t bytes) {
    CU(cudaMalloc(out, bytes));
    ws->owned.push_back(*out);
    return PSC_OK;
}

struct Ctx {
    psc_handle *h;
    AdjWS *ws;
    int N, H, nf, prec, alpha, model;
    long long modes, sites;
    double kIR2, gsq, C, N3;
    cudaStream_t st;
    int grid;
};

template <typename T>
int run_lin(const Ctx &c, void *y, const void *x, double c0, double ck2) {
    ka_lin<T><<<c.grid, kThreads, 0, c.st>>>((long long)c.nf * c.modes, c.modes, c.N, c.H, (psc::cplx<T> *)y,
                                              (const psc::cplx<T> *)x, c0, ck2);
    CU(cudaGetLastError());
    return PSC_OK;
}

int lin(const Ctx &c, void *y, const void *x, double c0, double ck2) {
    return c.prec == 32 ? run_lin<float>(c, y, x, c0, ck2) : run_lin<double>(c, y, x, c0, ck2);
}

int read_acc(const Ctx &c, double *out, int n) {
    CU(cudaMemcpyAsync(out, c.ws->acc, sizeof(double) * n, cudaMemcpyDeviceToHost, c.st));
    CU(cudaStreamSynchronize(c.st));
    return PSC_OK;
}

int zero_acc(const Ctx &c) {
    CU(cudaMemsetAsync(c.ws->acc, 0, sizeof(double) * 8, c.st));
    return PSC_OK;
}

// sum' w k^2 Re(conj X Y1) and sum' w Re(conj X Y2), divided by N^3
int dots(const Ctx &c, const void *X, const void *Y1, const void *Y2, double *d1, double *d2) {
    int rc;
    if ((rc = zero_acc(c))) return rc;
    const long long n = (long long)c.nf * c.modes;
    if (c.prec == 32)
        ka_dot2<float><<<c.grid, kThreads, 0, c.st>>>(n, c.modes, c.N, c.H, (const float2 *)X, (const float2 *)Y1,
                                                      (const float2 *)Y2, c.ws->acc);
    else
        ka_dot2<double><<<c.grid, kThreads, 0, c.st>>>(n, c.modes, c.N, c.H, (const double2 *)X, (const double2 *)Y1,
                                                       (const double2 *)Y2, c.ws->acc);
    CU(cudaGetLastError());
    double v[2];
    if ((rc = read_acc(c, v, 2))) return rc;
    if (d1) *d1 = v[0] / c.N3;
    if (d2) *d2 = v[1] / c.N3;
    return PSC_OK;
}

int c2r(const Ctx &c, const void *src, void *dst) {
    CU(c.prec == 32 ? psc::reg_c2r_f32(c.h->cfg, c.h->b, src, c.nf, dst, c.st)
                    : psc::reg_c2r_f64(c.h->cfg, c.h->b, src, c.nf, dst, c.st));
    return PSC_OK;
}

int r2c(const Ctx &c, const void *src, void *dst) {
    CU(c.prec == 32 ? psc::reg_r2c_f32(c.h->cfg, c.h->b, src, c.nf, dst, c.st)
                    : psc::reg_r2c_f64(c.h->cfg, c.h->b, src, c.nf, dst, c.st));
    return PSC_OK;
}

int model(const Ctx &c, int mode, const void *fx, const void *lam, void *out, double *acc3) {
    int rc;
    if ((rc = zero_acc(c))) return rc;
    if (c.prec == 32)
        kr_model<float><<<c.grid, kThreads, 0, c.st>>>(mode, c.sites, c.nf, c.model, c.gsq, (const float *)fx,
                                                       (const float *)lam, (float *)out, c.ws->acc);
    else
        kr_model<double><<<c.grid, kThreads, 0, c.st>>>(mode, c.sites, c.nf, c.model, c.gsq, (const double *)fx,
                                                        (const double *)lam, (double *)out, c.ws->acc);
    CU(cudaGetLastError());
    return read_acc(c, acc3, 3);
}

// F = -a^(1+al) kIR^2 k^2 f - a^(3+al) Vp, with fx = f(x) and Vp = r2c(V'(f(x)));
// vsum3 = {sum V, sum dV/dgsq, sum dV/dmu} over the sites
int force(const Ctx &c, const void *f, double a, void *fx, void *Vp, void *F, double *vsum3) {
    int rc;
    if ((rc = c2r(c, f, fx))) return rc;
    if ((rc = model(c, 0, fx, nullptr, c.ws->hout, vsum3))) return rc;
    if ((rc = r2c(c, c.ws->hout, Vp))) return rc;
    CU(cudaMemsetAsync(F, 0, c.ws->carr, c.st));
    if ((rc = lin(c, F, f, 0.0, -std::pow(a, 1 + c.alpha) * c.kIR2))) return rc;
    return lin(c, F, Vp, -std::pow(a, 3 + c.alpha), 0.0);
}

double A_of(const Ctx &c, double a, double K, double G, double V) {
    const int al = c.alpha;
    return c.C * std::pow(a, 1 + 2 * al) * ((al - 2) * K + al * G + (al + 1) * V);
}

int energies(const Ctx &c, const void *f, const void *p, double a, double vsum, double *K, double *G, double *V) {
    int rc;
    if ((rc = zero_acc(c))) return rc;
    const long long n = (long long)c.nf * c.modes;
    if (c.prec == 32)
        ka_kg<float><<<c.grid, kThreads, 0, c.st>>>(n, c.modes, c.N, c.H, (const float2 *)f, (const float2 *)p,
                                                    c.ws->acc);
    else
        ka_kg<double><<<c.grid, kThreads, 0, c.st>>>(n, c.modes, c.N, c.H, (const double2 *)f, (const double2 *)p,
                                                     c.ws->acc);
    CU(cudaGetLastError());
    double v[2];
    if ((rc = read_acc(c, v, 2))) return rc;
    *K = .5 * v[0] / std::pow(a, 6) / (c.N3 * c.N3);
    double grad = c.kIR2 * v[1];
    grad /= c.N3;
    grad /= 2.;
    *G = grad / (a * a) / c.N3;
    *V = vsum / c.N3;
    return PSC_OK;
}

// one stage forward: (f, p, bg) -> (fo, po, bgo); the intermediates stay in the workspace
int stage_fwd(const Ctx &c, const void *f, const void *p, BG3 bg, double w, double dt, void *fo, void *po, BG3 *bgo,
              double *vsum1_3 = nullptr, double *KGV = nullptr) {
    AdjWS *ws = c.ws;
    const double c1 = w * dt / 2;
    const double bh = bg.b + c1 * bg.add;
    double v0[3];
    int rc;
    if ((rc = force(c, f, bg.a, ws->fx0, ws->Vp0, ws->F0, v0))) return rc;
    CU(cudaMemcpyAsync(ws->ph, p, ws->carr, cudaMemcpyDeviceToDevice, c.st));
    if ((rc = lin(c, ws->ph, ws->F0, c1, 0.0))) return rc;
    const double ah = bg.a + bh * w * dt / 2.;
    const double c2 = w * dt * std::pow(ah, c.alpha - 3);
    CU(cudaMemcpyAsync(fo, f, ws->carr, cudaMemcpyDeviceToDevice, c.st));
    if ((rc = lin(c, fo, ws->ph, c2, 0.0))) return rc;
    const double a1 = ah + bh * w * dt / 2.;
    double v1[3];
    if ((rc = force(c, fo, a1, ws->fx1, ws->Vp1, ws->F1, v1))) return rc;
    CU(cudaMemcpyAsync(po, ws->ph, ws->carr, cudaMemcpyDeviceToDevice, c.st));
    if ((rc = lin(c, po, ws->F1, c1, 0.0))) return rc;
    double K, G, V;
    if ((rc = energies(c, fo, po, a1, v1[0], &K, &G, &V))) return rc;
    bgo->a = a1;
    bgo->add = A_of(c, a1, K, G, V);
    bgo->b = bh + c1 * bgo->add;
    if (vsum1_3)
        for (int i = 0; i < 3; ++i) vsum1_3[i] = v1[i];
    if (KGV) {
        KGV[0] = K;
        KGV[1] = G;
        KGV[2] = V;
    }
    return PSC_OK;
}

struct Adj {
    double la, lb, ladd;
    double gth[2];
};

// (dF/df)^T applied to the adjoint array L at (fx, a), added with factor s into Lf;
// returns <lambda, dV'/dtheta> sums in th[2]
int jt_add(const Ctx &c, const void *fx, double a, const void *L, void *Lf, double s, double *th) {
    AdjWS *ws = c.ws;
    int rc;
    if ((rc = c2r(c, L, ws->lam))) return rc;
    double acc[3];
    if ((rc = model(c, 1, fx, ws->lam, ws->hout, acc))) return rc;
    if ((rc = r2c(c, ws->hout, ws->tmp))) return rc;
    if ((rc = lin(c, Lf, L, 0.0, -s * std::pow(a, 1 + c.alpha) * c.kIR2))) return rc;
    if ((rc = lin(c, Lf, ws->tmp, -s * std::pow(a, 3 + c.alpha), 0.0))) return rc;
    th[0] = acc[0];
    th[1] = acc[1];
    return PSC_OK;
}

// reverse one stage given its inputs (f, p, bg); ws->Lf, ws->Lp and adj hold the
// adjoint of the stage outputs on entry and of its inputs on return
int stage_adj(const Ctx &c, const void *f, const void *p, BG3 bg, double w, double dt, Adj *adj) {
    AdjWS *ws = c.ws;
    const int al = c.alpha;
    const double c1 = w * dt / 2;
    int rc;
    double vs1[3], kgv[3];
    BG3 o;
    if ((rc = stage_fwd(c, f, p, bg, w, dt, ws->f1, ws->p1, &o, vs1, kgv))) return rc;
    const double bh = bg.b + c1 * bg.add;
    const double ah = bg.a + bh * w * dt / 2.;
    const double c2 = w * dt * std::pow(ah, al - 3);
    const double a1 = o.a;
    const double K1 = kgv[0], G1 = kgv[1], V1 = kgv[2];
    // b1 = bh + c1 add1
    const double lat = adj->ladd + c1 * adj->lb;
    double lbh = adj->lb;
    double la1 = adj->la;
    // add1 = A(f1, p1, a1)
    const double Cc = c.C * std::pow(a1, 1 + 2 * al);
    if ((rc = lin(c, ws->Lf, ws->f1, 0.0, lat * Cc * al / (a1 * a1 * c.N3) * c.kIR2))) return rc;
    if ((rc = lin(c, ws->Lf, ws->Vp1, lat * Cc * (al + 1) / c.N3, 0.0))) return rc;
    if ((rc = lin(c, ws->Lp, ws->p1, lat * Cc * (al - 2) / (std::pow(a1, 6) * c.N3), 0.0))) return rc;
    la1 += lat * (c.C * (1 + 2 * al) * std::pow(a1, 2 * al) * ((al - 2) * K1 + al * G1 + (al + 1) * V1) +
                  Cc * ((al - 2) * (-6 * K1 / a1) + al * (-2 * G1 / a1)));
    adj->gth[0] += lat * Cc * (al + 1) * vs1[1] / c.N3;
    adj->gth[1] += lat * Cc * (al + 1) * vs1[2] / c.N3;
    // p1 = ph + c1 F1(f1, a1): dots with Lp1 first, then Lf += c1 J^T Lp1
    double d1, d2, th[2];
    if ((rc = dots(c, ws->Lp, ws->f1, ws->Vp1, &d1, &d2))) return rc;
    la1 += c1 * ((1 + al) * std::pow(a1, al) * (-c.kIR2) * d1 - (3 + al) * std::pow(a1, 2 + al) * d2);
    if ((rc = jt_add(c, ws->fx1, a1, ws->Lp, ws->Lf, c1, th))) return rc;
    adj->gth[0] += c1 * (-std::pow(a1, 3 + al)) * th[0];
    adj->gth[1] += c1 * (-std::pow(a1, 3 + al)) * th[1];
    // a1 = ah + bh w dt/2
    double lah = la1;
    lbh += la1 * w * dt / 2.;
    // f1 = f + c2(ah) ph: Lph (= Lp buffer) += c2 Lf; lah += <lambda_f1, ph> dc2/dah
    double d3;
    if ((rc = dots(c, ws->Lf, nullptr, ws->ph, nullptr, &d3))) return rc;
    lah += d3 * w * dt * (al - 3) * std::pow(ah, al - 4);
    if ((rc = lin(c, ws->Lp, ws->Lf, c2, 0.0))) return rc;
    // ah = a + bh w dt/2
    double la = lah;
    lbh += lah * w * dt / 2.;
    // ph = pi + c1 F0(f, a)
    if ((rc = dots(c, ws->Lp, f, ws->Vp0, &d1, &d2))) return rc;
    la += c1 * ((1 + al) * std::pow(bg.a, al) * (-c.kIR2) * d1 - (3 + al) * std::pow(bg.a, 2 + al) * d2);
    if ((rc = jt_add(c, ws->fx0, bg.a, ws->Lp, ws->Lf, c1, th))) return rc;
    adj->gth[0] += c1 * (-std::pow(bg.a, 3 + al)) * th[0];
    adj->gth[1] += c1 * (-std::pow(bg.a, 3 + al)) * th[1];
    // bh = b + c1 add
    adj->la = la;
    adj->lb = lbh;
    adj->ladd = c1 * lbh;
    return PSC_OK;
}

int setup(psc_handle *h, Ctx *c) {
    if (!h->adj) {
        AdjWS *ws = new AdjWS();
        h->adj = ws;
        h->adj_free = ws_free;
        const psc::Geo &g = h->cfg.g;
        ws->carr = (size_t)g.nf * g.modes * h->csize;
        ws->rarr = (size_t)g.nf * g.sites * (h->csize / 2);
        void **cs[] = {&ws->ph, &ws->f1, &ws->p1, &ws->F0, &ws->Vp0, &ws->F1, &ws->Vp1, &ws->Lf, &ws->Lp, &ws->tmp};
        for (void **q : cs)
            if (int rc = ws_alloc(ws, q, ws->carr)) return rc;
        void **rs[] = {&ws->fx0, &ws->fx1, &ws->lam, &ws->hout};
        for (void **q : rs)
            if (int rc = ws_alloc(ws, q, ws->rarr)) return rc;
        void *acc;
        if (int rc = ws_alloc(ws, &acc, sizeof(double) * 8)) return rc;
        ws->acc = static_cast<double *>(acc);
    }
    const psc::Geo &g = h->cfg.g;
    const psc_params &p = h->p0();
    c->h = h;
    c->ws = static_cast<AdjWS *>(h->adj);
    c->N = g.N;
    c->H = g.H;
    c->nf = g.nf;
    c->prec = p.precision;
    c->alpha = p.alpha;
    c->model = p.model;
    c->modes = g.modes;
    c->sites = g.sites;
    c->kIR2 = p.kIR * p.kIR;
    c->gsq = p.gsq;
    psc::DevBG bg;
    if (int rc = psc::hapi::read_bg(h, 0, &bg)) return rc;
    c->C = bg.fs_over_mpl2 / 3.0;
    c->N3 = (double)g.sites;
    c->st = h->st;
    c->grid = 4 * 152;
    return PSC_OK;
}

int check(psc_handle *h) {
    if (h->R != 1) return fail(PSC_ERR_CONFIG, "the adjoint works on single-lattice handles");
    if (h->cfg.g.N < 32) return fail(PSC_ERR_CONFIG, "the adjoint needs N >= 32");
    if (h->cfg.g.mask)
        return fail(PSC_ERR_CONFIG, "the adjoint differentiates the unmasked step (spectral = 0 or simulate_inflation = 0)");
    if (h->p0().expansion != 2) return fail(PSC_ERR_CONFIG, "the adjoint needs self-consistent expansion (expansion = 2)");
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state: call psc_init_ic or psc_set_state first");
    return PSC_OK;
}

}  // namespace

extern "C" int psc_adjoint_chi2(psc_handle *h, double dt, int nsteps, int every, double *O, double *grad_fk,
                                double *grad_pik, double *grad_ad0, double *grad_theta) {
    if (!h || !O || nsteps < 1 || !(dt > 0)) return fail(PSC_ERR_ARG, "bad argument");
    if (int rc = check(h)) return rc;
    if (every < 1) every = nsteps;
    Ctx c;
    int rc;
    if ((rc = setup(h, &c))) return rc;
    AdjWS *ws = c.ws;
    const int s = h->s;
    const double *w = h->w;
    const int nseg = (nsteps + every - 1) / every;
    // storage: checkpoints and one segment's stage inputs
    while ((int)ws->ckpt_f.size() < nseg) {
        void *a, *b;
        if ((rc = ws_alloc(ws, &a, ws->carr)) || (rc = ws_alloc(ws, &b, ws->carr))) return rc;
        ws->ckpt_f.push_back(a);
        ws->ckpt_p.push_back(b);
    }
    ws->ckpt_bg.assign(nseg, BG3{});
    const int tape_len = every * s;
    while ((int)ws->tape_f.size() < tape_len) {
        void *a, *b;
        if ((rc = ws_alloc(ws, &a, ws->carr)) || (rc = ws_alloc(ws, &b, ws->carr))) return rc;
        ws->tape_f.push_back(a);
        ws->tape_p.push_back(b);
    }
    ws->tape_bg.assign(tape_len, BG3{});
    // initial state; a''(0) consistent with it
    psc::DevBG dbg;
    if ((rc = psc::hapi::read_bg(h, 0, &dbg))) return rc;
    BG3 bg0{dbg.a, dbg.ad, 0.0};
    {
        double v[3], K, G, V;
        if ((rc = c2r(c, h->b.fk, ws->fx0))) return rc;
        if ((rc = model(c, 0, ws->fx0, nullptr, ws->hout, v))) return rc;
        if ((rc = energies(c, h->b.fk, h->b.pk, bg0.a, v[0], &K, &G, &V))) return rc;
        bg0.add = A_of(c, bg0.a, K, G, V);
    }
    // forward with checkpoints (the handle's arrays carry the state)
    void *curf = h->b.fk, *curp = h->b.pk;
    BG3 bg = bg0;
    for (int seg = 0, done = 0; seg < nseg; ++seg) {
        CU(cudaMemcpyAsync(ws->ckpt_f[seg], curf, ws->carr, cudaMemcpyDeviceToDevice, c.st));
        CU(cudaMemcpyAsync(ws->ckpt_p[seg], curp, ws->carr, cudaMemcpyDeviceToDevice, c.st));
        ws->ckpt_bg[seg] = bg;
        const int n = std::min(every, nsteps - done);
        for (int k = 0; k < n; ++k)
            for (int q = 0; q < s; ++q) {
                BG3 o;
                if ((rc = stage_fwd(c, curf, curp, bg, w[q], dt, ws->f1, ws->p1, &o, nullptr))) return rc;
                CU(cudaMemcpyAsync(curf, ws->f1, ws->carr, cudaMemcpyDeviceToDevice, c.st));
                CU(cudaMemcpyAsync(curp, ws->p1, ws->carr, cudaMemcpyDeviceToDevice, c.st));
                bg = o;
            }
        done += n;
    }
    // observable O = <chi^2> and its adjoint: Lambda_chi = r2c(2 chi / N^3) = 2 chi_k / N^3
    {
        if ((rc = c2r(c, curf, ws->fx1))) return rc;
        std::vector<double> chi;
        const size_t rbytes = (size_t)c.sites * (h->csize / 2);
        const char *last = static_cast<const char *>(ws->fx1) + (size_t)(c.nf - 1) * rbytes;
        chi.resize(c.sites);
        if ((rc = psc::hapi::download_real(h, chi.data(), last, (size_t)c.sites))) return rc;
        double acc = 0.0;
        for (double x : chi) acc += x * x;
        *O = acc / c.N3;
    }
    CU(cudaMemsetAsync(ws->Lf, 0, ws->carr, c.st));
    CU(cudaMemsetAsync(ws->Lp, 0, ws->carr, c.st));
    {
        const size_t one = (size_t)c.modes * h->csize;
        char *Lf_last = static_cast<char *>(ws->Lf) + (size_t)(c.nf - 1) * one;
        const char *f_last = static_cast<const char *>(curf) + (size_t)(c.nf - 1) * one;
        Ctx c1 = c;
        c1.nf = 1;
        if ((rc = lin(c1, Lf_last, f_last, 2.0 / c.N3, 0.0))) return rc;
    }
    Adj adj{0.0, 0.0, 0.0, {0.0, 0.0}};
    // reverse sweep over segments
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int n = std::min(every, nsteps - seg * every);
        // recompute the segment keeping every stage input
        CU(cudaMemcpyAsync(curf, ws->ckpt_f[seg], ws->carr, cudaMemcpyDeviceToDevice, c.st));
        CU(cudaMemcpyAsync(curp, ws->ckpt_p[seg], ws->carr, cudaMemcpyDeviceToDevice, c.st));
        bg = ws->ckpt_bg[seg];
        int t = 0;
        for (int k = 0; k < n; ++k)
            for (int q = 0; q < s; ++q, ++t) {
                CU(cudaMemcpyAsync(ws->tape_f[t], curf, ws->carr, cudaMemcpyDeviceToDevice, c.st));
                CU(cudaMemcpyAsync(ws->tape_p[t], curp, ws->carr, cudaMemcpyDeviceToDevice, c.st));
                ws->tape_bg[t] = bg;
                BG3 o;
                if ((rc = stage_fwd(c, curf, curp, bg, w[q], dt, ws->f1, ws->p1, &o, nullptr))) return rc;
                CU(cudaMemcpyAsync(curf, ws->f1, ws->carr, cudaMemcpyDeviceToDevice, c.st));
                CU(cudaMemcpyAsync(curp, ws->p1, ws->carr, cudaMemcpyDeviceToDevice, c.st));
                bg = o;
            }
        for (int k = n - 1; k >= 0; --k)
            for (int q = s - 1; q >= 0; --q) {
                const int ti = k * s + q;
                if ((rc = stage_adj(c, ws->tape_f[ti], ws->tape_p[ti], ws->tape_bg[ti], w[q], dt, &adj))) return rc;
            }
    }
    // a''(0) = A(f0, pi0, a0): fold its adjoint into the initial state
    {
        const void *f0 = ws->ckpt_f[0], *p0 = ws->ckpt_p[0];
        const int al = c.alpha;
        const double a0 = bg0.a;
        double v[3], K, G, V;
        if ((rc = c2r(c, f0, ws->fx0))) return rc;
        if ((rc = model(c, 0, ws->fx0, nullptr, ws->hout, v))) return rc;
        if ((rc = r2c(c, ws->hout, ws->Vp0))) return rc;
        if ((rc = energies(c, f0, p0, a0, v[0], &K, &G, &V))) return rc;
        const double Cc = c.C * std::pow(a0, 1 + 2 * al);
        const double l = adj.ladd;
        if ((rc = lin(c, ws->Lf, f0, 0.0, l * Cc * al / (a0 * a0 * c.N3) * c.kIR2))) return rc;
        if ((rc = lin(c, ws->Lf, ws->Vp0, l * Cc * (al + 1) / c.N3, 0.0))) return rc;
        if ((rc = lin(c, ws->Lp, p0, l * Cc * (al - 2) / (std::pow(a0, 6) * c.N3), 0.0))) return rc;
        adj.gth[0] += l * Cc * (al + 1) * v[1] / c.N3;
        adj.gth[1] += l * Cc * (al + 1) * v[2] / c.N3;
    }
    // gradients with respect to the stored half spectrum: (w_k / N^3) Lambda_k
    const size_t ncplx = (size_t)c.nf * c.modes;
    auto to_grad = [&](const void *L, double *out) -> int {
        if (!out) return PSC_OK;
        int r = psc::hapi::download_real(h, out, L, 2 * ncplx);
        if (r) return r;
        for (size_t i = 0; i < ncplx; ++i) {
            const int kz = (int)((i % c.modes) % c.H);
            const double wk = (kz == 0 || kz == c.H - 1) ? 1.0 : 2.0;
            out[2 * i] *= wk / c.N3;
            out[2 * i + 1] *= wk / c.N3;
        }
        return PSC_OK;
    };
    if ((rc = to_grad(ws->Lf, grad_fk)) || (rc = to_grad(ws->Lp, grad_pik))) return rc;
    if (grad_ad0) *grad_ad0 = adj.lb;
    if (grad_theta) {
        grad_theta[0] = adj.gth[0];
        grad_theta[1] = adj.gth[1];
    }
    // leave the handle at the final state, as psc_step would
    dbg.a = bg.a;
    dbg.ad = bg.b;
    dbg.add = bg.add;
    dbg.t += dt * nsteps;
    if ((rc = psc::hapi::write_bg(h, 0, dbg))) return rc;
    return psc::hapi::evaluate(h, 0);
}

// Forward only with the same stage sequence (for finite differences of the
// adjoint's own discrete map): O = <chi^2> after nsteps, a''(0) from the state.
extern "C" int psc_adjoint_forward_chi2(psc_handle *h, double dt, int nsteps, double *O) {
    if (!h || !O || nsteps < 1 || !(dt > 0)) return fail(PSC_ERR_ARG, "bad argument");
    if (int rc = check(h)) return rc;
    Ctx c;
    int rc;
    if ((rc = setup(h, &c))) return rc;
    AdjWS *ws = c.ws;
    psc::DevBG dbg;
    if ((rc = psc::hapi::read_bg(h, 0, &dbg))) return rc;
    BG3 bg{dbg.a, dbg.ad, 0.0};
    double v[3], K, G, V;
    if ((rc = c2r(c, h->b.fk, ws->fx0))) return rc;
    if ((rc = model(c, 0, ws->fx0, nullptr, ws->hout, v))) return rc;
    if ((rc = energies(c, h->b.fk, h->b.pk, bg.a, v[0], &K, &G, &V))) return rc;
    bg.add = A_of(c, bg.a, K, G, V);
    for (int k = 0; k < nsteps; ++k)
        for (int q = 0; q < h->s; ++q) {
            BG3 o;
            if ((rc = stage_fwd(c, h->b.fk, h->b.pk, bg, h->w[q], dt, ws->f1, ws->p1, &o, nullptr))) return rc;
            CU(cudaMemcpyAsync(h->b.fk, ws->f1, ws->carr, cudaMemcpyDeviceToDevice, c.st));
            CU(cudaMemcpyAsync(h->b.pk, ws->p1, ws->carr, cudaMemcpyDeviceToDevice, c.st));
            bg = o;
        }
    if ((rc = c2r(c, h->b.fk, ws->fx1))) return rc;
    std::vector<double> chi(c.sites);
    const char *last = static_cast<const char *>(ws->fx1) + (size_t)(c.nf - 1) * c.sites * (h->csize / 2);
    if ((rc = psc::hapi::download_real(h, chi.data(), last, (size_t)c.sites))) return rc;
    double acc = 0.0;
    for (double x : chi) acc += x * x;
    *O = acc / c.N3;
    dbg.a = bg.a;
    dbg.ad = bg.b;
    dbg.add = bg.add;
    dbg.t += dt * nsteps;
    if ((rc = psc::hapi::write_bg(h, 0, dbg))) return rc;
    return psc::hapi::evaluate(h, 0);
}
