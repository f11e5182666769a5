// psc_ic_gpu.cu — initial conditions generated on the device, one thread per mode,
// from the reference's own random stream.
//
// The reference draws from one sequential Park-Miller stream (initialize.cpp:13-28,
// x_{n+1} = 16807 x_n mod (2^31 - 1), the first call discarding 99 values) while it
// walks the modes in a fixed order (initialize.cpp:686-749 for each field, then
// 356-444 for the GW tensors). Draw n of the stream is 16807^n x_0 mod (2^31 - 1),
// so a thread that knows the position of its mode in the walk computes its draws
// directly (skip-ahead by binary powers). The integer draws are exactly the
// reference's; the FP64 mode arithmetic (set_mode initialize.cpp:128-220,
// set_mode_GW initialize.cpp:273-340) uses the device's sqrt/log/sin/cos, so values
// can differ from the host generator in the last bits.
//
// The walk writes every stored element exactly once (a visited mode or the complex
// conjugate a visit fills in), so the threads never collide.
#include <cmath>
#include <string>
#include <vector>

#include "psc_dev.cuh"
#include "psc_handle.h"
#include "psc_ic.h"

using psc::hapi::fail;

namespace {

constexpr unsigned long long kPM = 2147483647ull;   // 2^31 - 1
constexpr double kPi = 3.14159265358979323846;      // 2 asin(1), pspectcosmo.h:27

__device__ __forceinline__ unsigned long long mulmod(unsigned long long a, unsigned long long b) {
    unsigned long long p = a * b;   // < 2^62
    p = (p & kPM) + (p >> 31);
    p = (p & kPM) + (p >> 31);
    return p >= kPM ? p - kPM : p;
}

// 16807^n mod (2^31 - 1) from the table pw[b] = 16807^(2^b)
__device__ __forceinline__ unsigned long long pm_pow(unsigned long long n, const unsigned long long *pw) {
    unsigned long long r = 1;
    for (int b = 0; n; ++b, n >>= 1)
        if (n & 1ull) r = mulmod(r, pw[b]);
    return r;
}

struct ICDev {
    int N, H, nf, model, gw, simulate_inflation, dpm;
    double k2c, dp2, kIR, gsq, a, hubble, aop, norm_s, norm_gw, n3;
    double m2[PSC_MAX_FIELDS], f0[PSC_MAX_FIELDS], fd0[PSC_MAX_FIELDS];
    long long visits;
    unsigned long long x0;   // seed (>= 1)
    unsigned long long pw[64];
};

struct Visit {
    int i, j, k, px, py;
    long long conj;   // element of the conjugate copy, or -1
    bool real;
};

// position v of the walk -> mode (initialize.cpp:686-749; corner_skip = 1 for the GW
// walk, which leaves out the (0,0,0) corner)
__device__ Visit decode(long long v, int N, int H, int corner_skip) {
    Visit o;
    const int h = N / 2, h1 = N / 2 - 1;
    const long long SA = (long long)h1 * (N + 2), SB = (long long)h1 * N * N;
    auto id = [&](int i, int j, int k) { return ((long long)i * N + j) * H + k; };
    o.real = false;
    o.conj = -1;
    if (v < 2 * SA) {
        const int k = v < SA ? 0 : h;
        long long w = v < SA ? v : v - SA;
        o.k = k;
        if (w < 2 * h1) {                       // i in {0, N/2}, j = 1 .. N/2-1
            o.i = (int)(w / h1) * h;
            o.j = 1 + (int)(w % h1);
            o.conj = id(o.i, N - o.j, k);
        } else if ((w -= 2 * h1) < 2 * h1) {    // j in {0, N/2}, i = 1 .. N/2-1
            o.j = (int)(w / h1) * h;
            o.i = 1 + (int)(w % h1);
            o.conj = id(N - o.i, o.j, k);
        } else {                                // i = 1 .. N/2-1, j = 1 .. N/2-1, N/2+1 .. N-1
            w -= 2 * h1;
            o.i = 1 + (int)(w / (N - 2));
            const int jj = (int)(w % (N - 2));
            o.j = jj < h1 ? 1 + jj : jj + 2;
            o.conj = id(N - o.i, N - o.j, k);
        }
        o.px = o.i;
        o.py = o.j <= h ? o.j : o.j - N;
        return o;
    }
    v -= 2 * SA;
    if (v < SB) {   // interior planes kz = 1 .. N/2-1, every (i, j)
        o.k = 1 + (int)(v / ((long long)N * N));
        const long long w = v % ((long long)N * N);
        o.i = (int)(w / N);
        o.j = (int)(w % N);
        o.px = psc::pcoord(o.i, N);
        o.py = psc::pcoord(o.j, N);
        return o;
    }
    const int c = (int)(v - SB) + corner_skip;   // the eight real corners
    o.k = (c >> 2) * h;
    o.i = ((c >> 1) & 1) * h;
    o.j = (c & 1) * h;
    o.px = o.i;
    o.py = o.j;
    o.real = true;
    return o;
}

template <typename T>
__device__ __forceinline__ void put(psc::cplx<T> *a, long long m, double re, double im) {
    a[m] = psc::mk<T>((T)re, (T)im);
}

// scalar field fld: one thread per visit (set_mode, initialize.cpp:128-220)
template <typename T>
__global__ void __launch_bounds__(256) k_ic_scalar(const ICDev *__restrict__ d, int fld, psc::cplx<T> *__restrict__ fk,
                                                   psc::cplx<T> *__restrict__ pk) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= d->visits) return;
    const int N = d->N, H = d->H;
    const Visit o = decode(v, N, H, 0);
    const long long m = ((long long)o.i * N + o.j) * H + o.k;
    const double p2 = d->dp2 * (double)(o.px * o.px + o.py * o.py + o.k * o.k);
    double f0 = 0, f1 = 0, q0 = 0, q1 = 0;
    if (!(d->k2c > 0. && p2 > d->k2c)) {
        // draw n (0-based) of the stream is x_{100 + n} (99 discarded, then one advance)
        const unsigned long long n0 = 100ull + (unsigned long long)(fld * d->visits + v) * d->dpm;
        unsigned long long x = mulmod(pm_pow(n0, d->pw), d->x0);
        double r[4];
        for (int q = 0; q < d->dpm; ++q) {
            r[q] = (double)x / (double)kPM;
            x = mulmod(x, 16807ull);
        }
        const double a = d->a, H0 = d->hubble, m2 = d->m2[fld];
        const double omega = (p2 + m2 > 0.) ? sqrt(p2 + a * a * m2) : sqrt(p2);
        const double rms = omega > 0. ? d->norm_s / sqrt(omega) : 0.;
        const double aop = d->aop;
        if (d->simulate_inflation) {
            const double amp = rms / a;
            const double phase = 2. * kPi * r[0];
            const double re = amp * cos(phase), im = amp * sin(phase);
            f0 = re;
            f1 = im;
            q0 = aop * (-omega * im - H0 * f0);
            q1 = aop * (omega * re - H0 * f1);
            if (o.real) {
                f0 = sqrt(f0 * f0 + f1 * f1);
                f1 = 0;
                q0 = sqrt(q0 * q0 + q1 * q1);
                q1 = 0.;
            }
        } else {
            const double al = rms / sqrt(2.) * sqrt(log(1. / r[0])) / a;
            const double ar = rms / sqrt(2.) * sqrt(log(1. / r[1])) / a;
            double ph = 2. * kPi * r[2];
            const double rel = al * cos(ph), iml = al * sin(ph);
            ph = 2. * kPi * r[3];
            const double rer = ar * cos(ph), imr = ar * sin(ph);
            f0 = rel + rer;
            f1 = iml + imr;
            q0 = aop * (-omega * (iml - imr) - H0 * f0);
            q1 = aop * (omega * (rel - rer) - H0 * f1);
            if (o.real) f1 = q1 = 0.;
        }
    }
    if (m == 0) {   // the homogeneous mode (initialize.cpp:760-765)
        f0 = d->f0[fld] * d->n3;
        f1 = 0.;
        q0 = d->aop * d->fd0[fld] * d->n3;
        q1 = 0.;
    }
    put<T>(fk, m, f0, f1);
    put<T>(pk, m, q0, q1);
    if (o.conj >= 0) {
        put<T>(fk, o.conj, f0, -f1);
        put<T>(pk, o.conj, q0, -q1);
    }
}

// e_TT(k) of TT_tensors (initialize.cpp:66-122)
__device__ void tt_tensor(const double k[3], double e[3][3]) {
    const double kn = sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
    const double kh[3] = {k[0] / kn, k[1] / kn, k[2] / kn};
    double tmp[3] = {0, 0, 1};
    if (fabs(kh[0]) < 1e-9 && fabs(kh[1]) < 1e-9 && fabs(kh[2] - 1) < 1e-9) {
        tmp[1] = 1;
        tmp[2] = 0;
    }
    double u[3] = {kh[1] * tmp[2] - kh[2] * tmp[1], kh[2] * tmp[0] - kh[0] * tmp[2], kh[0] * tmp[1] - kh[1] * tmp[0]};
    const double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (int q = 0; q < 3; ++q) u[q] /= un;
    double w[3] = {kh[1] * u[2] - kh[2] * u[1], kh[2] * u[0] - kh[0] * u[2], kh[0] * u[1] - kh[1] * u[0]};
    const double wn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    for (int q = 0; q < 3; ++q) w[q] /= wn;
    for (int i = 0; i < 3; i++)
        if (u[i] < 0) {
            for (int q = 0; q < 3; ++q) u[q] = -u[q];
            break;
        }
    for (int i = 0; i < 3; i++)
        if (w[i] < 0) {
            for (int q = 0; q < 3; ++q) w[q] = -w[q];
            break;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) e[i][j] = u[i] * u[j] - w[i] * w[j] + u[i] * w[j] + w[i] * u[j];
}

// GW tensors: one thread per visit of the GW walk (set_mode_GW, initialize.cpp:273-340)
template <typename T>
__global__ void __launch_bounds__(256) k_ic_gw(const ICDev *__restrict__ d, psc::cplx<T> *__restrict__ uk,
                                               psc::cplx<T> *__restrict__ puk, long long modes) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= d->visits - 1) return;
    const int N = d->N, H = d->H;
    const Visit o = decode(v, N, H, 1);
    const long long m = ((long long)o.i * N + o.j) * H + o.k;
    const double k2 = d->dp2 * (double)(o.px * o.px + o.py * o.py + o.k * o.k);
    const int ci[6] = {0, 0, 0, 1, 1, 2}, cj[6] = {0, 1, 2, 1, 2, 2};
    double uv[6][2], pv[6][2];
    for (int q = 0; q < 6; ++q) uv[q][0] = uv[q][1] = pv[q][0] = pv[q][1] = 0.;
    if (!(d->k2c > 0. && k2 > d->k2c)) {
        const unsigned long long n0 =
            100ull + (unsigned long long)(d->nf * d->visits) * d->dpm + (unsigned long long)v * 4ull;
        unsigned long long x = mulmod(pm_pow(n0, d->pw), d->x0);
        double r[4];
        for (int q = 0; q < 4; ++q) {
            r[q] = (double)x / (double)kPM;
            x = mulmod(x, 16807ull);
        }
        const double kv[3] = {o.px * d->kIR, o.py * d->kIR, o.k * d->kIR};
        double e[3][3];
        tt_tensor(kv, e);
        const double a = d->a, H0 = d->hubble;
        const double k = sqrt(k2);
        const double rms = d->norm_gw / sqrt(k);
        const double al = rms / sqrt(2.) * sqrt(log(1. / r[0])) / a;
        const double ar = rms / sqrt(2.) * sqrt(log(1. / r[1])) / a;
        double ph = 2. * kPi * r[2];
        const double rel = al * cos(ph), iml = al * sin(ph);
        ph = 2. * kPi * r[3];
        const double rer = ar * cos(ph), imr = ar * sin(ph);
        for (int q = 0; q < 6; ++q) {
            const double ec = e[ci[q]][cj[q]];
            uv[q][0] = ec * (rel + rer);
            uv[q][1] = ec * (iml + imr);
            pv[q][0] = d->aop * (ec * (-k * (iml - imr) - H0 * uv[q][0]));
            pv[q][1] = d->aop * (ec * (k * (rel - rer) - H0 * uv[q][1]));
            if (o.real) uv[q][1] = pv[q][1] = 0.;
        }
    }
    for (int q = 0; q < 6; ++q) {
        put<T>(uk + q * modes, m, uv[q][0], uv[q][1]);
        put<T>(puk + q * modes, m, pv[q][0], pv[q][1]);
        if (o.conj >= 0) {
            put<T>(uk + q * modes, o.conj, uv[q][0], -uv[q][1]);
            put<T>(puk + q * modes, o.conj, pv[q][0], -pv[q][1]);
        }
    }
    if (v == 0)   // the (0,0,0) mode is not visited and is zero (initialize.cpp:456-460)
        for (int q = 0; q < 6; ++q) {
            put<T>(uk + q * modes, 0, 0., 0.);
            put<T>(puk + q * modes, 0, 0., 0.);
        }
}

#define CU(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) return fail(PSC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

namespace psc {

// Generate the initial state of realization r of the handle on the device; returns
// the background values the host generator would (initialize.cpp:649-670).
int ic_device(psc_handle *h, int r, ICInfo *info) {
    const psc_params &p = h->p[r];
    if (p.seed < 1) return fail(PSC_ERR_CONFIG, "the device generator needs seed >= 1");
    const ICSetup s = ic_setup(p);
    ICDev d{};
    d.N = s.N;
    d.H = s.H;
    d.nf = s.nf;
    d.model = s.model;
    d.gw = s.gw;
    d.simulate_inflation = s.simulate_inflation;
    d.dpm = s.dpm;
    d.k2c = s.k2c;
    d.dp2 = s.dp2;
    d.kIR = s.kIR;
    d.gsq = s.gsq;
    d.a = s.a;
    d.hubble = s.hubble;
    d.aop = s.aop;
    d.norm_s = s.norm_s;
    d.norm_gw = s.norm_gw;
    d.n3 = s.n3;
    for (int q = 0; q < PSC_MAX_FIELDS; ++q) {
        d.m2[q] = s.m2[q];
        d.f0[q] = s.f0[q];
        d.fd0[q] = s.fd0[q];
    }
    d.visits = s.visits;
    d.x0 = (unsigned long long)p.seed;
    unsigned long long b = 16807ull;
    for (int q = 0; q < 64; ++q) {
        d.pw[q] = b;
        b = (b * b) % kPM;
    }
    void *dd = nullptr;
    CU(cudaMallocAsync(&dd, sizeof(ICDev), h->st));
    CU(cudaMemcpyAsync(dd, &d, sizeof(ICDev), cudaMemcpyHostToDevice, h->st));
    const ICDev *dp = static_cast<const ICDev *>(dd);
    const psc::Geo &g = h->cfg.g;
    const long long nb = (s.visits + 255) / 256;
    char *fk = static_cast<char *>(h->b.fk) + (size_t)r * g.fstride * h->csize;
    char *pk = static_cast<char *>(h->b.pk) + (size_t)r * g.fstride * h->csize;
    const size_t one = (size_t)g.modes * h->csize;
    for (int fld = 0; fld < s.nf; ++fld) {
        if (p.precision == 32)
            k_ic_scalar<float><<<(unsigned)nb, 256, 0, h->st>>>(dp, fld, (float2 *)(fk + fld * one),
                                                                (float2 *)(pk + fld * one));
        else
            k_ic_scalar<double><<<(unsigned)nb, 256, 0, h->st>>>(dp, fld, (double2 *)(fk + fld * one),
                                                                 (double2 *)(pk + fld * one));
        CU(cudaGetLastError());
    }
    if (g.gw) {
        char *uk = static_cast<char *>(h->b.uk) + (size_t)r * g.gstride * h->csize;
        char *puk = static_cast<char *>(h->b.puk) + (size_t)r * g.gstride * h->csize;
        if (p.precision == 32)
            k_ic_gw<float><<<(unsigned)nb, 256, 0, h->st>>>(dp, (float2 *)uk, (float2 *)puk, g.modes);
        else
            k_ic_gw<double><<<(unsigned)nb, 256, 0, h->st>>>(dp, (double2 *)uk, (double2 *)puk, g.modes);
        CU(cudaGetLastError());
    }
    CU(cudaFreeAsync(dd, h->st));
    *info = s.info;
    return PSC_OK;
}

}  // namespace psc
