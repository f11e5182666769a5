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
// mu = 1), at a''(0) = A(state(0)).
//
// Forward map, stage j from point P_j (f, p, a, b = a', add = a'') to P_{j+1},
// c = w_j dt/2 and F(f, a) = -a^(1+al) kIR^2 k^2 f - a^(3+al) r2c(V'(f(x))):
//   bh = b + c add;  ph = p + c F_j;  ah = a + c bh;  f' = f + w dt ah^(al-3) ph
//   a' = ah + c bh;  p' = ph + c F_{j+1};  add' = A(f', p', a');  b' = bh + c add'
// A = (fStar/MPl)^2/3 a^(1+2al) ((al-2) K + al G + (al+1) V). It is run by the
// product's own stage kernels, which write a tape of every stage point (f, p, V'_k
// and the real fields f(x)) and of the background record.
//
// Reverse sweep. Adjoint arrays are carried as Lambda = r2c(lambda(x)), so
// <lambda, y> = (1/N^3) sum' w Re(conj Lambda Y) and the gradient with respect to
// a stored mode is (w_k/N^3) Lambda_k. The two transposed force Jacobians that meet
// at a stage point P_j (the closing kick of stage j-1 and the opening kick of stage
// j use the same F at the same f and a) are applied together, once, to
//   M = (c_{j-1} + c_j) Lp + c_{j-1} beta p_j,
// linear in the adjoint: J^T M = -a^(1+al) kIR^2 k^2 M - a^(3+al) r2c(V''(f) m),
// together with the a''-adjoint terms of point j (dA/df, dA/dp, dA/da). All scalar
// adjoint arithmetic runs in one-thread device kernels on a device record, so the
// sweep has no host round trip. Memory: checkpoints of the state every `every`
// steps; each segment is re-run once with the tape on, then reversed.
#include <algorithm>
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

constexpr int kEW = 4 * 152;   // blocks of the elementwise kernels (grid-stride)
constexpr int kThreads = 256;

// The elementwise kernels walk the half spectrum one row (fixed field, x, y; kz
// fastest, H entries) per warp: no integer division per element, coalesced rows.
// Per-lane partial sums of a row are in the field precision, FP64 across rows.
struct RowIdx {
    int N, H, lg;   // lg = log2(N)
    __device__ __forceinline__ int kxy2(int r) const {
        const int xy = r & ((N * N) - 1);
        const int x = xy >> lg, y = xy & (N - 1);
        const int px = psc::pcoord(x, N), py = psc::pcoord(y, N);
        return px * px + py * py;
    }
};

__device__ __forceinline__ void warp_rows(int *r0, int *rstep, int *lane) {
    *lane = threadIdx.x & 31;
    *r0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    *rstep = (gridDim.x * blockDim.x) >> 5;
}

// point: M = alpha1 Lp + alpha2 p;  Lp += beta p;  part += sum' w k^2 Re(conj M f)
template <typename T>
__global__ void __launch_bounds__(kThreads) ka_point(int rows, RowIdx ri, psc::cplx<T> *__restrict__ Lp,
                                                     const psc::cplx<T> *__restrict__ p,
                                                     const psc::cplx<T> *__restrict__ f, psc::cplx<T> *__restrict__ Mk,
                                                     const psc::DevAdj *__restrict__ ad, double *__restrict__ part) {
    const T a1 = (T)ad->alpha1, a2 = (T)ad->alpha2, be = (T)ad->beta;
    int r, rs, lane;
    warp_rows(&r, &rs, &lane);
    double acc[1] = {0.0};
    for (; r < rows; r += rs) {
        const int kxy = ri.kxy2(r);
        T racc = T(0);
        for (int kz = lane; kz < ri.H; kz += 32) {
            const long long i = (long long)r * ri.H + kz;
            const psc::cplx<T> l = Lp[i], q = p[i], fv = f[i];
            const psc::cplx<T> mv = psc::mk<T>(a1 * l.x + a2 * q.x, a1 * l.y + a2 * q.y);
            Mk[i] = mv;
            Lp[i] = psc::mk<T>(l.x + be * q.x, l.y + be * q.y);
            const T w = (kz == 0 || kz == ri.H - 1) ? T(1) : T(2);
            racc += w * (T)(kxy + kz * kz) * (mv.x * fv.x + mv.y * fv.y);
        }
        acc[0] += (double)racc;
    }
    psc::block_reduce_store<1>(acc, part, gridDim.x, blockIdx.x);
}

// stage: ph = p + kc (-kn1 k^2 f - kn2 Vp);  part += sum' w Re(conj Lf ph);  Lp += c2 Lf
template <typename T>
__global__ void __launch_bounds__(kThreads) ka_stage(int rows, RowIdx ri, const psc::cplx<T> *__restrict__ Lf,
                                                     psc::cplx<T> *__restrict__ Lp, const psc::cplx<T> *__restrict__ p,
                                                     const psc::cplx<T> *__restrict__ f,
                                                     const psc::cplx<T> *__restrict__ vp,
                                                     const psc::DevAdj *__restrict__ ad, double *__restrict__ part) {
    const T kc = (T)ad->kc, kn1 = (T)ad->kn1, kn2 = (T)ad->kn2, c2 = (T)ad->c2;
    int r, rs, lane;
    warp_rows(&r, &rs, &lane);
    double acc[1] = {0.0};
    for (; r < rows; r += rs) {
        const int kxy = ri.kxy2(r);
        T racc = T(0);
        for (int kz = lane; kz < ri.H; kz += 32) {
            const long long i = (long long)r * ri.H + kz;
            const psc::cplx<T> l = Lf[i], q = p[i], fv = f[i], v = vp[i];
            const T fl = -kn1 * (T)(kxy + kz * kz);
            const psc::cplx<T> ph =
                psc::mk<T>(q.x + kc * (fl * fv.x - kn2 * v.x), q.y + kc * (fl * fv.y - kn2 * v.y));
            const T w = (kz == 0 || kz == ri.H - 1) ? T(1) : T(2);
            racc += w * (l.x * ph.x + l.y * ph.y);
            psc::cplx<T> lp = Lp[i];
            lp.x += c2 * l.x;
            lp.y += c2 * l.y;
            Lp[i] = lp;
        }
        acc[0] += (double)racc;
    }
    psc::block_reduce_store<1>(acc, part, gridDim.x, blockIdx.x);
}

// observable: part += sum' w |chi_k|^2 and, when Lf is given, Lf = 2 chi_k / N^3
template <typename T>
__global__ void __launch_bounds__(kThreads) ka_observable(int rows, RowIdx ri, const psc::cplx<T> *__restrict__ chi,
                                                          psc::cplx<T> *__restrict__ Lf, double scale,
                                                          double *__restrict__ part) {
    int r, rs, lane;
    warp_rows(&r, &rs, &lane);
    double acc[1] = {0.0};
    for (; r < rows; r += rs) {
        double racc = 0.0;
        for (int kz = lane; kz < ri.H; kz += 32) {
            const long long i = (long long)r * ri.H + kz;
            const psc::cplx<T> c = chi[i];
            const double w = (kz == 0 || kz == ri.H - 1) ? 1.0 : 2.0;
            racc += w * ((double)c.x * c.x + (double)c.y * c.y);
            if (Lf) Lf[i] = psc::mk<T>((T)(scale * c.x), (T)(scale * c.y));
        }
        acc[0] += racc;
    }
    psc::block_reduce_store<1>(acc, part, gridDim.x, blockIdx.x);
}

// GW point: Mu = alpha1 Lpu (the merged kicks' adjoint), Lu += eta1 k^2 Mu,
// part += sum' w Re(conj Mu Fu), Fu = -kIR^2 k^2 u + S_k from the tape (six components)
template <typename T>
__global__ void __launch_bounds__(kThreads) ka_point_gw(int rows, RowIdx ri, const psc::cplx<T> *__restrict__ Lpu,
                                                        psc::cplx<T> *__restrict__ Lu,
                                                        const psc::cplx<T> *__restrict__ fu,
                                                        psc::cplx<T> *__restrict__ Mu,
                                                        const psc::DevAdj *__restrict__ ad, double *__restrict__ part) {
    const T a1 = (T)ad->alpha1, e1 = (T)ad->eta1;
    int r, rs, lane;
    warp_rows(&r, &rs, &lane);
    double acc[1] = {0.0};
    for (; r < rows; r += rs) {
        const int kxy = ri.kxy2(r);
        T racc = T(0);
        for (int kz = lane; kz < ri.H; kz += 32) {
            const long long i = (long long)r * ri.H + kz;
            const psc::cplx<T> l = Lpu[i], fv = fu[i];
            psc::cplx<T> lu = Lu[i];
            const psc::cplx<T> mv = psc::mk<T>(a1 * l.x, a1 * l.y);
            const T k2 = (T)(kxy + kz * kz);
            Mu[i] = mv;
            lu.x += e1 * k2 * mv.x;
            lu.y += e1 * k2 * mv.y;
            Lu[i] = lu;
            const T w = (kz == 0 || kz == ri.H - 1) ? T(1) : T(2);
            racc += w * (mv.x * fv.x + mv.y * fv.y);
        }
        acc[0] += (double)racc;
    }
    psc::block_reduce_store<1>(acc, part, gridDim.x, blockIdx.x);
}

// GW stage: pu_half = pu + kfu Fu;  part += sum' w Re(conj Lu pu_half);  Lpu += c2 Lu
template <typename T>
__global__ void __launch_bounds__(kThreads) ka_stage_gw(int rows, RowIdx ri, const psc::cplx<T> *__restrict__ Lu,
                                                        psc::cplx<T> *__restrict__ Lpu,
                                                        const psc::cplx<T> *__restrict__ pu,
                                                        const psc::cplx<T> *__restrict__ fu,
                                                        const psc::DevAdj *__restrict__ ad, double *__restrict__ part) {
    const T kf = (T)ad->kfu, c2 = (T)ad->c2;
    int r, rs, lane;
    warp_rows(&r, &rs, &lane);
    double acc[1] = {0.0};
    for (; r < rows; r += rs) {
        T racc = T(0);
        for (int kz = lane; kz < ri.H; kz += 32) {
            const long long i = (long long)r * ri.H + kz;
            const psc::cplx<T> l = Lu[i], q = pu[i], fv = fu[i];
            psc::cplx<T> lp = Lpu[i];
            const T w = (kz == 0 || kz == ri.H - 1) ? T(1) : T(2);
            racc += w * (l.x * (q.x + kf * fv.x) + l.y * (q.y + kf * fv.y));
            lp.x += c2 * l.x;
            lp.y += c2 * l.y;
            Lpu[i] = lp;
        }
        acc[0] += (double)racc;
    }
    psc::block_reduce_store<1>(acc, part, gridDim.x, blockIdx.x);
}

// rho_GW of energy() (output.cpp:1030-1060) and its adjoint seed, one row (x, y) per
// warp: q_k = sum_ij |(P U)_ij|^2 - |tr P U|^2 / 2 with P = 1 - khat khat (spectra()'s
// projection, output.cpp:18-53), weighted as spectra()'s walk visits the stored modes
// (interior 2; on the kz = 0, N/2 planes the "+" half 2, the real corners 1, the rest 0),
// hz = sum |pi_u_ab(0)|^2 at k = 0. part += sum wq q; Lpu = fac 2 N^3 (wq / w) dq/d conj(U),
// fac = (fStar/MPl)^2 / (4 N^6 a^6).
template <typename T>
__global__ void __launch_bounds__(kThreads) ka_seed_gw(RowIdx ri, long long modes, const psc::cplx<T> *__restrict__ puk,
                                                       psc::cplx<T> *__restrict__ Lpu,
                                                       const psc::DevBG *__restrict__ fin, double n3,
                                                       double *__restrict__ part) {
    const int N = ri.N, h = N / 2, rows = N * N;
    const double kIR = fin->kIR, a = fin->a;
    const double fac = fin->fs_over_mpl2 / (4.0 * n3 * n3 * psc::ipow(a, 6));
    const int si[6] = {0, 0, 0, 1, 1, 2}, sj[6] = {0, 1, 2, 1, 2, 2};
    const int sy[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    int r, rs, lane;
    warp_rows(&r, &rs, &lane);
    double acc[1] = {0.0};
    for (; r < rows; r += rs) {
        const int x = r >> ri.lg, y = r & (N - 1);
        for (int kz = lane; kz < ri.H; kz += 32) {
            const long long m = (long long)r * ri.H + kz;
            double cr[6], ci[6];
            for (int c = 0; c < 6; ++c) {
                const psc::cplx<T> v = puk[c * modes + m];
                cr[c] = (double)v.x;
                ci[c] = (double)v.y;
            }
            const bool plane = (kz == 0 || kz == h);
            double wq = 2.0;
            if (plane) {
                if (x >= 1 && x < h) wq = 2.0;
                else if (x == 0 || x == h) wq = (y >= 1 && y < h) ? 2.0 : ((y == 0 || y == h) ? 1.0 : 0.0);
                else wq = 0.0;
            }
            const double wk = plane ? 1.0 : 2.0;
            double gr[6], gi[6], q;
            if (x == 0 && y == 0 && kz == 0) {
                q = 0.0;
                for (int c = 0; c < 6; ++c) {
                    const double mult = (si[c] == sj[c]) ? 1.0 : 2.0;
                    q += mult * (cr[c] * cr[c] + ci[c] * ci[c]);
                    gr[c] = mult * cr[c];
                    gi[c] = mult * ci[c];
                }
            } else {
                const double kv[3] = {kIR * psc::pcoord(x, N), kIR * psc::pcoord(y, N), kIR * kz};
                const double kn = sqrt(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
                double P[3][3];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) P[i][j] = (i == j ? 1.0 : 0.0) - (kv[i] / kn) * (kv[j] / kn);
                double Vr[3][3], Vi[3][3];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        double vr = 0, vi = 0;
                        for (int k = 0; k < 3; ++k) {
                            vr += P[i][k] * cr[sy[k][j]];
                            vi += P[i][k] * ci[sy[k][j]];
                        }
                        Vr[i][j] = vr;
                        Vi[i][j] = vi;
                    }
                const double tr = Vr[0][0] + Vr[1][1] + Vr[2][2], ti = Vi[0][0] + Vi[1][1] + Vi[2][2];
                q = -(tr * tr + ti * ti) / 2;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) q += Vr[i][j] * Vr[i][j] + Vi[i][j] * Vi[i][j];
                for (int c = 0; c < 6; ++c) {
                    const int i = si[c], j = sj[c];
                    double xr = Vr[i][j] - 0.5 * tr * P[i][j], xi = Vi[i][j] - 0.5 * ti * P[i][j];
                    if (i != j) {
                        xr += Vr[j][i] - 0.5 * tr * P[j][i];
                        xi += Vi[j][i] - 0.5 * ti * P[j][i];
                    }
                    gr[c] = xr;
                    gi[c] = xi;
                }
            }
            acc[0] += wq * q;
            const double s = fac * 2.0 * n3 * wq / wk;
            for (int c = 0; c < 6; ++c) Lpu[c * modes + m] = psc::mk<T>((T)(s * gr[c]), (T)(s * gi[c]));
        }
    }
    psc::block_reduce_store<1>(acc, part, gridDim.x, blockIdx.x);
}

enum AdjMode { ADJ_INIT = 0, ADJ_PRE = 1, ADJ_POST = 2, ADJ_STAGE_PRE = 3, ADJ_STAGE_POST = 4, ADJ_INIT_GW = 5 };

struct AdjArgs {
    int mode;
    int i;           // local point / stage index within the segment
    long long j;     // global point / stage index
    double n3;       // N^3
    // partial-sum regions: [offset, count]
    int d1_off, d1_n, z_off, z_n, d3_off, d3_n, o_off, o_n, dg_off, d3g_off;
    int gw;     // the GW adjoint runs (rho_GW observable)
    int last;   // the final point: no stage after it, only its GW kick adjoint
};

__device__ double block_sum(const double *__restrict__ v, int n, double *red) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += v[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

struct PointBG {
    double a, b, add, K, G, V, dVg, dVm;
};

// snapshots of the segment: snap[0] at its first point, snap[1] after the opening
// of stage 0, snap[i + 2] after the end of local stage i (evolution.cpp:1141-1197)
__device__ PointBG point_bg(const psc::DevBG *snap, int i) {
    const psc::DevBG &r = i == 0 ? snap[0] : snap[i + 1];
    PointBG o;
    o.a = i == 0 ? snap[0].a : snap[i].a;
    o.b = i == 0 ? snap[0].ad : r.b;
    o.add = r.add;
    o.K = 0;
    o.G = 0;
    for (int f = 0; f < r.nf; ++f) {
        o.K += r.K[f];
        o.G += r.G[f];
    }
    o.V = 0;
    for (int t = 0; t < r.nterms; ++t) o.V += r.V[t];
    o.dVm = r.V[0];
    o.dVg = (r.model == PSC_MODEL_PHI2CHI2) ? r.V[1] / r.gsq : 0.0;
    return o;
}

__global__ void __launch_bounds__(256) k_adj(AdjArgs A, psc::DevAdj *__restrict__ ad, const psc::DevBG *__restrict__ snap,
                                             const double *__restrict__ part) {
    __shared__ double red[256];
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (A.mode == ADJ_INIT || A.mode == ADJ_INIT_GW) s[0] = block_sum(part + A.o_off, A.o_n, red);
    if (A.mode == ADJ_POST) {
        if (!A.last) {
            s[0] = block_sum(part + A.d1_off, A.d1_n, red);
            for (int q = 0; q < 3; ++q) s[1 + q] = block_sum(part + A.z_off + q * A.z_n, A.z_n, red);
        }
        if (A.gw) s[4] = block_sum(part + A.dg_off, A.d1_n, red);
    }
    if (A.mode == ADJ_STAGE_POST) {
        s[0] = block_sum(part + A.d3_off, A.d3_n, red);
        if (A.gw) s[0] += block_sum(part + A.d3g_off, A.d3_n, red);
    }
    if (threadIdx.x != 0) return;
    const psc::DevBG &g0 = snap[0];
    const int al = g0.alpha, ns = g0.s;
    const double dt = g0.dt, kIR2 = g0.kIR2, C = g0.fs_over_mpl2 / 3.0, n3 = A.n3;
    if (A.mode == ADJ_INIT || A.mode == ADJ_INIT_GW) {
        ad->la = ad->lb = ad->ladd = ad->lbh = ad->lat = 0.0;
        ad->gth[0] = ad->gth[1] = 0.0;
        if (A.mode == ADJ_INIT) {
            ad->O = s[0] / (n3 * n3);   // <chi^2> by Parseval
        } else {
            // rho_GW = (fStar/MPl)^2 / (4 N^6 a^6) sum wq q; its a-adjoint -6 rho_GW / a
            const double a = g0.a;
            ad->O = g0.fs_over_mpl2 / (4.0 * n3 * n3 * psc::ipow(a, 6)) * s[0];
            ad->la = -6.0 * ad->O / a;
        }
        return;
    }
    const int q = (int)(A.j % ns);
    const double c = A.last ? 0.0 : g0.w[q] * dt / 2;   // the stage after the point (none after the last)
    const PointBG P = point_bg(snap, A.i);
    const double a = P.a;
    if (A.mode == ADJ_PRE) {
        const double cb = A.j > 0 ? g0.w[(q + ns - 1) % ns] * dt / 2 : 0.0;
        const double lat = ad->ladd + cb * ad->lb;
        ad->lat = lat;
        ad->lbh = ad->lb;
        const double Cc = C * psc::ipow(a, 1 + 2 * al);
        const double beta = lat * Cc * (al - 2) / (psc::ipow(a, 6) * n3);
        ad->beta = beta;
        ad->alpha1 = c + cb;
        ad->alpha2 = cb * beta;
        ad->gamma = lat * Cc * (al + 1) / n3;
        ad->delta = lat * Cc * al * kIR2 / (a * a * n3);
        ad->eta1 = -psc::ipow(a, 1 + al) * kIR2;
        ad->eta2 = -psc::ipow(a, 3 + al);
        ad->etaS = -psc::ipow(a, 1 + al);
        ad->la += lat * (C * (1 + 2 * al) * psc::ipow(a, 2 * al) * ((al - 2) * P.K + al * P.G + (al + 1) * P.V) +
                         Cc * ((al - 2) * (-6 * P.K / a) + al * (-2 * P.G / a)));
        ad->gth[0] += lat * Cc * (al + 1) * P.dVg;
        ad->gth[1] += lat * Cc * (al + 1) * P.dVm;
        return;
    }
    if (A.mode == ADJ_POST) {
        if (A.last) {   // the final point: only the closing GW kick of the last stage
            if (A.gw) ad->la += (1 + al) * psc::ipow(a, al) * s[4] / n3;
            return;
        }
        const double d1 = s[0] / n3, d2 = s[1];
        ad->la += (1 + al) * psc::ipow(a, al) * (-kIR2) * d1 - (3 + al) * psc::ipow(a, 2 + al) * d2;
        const double e2 = -psc::ipow(a, 3 + al);
        ad->gth[0] += e2 * s[2];
        ad->gth[1] += e2 * s[3];
        // GW kicks: dF_u/da = (1 + alpha) a^alpha (-kIR^2 k^2 u + S_k)
        if (A.gw) ad->la += (1 + al) * psc::ipow(a, al) * s[4] / n3;
        return;
    }
    if (A.mode == ADJ_STAGE_PRE) {
        ad->lbh += c * ad->la;
        ad->c2 = snap[A.i + 1].c_drift;
        ad->kc = c;
        ad->kn1 = psc::ipow(a, 1 + al) * kIR2;
        ad->kn2 = psc::ipow(a, 3 + al);
        ad->kfu = c * psc::ipow(a, 1 + al);
        return;
    }
    // ADJ_STAGE_POST
    const double d3 = s[0] / n3;
    const double bh = snap[A.i + 1].b_half;
    const double ah = a + bh * g0.w[q] * dt / 2.;
    ad->la += d3 * g0.w[q] * dt * (al - 3) * psc::ipow(ah, al - 4);
    ad->lbh += c * ad->la;
    ad->lb = ad->lbh;
    ad->ladd = c * ad->lbh;
}

struct AdjWS {
    size_t carr = 0, rarr = 0;   // bytes of nf complex / real arrays
    size_t garr = 0;             // bytes of the six GW component arrays (0 without GWs)
    void *M = nullptr, *Lf = nullptr, *Lp = nullptr;
    void *Mu = nullptr, *Lu = nullptr, *Lpu = nullptr, *Tarr = nullptr;   // GW adjoint
    psc::DevBG *fin = nullptr;   // the background at the final point
    double *part = nullptr;
    psc::DevAdj *rec = nullptr;
    psc::DevBG *snap = nullptr;
    int snap_n = 0;
    char *tape = nullptr;   // points x (f, p, vp, fx)
    int tape_n = 0;
    size_t tape_stride = 0;
    char *ckpt = nullptr;   // checkpoints x (f, p, bg)
    int ckpt_n = 0;
    size_t ckpt_stride = 0;
    int z_n = 0, part_n = 0;
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

int ws_grow(AdjWS *ws, char **ptr, int *have, int want, size_t stride) {
    if (*have >= want) return PSC_OK;
    if (*ptr) {
        auto it = std::find(ws->owned.begin(), ws->owned.end(), (void *)*ptr);
        if (it != ws->owned.end()) ws->owned.erase(it);
        cudaFree(*ptr);
        *ptr = nullptr;
        *have = 0;
    }
    void *p = nullptr;
    if (int rc = ws_alloc(ws, &p, stride * (size_t)want)) return rc;
    *ptr = static_cast<char *>(p);
    *have = want;
    return PSC_OK;
}

int check(psc_handle *h, int obs) {
    const psc_params &p = h->p0();
    if (obs != PSC_OBS_CHI2 && obs != PSC_OBS_RHO_GW) return fail(PSC_ERR_ARG, "unknown observable");
    if (h->R != 1) return fail(PSC_ERR_CONFIG, "the adjoint works on single-lattice handles");
    if (h->padded) return fail(PSC_ERR_CONFIG, "the adjoint differentiates the unpadded step (N_pad = 0)");
    h->force_valid = false;   // the reverse sweep rewrites the stage buffers
    if (!h->cfg.g.reg) return fail(PSC_ERR_CONFIG, "the adjoint needs the register engine (a power-of-two N >= 32)");
    if (h->cfg.g.mask)
        return fail(PSC_ERR_CONFIG, "the adjoint differentiates the unmasked step (spectral = 0 or simulate_inflation = 0)");
    if (p.expansion != 2) return fail(PSC_ERR_CONFIG, "the adjoint needs self-consistent expansion (expansion = 2)");
    if (obs == PSC_OBS_RHO_GW && !p.with_gw) return fail(PSC_ERR_CONFIG, "the rho_GW observable needs with_gw = 1");
    if (p.with_gw && p.spectral)
        return fail(PSC_ERR_CONFIG, "the adjoint differentiates evolved GW tensors (spectral = 0 with GWs)");
    if (p.with_gw && h->cfg.g.N > 512) return fail(PSC_ERR_CONFIG, "the adjoint with GWs needs N <= 512");
    if (psc::model_is_user(p.model))
        return fail(PSC_ERR_CONFIG, "the adjoint differentiates the built-in models (V'' and the coupling derivatives are "
                                    "written for them)");
    if (p.model == PSC_MODEL_PHI2CHI2 && !(p.gsq > 0)) return fail(PSC_ERR_CONFIG, "the adjoint needs gsq > 0");
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state: call psc_init_ic or psc_set_state first");
    return PSC_OK;
}

struct Run {
    psc_handle *h;
    AdjWS *ws;
    cudaStream_t st;
    int prec, nf, N, H;
    long long modes, n;   // n = nf * modes
    double n3;
    int z_n;
    RowIdx ri;
    bool gw;      // the handle evolves GWs (tape of pi_u and the GW force)
    bool gwadj;   // the GW adjoint runs (rho_GW observable)
};

int setup(psc_handle *h, Run *r) {
    if (!h->adj) {
        h->adj = new AdjWS();
        h->adj_free = ws_free;
    }
    AdjWS *ws = static_cast<AdjWS *>(h->adj);
    const psc::Geo &g = h->cfg.g;
    if (!ws->M) {
        ws->carr = (size_t)g.nf * g.modes * h->csize;
        ws->rarr = (size_t)g.nf * g.sites * (h->csize / 2);
        ws->garr = g.gw ? (size_t)6 * g.modes * h->csize : 0;
        void **cs[] = {&ws->M, &ws->Lf, &ws->Lp};
        for (void **q : cs)
            if (int rc = ws_alloc(ws, q, ws->carr)) return rc;
        if (g.gw) {
            void **gs[] = {&ws->Mu, &ws->Lu, &ws->Lpu};
            for (void **q : gs)
                if (int rc = ws_alloc(ws, q, ws->garr)) return rc;
            if (int rc = ws_alloc(ws, &ws->Tarr, (size_t)3 * ws->carr)) return rc;
        }
        ws->z_n = psc::adj_z_blocks(g.N, g.nf);   // the scalar adjoint Z pass's grid
        ws->part_n = 5 * kEW + 3 * ws->z_n;
        void *p;
        if (int rc = ws_alloc(ws, &p, sizeof(double) * ws->part_n)) return rc;
        ws->part = static_cast<double *>(p);
        if (int rc = ws_alloc(ws, &p, sizeof(psc::DevAdj))) return rc;
        ws->rec = static_cast<psc::DevAdj *>(p);
        if (int rc = ws_alloc(ws, &p, sizeof(psc::DevBG))) return rc;
        ws->fin = static_cast<psc::DevBG *>(p);
        ws->tape_stride = 3 * ws->carr + ws->rarr + 2 * ws->garr;
        ws->ckpt_stride = 2 * ws->carr + 2 * ws->garr + ((sizeof(psc::DevBG) + 255) / 256) * 256;
    }
    r->h = h;
    r->ws = ws;
    r->st = h->st;
    r->prec = h->p0().precision;
    r->nf = g.nf;
    r->N = g.N;
    r->H = g.H;
    r->modes = g.modes;
    r->n = (long long)g.nf * g.modes;
    r->n3 = (double)g.sites;
    r->z_n = ws->z_n;
    int lg = 0;
    while ((1 << lg) < g.N) ++lg;
    r->ri = RowIdx{g.N, g.H, lg};
    r->gw = g.gw != 0;
    r->gwadj = false;
    return PSC_OK;
}

AdjArgs args(const Run &r, int mode, int i, long long j) {
    AdjArgs A;
    A.mode = mode;
    A.i = i;
    A.j = j;
    A.n3 = r.n3;
    A.d1_off = 0;
    A.d1_n = kEW;
    A.z_off = kEW;
    A.z_n = r.z_n;
    A.d3_off = kEW + 3 * r.z_n;
    A.d3_n = kEW;
    A.o_off = 2 * kEW + 3 * r.z_n;
    A.o_n = kEW;
    A.dg_off = 3 * kEW + 3 * r.z_n;
    A.d3g_off = 4 * kEW + 3 * r.z_n;
    A.gw = r.gwadj ? 1 : 0;
    A.last = 0;
    return A;
}

int scalar(const Run &r, int mode, int i, long long j, const psc::DevBG *snap = nullptr, bool last = false) {
    AdjArgs A = args(r, mode, i, j);
    A.last = last ? 1 : 0;
    k_adj<<<1, 256, 0, r.st>>>(A, r.ws->rec, snap ? snap : r.ws->snap, r.ws->part);
    CU(cudaGetLastError());
    return PSC_OK;
}

char *tape_pt(const Run &r, int i) { return r.ws->tape + (size_t)i * r.ws->tape_stride; }
void *tp_f(const Run &r, int i) { return tape_pt(r, i); }
void *tp_p(const Run &r, int i) { return tape_pt(r, i) + r.ws->carr; }
void *tp_vp(const Run &r, int i) { return tape_pt(r, i) + 2 * r.ws->carr; }
void *tp_fx(const Run &r, int i) { return tape_pt(r, i) + 3 * r.ws->carr; }
void *tp_pu(const Run &r, int i) { return tape_pt(r, i) + 3 * r.ws->carr + r.ws->rarr; }
void *tp_fu(const Run &r, int i) { return tape_pt(r, i) + 3 * r.ws->carr + r.ws->rarr + r.ws->garr; }

// rho_GW from the handle's current pi_u and its adjoint seed into Lpu (and the a seed)
int observable_gw(const Run &r, void *Lpu) {
    CU(cudaMemcpyAsync(r.ws->fin, r.h->b.bg, sizeof(psc::DevBG), cudaMemcpyDeviceToDevice, r.st));
    double *part = r.ws->part + 2 * kEW + 3 * r.z_n;
    if (r.prec == 32)
        ka_seed_gw<float><<<kEW, kThreads, 0, r.st>>>(r.ri, r.modes, (const float2 *)r.h->b.puk, (float2 *)Lpu,
                                                      r.ws->fin, r.n3, part);
    else
        ka_seed_gw<double><<<kEW, kThreads, 0, r.st>>>(r.ri, r.modes, (const double2 *)r.h->b.puk, (double2 *)Lpu,
                                                       r.ws->fin, r.n3, part);
    CU(cudaGetLastError());
    return scalar(r, ADJ_INIT_GW, 0, 0, r.ws->fin);
}

// O from the handle's current state (Parseval: <chi^2> = sum' w |chi_k|^2 / N^6)
// and, with Lf_last, the adjoint seed Lambda_chi = r2c(2 chi / N^3) = 2 chi_k / N^3
int observable(const Run &r, void *Lf_last) {
    const size_t one = (size_t)r.modes * r.h->csize;
    const void *chi = static_cast<const char *>(r.h->b.fk) + (size_t)(r.nf - 1) * one;
    double *part = r.ws->part + 2 * kEW + 3 * r.z_n;
    const int rows = r.N * r.N;
    if (r.prec == 32)
        ka_observable<float><<<kEW, kThreads, 0, r.st>>>(rows, r.ri, (const float2 *)chi, (float2 *)Lf_last, 2.0 / r.n3,
                                                         part);
    else
        ka_observable<double><<<kEW, kThreads, 0, r.st>>>(rows, r.ri, (const double2 *)chi, (double2 *)Lf_last,
                                                          2.0 / r.n3, part);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(r.ws->fin, r.h->b.bg, sizeof(psc::DevBG), cudaMemcpyDeviceToDevice, r.st));
    return scalar(r, ADJ_INIT, 0, 0, r.ws->fin);
}

// the product's step sequence for n steps from the handle's state, writing the tape
// of points 0 .. n s - 1 and the background snapshots
int forward_taped(const Run &r, double dt, int n) {
    psc_handle *h = r.h;
    AdjWS *ws = r.ws;
    const int s = h->s, npts = n * s;
    psc::Buffers bt = h->b;
    auto tape_at = [&](int i) {
        if (i <= npts) {
            bt.tape_f = tp_f(r, i);
            bt.tape_p = tp_p(r, i);
            bt.tape_vp = tp_vp(r, i);
            bt.tape_fx = tp_fx(r, i);
            bt.tape_pu = r.gw ? tp_pu(r, i) : nullptr;
            bt.tape_fu = r.gw ? tp_fu(r, i) : nullptr;
        } else {
            bt.tape_f = bt.tape_p = bt.tape_vp = bt.tape_fx = bt.tape_pu = bt.tape_fu = nullptr;
        }
    };
    CU(psc::launch_set_run(h->b.bg, 1, dt, n, r.st));
    CU(cudaMemcpyAsync(ws->snap + 0, h->b.bg, sizeof(psc::DevBG), cudaMemcpyDeviceToDevice, r.st));
    CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_PRIME, 0, r.st));
    tape_at(0);
    CU(psc::launch_stage(h->cfg, bt, r.prec, 0, r.st));
    CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_BEGIN, 0, r.st));
    CU(cudaMemcpyAsync(ws->snap + 1, h->b.bg, sizeof(psc::DevBG), cudaMemcpyDeviceToDevice, r.st));
    for (int i = 0; i < npts; ++i) {
        tape_at(i + 1);
        CU(psc::launch_stage(h->cfg, bt, r.prec, 1, r.st));
        CU(psc::launch_scalar(h->cfg, h->b, psc::SCALAR_END, i % s, r.st));
        CU(cudaMemcpyAsync(ws->snap + i + 2, h->b.bg, sizeof(psc::DevBG), cudaMemcpyDeviceToDevice, r.st));
    }
    return PSC_OK;
}

template <typename T>
int reverse_segment_t(const Run &r, long long jbase, int npts, bool final_seg) {
    using C = psc::cplx<T>;
    AdjWS *ws = r.ws;
    psc_handle *h = r.h;
    double *p_d1 = ws->part, *p_z = ws->part + kEW, *p_d3 = ws->part + kEW + 3 * r.z_n;
    double *p_dg = ws->part + 3 * kEW + 3 * r.z_n, *p_d3g = ws->part + 4 * kEW + 3 * r.z_n;
    const int rows = r.nf * r.N * r.N, rows_gw = 6 * r.N * r.N;
    int rc;
    if (final_seg && r.gwadj) {
        // the final point P_S: the closing GW kick of the last stage (the scalar part is
        // zero there: nothing depends on pi(S) or on a''(S))
        const long long j = jbase + npts;
        if ((rc = scalar(r, ADJ_PRE, npts, j, nullptr, true))) return rc;
        ka_point_gw<T><<<kEW, kThreads, 0, r.st>>>(rows_gw, r.ri, (const C *)ws->Lpu, (C *)ws->Lu,
                                                   (const C *)tp_fu(r, npts), (C *)ws->Mu, ws->rec, p_dg);
        CU(cudaGetLastError());
        CU(r.prec == 32 ? psc::reg_adj_point_gw_f32(h->cfg, h->b, ws->Mu, tp_f(r, npts), ws->Tarr, ws->Lf, ws->rec, r.st)
                        : psc::reg_adj_point_gw_f64(h->cfg, h->b, ws->Mu, tp_f(r, npts), ws->Tarr, ws->Lf, ws->rec,
                                                    r.st));
        if ((rc = scalar(r, ADJ_POST, npts, j, nullptr, true))) return rc;
    }
    for (int i = npts - 1; i >= 0; --i) {
        const long long j = jbase + i;
        // the internals of stage j (its drift and a-updates)
        if ((rc = scalar(r, ADJ_STAGE_PRE, i, j))) return rc;
        ka_stage<T><<<kEW, kThreads, 0, r.st>>>(rows, r.ri, (const C *)ws->Lf, (C *)ws->Lp,
                                                (const C *)tp_p(r, i), (const C *)tp_f(r, i), (const C *)tp_vp(r, i),
                                                ws->rec, p_d3);
        CU(cudaGetLastError());
        if (r.gwadj) {
            ka_stage_gw<T><<<kEW, kThreads, 0, r.st>>>(rows_gw, r.ri, (const C *)ws->Lu, (C *)ws->Lpu,
                                                       (const C *)tp_pu(r, i), (const C *)tp_fu(r, i), ws->rec, p_d3g);
            CU(cudaGetLastError());
        }
        if ((rc = scalar(r, ADJ_STAGE_POST, i, j))) return rc;
        // point j: merged J^T of the kicks at P_j and the a''(P_j) terms
        if ((rc = scalar(r, ADJ_PRE, i, j))) return rc;
        ka_point<T><<<kEW, kThreads, 0, r.st>>>(rows, r.ri, (C *)ws->Lp, (const C *)tp_p(r, i),
                                                (const C *)tp_f(r, i), (C *)ws->M, ws->rec, p_d1);
        CU(cudaGetLastError());
        CU(r.prec == 32 ? psc::reg_adj_point_f32(h->cfg, h->b, ws->M, tp_f(r, i), tp_fx(r, i), ws->Lf, p_z, ws->rec,
                                                 r.st)
                        : psc::reg_adj_point_f64(h->cfg, h->b, ws->M, tp_f(r, i), tp_fx(r, i), ws->Lf, p_z, ws->rec,
                                                 r.st));
        if (r.gwadj) {
            // the merged GW kicks at P_j: Mu, Lu, the a-dot, then the transposed source into Lf
            ka_point_gw<T><<<kEW, kThreads, 0, r.st>>>(rows_gw, r.ri, (const C *)ws->Lpu, (C *)ws->Lu,
                                                       (const C *)tp_fu(r, i), (C *)ws->Mu, ws->rec, p_dg);
            CU(cudaGetLastError());
            CU(r.prec == 32 ? psc::reg_adj_point_gw_f32(h->cfg, h->b, ws->Mu, tp_f(r, i), ws->Tarr, ws->Lf, ws->rec,
                                                        r.st)
                            : psc::reg_adj_point_gw_f64(h->cfg, h->b, ws->Mu, tp_f(r, i), ws->Tarr, ws->Lf, ws->rec,
                                                        r.st));
        }
        if ((rc = scalar(r, ADJ_POST, i, j))) return rc;
    }
    return PSC_OK;
}

int reverse_segment(const Run &r, long long jbase, int npts, bool final_seg) {
    return r.prec == 32 ? reverse_segment_t<float>(r, jbase, npts, final_seg)
                        : reverse_segment_t<double>(r, jbase, npts, final_seg);
}

int save_state(const Run &r, char *dst) {
    const size_t c = r.ws->carr, g = r.ws->garr;
    CU(cudaMemcpyAsync(dst, r.h->b.fk, c, cudaMemcpyDeviceToDevice, r.st));
    CU(cudaMemcpyAsync(dst + c, r.h->b.pk, c, cudaMemcpyDeviceToDevice, r.st));
    if (g) {
        CU(cudaMemcpyAsync(dst + 2 * c, r.h->b.uk, g, cudaMemcpyDeviceToDevice, r.st));
        CU(cudaMemcpyAsync(dst + 2 * c + g, r.h->b.puk, g, cudaMemcpyDeviceToDevice, r.st));
    }
    CU(cudaMemcpyAsync(dst + 2 * c + 2 * g, r.h->b.bg, sizeof(psc::DevBG), cudaMemcpyDeviceToDevice, r.st));
    return PSC_OK;
}

int restore_state(const Run &r, const char *src) {
    const size_t c = r.ws->carr, g = r.ws->garr;
    CU(cudaMemcpyAsync(r.h->b.fk, src, c, cudaMemcpyDeviceToDevice, r.st));
    CU(cudaMemcpyAsync(r.h->b.pk, src + c, c, cudaMemcpyDeviceToDevice, r.st));
    if (g) {
        CU(cudaMemcpyAsync(r.h->b.uk, src + 2 * c, g, cudaMemcpyDeviceToDevice, r.st));
        CU(cudaMemcpyAsync(r.h->b.puk, src + 2 * c + g, g, cudaMemcpyDeviceToDevice, r.st));
    }
    CU(cudaMemcpyAsync(r.h->b.bg, src + 2 * c + 2 * g, sizeof(psc::DevBG), cudaMemcpyDeviceToDevice, r.st));
    return PSC_OK;
}

int grow_snap(AdjWS *ws, int want) {
    char *sp = reinterpret_cast<char *>(ws->snap);
    int rc = ws_grow(ws, &sp, &ws->snap_n, want, sizeof(psc::DevBG));
    ws->snap = reinterpret_cast<psc::DevBG *>(sp);
    return rc;
}

}  // namespace

extern "C" int psc_adjoint(psc_handle *h, int observable_id, double dt, int nsteps, int every, double *O,
                           double *grad_fk, double *grad_pik, double *grad_uk, double *grad_piuk, double *grad_ad0,
                           double *grad_theta) {
    if (!h || !O || nsteps < 1 || !(dt > 0) || !std::isfinite(dt)) return fail(PSC_ERR_ARG, "bad argument");
    int rc;
    if ((rc = check(h, observable_id))) return rc;
    if (every < 1 || every > nsteps) every = nsteps;
    Run r;
    if ((rc = setup(h, &r))) return rc;
    r.gwadj = observable_id == PSC_OBS_RHO_GW;
    AdjWS *ws = r.ws;
    const int s = h->s;
    const int nseg = (nsteps + every - 1) / every;
    const int npts_max = every * s;
    // storage: tape of one segment, snapshots, checkpoints (+ the final state)
    if ((rc = ws_grow(ws, &ws->tape, &ws->tape_n, npts_max + 1, ws->tape_stride))) return rc;
    if ((rc = grow_snap(ws, npts_max + 2))) return rc;
    if (nseg > 1 && (rc = ws_grow(ws, &ws->ckpt, &ws->ckpt_n, nseg + 1, ws->ckpt_stride))) return rc;
    CU(cudaEventRecord(h->ev0, r.st));
    // a''(0) = A(state(0)) and the reductions at the first point
    if ((rc = psc::hapi::evaluate(h, 0))) return rc;
    CU(cudaMemsetAsync(ws->Lf, 0, ws->carr, r.st));
    CU(cudaMemsetAsync(ws->Lp, 0, ws->carr, r.st));
    if (r.gw) {
        CU(cudaMemsetAsync(ws->Lu, 0, ws->garr, r.st));
        CU(cudaMemsetAsync(ws->Lpu, 0, ws->garr, r.st));
    }
    void *Lf_last = static_cast<char *>(ws->Lf) + (size_t)(r.nf - 1) * r.modes * h->csize;
    // the observable and its adjoint seed from the final state (the background record
    // goes to its own slot: the segment snapshots stay as the reverse sweep reads them)
    auto seed = [&]() -> int { return r.gwadj ? observable_gw(r, ws->Lpu) : observable(r, Lf_last); };
    if (nseg > 1) {
        // checkpoint pass on the product's captured step
        for (int seg = 0; seg < nseg; ++seg) {
            if ((rc = save_state(r, ws->ckpt + (size_t)seg * ws->ckpt_stride))) return rc;
            if ((rc = psc::hapi::step(h, dt, std::min(every, nsteps - seg * every)))) return rc;
        }
        if ((rc = save_state(r, ws->ckpt + (size_t)nseg * ws->ckpt_stride))) return rc;
        if ((rc = seed())) return rc;
    }
    // the segment replays below rewrite the state and the kept force
    h->force_valid = false;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int n = std::min(every, nsteps - seg * every);
        if (nseg > 1 && (rc = restore_state(r, ws->ckpt + (size_t)seg * ws->ckpt_stride))) return rc;
        if ((rc = forward_taped(r, dt, n))) return rc;
        if (nseg == 1 && (rc = seed())) return rc;
        if ((rc = reverse_segment(r, (long long)seg * every * s, n * s, seg == nseg - 1))) return rc;
    }
    CU(cudaEventRecord(h->ev1, r.st));
    psc::DevAdj rec;
    CU(cudaMemcpyAsync(&rec, ws->rec, sizeof(rec), cudaMemcpyDeviceToHost, r.st));
    CU(cudaStreamSynchronize(r.st));
    CU(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
    if (!std::isfinite(rec.O) || !std::isfinite(rec.lb) || !std::isfinite(rec.gth[0]) || !std::isfinite(rec.gth[1]))
        return fail(PSC_ERR_NONFINITE, "non-finite observable or gradient");
    *O = rec.O;
    if (grad_ad0) *grad_ad0 = rec.lb;
    if (grad_theta) {
        grad_theta[0] = rec.gth[0];
        grad_theta[1] = rec.gth[1];
    }
    // gradients with respect to the stored half spectrum: (w_k / N^3) Lambda_k
    auto to_grad = [&](const void *L, double *out, size_t ncplx) -> int {
        if (!out) return PSC_OK;
        if (!L) {
            std::memset(out, 0, sizeof(double) * 2 * ncplx);
            return PSC_OK;
        }
        int e = psc::hapi::download_real(h, out, L, 2 * ncplx);
        if (e) return e;
        for (size_t i = 0; i < ncplx; ++i) {
            const int kz = (int)((i % r.modes) % r.H);
            const double wk = (kz == 0 || kz == r.H - 1) ? 1.0 : 2.0;
            out[2 * i] *= wk / r.n3;
            out[2 * i + 1] *= wk / r.n3;
        }
        return PSC_OK;
    };
    if ((rc = to_grad(ws->Lf, grad_fk, (size_t)r.n)) || (rc = to_grad(ws->Lp, grad_pik, (size_t)r.n))) return rc;
    const size_t ng = (size_t)6 * r.modes;
    if (r.gw && ((rc = to_grad(r.gwadj ? ws->Lu : nullptr, grad_uk, ng)) ||
                 (rc = to_grad(r.gwadj ? ws->Lpu : nullptr, grad_piuk, ng))))
        return rc;
    // leave the handle at the final state, as psc_step(h, dt, nsteps) would
    if (nseg > 1) {
        if ((rc = restore_state(r, ws->ckpt + (size_t)nseg * ws->ckpt_stride))) return rc;
        CU(cudaStreamSynchronize(r.st));
    }
    h->diag_valid = true;
    return PSC_OK;
}

extern "C" int psc_adjoint_chi2(psc_handle *h, double dt, int nsteps, int every, double *O, double *grad_fk,
                                double *grad_pik, double *grad_ad0, double *grad_theta) {
    return psc_adjoint(h, PSC_OBS_CHI2, dt, nsteps, every, O, grad_fk, grad_pik, nullptr, nullptr, grad_ad0,
                       grad_theta);
}

extern "C" int psc_adjoint_forward(psc_handle *h, int observable_id, double dt, int nsteps, double *O) {
    if (!h || !O || nsteps < 1 || !(dt > 0) || !std::isfinite(dt)) return fail(PSC_ERR_ARG, "bad argument");
    int rc;
    if ((rc = check(h, observable_id))) return rc;
    Run r;
    if ((rc = setup(h, &r))) return rc;
    if ((rc = grow_snap(r.ws, 2))) return rc;
    if ((rc = psc::hapi::evaluate(h, 0))) return rc;
    if ((rc = psc::hapi::step(h, dt, nsteps))) return rc;
    if (observable_id == PSC_OBS_RHO_GW) {
        if ((rc = observable_gw(r, r.ws->Mu))) return rc;   // Mu: scratch for the seed
    } else {
        if ((rc = observable(r, nullptr))) return rc;
    }
    psc::DevAdj rec;
    CU(cudaMemcpyAsync(&rec, r.ws->rec, sizeof(rec), cudaMemcpyDeviceToHost, r.st));
    CU(cudaStreamSynchronize(r.st));
    *O = rec.O;
    return PSC_OK;
}

extern "C" int psc_adjoint_forward_chi2(psc_handle *h, double dt, int nsteps, double *O) {
    return psc_adjoint_forward(h, PSC_OBS_CHI2, dt, nsteps, O);
}
