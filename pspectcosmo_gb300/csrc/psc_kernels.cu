// psc_kernels.cu — the sm_103a kernels of one pseudo-spectral stage.
//
// A stage of evolve_VV_k_nopad (evolution.cpp:1131-1198) / evolve_VV
// (evolution.cpp:607-694) is one force evaluation here, because the closing
// half kick of a stage and the opening half kick of the next use the same
// force (same f and a): the two kicks are applied together in the epilogue of
// the last pass. Per stage and per field (GW terms in brackets):
//
//   k_ifft_x   X-axis inverse pass over f_k; prologue: the drift
//              f_k += w dt a_half^(alpha-3) pi_half (evolution.cpp:1164-1168);
//              [also i k_x f_k for the x-derivative (evolution.cpp:484-497)]
//   k_ifft_y   Y-axis inverse pass [+ i k_y for the y-derivative]
//   k_zpass    per (x,y) line: c2r along z and 1/N^3 (evolution.cpp:1171-1176)
//              [+ i k_z for the z-derivative], then pointwise V'(phi, chi)
//              (evolution.cpp:1103-1109) and <V> (evolution.cpp:1077-1085)
//              [and S_ab = 2 sum_f d_a f d_b f (evolution.cpp:592-597)], then
//              r2c along z of every product
//   k_fft_y    Y-axis forward pass of V' [and S_ab]
//   k_fft_x_final  X-axis forward pass, then the force
//              -a^(1+alpha) kIR^2 k^2 f_k - a^(3+alpha) V'_k (evolution.cpp:1115-1127),
//              the kicks, the masked K and G sums (evolution.cpp:923-1056)
//              [and for u_ij: the deferred drift, the force a^(1+alpha)(-k^2 u + S)
//              and the kicks (evolution.cpp:581-601, 635-684)]
//   k_scalar   one block: reductions -> a'' (evolution.cpp:1087) -> b, and the
//              next stage's coefficients (evolution.cpp:1141, 1161, 1180, 1193)
//
// All passes stage a tile of lines in shared memory and run a Stockham FFT
// there (psc_dev.cuh), so each pass is one read and one write of its arrays.
#include "psc_dev.cuh"
#include "psc_launch.h"

namespace psc {

// ------------------------------------------------------------------ X pass (inverse)
template <typename T, bool GW, bool DRIFT>
__global__ void __launch_bounds__(256) k_ifft_x(Geo g, cplx<T> *__restrict__ fk, const cplx<T> *__restrict__ pk,
                                                cplx<T> *__restrict__ TA, cplx<T> *__restrict__ TB,
                                                const DevBG *__restrict__ bg, const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int sh = g.tlx_shift, TL = 1 << sh, N = g.N;
    C *b0 = reinterpret_cast<C *>(smem_raw);
    C *b1 = b0 + TL * N;
    {
        const long long rf = (long long)blockIdx.z * g.fstride;
        fk += rf;
        if (DRIFT) pk += rf;
        TA += rf;
        if (GW) TB += rf;
        bg += blockIdx.z;
    }
    const long long off = (long long)blockIdx.y * g.modes;
    const int line0 = blockIdx.x * TL;
    const long long stride = g.lines_x;
    const T c = DRIFT ? (T)bg->c_drift : T(0);
    const int total = TL * N;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
        C v = mk<T>(0, 0);
        if (line < g.lines_x) {
            const long long a = off + n * stride + line;
            v = fk[a];
            if (DRIFT) {
                const C p = pk[a];
                v.x += c * p.x;
                v.y += c * p.y;
                // the homogeneous mode: the background kernel's FP64 shadow, already drifted
                if (a == off && bg->zero64) v = mk<T>((T)bg->z0f[blockIdx.y][0], (T)bg->z0f[blockIdx.y][1]);
                fk[a] = v;
            }
        }
        b0[idx] = v;
    }
    C *r = fft_tile<C, +1>(b0, b1, N, sh, TL, tw, N);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
        if (line < g.lines_x) TA[off + n * stride + line] = r[idx];
    }
    if (GW) {
        __syncthreads();
        const T kIR = (T)bg->kIR;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
            C v = mk<T>(0, 0);
            if (line < g.lines_x) {
                const C f = fk[off + n * stride + line];
                const T kx = (n == (N >> 1)) ? T(0) : kIR * (T)pcoord(n, N);
                v = mk<T>(-kx * f.y, kx * f.x);
            }
            b0[idx] = v;
        }
        r = fft_tile<C, +1>(b0, b1, N, sh, TL, tw, N);
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
            if (line < g.lines_x) TB[off + n * stride + line] = r[idx];
        }
    }
}

// ------------------------------------------------------------------ Y pass helpers
// Line l = x * H + kz of the Y pass; element y at (x N + y) H + kz.
__device__ __forceinline__ long long yaddr(const Geo &g, int line, int y) {
    const int x = line / g.H, kz = line - x * g.H;
    return ((long long)x * g.N + y) * g.H + kz;
}

// One Y-axis transform of a tile: src -> dst (may alias), optional i k_y multiplier.
template <typename T, int DIR>
__device__ __forceinline__ void ypass_tile(const Geo &g, const cplx<T> *src, cplx<T> *dst, bool deriv, T kIR,
                                           cplx<T> *b0, cplx<T> *b1, const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    const int sh = g.tlx_shift, TL = 1 << sh, N = g.N, total = TL * N;
    const int line0 = blockIdx.x * TL;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
        C v = mk<T>(0, 0);
        if (line < g.lines_x) {
            v = src[yaddr(g, line, n)];
            if (deriv) {
                const T ky = (n == (N >> 1)) ? T(0) : kIR * (T)pcoord(n, N);
                v = mk<T>(-ky * v.y, ky * v.x);
            }
        }
        b0[idx] = v;
    }
    C *r = fft_tile<C, DIR>(b0, b1, N, sh, TL, tw, N);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
        if (line < g.lines_x) dst[yaddr(g, line, n)] = r[idx];
    }
    __syncthreads();
}

template <typename T, bool GW>
__global__ void __launch_bounds__(256) k_ifft_y(Geo g, cplx<T> *__restrict__ TA, cplx<T> *__restrict__ TB,
                                                cplx<T> *__restrict__ TC, const DevBG *__restrict__ bg,
                                                const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int TL = 1 << g.tlx_shift;
    C *b0 = reinterpret_cast<C *>(smem_raw);
    C *b1 = b0 + TL * g.N;
    const long long off = (long long)blockIdx.y * g.modes + (long long)blockIdx.z * g.fstride;
    bg += blockIdx.z;
    const T kIR = (T)bg->kIR;
    if (GW) {
        // the y-derivative reads TA before TA is transformed in place
        ypass_tile<T, +1>(g, TA + off, TC + off, true, kIR, b0, b1, tw);
        ypass_tile<T, +1>(g, TA + off, TA + off, false, kIR, b0, b1, tw);
        ypass_tile<T, +1>(g, TB + off, TB + off, false, kIR, b0, b1, tw);
    } else {
        ypass_tile<T, +1>(g, TA + off, TA + off, false, kIR, b0, b1, tw);
    }
}

// Forward Y pass in place over a list of arrays (blockIdx.y selects the array; ArrList,
// psc_launch.h, holds up to PSC_MAX_FIELDS + 6 of them).

template <typename T>
__global__ void __launch_bounds__(256) k_fft_y(Geo g, ArrList arrs, const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int TL = 1 << g.tlx_shift;
    C *b0 = reinterpret_cast<C *>(smem_raw);
    C *b1 = b0 + TL * g.N;
    C *a = reinterpret_cast<C *>(arrs.p[blockIdx.y]) + (long long)blockIdx.z * arrs.rs[blockIdx.y];
    ypass_tile<T, -1>(g, a, a, false, T(0), b0, b1, tw);
}

// X-axis forward pass of the arrays of a list, no epilogue (the padded step's r2c at N_pad)
template <typename T>
__global__ void __launch_bounds__(256) k_fft_x_plain(Geo g, ArrList arrs, const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int sh = g.tlx_shift, TL = 1 << sh, N = g.N;
    C *b0 = reinterpret_cast<C *>(smem_raw);
    C *b1 = b0 + TL * N;
    C *a = reinterpret_cast<C *>(arrs.p[blockIdx.y]) + (long long)blockIdx.z * arrs.rs[blockIdx.y];
    const int line0 = blockIdx.x * TL;
    const long long stride = g.lines_x;
    const int total = TL * N;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
        b0[idx] = (line < g.lines_x) ? a[n * stride + line] : mk<T>(0, 0);
    }
    const C *r = fft_tile<C, -1>(b0, b1, N, sh, TL, tw, N);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
        if (line < g.lines_x) a[n * stride + line] = r[idx];
    }
}

// ------------------------------------------------------------------ fused Z pass
// Shared memory: b0, b1 (H rows x ldz) and nslot real-line slots (M rows x ldz,
// a complex element holding the two real sites 2m and 2m+1).
template <typename T, bool GW>
__global__ void __launch_bounds__(256) k_zpass(Geo g, const cplx<T> *__restrict__ TA, const cplx<T> *__restrict__ TB,
                                               const cplx<T> *__restrict__ TC, cplx<T> *__restrict__ QV,
                                               cplx<T> *__restrict__ QS, double *__restrict__ partV,
                                               const DevBG *__restrict__ bg, const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int sh = g.tlz_shift, TL = 1 << sh, LD = g.ldz, H = g.H, M = g.M, N = g.N;
    C *b0 = reinterpret_cast<C *>(smem_raw);
    C *b1 = b0 + H * LD;
    C *slots = b1 + H * LD;
    {
        const long long rf = (long long)blockIdx.z * g.fstride, rg = (long long)blockIdx.z * g.gstride;
        TA += rf;
        QV += rf;
        if (GW) {
            TB += rf;
            TC += rf;
            QS += rg;
        }
        partV += (size_t)blockIdx.z * g.pv_stride;
        bg += blockIdx.z;
    }
    const int line0 = blockIdx.x * TL;
    const int nf = g.nf;
    const int nin = nf * (GW ? 4 : 1);
    const int nout = nf + (GW ? 6 : 0);
    const T inv_n3 = (T)bg->inv_n3;
    const T kIR = (T)bg->kIR;

    // 1. complex-to-real along z of every input line
    for (int o = 0; o < nin; ++o) {
        const int fld = GW ? (o >> 2) : o;
        const int kind = GW ? (o & 3) : 0;   // 0: f, 1: d/dx f, 2: d/dy f, 3: d/dz f
        const C *src = (kind == 1 ? TB : (kind == 2 ? TC : TA)) + (long long)fld * g.modes;
        for (int idx = threadIdx.x; idx < TL * H; idx += blockDim.x) {
            const int t = idx / H, k = idx - t * H, line = line0 + t;
            C v = mk<T>(0, 0);
            if (line < g.lines_z) {
                v = src[(long long)line * H + k];
                if (kind == 3) {
                    const T kz = (k < M) ? kIR * (T)k : T(0);
                    v = mk<T>(-kz * v.y, kz * v.x);
                }
            }
            b1[k * LD + t] = v;
        }
        __syncthreads();
        // pack the half spectrum into an M-point complex transform:
        // Z[k] = (X[k] + conj X[M-k]) + i w^k (X[k] - conj X[M-k]), w = e^{+2 pi i/N};
        // Im X[0] and Im X[M] are ignored, as a c2r transform does.
        for (int idx = threadIdx.x; idx < TL * M; idx += blockDim.x) {
            const int t = idx & (TL - 1), k = idx >> sh;
            C x = b1[k * LD + t], y = cconj(b1[(M - k) * LD + t]);
            if (k == 0) { x.y = T(0); y.y = T(0); }
            const C s = cadd(x, y), d = csub(x, y);
            C w = __ldg(&tw[k]);
            w.y = -w.y;
            const C td = cmul(w, d);
            b0[k * LD + t] = mk<T>(s.x - td.y, s.y + td.x);
        }
        C *r = fft_tile<C, +1>(b0, b1, M, sh, LD, tw, N);
        C *so = slots + (size_t)o * M * LD;
        for (int idx = threadIdx.x; idx < TL * M; idx += blockDim.x) {
            const int t = idx & (TL - 1), k = idx >> sh;
            so[k * LD + t] = cscale(r[k * LD + t], inv_n3);
        }
        __syncthreads();
    }

    // 2. pointwise epilogue: V'(f), <V>, anisotropic stress
    Model mdl;
    mdl.kind = g.model;
    mdl.gsq = g.gsq;
    double pot[kMaxTerms] = {};
    constexpr int NIN = 4 * kMaxFields, NOUT = kMaxFields + 6;
    for (int idx = threadIdx.x; idx < TL * M; idx += blockDim.x) {
        const int t = idx & (TL - 1), k = idx >> sh;
        if (line0 + t >= g.lines_z) continue;
        const int e = k * LD + t;
        C in[NIN];
#pragma unroll
        for (int o = 0; o < NIN; ++o)
            if (o < nin) in[o] = slots[(size_t)o * M * LD + e];
        C out[NOUT];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            T f[kMaxFields], vp[kMaxFields];
#pragma unroll
            for (int fl = 0; fl < kMaxFields; ++fl) {
                if (fl < nf) {
                    const C c = in[GW ? fl * 4 : fl];
                    f[fl] = half ? c.y : c.x;
                } else {
                    f[fl] = T(0);
                }
            }
            model_dvdf<T, double, true>(mdl, f, vp, nf);
            model_potential<T, double, double, true>(mdl, f, pot);
#pragma unroll
            for (int fl = 0; fl < kMaxFields; ++fl)
                if (fl < nf) { if (half) out[fl].y = vp[fl]; else out[fl].x = vp[fl]; }
            if (GW) {
                T d[kMaxFields][3];
#pragma unroll
                for (int fl = 0; fl < kMaxFields; ++fl)
#pragma unroll
                    for (int ax = 0; ax < 3; ++ax)
                        d[fl][ax] = (fl < nf) ? (half ? in[fl * 4 + 1 + ax].y : in[fl * 4 + 1 + ax].x) : T(0);
                const int si[6] = {0, 0, 0, 1, 1, 2}, sj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    T sum = T(0);
#pragma unroll
                    for (int fl = 0; fl < kMaxFields; ++fl)
                        if (fl < nf) sum += T(2) * d[fl][si[c]] * d[fl][sj[c]];
                    if (half) out[nf + c].y = sum; else out[nf + c].x = sum;
                }
            }
        }
#pragma unroll
        for (int o = 0; o < NOUT; ++o)
            if (o < nout) slots[(size_t)o * M * LD + e] = out[o];
    }
    block_reduce_store<kMaxTerms>(pot, partV, gridDim.x, blockIdx.x);
    __syncthreads();

    // 3. real-to-complex along z of every product
    for (int o = 0; o < nout; ++o) {
        C *so = slots + (size_t)o * M * LD;
        C *r = fft_tile<C, -1>(so, b0, M, sh, LD, tw, N);
        C *dst = (o < nf) ? QV + (long long)o * g.modes : QS + (long long)(o - nf) * g.modes;
        for (int idx = threadIdx.x; idx < TL * H; idx += blockDim.x) {
            const int t = idx / H, k = idx - t * H, line = line0 + t;
            if (line >= g.lines_z) continue;
            const C zk = r[(k == M ? 0 : k) * LD + t];
            const C zc = cconj(r[(k == 0 ? 0 : M - k) * LD + t]);
            const C ev = cscale(cadd(zk, zc), T(0.5));
            const C dd = cscale(csub(zk, zc), T(0.5));
            const C od = mk<T>(dd.y, -dd.x);
            C w;
            if (k < M) w = __ldg(&tw[k]); else w = mk<T>(T(-1), T(0));
            dst[(long long)line * H + k] = cadd(ev, cmul(w, od));
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ X pass (forward) + kick epilogue
template <typename T, bool GW>
__global__ void __launch_bounds__(256) k_fft_x_final(Geo g, const cplx<T> *__restrict__ QV, const cplx<T> *__restrict__ QS,
                                                     const cplx<T> *__restrict__ fk, cplx<T> *__restrict__ pk,
                                                     cplx<T> *__restrict__ uk, cplx<T> *__restrict__ puk,
                                                     double *__restrict__ partKG, const DevBG *__restrict__ bg,
                                                     const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int sh = g.tlx_shift, TL = 1 << sh, N = g.N, H = g.H, M = g.M;
    C *b0 = reinterpret_cast<C *>(smem_raw);
    C *b1 = b0 + TL * N;
    {
        const long long rf = (long long)blockIdx.z * g.fstride, rg = (long long)blockIdx.z * g.gstride;
        QV += rf;
        fk += rf;
        pk += rf;
        if (GW) {
            QS += rg;
            uk += rg;
            puk += rg;
        }
        partKG += (size_t)blockIdx.z * g.pkg_stride;
        bg += blockIdx.z;
    }
    const int job = blockIdx.y;
    const bool field = job < g.nf;
    const long long off = (long long)(field ? job : job - g.nf) * g.modes;
    const C *src = (field ? QV : QS) + off;
    const int line0 = blockIdx.x * TL;
    const long long stride = g.lines_x;
    const int total = TL * N;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
        b0[idx] = (line < g.lines_x) ? src[n * stride + line] : mk<T>(0, 0);
    }
    const C *r = fft_tile<C, -1>(b0, b1, N, sh, TL, tw, N);

    const T norm1 = (T)bg->norm1, norm2 = (T)bg->norm2, kIR2 = (T)bg->kIR2;
    const T c_close = (T)bg->c_close, c_open = (T)bg->c_open;
    double accK = 0.0, accG = 0.0;
    if (field) {
        const bool mask = g.mask != 0;
        const T hub = (T)bg->hub, apow = (T)bg->apow, a3 = (T)bg->a3;
        const T dfdp = (T)bg->DFDP, eps = (T)bg->eps;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
            if (line >= g.lines_x) continue;
            const int y = line / H, kz = line - y * H;
            const int px = pcoord(n, N), py = pcoord(y, N);
            const T k2 = (T)(px * px + py * py + kz * kz);
            const long long a = off + n * stride + line;
            const C f = fk[a], p = pk[a], q = r[idx];
            if (a == off && bg->zero64) {   // the homogeneous mode: kicked in FP64 by the background kernel
                DevBG *bw = const_cast<DevBG *>(bg);
                bw->z0q[job][0] = (double)q.x;
                bw->z0q[job][1] = (double)q.y;
                bw->z0pending = 1;
                continue;
            }
            // force (evolution.cpp:1124-1125)
            const T fl = -norm1 * kIR2 * k2;
            const C F = mk<T>(fl * f.x - norm2 * q.x, fl * f.y - norm2 * q.y);
            const C pf = mk<T>(p.x + c_close * F.x, p.y + c_close * F.y);
            bool inc = true;
            if (mask && (n | line) != 0) {
                // R_Q2C (evolution.cpp:1038-1056) with the stale a' of the step
                const T fm = sqrt(f.x * f.x + f.y * f.y);
                const T gx = hub * f.x + apow * pf.x, gy = hub * f.y + apow * pf.y;
                const T R = dfdp / (fm * a3 * sqrt(gx * gx + gy * gy));
                inc = R < eps;
            }
            if (inc) {
                const double wgt = (kz == 0 || kz == M) ? 1.0 : 2.0;
                accK += wgt * ((double)pf.x * pf.x + (double)pf.y * pf.y);
                accG += wgt * (double)k2 * ((double)f.x * f.x + (double)f.y * f.y);
            }
            pk[a] = mk<T>(pf.x + c_open * F.x, pf.y + c_open * F.y);
        }
        double v[2] = {accK, accG};
        block_reduce_store<2>(v, partKG + (size_t)(2 * job) * gridDim.x, gridDim.x, blockIdx.x);
    } else if (GW) {
        const T c_drift = (T)bg->c_drift;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int t = idx & (TL - 1), n = idx >> sh, line = line0 + t;
            if (line >= g.lines_x) continue;
            const int y = line / H, kz = line - y * H;
            const int px = pcoord(n, N), py = pcoord(y, N);
            const T k2 = (T)(px * px + py * py + kz * kz);
            const long long a = off + n * stride + line;
            C u = uk[a];
            const C v = puk[a], q = r[idx];
            // drift of u_ij deferred from the stage prologue (evolution.cpp:655-662)
            u.x += c_drift * v.x;
            u.y += c_drift * v.y;
            // a^(1+alpha) (lapl u + 2 sum d_i f d_j f)  (evolution.cpp:586-598)
            const T l = -kIR2 * k2;
            const C F = mk<T>(norm1 * (l * u.x + q.x), norm1 * (l * u.y + q.y));
            const C vf = mk<T>(v.x + c_close * F.x, v.y + c_close * F.y);
            uk[a] = u;
            puk[a] = mk<T>(vf.x + c_open * F.x, vf.y + c_open * F.y);
        }
    }
}

// ------------------------------------------------------------------ scalar background update
// The homogeneous mode's FP64 shadow (DevBG::z0*): element 0 of field f's array, rounded
// to the array's precision
__device__ void zero_store(const DevBG *bg, void *arr, long long modes, int f, const double *v) {
    if (bg->fp32) reinterpret_cast<float2 *>(arr)[(long long)f * modes] = make_float2((float)v[0], (float)v[1]);
    else reinterpret_cast<double2 *>(arr)[(long long)f * modes] = make_double2(v[0], v[1]);
}

// The kicks of the last kick pass, applied to the shadow: F = -a^(3+alpha) V'_k(0) (no
// gradient term at k = 0, kernel_field_k_nopad evolution.cpp:1124-1125), pf = p + c_close F
// (synchronised: K0[f] = |pf|^2, the zero mode's term of the kinetic sum), p = pf + c_open F.
__device__ void zero_kick(DevBG *bg, void *pk, long long modes, double *K0) {
    for (int f = 0; f < bg->nf; ++f) {
        const double F[2] = {-bg->norm2 * bg->z0q[f][0], -bg->norm2 * bg->z0q[f][1]};
        const double pf[2] = {bg->z0p[f][0] + bg->c_close * F[0], bg->z0p[f][1] + bg->c_close * F[1]};
        if (K0) K0[f] = pf[0] * pf[0] + pf[1] * pf[1];
        for (int c = 0; c < 2; ++c) {
            bg->z0p[f][c] = pf[c] + bg->c_open * F[c];
            if (bg->c_open == 0.0) bg->z0F[f][c] = F[c];
        }
        zero_store(bg, pk, modes, f, bg->z0p[f]);
    }
    bg->z0pending = 0;
}

__device__ void begin_stage(DevBG *bg, int p) {
    const double w = bg->w[p], dt = bg->dt;
    const int al = bg->alpha;
    // evolution.cpp:1141, 1161, 1165, 1180
    bg->b_half = bg->b + w * dt / 2. * bg->add;
    const double a_half = bg->a + bg->b_half * w * dt / 2.;
    bg->c_drift = w * dt * ipow(a_half, al - 3);
    bg->a = a_half + bg->b_half * w * dt / 2.;
    bg->norm1 = ipow(bg->a, 1 + al);
    bg->norm2 = ipow(bg->a, 3 + al);
    bg->c_close = w * dt / 2;
    if (p + 1 < bg->s) bg->c_open = bg->w[p + 1] * dt / 2;
    else bg->c_open = (bg->steps_left > 1) ? bg->w[0] * dt / 2 : 0.0;
    bg->hub = bg->ad_stale / bg->a;
    bg->apow = ipow(bg->a, al - 3);
    bg->a3 = ipow(bg->a, 3 - al);
    bg->stage = p;
    if (bg->zero64)   // the drift of the homogeneous mode (the drift pass reads the shadow)
        for (int f = 0; f < bg->nf; ++f)
            for (int c = 0; c < 2; ++c) bg->z0f[f][c] += bg->c_drift * bg->z0p[f][c];
}

__device__ void eval_coeffs(DevBG *bg) {
    const int al = bg->alpha;
    bg->c_drift = 0.0;
    bg->c_close = 0.0;
    bg->norm1 = ipow(bg->a, 1 + al);
    bg->norm2 = ipow(bg->a, 3 + al);
    bg->ad_stale = bg->ad;
    bg->hub = bg->ad / bg->a;
    bg->apow = ipow(bg->a, al - 3);
    bg->a3 = ipow(bg->a, 3 - al);
}

// a'' = (1/3)(fStar/MPl)^2 a^(1+2 alpha) ((alpha-2) K + alpha G + (alpha+1) V)  (evolution.cpp:1087)
__device__ double friedmann_add(const DevBG *bg, double K, double G, double V) {
    const int al = bg->alpha;
    return 1. / 3. * bg->fs_over_mpl2 * ipow(bg->a, 1 + 2 * al) * ((al - 2) * K + al * G + (al + 1) * V);
}

// fk, pk: the realizations' field arrays (realization blockIdx.x at blockIdx.x fstride
// elements), for the homogeneous mode's shadow. SCALAR_PRIME with p = 1: the opening half
// kick uses the kept force.
// r: the realization (the block of one configuration's kernel; the batched background kernel
// passes a realization of one of its configurations)
// threads of the background kernel's block (the reduction of the block partials; the rest is
// one thread's FP64 arithmetic): 256 against 1024 cut its FP64 shuffle trees by four
constexpr int kScalarThreads = 256;

__device__ __forceinline__ void k_scalar_body(unsigned r, DevBG *bg, const double *__restrict__ partKG,
                                              const double *__restrict__ partV, int mode, int p, int pkg_stride,
                                              int pv_stride, void *fk, void *pk, long long fstride, long long modes) {
    constexpr int NQ = 2 * kMaxFields + kMaxTerms;
    __shared__ double red[32][NQ];
    bg += r;
    partKG += (size_t)r * pkg_stride;
    partV += (size_t)r * pv_stride;
    {
        const size_t off = (size_t)r * fstride * (bg->fp32 ? sizeof(float2) : sizeof(double2));
        fk = static_cast<char *>(fk) + off;
        pk = static_cast<char *>(pk) + off;
    }
    // a failed step (a wait ran out, a non-finite background) keeps its background as the
    // failure left it; evaluations of the state still run
    if (bg->err && mode != SCALAR_EVAL && mode != SCALAR_EVAL_END) return;
    __shared__ double sums[NQ];
    const bool reduce = (mode == SCALAR_END || mode == SCALAR_EVAL_END);
    if (reduce) {
        // every quantity in one sweep (all loads of a thread in flight together), then
        // one warp-shuffle + shared-memory tree for all of them
        const int nbx = bg->nbx, nbz = bg->nbz, nf = bg->nf, nt = bg->nterms;
        double acc[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
#pragma unroll 4
        for (int i = threadIdx.x; i < nbx; i += blockDim.x)
#pragma unroll
            for (int q = 0; q < 2 * kMaxFields; ++q)
                if (q < 2 * nf) acc[q] += partKG[(size_t)q * nbx + i];
        // fixed slots (K, G of field f at 2f, 2f+1; term t at 2 kMaxFields + t): no
        // run-time register index
#pragma unroll 8
        for (int i = threadIdx.x; i < nbz; i += blockDim.x)
#pragma unroll
            for (int q = 0; q < kMaxTerms; ++q)
                if (q < nt) acc[2 * kMaxFields + q] += partV[(size_t)q * nbz + i];
        // only the live quantities (2 nf field sums, nt terms) go through the shuffle trees:
        // on this part's narrow FP64 pipe the trees of every slot dominated the kernel
        auto live = [&](int q) { return q < 2 * kMaxFields ? q < 2 * nf : q - 2 * kMaxFields < nt; };
#pragma unroll
        for (int q = 0; q < NQ; ++q)
            if (live(q))
                for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < NQ; ++q) red[warp][q] = acc[q];
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                if (!live(q)) continue;
                double x = lane < nw ? red[lane][q] : 0.0;
                for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
                if (lane == 0) {
                    if (q < 2 * kMaxFields) {
                        if (q < 2 * nf) sums[q] = x;
                    } else if (q - 2 * kMaxFields < nt) {
                        sums[2 * nf + (q - 2 * kMaxFields)] = x;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const bool z0 = bg->zero64 != 0;
    if (mode == SCALAR_PRIME) {
        eval_coeffs(bg);
        bg->c_open = bg->w[0] * bg->dt / 2;
        if (z0 && p)   // the opening half kick of the homogeneous mode from its kept force
            for (int f = 0; f < bg->nf; ++f) {
                for (int c = 0; c < 2; ++c) bg->z0p[f][c] += bg->c_open * bg->z0F[f][c];
                zero_store(bg, pk, modes, f, bg->z0p[f]);
            }
        return;
    }
    if (mode == SCALAR_EVAL) {
        eval_coeffs(bg);
        bg->c_open = 0.0;
        return;
    }
    if (mode == SCALAR_BEGIN) {
        if (z0 && bg->z0pending) zero_kick(bg, pk, modes, nullptr);   // the prologue's evaluated kick
        bg->b = bg->ad;
        bg->ad_stale = bg->ad;
        begin_stage(bg, 0);
        return;
    }
    // reductions -> K, G, V (kinetic_energy_k / gradient_energy_k evolution.cpp:966-1034,
    // V_E evolution.cpp:1077-1085)
    double K = 0, G = 0, V = 0;
    const double a = bg->a;
    double K0[kMaxFields] = {0.0, 0.0};   // the homogeneous mode's kinetic term, from the shadow
    if (z0 && bg->z0pending) zero_kick(bg, pk, modes, K0);
    for (int f = 0; f < bg->nf; ++f) {
        const double k = .5 * (sums[2 * f] + K0[f]) / ipow(a, 6) * bg->inv_n3sq;
        double grad = bg->kIR2 * sums[2 * f + 1];
        grad *= bg->inv_n3;
        grad /= 2.;
        const double gq = grad / (a * a) * bg->inv_n3;
        bg->K[f] = k;
        bg->G[f] = gq;
        K += k;
        G += gq;
    }
    for (int tt = 0; tt < bg->nterms; ++tt) {
        const double v = sums[2 * bg->nf + tt] * bg->inv_nv;   // V_E /= N3 (or N3_pad, evolution.cpp:1631)
        bg->V[tt] = v;
        V += v;
    }
    const double add_new = friedmann_add(bg, K, G, V);
    if (!isfinite(add_new) || !isfinite(bg->a)) report_err(&bg->err, PSC_ERR_NONFINITE);
    if (mode == SCALAR_EVAL_END) {
        if (p == 0) bg->add = add_new;   // p == 1: diagnostics only, a'' kept as set by the caller
        return;
    }
    bg->add = add_new;
    // SCALAR_END: close stage p (evolution.cpp:1193), then open the next stage or step
    bg->b = bg->b_half + bg->w[p] * bg->dt / 2. * bg->add;
    if (p + 1 < bg->s) {
        begin_stage(bg, p + 1);
        return;
    }
    bg->ad = bg->b;        // evolution.cpp:1196-1197
    bg->t += bg->dt;
    bg->steps_left -= 1;
    if (!isfinite(bg->ad)) report_err(&bg->err, PSC_ERR_NONFINITE);
    if (bg->steps_left > 0) {
        bg->b = bg->ad;
        bg->ad_stale = bg->ad;
        begin_stage(bg, 0);
    }
}

__global__ void __launch_bounds__(kScalarThreads) k_scalar(DevBG *bg, const double *__restrict__ partKG,
                                                const double *__restrict__ partV, int mode, int p, int pkg_stride,
                                                int pv_stride, void *fk, void *pk, long long fstride,
                                                long long modes) {
    k_scalar_body(blockIdx.x, bg, partKG, partV, mode, p, pkg_stride, pv_stride, fk, pk, fstride, modes);
}

// the homogeneous modes' FP64 shadow taken from the arrays (after a device-side writer)
__global__ void k_zero_sync(DevBG *bg, const void *fk, const void *pk, long long fstride, long long modes) {
    if (threadIdx.x != 0) return;
    bg += blockIdx.x;
    const size_t cs = bg->fp32 ? sizeof(float2) : sizeof(double2);
    const char *f = static_cast<const char *>(fk) + (size_t)blockIdx.x * fstride * cs;
    const char *p = static_cast<const char *>(pk) + (size_t)blockIdx.x * fstride * cs;
    for (int q = 0; q < bg->nf; ++q) {
        const size_t o = (size_t)q * modes * cs;
        if (bg->fp32) {
            const float2 a = *reinterpret_cast<const float2 *>(f + o), b = *reinterpret_cast<const float2 *>(p + o);
            bg->z0f[q][0] = a.x, bg->z0f[q][1] = a.y, bg->z0p[q][0] = b.x, bg->z0p[q][1] = b.y;
        } else {
            const double2 a = *reinterpret_cast<const double2 *>(f + o), b = *reinterpret_cast<const double2 *>(p + o);
            bg->z0f[q][0] = a.x, bg->z0f[q][1] = a.y, bg->z0p[q][0] = b.x, bg->z0p[q][1] = b.y;
        }
    }
    bg->zero64 = 1;
    bg->z0pending = 0;
}

cudaError_t launch_zero_sync(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st) {
    k_zero_sync<<<cfg.R, 32, 0, st>>>(b.bg, b.fk, b.pk, cfg.g.fstride, cfg.g.modes);
    return cudaGetLastError();
}

__global__ void k_set_run(DevBG *bg, int R, double dt, int nsteps) {
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        bg[r].dt = dt;
        bg[r].steps_left = nsteps;
    }
}

// ------------------------------------------------------------------ real-space view
template <typename T>
__global__ void __launch_bounds__(256) k_z_c2r_real(Geo g, const cplx<T> *__restrict__ TA, T *__restrict__ out,
                                                    const cplx<T> *__restrict__ tw, T inv_n3) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int sh = g.tlz_shift, TL = 1 << sh, LD = g.ldz, H = g.H, M = g.M, N = g.N;
    C *b0 = reinterpret_cast<C *>(smem_raw);
    C *b1 = b0 + H * LD;
    const int line0 = blockIdx.x * TL;
    const long long off = (long long)blockIdx.y * g.modes;
    const C *src = TA + off;
    for (int idx = threadIdx.x; idx < TL * H; idx += blockDim.x) {
        const int t = idx / H, k = idx - t * H, line = line0 + t;
        b1[k * LD + t] = (line < g.lines_z) ? src[(long long)line * H + k] : mk<T>(0, 0);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < TL * M; idx += blockDim.x) {
        const int t = idx & (TL - 1), k = idx >> sh;
        C x = b1[k * LD + t], y = cconj(b1[(M - k) * LD + t]);
        if (k == 0) { x.y = T(0); y.y = T(0); }
        const C s = cadd(x, y), d = csub(x, y);
        C w = __ldg(&tw[k]);
        w.y = -w.y;
        const C td = cmul(w, d);
        b0[k * LD + t] = mk<T>(s.x - td.y, s.y + td.x);
    }
    const C *r = fft_tile<C, +1>(b0, b1, M, sh, LD, tw, N);
    T *o = out + (long long)blockIdx.y * g.sites;
    for (int idx = threadIdx.x; idx < TL * N; idx += blockDim.x) {
        const int t = idx / N, z = idx - t * N, line = line0 + t;
        if (line >= g.lines_z) continue;
        const C c = r[(z >> 1) * LD + t];
        o[(long long)line * N + z] = ((z & 1) ? c.y : c.x) * inv_n3;
    }
}

// ------------------------------------------------------------------ spectra
// Scalar spectra bin sums (output.cpp:626-669): every stored mode, weight 2 for
// 0 < kz < N/2; bin l = floor(sqrt(px^2 + py^2 + kz^2) + 0.5).
template <typename T>
__global__ void k_spectra_scalar(Geo g, const cplx<T> *__restrict__ fk, const cplx<T> *__restrict__ pk,
                                 const DevBG *__restrict__ bg, int nb, double *__restrict__ acc,
                                 int *__restrict__ cnt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sF = reinterpret_cast<double *>(smem_raw);
    double *sP = sF + nb, *sN = sP + nb;
    int *sC = reinterpret_cast<int *>(sN + nb);
    for (int i = threadIdx.x; i < nb; i += blockDim.x) { sF[i] = sP[i] = sN[i] = 0.0; sC[i] = 0; }
    __syncthreads();
    const int fld = blockIdx.y, N = g.N, H = g.H, M = g.M;
    const double a = bg->a, hub = bg->ad / a, aop = ipow(a, bg->alpha - 3);
    const cplx<T> *f = fk + (long long)fld * g.modes, *p = pk + (long long)fld * g.modes;
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < g.modes;
         m += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(m % H);
        const long long xy = m / H;
        const int y = (int)(xy % N), x = (int)(xy / N);
        const int px = pcoord(x, N), py = pcoord(y, N);
        const int l = (int)floor(sqrt((double)(px * px + py * py + kz * kz)) + 0.5);
        const double fr = f[m].x, fi = f[m].y, pr = p[m].x, pi = p[m].y;
        const double w = (kz == 0 || kz == M) ? 1.0 : 2.0;
        const double nr = aop * pr + hub * fr, ni = aop * pi + hub * fi;
        atomicAdd(&sF[l], w * (fr * fr + fi * fi));
        atomicAdd(&sP[l], w * (pr * pr + pi * pi));
        atomicAdd(&sN[l], w * (nr * nr + ni * ni));
        atomicAdd(&sC[l], (int)w);
    }
    __syncthreads();
    double *aF = acc + (size_t)fld * 3 * nb;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        if (sC[i] == 0) continue;
        atomicAdd(&aF[i], sF[i]);
        atomicAdd(&aF[nb + i], sP[i]);
        atomicAdd(&aF[2 * nb + i], sN[i]);
        atomicAdd(&cnt[(size_t)fld * nb + i], sC[i]);
    }
}

// GW spectra bin sums (output.cpp:780-1025): on the kz = 0 and kz = N/2 planes
// only the reference's "+" representatives count (weight 2), plus the seven
// non-zero real corners (weight 1); interior planes have weight 2. Per mode
// v = P u with P = 1 - khat khat, h^2 += sum |v_ij|^2 - |tr v|^2 / 2.
template <typename T>
__global__ void k_spectra_gw(Geo g, const cplx<T> *__restrict__ uk, const cplx<T> *__restrict__ puk,
                             const DevBG *__restrict__ bg, int nb, double *__restrict__ acc, int *__restrict__ cnt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sH = reinterpret_cast<double *>(smem_raw);
    double *sD = sH + nb;
    int *sC = reinterpret_cast<int *>(sD + nb);
    for (int i = threadIdx.x; i < nb; i += blockDim.x) { sH[i] = sD[i] = 0.0; sC[i] = 0; }
    __syncthreads();
    const int N = g.N, H = g.H, M = g.M;
    const double kIR = bg->kIR;
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < g.modes;
         m += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(m % H);
        const long long xy = m / H;
        const int j = (int)(xy % N), i = (int)(xy / N);
        int w = 2;
        if (kz == 0 || kz == M) {
            const bool ie = (i == 0 || i == M), je = (j == 0 || j == M);
            const bool iin = (i >= 1 && i < M), jlo = (j >= 1 && j < M), jhi = (j > M && j < N);
            if (ie && je) w = (i == 0 && j == 0 && kz == 0) ? 0 : 1;
            else if (ie && jlo) w = 2;
            else if (je && iin) w = 2;
            else if (iin && (jlo || jhi)) w = 2;
            else w = 0;
        }
        if (w == 0) continue;
        const int px = pcoord(i, N), py = pcoord(j, N);
        const int l = (int)floor(sqrt((double)(px * px + py * py + kz * kz)) + 0.5);
        const double kv[3] = {px * kIR, py * kIR, kz * kIR};
        const double kn = sqrt(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
        const double kh[3] = {kv[0] / kn, kv[1] / kn, kv[2] / kn};
        double res[2];
#pragma unroll
        for (int which = 0; which < 2; ++which) {
            const cplx<T> *arr = which ? puk : uk;
            double ur[6], ui[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const cplx<T> v = arr[(long long)c * g.modes + m];
                ur[c] = v.x;
                ui[c] = v.y;
            }
            const int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
            double s = 0.0, trr = 0.0, tri = 0.0;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    double vr = 0.0, vi = 0.0;
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const double P = (a == k ? 1.0 : 0.0) - kh[a] * kh[k];
                        vr += P * ur[sym[k][b]];
                        vi += P * ui[sym[k][b]];
                    }
                    s += vr * vr + vi * vi;
                    if (a == b) { trr += vr; tri += vi; }
                }
            res[which] = s - (trr * trr + tri * tri) / 2.;
        }
        atomicAdd(&sH[l], w * res[0]);
        atomicAdd(&sD[l], w * res[1]);
        atomicAdd(&sC[l], w);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        if (sC[q] == 0) continue;
        atomicAdd(&acc[q], sH[q]);
        atomicAdd(&acc[nb + q], sD[q]);
        atomicAdd(&cnt[q], sC[q]);
    }
}

// ------------------------------------------------------------------ host side
static int ilog2i(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

void plan(const psc_params &p, int R, LaunchCfg *cfg, const TileChoice *tc) {
    Geo &g = cfg->g;
    cfg->R = R;
    g.N = p.N;
    g.H = p.N / 2 + 1;
    g.M = p.N / 2;
    g.nf = p.nflds;
    g.gw = p.with_gw ? 1 : 0;
    g.gwev = (p.with_gw && !p.spectral) ? 1 : 0;
    g.model = p.model;
    g.nterms = model_nterms(p.model);
    g.mask = (p.spectral && p.simulate_inflation) ? 1 : 0;
    g.gsq = p.gsq;
    g.kIR = p.kIR;
    g.lines_x = g.N * g.H;
    g.lines_z = g.N * g.N;
    g.modes = (long long)g.N * g.N * g.H;
    g.sites = (long long)g.N * g.N * g.N;
    // the register engine: power-of-two lines from 32 on; the generic engine takes the rest
    // (N = 8, 16 and the sizes with factors 3, 5, 7)
    g.reg = (g.N >= 32 && (g.N & (g.N - 1)) == 0) ? 1 : 0;
    g.fstride = (long long)g.nf * g.modes;
    g.gstride = g.gw ? 6LL * g.modes : 0;
    const int csize = p.precision == 32 ? 8 : 16;
    const int nin = g.nf * (g.gwev ? 4 : 1), nout = g.nf + (g.gwev ? 6 : 0);
    const int nslot = nin > nout ? nin : nout;
    if (g.reg) {
        // register engine: P = L/16 threads per line, 256 threads per block (512 for FP32
        // 1024-point lines: 8 lines per block, 64 contiguous bytes per row; in FP64 the X
        // forward pass's three tiles would not fit in shared memory at that width)
        const int P = g.N / 16;
        const int xy_thr = (g.N >= 1024 && p.precision == 32) ? 512 : 256;
        int tl = xy_thr / P;
        while (tl > 1 && tl / 2 >= g.lines_x) tl /= 2;
        if (tc && tc->xy_shift >= 0 && (1 << tc->xy_shift) < tl) tl = 1 << tc->xy_shift;
        g.tlx_shift = ilog2i(tl);
        cfg->tc.xy_shift = g.tlx_shift;
        cfg->thr_xy = tl * P;
        cfg->smem_xy = (size_t)tl * g.N * csize;
        cfg->smem_xf = 3 * cfg->smem_xy + 128;   // + the alignment of the TMA operand tiles
        cfg->smem_xi = 3 * cfg->smem_xy + 128;
        // a Y tile staged by tensor copies: TL even rows and TL + 2 odd rows (FP32) of N/2
        cfg->smem_ys = (size_t)(tl + (csize == 8 ? 1 : 0)) * g.N * csize;
        cfg->nbx = (g.lines_x + tl - 1) / tl;
        const int Pz = g.M / 16;
        int tlz = 1;   // lines per tile: the largest power of two with nin x tlz x Pz <= 256 threads
        while (2 * tlz * nin * Pz <= 256) tlz *= 2;
        if (tc && tc->z_shift >= 0 && (1 << tc->z_shift) < tlz) tlz = 1 << tc->z_shift;
        g.tlz_shift = ilog2i(tlz);
        cfg->tc.z_shift = g.tlz_shift;
        g.ldz = 0;
        cfg->thr_z = nin * tlz * Pz;
        // Z pass shared memory. Without GWs (kr_zpass): nf work slots + nf staging slots of
        // half-length lines, persistent (2 blocks per SM). With GWs (kr_zpass_gw): four
        // slots of N-point lines and, in FP32 (persistent, 2 blocks per SM at up to 128
        // registers: 0.384 against 0.402 ms at 3 blocks and 80 registers, 256^3; next tile
        // staged), the nf x 3 input lines of a tile; in FP64 one tile per block.
        // A user model (up to kMaxFields fields) runs the USER instantiations: nslot work
        // slots (input pairs 2 nf, output pairs (nf + 7) / 2).
        const bool gw_staged = g.gwev && p.precision == 32;
        const bool user = model_is_user(p.model);
        const int gw_slots = user ? ((2 * g.nf > (g.nf + 7) / 2) ? 2 * g.nf : (g.nf + 7) / 2) : 4;
        if (g.gwev)
            cfg->smem_z = ((size_t)gw_slots * tlz * (g.N + g.N / 16 + 1) +
                           (gw_staged ? (size_t)g.nf * 3 * tlz * (g.M + 2) : 0)) * csize;
        else
            cfg->smem_z = (size_t)2 * g.nf * tlz * (g.M + g.M / 16 + 1) * csize;
        const int ntiles = (g.lines_z + tlz - 1) / tlz;
        int sms = 0, dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                      cudaSuccess || sms <= 0)
            sms = 152;
        cfg->sms = sms;
        const size_t smem_sm = 227 * 1024;
        int per_sm = (int)(smem_sm / cfg->smem_z);
        if (per_sm > 2) per_sm = 2;   // the Z passes' launch bounds
        if (tc && tc->z_per_sm > 0 && tc->z_per_sm < per_sm) per_sm = tc->z_per_sm;
        if (per_sm < 1) per_sm = 1;
        cfg->tc.z_per_sm = per_sm;
        cfg->nbz = ((g.gwev && !gw_staged) || ntiles < per_sm * sms) ? ntiles : per_sm * sms;
        g.pkg_stride = 2 * kMaxFields * cfg->nbx;
        g.pv_stride = kMaxTerms * cfg->nbz;
        return;
    }
    // generic engine: a tile of TL lines x N elements (TL a power of two: the kernels take
    // a line's index and element from the low and high bits of a thread index), two
    // ping-pong buffers of <= 32 KiB each
    int tl = 1;
    while (2 * tl <= (32768 / csize) / g.N) tl *= 2;
    if (tl < 4) tl = 4;
    if (tl > 256) tl = 256;
    while (tl > 1 && tl / 2 >= g.lines_x) tl /= 2;
    g.tlx_shift = ilog2i(tl);
    cfg->thr_xy = 256;
    cfg->smem_xy = (size_t)2 * tl * g.N * csize;
    cfg->smem_xf = cfg->smem_xy;
    cfg->smem_xi = cfg->smem_xy;
    cfg->smem_ys = 0;
    cfg->nbx = (g.lines_x + tl - 1) / tl;
    // Z pass: TLz lines, two H-row buffers + nslot M-row real-line slots.
    int tlz = 32;
    auto zbytes = [&](int t) { return (size_t)(t + 1) * (2 * g.H + nslot * g.M) * csize; };
    while (tlz > 1 && zbytes(tlz) > 100 * 1024) tlz /= 2;
    while (tlz > 1 && tlz / 2 >= g.lines_z) tlz /= 2;
    g.tlz_shift = ilog2i(tlz);
    g.ldz = tlz + 1;
    cfg->thr_z = 256;
    cfg->smem_z = zbytes(tlz);
    cfg->nbz = (g.lines_z + tlz - 1) / tlz;
    g.pkg_stride = 2 * kMaxFields * cfg->nbx;
    g.pv_stride = kMaxTerms * cfg->nbz;
}

template <typename T>
static cudaError_t configure_t(const LaunchCfg &cfg) {
    const int sxy = (int)cfg.smem_xy, sz = (int)cfg.smem_z;
    cudaError_t e;
#define SETA(kern, bytes)                                                                                  \
    e = cudaFuncSetAttribute((const void *)(kern), cudaFuncAttributeMaxDynamicSharedMemorySize, (bytes));  \
    if (e != cudaSuccess) return e;
    SETA((k_ifft_x<T, false, true>), sxy);
    SETA((k_ifft_x<T, true, true>), sxy);
    SETA((k_ifft_x<T, false, false>), sxy);
    SETA((k_ifft_x<T, true, false>), sxy);
    SETA((k_ifft_y<T, false>), sxy);
    SETA((k_ifft_y<T, true>), sxy);
    SETA((k_fft_y<T>), sxy);
    SETA((k_zpass<T, false>), sz);
    SETA((k_zpass<T, true>), sz);
    SETA((k_fft_x_final<T, false>), sxy);
    SETA((k_fft_x_final<T, true>), sxy);
    SETA((k_z_c2r_real<T>), sz);
    SETA((k_fft_x_plain<T>), sxy);
#undef SETA
    return cudaSuccess;
}

cudaError_t configure(const LaunchCfg &cfg, int precision) {
    if (cfg.g.reg) return precision == 32 ? reg_configure_f32(cfg) : reg_configure_f64(cfg);
    return precision == 32 ? configure_t<float>(cfg) : configure_t<double>(cfg);
}

template <typename T>
static cudaError_t launch_stage_t(const LaunchCfg &cfg, const Buffers &b, int drift, cudaStream_t st,
                                  cudaEvent_t *ev = nullptr, int scalar_mode = -1) {
    using C = cplx<T>;
    const Geo &g = cfg.g;
    const C *tw = reinterpret_cast<const C *>(b.tw);
    C *fk = (C *)b.fk, *pk = (C *)b.pk, *uk = (C *)b.uk, *puk = (C *)b.puk;
    C *TA = (C *)b.TA, *TB = (C *)b.TB, *TC = (C *)b.TC, *QV = (C *)b.QV, *QS = (C *)b.QS;
    const int R = cfg.R;
    const dim3 gx(cfg.nbx, g.nf, R);
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], st);
    };
    mark(0);
    if (g.gwev) {
        if (drift) k_ifft_x<T, true, true><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, fk, pk, TA, TB, b.bg, tw);
        else k_ifft_x<T, true, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, fk, pk, TA, TB, b.bg, tw);
        mark(1);
        k_ifft_y<T, true><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, TA, TB, TC, b.bg, tw);
        mark(2);
        k_zpass<T, true><<<dim3(cfg.nbz, 1, R), cfg.thr_z, cfg.smem_z, st>>>(g, TA, TB, TC, QV, QS, b.partV, b.bg, tw);
    } else {
        if (drift) k_ifft_x<T, false, true><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, fk, pk, TA, TB, b.bg, tw);
        else k_ifft_x<T, false, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, fk, pk, TA, TB, b.bg, tw);
        mark(1);
        k_ifft_y<T, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, TA, TB, TC, b.bg, tw);
        mark(2);
        k_zpass<T, false><<<dim3(cfg.nbz, 1, R), cfg.thr_z, cfg.smem_z, st>>>(g, TA, TB, TC, QV, QS, b.partV, b.bg, tw);
    }
    mark(3);
    ArrList al{};
    int nj = 0;
    for (int f = 0; f < g.nf; ++f) {
        al.rs[nj] = g.fstride;
        al.p[nj++] = QV + (long long)f * g.modes;
    }
    if (g.gwev)
        for (int c = 0; c < 6; ++c) {
            al.rs[nj] = g.gstride;
            al.p[nj++] = QS + (long long)c * g.modes;
        }
    k_fft_y<T><<<dim3(cfg.nbx, nj, R), cfg.thr_xy, cfg.smem_xy, st>>>(g, al, tw);
    mark(4);
    const dim3 gf(cfg.nbx, nj, R);
    if (g.gwev) k_fft_x_final<T, true><<<gf, cfg.thr_xy, cfg.smem_xy, st>>>(g, QV, QS, fk, pk, uk, puk, b.partKG, b.bg, tw);
    else k_fft_x_final<T, false><<<gf, cfg.thr_xy, cfg.smem_xy, st>>>(g, QV, QS, fk, pk, uk, puk, b.partKG, b.bg, tw);
    mark(5);
    if (scalar_mode >= 0) {
        k_scalar<<<cfg.R, kScalarThreads, 0, st>>>(b.bg, b.partKG, b.partV, scalar_mode, 1, cfg.g.pkg_stride, cfg.g.pv_stride,
                                         b.fk, b.pk, cfg.g.fstride, cfg.g.modes);
        mark(6);
    }
    return cudaGetLastError();
}

// The transforms of the padded step on the generic engine (N_pad not a power of two, or below
// 32), as RegLaunch::pad_passes: c2r of the padded spectra b.fk with the lattice's 1/N^3 (the
// background record's inv_n3), V'(f_pad) and the <V> partials over the padded sites, r2c into
// b.QV.
template <typename T>
static cudaError_t pad_passes_t(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st) {
    using C = cplx<T>;
    const Geo &g = cfg.g;
    const C *tw = reinterpret_cast<const C *>(b.tw);
    C *fk = (C *)b.fk, *TA = (C *)b.TA, *QV = (C *)b.QV;
    const dim3 gx(cfg.nbx, g.nf);
    k_ifft_x<T, false, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, fk, nullptr, TA, nullptr, b.bg, tw);
    k_ifft_y<T, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, TA, nullptr, nullptr, b.bg, tw);
    k_zpass<T, false><<<cfg.nbz, cfg.thr_z, cfg.smem_z, st>>>(g, TA, nullptr, nullptr, QV, nullptr, b.partV, b.bg, tw);
    ArrList al{};
    for (int f = 0; f < g.nf; ++f) {
        al.rs[f] = g.fstride;
        al.p[f] = QV + (long long)f * g.modes;
    }
    k_fft_y<T><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, al, tw);
    k_fft_x_plain<T><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, al, tw);
    return cudaGetLastError();
}

cudaError_t generic_pad_passes(const LaunchCfg &cfg, const Buffers &b, int precision, cudaStream_t st) {
    return precision == 32 ? pad_passes_t<float>(cfg, b, st) : pad_passes_t<double>(cfg, b, st);
}

cudaError_t launch_stage_timed(const LaunchCfg &cfg, const Buffers &b, int precision, int drift, int scalar_mode,
                               cudaEvent_t *ev, cudaStream_t st) {
    if (cfg.g.reg)
        return precision == 32 ? reg_stage_f32(cfg, b, drift, st, ev, scalar_mode)
                               : reg_stage_f64(cfg, b, drift, st, ev, scalar_mode);
    return precision == 32 ? launch_stage_t<float>(cfg, b, drift, st, ev, scalar_mode)
                           : launch_stage_t<double>(cfg, b, drift, st, ev, scalar_mode);
}

cudaError_t launch_stage(const LaunchCfg &cfg, const Buffers &b, int precision, int drift, cudaStream_t st) {
    if (cfg.g.reg)
        return precision == 32 ? reg_stage_f32(cfg, b, drift, st, nullptr, -1)
                               : reg_stage_f64(cfg, b, drift, st, nullptr, -1);
    return precision == 32 ? launch_stage_t<float>(cfg, b, drift, st) : launch_stage_t<double>(cfg, b, drift, st);
}

// SCALAR_END of stage p for every realization of every configuration of a batch: block i is
// realization i of the concatenated list (the groups' realizations in order). kScalarThreads
// threads, as k_scalar: the partial sums add up in the same order, so the background is the
// same bits.
__global__ void __launch_bounds__(kScalarThreads) k_scalar_batch(const __grid_constant__ BatchTable bt, int p) {
    unsigned r = blockIdx.x;
    int gi = 0;
    while (gi + 1 < bt.ngroups && r >= (unsigned)bt.grp[gi].R) {
        r -= (unsigned)bt.grp[gi].R;
        ++gi;
    }
    const BatchGroup &G = bt.grp[gi];
    k_scalar_body(r, G.bg, G.partKG, G.partV, SCALAR_END, p, G.g.pkg_stride, G.g.pv_stride, G.fk, G.pk, G.g.fstride,
                  G.g.modes);
}

cudaError_t launch_scalar_batch(const BatchTable &bt, int p, cudaStream_t st) {
    int n = 0;
    for (int i = 0; i < bt.ngroups; ++i) n += bt.grp[i].R;
    k_scalar_batch<<<n, kScalarThreads, 0, st>>>(bt, p);
    return cudaGetLastError();
}

cudaError_t launch_scalar(const LaunchCfg &cfg, const Buffers &b, int mode, int p, cudaStream_t st) {
    k_scalar<<<cfg.R, kScalarThreads, 0, st>>>(b.bg, b.partKG, b.partV, mode, p, cfg.g.pkg_stride, cfg.g.pv_stride, b.fk, b.pk,
                                     cfg.g.fstride, cfg.g.modes);
    return cudaGetLastError();
}

// pi += c_open F (pi_u += c_open F_u) for every realization: the opening half kick of a step
// call (evolution.cpp:1144-1158) from the force the previous call's last kick kept, with the
// epilogue's own arithmetic (pf = p + c_close F, then pf + c_open F).
template <typename T>
__global__ void __launch_bounds__(256) k_open_kick(Geo g, cplx<T> *__restrict__ pk, const cplx<T> *__restrict__ Fk,
                                                   cplx<T> *__restrict__ puk, const cplx<T> *__restrict__ Fu,
                                                   const DevBG *__restrict__ bg) {
    const int arr = blockIdx.y, r = blockIdx.z;
    bg += r;
    cplx<T> *p;
    const cplx<T> *F;
    if (arr < g.nf) {
        const long long off = (long long)r * g.fstride + (long long)arr * g.modes;
        p = pk + off;
        F = Fk + off;
    } else {
        const long long off = (long long)r * g.gstride + (long long)(arr - g.nf) * g.modes;
        p = puk + off;
        F = Fu + off;
    }
    const T c_close = (T)bg->c_close, c_open = (T)bg->c_open;
    const long long stride = (long long)gridDim.x * blockDim.x;
    // the homogeneous mode of a field has its opening kick in the background kernel (FP64)
    const long long m0 = (arr < g.nf && bg->zero64) ? 1 : 0;
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x + m0; m < g.modes; m += stride) {
        const cplx<T> f = F[m], q = p[m];
        const cplx<T> pf = mk<T>(q.x + c_close * f.x, q.y + c_close * f.y);
        p[m] = mk<T>(pf.x + c_open * f.x, pf.y + c_open * f.y);
    }
}

cudaError_t launch_open_kick(const LaunchCfg &cfg, const Buffers &b, int precision, cudaStream_t st) {
    const Geo &g = cfg.g;
    const dim3 grid(2 * 152, g.nf + (g.gwev ? 6 : 0), cfg.R);
    if (precision == 32)
        k_open_kick<float><<<grid, 256, 0, st>>>(g, (float2 *)b.pk, (const float2 *)b.Fk, (float2 *)b.puk,
                                                 (const float2 *)b.Fu, b.bg);
    else
        k_open_kick<double><<<grid, 256, 0, st>>>(g, (double2 *)b.pk, (const double2 *)b.Fk, (double2 *)b.puk,
                                                  (const double2 *)b.Fu, b.bg);
    return cudaGetLastError();
}

cudaError_t launch_set_run(DevBG *bg, int R, double dt, int nsteps, cudaStream_t st) {
    k_set_run<<<1, 128, 0, st>>>(bg, R, dt, nsteps);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_c2r_real_t(const LaunchCfg &cfg, const Buffers &b, const void *src, int nsrc,
                                     cudaStream_t st) {
    using C = cplx<T>;
    const Geo &g = cfg.g;
    const C *tw = reinterpret_cast<const C *>(b.tw);
    C *TA = (C *)b.TA;
    // one source array at a time through TA (TA holds nf arrays)
    for (int s0 = 0; s0 < nsrc; s0 += g.nf) {
        const int cnt = (nsrc - s0) < g.nf ? (nsrc - s0) : g.nf;
        const C *s = (const C *)src + (long long)s0 * g.modes;
        k_ifft_x<T, false, false><<<dim3(cfg.nbx, cnt), cfg.thr_xy, cfg.smem_xy, st>>>(g, (C *)s, nullptr, TA, nullptr,
                                                                                      b.bg, tw);
        k_ifft_y<T, false><<<dim3(cfg.nbx, cnt), cfg.thr_xy, cfg.smem_xy, st>>>(g, TA, nullptr, nullptr, b.bg, tw);
        k_z_c2r_real<T><<<dim3(cfg.nbz, cnt), cfg.thr_z, cfg.smem_z, st>>>(
            g, TA, (T *)b.real + (long long)s0 * g.sites, tw, (T)(1.0 / (double)g.sites));
    }
    return cudaGetLastError();
}

cudaError_t launch_c2r_real(const LaunchCfg &cfg, const Buffers &b, int precision, const void *src, int nsrc,
                            cudaStream_t st) {
    if (cfg.g.reg)
        return precision == 32 ? reg_c2r_real_f32(cfg, b, src, nsrc, st) : reg_c2r_real_f64(cfg, b, src, nsrc, st);
    return precision == 32 ? launch_c2r_real_t<float>(cfg, b, src, nsrc, st)
                           : launch_c2r_real_t<double>(cfg, b, src, nsrc, st);
}

template <typename T>
static cudaError_t launch_spectra_t(const LaunchCfg &cfg, const Buffers &b, int nb, cudaStream_t st) {
    using C = cplx<T>;
    const Geo &g = cfg.g;
    const size_t nacc = (size_t)g.nf * 3 * nb + 2 * nb, ncnt = (size_t)g.nf * nb + nb;
    cudaError_t e = cudaMemsetAsync(b.spec, 0, nacc * sizeof(double), st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(b.spec_cnt, 0, ncnt * sizeof(int), st);
    if (e != cudaSuccess) return e;
    const int blocks = 4 * 152;
    const size_t sm_s = (size_t)nb * (3 * sizeof(double) + sizeof(int));
    k_spectra_scalar<T><<<dim3(blocks, g.nf), 256, sm_s, st>>>(g, (const C *)b.fk, (const C *)b.pk, b.bg, nb, b.spec,
                                                               b.spec_cnt);
    if (g.gw) {
        const size_t sm_g = (size_t)nb * (2 * sizeof(double) + sizeof(int));
        k_spectra_gw<T><<<blocks, 256, sm_g, st>>>(g, (const C *)b.uk, (const C *)b.puk, b.bg, nb,
                                                   b.spec + (size_t)g.nf * 3 * nb, b.spec_cnt + (size_t)g.nf * nb);
    }
    return cudaGetLastError();
}

cudaError_t launch_spectra(const LaunchCfg &cfg, const Buffers &b, int precision, int nb, cudaStream_t st) {
    return precision == 32 ? launch_spectra_t<float>(cfg, b, nb, st) : launch_spectra_t<double>(cfg, b, nb, st);
}

}  // namespace psc
