// psc_pad.cu — the dealiased spectral step evolve_VV_k_pad (evolution.cpp:1271-1759) and
// the spectral prolongation of a coarser lattice's state.
//
// The padded step is the spectral step with V'(phi) and <V> evaluated on an N_pad grid:
//   padding()          evolution.cpp:1271-1443  f_k (N) -> f_k_pad (N_pad), zero outside the
//                       band |k_x|, |k_y|, k_z <= N/2, every Nyquist index (x, y or z = N/2)
//                       split over its +-N/2 images with a factor 1/2 per Nyquist axis;
//   c2r at N_pad / N^3, V'(f_pad), r2c at N_pad     (the register-engine passes at N_pad, or
//                       the generic engine's where N_pad is not a power of two >= 32);
//   extract_padding()  evolution.cpp:1446-1609  V'_k_pad -> V'_k, Nyquist entries taken from
//                       the +N/2 image times 2 per Nyquist axis, divided by (N_pad/N)^3;
//   kernel_field_k_pad evolution.cpp:1643-1682  the force, then the kicks as in the unpadded
//                       step; kernel_a_k_pad (evolution.cpp:1611-1637): K, G over every mode
//                       (the padded step never fills the R_Q2C mask, so none is excluded) and
//                       <V> over the padded sites.
// One thread per lattice mode scatters its value to its 1, 2 or 4 padded images; the
// padded entries outside the band are zero once and never written again.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "psc_dev.cuh"
#include "psc_handle.h"

namespace psc {
namespace {

constexpr int kPadThreads = 256;

// source mode (i, j, kz) of an Ns grid -> its images in the Nd grid (Nd > Ns), values
// scaled by `scale` and 1/2 per Nyquist axis; with DRIFT the source is first drifted,
// f_k += c_drift pi_half (evolution.cpp:1664-1668), and written back.
template <typename T, bool DRIFT>
__global__ void __launch_bounds__(kPadThreads) k_pad_scatter(cplx<T> *__restrict__ src, const cplx<T> *__restrict__ pk,
                                                             cplx<T> *__restrict__ dst, int Ns, int Nd,
                                                             long long modes_s, long long modes_d, T scale,
                                                             const DevBG *__restrict__ bg) {
    const int Hs = Ns / 2 + 1, Hd = Nd / 2 + 1, h = Ns / 2;
    src += (long long)blockIdx.y * modes_s;
    dst += (long long)blockIdx.y * modes_d;
    if (DRIFT) pk += (long long)blockIdx.y * modes_s;
    const T c = DRIFT ? (T)bg->c_drift : T(0);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < modes_s; m += stride) {
        const int kz = (int)(m % Hs);
        const long long l = m / Hs;
        const int j = (int)(l % Ns), i = (int)(l / Ns);
        cplx<T> v = src[m];
        if (DRIFT) {
            const cplx<T> p = pk[m];
            v.x += c * p.x;
            v.y += c * p.y;
            // the homogeneous mode: the background kernel's FP64 shadow, already drifted
            if (m == 0 && bg->zero64) v = mk<T>((T)bg->z0f[blockIdx.y][0], (T)bg->z0f[blockIdx.y][1]);
            src[m] = v;
        }
        T f = scale;
        if (i == h) f *= T(0.5);
        if (j == h) f *= T(0.5);
        if (kz == h) f *= T(0.5);
        v.x *= f;
        v.y *= f;
        const int I0 = i <= h ? i : Nd - (Ns - i), J0 = j <= h ? j : Nd - (Ns - j);
        const int I1 = (i == h) ? Nd - h : I0, J1 = (j == h) ? Nd - h : J0;
        dst[((long long)I0 * Nd + J0) * Hd + kz] = v;
        if (I1 != I0) dst[((long long)I1 * Nd + J0) * Hd + kz] = v;
        if (J1 != J0) dst[((long long)I0 * Nd + J1) * Hd + kz] = v;
        if (I1 != I0 && J1 != J0) dst[((long long)I1 * Nd + J1) * Hd + kz] = v;
    }
}

// extract_padding of V'_k_pad, the force of kernel_field_k_pad and the kicks of the
// stage (as the unpadded kick epilogue: closing half kick -> synchronised pi for the
// K, G partials, then the opening half kick of the next stage). One field per blockIdx.y;
// gridDim.x = the lattice's nbx (the K, G partial layout the background kernel reads).
template <typename T, typename C_ = cplx<T>>
__global__ void __launch_bounds__(kPadThreads) k_pad_kick(const cplx<T> *__restrict__ qvp, const cplx<T> *__restrict__ fk,
                                                          cplx<T> *__restrict__ pk, double *__restrict__ partKG,
                                                          int N, int Np, long long modes, long long modes_p,
                                                          T ratio3, const DevBG *__restrict__ bg,
                                                          C_ *__restrict__ fcache) {
    using C = cplx<T>;
    const int H = N / 2 + 1, Hp = Np / 2 + 1, h = N / 2;
    const int fld = blockIdx.y;
    qvp += (long long)fld * modes_p;
    fk += (long long)fld * modes;
    pk += (long long)fld * modes;
    if (fcache) fcache += (long long)fld * modes;
    const T norm1 = (T)bg->norm1, norm2 = (T)bg->norm2, kIR2 = (T)bg->kIR2;
    const T c_close = (T)bg->c_close, c_open = (T)bg->c_open;
    const bool keep = bg->c_open == 0.0 && fcache != nullptr;   // the force of a synchronising kick
    T accK = T(0), accG = T(0);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < modes; m += stride) {
        const int kz = (int)(m % H);
        const long long l = m / H;
        const int j = (int)(l % N), i = (int)(l / N);
        const int I = i <= h ? i : Np - (N - i), J = j <= h ? j : Np - (N - j);
        C q = qvp[((long long)I * Np + J) * Hp + kz];
        T g = T(1);
        if (i == h) g *= T(2);
        if (j == h) g *= T(2);
        if (kz == h) g *= T(2);
        // x 2 per Nyquist axis, / (N_pad/N)^3 (evolution.cpp:1602)
        q.x = q.x * g / ratio3;
        q.y = q.y * g / ratio3;
        const int px = pcoord(i, N), py = pcoord(j, N);
        const T k2 = (T)(px * px + py * py + kz * kz);
        const C f = fk[m], p = pk[m];
        if (m == 0 && bg->zero64) {   // the homogeneous mode: kicked in FP64 by the background kernel
            DevBG *bw = const_cast<DevBG *>(bg);
            bw->z0q[fld][0] = (double)q.x;
            bw->z0q[fld][1] = (double)q.y;
            bw->z0pending = 1;
            continue;
        }
        const T fl = -norm1 * kIR2 * k2;
        const C F = mk<T>(fl * f.x - norm2 * q.x, fl * f.y - norm2 * q.y);
        const C pf = mk<T>(p.x + c_close * F.x, p.y + c_close * F.y);
        const T wgt = (kz == 0 || kz == h) ? T(1) : T(2);
        accK += wgt * (pf.x * pf.x + pf.y * pf.y);
        accG += wgt * k2 * (f.x * f.x + f.y * f.y);
        pk[m] = mk<T>(pf.x + c_open * F.x, pf.y + c_open * F.y);
        if (keep) fcache[m] = F;
    }
    T vals[2] = {accK, accG};
    block_reduce_store_t<T, 2>(vals, partKG + (size_t)(2 * fld) * gridDim.x, gridDim.x, blockIdx.x);
}

template <typename T>
cudaError_t pad_stage_t(const LaunchCfg &cfg, const LaunchCfg &cfgp, const Buffers &b, const Buffers &bp, int drift,
                        cudaStream_t st) {
    using C = cplx<T>;
    const Geo &g = cfg.g, &gp = cfgp.g;
    const dim3 grid(cfg.nbx, g.nf);
    if (drift)
        k_pad_scatter<T, true><<<grid, kPadThreads, 0, st>>>((C *)b.fk, (const C *)b.pk, (C *)bp.fk, g.N, gp.N,
                                                             g.modes, gp.modes, T(1), b.bg);
    else
        k_pad_scatter<T, false><<<grid, kPadThreads, 0, st>>>((C *)b.fk, nullptr, (C *)bp.fk, g.N, gp.N, g.modes,
                                                              gp.modes, T(1), b.bg);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (gp.reg)
        e = sizeof(T) == 4 ? reg_pad_passes_f32(cfgp, bp, st) : reg_pad_passes_f64(cfgp, bp, st);
    else
        e = generic_pad_passes(cfgp, bp, sizeof(T) == 4 ? 32 : 64, st);
    if (e != cudaSuccess) return e;
    // extract_padding divides by pow((double)N_pad / N, 3) (evolution.cpp:1602)
    const double r3 = std::pow((double)gp.N / (double)g.N, 3);
    k_pad_kick<T><<<grid, kPadThreads, 0, st>>>((const C *)bp.QV, (const C *)b.fk, (C *)b.pk, b.partKG, g.N, gp.N,
                                                g.modes, gp.modes, (T)r3, b.bg, (C *)b.Fk);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pad_stage(const LaunchCfg &cfg, const LaunchCfg &cfgp, const Buffers &b, const Buffers &bp,
                             int precision, int drift, cudaStream_t st) {
    return precision == 32 ? pad_stage_t<float>(cfg, cfgp, b, bp, drift, st)
                           : pad_stage_t<double>(cfg, cfgp, b, bp, drift, st);
}

cudaError_t launch_prolong(const void *src, void *dst, int nsrc_arrays, int Ns, int Nd, int precision,
                           cudaStream_t st) {
    const long long ms = (long long)Ns * Ns * (Ns / 2 + 1), md = (long long)Nd * Nd * (Nd / 2 + 1);
    const double r = (double)Nd / (double)Ns, scale = r * r * r;
    const size_t csize = precision == 32 ? 8 : 16;
    cudaError_t e = cudaMemsetAsync(dst, 0, (size_t)md * nsrc_arrays * csize, st);
    if (e != cudaSuccess) return e;
    const dim3 grid(4 * 152, nsrc_arrays);
    if (precision == 32)
        k_pad_scatter<float, false><<<grid, kPadThreads, 0, st>>>((float2 *)src, nullptr, (float2 *)dst, Ns, Nd, ms, md,
                                                                 (float)scale, nullptr);
    else
        k_pad_scatter<double, false><<<grid, kPadThreads, 0, st>>>((double2 *)src, nullptr, (double2 *)dst, Ns, Nd, ms,
                                                                  md, scale, nullptr);
    return cudaGetLastError();
}

}  // namespace psc
