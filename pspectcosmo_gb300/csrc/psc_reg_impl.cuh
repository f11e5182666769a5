// psc_reg_impl.cuh — launchers of the register-engine passes for one precision
// (included by psc_reg_f32.cu / psc_reg_f64.cu so the two precisions compile in
// parallel). Dispatches the run-time lattice size to the compile-time line
// lengths L = N (X, Y passes) and L = N/2 (Z pass).
#pragma once

#include "psc_passes.cuh"

namespace psc {

template <typename T, int N>
struct RegLaunch {
    using C = cplx<T>;
    static constexpr int M = N / 2;
    // the Y forward pass staged by tensor maps (kr_fft_y_pipe): FP32, N = 128 .. 1024
    static constexpr bool kYPipe = sizeof(T) == 4 && y_pipe_size(N);

    static void gw_adj_tile(int nf, int *tl, int *sh);
    // the scalar adjoint Z pass (adj_z_tile / adj_z_blocks, psc_launch.h)
    static void zadj_tile(int nf, int *tl, int *sh) {
        const int t = adj_z_tile(N, nf);
        int s = 0;
        while ((1 << s) < t) ++s;
        *tl = t;
        *sh = s;
    }

    static cudaError_t configure(const LaunchCfg &cfg) {
        const int sxy = (int)cfg.smem_xy, sz = (int)cfg.smem_z;
        cudaError_t e;
#define SETA(kern, bytes)                                                                                   \
    e = cudaFuncSetAttribute((const void *)(kern), cudaFuncAttributeMaxDynamicSharedMemorySize, (bytes));   \
    if (e != cudaSuccess) return e;                                                                         \
    e = cudaFuncSetAttribute((const void *)(kern), cudaFuncAttributePreferredSharedMemoryCarveout,         \
                             cudaSharedmemCarveoutMaxShared);                                               \
    if (e != cudaSuccess) return e;
        SETA((kr_ifft_x<T, N, false, true>), (int)cfg.smem_xi);
        SETA((kr_ifft_x<T, N, true, true>), (int)cfg.smem_xi);
        SETA((kr_ifft_x<T, N, false, false>), (int)cfg.smem_xi);
        SETA((kr_ifft_x<T, N, true, false>), (int)cfg.smem_xi);
        SETA((kr_ifft_y<T, N, false>), sxy);
        SETA((kr_ifft_y<T, N, true>), 3 * sxy);   // exchange tile + TA and TB staging tiles
        SETA((kr_fft_y<T, N>), sxy);
        if constexpr (kYPipe) {   // the Y passes staged by tensor maps: 128-byte aligned buffers
            SETA((kr_fft_y_pipe<T, N>), 2 * (int)cfg.smem_ys + 128);
            SETA((kr_ifft_y_pipe<T, N>), 2 * (int)cfg.smem_ys + sxy + 128);   // + the exchange tile
        }
        SETA((kr_fft_x_final<T, N, false>), (int)cfg.smem_xf);
        SETA((kr_fft_x_final<T, N, true>), (int)cfg.smem_xf);
        SETA((kr_zpass<T, M>), sz);
        SETA((kr_zpass_gw<T, N, sizeof(T) == 4>), sz);
        if (model_is_user(cfg.g.model)) {   // the Z passes of the user models (psc_reg_user_*.cu)
            if constexpr (sizeof(T) == 4) e = reg_configure_user_f32(cfg);
            else e = reg_configure_user_f64(cfg);
            if (e != cudaSuccess) return e;
        }
        SETA((kr_z_c2r_real<T, M>), (int)((256 / (M / 16)) * ZIdx<M>::LS * sizeof(C)));
        {
            int tl = 1, sh = 0;
            zadj_tile(cfg.g.nf, &tl, &sh);
            SETA((kr_zpass_adj<T, M>), (int)(cfg.g.nf * tl * ZIdx<M>::LS * sizeof(C)));
        }
        SETA((kr_fft_x_plain<T, N>), sxy);
        SETA((kr_fft_x_adj<T, N>), sxy);
        SETA((kr_fft_x_gwadj<T, N>), sxy);
        {
            int tl = 1, sh = 0;
            gw_adj_tile(cfg.g.nf, &tl, &sh);
            SETA((kr_zpass_adj_gw<T, N>), (int)((cfg.g.nf + 4) * tl * ZIdx<N>::LS * sizeof(C)));
        }
#undef SETA
        return cudaSuccess;
    }

    // The fused Z pass of R realizations: kr_zpass_gw on the real-space path with GWs,
    // kr_zpass otherwise. USER = true: the instantiations of the user models (up to
    // kMaxFields fields), compiled in psc_reg_user_*.cu only.
    template <bool USER>
    static cudaError_t zpass(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st, int R) {
        const Geo &g = cfg.g;
        const C *tw = reinterpret_cast<const C *>(b.tw);
        C *TA = (C *)b.TA, *TB = (C *)b.TB, *TC = (C *)b.TC, *QV = (C *)b.QV, *QS = (C *)b.QS;
        if (g.gwev)
            kr_zpass_gw<T, N, sizeof(T) == 4, USER><<<dim3(cfg.nbz, 1, R), cfg.thr_z, cfg.smem_z, st>>>(
                g, TA, TB, TC, QV, QS, b.partV, b.bg, tw, (T *)b.tape_fx);
        else
            kr_zpass<T, M, USER><<<dim3(cfg.nbz, 1, R), cfg.thr_z, cfg.smem_z, st>>>(g, TA, QV, b.partV, b.bg, tw,
                                                                                  (T *)b.tape_fx);
        return cudaGetLastError();
    }
    template <bool USER>
    static cudaError_t configure_z(const LaunchCfg &cfg) {
        const void *kz[2] = {(const void *)kr_zpass<T, M, USER>, (const void *)kr_zpass_gw<T, N, sizeof(T) == 4, USER>};
        for (const void *k : kz) {
            cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem_z);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    static void zpass_any(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st, int R) {
        if (model_is_user(cfg.g.model)) {
            if constexpr (sizeof(T) == 4) reg_zpass_user_f32(cfg, b, st, R);
            else reg_zpass_user_f64(cfg, b, st, R);
        } else {
            zpass<false>(cfg, b, st, R);
        }
    }

    static cudaError_t stage(const LaunchCfg &cfg, const Buffers &b, int drift, cudaStream_t st, cudaEvent_t *ev,
                             int scalar_mode) {
        const Geo &g = cfg.g;
        const C *tw = reinterpret_cast<const C *>(b.tw);
        C *fk = (C *)b.fk, *pk = (C *)b.pk, *uk = (C *)b.uk, *puk = (C *)b.puk;
        C *TA = (C *)b.TA, *TB = (C *)b.TB, *TC = (C *)b.TC, *QV = (C *)b.QV, *QS = (C *)b.QS;
        const int R = cfg.R;
        const dim3 gx(cfg.nbx, g.nf, R);
        const int txy = cfg.thr_xy, tz = cfg.thr_z;
        auto mark = [&](int i) {
            if (ev) cudaEventRecord(ev[i], st);
        };
        // the X passes' operand tiles by tensor copies where the handle has tensor maps
        const XTma xt = (b.xtma && b.xtma->on) ? *b.xtma : XTma{};
        const size_t sxi = (xt.on && xt.xi) ? cfg.smem_xi : cfg.smem_xy;
        // the Y forward pass's tiles by tensor copies where the handle has tensor maps for them
        // (the encoder gives them only to FP32 and the sizes with the tensor-map instantiation)
        const bool ypl = kYPipe && b.ytma && b.ytma->on;
        mark(0);
        if (g.gwev) {
            if (drift) kr_ifft_x<T, N, true, true><<<gx, txy, sxi, st>>>(g, fk, pk, TA, TB, b.bg, tw, xt);
            else kr_ifft_x<T, N, true, false><<<gx, txy, sxi, st>>>(g, fk, pk, TA, TB, b.bg, tw, xt);
            mark(1);
            bool ipiped = false;
            if constexpr (kYPipe) {
                if (b.ytma_i && b.ytma_i->on) {
                    // persistent and pipelined: two blocks per SM (one for 1024-point lines)
                    const long long items = (long long)cfg.nbx * g.nf * R, wave = (long long)xy_blocks<N>(2) * cfg.sms;
                    const int grid = (int)(items < wave ? items : wave);
                    kr_ifft_y_pipe<T, N><<<grid, txy, 2 * cfg.smem_ys + cfg.smem_xy + 128, st>>>(g, TA, TB, TC, b.bg, tw,
                                                                                              *b.ytma_i, R);
                    ipiped = true;
                }
            }
            if (!ipiped) kr_ifft_y<T, N, true><<<gx, txy, 3 * cfg.smem_xy, st>>>(g, TA, TB, TC, b.bg, tw);
            mark(2);
            zpass_any(cfg, b, st, R);
        } else {
            if (drift) kr_ifft_x<T, N, false, true><<<gx, txy, sxi, st>>>(g, fk, pk, TA, TB, b.bg, tw, xt);
            else kr_ifft_x<T, N, false, false><<<gx, txy, sxi, st>>>(g, fk, pk, TA, TB, b.bg, tw, xt);
            mark(1);
            kr_ifft_y<T, N, false><<<gx, txy, cfg.smem_xy, st>>>(g, TA, TB, TC, b.bg, tw);
            mark(2);
            zpass_any(cfg, b, st, R);
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
        if (!ypl) {
            kr_fft_y<T, N><<<dim3(cfg.nbx, nj, R), txy, cfg.smem_xy, st>>>(g, al, tw);
        } else if constexpr (kYPipe) {
            // persistent and pipelined: two blocks per SM (one for 1024-point lines) walk the items
            const long long items = (long long)cfg.nbx * nj * R, wave = (long long)xy_blocks<N>(2) * cfg.sms;
            const int grid = (int)(items < wave ? items : wave);
            kr_fft_y_pipe<T, N><<<grid, txy, 2 * cfg.smem_ys + 128, st>>>(g, al, tw, b.bg, *b.ytma, nj, R);
        }
        mark(4);
        const dim3 gf(cfg.nbx, nj, R);
        if (g.gwev)
            kr_fft_x_final<T, N, true><<<gf, txy, cfg.smem_xf, st>>>(g, QV, QS, fk, pk, uk, puk, b.partKG, b.bg, tw,
                                                                      (C *)b.tape_f, (C *)b.tape_p, (C *)b.tape_vp,
                                                                      (C *)b.tape_pu, (C *)b.tape_fu, (C *)b.Fk,
                                                                      (C *)b.Fu, xt);
        else
            kr_fft_x_final<T, N, false><<<gf, txy, cfg.smem_xf, st>>>(g, QV, QS, fk, pk, uk, puk, b.partKG, b.bg, tw,
                                                                       (C *)b.tape_f, (C *)b.tape_p, (C *)b.tape_vp,
                                                                       nullptr, nullptr, (C *)b.Fk, nullptr, xt);
        mark(5);
        if (scalar_mode >= 0) {
            cudaError_t e = launch_scalar(cfg, b, scalar_mode, 1, st);
            if (e != cudaSuccess) return e;
            mark(6);
        }
        return cudaGetLastError();
    }

    // The transforms of the padded step (evolution.cpp:1639-1661) on the padded grid, this
    // N being N_pad: c2r of the padded spectra b.fk with the lattice's 1/N^3, V'(f_pad)
    // and the <V> partials over the padded sites, r2c, ending in k-space in b.QV.
    static cudaError_t pad_passes(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st) {
        const Geo &g = cfg.g;
        const C *tw = reinterpret_cast<const C *>(b.tw);
        C *fk = (C *)b.fk, *TA = (C *)b.TA, *QV = (C *)b.QV;
        const dim3 gx(cfg.nbx, g.nf);
        kr_ifft_x<T, N, false, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, fk, nullptr, TA, nullptr, b.bg, tw);
        kr_ifft_y<T, N, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, TA, nullptr, nullptr, b.bg, tw);
        zpass_any(cfg, b, st, 1);
        ArrList al{};
        for (int f = 0; f < g.nf; ++f) {
            al.rs[f] = g.fstride;
            al.p[f] = QV + (long long)f * g.modes;
        }
        kr_fft_y<T, N><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, al, tw);
        kr_fft_x_plain<T, N><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, al, tw);
        return cudaGetLastError();
    }

    static cudaError_t c2r_real(const LaunchCfg &cfg, const Buffers &b, const void *src, int nsrc, cudaStream_t st) {
        const Geo &g = cfg.g;
        const C *tw = reinterpret_cast<const C *>(b.tw);
        C *TA = (C *)b.TA;
        constexpr int P = M / 16;
        int tl = 256 / P;
        int sh = 0;
        while ((1 << sh) < tl) ++sh;
        const size_t smem = (size_t)tl * ZIdx<M>::LS * sizeof(C);
        const int nbz = (g.lines_z + tl - 1) / tl;
        for (int s0 = 0; s0 < nsrc; s0 += g.nf) {
            const int cnt = (nsrc - s0) < g.nf ? (nsrc - s0) : g.nf;
            const C *s = (const C *)src + (long long)s0 * g.modes;
            kr_ifft_x<T, N, false, false><<<dim3(cfg.nbx, cnt), cfg.thr_xy, cfg.smem_xy, st>>>(
                g, (C *)s, nullptr, TA, nullptr, b.bg, tw);
            kr_ifft_y<T, N, false><<<dim3(cfg.nbx, cnt), cfg.thr_xy, cfg.smem_xy, st>>>(g, TA, nullptr, nullptr, b.bg,
                                                                                      tw);
            kr_z_c2r_real<T, M><<<dim3(nbz, cnt), tl * P, smem, st>>>(g, TA, (T *)b.real + (long long)s0 * g.sites,
                                                                     tw, (T)(1.0 / (double)g.sites), sh);
        }
        return cudaGetLastError();
    }

    // J^T application of the adjoint at a stage point (no GW, one lattice): c2r of
    // Mk (X, Y inverse passes into TA), the fused Z pass with the taped real fields,
    // the Y forward pass and the X forward pass adding into Lf.
    static cudaError_t adj_point(const LaunchCfg &cfg, const Buffers &b, const void *Mk, const void *f_tape,
                                 const void *fx_tape, void *Lf, double *part, const DevAdj *ad, cudaStream_t st) {
        const Geo &g = cfg.g;
        const C *tw = reinterpret_cast<const C *>(b.tw);
        C *TA = (C *)b.TA, *QV = (C *)b.QV;
        const dim3 gx(cfg.nbx, g.nf);
        kr_ifft_x<T, N, false, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, (C *)Mk, nullptr, TA, nullptr, b.bg, tw);
        kr_ifft_y<T, N, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, TA, nullptr, nullptr, b.bg, tw);
        int tl = 1, sh = 0;
        zadj_tile(g.nf, &tl, &sh);
        const int nbz = adj_z_blocks(N, g.nf);
        kr_zpass_adj<T, M><<<nbz, g.nf * (M / 16) * tl, (size_t)g.nf * tl * ZIdx<M>::LS * sizeof(C), st>>>(
            g, TA, (const T *)fx_tape, QV, part, ad, tw, sh);
        ArrList al{};
        for (int f = 0; f < g.nf; ++f) al.p[f] = QV + (long long)f * g.modes;
        kr_fft_y<T, N><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, al, tw);
        kr_fft_x_adj<T, N><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, QV, (const C *)Mk, (const C *)f_tape, (C *)Lf, ad,
                                                                 tw);
        return cudaGetLastError();
    }

    // transposed GW source at a stage point (one lattice with GWs): the field gradients of
    // the taped f (X, Y inverse GW passes into TA, TB, TC), the six adjoint components Mu
    // (X, Y inverse into QS), the GW adjoint Z pass into Tarr (3 nf arrays), the Y forward
    // pass and the X forward pass adding etaS sum_a i k_a T_a into Lf.
    static cudaError_t adj_point_gw(const LaunchCfg &cfg, const Buffers &b, const void *Mu, const void *f_tape,
                                    void *Tarr, void *Lf, const DevAdj *ad, cudaStream_t st) {
        const Geo &g = cfg.g;
        const C *tw = reinterpret_cast<const C *>(b.tw);
        C *TA = (C *)b.TA, *TB = (C *)b.TB, *TC = (C *)b.TC, *QS = (C *)b.QS;
        const dim3 gx(cfg.nbx, g.nf), g6(cfg.nbx, 6);
        kr_ifft_x<T, N, true, false><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, (C *)f_tape, nullptr, TA, TB, b.bg, tw);
        kr_ifft_y<T, N, true><<<gx, cfg.thr_xy, 3 * cfg.smem_xy, st>>>(g, TA, TB, TC, b.bg, tw);
        kr_ifft_x<T, N, false, false><<<g6, cfg.thr_xy, cfg.smem_xy, st>>>(g, (C *)Mu, nullptr, QS, nullptr, b.bg, tw);
        kr_ifft_y<T, N, false><<<g6, cfg.thr_xy, cfg.smem_xy, st>>>(g, QS, nullptr, nullptr, b.bg, tw);
        int tl = 1, sh = 0;
        gw_adj_tile(g.nf, &tl, &sh);
        const int pin = g.nf + 4, P = N / 16;
        const size_t smem = (size_t)pin * tl * ZIdx<N>::LS * sizeof(C);
        kr_zpass_adj_gw<T, N><<<(g.lines_z + tl - 1) / tl, pin * P * tl, smem, st>>>(g, TA, TB, TC, QS, (C *)Tarr, tw,
                                                                                    sh);
        ArrList al{};
        for (int i = 0; i < 3 * g.nf; ++i) al.p[i] = (C *)Tarr + (long long)i * g.modes;
        kr_fft_y<T, N><<<dim3(cfg.nbx, 3 * g.nf), cfg.thr_xy, cfg.smem_xy, st>>>(g, al, tw);
        kr_fft_x_gwadj<T, N><<<gx, cfg.thr_xy, cfg.smem_xy, st>>>(g, (const C *)Tarr, (C *)Lf, ad, tw);
        return cudaGetLastError();
    }
};

// the GW adjoint Z pass: nf + 4 input pairs of P = N/16 threads each per line
template <typename T, int N>
void RegLaunch<T, N>::gw_adj_tile(int nf, int *tl, int *sh) {
    const int pin = nf + 4, P = N / 16;
    int t = 1;
    while (pin * P * t * 2 <= 256) t *= 2;
    int s = 0;
    while ((1 << s) < t) ++s;
    *tl = t;
    *sh = s;
}

template <typename T>
struct RegDispatch {
    template <typename F>
    static cudaError_t on(int N, F &&f) {
        switch (N) {
        case 32: return f(RegLaunch<T, 32>());
        case 64: return f(RegLaunch<T, 64>());
        case 128: return f(RegLaunch<T, 128>());
        case 256: return f(RegLaunch<T, 256>());
        case 512: return f(RegLaunch<T, 512>());
        case 1024: return f(RegLaunch<T, 1024>());
        default: return cudaErrorInvalidValue;
        }
    }
};

}  // namespace psc

// The user-model Z passes of one precision (psc_reg_user_f32.cu, psc_reg_user_f64.cu).
#define PSC_DEFINE_REG_USER_ENTRY(T, SUFFIX)                                                                     \
    namespace psc {                                                                                              \
    cudaError_t reg_configure_user_##SUFFIX(const LaunchCfg &cfg) {                                              \
        return RegDispatch<T>::on(cfg.g.N, [&](auto L) { return decltype(L)::template configure_z<true>(cfg); }); \
    }                                                                                                            \
    cudaError_t reg_zpass_user_##SUFFIX(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st, int R) {        \
        return RegDispatch<T>::on(cfg.g.N, [&](auto L) { return decltype(L)::template zpass<true>(cfg, b, st, R); }); \
    }                                                                                                            \
    }

#define PSC_DEFINE_REG_ENTRY(T, SUFFIX)                                                                          \
    namespace psc {                                                                                              \
    cudaError_t reg_adj_point_##SUFFIX(const LaunchCfg &cfg, const Buffers &b, const void *Mk, const void *f_tape, \
                                       const void *fx_tape, void *Lf, double *part, const DevAdj *ad,             \
                                       cudaStream_t st) {                                                         \
        return RegDispatch<T>::on(cfg.g.N, [&](auto L) {                                                         \
            return decltype(L)::adj_point(cfg, b, Mk, f_tape, fx_tape, Lf, part, ad, st);                        \
        });                                                                                                      \
    }                                                                                                            \
    cudaError_t reg_adj_point_gw_##SUFFIX(const LaunchCfg &cfg, const Buffers &b, const void *Mu,               \
                                          const void *f_tape, void *Tarr, void *Lf, const DevAdj *ad,             \
                                          cudaStream_t st) {                                                      \
        return RegDispatch<T>::on(cfg.g.N, [&](auto L) {                                                         \
            return decltype(L)::adj_point_gw(cfg, b, Mu, f_tape, Tarr, Lf, ad, st);                              \
        });                                                                                                      \
    }                                                                                                            \
    cudaError_t reg_configure_##SUFFIX(const LaunchCfg &cfg) {                                                   \
        return RegDispatch<T>::on(cfg.g.N, [&](auto L) { return decltype(L)::configure(cfg); });                 \
    }                                                                                                            \
    cudaError_t reg_stage_##SUFFIX(const LaunchCfg &cfg, const Buffers &b, int drift, cudaStream_t st,           \
                                   cudaEvent_t *ev, int scalar_mode) {                                           \
        return RegDispatch<T>::on(cfg.g.N,                                                                       \
                                  [&](auto L) { return decltype(L)::stage(cfg, b, drift, st, ev, scalar_mode); }); \
    }                                                                                                            \
    cudaError_t reg_pad_passes_##SUFFIX(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st) {               \
        return RegDispatch<T>::on(cfg.g.N, [&](auto L) { return decltype(L)::pad_passes(cfg, b, st); });          \
    }                                                                                                            \
    cudaError_t reg_c2r_real_##SUFFIX(const LaunchCfg &cfg, const Buffers &b, const void *src, int nsrc,         \
                                      cudaStream_t st) {                                                         \
        return RegDispatch<T>::on(cfg.g.N, [&](auto L) { return decltype(L)::c2r_real(cfg, b, src, nsrc, st); }); \
    }                                                                                                            \
    }
