// psc_passes.cuh — the pass kernels on the register-resident FFT engine
// (psc_fftreg.cuh), templated on precision T and line length L. Used for
// N >= 32; the generic shared-memory engine of psc_kernels.cu covers N = 8, 16.
//
// Thread layout of the X/Y passes (strided lines): TL lines x P = L/16 threads,
// t fastest, so each of a thread's 16 loads is one coalesced TL-wide row.
// Thread layout of the Z passes (contiguous lines): (input, line, j) with j
// fastest, so consecutive threads read consecutive kz of one line; all inputs
// of a tile are transformed at the same time and meet in shared memory for the
// pointwise epilogue. Without GWs an input is one field's line, transformed by
// half-length packing (kr_zpass); with GWs an input is a pair of real lines
// carried as one complex line through a full-length transform (kr_zpass_gw, and
// the adjoint's kr_zpass_adj_gw).
#pragma once

#include "psc_fftreg.cuh"
#include "psc_launch.h"

namespace psc {

// X/Y pass block sizes: 256 threads, except 512 for 1024-point lines, so that a block
// still holds 8 lines (64 contiguous bytes of every FP32 row it streams instead of 32).
// Both give the kernels the same 128-register budget.
template <int L> constexpr int xy_threads() { return L >= 1024 ? 512 : 256; }
template <int L> constexpr int xy_blocks(int k) { return L >= 1024 ? 1 : k; }

// The block a pass body works on: its indices and the width of the grid along x (the stride
// of the persistent Z passes). A kernel of one lattice (or of R realizations of one
// configuration) passes its own blockIdx and gridDim; the batched kernels of several
// configurations pass a block of one configuration's grid.
// HwBlock reads the hardware indices where they are used (no registers held for them, as in a
// kernel written with blockIdx); VBlock carries the indices of a block of another grid.
struct HwBlock {
    __device__ __forceinline__ unsigned x() const { return blockIdx.x; }
    __device__ __forceinline__ unsigned y() const { return blockIdx.y; }
    __device__ __forceinline__ unsigned z() const { return blockIdx.z; }
    __device__ __forceinline__ unsigned gx() const { return gridDim.x; }
};
struct VBlock {
    unsigned x_, y_, z_, gx_;
    __device__ __forceinline__ unsigned x() const { return x_; }
    __device__ __forceinline__ unsigned y() const { return y_; }
    __device__ __forceinline__ unsigned z() const { return z_; }
    __device__ __forceinline__ unsigned gx() const { return gx_; }
};
__device__ __forceinline__ HwBlock vblock_hw() { return HwBlock{}; }

// One X-pass tile (TL lines x L points, line fastest) of array `arr`, realization z, by tensor
// copies from the map m (box {TL lines, XB x}): L / XB boxes stacked along x, since a box edge
// is at most 256 (XB = min(L, 256)). c0: the tile's first line in 8-byte elements.
template <int L, typename C>
__device__ __forceinline__ void x_tile_tma(C *dst, const CUtensorMap *m, int c0, int TL, int arr, int z,
                                           uint64_t *bar) {
    constexpr int XB = L < 256 ? L : 256;
#pragma unroll
    for (int x0 = 0; x0 < L; x0 += XB) tma_load_4d(dst + x0 * TL, m, c0, x0, arr, z, bar);
}


// ------------------------------------------------------------------ X inverse (+ drift, + x-derivative)
template <typename T, int L, bool GW, bool DRIFT, class VB>
__device__ __forceinline__ void kr_ifft_x_body(const VB &vb, Geo g, cplx<T> *__restrict__ fk, const cplx<T> *__restrict__ pk, cplx<T> *__restrict__ TA, cplx<T> *__restrict__ TB, const DevBG *__restrict__ bg, const cplx<T> *__restrict__ tw, const XTma *tma) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);
    {
        const long long rf = (long long)vb.z() * g.fstride;
        fk += rf;
        if (DRIFT) pk += rf;
        TA += rf;
        if (GW) TB += rf;
        bg += vb.z();
    }
    const int sh = g.tlx_shift, TL = 1 << sh;
    const int t = threadIdx.x & (TL - 1), j = threadIdx.x >> sh;
    const int line = vb.x() * TL + t;
    const bool valid = line < g.lines_x;
    const long long stride = g.lines_x;
    const long long base = (long long)vb.y() * g.modes + line;
    auto ix = [&](int n) { return n * TL + t; };
    const T c = DRIFT ? (T)bg->c_drift : T(0);
    const T kIR = GW ? (T)bg->kIR : T(0);
    // With tensor maps (tma): the tile of f_k (and, drifting, of pi_half) comes into shared
    // memory by tiled copies of the tensor memory accelerator, issued by one thread and landing
    // on an mbarrier (128-byte aligned tiles: the launch adds 128 bytes of shared memory);
    // the drift updates the staged f_k too, so the GW derivative pass reads it from there.
    // Otherwise every thread loads its elements from global memory.
    __shared__ uint64_t ibar;
    const bool use_tma = tma != nullptr;
    C *opF = nullptr, *opP = nullptr;
    if (use_tma) {
        // a failed stage: no further waits (the block decides as one)
        if (__syncthreads_or(threadIdx.x == 0 && bg->err != 0)) return;
        opF = reinterpret_cast<C *>((reinterpret_cast<uintptr_t>(sm + TL * L) + 127) & ~(uintptr_t)127);
        opP = opF + TL * L;
        if (threadIdx.x == 0) {
            mbar_init(&ibar, 1);
            mbar_fence_init();
            mbar_arrive_expect_tx(&ibar, (DRIFT ? 2u : 1u) * (unsigned)(TL * L * sizeof(C)) + planted(bg, 0));
            const int w8 = (int)(sizeof(C) / 8), c0 = (int)(vb.x() * TL) * w8;
            x_tile_tma<L>(opF, &tma->fk, c0, TL, (int)vb.y(), (int)vb.z(), &ibar);
            if (DRIFT) x_tile_tma<L>(opP, &tma->pk, c0, TL, (int)vb.y(), (int)vb.z(), &ibar);
        }
        __syncthreads();   // the mbarrier is initialised before any thread waits on it
        // bounded wait, as the X forward + kick pass's: a timeout is reported, the copies in
        // flight are waited for once more, and the block leaves only after they landed
        const bool ok = mbar_wait_bounded(&ibar, 0, bg->wait_ns);
        if (__syncthreads_or(!ok)) {
            int *err = &const_cast<DevBG *>(bg)->err;
            if (threadIdx.x == 0) {
                report_err(err, PSC_ERR_TIMEOUT);
                if (planted(bg, 0)) mbar_complete_tx(&ibar, planted(bg, 0));   // the test hook's bytes
            }
            const bool landed = mbar_wait_bounded(&ibar, 0, bg->wait_ns);
            if (__syncthreads_or(!landed) && threadIdx.x == 0) report_err(err, PSC_ERR_DEVICE);
            return;
        }
    }
    // pass 0: (drifted) f -> TA; with GWs pass 1: i k_x f -> TB (one copy of the
    // transform code for both keeps the register allocation spill-free)
#pragma unroll 1
    for (int pass = 0; pass < (GW ? 2 : 1); ++pass) {
        if (pass) __syncthreads();   // the exchange buffer is free again
        // every load of the line before the first store back to f_k: the drift's
        // read-modify-write of f_k through one pointer would otherwise keep each load
        // behind the previous store (no alias proof at run-time strides)
        C v[16];
        if (use_tma) {
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = opF[ix(j + r * RP::P)];
        } else {
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = valid ? fk[base + (long long)(j + r * RP::P) * stride] : mk<T>(0, 0);
        }
        if (pass == 0 && DRIFT) {
            C pv[16];
            if (use_tma) {
#pragma unroll
                for (int r = 0; r < 16; ++r) pv[r] = opP[ix(j + r * RP::P)];
            } else {
#pragma unroll
                for (int r = 0; r < 16; ++r)
                    pv[r] = valid ? pk[base + (long long)(j + r * RP::P) * stride] : mk<T>(0, 0);
            }
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                v[r].x += c * pv[r].x;
                v[r].y += c * pv[r].y;
                if (valid) fk[base + (long long)(j + r * RP::P) * stride] = v[r];
                if (GW && use_tma) opF[ix(j + r * RP::P)] = v[r];   // this thread's own elements
            }
            if (line == 0 && j == 0 && bg->zero64) {
                // the homogeneous mode (element 0 of the line x = y = kz = 0) is the background
                // kernel's FP64 shadow, already drifted
                v[0] = mk<T>((T)bg->z0f[vb.y()][0], (T)bg->z0f[vb.y()][1]);
                fk[base] = v[0];
                if (GW && use_tma) opF[ix(0)] = v[0];
            }
        }
        if (pass == 1) {
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int n = j + r * RP::P;
                const T kx = (n == (g.N >> 1)) ? T(0) : kIR * (T)pcoord(n, g.N);
                v[r] = mk<T>(-kx * v[r].y, kx * v[r].x);
            }
        }
        fft_reg<C, L, +1>(v, sm, ix, j, tw, g.N / L);
        C *dst = pass ? TB : TA;
        if (valid) {
#pragma unroll
            for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                for (int r = 0; r < RP::RL; ++r) dst[base + (long long)RP::out(j, q, r) * stride] = v[q * RP::RL + r];
        }
    }
}

template <typename T, int L, bool GW, bool DRIFT>
__global__ void __launch_bounds__(xy_threads<L>(), xy_blocks<L>(2)) kr_ifft_x(Geo g, cplx<T> *__restrict__ fk, const cplx<T> *__restrict__ pk,
                                                 cplx<T> *__restrict__ TA, cplx<T> *__restrict__ TB,
                                                 const DevBG *__restrict__ bg, const cplx<T> *__restrict__ tw,
                                                 const __grid_constant__ XTma tma = XTma{}) {
    kr_ifft_x_body<T, L, GW, DRIFT, HwBlock>(vblock_hw(), g, fk, pk, TA, TB, bg, tw,
                                             (tma.on && tma.xi) ? &tma : nullptr);
}

// ------------------------------------------------------------------ Y passes
// One transform of a tile of Y lines (l = x H + kz, element y at (x N + y) H + kz):
// src -> dst (may alias), optional i k_y multiplier. Ends with a barrier.
template <typename T, int L, int DIR, class VB>
__device__ __forceinline__ void ry_tile(const VB &vb, const Geo &g, const cplx<T> *src, cplx<T> *dst, bool deriv, T kIR,
                                        cplx<T> *sm, const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    const int sh = g.tlx_shift, TL = 1 << sh;
    const int t = threadIdx.x & (TL - 1), j = threadIdx.x >> sh;
    const int line = vb.x() * TL + t;
    const bool valid = line < g.lines_x;
    const int x = line / g.H, kz = line - x * g.H;
    const long long base = (long long)x * g.N * g.H + kz;
    const long long stride = g.H;
    auto ix = [&](int n) { return n * TL + t; };
    C v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const int n = j + r * RP::P;
        C a = mk<T>(0, 0);
        if (valid) {
            a = src[base + (long long)n * stride];
            if (deriv) {
                const T ky = (n == (g.N >> 1)) ? T(0) : kIR * (T)pcoord(n, g.N);
                a = mk<T>(-ky * a.y, ky * a.x);
            }
        }
        v[r] = a;
    }
    fft_reg<C, L, DIR>(v, sm, ix, j, tw, g.N / L);
    if (valid) {
#pragma unroll
        for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
            for (int r = 0; r < RP::RL; ++r) dst[base + (long long)RP::out(j, q, r) * stride] = v[q * RP::RL + r];
    }
    __syncthreads();
}

template <typename T, int L, bool GW, class VB>
__device__ __forceinline__ void kr_ifft_y_body(const VB &vb, Geo g, cplx<T> *__restrict__ TA, cplx<T> *__restrict__ TB, cplx<T> *__restrict__ TC, const DevBG *__restrict__ bg, const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);
    const long long off = (long long)vb.y() * g.modes + (long long)vb.z() * g.fstride;
    bg += vb.z();
    const T kIR = (T)bg->kIR;
    if (GW) {
        // This thread's TA and TB elements are copied into two shared staging tiles by
        // cp.async at once (every load in flight together, TA read from HBM once); then
        // three transforms from the tiles: d/dy TA -> TC, TA -> TA, TB -> TB (one copy of the
        // transform code keeps the register allocation spill-free). (Staged by tensor copies
        // instead, as the Y forward pass is, this pass measured slower on GB300: 0.215 against
        // 0.201 ms at 256^3.)
        using RP = RegPlan<L>;
        const int sh = g.tlx_shift, TL = 1 << sh;
        const int t = threadIdx.x & (TL - 1), j = threadIdx.x >> sh;
        const int line = vb.x() * TL + t;
        const bool valid = line < g.lines_x;
        const int x = line / g.H, kz = line - x * g.H;
        const long long base = off + (long long)x * g.N * g.H + kz;
        const long long stride = g.H;
        auto ix = [&](int n) { return n * TL + t; };
        C *stA = sm + TL * L, *stB = stA + TL * L;
        if (valid) {
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int n = j + r * RP::P;
                cp_async_elem(stA + ix(n), TA + base + (long long)n * stride);
                cp_async_elem(stB + ix(n), TB + base + (long long)n * stride);
            }
        }
        cp_async_commit();
        cp_async_wait_all();   // own elements only: no barrier needed to read them
#pragma unroll 1
        for (int a = 0; a < 3; ++a) {
            if (a) __syncthreads();   // the exchange buffer is free again
            const C *st = (a == 2) ? stB : stA;
            C v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int n = j + r * RP::P;
                C e = valid ? st[ix(n)] : mk<T>(0, 0);
                if (a == 0) {
                    const T ky = (n == (g.N >> 1)) ? T(0) : kIR * (T)pcoord(n, g.N);
                    e = mk<T>(-ky * e.y, ky * e.x);
                }
                v[r] = e;
            }
            fft_reg<C, L, +1>(v, sm, ix, j, tw, g.N / L);
            C *dst = (a == 0 ? TC : (a == 1 ? TA : TB));
            if (valid) {
#pragma unroll
                for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                    for (int r = 0; r < RP::RL; ++r)
                        dst[base + (long long)RP::out(j, q, r) * stride] = v[q * RP::RL + r];
            }
        }
    } else {
        ry_tile<T, L, +1, VB>(vb, g, TA + off, TA + off, false, kIR, sm, tw);
    }
}

template <typename T, int L, bool GW>
__global__ void __launch_bounds__(xy_threads<L>(), xy_blocks<L>(2)) kr_ifft_y(Geo g, cplx<T> *__restrict__ TA, cplx<T> *__restrict__ TB,
                                                 cplx<T> *__restrict__ TC, const DevBG *__restrict__ bg,
                                                 const cplx<T> *__restrict__ tw) {
    kr_ifft_y_body<T, L, GW, HwBlock>(vblock_hw(), g, TA, TB, TC, bg, tw);
}


template <typename T, int L, class VB>
__device__ __forceinline__ void kr_fft_y_body(const VB &vb, Geo g, const ArrList &arrs, const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);
    C *a = reinterpret_cast<C *>(arrs.p[vb.y()]) + (long long)vb.z() * arrs.rs[vb.y()];
    ry_tile<T, L, -1, VB>(vb, g, a, a, false, T(0), sm, tw);
}

template <typename T, int L>
__global__ void __launch_bounds__(xy_threads<L>(), xy_blocks<L>(3)) kr_fft_y(Geo g, const __grid_constant__ ArrList arrs,
                                                 const cplx<T> *__restrict__ tw) {
    kr_fft_y_body<T, L, HwBlock>(vblock_hw(), g, arrs, tw);
}

// Y forward pass staged by tensor maps (YTma, psc_launch.h). Its tiles: the first N (N/2)/TL
// hold TL consecutive kz < N/2 of one x plane, staged by two tensor copies (the even and the
// odd rows); the last N/TL hold the kz = N/2 column of TL consecutive x, staged by each
// thread's cp.async copies into the same layout. Together they cover the N H lines in the
// same number of tiles as kr_fft_y (TL divides N/2), and every line is transformed alike.
struct YTile {
    int x, kz;     // this thread's line
    int x0, kz0;   // the tile's first line
    bool column;   // a kz = N/2 tile
};

// Staged tile of one array: the even rows y = 2p as [p][TL], then the odd rows y = 2p + 1 as
// [p][TL + 2 OX] from element OX on. OX = 1 in FP32, where the odd rows' box starts one element
// before kz0 (its start must be a multiple of 16 bytes), 0 in FP64.
template <typename C> __host__ __device__ constexpr int y_ox() { return sizeof(C) == 8 ? 1 : 0; }
template <typename C>
__device__ __forceinline__ int y_slot(int n, int t, int TL, int M) {
    constexpr int OX = y_ox<C>();
    return (n & 1) ? TL * M + (n >> 1) * (TL + 2 * OX) + OX + t : (n >> 1) * TL + t;
}
// A thread's elements n = j + r P (P = L/16, even) all have the parity of j, so their slots
// are s0 + r sp: y_slot(j) + r (P/2) (row pitch).
template <typename C, int L>
__device__ __forceinline__ void y_slots(int j, int t, int TL, int M, int &s0, int &sp) {
    constexpr int P = RegPlan<L>::P, OX = y_ox<C>();
    s0 = y_slot<C>(j, t, TL, M);
    sp = (P / 2) * ((j & 1) ? TL + 2 * OX : TL);
}
// elements of one staged array tile: (2 TL + 2 OX) rows of N/2
template <typename C> __device__ __forceinline__ int y_stage_elems(int TL, int N) { return (TL + y_ox<C>()) * N; }

// Thread 0: the tensor copies of plane tile y of array `arr`, realization z, into st (128-byte
// aligned), completing on bar: the even rows, then the odd rows, each in boxes of
// YB = min(N/2, 256) pairs (a box edge is at most 256).
template <typename C, int L>
__device__ __forceinline__ void y_issue(C *st, const CUtensorMap *me, const CUtensorMap *mo, const YTile &y,
                                        const Geo &g, int arr, int z, uint64_t *bar) {
    constexpr int OX = y_ox<C>(), W = (int)(sizeof(C) / 8), M = L / 2, YB = M < 256 ? M : 256;
    const int TL = 1 << g.tlx_shift, q0 = y.x0 * M;
    C *odd = st + TL * M;
#pragma unroll
    for (int p0 = 0; p0 < M; p0 += YB) {
        tma_load_4d(st + p0 * TL, me, y.kz0 * W, q0 + p0, arr, z, bar);
        tma_load_4d(odd + p0 * (TL + 2 * OX), mo, (g.H + y.kz0) * W - OX, q0 + p0, arr, z, bar);
    }
}

// Each thread of a column tile copies its own elements of array src (cp.async) into the
// staged layout.
template <typename C, int L>
__device__ __forceinline__ void y_column_async(C *st, const C *src, const YTile &y, int t, int j, const Geo &g) {
    using RP = RegPlan<L>;
    int s0, sp;
    y_slots<C, L>(j, t, 1 << g.tlx_shift, g.M, s0, sp);
    const C *p = src + (long long)y.x * g.N * g.H + y.kz + (long long)j * g.H;
#pragma unroll
    for (int r = 0; r < 16; ++r) cp_async_elem(st + s0 + r * sp, p + (long long)r * RP::P * g.H);
}

// Y forward pass, FP32 tensor-map form, persistent and pipelined: one wave of blocks (two per
// SM, one for 1024-point lines; three, at 80 registers, measured slower) walks the items
// w = (tile, array, realization),
// tile fastest. While an item's tile is transformed, thread 0 has already issued the tensor
// copies of the block's next item into the other of two staging buffers (the current one
// doubles as the exchange buffer), so each tile's load overlaps the previous tile's transform.
// Column tiles (kz = N/2) are staged by the block's own cp.async copies when their turn comes.
// Same transform per line: the bits of kr_fft_y.
template <typename T, int L>
__global__ void __launch_bounds__(xy_threads<L>(), xy_blocks<L>(2)) kr_fft_y_pipe(Geo g, const __grid_constant__ ArrList arrs,
                                                       const cplx<T> *__restrict__ tw, const DevBG *bg,
                                                       const __grid_constant__ YTma ym, int nj, int R) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t bar[2];   // completion of the tensor copies into staging buffer 0 / 1
    const int sh = g.tlx_shift, TL = 1 << sh;
    const int t = threadIdx.x & (TL - 1), j = threadIdx.x >> sh;
    const unsigned per = (unsigned)(g.M >> sh), nplane = (unsigned)g.N * per, nbx = nplane + (unsigned)(g.N >> sh);
    const unsigned total = nbx * (unsigned)nj * (unsigned)R;
    const int se = y_stage_elems<C>(TL, g.N);
    C *S0 = reinterpret_cast<C *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
    auto ix = [&](int n) { return n * TL + t; };
    // thread 0: the two tensor copies of plane-tile item w into st, on br
    auto issue = [&](unsigned w, C *st, uint64_t *br) {
        const unsigned b = w % nbx, rest = w / nbx;
        const int jy = (int)(rest % (unsigned)nj), z = (int)(rest / (unsigned)nj);
        const bool first = jy < ym.na;
        YTile y;
        y.x0 = (int)(b / per);
        y.kz0 = (int)(b - (unsigned)y.x0 * per) << sh;
        fence_proxy_async();   // the previous use of st (staging reads, exchange) comes first
        mbar_arrive_expect_tx(br, (unsigned)(se * sizeof(C)) + planted(bg + z, 3));
        y_issue<C, L>(st, first ? &ym.ae : &ym.be, first ? &ym.ao : &ym.bo, y, g, first ? jy : jy - ym.na, z, br);
    };
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    // a failed stage: no work (one thread reads the error words; the barrier also makes the
    // initialised mbarriers visible to every thread)
    bool failed = false;
    if (threadIdx.x == 0)
        for (int z = 0; z < R; ++z) failed |= bg[z].err != 0;
    if (__syncthreads_or(failed)) return;
    unsigned w = blockIdx.x;
    if (threadIdx.x == 0 && w < total && w % nbx < nplane) issue(w, S0, &bar[0]);
    unsigned phase = 0;   // bit i: parity of the next completion of bar[i]
    int cur = 0;
    for (; w < total; w += gridDim.x, cur ^= 1) {
        const unsigned wn = w + gridDim.x;
        C *Sc = S0 + cur * se;
        const bool next_tma = wn < total && wn % nbx < nplane;
        if (threadIdx.x == 0 && next_tma) issue(wn, S0 + (cur ^ 1) * se, &bar[cur ^ 1]);
        const unsigned b = w % nbx, rest = w / nbx;
        const int jy = (int)(rest % (unsigned)nj), z = (int)(rest / (unsigned)nj);
        C *a = reinterpret_cast<C *>(arrs.p[jy]) + (long long)z * arrs.rs[jy];
        YTile y;
        if (b < nplane) {
            y.x0 = (int)(b / per);
            y.x = y.x0;
            y.kz = ((int)(b - (unsigned)y.x0 * per) << sh) + t;
            y.column = false;
        } else {
            y.x = ((int)(b - nplane) << sh) + t;
            y.kz = g.M;
            y.column = true;
        }
        if (y.column) {
            y_column_async<C, L>(Sc, a, y, t, j, g);
            cp_async_commit();
            cp_async_wait_all();   // own elements only
        } else {
            const bool ok = mbar_wait_bounded(&bar[cur], (phase >> cur) & 1u, bg[z].wait_ns);
            if (__syncthreads_or(!ok)) {
                // report the timeout, count the test hook's planted bytes, wait once more
                // (bounded) for every copy still in flight (this tile's and the next one's)
                // and leave; PSC_ERR_DEVICE when they never land
                int *err = &const_cast<DevBG *>(bg)[z].err;
                const int zn = next_tma ? (int)(wn / nbx / (unsigned)nj) : 0;
                if (threadIdx.x == 0) {
                    report_err(err, PSC_ERR_TIMEOUT);
                    if (planted(bg + z, 3)) mbar_complete_tx(&bar[cur], planted(bg + z, 3));
                    if (next_tma && planted(bg + zn, 3)) mbar_complete_tx(&bar[cur ^ 1], planted(bg + zn, 3));
                }
                bool landed = mbar_wait_bounded(&bar[cur], (phase >> cur) & 1u, bg[z].wait_ns);
                if (next_tma)
                    landed = mbar_wait_bounded(&bar[cur ^ 1], (phase >> (cur ^ 1)) & 1u, bg[z].wait_ns) && landed;
                if (__syncthreads_or(!landed) && threadIdx.x == 0) report_err(err, PSC_ERR_DEVICE);
                return;
            }
            phase ^= 1u << cur;
        }
        int s0, sp;
        y_slots<C, L>(j, t, TL, g.M, s0, sp);
        C v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = Sc[s0 + r * sp];
        __syncthreads();   // every thread holds its elements before the transform reuses the tile
        fft_reg<C, L, -1>(v, Sc, ix, j, tw, g.N / L);
        const long long base = (long long)y.x * g.N * g.H + y.kz;
#pragma unroll
        for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
            for (int r = 0; r < RP::RL; ++r) a[base + (long long)RP::out(j, q, r) * g.H] = v[q * RP::RL + r];
        __syncthreads();   // the exchange reads are done before the buffer is refilled
    }
}


// Y inverse pass with GWs, FP32 tensor-map form, persistent and pipelined: one wave of blocks
// walks the items w = (tile, field, realization), tile fastest, with the Y forward pass's tiles
// (row-pair boxes; the kz = N/2 column by the threads' own cp.async copies). An item's TA and TB
// tiles sit in one staging buffer each; the block transforms TB -> TB first, then
// d/dy TA -> TC and TA -> TA, through a separate exchange buffer. As soon as a buffer's last
// transform has read it, thread 0 refills it with the block's next item (TB after the first
// transform, TA after the third), so each tile's load overlaps the transforms that follow.
// Same transform per line: the bits of kr_ifft_y.
template <typename T, int L>
__global__ void __launch_bounds__(xy_threads<L>(), xy_blocks<L>(2)) kr_ifft_y_pipe(Geo g, cplx<T> *__restrict__ TA,
                                                       cplx<T> *__restrict__ TB, cplx<T> *__restrict__ TC,
                                                       const DevBG *bg, const cplx<T> *__restrict__ tw,
                                                       const __grid_constant__ YTma ym, int R) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t barA, barB;   // completion of the tensor copies into the TA / TB buffer
    const int sh = g.tlx_shift, TL = 1 << sh;
    const int t = threadIdx.x & (TL - 1), j = threadIdx.x >> sh;
    const unsigned per = (unsigned)(g.M >> sh), nplane = (unsigned)g.N * per, nbx = nplane + (unsigned)(g.N >> sh);
    const unsigned nf = (unsigned)g.nf, total = nbx * nf * (unsigned)R;
    const int se = y_stage_elems<C>(TL, g.N);
    C *stA = reinterpret_cast<C *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
    C *stB = stA + se, *xb = stB + se;
    auto ix = [&](int n) { return n * TL + t; };
    unsigned plantA = 0, plantB = 0;   // thread 0: the test hook's bytes in the pending copies
    // thread 0: the tensor copies of plane-tile item w's array (maps me, mo) into st, on br
    auto issue = [&](unsigned w, C *st, const CUtensorMap *me, const CUtensorMap *mo, uint64_t *br) -> unsigned {
        const unsigned b = w % nbx, rest = w / nbx;
        const int jy = (int)(rest % nf), z = (int)(rest / nf);
        YTile y;
        y.x0 = (int)(b / per);
        y.kz0 = (int)(b - (unsigned)y.x0 * per) << sh;
        const unsigned plant = planted(bg + z, 1);
        fence_proxy_async();   // the previous reads of st come first
        mbar_arrive_expect_tx(br, (unsigned)(se * sizeof(C)) + plant);
        y_issue<C, L>(st, me, mo, y, g, jy, z, br);
        return plant;
    };
    if (threadIdx.x == 0) {
        mbar_init(&barA, 1);
        mbar_init(&barB, 1);
        mbar_fence_init();
    }
    // a failed stage: no work (one thread reads the error words; the barrier also makes the
    // initialised mbarriers visible to every thread)
    bool failed = false;
    if (threadIdx.x == 0)
        for (int z = 0; z < R; ++z) failed |= bg[z].err != 0;
    if (__syncthreads_or(failed)) return;
    unsigned w = blockIdx.x;
    bool pendA = false, pendB = false;   // copies in flight into the TA / TB buffer (every thread)
    unsigned pa = 0, pb = 0;             // parities of the next completions of barA / barB
    if (w < total && w % nbx < nplane) {
        if (threadIdx.x == 0) {
            plantB = issue(w, stB, &ym.be, &ym.bo, &barB);
            plantA = issue(w, stA, &ym.ae, &ym.ao, &barA);
        }
        pendA = pendB = true;
    }
    // every thread waits (bounded) for the copies into one buffer. On a timeout the block
    // reports it, counts the test hook's planted bytes, waits once more (bounded) for every copy
    // still in flight and returns false (PSC_ERR_DEVICE when they never land).
    auto wait = [&](uint64_t *br, unsigned par, int z) -> bool {
        if (!__syncthreads_or(!mbar_wait_bounded(br, par, bg[z].wait_ns))) return true;
        int *err = &const_cast<DevBG *>(bg)[z].err;
        if (threadIdx.x == 0) {
            report_err(err, PSC_ERR_TIMEOUT);
            if (pendA && plantA) mbar_complete_tx(&barA, plantA);
            if (pendB && plantB) mbar_complete_tx(&barB, plantB);
        }
        bool landed = true;
        if (pendA) landed = mbar_wait_bounded(&barA, pa, bg[z].wait_ns) && landed;
        if (pendB) landed = mbar_wait_bounded(&barB, pb, bg[z].wait_ns) && landed;
        if (__syncthreads_or(!landed) && threadIdx.x == 0) report_err(err, PSC_ERR_DEVICE);
        return false;
    };
    for (; w < total; w += gridDim.x) {
        const unsigned wn = w + gridDim.x;
        const bool next_tma = wn < total && wn % nbx < nplane;
        const unsigned b = w % nbx, rest = w / nbx;
        const int jy = (int)(rest % nf), z = (int)(rest / nf);
        YTile y;
        if (b < nplane) {
            y.x0 = (int)(b / per);
            y.x = y.x0;
            y.kz = ((int)(b - (unsigned)y.x0 * per) << sh) + t;
            y.column = false;
        } else {
            y.x = ((int)(b - nplane) << sh) + t;
            y.kz = g.M;
            y.column = true;
        }
        const long long off = (long long)jy * g.modes + (long long)z * g.fstride;
        if (y.column) {
            // nothing is in flight into the buffers (this item issued no copies)
            y_column_async<C, L>(stA, TA + off, y, t, j, g);
            y_column_async<C, L>(stB, TB + off, y, t, j, g);
            cp_async_commit();
            cp_async_wait_all();   // own elements only
            __syncthreads();       // the previous item's last exchange reads are done
        }
        const T kIR = (T)bg[z].kIR;
        int s0, sp;
        y_slots<C, L>(j, t, TL, g.M, s0, sp);
        const long long base = off + (long long)y.x * g.N * g.H + y.kz;
#pragma unroll 1
        for (int k = 0; k < 3; ++k) {
            // k = 0: TB -> TB; 1: d/dy TA -> TC; 2: TA -> TA
            if (k) __syncthreads();   // the exchange buffer is free again (k = 0: the wait's barrier)
            if (!y.column && k < 2) {
                if (!wait(k == 0 ? &barB : &barA, k == 0 ? pb : pa, z)) return;
                if (k == 0) {
                    pb ^= 1u;
                    pendB = false;
                } else {
                    pa ^= 1u;
                    pendA = false;
                }
            }
            const C *st = k == 0 ? stB : stA;
            C v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int n = j + r * RP::P;
                C e = st[s0 + r * sp];
                if (k == 1) {
                    const T ky = (n == (g.N >> 1)) ? T(0) : kIR * (T)pcoord(n, g.N);
                    e = mk<T>(-ky * e.y, ky * e.x);
                }
                v[r] = e;
            }
            fft_reg<C, L, +1>(v, xb, ix, j, tw, g.N / L);
            C *dst = k == 0 ? TB : (k == 1 ? TC : TA);
#pragma unroll
            for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                for (int r = 0; r < RP::RL; ++r) dst[base + (long long)RP::out(j, q, r) * g.H] = v[q * RP::RL + r];
            // every thread has passed the transform's barriers, so every read of the buffer
            // this transform used is done: refill it with the next item's tile
            if (next_tma && k != 1) {
                if (threadIdx.x == 0) {
                    if (k == 0) plantB = issue(wn, stB, &ym.be, &ym.bo, &barB);
                    else plantA = issue(wn, stA, &ym.ae, &ym.ao, &barA);
                }
                if (k == 0) pendB = true;
                else pendA = true;
            }
        }
    }
}


// ------------------------------------------------------------------ X forward + kick epilogue
template <typename T, int L, bool GW, class VB>
__device__ __forceinline__ void kr_fft_x_final_body(const VB &vb, Geo g, const cplx<T> *__restrict__ QV, const cplx<T> *__restrict__ QS, const cplx<T> *__restrict__ fk, cplx<T> *__restrict__ pk, cplx<T> *__restrict__ uk, cplx<T> *__restrict__ puk, double *__restrict__ partKG, const DevBG *__restrict__ bg, const cplx<T> *__restrict__ tw, cplx<T> *__restrict__ tape_f, cplx<T> *__restrict__ tape_p, cplx<T> *__restrict__ tape_vp, cplx<T> *__restrict__ tape_pu, cplx<T> *__restrict__ tape_fu, cplx<T> *__restrict__ fcache, cplx<T> *__restrict__ ucache, const XTma *tma) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);
    __shared__ uint64_t qbar, xbar;   // completion of the input tile's / operand tiles' tensor copies (TMA)
    {
        const long long rf = (long long)vb.z() * g.fstride, rg = (long long)vb.z() * g.gstride;
        QV += rf;
        fk += rf;
        pk += rf;
        if (fcache) fcache += rf;
        if (GW) {
            if (ucache) ucache += rg;
            QS += rg;
            uk += rg;
            puk += rg;
        }
        partKG += (size_t)vb.z() * g.pkg_stride;
        bg += vb.z();
    }
    const int sh = g.tlx_shift, TL = 1 << sh, N = g.N, H = g.H, M = g.M;
    const int t = threadIdx.x & (TL - 1), j = threadIdx.x >> sh;
    const int line = vb.x() * TL + t;
    const bool valid = line < g.lines_x;
    const int job = vb.y();
    const bool field = job < g.nf;
    const long long off = (long long)(field ? job : job - g.nf) * g.modes;
    const C *src = (field ? QV : QS) + off;
    const long long stride = g.lines_x;
    const long long base = off + line;
    auto ix = [&](int n) { return n * TL + t; };
    // Prefetch the kick operands (f_k, pi_half or u_k, pi_u_half) of this tile into shared
    // memory, overlapping their latency with the FFT: with tensor maps (tma), two tiled copies
    // by the tensor memory accelerator issued by one thread, landing on an mbarrier (the tiles
    // 128-byte aligned: the launch adds 128 bytes of shared memory for it); otherwise each
    // thread copies its own elements with cp.async.
    const bool use_tma = tma != nullptr;
    // with tensor maps the three tiles (the transform's input, then the two operands) sit
    // 128-byte aligned from the start of the buffer: the input tile doubles as the exchange
    // buffer once every thread holds its elements
    if (use_tma) sm = reinterpret_cast<C *>((reinterpret_cast<uintptr_t>(sm) + 127) & ~(uintptr_t)127);
    C *opA = sm + TL * L;
    C *opB = opA + TL * L;
    const C *gA = field ? fk : uk, *gB = field ? pk : puk;
    C v[16];
    if (use_tma) {
        // a failed stage: no further waits (one thread reads the error word, so that the block
        // decides as one while another block may be writing it)
        if (__syncthreads_or(threadIdx.x == 0 && bg->err != 0)) return;
        if (threadIdx.x == 0) {
            mbar_init(&qbar, 1);
            mbar_init(&xbar, 1);
            mbar_fence_init();
            const int w8 = (int)(sizeof(C) / 8), arr = field ? job : job - g.nf, c0 = (int)(vb.x() * TL) * w8;
            mbar_arrive_expect_tx(&qbar, (unsigned)(TL * L * sizeof(C)) + planted(bg, 4));
            x_tile_tma<L>(sm, field ? &tma->qv : &tma->qs, c0, TL, arr, (int)vb.z(), &qbar);
            mbar_arrive_expect_tx(&xbar, 2u * (unsigned)(TL * L * sizeof(C)));
            const CUtensorMap *ma = field ? &tma->fk : &tma->uk, *mb = field ? &tma->pk : &tma->puk;
            x_tile_tma<L>(opA, ma, c0, TL, arr, (int)vb.z(), &xbar);
            x_tile_tma<L>(opB, mb, c0, TL, arr, (int)vb.z(), &xbar);
        }
        __syncthreads();   // the mbarriers are initialised before any thread waits on them
        const bool ok = mbar_wait_bounded(&qbar, 0, bg->wait_ns);
        if (__syncthreads_or(!ok)) {
            // the input tile did not land in time: report it, wait once more (bounded) for all
            // three tiles still in flight so that none can write into shared memory after the
            // block has left, and leave (PSC_ERR_DEVICE when they never land)
            int *err = &const_cast<DevBG *>(bg)->err;
            if (threadIdx.x == 0) {
                report_err(err, PSC_ERR_TIMEOUT);
                if (planted(bg, 4)) mbar_complete_tx(&qbar, planted(bg, 4));   // the test hook's bytes
            }
            const bool landed = mbar_wait_bounded(&qbar, 0, bg->wait_ns) && mbar_wait_bounded(&xbar, 0, bg->wait_ns);
            if (__syncthreads_or(!landed) && threadIdx.x == 0) report_err(err, PSC_ERR_DEVICE);
            return;
        }
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[ix(j + r * RP::P)];
        __syncthreads();   // every thread holds its elements before the transform reuses the tile
    } else {
        if (valid) {
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int n = RP::out(j, r / RP::RL, r % RP::RL);
                const long long a = base + (long long)n * stride;
                cp_async_elem(opA + ix(n), gA + a);
                cp_async_elem(opB + ix(n), gB + a);
            }
        }
        cp_async_commit();
#pragma unroll
        for (int r = 0; r < 16; ++r)
            v[r] = valid ? src[(long long)(j + r * RP::P) * stride + line] : mk<T>(0, 0);
    }
    fft_reg<C, L, -1>(v, sm, ix, j, tw, N / L);
    if (use_tma) {
        // every thread waits for the tiles (bounded). If they did not land in time: report the
        // timeout, wait once more for the copies in flight (bounded) so that the block never
        // leaves while one can still write into its shared memory, and leave; if they never
        // land, PSC_ERR_DEVICE (the context can no longer be trusted)
        const bool ok = mbar_wait_bounded(&xbar, 0, bg->wait_ns);
        if (__syncthreads_or(!ok)) {
            int *err = &const_cast<DevBG *>(bg)->err;
            if (threadIdx.x == 0) report_err(err, PSC_ERR_TIMEOUT);
            const bool landed = mbar_wait_bounded(&xbar, 0, bg->wait_ns);
            if (__syncthreads_or(!landed) && threadIdx.x == 0) report_err(err, PSC_ERR_DEVICE);
            return;
        }
    } else {
        cp_async_wait_all();
    }

    const T norm1 = (T)bg->norm1, norm2 = (T)bg->norm2, kIR2 = (T)bg->kIR2;
    const T c_close = (T)bg->c_close, c_open = (T)bg->c_open;
    // a synchronising kick (the last of a step call, or an evaluation) keeps its force
    const bool keep = bg->c_open == 0.0;
    const int y = line / H, kz = line - y * H;
    const int py = pcoord(y, N);
    if (field) {
        T accK = T(0), accG = T(0);   // per-thread partials (16 modes), FP64 across threads
        // the homogeneous mode (n = 0 of line 0) is kicked by the background kernel in FP64:
        // here its V'_k is handed over and it stays out of the partials
        const bool z0 = line == 0 && j == 0 && bg->zero64;
        if (valid) {
            const bool mask = g.mask != 0;
            const T hub = (T)bg->hub, apow = (T)bg->apow, a3 = (T)bg->a3;
            const T dfdp = (T)bg->DFDP, eps = (T)bg->eps;
            const T wgt = (kz == 0 || kz == M) ? T(1) : T(2);
#pragma unroll
            for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                for (int r = 0; r < RP::RL; ++r) {
                    const int n = RP::out(j, q, r);
                    const int px = pcoord(n, N);
                    const T k2 = (T)(px * px + py * py + kz * kz);
                    const long long a = base + (long long)n * stride;
                    const C f = opA[ix(n)], p = opB[ix(n)], qv = v[q * RP::RL + r];
                    if (q == 0 && r == 0 && z0) {   // n = 0 (out(0, 0, 0))
                        DevBG *bw = const_cast<DevBG *>(bg);
                        bw->z0q[job][0] = (double)qv.x;
                        bw->z0q[job][1] = (double)qv.y;
                        bw->z0pending = 1;
                        if (tape_p) {   // the tape as the kick below would write it (k = 0: no -k^2 f term)
                            tape_f[a] = f;
                            tape_p[a] = mk<T>(p.x + c_close * (-norm2 * qv.x), p.y + c_close * (-norm2 * qv.y));
                            tape_vp[a] = qv;
                        }
                        continue;
                    }
                    // force (evolution.cpp:1124-1125)
                    const T fl = -norm1 * kIR2 * k2;
                    const C F = mk<T>(fl * f.x - norm2 * qv.x, fl * f.y - norm2 * qv.y);
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
                        accK += wgt * (pf.x * pf.x + pf.y * pf.y);
                        accG += wgt * k2 * (f.x * f.x + f.y * f.y);
                    }
                    pk[a] = mk<T>(pf.x + c_open * F.x, pf.y + c_open * F.y);
                    if (keep && fcache) fcache[a] = F;
                    if (tape_p) {   // adjoint tape: the synchronised stage-point state
                        tape_f[a] = f;
                        tape_p[a] = pf;
                        tape_vp[a] = qv;
                    }
                }
        }
        T vals[2] = {accK, accG};
        block_reduce_store_t<T, 2>(vals, partKG + (size_t)(2 * job) * vb.gx(), vb.gx(), vb.x());
    } else if (GW && valid) {
        const T c_drift = (T)bg->c_drift;
#pragma unroll
        for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
            for (int r = 0; r < RP::RL; ++r) {
                const int n = RP::out(j, q, r);
                const int px = pcoord(n, N);
                const T k2 = (T)(px * px + py * py + kz * kz);
                const long long a = base + (long long)n * stride;
                C u = opA[ix(n)];
                const C w = opB[ix(n)], qv = v[q * RP::RL + r];
                // drift of u_ij deferred from the stage prologue (evolution.cpp:655-662)
                u.x += c_drift * w.x;
                u.y += c_drift * w.y;
                // a^(1+alpha) (lapl u + 2 sum d_i f d_j f)  (evolution.cpp:586-598)
                const T l = -kIR2 * k2;
                const C fu = mk<T>(l * u.x + qv.x, l * u.y + qv.y);
                const C F = mk<T>(norm1 * fu.x, norm1 * fu.y);
                const C wf = mk<T>(w.x + c_close * F.x, w.y + c_close * F.y);
                uk[a] = u;
                puk[a] = mk<T>(wf.x + c_open * F.x, wf.y + c_open * F.y);
                if (keep && ucache) ucache[a] = F;
                if (tape_pu) {   // adjoint tape: synchronised pi_u and the force without a^(1+alpha)
                    tape_pu[a] = wf;
                    tape_fu[a] = fu;
                }
            }
    }
}

template <typename T, int L, bool GW>
__global__ void __launch_bounds__(xy_threads<L>(), xy_blocks<L>(2)) kr_fft_x_final(Geo g, const cplx<T> *__restrict__ QV,
                                                      const cplx<T> *__restrict__ QS, const cplx<T> *__restrict__ fk,
                                                      cplx<T> *__restrict__ pk, cplx<T> *__restrict__ uk,
                                                      cplx<T> *__restrict__ puk, double *__restrict__ partKG,
                                                      const DevBG *__restrict__ bg, const cplx<T> *__restrict__ tw,
                                                      cplx<T> *__restrict__ tape_f = nullptr,
                                                      cplx<T> *__restrict__ tape_p = nullptr,
                                                      cplx<T> *__restrict__ tape_vp = nullptr,
                                                      cplx<T> *__restrict__ tape_pu = nullptr,
                                                      cplx<T> *__restrict__ tape_fu = nullptr,
                                                      cplx<T> *__restrict__ fcache = nullptr,
                                                      cplx<T> *__restrict__ ucache = nullptr,
                                                      const __grid_constant__ XTma tma = XTma{}) {
    kr_fft_x_final_body<T, L, GW, HwBlock>(vblock_hw(), g, QV, QS, fk, pk, uk, puk, partKG, bg, tw, tape_f, tape_p, tape_vp, tape_pu, tape_fu, fcache, ucache, tma.on ? &tma : nullptr);
}

// ------------------------------------------------------------------ fused Z pass
// Shared memory: nslot real-line slots of TL lines x LS complex (a complex
// element holds the real sites 2m, 2m+1), index t*LS + m + m/16 (the pad keeps
// the radix-16 exchange free of bank conflicts).
template <int L>
struct ZIdx {
    static constexpr int LS = L + L / 16 + 1;   // one spare entry holds X[M] while staging
    int base;
    __device__ __forceinline__ int operator()(int n) const { return base + n + (n >> 4); }
};

// Half-length packing partners by warp shuffle. The P = M/16 lanes of a z line are
// consecutive lanes of one warp. Input order (thread j holds x[j + rP], r < 16): the
// partner of k = j + rP is M - k = (15 - r) P + (P - j), held by lane P - j in its
// register 15 - r (lane 0: its own register 16 - r, and x[M] for r = 0).
template <typename C>
__device__ __forceinline__ C shfl_c(C a, int src, int width) {
    C r;
    r.x = __shfl_sync(0xffffffffu, a.x, src, width);
    r.y = __shfl_sync(0xffffffffu, a.y, src, width);
    return r;
}

template <typename C, int M>
__device__ __forceinline__ void partners_in(const C (&v)[16], C xM, int j, C (&y)[16]) {
    constexpr int P = M / 16;
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const C s = shfl_c(v[15 - r], (P - j) & (P - 1), P);
        y[r] = (j == 0) ? (r == 0 ? xM : v[(16 - r) & 15]) : s;
    }
}

// Output order of the forward transform (thread j holds Z[out(j, q, r)] in v[q RL + r]):
// the partner of k = (j NBL + q) + r NSL is M - k, held by lane P - j (q = 0) or
// P - 1 - j (q > 0) in register ((NBL - q) mod NBL) RL + RL - 1 - r; lane 0 with q = 0
// holds it itself (register RL - r, and Z[0] for r = 0). Returns conj Z[M - k].
template <typename C, int M>
__device__ __forceinline__ C partner_out(const C (&v)[16], int j, int q, int r) {
    using RP = RegPlan<M>;
    constexpr int P = RP::P, RL = RP::RL, NBL = RP::NBL;
    const C a = v[(q == 0 ? 0 : NBL - q) * RL + (RL - 1 - r)];
    const C s = shfl_c(a, q == 0 ? ((P - j) & (P - 1)) : (P - 1 - j), P);
    C z = s;
    if (q == 0 && j == 0) z = (r == 0) ? v[0] : v[(RL - r) % RL];
    return cconj(z);
}

// Z pass without GWs (one or two fields, one input line per field). Persistent: a block
// walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ...; while one tile is transformed,
// the input lines of the next are copied into a staging area by cp.async (no register
// round trip), so the HBM reads overlap the FFT work. Shared memory: nf work slots, then
// nf staging slots, TL lines x LS complex each (a complex element holds the real sites
// 2m, 2m+1). The GW form is kr_zpass_gw. USER = false: the built-in models (nf <= 2);
// USER = true: any model, up to kMaxFields fields and kMaxTerms potential terms.
template <typename T, int L, bool USER, class VB>
__device__ __forceinline__ void kr_zpass_body(const VB &vb, Geo g, const cplx<T> *__restrict__ TA, cplx<T> *__restrict__ QV, double *__restrict__ partV, const DevBG *__restrict__ bg, const cplx<T> *__restrict__ tw, T *__restrict__ tape_fx) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    constexpr int M = L, P = RP::P, LS = ZIdx<L>::LS;
    constexpr int NF = USER ? kMaxFields : 2, NT = USER ? kMaxTerms : 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *slots = reinterpret_cast<C *>(smem_raw);
    {
        const long long rf = (long long)vb.z() * g.fstride;
        TA += rf;
        QV += rf;
        partV += (size_t)vb.z() * g.pv_stride;
        bg += vb.z();
    }
    const int sh = g.tlz_shift, TL = 1 << sh, H = g.H, N = g.N;
    const int nf = g.nf;
    const int j = threadIdx.x % P;
    const int t = (threadIdx.x / P) & (TL - 1);
    const int grp = threadIdx.x / (P * TL);   // the field this thread transforms
    const size_t slot_elems = (size_t)TL * LS;
    C *stage = slots + (size_t)nf * slot_elems;
    const T inv_n3 = (T)bg->inv_n3;
    const C *src0 = TA + (long long)grp * g.modes;
    const ZIdx<L> ix{(int)(grp * slot_elems + t * LS)};
    const int ntiles = (g.lines_z + TL - 1) >> sh;
    // stage X[0..M] of this thread's line of tile `tile` (M+1 entries fit: the pad leaves room)
    auto prefetch = [&](int tile) {
        const int ln = tile * TL + t;
        if (tile < ntiles && ln < g.lines_z) {
            const C *src = src0 + (long long)ln * H;
#pragma unroll
            for (int r = 0; r < 16; ++r) cp_async_elem(stage + ix(j + r * P), src + j + r * P);
            if (j == 0) cp_async_elem(stage + ix(M), src + M);
        }
        cp_async_commit();
    };
    ModelG<T> mdl;
    mdl.kind = g.model;
    mdl.gsq = (T)g.gsq;
    // <V> partial sums: up to 16 tiles' sites in the field precision, then folded into
    // FP64 (a persistent block walks thousands of tiles at N = 1024; a fold per tile
    // would put a conversion and an add per thread and tile on the narrow FP64 pipe)
    T pot_t[NT] = {};
    double pot_d[NT] = {};
    int nfold = 0;
    // the sums run over V(site) - vref (model_potential_shifted), vref the potential terms of
    // the homogeneous fields (the FP64 shadow of the zero modes / N^3), a value of the state
    // alone; vref is added back once per site summed (every tile gives a thread the same
    // number of sites: the line count is a multiple of the tile's)
    T vref[NT];
    homogeneous_potential<T, T, USER>(mdl, bg, vref);
    prefetch(vb.x());
    for (int tile = vb.x(); tile < ntiles; tile += vb.gx()) {
        const int line = tile * TL + t;
        const bool valid = line < g.lines_z;
        // 1. complex-to-real along z of field grp: pack X[k], X[M-k] into the M-point
        //    transform Z[k] = (X[k] + conj X[M-k]) + i w^k (X[k] - conj X[M-k]),
        //    w = e^{+2 pi i/N}; Im X[0] and Im X[M] are ignored, as a c2r does. Own
        //    elements from the staging area, partners by warp shuffle.
        C v[16], yv[16];
        {
            cp_async_wait_all();
            __syncthreads();
            C xM = mk<T>(0, 0);
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = stage[ix(j + r * P)];
            if (j == 0) xM = stage[ix(M)];
            partners_in<C, M>(v, xM, j, yv);
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int k = j + r * P;
                C x = mk<T>(0, 0), y = mk<T>(0, 0);
                if (valid) {
                    x = v[r];
                    y = yv[r];
                }
                y.y = -y.y;
                if (k == 0) { x.y = T(0); y.y = T(0); }
                const C s = cadd(x, y), d = csub(x, y);
                C w = __ldg(&tw[k]);
                w.y = -w.y;
                const C td = cmul(w, d);
                v[r] = mk<T>(s.x - td.y, s.y + td.x);
            }
            __syncthreads();   // every thread has read the staging area
            prefetch(tile + vb.gx());
            fft_reg<C, L, +1, true>(v, slots, ix, j, tw, N / L);
            __syncthreads();
#pragma unroll
            for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                for (int r = 0; r < RP::RL; ++r) slots[ix(RP::out(j, q, r))] = cscale_k<true>(v[q * RP::RL + r], inv_n3);
        }
        __syncthreads();

        // 2. pointwise epilogue: V'(f), <V>
        for (int idx = threadIdx.x; idx < TL * M; idx += blockDim.x) {
            const int tt = idx / M, m = idx - tt * M;
            const long long ln = (long long)tile * TL + tt;
            if (ln >= g.lines_z) continue;
            const int e = tt * LS + m + (m >> 4);
            C in[NF];
#pragma unroll
            for (int o = 0; o < NF; ++o)
                if (o < nf) in[o] = slots[o * slot_elems + e];
            if (tape_fx) {   // adjoint tape: the real fields (sites 2m, 2m+1 of the line)
#pragma unroll
                for (int fl = 0; fl < NF; ++fl)
                    if (fl < nf) reinterpret_cast<C *>(tape_fx + fl * g.sites + ln * N)[m] = in[fl];
            }
            C out[NF];
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                T f[NF], vp[NF];
#pragma unroll
                for (int fl = 0; fl < NF; ++fl) f[fl] = (fl < nf) ? (half ? in[fl].y : in[fl].x) : T(0);
                model_dvdf<T, T, USER>(mdl, f, vp, nf);
                model_potential_shifted<T, T, USER>(mdl, f, vref, pot_t);
#pragma unroll
                for (int fl = 0; fl < NF; ++fl)
                    if (fl < nf) { if (half) out[fl].y = vp[fl]; else out[fl].x = vp[fl]; }
            }
#pragma unroll
            for (int o = 0; o < NF; ++o)
                if (o < nf) slots[o * slot_elems + e] = out[o];
        }
        if ((++nfold & 15) == 0) {
#pragma unroll
            for (int i = 0; i < NT; ++i) {
                pot_d[i] += (double)pot_t[i];
                pot_t[i] = T(0);
            }
        }
        __syncthreads();

        // 3. real-to-complex along z of V'(f) of field grp; X[k] = (Z[k] + conj Z[M-k])/2
        //    + e^{-2 pi i k/N} (Z[k] - conj Z[M-k])/(2i), k = 0..M (Z[M] = Z[0])
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = slots[ix(j + r * P)];
        __syncthreads();   // all loads precede the first exchange write
        fft_reg<C, L, -1, true>(v, slots, ix, j, tw, N / L);
        {
            // the partners Z[M-k] by warp shuffle, X[k] straight out
            C *dst = QV + (long long)grp * g.modes + (long long)line * H;
#pragma unroll
            for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                for (int r = 0; r < RP::RL; ++r) {
                    const int k = RP::out(j, q, r);
                    const C zk = v[q * RP::RL + r];
                    const C zc = partner_out<C, M>(v, j, q, r);
                    const C ev = cscale_k<true>(cadd_k<true>(zk, zc), T(0.5));
                    const C dd = cscale_k<true>(csub_k<true>(zk, zc), T(0.5));
                    const C od = mk<T>(dd.y, -dd.x);
                    const C w = __ldg(&tw[k]);
                    if (valid) dst[k] = cadd(ev, cmul(w, od));
                }
            if (valid && j == 0) {   // X[M] = Re Z[0] - Im Z[0]
                const C z0 = v[0];
                dst[M] = mk<T>(z0.x - z0.y, T(0));
            }
        }
        __syncthreads();   // the transform's last exchange read precedes the next writes
    }
    cp_async_wait_all();
#pragma unroll
    const double nsite = (double)nfold * (2 * ((TL * M - 1 - (int)threadIdx.x) / (int)blockDim.x + 1));
    for (int i = 0; i < NT; ++i) pot_d[i] += (double)pot_t[i] + nsite * (double)vref[i];
    block_reduce_store_t<double, NT>(pot_d, partV, vb.gx(), vb.x());
}

template <typename T, int L, bool USER = false>
__global__ void __launch_bounds__(256, 2) kr_zpass(Geo g, const cplx<T> *__restrict__ TA, cplx<T> *__restrict__ QV,
                                                double *__restrict__ partV, const DevBG *__restrict__ bg,
                                                const cplx<T> *__restrict__ tw, T *__restrict__ tape_fx = nullptr) {
    kr_zpass_body<T, L, USER, HwBlock>(vblock_hw(), g, TA, QV, partV, bg, tw, tape_fx);
}

// GW form of the Z pass on full-length line transforms. The eight real lines of a z line
// (f, d/dx f, d/dy f, d/dz f of each field) travel as complex lines a + i b: pair 2 fld =
// f + i d/dz f (both from TA), pair 2 fld + 1 = d/dx f + i d/dy f (TB, TC). One N-point
// inverse transform of Z[n] = A[n] + i B[n] (n <= N/2), conj A[N-n] + i conj B[N-n]
// (n > N/2) gives both real lines, with no packing step: Im of the kz = 0 and N/2 entries
// is dropped first, as a c2r does. The products (V' of each field, then S_00, S_01, S_02,
// S_11, S_12, S_22) return as four pairs, each split after one N-point forward transform:
// P[k] = (Z[k] + conj Z[N-k]) / 2, Q[k] = (Z[k] - conj Z[N-k]) / 2i, k = 0..N/2, the
// partner Z[N-k] by warp shuffle (N <= 512) or through shared memory (N = 1024, where the
// 64 lanes of a line span two warps). Thread layout as kr_zpass (pair, line, j).
// STAGED (FP32): persistent, one wave of blocks walking the tiles; the input lines of the
// next tile are copied into a staging area by cp.async while the current one is
// transformed. Otherwise one tile per block, inputs read straight from global memory.
// Shared memory: four slots of TL lines x LS complex, then (STAGED) the staging area.
template <typename T, int L, bool STAGED, bool USER, class VB>
__device__ __forceinline__ void kr_zpass_gw_body(const VB &vb, Geo g, const cplx<T> *__restrict__ TA, const cplx<T> *__restrict__ TB, const cplx<T> *__restrict__ TC, cplx<T> *__restrict__ QV, cplx<T> *__restrict__ QS, double *__restrict__ partV, const DevBG *bg, const cplx<T> *__restrict__ tw, T *__restrict__ tape_fx) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    constexpr int P = RP::P, LS = ZIdx<L>::LS, HL = L / 2;
    constexpr int NF = USER ? kMaxFields : 2, NT = USER ? kMaxTerms : 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t zbar;   // completion of a tile's bulk copies
    C *slots = reinterpret_cast<C *>(smem_raw);
    {
        const long long rf = (long long)vb.z() * g.fstride, rg = (long long)vb.z() * g.gstride;
        TA += rf;
        TB += rf;
        TC += rf;
        QV += rf;
        QS += rg;
        partV += (size_t)vb.z() * g.pv_stride;
        bg += vb.z();
    }
    // a failed stage (an earlier wait ran out, or a non-finite background) leaves the rest
    // of the step call without work: no further waits. One thread reads the error word, so
    // that the block decides as one while another block may be writing it.
    if (__syncthreads_or(threadIdx.x == 0 && bg->err != 0)) return;
    const int TL = 1 << g.tlz_shift, H = g.H, N = g.N;
    const int nf = g.nf;
    const int pin = 2 * nf;                         // input pairs of a line
    // output pairs (V' of each field, then the six S_ab, two by two) and work slots: four
    // for up to two fields
    const int pout = USER ? (nf + 7) / 2 : 4;
    const int nslot = USER ? (pin > pout ? pin : pout) : 4;
    const int j = threadIdx.x % P;
    const int t = (threadIdx.x / P) & (TL - 1);
    const int grp = threadIdx.x / (P * TL);         // this thread's input pair in phase 1
    const size_t slot_elems = (size_t)TL * LS;
    // staging (STAGED): the next tile's input lines, [field][TA, TB, TC][line][hs]. The TL
    // lines of one array in a tile are contiguous in global memory; when that run is a
    // multiple of 16 bytes (TL even in FP32) it is one bulk copy by the tensor memory
    // accelerator (line stride hs = H), otherwise warps copy it by cp.async (hs = H + 1).
    C *stage = slots + nslot * slot_elems;
    const bool bulk = STAGED && ((size_t)TL * H * sizeof(C)) % 16 == 0;
    const int hs = bulk ? H : H + 1;
    const T inv_n3 = (T)bg->inv_n3;
    const T kIR = (T)bg->kIR;
    const T fj = (T)j;
    const int fld = grp >> 1, kind = grp & 1;
    const C *srcA = (kind ? TB : TA) + (long long)fld * g.modes;
    const C *srcB = TC + (long long)fld * g.modes;
    const C *stA = stage + ((size_t)(fld * 3 + (kind ? 1 : 0)) * TL + t) * hs;
    const C *stB = stage + ((size_t)(fld * 3 + 2) * TL + t) * hs;
    const int ntiles = (g.lines_z + TL - 1) / TL;
    if (bulk && threadIdx.x == 0) {
        mbar_init(&zbar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    // copy the input lines of tile `tl` into the staging area. Bulk: thread 0 issues one
    // copy per array (lines_z is a multiple of TL, so a tile never runs past the array).
    // Otherwise warp w takes the lines w, w + 8, ... of the nf x 3 x TL, its lanes
    // consecutive entries of each.
    auto prefetch = [&](int tl) {
        if (bulk) {
            if (threadIdx.x == 0 && tl < ntiles) {
                const unsigned run = (unsigned)((size_t)TL * H * sizeof(C));
                fence_proxy_async();   // the staging reads of the previous tile come first
                // + the test hook's planted bytes (0 in normal runs)
                mbar_arrive_expect_tx(&zbar, (unsigned)(nf * 3) * run + planted(bg, 2));
                for (int a = 0; a < nf * 3; ++a) {
                    const int fl = USER ? a / 3 : (a >= 3 ? 1 : 0), w = a - 3 * fl;
                    const C *src = (w == 0 ? TA : (w == 1 ? TB : TC)) + (long long)fl * g.modes +
                                   (long long)tl * TL * H;
                    bulk_copy_g2s(stage + (size_t)a * TL * H, src, run, &zbar);
                }
            }
            return;
        }
        if (tl < ntiles) {
            const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
            const int nl = nf * 3 * TL;
            for (int li = threadIdx.x >> 5; li < nl; li += nw) {
                const int a = li >> g.tlz_shift, tt = li & (TL - 1);
                const long long ln = (long long)tl * TL + tt;
                if (ln >= g.lines_z) continue;
                const int fl = USER ? a / 3 : (a >= 3 ? 1 : 0), w = a - 3 * fl;
                const C *src = (w == 0 ? TA : (w == 1 ? TB : TC)) + (long long)fl * g.modes + ln * H;
                C *dst = stage + (size_t)li * hs;
                for (int m = lane; m < H; m += 32) cp_async_elem(dst + m, src + m);
            }
        }
        cp_async_commit();
    };
    ModelG<T> mdl;
    mdl.kind = g.model;
    mdl.gsq = (T)g.gsq;
    // <V> partial sums: up to 16 tiles' sites in the field precision, then folded into
    // FP64 (a persistent block walks thousands of tiles at N = 1024; a fold per tile
    // would put a conversion and an add per thread and tile on the narrow FP64 pipe)
    T pot_t[NT] = {};
    double pot_d[NT] = {};
    int nfold = 0;
    // the sums run over V(site) - vref (model_potential_shifted), vref the potential terms of
    // the homogeneous fields (the FP64 shadow of the zero modes / N^3), a value of the state
    // alone; vref is added back once per site summed (every tile gives a thread the same
    // number of sites: the line count is a multiple of the tile's)
    T vref[NT];
    homogeneous_potential<T, T, USER>(mdl, bg, vref);
    if (STAGED) prefetch(vb.x());
    unsigned phase = 0;   // parity of the bulk-copy phase the next tile completes
    for (int tile = vb.x(); tile < ntiles; tile = STAGED ? tile + vb.gx() : ntiles) {
        const int line = tile * TL + t;
        const bool valid = line < g.lines_z;
        C v[16];
        {
            // 1. two real c2r in one N-point transform
            const ZIdx<L> ix{(int)(grp * slot_elems + t * LS)};
            const long long lo = (long long)line * H;
            if (bulk) {
                const bool ok = mbar_wait_bounded(&zbar, phase, bg->wait_ns);
                if (__syncthreads_or(!ok)) {
                    // The tile's copies did not complete in time. Only this tile's copies can
                    // be in flight (the next tile's are issued after this wait), and the block
                    // must not leave while one of them can still write into its shared memory:
                    // report the timeout, wait for them once more (bounded), and leave only
                    // after they landed. If they never do, the copies may still write into
                    // shared memory the SM gives to another block: PSC_ERR_DEVICE says the
                    // context can no longer be trusted. With the test hook the planted bytes
                    // are counted here, so the phase completes once the real copies have.
                    int *err = &const_cast<DevBG *>(bg)->err;
                    if (threadIdx.x == 0) {
                        report_err(err, PSC_ERR_TIMEOUT);
                        if (planted(bg, 2)) mbar_complete_tx(&zbar, planted(bg, 2));
                    }
                    const bool landed = mbar_wait_bounded(&zbar, phase, bg->wait_ns);
                    if (__syncthreads_or(!landed) && threadIdx.x == 0) report_err(err, PSC_ERR_DEVICE);
                    return;
                }
                phase ^= 1u;
            } else if (STAGED) {
                cp_async_wait_all();
                __syncthreads();   // every thread's copies of this tile have landed
            }
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int n = j + r * P;
                const int m = n <= HL ? n : L - n;
                const T fm = n <= HL ? fj + T(r * P) : T(L - r * P) - fj;   // (T)m without a conversion
                C a = mk<T>(0, 0), b = mk<T>(0, 0);
                if (valid) {
                    a = STAGED ? stA[m] : srcA[lo + m];
                    if (kind) {
                        b = STAGED ? stB[m] : srcB[lo + m];
                    } else {
                        const T kz = (m == HL) ? T(0) : kIR * fm;   // d/dz, Nyquist zeroed
                        b = mk<T>(-kz * a.y, kz * a.x);
                    }
                    if (m == 0 || m == HL) {
                        a.y = T(0);
                        b.y = T(0);
                    }
                }
                v[r] = (n <= HL) ? mk<T>(a.x - b.y, a.y + b.x) : mk<T>(a.x + b.y, b.x - a.y);
            }
            if (STAGED) {
                __syncthreads();   // every staging read of this tile is done
                prefetch(tile + vb.gx());
            }
            fft_reg<C, L, +1, true>(v, slots, ix, j, tw, N / L);
            __syncthreads();
#pragma unroll
            for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                for (int r = 0; r < RP::RL; ++r) slots[ix(RP::out(j, q, r))] = cscale_k<true>(v[q * RP::RL + r], inv_n3);
        }
        __syncthreads();
        // 2. pointwise epilogue per site: V'(f), <V>, anisotropic stress
        for (int idx = threadIdx.x; idx < TL * L; idx += blockDim.x) {
            const int tt = idx / L, z = idx - tt * L;
            const long long ln = (long long)tile * TL + tt;
            if (ln >= g.lines_z) continue;
            const int e = tt * LS + z + (z >> 4);
            T f[NF], d[NF][3];
#pragma unroll
            for (int fl = 0; fl < NF; ++fl) {
                if (fl < nf) {
                    const C p0 = slots[(2 * fl) * slot_elems + e], p1 = slots[(2 * fl + 1) * slot_elems + e];
                    f[fl] = p0.x;
                    d[fl][2] = p0.y;
                    d[fl][0] = p1.x;
                    d[fl][1] = p1.y;
                } else {
                    f[fl] = T(0);
                    d[fl][0] = d[fl][1] = d[fl][2] = T(0);
                }
            }
            if (tape_fx) {   // adjoint tape: the real fields
#pragma unroll
                for (int fl = 0; fl < NF; ++fl)
                    if (fl < nf) tape_fx[fl * g.sites + ln * N + z] = f[fl];
            }
            T vp[NF] = {};
            model_dvdf<T, T, USER>(mdl, f, vp, nf);
            model_potential_shifted<T, T, USER>(mdl, f, vref, pot_t);
            const int si[6] = {0, 0, 0, 1, 1, 2}, sj[6] = {0, 1, 2, 1, 2, 2};
            if constexpr (!USER) {
                T o[8];
                o[0] = vp[0];
                o[1] = vp[1];
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    T sum = T(0);
#pragma unroll
                    for (int fl = 0; fl < 2; ++fl)
                        if (fl < nf) sum += T(2) * d[fl][si[c]] * d[fl][sj[c]];
                    o[2 + c] = sum;
                }
                if (nf == 1) {   // V', S_00, ..., S_22, 0
#pragma unroll
                    for (int c = 1; c < 7; ++c) o[c] = o[c + 1];
                    o[7] = T(0);
                }
#pragma unroll
                for (int p = 0; p < 4; ++p) slots[p * slot_elems + e] = mk<T>(o[2 * p], o[2 * p + 1]);
            } else {
                // the products in order V'_0 .. V'_{nf-1}, S_00, ..., S_22, padded with 0
                constexpr int NPO = (kMaxFields + 7) / 2;
                T o[2 * NPO];
#pragma unroll
                for (int q = 0; q < 2 * NPO; ++q) o[q] = q < nf ? vp[q < NF ? q : 0] : T(0);
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    T sum = T(0);
#pragma unroll
                    for (int fl = 0; fl < NF; ++fl)
                        if (fl < nf) sum += T(2) * d[fl][si[c]] * d[fl][sj[c]];
#pragma unroll
                    for (int q = 0; q < 2 * NPO; ++q)
                        if (q == nf + c) o[q] = sum;
                }
#pragma unroll
                for (int p = 0; p < NPO; ++p)
                    if (p < pout) slots[p * slot_elems + e] = mk<T>(o[2 * p], o[2 * p + 1]);
            }
        }
        if ((++nfold & 15) == 0) {
#pragma unroll
            for (int i = 0; i < NT; ++i) {
                pot_d[i] += (double)pot_t[i];
                pot_t[i] = T(0);
            }
        }
        __syncthreads();

        // 3. two real r2c per N-point forward transform of output pair o
        const int nreal = nf + 6;
        const int rounds = (pout + pin - 1) / pin;
        for (int it = 0; it < rounds; ++it) {
            const int o = grp + it * pin;
            const bool act = o < pout;
            const ZIdx<L> ix{(int)((act ? o : 0) * slot_elems + t * LS)};
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = act ? slots[ix(j + r * P)] : mk<T>(0, 0);
            __syncthreads();   // all loads of this round precede the first exchange write
            fft_reg<C, L, -1, true>(v, slots, ix, j, tw, N / L, act);
            {
                const int r0 = 2 * o, r1 = 2 * o + 1;
                auto arr = [&](int ri) -> C * {
                    return ri < nf ? QV + (long long)ri * g.modes : QS + (long long)(ri - nf) * g.modes;
                };
                const bool wr = act && valid;
                C *d0 = wr ? arr(r0) + (long long)line * H : nullptr;
                C *d1 = (wr && r1 < nreal) ? arr(r1) + (long long)line * H : nullptr;
                if constexpr (P <= 32) {
                    // the partners Z[N-k] by warp shuffle (the P lanes of a line in one warp)
#pragma unroll
                    for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                        for (int r = 0; r < RP::RL; ++r) {
                            // out(j, q, r) grows with j: a register whose lane-0 index is above
                            // N/2 holds no written k in any lane (a compile-time skip)
                            if (RP::out(0, q, r) > HL) continue;
                            const int k = RP::out(j, q, r);
                            const C zk = v[q * RP::RL + r];
                            const C zc = partner_out<C, L>(v, j, q, r);   // conj Z[N - k]
                            if (wr && k <= HL) {
                                const C ev = cscale_k<true>(cadd_k<true>(zk, zc), T(0.5));
                                const C dd = cscale_k<true>(csub_k<true>(zk, zc), T(0.5));
                                d0[k] = ev;
                                if (d1) d1[k] = mk<T>(dd.y, -dd.x);
                            }
                        }
                } else {
                    // a line's lanes span two warps (N = 1024): Z goes through its slot and
                    // each lane splits k = j, j + P, ... <= N/2 from there
                    __syncthreads();   // the transform's last exchange reads are done
                    if (act) {
#pragma unroll
                        for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                            for (int r = 0; r < RP::RL; ++r) slots[ix(RP::out(j, q, r))] = v[q * RP::RL + r];
                    }
                    __syncthreads();
                    if (wr) {
                        for (int k = j; k <= HL; k += P) {
                            const C zk = slots[ix(k)], zc = cconj(slots[ix((L - k) & (L - 1))]);
                            const C ev = cscale_k<true>(cadd_k<true>(zk, zc), T(0.5));
                            const C dd = cscale_k<true>(csub_k<true>(zk, zc), T(0.5));
                            d0[k] = ev;
                            if (d1) d1[k] = mk<T>(dd.y, -dd.x);
                        }
                    }
                }
            }
            __syncthreads();   // the transform's last exchange read precedes the next writes
        }
    }
    if (STAGED) cp_async_wait_all();
#pragma unroll
    const double nsite = (double)nfold * ((TL * L - 1 - (int)threadIdx.x) / (int)blockDim.x + 1);
    for (int i = 0; i < NT; ++i) pot_d[i] += (double)pot_t[i] + nsite * (double)vref[i];
    block_reduce_store_t<double, NT>(pot_d, partV, vb.gx(), vb.x());
}

template <typename T, int L, bool STAGED, bool USER = false>
__global__ void __launch_bounds__(256, 2) kr_zpass_gw(Geo g, const cplx<T> *__restrict__ TA,
                                                     const cplx<T> *__restrict__ TB, const cplx<T> *__restrict__ TC,
                                                     cplx<T> *__restrict__ QV, cplx<T> *__restrict__ QS,
                                                     double *__restrict__ partV, const DevBG *bg,
                                                     const cplx<T> *__restrict__ tw, T *__restrict__ tape_fx) {
    kr_zpass_gw_body<T, L, STAGED, USER, HwBlock>(vblock_hw(), g, TA, TB, TC, QV, QS, partV, bg, tw, tape_fx);
}

// ------------------------------------------------------------------ real-space view (c2r along z)
template <typename T, int L>
__global__ void __launch_bounds__(256) kr_z_c2r_real(Geo g, const cplx<T> *__restrict__ TA, T *__restrict__ out,
                                                     const cplx<T> *__restrict__ tw, T inv_n3, int tl_shift) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    constexpr int M = L, P = RP::P, LS = ZIdx<L>::LS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);
    const int TL = 1 << tl_shift, H = g.H, N = g.N;
    const int j = threadIdx.x % P, t = threadIdx.x / P;
    const int line = blockIdx.x * TL + t;
    const bool valid = line < g.lines_z;
    const C *src = TA + (long long)blockIdx.y * g.modes + (long long)line * H;
    C v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const int k = j + r * P;
        C x = mk<T>(0, 0), y = mk<T>(0, 0);
        if (valid) {
            x = src[k];
            y = src[M - k];
        }
        y.y = -y.y;
        if (k == 0) { x.y = T(0); y.y = T(0); }
        const C s = cadd(x, y), d = csub(x, y);
        C w = __ldg(&tw[k]);
        w.y = -w.y;
        const C td = cmul(w, d);
        v[r] = mk<T>(s.x - td.y, s.y + td.x);
    }
    const ZIdx<L> ix{t * LS};
    fft_reg<C, L, +1>(v, sm, ix, j, tw, N / L);
    if (valid) {
        T *o = out + (long long)blockIdx.y * g.sites + (long long)line * N;
#pragma unroll
        for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
            for (int r = 0; r < RP::RL; ++r) {
                const int m = RP::out(j, q, r);
                const C c = cscale(v[q * RP::RL + r], inv_n3);
                o[2 * m] = c.x;
                o[2 * m + 1] = c.y;
            }
    }
}

// ------------------------------------------------------------------ adjoint passes
// Z pass of the adjoint's J^T application at a stage point (no GW): per z line,
// m = c2r(M) / N^3 of every field, the taped real fields f(x) of the point,
// out = eta2 V''(f) m + gamma V'(f) and r2c(out) -> QV; block partial sums of
// sum m.V'(f), sum m.dV'/dgsq, sum m.dV'/dmu (V = mu phi^2/2 + gsq phi^2 chi^2/2, mu = 1).
// Same thread layout, slots and phases as the product's Z pass.
template <typename T, int L>
__global__ void __launch_bounds__(256, 2) kr_zpass_adj(Geo g, const cplx<T> *__restrict__ TA, const T *__restrict__ fx,
                                                    cplx<T> *__restrict__ QV, double *__restrict__ part,
                                                    const DevAdj *__restrict__ ad, const cplx<T> *__restrict__ tw,
                                                    int tl_shift) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    constexpr int M = L, P = RP::P, LS = ZIdx<L>::LS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *slots = reinterpret_cast<C *>(smem_raw);
    // tile of TL lines x nf inputs (its own geometry: a GW handle's Z pass has 4 nf inputs)
    const int sh = tl_shift, TL = 1 << sh, H = g.H, N = g.N;
    const int j = threadIdx.x % P;
    const int t = (threadIdx.x / P) & (TL - 1);
    const int grp = threadIdx.x / (P * TL);
    const size_t slot_elems = (size_t)TL * LS;
    const T inv_n3 = (T)(1.0 / (double)g.sites);
    const T eta2 = (T)ad->eta2, gam = (T)ad->gamma, gsq = (T)g.gsq;
    const bool two = g.model == PSC_MODEL_PHI2CHI2;
    const int ntiles = (g.lines_z + TL - 1) >> sh;
    // per-thread partials: a tile's sites in the field precision, the block's tiles in FP64
    T acc_t[3] = {T(0), T(0), T(0)};
    double acc_d[3] = {0.0, 0.0, 0.0};
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int line = tile * TL + t;
        const bool valid = line < g.lines_z;
        // 1. c2r along z of field grp (own elements into registers, partners by shuffle)
        {
            const C *src = TA + (long long)grp * g.modes + (long long)line * H;
            const ZIdx<L> ix{(int)(grp * slot_elems + t * LS)};
            C v[16], yv[16], xM = mk<T>(0, 0);
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = valid ? src[j + r * P] : mk<T>(0, 0);
            if (valid && j == 0) xM = src[M];
            partners_in<C, M>(v, xM, j, yv);
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int k = j + r * P;
                C x = mk<T>(0, 0), y = mk<T>(0, 0);
                if (valid) {
                    x = v[r];
                    y = yv[r];
                }
                y.y = -y.y;
                if (k == 0) { x.y = T(0); y.y = T(0); }
                const C s = cadd(x, y), d = csub(x, y);
                C w = __ldg(&tw[k]);
                w.y = -w.y;
                const C td = cmul(w, d);
                v[r] = mk<T>(s.x - td.y, s.y + td.x);
            }
            fft_reg<C, L, +1>(v, slots, ix, j, tw, N / L);
            __syncthreads();
#pragma unroll
            for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                for (int r = 0; r < RP::RL; ++r) slots[ix(RP::out(j, q, r))] = cscale(v[q * RP::RL + r], inv_n3);
        }
        __syncthreads();
        // 2. pointwise: Hessian and V' of the taped fields
        for (int idx = threadIdx.x; idx < TL * M; idx += blockDim.x) {
            const int tt = idx / M, m = idx - tt * M;
            const long long ln = (long long)tile * TL + tt;
            if (ln >= g.lines_z) continue;
            const int e = tt * LS + m + (m >> 4);
            const C l0 = slots[e];
            const C f0 = reinterpret_cast<const C *>(fx + ln * N)[m];
            if (two) {
                const C l1 = slots[slot_elems + e];
                const C f1 = reinterpret_cast<const C *>(fx + g.sites + ln * N)[m];
                C o0, o1;
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    const T p = half ? f0.y : f0.x, c = half ? f1.y : f1.x;
                    const T a0 = half ? l0.y : l0.x, a1 = half ? l1.y : l1.x;
                    const T vp0 = p + gsq * p * (c * c), vp1 = gsq * (p * p) * c;
                    const T h00 = T(1) + gsq * (c * c), h01 = T(2) * gsq * p * c, h11 = gsq * (p * p);
                    const T r0 = eta2 * (h00 * a0 + h01 * a1) + gam * vp0;
                    const T r1 = eta2 * (h01 * a0 + h11 * a1) + gam * vp1;
                    if (half) { o0.y = r0; o1.y = r1; } else { o0.x = r0; o1.x = r1; }
                    acc_t[0] += a0 * vp0 + a1 * vp1;
                    acc_t[1] += a0 * p * (c * c) + a1 * (p * p) * c;
                    acc_t[2] += a0 * p;
                }
                slots[e] = o0;
                slots[slot_elems + e] = o1;
            } else {
                C o0;
                o0.x = eta2 * l0.x + gam * f0.x;
                o0.y = eta2 * l0.y + gam * f0.y;
                const T d = l0.x * f0.x + l0.y * f0.y;
                acc_t[0] += d;
                acc_t[2] += d;
                slots[e] = o0;
            }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            acc_d[i] += (double)acc_t[i];
            acc_t[i] = T(0);
        }
        __syncthreads();
        // 3. r2c along z of field grp
        {
            const ZIdx<L> ix{(int)(grp * slot_elems + t * LS)};
            C v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = slots[ix(j + r * P)];
            __syncthreads();
            fft_reg<C, L, -1>(v, slots, ix, j, tw, N / L);
            C *dst = QV + (long long)grp * g.modes + (long long)line * H;
#pragma unroll
            for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                for (int r = 0; r < RP::RL; ++r) {
                    const int k = RP::out(j, q, r);
                    const C zk = v[q * RP::RL + r];
                    const C zc = partner_out<C, M>(v, j, q, r);
                    const C ev = cscale(cadd(zk, zc), T(0.5));
                    const C dd = cscale(csub(zk, zc), T(0.5));
                    const C od = mk<T>(dd.y, -dd.x);
                    const C w = __ldg(&tw[k]);
                    if (valid) dst[k] = cadd(ev, cmul(w, od));
                }
            if (valid && j == 0) dst[M] = mk<T>(v[0].x - v[0].y, T(0));   // X[M] = Re Z[0] - Im Z[0]
            __syncthreads();
        }
    }
    block_reduce_store_t<double, 3>(acc_d, part, gridDim.x, blockIdx.x);
}

// X forward transform of the adjoint's J^T application with its epilogue:
// Lf += fft_x(QV) + eta1 k^2 M + delta k^2 f  (blockIdx.y = field).
template <typename T, int L>
__global__ void __launch_bounds__(xy_threads<L>(), xy_blocks<L>(2)) kr_fft_x_adj(Geo g, const cplx<T> *__restrict__ QV,
                                                    const cplx<T> *__restrict__ Mk, const cplx<T> *__restrict__ fk,
                                                    cplx<T> *__restrict__ Lf, const DevAdj *__restrict__ ad,
                                                    const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);
    const int sh = g.tlx_shift, TL = 1 << sh, N = g.N, H = g.H;
    const int t = threadIdx.x & (TL - 1), j = threadIdx.x >> sh;
    const int line = blockIdx.x * TL + t;
    const bool valid = line < g.lines_x;
    const long long stride = g.lines_x;
    const long long base = (long long)blockIdx.y * g.modes + line;
    auto ix = [&](int n) { return n * TL + t; };
    C v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = valid ? QV[base + (long long)(j + r * RP::P) * stride] : mk<T>(0, 0);
    fft_reg<C, L, -1>(v, sm, ix, j, tw, N / L);
    if (!valid) return;
    const T eta1 = (T)ad->eta1, delta = (T)ad->delta;
    const int y = line / H, kz = line - y * H;
    const int py = pcoord(y, N);
    C lv[16];   // every Lf load before the first Lf store (no alias proof at run-time strides)
#pragma unroll
    for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
        for (int r = 0; r < RP::RL; ++r) lv[q * RP::RL + r] = Lf[base + (long long)RP::out(j, q, r) * stride];
#pragma unroll
    for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
        for (int r = 0; r < RP::RL; ++r) {
            const int n = RP::out(j, q, r);
            const int px = pcoord(n, N);
            const T k2 = (T)(px * px + py * py + kz * kz);
            const long long a = base + (long long)n * stride;
            const C mv = Mk[a], fv = fk[a], y0 = v[q * RP::RL + r];
            C l = lv[q * RP::RL + r];
            l.x += y0.x + k2 * (eta1 * mv.x + delta * fv.x);
            l.y += y0.y + k2 * (eta1 * mv.y + delta * fv.y);
            Lf[a] = l;
        }
}

// ------------------------------------------------------------------ GW adjoint passes
// Z pass of the transposed GW source at a stage point: per z line, the c2r / N^3 of the
// field gradients d_x f (TB), d_y f (TC), d_z f (i k_z TA) of every field and of the six
// adjoint tensor components lambda_ab (LAM), then per site and field
// T_a = 2 sum_b (1 + delta_ab) lambda_ab d_b f (the transpose of S_ab = 2 sum_f d_a f d_b f,
// kernel_GW evolution.cpp:581-601) and the r2c of the 3 nf T_a into Tout.
// Full-length transforms of real-line pairs, as in kr_zpass_gw: input pairs
// (d_x f, d_y f) of each field, (d_z f_0, d_z f_1 or 0), (lambda_0, lambda_1),
// (lambda_2, lambda_3), (lambda_4, lambda_5): nf + 4 pairs; output pairs: the 3 nf T_a
// (field-major) two by two. One tile of TL lines per block; shared memory: nf + 4 slots
// of TL lines x LS complex.
template <typename T, int L>
__global__ void __launch_bounds__(256) kr_zpass_adj_gw(Geo g, const cplx<T> *__restrict__ TA,
                                                     const cplx<T> *__restrict__ TB, const cplx<T> *__restrict__ TC,
                                                     const cplx<T> *__restrict__ LAM, cplx<T> *__restrict__ Tout,
                                                     const cplx<T> *__restrict__ tw, int tl_shift) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    constexpr int P = RP::P, LS = ZIdx<L>::LS, HL = L / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *slots = reinterpret_cast<C *>(smem_raw);
    const int TL = 1 << tl_shift, H = g.H, N = g.N;
    const int nf = g.nf;
    const int pin = nf + 4;          // input pairs
    const int nreal = 3 * nf;        // output reals
    const int pout = (nreal + 1) / 2;
    const int j = threadIdx.x % P;
    const int t = (threadIdx.x / P) & (TL - 1);
    const int grp = threadIdx.x / (P * TL);
    const int line = blockIdx.x * TL + t;
    const bool valid = line < g.lines_z;
    const size_t slot_elems = (size_t)TL * LS;
    const T inv_n3 = (T)(1.0 / (double)g.sites);
    const T kIR = (T)g.kIR;
    const T fj = (T)j;
    // this thread's pair: kind 0 (d_x f, d_y f) of field grp, 1 (d_z f_0, d_z f_1), 2 lambda
    const int kind = grp < nf ? 0 : (grp == nf ? 1 : 2);
    const C *srcA, *srcB;
    if (kind == 0) {
        srcA = TB + (long long)grp * g.modes;
        srcB = TC + (long long)grp * g.modes;
    } else if (kind == 1) {
        srcA = TA;
        srcB = nf > 1 ? TA + g.modes : nullptr;
    } else {
        const int c = 2 * (grp - nf - 1);
        srcA = LAM + (long long)c * g.modes;
        srcB = LAM + (long long)(c + 1) * g.modes;
    }
    const ZIdx<L> ix{(int)(grp * slot_elems + t * LS)};
    C v[16];
    // 1. two real c2r in one N-point transform
    {
        const long long lo = (long long)line * H;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const int n = j + r * P;
            const int m = n <= HL ? n : L - n;
            C a = mk<T>(0, 0), b = mk<T>(0, 0);
            if (valid) {
                a = srcA[lo + m];
                if (srcB) b = srcB[lo + m];
                if (kind == 1) {   // d/dz of both: i k_z, Nyquist zeroed
                    const T fm = n <= HL ? fj + T(r * P) : T(L - r * P) - fj;
                    const T kz = (m == HL) ? T(0) : kIR * fm;
                    a = mk<T>(-kz * a.y, kz * a.x);
                    b = mk<T>(-kz * b.y, kz * b.x);
                }
                if (m == 0 || m == HL) {
                    a.y = T(0);
                    b.y = T(0);
                }
            }
            v[r] = (n <= HL) ? mk<T>(a.x - b.y, a.y + b.x) : mk<T>(a.x + b.y, b.x - a.y);
        }
        fft_reg<C, L, +1>(v, slots, ix, j, tw, N / L);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
            for (int r = 0; r < RP::RL; ++r) slots[ix(RP::out(j, q, r))] = cscale(v[q * RP::RL + r], inv_n3);
    }
    __syncthreads();
    // 2. T_a = 2 sum_b (1 + delta_ab) lambda_ab d_b f per field and site
    for (int idx = threadIdx.x; idx < TL * L; idx += blockDim.x) {
        const int tt = idx / L, z = idx - tt * L;
        if (blockIdx.x * TL + tt >= g.lines_z) continue;
        const int e = tt * LS + z + (z >> 4);
        T lam[6];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const C l = slots[(nf + 1 + c) * slot_elems + e];
            lam[2 * c] = l.x;
            lam[2 * c + 1] = l.y;
        }
        const C dz = slots[nf * slot_elems + e];
        T d[2][3];
#pragma unroll
        for (int fl = 0; fl < 2; ++fl) {
            if (fl < nf) {
                const C dxy = slots[fl * slot_elems + e];
                d[fl][0] = dxy.x;
                d[fl][1] = dxy.y;
                d[fl][2] = fl ? dz.y : dz.x;
            } else {
                d[fl][0] = d[fl][1] = d[fl][2] = T(0);
            }
        }
        // symmetric index of (a, b): 00 0, 01 1, 02 2, 11 3, 12 4, 22 5
        const int sy[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
        T o[6];
#pragma unroll
        for (int fl = 0; fl < 2; ++fl)
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                T acc = T(0);
#pragma unroll
                for (int b2 = 0; b2 < 3; ++b2) acc += ((a == b2) ? T(4) : T(2)) * lam[sy[a][b2]] * d[fl][b2];
                o[fl * 3 + a] = acc;
            }
        if (nf == 1) o[3] = T(0);
#pragma unroll
        for (int p = 0; p < 3; ++p)
            if (p < pout) slots[p * slot_elems + e] = mk<T>(o[2 * p], o[2 * p + 1]);
    }
    __syncthreads();
    // 3. two real r2c per N-point forward transform of output pair grp (groups >= pout
    //    only keep the barriers)
    {
        const bool act = grp < pout;
        const ZIdx<L> ixo{(int)((act ? grp : 0) * slot_elems + t * LS)};
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = act ? slots[ixo(j + r * P)] : mk<T>(0, 0);
        __syncthreads();
        fft_reg<C, L, -1>(v, slots, ixo, j, tw, N / L, act);
        const int r0 = 2 * grp, r1 = 2 * grp + 1;
        const bool wr = act && valid;
        C *d0 = wr ? Tout + (long long)r0 * g.modes + (long long)line * H : nullptr;
        C *d1 = (wr && r1 < nreal) ? Tout + (long long)r1 * g.modes + (long long)line * H : nullptr;
        if constexpr (P <= 32) {
#pragma unroll
            for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                for (int r = 0; r < RP::RL; ++r) {
                    if (RP::out(0, q, r) > HL) continue;   // no lane holds a written k
                    const int k = RP::out(j, q, r);
                    const C zk = v[q * RP::RL + r];
                    const C zc = partner_out<C, L>(v, j, q, r);   // conj Z[N - k]
                    if (wr && k <= HL) {
                        const C ev = cscale(cadd(zk, zc), T(0.5));
                        const C dd = cscale(csub(zk, zc), T(0.5));
                        d0[k] = ev;
                        if (d1) d1[k] = mk<T>(dd.y, -dd.x);
                    }
                }
        } else {
            // a line's lanes span two warps: Z through its slot, then the split from there
            __syncthreads();
            if (act) {
#pragma unroll
                for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
                    for (int r = 0; r < RP::RL; ++r) slots[ixo(RP::out(j, q, r))] = v[q * RP::RL + r];
            }
            __syncthreads();
            if (wr) {
                for (int k = j; k <= HL; k += P) {
                    const C zk = slots[ixo(k)], zc = cconj(slots[ixo((L - k) & (L - 1))]);
                    const C ev = cscale(cadd(zk, zc), T(0.5));
                    const C dd = cscale(csub(zk, zc), T(0.5));
                    d0[k] = ev;
                    if (d1) d1[k] = mk<T>(dd.y, -dd.x);
                }
            }
        }
    }
}

// X forward transform of the three T_a of field blockIdx.y and the transposed source
// gradient: Lf += etaS sum_a i k_a fft_x(T_a), k_a with the Nyquist bin zeroed
// (field_1st_derivative evolution.cpp:466-578), etaS = -a^(1+alpha).
template <typename T, int L>
__global__ void __launch_bounds__(xy_threads<L>(), xy_blocks<L>(2)) kr_fft_x_gwadj(Geo g, const cplx<T> *__restrict__ Tin,
                                                      cplx<T> *__restrict__ Lf, const DevAdj *__restrict__ ad,
                                                      const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);
    const int sh = g.tlx_shift, TL = 1 << sh, N = g.N, H = g.H;
    const int t = threadIdx.x & (TL - 1), j = threadIdx.x >> sh;
    const int line = blockIdx.x * TL + t;
    const bool valid = line < g.lines_x;
    const long long stride = g.lines_x;
    const int fl = blockIdx.y;
    auto ix = [&](int n) { return n * TL + t; };
    const T kIR = (T)g.kIR;
    const int y = line / H, kz = line - y * H;
    const T ky = (y == (N >> 1)) ? T(0) : kIR * (T)pcoord(y, N);
    const T kzv = (kz == (N >> 1)) ? T(0) : kIR * (T)kz;
    C acc[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) acc[r] = mk<T>(0, 0);
#pragma unroll 1
    for (int a = 0; a < 3; ++a) {
        if (a) __syncthreads();   // the exchange buffer is free again
        const long long base = (long long)(fl * 3 + a) * g.modes + line;
        C v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = valid ? Tin[base + (long long)(j + r * RP::P) * stride] : mk<T>(0, 0);
        fft_reg<C, L, -1>(v, sm, ix, j, tw, N / L);
#pragma unroll
        for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
            for (int r = 0; r < RP::RL; ++r) {
                const int n = RP::out(j, q, r);
                const T kk = (a == 0) ? ((n == (N >> 1)) ? T(0) : kIR * (T)pcoord(n, N)) : (a == 1 ? ky : kzv);
                const C z = v[q * RP::RL + r];
                C &o = acc[q * RP::RL + r];
                o.x -= kk * z.y;
                o.y += kk * z.x;
            }
    }
    if (!valid) return;
    const T etaS = (T)ad->etaS;
    const long long base = (long long)fl * g.modes + line;
    C lv[16];
#pragma unroll
    for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
        for (int r = 0; r < RP::RL; ++r) lv[q * RP::RL + r] = Lf[base + (long long)RP::out(j, q, r) * stride];
#pragma unroll
    for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
        for (int r = 0; r < RP::RL; ++r) {
            C l = lv[q * RP::RL + r];
            const C o = acc[q * RP::RL + r];
            l.x += etaS * o.x;
            l.y += etaS * o.y;
            Lf[base + (long long)RP::out(j, q, r) * stride] = l;
        }
}

// Forward transform along x in place (blockIdx.y selects the array of the list): the
// last pass of the padded step's r2c on the padded grid, whose kick runs on the
// lattice grid afterwards.
template <typename T, int L>
__global__ void __launch_bounds__(xy_threads<L>(), xy_blocks<L>(3)) kr_fft_x_plain(Geo g, const __grid_constant__ ArrList arrs,
                                                       const cplx<T> *__restrict__ tw) {
    using C = cplx<T>;
    using RP = RegPlan<L>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);
    C *a = reinterpret_cast<C *>(arrs.p[blockIdx.y]);
    const int sh = g.tlx_shift, TL = 1 << sh;
    const int t = threadIdx.x & (TL - 1), j = threadIdx.x >> sh;
    const int line = blockIdx.x * TL + t;
    const bool valid = line < g.lines_x;
    const long long stride = g.lines_x;
    auto ix = [&](int n) { return n * TL + t; };
    C v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = valid ? a[(long long)(j + r * RP::P) * stride + line] : mk<T>(0, 0);
    fft_reg<C, L, -1>(v, sm, ix, j, tw, g.N / L);
    if (valid) {
#pragma unroll
        for (int q = 0; q < RP::NBL; ++q)
#pragma unroll
            for (int r = 0; r < RP::RL; ++r) a[(long long)RP::out(j, q, r) * stride + line] = v[q * RP::RL + r];
    }
}

}  // namespace psc
