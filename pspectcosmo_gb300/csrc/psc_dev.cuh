// psc_dev.cuh — device-side building blocks of the GB300 lattice step:
// complex types, the background record, the model, and the shared-memory
// Stockham FFT engine used by every pass kernel.
//
// Layout conventions (match the reference's FFTW arrays, pspectcosmo.h:179-190):
//   half spectrum  [x][y][kz], kz in [0, N/2], kz fastest, H = N/2 + 1
//   real lattice   [x][y][z],  z fastest
// Transforms are unnormalised like FFTW's; the 1/N^3 of every c2r
// (evolution.cpp:1150, 1176) is applied in the Z-pass epilogue.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "psc.h"
#include "psc_bg.h"
#include "psc_model.h"

namespace psc {

// ------------------------------------------------------------------ types
template <typename T> struct CplxOf;
template <> struct CplxOf<float> { using type = float2; };
template <> struct CplxOf<double> { using type = double2; };
template <typename T> using cplx = typename CplxOf<T>::type;

template <typename T> __device__ __forceinline__ cplx<T> mk(T re, T im) { cplx<T> c; c.x = re; c.y = im; return c; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename C, typename T> __device__ __forceinline__ C cscale(C a, T s) { a.x *= s; a.y *= s; return a; }
template <typename C> __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
// Complex add, subtract and real scale with a choice of arithmetic: PK = true puts FP32
// values on the packed f32x2 instructions of sm_100 and later (one instruction for both
// components, each rounded as the scalar operation would be; a - b as the exact fma
// b (-1) + a). Packed operands need aligned register pairs, which costs registers: it pays
// in the instruction-bound Z passes (GW Z pass 0.428 -> 0.400 ms at 256^3) and not in the
// latency-bound X and Y passes (X forward + kick 0.559 -> 0.580 ms), so only the Z passes
// ask for it.
template <bool PK, typename C> __device__ __forceinline__ C cadd_k(C a, C b) {
    if constexpr (PK && sizeof(a.x) == 4) return __fadd2_rn(a, b);
    else return cadd(a, b);
}
template <bool PK, typename C> __device__ __forceinline__ C csub_k(C a, C b) {
    if constexpr (PK && sizeof(a.x) == 4) return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
    else return csub(a, b);
}
template <bool PK, typename C, typename T> __device__ __forceinline__ C cscale_k(C a, T s) {
    if constexpr (PK && sizeof(a.x) == 4) return __fmul2_rn(a, make_float2(s, s));
    else return cscale(a, s);
}


// ------------------------------------------------------------------ model (model.h)
// Per-site evaluation of the model in the arithmetic of the pass: V'(phi) and the potential
// terms. The built-in models (PSC_MODEL_PHI2, model.h:35-99, and the two-field
// phi^2 chi^2 model) are written out here; a user model (PSC_MODEL_USER + i) is its model.h
// compiled in the same precision (psc_user_models.cuh). USER = false compiles the built-in
// models only: the pass instantiations of the built-in models (nf <= 2) keep the code and
// registers of the hand-written forms; USER = true adds the user models.
// The coupling is held in the precision G of the arithmetic that uses it (the field
// precision in the register engine: no per-site FP64 -> FP32 conversion).
template <typename G = double>
struct ModelG {
    int kind;   // PSC_MODEL_*
    G gsq;
};
using Model = ModelG<double>;

template <typename T, typename G, bool USER = false>
__host__ __device__ __forceinline__ void model_dvdf(const ModelG<G> &m, const T *v, T *out, int nf) {
    if constexpr (USER) {
        if (m.kind >= PSC_MODEL_USER) {
            um_dvdf<T>(m.kind - PSC_MODEL_USER, v, out, nf);
            return;
        }
    }
    if (m.kind == PSC_MODEL_PHI2) {
        out[0] = v[0];
    } else {
        const T g = (T)m.gsq;
        out[0] = v[0] + g * v[0] * (v[1] * v[1]);
        if (nf > 1) out[1] = g * (v[0] * v[0]) * v[1];
    }
}

// Accumulates in A: the field precision for the per-thread partial sums of the
// register engine (a thread adds a handful of sites before the FP64 block sum),
// double in the generic engine.
template <typename T, typename A = double, typename G = double, bool USER = false>
__host__ __device__ __forceinline__ void model_potential(const ModelG<G> &m, const T *v, A *terms) {
    if constexpr (USER) {
        if (m.kind >= PSC_MODEL_USER) {
            T t[kMaxTerms] = {};
            um_potential<T>(m.kind - PSC_MODEL_USER, v, t);
#pragma unroll
            for (int i = 0; i < kMaxTerms; ++i) terms[i] += (A)t[i];
            return;
        }
    }
    const A p = (A)v[0];
    terms[0] += A(0.5) * p * p;
    if (m.kind == PSC_MODEL_PHI2CHI2) {
        const A c = (A)v[1];
        terms[1] += A(0.5) * (A)m.gsq * p * p * c * c;
    }
}

// The potential terms of one site minus a reference value per term, accumulated in the
// field precision: terms[t] += V_t(v) - ref[t]. A plain FP32 sum of a thread's sites adds a
// long run of nearly equal values (phi^2/2 of a lattice dominated by its homogeneous mode),
// and its roundings do not cancel: at 256^3 two-field preheating <V> came out 5e-7 high
// after one step, which a'' ~ (V - 2K) amplifies tenfold. Shifted by the terms of the
// homogeneous fields (homogeneous_potential), the summands are the sites' small deviations.
// The caller counts its sites and adds count x ref in FP64.
template <typename T, typename G, bool USER = false>
__host__ __device__ __forceinline__ void model_potential_shifted(const ModelG<G> &m, const T *v, const T *ref, T *terms) {
    if constexpr (USER) {
        if (m.kind >= PSC_MODEL_USER) {
            T t[kMaxTerms] = {};
            um_potential<T>(m.kind - PSC_MODEL_USER, v, t);
#pragma unroll
            for (int i = 0; i < kMaxTerms; ++i) terms[i] += t[i] - ref[i];
            return;
        }
    }
    const T p = v[0];
    terms[0] += fma(T(0.5) * p, p, -ref[0]);
    if (m.kind == PSC_MODEL_PHI2CHI2) {
        const T c = v[1];
        terms[1] += fma(T(0.5) * (T)m.gsq * p * p * c, c, -ref[1]);
    }
}

// The potential terms of the homogeneous fields, the FP64 shadow of the zero modes over
// N^3 (zero when the shadow is not set): a reference for model_potential_shifted that depends
// on the state alone, so that resumed and uninterrupted runs sum identically.
template <typename T, typename G, bool USER = false>
__device__ __forceinline__ void homogeneous_potential(const ModelG<G> &m, const DevBG *bg, T *ref) {
    T f[kMaxFields] = {};
    if (bg->zero64)
        for (int q = 0; q < kMaxFields; ++q)
            if (q < bg->nf) f[q] = (T)(bg->z0f[q][0] * bg->inv_n3);
    if constexpr (USER) {   // ref has kMaxTerms entries (two in the built-in instantiations)
        for (int i = 0; i < kMaxTerms; ++i) ref[i] = T(0);
        if (m.kind >= PSC_MODEL_USER) {
            um_potential<T>(m.kind - PSC_MODEL_USER, f, ref);
            return;
        }
    }
    ref[0] = T(0.5) * f[0] * f[0];
    ref[1] = m.kind == PSC_MODEL_PHI2CHI2 ? T(0.5) * (T)m.gsq * f[0] * f[0] * f[1] * f[1] : T(0);
}

// ------------------------------------------------------------------ FFT engine
// cos/sin(2 pi k / 16): exact decimal expansions of the algebraic values.
__host__ __device__ constexpr double cos16(int k) {
    switch (k & 15) {
    case 0: return 1.0;
    case 1: return 0.92387953251128675613;
    case 2: return 0.70710678118654752440;
    case 3: return 0.38268343236508977173;
    case 4: return 0.0;
    case 5: return -0.38268343236508977173;
    case 6: return -0.70710678118654752440;
    case 7: return -0.92387953251128675613;
    case 8: return -1.0;
    case 9: return -0.92387953251128675613;
    case 10: return -0.70710678118654752440;
    case 11: return -0.38268343236508977173;
    case 12: return 0.0;
    case 13: return 0.38268343236508977173;
    case 14: return 0.70710678118654752440;
    default: return 0.92387953251128675613;
    }
}
__host__ __device__ constexpr double sin16(int k) { return cos16(k - 4); }

template <int R> __host__ __device__ constexpr int brev(int i) {
    int r = 0;
    for (int b = 1, m = R >> 1; b < R; b <<= 1, m >>= 1)
        if (i & b) r |= m;
    return r;
}

// In-register R-point DFT (R = 2, 4, 8, 16), direction DIR = -1 (forward,
// e^{-2 pi i}) or +1 (backward): bit reversal + radix-2 butterflies with
// compile-time twiddles.
template <int R, int DIR, typename C, bool PK = false>
__device__ __forceinline__ void dft(C (&v)[R]) {
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int j = brev<R>(i);
        if (i < j) { C t = v[i]; v[i] = v[j]; v[j] = t; }
    }
#pragma unroll
    for (int len = 2; len <= R; len <<= 1) {
#pragma unroll
        for (int i = 0; i < R; i += len) {
#pragma unroll
            for (int k = 0; k < len / 2; ++k) {
                const int ti = k * (16 / len);
                C u = v[i + k], x = v[i + k + len / 2], t;
                if (PK && ti == 4) {
                    // t = -+i x: the swapped components go straight into scalar adds (a packed
                    // add would first need them swapped in registers)
                    C a = u, b = u;
                    if (DIR < 0) {
                        a.x += x.y; a.y -= x.x; b.x -= x.y; b.y += x.x;
                    } else {
                        a.x -= x.y; a.y += x.x; b.x += x.y; b.y -= x.x;
                    }
                    v[i + k] = a;
                    v[i + k + len / 2] = b;
                    continue;
                }
                if (ti == 0) {
                    t = x;
                } else if (ti == 4) {
                    if (DIR < 0) { t.x = x.y; t.y = -x.x; } else { t.x = -x.y; t.y = x.x; }
                } else {
                    using T = decltype(x.x);
                    const T c = (T)cos16(ti), s = (T)(DIR * sin16(ti));
                    t.x = x.x * c - x.y * s;
                    t.y = x.x * s + x.y * c;
                }
                v[i + k] = cadd_k<PK>(u, t);
                v[i + k + len / 2] = csub_k<PK>(u, t);
            }
        }
    }
}

// cos/sin(2 pi k / R) for the odd radices R = 3, 5, 7 of the generic engine (lattice sizes
// that are not powers of two): decimal expansions of the algebraic values, k = 0 .. R/2.
__host__ __device__ constexpr double cos_odd(int R, int k) {
    return R == 3 ? (k == 0 ? 1.0 : -0.5)
         : R == 5 ? (k == 0 ? 1.0 : k == 1 ? 0.30901699437494742410 : -0.80901699437494742410)
                  : (k == 0 ? 1.0 : k == 1 ? 0.62348980185873353053 : k == 2 ? -0.22252093395631440429
                                                                               : -0.90096886790241912624);
}
__host__ __device__ constexpr double sin_odd(int R, int k) {
    return R == 3 ? (k == 0 ? 0.0 : 0.86602540378443864676)
         : R == 5 ? (k == 0 ? 0.0 : k == 1 ? 0.95105651629515357212 : 0.58778525229247312917)
                  : (k == 0 ? 0.0 : k == 1 ? 0.78183148246802980871 : k == 2 ? 0.97492791218182360702
                                                                               : 0.43388373911755812048);
}

// In-register R-point DFT for odd prime R (3, 5, 7), direction DIR: the symmetric form
// Y[k] = v0 + sum_{m=1}^{(R-1)/2} [(v_m + v_{R-m}) cos(2 pi k m / R)
//        + DIR i (v_m - v_{R-m}) sin(2 pi k m / R)], with compile-time constants.
template <int R, int DIR, typename C>
__device__ __forceinline__ void dft_odd(C (&v)[R]) {
    using T = decltype(v[0].x);
    constexpr int H2 = R / 2;
    C s[H2 + 1], d[H2 + 1];
#pragma unroll
    for (int m = 1; m <= H2; ++m) {
        s[m] = mk<T>(v[m].x + v[R - m].x, v[m].y + v[R - m].y);
        d[m] = mk<T>(v[m].x - v[R - m].x, v[m].y - v[R - m].y);
    }
    C y[R];
    y[0] = v[0];
#pragma unroll
    for (int m = 1; m <= H2; ++m) {
        y[0].x += s[m].x;
        y[0].y += s[m].y;
    }
#pragma unroll
    for (int k = 1; k <= H2; ++k) {
        T ar = v[0].x, ai = v[0].y, br = T(0), bi = T(0);
#pragma unroll
        for (int m = 1; m <= H2; ++m) {
            const int q = (k * m) % R, qq = q <= H2 ? q : R - q;
            const T c = (T)cos_odd(R, qq), sn = (T)(q <= H2 ? sin_odd(R, qq) : -sin_odd(R, qq));
            ar += c * s[m].x;
            ai += c * s[m].y;
            br += sn * d[m].x;
            bi += sn * d[m].y;
        }
        // DIR i (br + i bi) = DIR (-bi + i br)
        y[k] = mk<T>(ar - T(DIR) * bi, ai + T(DIR) * br);
        y[R - k] = mk<T>(ar + T(DIR) * bi, ai - T(DIR) * br);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = y[k];
}

// One Stockham autosort stage (radix R, span Ns) over a tile of TL lines of
// length L held in shared memory as s[n * LD + t] (element n of line t).
// Twiddles come from tw[q] = e^{-2 pi i q / Ntw}, the table of the lattice
// length; a length-L transform uses every (Ntw/L)-th entry.
template <typename C, int R, int DIR>
__device__ __forceinline__ void stockham_stage(const C *__restrict__ src, C *__restrict__ dst, int L, int Ns, int tl_shift,
                                               int LD, const C *__restrict__ tw, int Ntw) {
    const int LR = L / R;
    const int TL = 1 << tl_shift;
    const int nb = LR << tl_shift;
    const int tws = Ntw / (Ns * R);
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const int t = b & (TL - 1);
        const int j = b >> tl_shift;
        const int jm = j % Ns;
        C v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[(j + r * LR) * LD + t];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                C w = __ldg(&tw[jm * r * tws]);
                if (DIR > 0) w.y = -w.y;
                v[r] = cmul(v[r], w);
            }
        }
        if constexpr (R == 3 || R == 5 || R == 7) dft_odd<R, DIR>(v);
        else dft<R, DIR>(v);
        const int idxD = (j - jm) * R + jm;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[(idxD + r * Ns) * LD + t] = v[r];
    }
}

// Transform all TL lines of a tile (length L >= 2 with prime factors 2, 3, 5, 7: radix 16,
// 8, 4, 2 while L's power of two lasts, then 3, 5, 7). Ping-pongs between a and b; returns
// the buffer holding the result. Begins and ends with a block barrier.
template <typename C, int DIR>
__device__ C *fft_tile(C *a, C *b, int L, int tl_shift, int LD, const C *__restrict__ tw, int Ntw) {
    C *src = a, *dst = b;
    int Ns = 1, rem = L;
    while (rem > 1) {
        __syncthreads();
        int R;
        if (rem % 16 == 0) {
            stockham_stage<C, 16, DIR>(src, dst, L, Ns, tl_shift, LD, tw, Ntw);
            R = 16;
        } else if (rem % 8 == 0) {
            stockham_stage<C, 8, DIR>(src, dst, L, Ns, tl_shift, LD, tw, Ntw);
            R = 8;
        } else if (rem % 4 == 0) {
            stockham_stage<C, 4, DIR>(src, dst, L, Ns, tl_shift, LD, tw, Ntw);
            R = 4;
        } else if (rem % 2 == 0) {
            stockham_stage<C, 2, DIR>(src, dst, L, Ns, tl_shift, LD, tw, Ntw);
            R = 2;
        } else if (rem % 3 == 0) {
            stockham_stage<C, 3, DIR>(src, dst, L, Ns, tl_shift, LD, tw, Ntw);
            R = 3;
        } else if (rem % 5 == 0) {
            stockham_stage<C, 5, DIR>(src, dst, L, Ns, tl_shift, LD, tw, Ntw);
            R = 5;
        } else {
            stockham_stage<C, 7, DIR>(src, dst, L, Ns, tl_shift, LD, tw, Ntw);
            R = 7;
        }
        Ns *= R;
        rem /= R;
        C *x = src; src = dst; dst = x;
    }
    __syncthreads();
    return src;
}

// ------------------------------------------------------------------ asynchronous copies
// One complex element global -> shared with cp.async (sm_80+ LDGSTS); 8-byte
// elements use the .ca form, 16-byte elements the .cg form.
__device__ __forceinline__ void cp_async_elem(float2 *dst, const float2 *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_elem(double2 *dst, const double2 *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// ------------------------------------------------------------------ bulk copies (TMA) and mbarriers
// One-dimensional bulk copies global -> shared by the tensor memory accelerator, completed
// on an mbarrier (transaction bytes). Addresses and sizes must be multiples of 16 bytes.
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// makes an initialised mbarrier visible to the asynchronous proxy
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
// orders this thread's earlier shared-memory accesses before later bulk-copy writes
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// arrives on bar (count 1) and adds `bytes` to the transactions its phase waits for
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// Tiled tensor copy global -> shared by the tensor memory accelerator: the box of the tensor
// map at coordinates (c0, c1, c2, c3), innermost first, written to dst (128-byte aligned) in
// the box's row-major order and completed on an mbarrier. map is the address of a
// __grid_constant__ kernel parameter.
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];\n" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}
// Waits until phase `parity` of bar has completed, for at most limit_ns of wall time:
// true when it completed, false when the limit ran out (the caller reports a timeout).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer_ns() - t0 > limit_ns) return false;
    }
}
// the default limit of the waits on bulk copies (DevBG::wait_ns): far above any copy's
// time, short enough that a lost completion returns an error instead of holding the GPU
constexpr unsigned long long kBulkWaitNs = 1000000000ull;
// counts `bytes` of transactions as complete on bar's current phase, as an arriving copy does
__device__ __forceinline__ void mbar_complete_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.complete_tx.relaxed.cta.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// The test hook's planted bytes for a staged tile of pass `pass` (0 in normal runs).
__device__ __forceinline__ unsigned planted(const DevBG *bg, int pass) {
    return bg->wait_plant_pass == pass ? (unsigned)bg->wait_plant : 0u;
}
// Error word of a device record: the first cause wins (a later failure does not overwrite
// it), except that PSC_ERR_DEVICE, which says the context can no longer be trusted,
// replaces a PSC_ERR_TIMEOUT.
__device__ __forceinline__ void report_err(int *err, int code) {
    const int old = atomicCAS(err, 0, code);
    if (old == PSC_ERR_TIMEOUT && code == PSC_ERR_DEVICE) atomicCAS(err, PSC_ERR_TIMEOUT, code);
}

// ------------------------------------------------------------------ reductions
// Block reduction of NV doubles; thread 0 stores out[i * stride + blockIdx.x].
// Deterministic for a fixed block size.
template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double *out, int stride, int slot) {
    __shared__ double red[32][NV > 0 ? NV : 1];
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
            if (lane == 0) out[i * stride + slot] = x;
        }
    }
}

// The same with the per-thread values in the field precision T: the warp-level
// shuffle sums run in T, only the per-warp partials are summed in FP64 (GB300's FP64
// pipe is narrow; a full FP64 tree per block showed up as 10-17 % FP64-pipe time in
// the passes that reduce).
template <typename T, int NV>
__device__ __forceinline__ void block_reduce_store_t(T (&v)[NV], double *out, int stride, int slot) {
    __shared__ double red[32][NV > 0 ? NV : 1];
#pragma unroll
    for (int i = 0; i < NV; ++i)
        for (int off = 16; off > 0; off >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) red[warp][i] = (double)v[i];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double x = lane < nw ? red[lane][i] : 0.0;
            for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
            if (lane == 0) out[i * stride + slot] = x;
        }
    }
}

__device__ __forceinline__ int pcoord(int i, int N) { return i <= (N >> 1) ? i : i - N; }

// x^n for a small integer n by repeated squaring: the scale-factor powers a^(1+alpha),
// a^(3+alpha), a^(alpha-3), ... of the background update. A one-thread kernel runs
// these on the FP64 pipe, where a general pow() costs microseconds.
__device__ __forceinline__ double ipow(double x, int n) {
    unsigned m = n < 0 ? (unsigned)(-n) : (unsigned)n;
    double r = 1.0, b = x;
    while (m) {
        if (m & 1u) r *= b;
        b *= b;
        m >>= 1;
    }
    return n < 0 ? 1.0 / r : r;
}

}  // namespace psc
