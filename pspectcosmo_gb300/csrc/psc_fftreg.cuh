// psc_fftreg.cuh — register-resident Stockham FFT for lines of compile-time
// length L (16 <= L <= 1024, power of two).
//
// P = L/16 threads cooperate on one line and each owns 16 elements. Stage 0 is a
// radix-16 butterfly on the elements j + r P (r < 16) that thread j loaded
// itself, so the first stage needs no shared memory; every later stage reads
// its inputs from a per-line shared exchange buffer, and the last stage leaves
// its outputs in registers for the caller to store (or to consume in a fused
// epilogue). A 256-point line costs one shared-memory round trip and one block
// barrier. Radix plan: 16, 16, ..., then one radix 2/4/8 stage for the rest.
#pragma once

#include "psc_dev.cuh"

namespace psc {

__host__ __device__ constexpr int reg_rad(int L, int s) {
    int rem = L;
    for (int i = 0; i < s; ++i) rem /= (rem >= 16 ? 16 : rem);
    return rem >= 16 ? 16 : rem;
}
__host__ __device__ constexpr int reg_nstages(int L) {
    int n = 0, rem = L;
    while (rem > 1) {
        rem /= (rem >= 16 ? 16 : rem);
        ++n;
    }
    return n;
}
__host__ __device__ constexpr int reg_span(int L, int s) {
    int ns = 1;
    for (int i = 0; i < s; ++i) ns *= reg_rad(L, i);
    return ns;
}

template <int L>
struct RegPlan {
    static constexpr int P = L / 16;                       // threads per line
    static constexpr int S = reg_nstages(L);               // stages
    static constexpr int RL = reg_rad(L, S - 1);           // radix of the last stage
    static constexpr int NSL = reg_span(L, S - 1);         // span of the last stage
    static constexpr int NBL = 16 / RL;                    // last-stage butterflies per thread
    // element index of output v[q * RL + r] of thread j
    __device__ __forceinline__ static int out(int j, int q, int r) { return (j * NBL + q) + r * NSL; }
};

template <typename C, int L, int DIR, int S, bool PK, typename IX>
__device__ __forceinline__ void reg_stage(C (&v)[16], C *sm, const IX &ix, int j, const C *__restrict__ tw,
                                          int twmul, bool act) {
    constexpr int R = reg_rad(L, S), NS = reg_span(L, S), NB = 16 / R, LR = L / R;
    __syncthreads();   // the previous stage's outputs are in shared memory
    const int tf = (L / (NS * R)) * twmul;
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int b = j * NB + q;
        const int jm = b & (NS - 1);
        C u[R];
#pragma unroll
        for (int r = 0; r < R; ++r) u[r] = act ? sm[ix(b + r * LR)] : v[q * R + r];
#pragma unroll
        for (int r = 1; r < R; ++r) {
            C w = __ldg(&tw[(jm * r) * tf]);
            if (DIR > 0) w.y = -w.y;
            u[r] = cmul(u[r], w);
        }
        dft<R, DIR, C, PK>(u);
#pragma unroll
        for (int r = 0; r < R; ++r) v[q * R + r] = u[r];
    }
    if constexpr (S + 1 < reg_nstages(L)) {
        __syncthreads();   // every read of this stage is done before the buffer is rewritten
        if (act) {
#pragma unroll
            for (int q = 0; q < NB; ++q) {
                const int b = j * NB + q, jm = b & (NS - 1), idxD = (b - jm) * R + jm;
#pragma unroll
                for (int r = 0; r < R; ++r) sm[ix(idxD + r * NS)] = v[q * R + r];
            }
        }
        reg_stage<C, L, DIR, S + 1, PK>(v, sm, ix, j, tw, twmul, act);
    }
}

// v holds the elements j + r P of this thread's line on entry and the outputs
// RegPlan<L>::out(j, q, r) on return. ix(n) maps an element index of the line to
// its shared-memory slot. The exchange buffer must be free on entry (the caller
// synchronizes after any earlier use); on return the last stage has read it, so
// the caller synchronizes again before writing it. `act` = false runs the
// barriers without touching memory (threads without a line this round).
// Twiddles: tw[q] = e^{-2 pi i q / (L twmul)}. PK: packed FP32 butterflies (cadd_k).
template <typename C, int L, int DIR, bool PK = false, typename IX>
__device__ __forceinline__ void fft_reg(C (&v)[16], C *sm, const IX &ix, int j, const C *__restrict__ tw, int twmul,
                                        bool act = true) {
    static_assert(L >= 16 && (L & (L - 1)) == 0 && L <= 1024, "line length");
    dft<16, DIR, C, PK>(v);
    if constexpr (reg_nstages(L) > 1) {
        if (act) {
#pragma unroll
            for (int r = 0; r < 16; ++r) sm[ix(j * 16 + r)] = v[r];
        }
        reg_stage<C, L, DIR, 1, PK>(v, sm, ix, j, tw, twmul, act);
    }
}

}  // namespace psc
