// psc_batch.cuh — one launch per pass for a batch of several configurations (lattice sizes).
//
// Each pass kernel walks a work list that concatenates the blocks of every configuration of
// the batch (BatchTable, psc_launch.h): item w belongs to the group whose range holds it, and
// runs the same pass body as the configuration's own kernel (psc_passes.cuh) on a VBlock that
// names the block of that configuration's grid. The block walks the items blockIdx.x,
// blockIdx.x + gridDim.x, ...: a persistent kernel over (configuration, realization, array,
// tile). Same bodies, same block indices, same geometry: every realization evolves bit for bit
// as it would alone. Line lengths 32 .. 256; every configuration's blocks have 256 threads.
#pragma once

#include "psc_passes.cuh"

namespace psc {

template <typename T, int L, int PASS, bool DRIFT>
__device__ __forceinline__ void batch_item(const BatchGroup &G, unsigned w) {
    using C = cplx<T>;
    const Geo &g = G.g;
    const C *tw = reinterpret_cast<const C *>(G.tw);
    C *fk = (C *)G.fk, *pk = (C *)G.pk, *uk = (C *)G.uk, *puk = (C *)G.puk;
    C *TA = (C *)G.TA, *TB = (C *)G.TB, *TC = (C *)G.TC, *QV = (C *)G.QV, *QS = (C *)G.QS;
    if constexpr (PASS == 0 || PASS == 1) {
        // blocks (x tile, field, realization), x fastest
        const unsigned nbx = (unsigned)G.nbx, nf = (unsigned)g.nf, rest = w / nbx;
        const VBlock vb{w - rest * nbx, rest % nf, rest / nf, nbx};
        if constexpr (PASS == 0) {
            if (g.gwev) kr_ifft_x_body<T, L, true, DRIFT, VBlock>(vb, g, fk, pk, TA, TB, G.bg, tw, nullptr);
            else kr_ifft_x_body<T, L, false, DRIFT, VBlock>(vb, g, fk, pk, TA, TB, G.bg, tw, nullptr);
        } else {
            if (g.gwev) kr_ifft_y_body<T, L, true, VBlock>(vb, g, TA, TB, TC, G.bg, tw);
            else kr_ifft_y_body<T, L, false, VBlock>(vb, g, TA, TB, TC, G.bg, tw);
        }
    } else if constexpr (PASS == 2) {
        // persistent Z blocks (block, realization)
        const unsigned nbz = (unsigned)G.nbz, r = w / nbz;
        const VBlock vb{w - r * nbz, 0u, r, nbz};
        if (g.gwev)
            kr_zpass_gw_body<T, L, sizeof(T) == 4, false, VBlock>(vb, g, TA, TB, TC, QV, QS, G.partV, G.bg, tw,
                                                                  nullptr);
        else
            kr_zpass_body<T, L / 2, false, VBlock>(vb, g, TA, QV, G.partV, G.bg, tw, nullptr);
    } else {
        // blocks (x tile, forward array, realization)
        const unsigned nbx = (unsigned)G.nbx, nj = (unsigned)G.nj, rest = w / nbx;
        const VBlock vb{w - rest * nbx, rest % nj, rest / nj, nbx};
        if constexpr (PASS == 3) {
            kr_fft_y_body<T, L, VBlock>(vb, g, G.fwd, tw);
        } else {
            if (g.gwev)
                kr_fft_x_final_body<T, L, true, VBlock>(vb, g, QV, QS, fk, pk, uk, puk, G.partKG, G.bg, tw, nullptr,
                                                        nullptr, nullptr, nullptr, nullptr, (C *)G.Fk, (C *)G.Fu, nullptr);
            else
                kr_fft_x_final_body<T, L, false, VBlock>(vb, g, QV, QS, fk, pk, uk, puk, G.partKG, G.bg, tw, nullptr,
                                                         nullptr, nullptr, nullptr, nullptr, (C *)G.Fk, nullptr, nullptr);
        }
    }
}

// Y forward keeps its three blocks per SM (80 registers), the other passes two.
template <typename T, int PASS, bool DRIFT>
__global__ void __launch_bounds__(256, PASS == 3 ? 3 : 2) kr_batch_pass(const __grid_constant__ BatchTable bt) {
    const unsigned total = (unsigned)bt.total[PASS];
    for (unsigned w = blockIdx.x; w < total; w += gridDim.x) {
        int gi = 0;
        while (gi + 1 < bt.ngroups && w >= (unsigned)bt.grp[gi + 1].start[PASS]) ++gi;
        const BatchGroup &G = bt.grp[gi];
        const unsigned local = w - (unsigned)G.start[PASS];
        switch (G.L) {
        case 32: batch_item<T, 32, PASS, DRIFT>(G, local); break;
        case 64: batch_item<T, 64, PASS, DRIFT>(G, local); break;
        case 128: batch_item<T, 128, PASS, DRIFT>(G, local); break;
        case 256: batch_item<T, 256, PASS, DRIFT>(G, local); break;
        default: break;
        }
        __syncthreads();   // the next item reuses the shared memory
    }
}

template <typename T>
const void *batch_kernel(int pass, int drift) {
    switch (pass) {
    case 0: return drift ? (const void *)kr_batch_pass<T, 0, true> : (const void *)kr_batch_pass<T, 0, false>;
    case 1: return (const void *)kr_batch_pass<T, 1, false>;
    case 2: return (const void *)kr_batch_pass<T, 2, false>;
    case 3: return (const void *)kr_batch_pass<T, 3, false>;
    case 4: return (const void *)kr_batch_pass<T, 4, false>;
    default: return nullptr;
    }
}

template <typename T>
cudaError_t batch_pass(const BatchTable &bt, int pass, int drift, int grid, size_t smem, cudaStream_t st) {
    switch (pass) {
    case 0:
        if (drift) kr_batch_pass<T, 0, true><<<grid, 256, smem, st>>>(bt);
        else kr_batch_pass<T, 0, false><<<grid, 256, smem, st>>>(bt);
        break;
    case 1: kr_batch_pass<T, 1, false><<<grid, 256, smem, st>>>(bt); break;
    case 2: kr_batch_pass<T, 2, false><<<grid, 256, smem, st>>>(bt); break;
    case 3: kr_batch_pass<T, 3, false><<<grid, 256, smem, st>>>(bt); break;
    case 4: kr_batch_pass<T, 4, false><<<grid, 256, smem, st>>>(bt); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace psc

#define PSC_DEFINE_BATCH_ENTRY(T, SUFFIX)                                                                        \
    namespace psc {                                                                                              \
    cudaError_t reg_batch_pass_##SUFFIX(const BatchTable &bt, int pass, int drift, int grid, size_t smem,        \
                                        cudaStream_t st) {                                                       \
        return batch_pass<T>(bt, pass, drift, grid, smem, st);                                                   \
    }                                                                                                            \
    const void *reg_batch_kernel_##SUFFIX(int pass, int drift) { return batch_kernel<T>(pass, drift); }           \
    }
