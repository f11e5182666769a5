// psc_noalloc.cu — the scalar power spectrum computed without any device
// allocation, for callers that cannot call cudaMalloc.
//
// Some callers own all device memory themselves: a host application that
// hands every byte of the GPU to its own memory pool up front, or code that
// must not allocate once it is set up (allocation synchronises the device and
// can fail late). psc_spectra needs a handle, and a handle allocates its bin
// accumulators with cudaMalloc. psc_spectra_noalloc takes the caller's device
// arrays instead and keeps its bin accumulators in one fixed array of device
// memory that is part of the library image: `g_spectra_scratch` below, sized for
// N <= PSC_NOALLOC_MAX_N and nflds <= 2 (about 50 KB). Every GPU that loads the
// library holds that array until the process exits.
//
// The accumulators are shared by every call on a device and keep the last
// call's sums; each call clears them before use. Calls whose work overlaps on
// the GPU (different streams, or different host threads) race on them.
#include <cmath>

#include "../../include/psc.h"
#include "psc_dev.cuh"
#include "psc_launch.h"

namespace {

constexpr int kMaxBins = 888;   // psc_maxnumbins(PSC_NOALLOC_MAX_N)
constexpr int kMaxFlds = 2;
constexpr int kSumDoubles = kMaxFlds * 3 * kMaxBins;   // sums of |f|^2, |pi|^2, n^2 per field and bin
constexpr int kCountInts = kMaxFlds * kMaxBins;        // mode counts per field and bin

// Bin sums then counts (the ints start on a 256-byte boundary).
struct SpectraScratch {
    double sums[kSumDoubles];
    alignas(256) int counts[kCountInts];
};
static __device__ __align__(256) SpectraScratch g_spectra_scratch;

int fail(int code, const char *msg) {
    psc::set_last_error(msg);
    return code;
}

// The bin sums of output.cpp:626-669 for one field: every stored mode, weight 2
// for 0 < kz < N/2, bin l = floor(sqrt(px^2 + py^2 + kz^2) + 0.5). Same
// arithmetic as the handle-based spectrum kernel; the accumulators are the
// static scratch instead of handle memory.
template <typename T>
__global__ void k_spectra_noalloc(int N, long long modes, const psc::cplx<T> *__restrict__ fk,
                                  const psc::cplx<T> *__restrict__ pk, double aop, double hub, int nb,
                                  SpectraScratch *scratch) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sF = reinterpret_cast<double *>(smem_raw);
    double *sP = sF + nb, *sN = sP + nb;
    int *sC = reinterpret_cast<int *>(sN + nb);
    for (int i = threadIdx.x; i < nb; i += blockDim.x) { sF[i] = sP[i] = sN[i] = 0.0; sC[i] = 0; }
    __syncthreads();
    const int fld = blockIdx.y, H = N / 2 + 1, M = N / 2;
    const psc::cplx<T> *f = fk + (long long)fld * modes, *p = pk + (long long)fld * modes;
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < modes;
         m += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(m % H);
        const long long xy = m / H;
        const int y = (int)(xy % N), x = (int)(xy / N);
        const int px = psc::pcoord(x, N), py = psc::pcoord(y, N);
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
    double *aF = scratch->sums + (size_t)fld * 3 * nb;
    int *cnt = scratch->counts + (size_t)fld * nb;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        if (sC[i] == 0) continue;
        atomicAdd(&aF[i], sF[i]);
        atomicAdd(&aF[nb + i], sP[i]);
        atomicAdd(&aF[2 * nb + i], sN[i]);
        atomicAdd(&cnt[i], sC[i]);
    }
}

// Per-bin means into the caller's arrays (the division spectra() does before
// printing, output.cpp:674-680).
__global__ void k_spectra_noalloc_finish(int nf, int nb, const SpectraScratch *scratch, int32_t *numpoints, double *f2,
                                         double *pi2, double *n2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf * nb) return;
    const int fld = i / nb, l = i - fld * nb;
    const int c = scratch->counts[i];
    const double d = c > 0 ? (double)c : 1.0;
    const double *s = scratch->sums + (size_t)fld * 3 * nb;
    if (numpoints) numpoints[i] = c;
    if (f2) f2[i] = s[l] / d;
    if (pi2) pi2[i] = s[nb + l] / d;
    if (n2) n2[i] = s[2 * nb + l] / d;
}

}  // namespace

extern "C" int psc_spectra_noalloc(const psc_params *p, double a, double ad, const void *f_k, const void *pi_k,
                                   int32_t *numpoints, double *f2, double *pi2, double *n2, void *stream) {
    if (!p || !f_k || !pi_k) return fail(PSC_ERR_ARG, "null argument");
    if (p->N < 8 || p->N > PSC_NOALLOC_MAX_N || (p->N & (p->N - 1)) != 0)
        return fail(PSC_ERR_CONFIG, "psc_spectra_noalloc: N must be a power of two in [8, PSC_NOALLOC_MAX_N]");
    if (p->nflds < 1 || p->nflds > kMaxFlds) return fail(PSC_ERR_CONFIG, "psc_spectra_noalloc: nflds must be 1 or 2");
    if (p->precision != 32 && p->precision != 64) return fail(PSC_ERR_CONFIG, "precision must be 32 or 64");
    const int nb = psc_maxnumbins(p->N);
    if (nb > kMaxBins) return fail(PSC_ERR_CONFIG, "psc_spectra_noalloc: too many bins");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(PSC_ERR_CUDA, "psc_spectra_noalloc: no current CUDA device");
    if (st) {
        // the scratch address below is the current device's copy: the stream must be on it
        int sdev = -1;
        if (cudaStreamGetDevice(st, &sdev) != cudaSuccess)
            return fail(PSC_ERR_ARG, "psc_spectra_noalloc: not a valid CUDA stream");
        if (sdev != dev)
            return fail(PSC_ERR_ARG, "psc_spectra_noalloc: the stream belongs to another device than the current one");
    }
    // Device address of g_spectra_scratch on the current device. In host code the symbol
    // itself is only a host-side stand-in, never a device address. The lookup is made on
    // every call, so a context created anew on the device (after cudaDeviceReset) is served
    // by its own copy; the first lookup in a context loads the library's device code there,
    // which is the set-up that should come before any stream capture.
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_spectra_scratch);
    if (e != cudaSuccess) return fail(PSC_ERR_CUDA, cudaGetErrorString(e));
    SpectraScratch *scratch = static_cast<SpectraScratch *>(ptr);
    // clear the accumulators this call uses (the previous call's sums are still there)
    e = cudaMemsetAsync(scratch->sums, 0, sizeof(double) * 3 * nb * p->nflds, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch->counts, 0, sizeof(int) * nb * p->nflds, st);
    if (e != cudaSuccess) return fail(PSC_ERR_CUDA, cudaGetErrorString(e));
    const long long modes = (long long)p->N * p->N * (p->N / 2 + 1);
    const double aop = std::pow(a, p->alpha - 3), hub = ad / a;
    const size_t smem = (size_t)nb * (3 * sizeof(double) + sizeof(int));
    const dim3 grid(4 * 152, p->nflds);
    if (p->precision == 32)
        k_spectra_noalloc<float><<<grid, 256, smem, st>>>(p->N, modes, static_cast<const float2 *>(f_k),
                                                          static_cast<const float2 *>(pi_k), aop, hub, nb, scratch);
    else
        k_spectra_noalloc<double><<<grid, 256, smem, st>>>(p->N, modes, static_cast<const double2 *>(f_k),
                                                           static_cast<const double2 *>(pi_k), aop, hub, nb, scratch);
    const int total = p->nflds * nb;
    k_spectra_noalloc_finish<<<(total + 255) / 256, 256, 0, st>>>(p->nflds, nb, scratch, numpoints, f2, pi2, n2);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(PSC_ERR_CUDA, cudaGetErrorString(e));
    return PSC_OK;
}
