// psc_outputs.cu — output-step quantities of the real-space fields, on the device, and
// the checkpoint files:
//   * histograms()      output.cpp:1193-1297 (bin frequencies, lower edge, bin width);
//   * snapshots()       output.cpp:1541-1648 (the fields and, with SNAPSHOTS_ENERGY,
//     the lattice energy densities: kinetic_energy_lattice / gradient_energy_lattice
//     evolution.cpp:7-138, potential and total output.cpp:1614-1627), written as the
//     reference's HDF5 file by the host writer in psc_h5.cpp.
// The real-space fields come from the c2r of the state (the reference's isChanged
// block, output.cpp:1219-1240 / 1555-1578); the gradients are c2r's of i kIR k_a f_k
// with that axis' Nyquist bin zeroed, which is what the reference's 1-D r2c, multiply
// and c2r along each axis compute (evolution.cpp:34-127).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "psc_dev.cuh"
#include "psc_h5.h"
#include "psc_handle.h"

namespace psc {
namespace {

constexpr int kOutBlocks = 4 * 152;
constexpr int kOutThreads = 256;

// out = i kIR k_axis f_k, k_axis the signed wavenumber along axis (0 = x, 1 = y,
// 2 = z), zero on that axis' Nyquist bin (evolution.cpp:47-56, 79-88, 107-116)
template <typename T>
__global__ void __launch_bounds__(kOutThreads) k_deriv_axis(const cplx<T> *__restrict__ fk, cplx<T> *__restrict__ out,
                                                            int N, int H, long long modes, int axis, double kIR) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < modes; m += stride) {
        int n;
        if (axis == 2) {
            n = (int)(m % H);
        } else if (axis == 1) {
            n = (int)((m / H) % N);
        } else {
            n = (int)(m / ((long long)N * H));
        }
        const int kap = (n == N / 2) ? 0 : (n < N / 2 ? n : n - N);
        const T s = (T)(kIR * kap);
        const cplx<T> v = fk[m];
        out[m] = mk<T>(-s * v.y, s * v.x);
    }
}

// potential energy density per site (output.cpp:1618-1625): the sum over the model's
// terms of potential_energy(term, f(x)); tot = pot
template <typename T>
__global__ void __launch_bounds__(kOutThreads) k_snap_pot(const T *__restrict__ real, double *__restrict__ pot,
                                                          double *__restrict__ tot, long long sites, int model,
                                                          double gsq, int nf) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int nt = model_nterms(model);
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < sites; s += stride) {
        double v = 0.0;
        if (model_is_user(model)) {
            double f[kMaxFields] = {};
            for (int q = 0; q < nf; ++q) f[q] = (double)real[q * sites + s];
            for (int t = 0; t < nt; ++t) v += model_potential_term(model, gsq, t, f);
        } else {
            const double phi = (double)real[s];
            v += 0.5 * (phi * phi);
            if (model == PSC_MODEL_PHI2CHI2) {
                const double chi = (double)real[sites + s];
                v += 0.5 * gsq * (phi * phi) * (chi * chi);
            }
        }
        pot[s] = v;
        tot[s] = v;
    }
}

// kinetic energy density (evolution.cpp:7-19): norm * sum_f pi_f(x)^2; tot += it
template <typename T>
__global__ void __launch_bounds__(kOutThreads) k_snap_kin(const T *__restrict__ real, double *__restrict__ kin,
                                                          double *__restrict__ tot, long long sites, int nf,
                                                          double norm) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < sites; s += stride) {
        double k = 0.0;
        for (int f = 0; f < nf; ++f) {
            const double p = (double)real[(long long)f * sites + s];
            k += p * p;
        }
        k *= norm;
        kin[s] = k;
        tot[s] += k;
    }
}

// gradient energy density (evolution.cpp:23-138): grad += (d_a f)^2 for one field and
// axis (first: grad = ...); the final call scales by norm and adds to tot
template <typename T>
__global__ void __launch_bounds__(kOutThreads) k_snap_grad(const T *__restrict__ d, double *__restrict__ grad,
                                                           double *__restrict__ tot, long long sites, int first,
                                                           int last, double norm) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < sites; s += stride) {
        const double x = (double)d[s];
        double g = first ? 0.0 : grad[s];
        g += x * x;
        if (last) {
            g *= norm;
            tot[s] += g;
        }
        grad[s] = g;
    }
}

// block partial minimum and maximum of x[0..n) (output.cpp:1250-1256)
template <typename T>
__global__ void __launch_bounds__(kOutThreads) k_minmax(const T *__restrict__ x, long long n, double *__restrict__ part) {
    __shared__ double smin[kOutThreads / 32], smax[kOutThreads / 32];
    double lo = (double)x[0], hi = lo;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double v = (double)x[i];
        lo = v < lo ? v : lo;
        hi = v > hi ? v : hi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double a = __shfl_xor_sync(0xffffffffu, lo, o), b = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        smin[w] = lo;
        smax[w] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
            lo = smin[i] < lo ? smin[i] : lo;
            hi = smax[i] > hi ? smax[i] : hi;
        }
        part[2 * blockIdx.x] = lo;
        part[2 * blockIdx.x + 1] = hi;
    }
}

// bin counts of x[0..n) over [bmin, bmax] in nbins bins (output.cpp:1244-1279):
// binnum = (int)((x - bmin) / df), x == bmax in the last bin, values whose bin falls
// outside [0, nbins) not counted. With auto_range the limits are the minimum and
// maximum of the block partials. edges = {bmin, df}.
template <typename T>
__global__ void __launch_bounds__(kOutThreads) k_hist(const T *__restrict__ x, long long n,
                                                      const double *__restrict__ part, int nparts, int auto_range,
                                                      double hmin, double hmax, int nbins,
                                                      unsigned *__restrict__ counts, double *__restrict__ edges) {
    extern __shared__ unsigned sc[];
    __shared__ double lim[2];
    if (threadIdx.x == 0) {
        double lo = hmin, hi = hmax;
        if (auto_range) {
            lo = part[0];
            hi = part[1];
            for (int i = 1; i < nparts; ++i) {
                lo = part[2 * i] < lo ? part[2 * i] : lo;
                hi = part[2 * i + 1] > hi ? part[2 * i + 1] : hi;
            }
        }
        lim[0] = lo;
        lim[1] = hi;
        if (blockIdx.x == 0) {
            edges[0] = lo;
            edges[1] = (hi - lo) / (double)nbins;
        }
    }
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) sc[i] = 0u;
    __syncthreads();
    const double bmin = lim[0], bmax = lim[1];
    const double df = (bmax - bmin) / (double)nbins;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double v = (double)x[i];
        int bin;
        if (v == bmax) {
            bin = nbins - 1;
        } else {
            const double q = (v - bmin) / df;
            if (q != q) continue;           // NaN: no bin
            bin = __double2int_rz(q);       // truncation toward zero; saturates out of range
        }
        if (bin >= 0 && bin < nbins) atomicAdd(&sc[bin], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nbins; i += blockDim.x)
        if (sc[i]) atomicAdd(&counts[i], sc[i]);
}

// 2-D histogram of a field pair (output.cpp:1369-1410): both bin indices as the 1-D
// histogram computes them; lim = {bmin0, bmax0, bmin1, bmax1}
template <typename T>
__global__ void __launch_bounds__(kOutThreads) k_hist2d(const T *__restrict__ x, const T *__restrict__ y, long long n,
                                                        const double *__restrict__ lim, int nb0, int nb1,
                                                        unsigned *__restrict__ counts) {
    extern __shared__ unsigned sc2[];
    const int nb = nb0 * nb1;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) sc2[i] = 0u;
    __syncthreads();
    const double b0 = lim[0], e0 = lim[1], b1 = lim[2], e1 = lim[3];
    const double d0 = (e0 - b0) / (double)nb0, d1 = (e1 - b1) / (double)nb1;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double u = (double)x[i], v = (double)y[i];
        int i0, i1;
        if (u == e0) {
            i0 = nb0 - 1;
        } else {
            const double q = (u - b0) / d0;
            if (q != q) continue;
            i0 = __double2int_rz(q);
        }
        if (v == e1) {
            i1 = nb1 - 1;
        } else {
            const double q = (v - b1) / d1;
            if (q != q) continue;
            i1 = __double2int_rz(q);
        }
        if (i0 >= 0 && i0 < nb0 && i1 >= 0 && i1 < nb1) atomicAdd(&sc2[i0 * nb1 + i1], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
        if (sc2[i]) atomicAdd(&counts[i], sc2[i]);
}

// the global minimum and maximum of the block partials of k_minmax into lim[0], lim[1]
__global__ void k_minmax_final(const double *__restrict__ part, int nparts, double *__restrict__ lim) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double lo = part[0], hi = part[1];
    for (int i = 1; i < nparts; ++i) {
        lo = part[2 * i] < lo ? part[2 * i] : lo;
        hi = part[2 * i + 1] > hi ? part[2 * i + 1] : hi;
    }
    lim[0] = lo;
    lim[1] = hi;
}

// slices() (output.cpp:1456-1534): output value o of a dim-dimensional slice with side
// `side` points (every skip-th site from the origin), each the mean of its skip block when
// average != 0 (sequential sum in the reference's loop order; 3-D multiplies by 1/n)
template <typename T>
__global__ void __launch_bounds__(kOutThreads) k_slices(const T *__restrict__ f, int N, int dim, int side, int skip,
                                                        int average, double *__restrict__ out) {
    long long total = side;
    for (int d = 1; d < dim; ++d) total *= side;
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= total) return;
    int c[3] = {0, 0, 0};   // x, y, z start of the block
    long long r = o;
    for (int d = 2; d >= 3 - dim; --d) {
        c[d] = (int)(r % side) * skip;
        r /= side;
    }
    const size_t NN = (size_t)N;
    double v;
    if (average) {
        v = 0.0;
        int n = 0;
        const int xe = dim == 3 ? min(c[0] + skip, N) : 1, ye = dim >= 2 ? min(c[1] + skip, N) : 1;
        const int ze = min(c[2] + skip, N);
        for (int x = c[0]; x < xe; ++x)
            for (int y = c[1]; y < ye; ++y)
                for (int z = c[2]; z < ze; ++z) {
                    v += (double)f[((size_t)x * NN + y) * NN + z];
                    ++n;
                }
        v = dim == 3 ? v * (1 / (double)n) : v / (double)n;
    } else {
        v = (double)f[((size_t)c[0] * NN + c[1]) * NN + c[2]];
    }
    out[o] = v;
}

template <typename T>
cudaError_t launch_deriv(const Geo &g, const void *fk, void *out, int axis, cudaStream_t st) {
    k_deriv_axis<T><<<kOutBlocks, kOutThreads, 0, st>>>((const cplx<T> *)fk, (cplx<T> *)out, g.N, g.H, g.modes, axis,
                                                         g.kIR);
    return cudaGetLastError();
}

}  // namespace

namespace hapi {

#define CU(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return fail(e_ == cudaErrorMemoryAllocation ? PSC_ERR_NOMEM : PSC_ERR_CUDA,                  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                             \
    } while (0)

namespace {

int ensure_real(psc_handle *h) {
    const Geo &g = h->cfg.g;
    if (h->b.real) return PSC_OK;
    return dalloc(h, &h->b.real, (size_t)g.sites * g.nf * (h->csize / 2));
}

// c2r of nsrc arrays of realization r into h->b.real
int to_real(psc_handle *h, int r, const void *src, int nsrc) {
    int rc = ensure_real(h);
    if (rc) return rc;
    const Buffers b1 = buffers_of(h, r);
    CU(launch_c2r_real(single_cfg(h), b1, h->p0().precision, src, nsrc, h->st));
    return PSC_OK;
}

template <typename T>
int histograms_t(psc_handle *h, int r, int nbins, double hmin, double hmax, double *binfreq, double *bmin,
                 double *df) {
    const Geo &g = h->cfg.g;
    const Buffers b1 = buffers_of(h, r);
    int rc = to_real(h, r, b1.fk, g.nf);
    if (rc) return rc;
    // device scratch: block partials and the two edges (doubles, 8-byte aligned) first,
    // then the nbins 4-byte counters
    const size_t part_b = 2 * kOutBlocks * sizeof(double), edge_b = 2 * sizeof(double);
    const size_t cnt_b = (size_t)nbins * sizeof(unsigned);
    void *scratch = nullptr;
    CU(cudaMallocAsync(&scratch, part_b + edge_b + cnt_b, h->st));
    double *part = static_cast<double *>(scratch);
    double *edges = part + 2 * kOutBlocks;
    unsigned *cnt = reinterpret_cast<unsigned *>(static_cast<char *>(scratch) + part_b + edge_b);
    std::vector<unsigned> hc((size_t)nbins);
    double he[2];
    const int auto_range = (hmin == hmax);
    cudaError_t e = cudaSuccess;
    if (cnt_b > 48 * 1024)
        e = cudaFuncSetAttribute(k_hist<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cnt_b);
    for (int f = 0; f < g.nf && e == cudaSuccess; ++f) {
        const T *x = static_cast<const T *>(h->b.real) + (long long)f * g.sites;
        if (auto_range) k_minmax<T><<<kOutBlocks, kOutThreads, 0, h->st>>>(x, g.sites, part);
        if ((e = cudaMemsetAsync(cnt, 0, cnt_b, h->st)) != cudaSuccess) break;
        k_hist<T><<<kOutBlocks, kOutThreads, cnt_b, h->st>>>(x, g.sites, part, kOutBlocks, auto_range, hmin, hmax,
                                                            nbins, cnt, edges);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(hc.data(), cnt, cnt_b, cudaMemcpyDeviceToHost, h->st)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(he, edges, sizeof he, cudaMemcpyDeviceToHost, h->st)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(h->st)) != cudaSuccess) break;
        unsigned long long numpts = 0;
        for (unsigned c : hc) numpts += c;
        if (binfreq)
            for (int i = 0; i < nbins; ++i) binfreq[(size_t)f * nbins + i] = (double)hc[i] / (double)numpts;
        if (bmin) bmin[f] = he[0];
        if (df) df[f] = he[1];
    }
    cudaFreeAsync(scratch, h->st);
    CU(e);
    CU(cudaStreamSynchronize(h->st));
    return PSC_OK;
}

template <typename T>
int histograms2d_t(psc_handle *h, int r, int f1, int f2, int nb0, int nb1, double hmin, double hmax, double *binfreq,
                   double *bmin, double *df) {
    const Geo &g = h->cfg.g;
    const Buffers b1 = buffers_of(h, r);
    int rc = to_real(h, r, b1.fk, g.nf);
    if (rc) return rc;
    const size_t part_b = 2 * kOutBlocks * sizeof(double), lim_b = 4 * sizeof(double);
    const size_t cnt_b = (size_t)nb0 * nb1 * sizeof(unsigned);
    void *scratch = nullptr;
    CU(cudaMallocAsync(&scratch, part_b + lim_b + cnt_b, h->st));
    double *part = static_cast<double *>(scratch);
    double *lim = part + 2 * kOutBlocks;
    unsigned *cnt = reinterpret_cast<unsigned *>(static_cast<char *>(scratch) + part_b + lim_b);
    const T *x = static_cast<const T *>(h->b.real) + (long long)f1 * g.sites;
    const T *y = static_cast<const T *>(h->b.real) + (long long)f2 * g.sites;
    cudaError_t e = cudaSuccess;
    if (hmin == hmax) {
        k_minmax<T><<<kOutBlocks, kOutThreads, 0, h->st>>>(x, g.sites, part);
        k_minmax_final<<<1, 32, 0, h->st>>>(part, kOutBlocks, lim);
        k_minmax<T><<<kOutBlocks, kOutThreads, 0, h->st>>>(y, g.sites, part);
        k_minmax_final<<<1, 32, 0, h->st>>>(part, kOutBlocks, lim + 2);
    } else {
        const double l[4] = {hmin, hmax, hmin, hmax};
        e = cudaMemcpyAsync(lim, l, sizeof l, cudaMemcpyHostToDevice, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, cnt_b, h->st);
    if (e == cudaSuccess && cnt_b > 48 * 1024)
        e = cudaFuncSetAttribute(k_hist2d<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cnt_b);
    std::vector<unsigned> hc((size_t)nb0 * nb1);
    double hl[4];
    if (e == cudaSuccess) {
        k_hist2d<T><<<kOutBlocks, kOutThreads, cnt_b, h->st>>>(x, y, g.sites, lim, nb0, nb1, cnt);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), cnt, cnt_b, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hl, lim, sizeof hl, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    cudaFreeAsync(scratch, h->st);
    CU(e);
    // binfreq / N^3 (output.cpp:1407), df = (bmax - bmin) / nbins
    const double n3 = (double)g.sites;
    if (binfreq)
        for (size_t i = 0; i < hc.size(); ++i) binfreq[i] = (double)hc[i] / n3;
    if (bmin) {
        bmin[0] = hl[0];
        bmin[1] = hl[2];
    }
    if (df) {
        df[0] = (hl[1] - hl[0]) / (double)nb0;
        df[1] = (hl[3] - hl[2]) / (double)nb1;
    }
    return PSC_OK;
}

template <typename T>
int slices_t(psc_handle *h, int r, int dim, int length, int skip, int average, double *out, long long count) {
    const Geo &g = h->cfg.g;
    const Buffers b1 = buffers_of(h, r);
    int rc = to_real(h, r, b1.fk, g.nf);
    if (rc) return rc;
    const int N = g.N;
    const int fin = std::min((long long)length * skip, (long long)N) > 0 ? (int)std::min((long long)length * skip,
                                                                                         (long long)N)
                                                                       : 0;
    const int side = (fin + skip - 1) / skip;
    double *dout = nullptr;
    CU(cudaMallocAsync(reinterpret_cast<void **>(&dout), (size_t)count * g.nf * sizeof(double), h->st));
    cudaError_t e = cudaSuccess;
    for (int f = 0; f < g.nf && e == cudaSuccess; ++f) {
        const T *x = static_cast<const T *>(h->b.real) + (long long)f * g.sites;
        const unsigned blocks = (unsigned)((count + kOutThreads - 1) / kOutThreads);
        k_slices<T><<<blocks, kOutThreads, 0, h->st>>>(x, N, dim, side, skip, average, dout + (size_t)f * count);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, dout, (size_t)count * g.nf * sizeof(double), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    cudaFreeAsync(dout, h->st);
    CU(e);
    return PSC_OK;
}

// Runs the snapshot datasets through `sink(name, device_or_host_data)`: the fields
// (host arrays, converted to FP64) and, with energy, the four densities (device FP64).
struct Sink {
    virtual int fields(const double *host_f) = 0;            // [nf][sites]
    virtual int energy(int which, const double *dev) = 0;    // 0 pot, 1 kin, 2 grad, 3 tot
    virtual ~Sink() {}
};

template <typename T>
int snapshot_t(psc_handle *h, int r, int want_fields, int with_energy, Sink &sink) {
    const Geo &g = h->cfg.g;
    const Buffers b1 = buffers_of(h, r);
    int rc;
    DevBG bg;
    if ((rc = read_bg(h, r, &bg))) return rc;
    if ((rc = to_real(h, r, b1.fk, g.nf))) return rc;
    if (want_fields) {
        std::vector<double> hf((size_t)g.sites * g.nf);
        if ((rc = download_real(h, hf.data(), h->b.real, hf.size()))) return rc;
        if ((rc = sink.fields(hf.data()))) return rc;
    }
    if (!with_energy) return PSC_OK;
    double *work = nullptr, *tot = nullptr;
    const size_t bytes = (size_t)g.sites * sizeof(double);
    CU(cudaMallocAsync(reinterpret_cast<void **>(&work), 2 * bytes, h->st));
    tot = work + g.sites;
    auto run = [&]() -> int {
        const T *real = static_cast<const T *>(h->b.real);
        k_snap_pot<T><<<kOutBlocks, kOutThreads, 0, h->st>>>(real, work, tot, g.sites, g.model, g.gsq, g.nf);
        CU(cudaGetLastError());
        int rc2 = sink.energy(0, work);
        if (rc2) return rc2;
        if ((rc2 = to_real(h, r, b1.pk, g.nf))) return rc2;
        // kinetic_energy_lattice: pow(a, 6) / 2 (evolution.cpp:9)
        k_snap_kin<T><<<kOutBlocks, kOutThreads, 0, h->st>>>(real, work, tot, g.sites, g.nf, std::pow(bg.a, 6) / 2.);
        CU(cudaGetLastError());
        if ((rc2 = sink.energy(1, work))) return rc2;
        // gradient_energy_lattice: field by field, axes x, y, z; pw2(a) / 2 (evolution.cpp:133)
        const double gnorm = bg.a * bg.a / 2.;
        for (int f = 0; f < g.nf; ++f)
            for (int ax = 0; ax < 3; ++ax) {
                const void *src = static_cast<const char *>(b1.fk) + (size_t)f * g.modes * h->csize;
                CU(launch_deriv<T>(g, src, b1.QV, ax, h->st));
                if ((rc2 = to_real(h, r, b1.QV, 1))) return rc2;
                const int first = (f == 0 && ax == 0), last = (f == g.nf - 1 && ax == 2);
                k_snap_grad<T><<<kOutBlocks, kOutThreads, 0, h->st>>>(real, work, tot, g.sites, first, last, gnorm);
                CU(cudaGetLastError());
            }
        if ((rc2 = sink.energy(2, work))) return rc2;
        return sink.energy(3, tot);
    };
    rc = run();
    cudaFreeAsync(work, h->st);
    if (rc) return rc;
    CU(cudaStreamSynchronize(h->st));
    return PSC_OK;
}

struct ArraySink : Sink {
    psc_handle *h;
    size_t n, nf;
    double *f, *out[4];
    int fields(const double *hf) override {
        if (f) std::copy(hf, hf + n * nf, f);
        return PSC_OK;
    }
    int energy(int which, const double *dev) override {
        if (!out[which]) return PSC_OK;
        CU(cudaMemcpyAsync(out[which], dev, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        CU(cudaStreamSynchronize(h->st));
        return PSC_OK;
    }
};

struct FileSink : Sink {
    psc_handle *h;
    size_t n, nf;
    h5::Writer *w;
    std::vector<double> host;
    int fields(const double *hf) override {
        for (size_t f = 0; f < nf; ++f)
            if (w->write((int)f, hf + f * n)) return fail(PSC_ERR_IO, w->error());
        return PSC_OK;
    }
    int energy(int which, const double *dev) override {
        host.resize(n);
        CU(cudaMemcpyAsync(host.data(), dev, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        CU(cudaStreamSynchronize(h->st));
        if (w->write((int)(nf + which), host.data())) return fail(PSC_ERR_IO, w->error());
        return PSC_OK;
    }
};

}  // namespace

int histograms(psc_handle *h, int r, int nbins, double hmin, double hmax, double *binfreq, double *bmin,
               double *df) {
    if (nbins < 1 || nbins > 16384) return fail(PSC_ERR_ARG, "nbins must be in [1, 16384]");
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state");
    return h->p0().precision == 32 ? histograms_t<float>(h, r, nbins, hmin, hmax, binfreq, bmin, df)
                                   : histograms_t<double>(h, r, nbins, hmin, hmax, binfreq, bmin, df);
}

int histograms2d(psc_handle *h, int r, int f1, int f2, int nb0, int nb1, double hmin, double hmax, double *binfreq,
                 double *bmin, double *df) {
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state");
    const int nf = h->cfg.g.nf;
    if (f1 < 0 || f1 >= nf || f2 < 0 || f2 >= nf) return fail(PSC_ERR_ARG, "field index out of range");
    if (nb0 < 1 || nb1 < 1 || (long long)nb0 * nb1 > 16384) return fail(PSC_ERR_ARG, "nbins0 * nbins1 must be in [1, 16384]");
    return h->p0().precision == 32 ? histograms2d_t<float>(h, r, f1, f2, nb0, nb1, hmin, hmax, binfreq, bmin, df)
                                   : histograms2d_t<double>(h, r, f1, f2, nb0, nb1, hmin, hmax, binfreq, bmin, df);
}

long long slice_count(int N, int dim, int length, int skip) {
    if (dim < 1 || length < 1 || skip < 1) return -1;
    if (dim > 3) dim = 3;
    const long long fin = std::min((long long)length * skip, (long long)N);
    const long long side = (fin + skip - 1) / skip;
    long long c = side;
    for (int d = 1; d < dim; ++d) c *= side;
    return c;
}

int slices(psc_handle *h, int r, int dim, int length, int skip, int average, double *out, long long *count) {
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state");
    const long long c = slice_count(h->cfg.g.N, dim, length, skip);
    if (c < 0) return fail(PSC_ERR_ARG, "slicedim, slicelength and sliceskip must be positive");
    if (count) *count = c;
    if (!out) return PSC_OK;
    if (dim > 3) dim = 3;
    return h->p0().precision == 32 ? slices_t<float>(h, r, dim, length, skip, average, out, c)
                                   : slices_t<double>(h, r, dim, length, skip, average, out, c);
}

int snapshot_arrays(psc_handle *h, int r, double *f, double *pot, double *kin, double *grad, double *tot) {
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state");
    const Geo &g = h->cfg.g;
    ArraySink s;
    s.h = h;
    s.n = (size_t)g.sites;
    s.nf = (size_t)g.nf;
    s.f = f;
    s.out[0] = pot;
    s.out[1] = kin;
    s.out[2] = grad;
    s.out[3] = tot;
    const int energy = pot || kin || grad || tot;
    return h->p0().precision == 32 ? snapshot_t<float>(h, r, f != nullptr, energy, s)
                                   : snapshot_t<double>(h, r, f != nullptr, energy, s);
}

int write_snapshot(psc_handle *h, int r, const char *path, int with_energy) {
    if (!path) return fail(PSC_ERR_ARG, "null path");
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state");
    const Geo &g = h->cfg.g;
    // dataset names of snapshots() (output.cpp:1581-1593)
    std::vector<std::string> names;
    for (int f = 0; f < g.nf; ++f) names.push_back("/ScalarField_" + std::to_string(f));
    if (with_energy)
        for (const char *e : {"/PotentialEnergy", "/KineticEnergy", "/GradientEnergy", "/TotalEnergy"})
            names.push_back(e);
    h5::Writer w;
    const uint64_t N = (uint64_t)g.N;
    if (w.open(path, names, {N, N, N})) return fail(PSC_ERR_IO, w.error());
    FileSink s;
    s.h = h;
    s.n = (size_t)g.sites;
    s.nf = (size_t)g.nf;
    s.w = &w;
    const int rc = h->p0().precision == 32 ? snapshot_t<float>(h, r, 1, with_energy, s)
                                           : snapshot_t<double>(h, r, 1, with_energy, s);
    if (rc) return rc;
    if (w.close()) return fail(PSC_ERR_IO, w.error());
    return PSC_OK;
}

// Checkpoint file (HDF5, the library's writer): f_k, pi_k [nflds][modes][2] and with GWs
// u_k, pi_u_k [6][modes][2] in the layout of psc_get_state, background = {t, a, a', a''},
// lattice = {N, nflds, with_gw, spectral, N_pad, vv, model, precision}.
int checkpoint_write(psc_handle *h, int r, const char *path) {
    if (!path) return fail(PSC_ERR_ARG, "null path");
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state");
    const Geo &g = h->cfg.g;
    const psc_params &q = h->p[r];
    const uint64_t n = (uint64_t)g.modes, nf = (uint64_t)g.nf;
    std::vector<double> fk(2 * n * nf), pk(2 * n * nf), uk, puk;
    if (g.gw) {
        uk.resize(2 * n * 6);
        puk.resize(2 * n * 6);
    }
    double bgv[4];
    int rc = get_state(h, r, fk.data(), pk.data(), bgv + 1, bgv + 2, bgv + 3, g.gw ? uk.data() : nullptr,
                       g.gw ? puk.data() : nullptr);
    if (rc) return rc;
    DevBG bg;
    if ((rc = read_bg(h, r, &bg))) return rc;
    bgv[0] = bg.t;
    const double lat[8] = {(double)q.N, (double)q.nflds, (double)q.with_gw, (double)q.spectral, (double)q.N_pad,
                           (double)q.vv, (double)q.model, (double)q.precision};
    std::vector<std::string> names = {"/f_k", "/pi_k", "/background", "/lattice"};
    std::vector<std::vector<uint64_t>> shapes = {{nf, n, 2}, {nf, n, 2}, {4}, {8}};
    std::vector<const double *> data = {fk.data(), pk.data(), bgv, lat};
    if (g.gw) {
        names.push_back("/u_k");
        names.push_back("/pi_u_k");
        shapes.push_back({6, n, 2});
        shapes.push_back({6, n, 2});
        data.push_back(uk.data());
        data.push_back(puk.data());
    }
    h5::Writer w;
    if (w.open(path, names, shapes)) return fail(PSC_ERR_IO, w.error());
    for (size_t i = 0; i < data.size(); ++i)
        if (w.write((int)i, data[i])) return fail(PSC_ERR_IO, w.error());
    if (w.close()) return fail(PSC_ERR_IO, w.error());
    return PSC_OK;
}

int checkpoint_read(psc_handle *h, int r, const char *path) {
    if (!path) return fail(PSC_ERR_ARG, "null path");
    const Geo &g = h->cfg.g;
    const psc_params &q = h->p[r];
    h5::Reader rd;
    if (rd.open(path)) return fail(PSC_ERR_IO, rd.error());
    double lat[8], bgv[4];
    if (rd.read("/lattice", lat, 8) || rd.read("/background", bgv, 4)) return fail(PSC_ERR_IO, rd.error());
    if ((int)lat[0] != q.N || (int)lat[1] != q.nflds || (int)lat[2] != q.with_gw)
        return fail(PSC_ERR_CONFIG, "checkpoint of another lattice (N, nflds or with_gw differ)");
    const size_t n = (size_t)g.modes;
    std::vector<double> fk(2 * n * g.nf), pk(2 * n * g.nf), uk, puk;
    if (rd.read("/f_k", fk.data(), fk.size()) || rd.read("/pi_k", pk.data(), pk.size()))
        return fail(PSC_ERR_IO, rd.error());
    if (g.gw) {
        uk.resize(2 * n * 6);
        puk.resize(2 * n * 6);
        if (rd.read("/u_k", uk.data(), uk.size()) || rd.read("/pi_u_k", puk.data(), puk.size()))
            return fail(PSC_ERR_IO, rd.error());
    }
    int rc = set_state(h, r, fk.data(), pk.data(), bgv[1], bgv[2], bgv[3], g.gw ? uk.data() : nullptr,
                       g.gw ? puk.data() : nullptr);
    if (rc) return rc;
    DevBG bg;
    if ((rc = read_bg(h, r, &bg))) return rc;
    bg.t = bgv[0];
    return write_bg(h, r, bg);
}

}  // namespace hapi
}  // namespace psc

using namespace psc::hapi;

extern "C" {

int psc_histograms(psc_handle *h, int nbins, double hmin, double hmax, double *binfreq, double *bmin, double *df) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return histograms(h, 0, nbins, hmin, hmax, binfreq, bmin, df);
}

int psc_histograms_2d(psc_handle *h, int fld1, int fld2, int nbins0, int nbins1, double hmin, double hmax,
                      double *binfreq, double *bmin, double *df) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return histograms2d(h, 0, fld1, fld2, nbins0, nbins1, hmin, hmax, binfreq, bmin, df);
}

int psc_slices(psc_handle *h, int slicedim, int slicelength, int sliceskip, int sliceaverage, double *out,
               long long *count) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return slices(h, 0, slicedim, slicelength, sliceskip, sliceaverage, out, count);
}

int psc_snapshot_arrays(psc_handle *h, double *f, double *pot, double *kin, double *grad, double *tot) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return snapshot_arrays(h, 0, f, pot, kin, grad, tot);
}

int psc_write_snapshot(psc_handle *h, const char *path, int with_energy) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return write_snapshot(h, 0, path, with_energy);
}

int psc_time_c2r(psc_handle *h, int reps, float *ms) {
    if (!h || !ms || reps < 1) return fail(PSC_ERR_ARG, "bad arguments");
    if (!h->have_state) return fail(PSC_ERR_STATE, "no state");
    const psc::Buffers b1 = buffers_of(h, 0);
    int rc = to_real(h, 0, b1.fk, h->cfg.g.nf);   // warm-up (and allocation of the real buffer)
    if (rc) return rc;
    CU(cudaEventRecord(h->ev0, h->st));
    for (int i = 0; i < reps; ++i)
        if ((rc = to_real(h, 0, b1.fk, h->cfg.g.nf))) return rc;
    CU(cudaEventRecord(h->ev1, h->st));
    CU(cudaEventSynchronize(h->ev1));
    float t = 0.f;
    CU(cudaEventElapsedTime(&t, h->ev0, h->ev1));
    *ms = t / (float)reps;
    return PSC_OK;
}

int psc_checkpoint_write(psc_handle *h, const char *path) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return checkpoint_write(h, 0, path);
}

int psc_checkpoint_read(psc_handle *h, const char *path) {
    if (!h) return fail(PSC_ERR_ARG, "null handle");
    return checkpoint_read(h, 0, path);
}

int psc_h5_write_f64(const char *path, int n, const char *const *names, const double *const *data, int rank,
                     const uint64_t *dims) {
    if (!path || n < 1 || !names || !data || rank < 1 || !dims) return fail(PSC_ERR_ARG, "bad arguments");
    std::vector<std::string> nm;
    for (int i = 0; i < n; ++i) {
        if (!names[i] || !data[i]) return fail(PSC_ERR_ARG, "null dataset name or data");
        nm.push_back(names[i]);
    }
    psc::h5::Writer w;
    if (w.open(path, nm, std::vector<uint64_t>(dims, dims + rank))) return fail(PSC_ERR_IO, w.error());
    for (int i = 0; i < n; ++i)
        if (w.write(i, data[i])) return fail(PSC_ERR_IO, w.error());
    if (w.close()) return fail(PSC_ERR_IO, w.error());
    return PSC_OK;
}

int psc_h5_dataset_shape(const char *path, const char *name, uint64_t *dims, int maxrank, int *rank) {
    if (!path || !name || !rank || (maxrank > 0 && !dims)) return fail(PSC_ERR_ARG, "bad arguments");
    psc::h5::Reader rd;
    std::vector<uint64_t> d;
    if (rd.open(path) || rd.shape(name, &d)) return fail(PSC_ERR_IO, rd.error());
    *rank = (int)d.size();
    for (int i = 0; i < maxrank && i < (int)d.size(); ++i) dims[i] = d[i];
    return PSC_OK;
}

int psc_h5_read_f64(const char *path, const char *name, double *out, uint64_t count) {
    if (!path || !name || !out) return fail(PSC_ERR_ARG, "bad arguments");
    psc::h5::Reader rd;
    if (rd.open(path) || rd.read(name, out, (size_t)count)) return fail(PSC_ERR_IO, rd.error());
    return PSC_OK;
}

}  // extern "C"
