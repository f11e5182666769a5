// psc_launch.h — host-side interface between the C-ABI layer (psc_api.cpp) and
// the CUDA kernels (psc_kernels.cu). No CUDA C++ device code here.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/psc.h"

namespace psc {

struct DevBG;
struct DevAdj;
struct XTma;
struct YTma;

// Lattice geometry and tiling, passed by value to every pass kernel.
struct Geo {
    int N, H, M;                 // edge, half-spectrum length N/2+1, N/2
    int nf, gw, nterms, mask;    // fields, GW tensors held, potential terms, R_Q2C mask on
    int gwev;                    // the step evolves the GW tensors (the real-space path; on the
                                 // spectral path they stay as initialised, as in the reference)
    int model;                   // PSC_MODEL_*
    int reg;                     // 1: register-engine passes (N >= 32), 0: generic shared-memory engine
    int tlx_shift, tlz_shift;    // log2 lines per tile: X/Y passes, Z pass
    int ldz;                     // shared-memory leading dimension of the Z pass (lines + 1)
    int lines_x;                 // N * H  (X-pass and Y-pass line count per array)
    int lines_z;                 // N * N  (Z-pass line count)
    long long modes, sites;
    double gsq, kIR;
    // batches of R same-configuration lattices: realization r = blockIdx.z owns
    // the arrays at r * fstride (field-sized) / r * gstride (GW-sized), the
    // background record bg[r] and the partial sums at r * pkg_stride / r * pv_stride.
    long long fstride, gstride;
    int pkg_stride, pv_stride;
};

// Tile and grid shapes of the register-engine passes that the autotuner (psc_autotune)
// chooses among; -1 / 0 = the planner's default. xy_shift: log2 lines per tile of the X and Y
// passes (at most the default, which fills the passes' block size); z_shift: log2 lines per
// tile of the Z pass (at most the default); z_per_sm: resident blocks per SM of the persistent
// Z passes (1 .. the kernel's launch-bound minimum).
struct TileChoice {
    int xy_shift = -1, z_shift = -1, z_per_sm = 0;
};

struct LaunchCfg {
    Geo g;
    TileChoice tc;               // the shapes in use (defaults resolved)
    int R;                       // realizations advanced together (1 for a single lattice)
    int thr_xy, thr_z;           // threads per block
    size_t smem_xy, smem_z;      // dynamic shared memory bytes
    size_t smem_xf;              // X forward + kick pass (exchange tile + two prefetched operand tiles)
    size_t smem_xi;              // X inverse pass with tensor-map staging (exchange tile + f_k and pi tiles)
    size_t smem_ys;              // one array's tile of a Y pass staged by tensor copies (even + odd rows)
    int nbx;                     // blocks of the X / Y passes (per array)
    int nbz;                     // blocks of the Z pass
    int sms = 0;                 // SMs of the device (the persistent passes' waves)
};

// Device buffers of one lattice. Complex arrays hold cplx<T> of the handle's
// precision (T = float for 32, double for 64).
struct Buffers {
    void *fk, *pk;               // [nf][modes]   f_k, pi_k (pi_half between the stages of a step)
    void *uk, *puk;              // [6][modes]    u_k, pi_u_k (GW)
    void *TA, *TB, *TC;          // [nf][modes]   inverse-transform intermediates (f, d/dx f, d/dy f)
    void *QV, *QS;               // [nf][modes], [6][modes]   forward-transform intermediates (V', S_ab)
    void *tw;                    // [N] e^{-2 pi i q/N}
    void *real;                  // [nf][sites] real-space output buffer (optional)
    double *partKG;              // [2 nf][nbx]   block partial sums of K and G
    double *partV;               // [nterms][nbz] block partial sums of V
    double *spec;                // spectra accumulators
    int *spec_cnt;
    DevBG *bg;
    // forward tape of the adjoint (single lattice; null otherwise): the stage-point
    // state f, pi (synchronised), V'_k and the real fields f(x); with GWs also pi_u
    // (synchronised) and -kIR^2 k^2 u + S_k (the GW force without its a^(1+alpha))
    void *tape_f, *tape_p, *tape_vp, *tape_fx, *tape_pu, *tape_fu;
    // the force of the last synchronising kick (c_open = 0), per mode: F of the fields
    // [nf][modes] and a^(1+alpha)(-k^2 u + S) of the GW [6][modes]. The opening half kick of
    // the next step call uses it instead of a force evaluation (null: not kept)
    void *Fk, *Fu;
    const XTma *xtma;            // host copy of the kick operands' tensor maps (null: cp.async staging)
    const YTma *ytma;            // the Y forward pass's tensor maps (V', S_ab); null: direct loads
    const YTma *ytma_i;          // the GW Y inverse pass's tensor maps (TA, TB); null: direct loads
};

// Tensor maps of the X passes' tiles (TMA): f_k, pi_k, QV as {lines, x, field, realization}
// and u_k, pi_u_k, QS as {lines, x, component, realization}, in 8-byte elements, box {lines
// per tile, min(N, 256), 1, 1} (N/256 boxes per tile above 256). on = 0: the pass stages its
// operands by cp.async instead (batched launches, the generic engine, or no tensor-map
// encoder).
struct XTma {
    CUtensorMap fk, pk, uk, puk;
    CUtensorMap qv, qs;   // the forward passes' V'_k and S_k arrays: the X forward's input tiles
    int on;
    int xi;   // the X inverse pass stages f_k and pi too (FP32: its two tiles keep two blocks per SM)
};

// Tensor maps of the Y passes' tiles (TMA). A Y line's element stride is H = N/2 + 1 complex,
// in FP32 8 H bytes, never a multiple of 16, so an array is mapped as rows of two y (pairs):
// {2 H, N N / 2, array, realization} in 8-byte elements (an FP64 complex being two), pair stride
// 16 H bytes. A tile of TL consecutive kz < N/2 at one x is two boxes of N/2 pairs (each split
// into boxes of 256 pairs above N = 512, a box edge being at most 256): the even
// rows {TL, N/2} at kz0, the odd rows at H + kz0; in FP32 that start is odd, so the odd box
// starts one element earlier (H - 1 + kz0, even) and is TL + 2 wide (a multiple of 16 bytes).
// The FP32 Y forward pass uses them (in FP64 the staging measured no faster): a* map the fields'
// V' (the first na arrays of the pass), b* the six S_ab; and the FP32 GW Y inverse pass in its
// pipelined form: a* TA, b* TB of each field. on = 0: direct loads.
struct YTma {
    CUtensorMap ae, ao, be, bo;   // even-row and odd-row boxes of the two array groups
    int na;
    int on;
};
// the lattice sizes whose Y forward pass has its tensor-map instantiation (FP32)
constexpr bool y_pipe_size(int N) { return N == 128 || N == 256 || N == 512 || N == 1024; }

// The arrays of the forward passes (V' of each field, then the six S_ab: up to
// PSC_MAX_FIELDS + 6) with the realization stride of each (elements).
constexpr int kMaxArrays = PSC_MAX_FIELDS + 6;
struct ArrList {
    void *p[kMaxArrays];
    long long rs[kMaxArrays];
};

// Batches of several configurations (lattice sizes) advanced by ONE launch per pass: the work
// list of each pass is the concatenation of every configuration's blocks (group i owns the
// items [start[pass], start[pass] + count)); a block of the batched kernel walks the items
// blockIdx.x, blockIdx.x + gridDim.x, ... and runs each with its configuration's geometry and
// buffers. Passes: 0 X inverse (+ drift), 1 Y inverse, 2 Z, 3 Y forward, 4 X forward + kick.
constexpr int kMaxBatchGroups = 4;
constexpr int kBatchPasses = 5;
struct BatchGroup {
    Geo g;
    int L;                       // N: line length of the X / Y passes
    int nbx, nbz, R, nj;         // X/Y blocks per array, Z blocks per realization, realizations, forward arrays
    int start[kBatchPasses];     // first item of this group in each pass's work list
    void *fk, *pk, *uk, *puk, *TA, *TB, *TC, *QV, *QS, *tw, *Fk, *Fu;
    double *partKG, *partV;
    DevBG *bg;
    ArrList fwd;                // the forward passes' arrays
};
struct BatchTable {
    int ngroups;
    int total[kBatchPasses];     // items of each pass
    BatchGroup grp[kMaxBatchGroups];
};

enum ScalarMode {
    SCALAR_PRIME = 0,   // coefficients for the opening half kick of a call
    SCALAR_BEGIN = 1,   // start of a step: b = ad, begin stage 0
    SCALAR_END = 2,     // end of stage p: reductions -> a'' -> b; begin the next stage/step
    SCALAR_EVAL = 3,    // coefficients for a pure force/energy evaluation
    SCALAR_EVAL_END = 4 // reductions of an evaluation -> K, G, V, a''
};

// Tile sizes, block sizes and shared memory for R lattices of one configuration; tc (may be
// null) overrides the default shapes of the register engine within their limits.
void plan(const psc_params &p, int R, LaunchCfg *cfg, const TileChoice *tc = nullptr);
// Set the dynamic shared-memory limits of the kernels a configuration uses.
cudaError_t configure(const LaunchCfg &cfg, int precision);

// One force evaluation of a stage: X-iFFT (with the drift when drift != 0),
// Y-iFFT, fused Z pass (c2r, V' and anisotropic stress, r2c), Y-fFFT and the
// X-fFFT with the kick epilogue and the K, G reductions.
cudaError_t launch_stage(const LaunchCfg &cfg, const Buffers &b, int precision, int drift, cudaStream_t st);
// The same sequence with an event recorded after each pass (ev[0] before the
// first, ev[i + 1] after pass i; 5 passes + the scalar kernel of `scalar_mode`).
cudaError_t launch_stage_timed(const LaunchCfg &cfg, const Buffers &b, int precision, int drift, int scalar_mode,
                               cudaEvent_t *ev, cudaStream_t st);
cudaError_t launch_scalar(const LaunchCfg &cfg, const Buffers &b, int mode, int p, cudaStream_t st);
cudaError_t launch_set_run(DevBG *bg, int R, double dt, int nsteps, cudaStream_t st);
// The homogeneous modes' FP64 shadow (DevBG::z0f, z0p) read from the arrays' element 0.
cudaError_t launch_zero_sync(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st);
// The opening half kick of a step call from the kept force: pi += c_open F (and pi_u).
cudaError_t launch_open_kick(const LaunchCfg &cfg, const Buffers &b, int precision, cudaStream_t st);
// Real-space view of nsrc complex arrays (c2r / N^3) into b.real (precision T).
cudaError_t launch_c2r_real(const LaunchCfg &cfg, const Buffers &b, int precision, const void *src, int nsrc,
                            cudaStream_t st);
// Bin sums of the scalar spectra (output.cpp:626-669) and of the GW spectra
// (output.cpp:780-1025). Layout of b.spec: [nf][3][nb] then GW [2][nb];
// b.spec_cnt: [nf][nb] then GW [nb]. Zeroes the accumulators first.
cudaError_t launch_spectra(const LaunchCfg &cfg, const Buffers &b, int precision, int nb, cudaStream_t st);

// Record the message psc_last_error() returns on this thread.
void set_last_error(const char *msg);

// Register-engine passes (psc_reg_f32.cu, psc_reg_f64.cu), N = 32..1024.
cudaError_t reg_configure_f32(const LaunchCfg &cfg);
cudaError_t reg_configure_f64(const LaunchCfg &cfg);
cudaError_t reg_stage_f32(const LaunchCfg &cfg, const Buffers &b, int drift, cudaStream_t st, cudaEvent_t *ev,
                          int scalar_mode);
cudaError_t reg_stage_f64(const LaunchCfg &cfg, const Buffers &b, int drift, cudaStream_t st, cudaEvent_t *ev,
                          int scalar_mode);
// The fused Z pass for the user models (model.h files compiled in, up to PSC_MAX_FIELDS
// fields): its shared-memory limits and its launch for R realizations.
cudaError_t reg_configure_user_f32(const LaunchCfg &cfg);
cudaError_t reg_configure_user_f64(const LaunchCfg &cfg);
cudaError_t reg_zpass_user_f32(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st, int R);
cudaError_t reg_zpass_user_f64(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st, int R);
// One pass of a batch over all its configurations (BatchTable): grid blocks of 256 threads with
// smem bytes of dynamic shared memory; the line lengths of the register engine up to 256.
cudaError_t reg_batch_pass_f32(const BatchTable &bt, int pass, int drift, int grid, size_t smem, cudaStream_t st);
cudaError_t reg_batch_pass_f64(const BatchTable &bt, int pass, int drift, int grid, size_t smem, cudaStream_t st);
// The kernel behind reg_batch_pass_* (for occupancy queries and shared-memory limits).
const void *reg_batch_kernel_f32(int pass, int drift);
const void *reg_batch_kernel_f64(int pass, int drift);
// The background update at the end of stage p for every realization of every configuration
// of the batch (k_scalar's SCALAR_END), one launch.
cudaError_t launch_scalar_batch(const BatchTable &bt, int p, cudaStream_t st);
cudaError_t generic_pad_passes(const LaunchCfg &cfg, const Buffers &b, int precision, cudaStream_t st);
cudaError_t reg_pad_passes_f32(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st);
cudaError_t reg_pad_passes_f64(const LaunchCfg &cfg, const Buffers &b, cudaStream_t st);
// The padded step's force evaluation (psc_pad.cu): drift (drift != 0) and padding of f_k
// into bp.fk, the passes at N_pad (cfgp, bp), extraction, force and kicks at N.
cudaError_t launch_pad_stage(const LaunchCfg &cfg, const LaunchCfg &cfgp, const Buffers &b, const Buffers &bp,
                             int precision, int drift, cudaStream_t st);
// nsrc_arrays half spectra of an Ns lattice -> the Nd lattice (Nd > Ns): zero-padding as
// padding() does, amplitudes times (Nd/Ns)^3 (dst is zeroed first).
cudaError_t launch_prolong(const void *src, void *dst, int nsrc_arrays, int Ns, int Nd, int precision,
                           cudaStream_t st);
cudaError_t reg_c2r_real_f32(const LaunchCfg &cfg, const Buffers &b, const void *src, int nsrc, cudaStream_t st);
cudaError_t reg_c2r_real_f64(const LaunchCfg &cfg, const Buffers &b, const void *src, int nsrc, cudaStream_t st);
// Tiling of the adjoint's scalar Z pass (nf inputs of P = N/32 threads per z line, TL
// lines per block, at most kAdjZBlocks blocks walking the tiles); its block partial sums
// have adj_z_blocks() slots per quantity.
constexpr int kAdjZBlocks = 2 * 152;
inline int adj_z_tile(int N, int nf) {
    const int P = N / 32;
    int t = 1;
    while (nf * P * t * 2 <= 256) t *= 2;
    return t;
}
inline int adj_z_blocks(int N, int nf) {
    const int tl = adj_z_tile(N, nf);
    const int ntiles = (N * N + tl - 1) / tl;
    return ntiles < kAdjZBlocks ? ntiles : kAdjZBlocks;
}

// The adjoint's J^T application at a stage point (register engine, one lattice, no GW):
// Lf += eta1 k^2 Mk + delta k^2 f_tape + r2c(eta2 V''(f(x)) m + gamma V'(f(x))), m = c2r(Mk) / N^3,
// coefficients from the device record ad; block partial sums of m.V', m.dV'/dgsq, m.dV'/dmu
// into part[i * kAdjZBlocks + block]. Uses TA and QV as scratch.
cudaError_t reg_adj_point_f32(const LaunchCfg &cfg, const Buffers &b, const void *Mk, const void *f_tape,
                              const void *fx_tape, void *Lf, double *part, const DevAdj *ad, cudaStream_t st);
cudaError_t reg_adj_point_f64(const LaunchCfg &cfg, const Buffers &b, const void *Mk, const void *f_tape,
                              const void *fx_tape, void *Lf, double *part, const DevAdj *ad, cudaStream_t st);
// The transposed GW source at a stage point (N <= 512, one lattice with GWs):
// Lf += -a^(1+alpha) sum_a i k_a r2c(T_a), T_a = 2 sum_b (1 + delta_ab) lambda_ab d_b f,
// lambda = c2r(Mu) / N^3 (six components), f the taped stage-point fields; etaS from ad.
// Uses TA, TB, TC, QS and Tarr ([3 nf][modes]) as scratch.
cudaError_t reg_adj_point_gw_f32(const LaunchCfg &cfg, const Buffers &b, const void *Mu, const void *f_tape,
                                 void *Tarr, void *Lf, const DevAdj *ad, cudaStream_t st);
cudaError_t reg_adj_point_gw_f64(const LaunchCfg &cfg, const Buffers &b, const void *Mu, const void *f_tape,
                                 void *Tarr, void *Lf, const DevAdj *ad, cudaStream_t st);

}  // namespace psc
