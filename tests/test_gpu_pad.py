"""The padded (dealiased) spectral step and the spectral prolongation on the device.

* FP64 padded step (N = 16, N_pad = 32; N = 16, N_pad = 24; N = 20, N_pad = 30) against the
  reference's own evolve_VV_k_pad (golden runs pad1_n16, pad2_n16_vv4, pad3_n16_vv4 with the
  three-field model.h, pad1_n16_np24, pad2_n20_vv4_np30): initial a'' (kernel_a_k_pad) to 1e-12, the state
  after 20 steps to 1e-10 of its largest mode and, for the two-field model where the
  padding changes the result, the fluctuation modes (all but k = 0) to 1e-8 of theirs
  (the unpadded step differs from the padded one by ~5e-7 there).
* FP32 padded step within 2e-4 of the FP64 one (the FP32 field tolerance of the parity tests).
* psc_set_state_padded bit-exact with the oracle's padding() x (N/Nsrc)^3 (FP64).
* Lattice sizes without a CPU oracle (up to 1024^3): a band-limited state (|k| <= 5 per
  axis) on a 32^3 lattice prolonged to N. V' is cubic and the GW source quadratic, so
  no product reaches the 32^3 Nyquist and every volume average (K, G, V, rho_GW) and the
  background a, a', a'' evolve identically on every N: equal to 1e-11 (FP64) / 2e-5 (FP32)
  after 3 Yoshida-4 steps of the GW path; in FP32 a'' to 1e-4, the parity tests' FP32
  bound for it (a'' ~ (V - 2K)/3 cancels). The step is the reference's adaptive
  dt = 0.2 a / (kIR N sqrt(3)/2) of the large lattice (pspectcosmo.cpp:213-233): at a fixed
  dt = 0.005 the modes of a 1024^3 lattice have omega dt up to 4.4, beyond the Yoshida-4
  bound (~1.57), and the FP32 rounding noise there grows by orders of magnitude per step.
"""
import os
import re
import sys

import numpy as np
import pytest

from golden_util import load, params_for, rel

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))


def _padded(run, precision=64):
    from pspectcosmo_gb300 import Lattice

    g, meta = load(run)
    p = params_for(meta, precision)
    m = re.search(r"np(\d+)", run)
    p.N_pad = int(m.group(1)) if m else 2 * p.N
    return g, meta, p, Lattice(p)


# pad1_n16_np24: a padded grid that is not a power of two (24^3, the generic engine, ratio 1.5);
# pad2_n20_vv4_np30: both grids mixed-radix (20^3 and 30^3)
@pytest.mark.parametrize("run", ["pad1_n16", "pad2_n16_vv4", "pad3_n16_vv4", "pad1_n16_np24", "pad2_n20_vv4_np30"])
def test_padded_step_matches_reference(run):
    g, meta, p, lat = _padded(run)
    lat.initialize()
    bg0 = lat.background()
    assert rel(bg0["add"], meta["ic_info"]["add"]) < 1e-12
    st = lat.get_state()
    assert rel(st["f_k"][:, :4096], g["ic_f_k"][:, :4096]) < 1e-13
    dt, n = meta["dt"], meta["nsteps"]
    lat.evolve(dt, n)
    st = lat.get_state()
    assert rel(st["f_k"], g["fin_f_k"]) < 1e-10
    assert rel(st["pi_k"], g["fin_pi_k"]) < 1e-10
    fl, ref = st["f_k"].copy(), g["fin_f_k"].copy()
    fl[:, 0] = 0
    ref[:, 0] = 0
    assert rel(fl, ref) < 1e-8
    row = g["bg"][-1]
    bg = lat.background()
    assert rel(bg["a"], row[2]) < 1e-12 and rel(bg["ad"], row[3]) < 1e-11 and rel(bg["add"], row[4]) < 1e-10


def test_padded_differs_from_unpadded():
    """Two-field model: the padded step is not the unpadded one (the aliasing it removes)."""
    from pspectcosmo_gb300 import Lattice

    g, meta, p, lat = _padded("pad2_n16_vv4")
    q = params_for(meta, 64)
    plain = Lattice(q)
    for x in (lat, plain):
        x.initialize()
        x.evolve(meta["dt"], meta["nsteps"])
    a, b = lat.get_state()["f_k"], plain.get_state()["f_k"]
    a[:, 0] = 0
    b[:, 0] = 0
    assert rel(a, b) > 1e-8


def test_padded_fp32_vs_fp64():
    from pspectcosmo_gb300 import Lattice, Params

    res = {}
    for prec in (64, 32):
        p = Params.preheating(N=64, N_pad=128, spectral=1, with_gw=0, vv=4, precision=prec)
        lat = Lattice(p)
        lat.initialize()
        lat.evolve(0.005, 10)
        res[prec] = (lat.get_state(), lat.background(), lat.energies())
    s64, b64, e64 = res[64]
    s32, b32, e32 = res[32]
    assert rel(s32["f_k"], s64["f_k"]) < 2e-4 and rel(s32["pi_k"], s64["pi_k"]) < 2e-4
    assert rel(b32["a"], b64["a"]) < 1e-6 and rel(b32["ad"], b64["ad"]) < 1e-6
    assert rel(e32["V"], e64["V"]) < 1e-4


def test_prolongation_is_padding():
    import pad_ref
    from pspectcosmo_gb300 import Lattice, Params

    rng = np.random.default_rng(11)
    Ns, N = 16, 32
    Hs = Ns // 2 + 1
    shape = (2, Ns * Ns * Hs)
    fk = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    pk = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    lat = Lattice(Params.preheating(N=N, spectral=1, with_gw=0))
    lat.set_state_padded(Ns, fk, pk, 1.0, 0.1, 0.0)
    st = lat.get_state()
    for fld in range(2):
        want = pad_ref.padding(fk[fld], Ns, N).ravel() * 8.0
        assert np.array_equal(st["f_k"][fld], want)
        assert np.array_equal(st["pi_k"][fld], pad_ref.padding(pk[fld], Ns, N).ravel() * 8.0)


def _band_limited_state(rng, Ns=32, K=5, gw=True):
    """Real band-limited fields on an Ns lattice: phi0 + small fluctuations, chi small,
    u_ij and pi_u small; returned as half spectra [arrays][Ns*Ns*(Ns/2+1)]."""
    Hs = Ns // 2 + 1
    kx = np.fft.fftfreq(Ns, 1.0 / Ns)
    kz = np.arange(Hs)
    band = (np.abs(kx)[:, None, None] <= K) & (np.abs(kx)[None, :, None] <= K) & (kz[None, None, :] <= K)

    def field(amp, mean=0.0):
        x = rng.standard_normal((Ns, Ns, Ns)) * amp + mean
        k = np.fft.rfftn(x, axes=(0, 1, 2))
        k[~band] = 0
        return k.ravel()

    f = np.stack([field(1e-4, 0.193), field(1e-6)])
    pi = np.stack([field(1e-6, -0.142), field(1e-7)])
    u = np.stack([field(1e-9) for _ in range(6)]) if gw else None
    pu = np.stack([field(1e-9) for _ in range(6)]) if gw else None
    return f, pi, u, pu


@pytest.mark.parametrize("N,precision", [(64, 64), (128, 64), (256, 64), (512, 64), (512, 32), (1024, 32)])
def test_large_lattices_band_limited(N, precision):
    from pspectcosmo_gb300 import Lattice, Params

    rng = np.random.default_rng(5)
    f, pi, u, pu = _band_limited_state(rng)
    a0, ad0, add0 = 1.0, 0.0978, -5e-4
    out = {}
    for n in (32, N):
        p = Params.preheating(N=n, spectral=0, with_gw=1, vv=4, precision=precision)
        lat = Lattice(p)
        if n == 32:
            lat.set_state(f, pi, a0, ad0, add0, u, pu)
        else:
            lat.set_state_padded(32, f, pi, a0, ad0, add0, u, pu)
        lat.evolve(0.2 / (N * 3 ** 0.5 / 2), 3)
        e = lat.energies()
        out[n] = (lat.background(), e)
        lat.close()
    (b0, e0), (b1, e1) = out[32], out[N]
    tol = 1e-11 if precision == 64 else 2e-5
    for k in ("a", "ad", "add"):
        assert rel(b1[k], b0[k]) < (max(tol, 1e-4) if k == "add" else tol), k
    for k in ("K", "G", "V"):
        assert rel(e1[k], e0[k]) < tol, k
    assert rel(e1["rho_gw"], e0["rho_gw"]) < (tol if precision == 64 else 1e-4)


def test_padded_rejections():
    from pspectcosmo_gb300 import Ensemble, Lattice, Params
    from pspectcosmo_gb300.lattice import PscError

    with pytest.raises(PscError):
        Lattice(Params.preheating(N=32, N_pad=64, spectral=0, with_gw=1))   # GWs: real-space path
    with pytest.raises(PscError):
        Lattice(Params.preheating(N=32, N_pad=32, spectral=1, with_gw=0))   # N_pad <= N
    with pytest.raises(PscError):
        Ensemble([Params.preheating(N=32, N_pad=64, spectral=1, with_gw=0)])
    lat = Lattice(Params.preheating(N=32, N_pad=64, spectral=1, with_gw=0, simulate_inflation=0))
    lat.initialize()
    with pytest.raises(PscError):
        lat.adjoint("chi2", 0.005, 2)
