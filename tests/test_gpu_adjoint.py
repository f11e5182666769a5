"""The CUDA adjoint (psc_adjoint_chi2 through the C ABI) on the GPU.

FP64: O and every gradient within 1e-9 (max-norm relative) of the FP64 numpy adjoint
(oracle/adjoint_ref.py, itself pinned to the reference step and to finite differences),
and within 1e-5 of central finite differences of the device forward map. The adjoint's
forward map matches the product step (psc_step) to 1e-11. FP32 gradients are within 2e-3
of the FP64 ones (measured; FP32 state, FP64 reductions and background)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import adjoint_ref as A  # noqa: E402

from golden_util import rel  # noqa: E402

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-9
FD_TOL = 1e-5
FP32_TOL = 2e-3

CASES = {
    # name: (nflds, vv, dt, nsteps, every, fd scale)
    "preheat_vv4": (2, 4, 0.005, 8, 3, 1e-6),
    "preheat_vv2": (2, 2, 0.005, 6, 0, 1e-6),
    "phi2_vv2": (1, 2, 2e-4, 6, 2, 1e-2),
}


def _params(nf, vv, N=32, precision=64):
    from pspectcosmo_gb300.params import Params

    p = Params.preheating(N=N) if nf == 2 else Params.reference_default(N=N)
    p.vv = vv
    p.spectral = 0
    p.precision = precision
    return p


def _ic(p):
    from pspectcosmo_gb300 import generate_ic

    f, pi, _, _, info = generate_ic(p)
    return f, pi, info


def _lattice(p, f, pi, info, ad=None):
    from pspectcosmo_gb300 import Lattice

    lat = Lattice(p)
    lat.set_state(f, pi, info["a"], info["ad"] if ad is None else ad, info["add_printed"])
    return lat


def _ref_lattice(p):
    fs = p.fStar if p.fStar > 0 else p.MPl
    return A.Lattice(p.N, p.kIR, p.nflds, p.gsq, alpha=p.alpha, fs_over_mpl2=(fs / p.MPl) ** 2, vv=p.vv)


def _ref(p, f, pi, info, dt, nsteps):
    lat = _ref_lattice(p)
    sh = (p.nflds, p.N, p.N, p.N // 2 + 1)
    st0 = [f.reshape(sh), pi.reshape(sh), info["a"], info["ad"], 0.0]
    O, gf, gp, _, gb, gth = A.gradient(lat, st0, dt, nsteps)
    return O, gf.reshape(f.shape), gp.reshape(pi.shape), gb, gth


@pytest.mark.parametrize("case", list(CASES))
def test_gradients_match_fp64_adjoint(psc_lib, case):
    nf, vv, dt, nsteps, every, _ = CASES[case]
    p = _params(nf, vv)
    f, pi, info = _ic(p)
    with _lattice(p, f, pi, info) as lat:
        g = lat.adjoint_chi2(dt, nsteps, every)
    O, gf, gp, gb, gth = _ref(p, f, pi, info, dt, nsteps)
    assert abs(g["O"] / O - 1) < FP64_TOL
    assert rel(g["grad_f_k"], gf) < FP64_TOL
    assert rel(g["grad_pi_k"], gp) < FP64_TOL
    assert abs(g["grad_ad0"] / gb - 1) < FP64_TOL
    for k in range(2):
        if gth[k] != 0:
            assert abs(g["grad_theta"][k] / gth[k] - 1) < FP64_TOL, k
        else:
            assert g["grad_theta"][k] == 0


@pytest.mark.parametrize("case", ["preheat_vv4", "phi2_vv2"])
def test_forward_map_is_the_product_step(psc_lib, case):
    nf, vv, dt, nsteps, _, _ = CASES[case]
    p = _params(nf, vv)
    f, pi, info = _ic(p)
    with _lattice(p, f, pi, info) as lat:
        O = lat.adjoint_forward_chi2(dt, nsteps)
        st_adj = lat.get_state()
    # the adjoint starts from a''(0) = A(state); give the product step the same a''
    sh = (p.nflds, p.N, p.N, p.N // 2 + 1)
    add0 = _ref_lattice(p).A(f.reshape(sh), pi.reshape(sh), info["a"])
    with _lattice(p, f, pi, dict(info, add_printed=add0)) as lat:
        lat.evolve(dt, nsteps)
        st = lat.get_state()
        fx, _ = lat.fields_real()
    assert abs(np.mean(fx[-1] ** 2) / O - 1) < 1e-11
    assert rel(st_adj["f_k"], st["f_k"]) < 1e-11
    assert rel(st_adj["pi_k"], st["pi_k"]) < 1e-11
    for k in ("a", "ad", "add"):
        assert abs(st_adj[k] / st[k] - 1) < 1e-11, k


@pytest.mark.parametrize("case", ["preheat_vv4", "phi2_vv2"])
def test_gradients_against_device_central_differences(psc_lib, case):
    nf, vv, dt, nsteps, every, scale = CASES[case]
    p = _params(nf, vv)
    f, pi, info = _ic(p)
    with _lattice(p, f, pi, info) as lat:
        g = lat.adjoint_chi2(dt, nsteps, every)
    rng = np.random.default_rng(11)
    N = p.N

    def run(ff, pp, ad=None, gsq=None):
        q = _params(nf, vv)
        if gsq is not None:
            q.gsq = gsq
        with _lattice(q, ff, pp, info, ad) as lat:
            return lat.adjoint_forward_chi2(dt, nsteps)

    for name in ("f", "pi"):
        d = np.fft.rfftn(rng.standard_normal((nf, N, N, N)), axes=(-3, -2, -1)).reshape(f.shape)
        base = f if name == "f" else pi
        d *= scale * np.abs(base).mean() / np.abs(d).mean()
        if name == "f":
            fd = (run(f + d, pi) - run(f - d, pi)) / 2
        else:
            fd = (run(f, pi + d) - run(f, pi - d)) / 2
        pred = float(np.sum(np.real(np.conj(g["grad_f_k" if name == "f" else "grad_pi_k"]) * d)))
        assert abs(fd - pred) <= FD_TOL * abs(fd), (name, fd, pred)
    hb = scale * abs(info["ad"])
    fd = (run(f, pi, ad=info["ad"] + hb) - run(f, pi, ad=info["ad"] - hb)) / 2
    assert abs(fd - g["grad_ad0"] * hb) <= FD_TOL * abs(fd), ("ad", fd, g["grad_ad0"] * hb)
    if p.gsq != 0:
        h = scale * p.gsq
        fd = (run(f, pi, gsq=p.gsq + h) - run(f, pi, gsq=p.gsq - h)) / 2
        assert abs(fd - g["grad_theta"][0] * h) <= FD_TOL * abs(fd), ("gsq", fd, g["grad_theta"][0] * h)


def test_checkpoint_spacing_does_not_change_the_gradient(psc_lib):
    nf, vv, dt, nsteps, _, _ = CASES["preheat_vv4"]
    p = _params(nf, vv)
    f, pi, info = _ic(p)
    out = []
    for every in (1, 3, 0):
        with _lattice(p, f, pi, info) as lat:
            out.append(lat.adjoint_chi2(dt, nsteps, every))
    for g in out[1:]:
        assert abs(g["O"] / out[0]["O"] - 1) < 1e-13
        assert rel(g["grad_f_k"], out[0]["grad_f_k"]) < 1e-12
        assert rel(g["grad_pi_k"], out[0]["grad_pi_k"]) < 1e-12


def test_fp32_gradients(psc_lib):
    nf, vv, dt, nsteps, every, _ = CASES["preheat_vv4"]
    p = _params(nf, vv, precision=32)
    f, pi, info = _ic(p)
    with _lattice(p, f, pi, info) as lat:
        g = lat.adjoint_chi2(dt, nsteps, every)
    O, gf, gp, gb, gth = _ref(_params(nf, vv), f, pi, info, dt, nsteps)
    assert abs(g["O"] / O - 1) < FP32_TOL
    assert rel(g["grad_f_k"], gf) < FP32_TOL
    assert rel(g["grad_pi_k"], gp) < FP32_TOL
    assert abs(g["grad_ad0"] / gb - 1) < FP32_TOL
    assert abs(g["grad_theta"][0] / gth[0] - 1) < FP32_TOL


def test_unsupported_configurations_are_rejected(psc_lib):
    from pspectcosmo_gb300 import Lattice, PscError

    p = _params(2, 4)
    p.spectral = 1
    p.simulate_inflation = 1
    f, pi, info = _ic(p)
    with _lattice(p, f, pi, info) as lat:
        with pytest.raises(PscError) as e:
            lat.adjoint_chi2(0.005, 2)
        assert e.value.code == -1
    q = _params(2, 4, N=16)
    with Lattice(q) as lat:
        lat.initialize()
        with pytest.raises(PscError) as e:
            lat.adjoint_chi2(0.005, 2)
        assert e.value.code == -1


# ---------------------------------------------------------------- rho_GW (GW energy density)
def _gw_params(N=32, precision=64):
    from pspectcosmo_gb300.params import Params

    p = Params.preheating(N=N, vv=2, spectral=0, with_gw=1)
    p.precision = precision
    return p


def _gw_setup(p, zero_gw):
    from pspectcosmo_gb300 import generate_ic

    f, pi, u, pu, info = generate_ic(p)
    z = 0.0 if zero_gw else 1.0
    return f, pi, z * u, z * pu, info


def _gw_lattice(p, f, pi, u, pu, info, ad=None, add=None):
    from pspectcosmo_gb300 import Lattice

    lat = Lattice(p)
    lat.set_state(f, pi, info["a"], info["ad"] if ad is None else ad, info["add_printed"] if add is None else add,
                  u, pu)
    return lat


def _gw_ref(p, f, pi, u, pu, info, dt, nsteps):
    fs = p.fStar if p.fStar > 0 else p.MPl
    lat = A.Lattice(p.N, p.kIR, p.nflds, p.gsq, alpha=p.alpha, fs_over_mpl2=(fs / p.MPl) ** 2, vv=p.vv, gw=True)
    sh, sg = (p.nflds, p.N, p.N, p.N // 2 + 1), (6, p.N, p.N, p.N // 2 + 1)
    st0 = [f.reshape(sh), pi.reshape(sh), info["a"], info["ad"], 0.0, u.reshape(sg), pu.reshape(sg)]
    O, gf, gp, _, gb, gth, gu, gpu = A.gradient(lat, st0, dt, nsteps, observable="rho_gw")
    return O, gf.reshape(f.shape), gp.reshape(pi.shape), gu.reshape(u.shape), gpu.reshape(pu.shape), gb, gth, lat


@pytest.mark.parametrize("zero_gw", [True, False])
def test_rho_gw_gradients_match_fp64_adjoint(psc_lib, zero_gw):
    """rho_GW generated from u = pi_u = 0 by the scalar source, and from the GW vacuum."""
    p = _gw_params()
    f, pi, u, pu, info = _gw_setup(p, zero_gw)
    dt, nsteps = 0.005, 6
    with _gw_lattice(p, f, pi, u, pu, info) as lat:
        g = lat.adjoint("rho_gw", dt, nsteps, 4)
    O, gf, gp, gu, gpu, gb, gth, _ = _gw_ref(p, f, pi, u, pu, info, dt, nsteps)
    assert abs(g["O"] / O - 1) < FP64_TOL
    assert rel(g["grad_f_k"], gf) < FP64_TOL
    assert rel(g["grad_pi_k"], gp) < FP64_TOL
    assert rel(g["grad_u_k"], gu) < FP64_TOL
    assert rel(g["grad_pi_u_k"], gpu) < FP64_TOL
    assert abs(g["grad_ad0"] / gb - 1) < FP64_TOL
    for k in range(2):
        assert abs(g["grad_theta"][k] - gth[k]) <= FP64_TOL * abs(gth[k]) + 1e-300, k


def test_rho_gw_is_the_product_energy(psc_lib):
    """The adjoint's rho_GW is psc_energies' rho_GW of the same final state (energy(), the GW walk)."""
    p = _gw_params()
    f, pi, u, pu, info = _gw_setup(p, False)
    with _gw_lattice(p, f, pi, u, pu, info) as lat:
        O = lat.adjoint_forward("rho_gw", 0.005, 5)
        rho = lat.energies()["rho_gw"]
    assert abs(O / rho - 1) < 1e-12


def test_rho_gw_gradients_against_device_central_differences(psc_lib):
    p = _gw_params()
    f, pi, u, pu, info = _gw_setup(p, True)
    dt, nsteps = 0.005, 6
    with _gw_lattice(p, f, pi, u, pu, info) as lat:
        g = lat.adjoint("rho_gw", dt, nsteps)
    N = p.N
    rng = np.random.default_rng(13)

    def run(ff, pp, ad=None, gsq=None):
        q = _gw_params()
        if gsq is not None:
            q.gsq = gsq
        with _gw_lattice(q, ff, pp, u, pu, info, ad) as lat:
            return lat.adjoint_forward("rho_gw", dt, nsteps)

    for name in ("f", "pi"):
        d = np.fft.rfftn(rng.standard_normal((2, N, N, N)), axes=(-3, -2, -1)).reshape(f.shape)
        base = (f if name == "f" else pi).copy()
        base[:, 0] = 0
        d *= 1e-3 * np.abs(base).mean() / np.abs(d).mean()
        if name == "f":
            fd = (run(f + d, pi) - run(f - d, pi)) / 2
        else:
            fd = (run(f, pi + d) - run(f, pi - d)) / 2
        pred = float(np.sum(np.real(np.conj(g["grad_f_k" if name == "f" else "grad_pi_k"]) * d)))
        assert abs(fd - pred) <= FD_TOL * abs(fd), (name, fd, pred)
    hb = 1e-6 * abs(info["ad"])
    fd = (run(f, pi, ad=info["ad"] + hb) - run(f, pi, ad=info["ad"] - hb)) / 2
    assert abs(fd - g["grad_ad0"] * hb) <= FD_TOL * abs(fd), ("ad", fd, g["grad_ad0"] * hb)
    h = 1e-4 * p.gsq
    fd = (run(f, pi, gsq=p.gsq + h) - run(f, pi, gsq=p.gsq - h)) / 2
    assert abs(fd - g["grad_theta"][0] * h) <= FD_TOL * abs(fd), ("gsq", fd, g["grad_theta"][0] * h)


def test_rho_gw_checkpoint_spacing_and_fp32(psc_lib):
    p = _gw_params()
    f, pi, u, pu, info = _gw_setup(p, True)
    dt, nsteps = 0.005, 6
    out = []
    for every in (1, 0):
        with _gw_lattice(p, f, pi, u, pu, info) as lat:
            out.append(lat.adjoint("rho_gw", dt, nsteps, every))
    assert abs(out[1]["O"] / out[0]["O"] - 1) < 1e-13
    for k in ("grad_f_k", "grad_pi_k", "grad_pi_u_k"):
        assert rel(out[1][k], out[0][k]) < 1e-12, k
    q = _gw_params(precision=32)
    with _gw_lattice(q, f, pi, u, pu, info) as lat:
        g32 = lat.adjoint("rho_gw", dt, nsteps)
    assert abs(g32["O"] / out[1]["O"] - 1) < 5e-3
    assert rel(g32["grad_f_k"], out[1]["grad_f_k"]) < 5e-3
    assert rel(g32["grad_pi_u_k"], out[1]["grad_pi_u_k"]) < 5e-3
