"""The FP64 numpy adjoint (oracle/adjoint_ref.py) on the CPU.

Its forward map is pinned to the C oracle port of the reference's step (unmasked: the
real-space evolve_VV path), and its gradients to central finite differences of that same
forward map. The mode-space step is a fraction `scale` of the mean mode amplitude, chosen
per case so that the truncation error O(h^2) and the rounding error eps O / (h |dO/dh|) both
stay below the 1e-5 bar: <chi^2> of the two-field case is a small fluctuation observable
(scale 1e-6), <phi^2> of the one-field case is dominated by the homogeneous mode (1e-2)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import adjoint_ref as A  # noqa: E402

from golden_util import rel  # noqa: E402
from pspectcosmo_gb300.params import Params  # noqa: E402


def _params(nf, vv, N):
    if nf == 2:
        p = Params.preheating(N=N)
    else:
        p = Params.reference_default(N=N)
    p.vv = vv
    p.spectral = 0
    return p


def _ref_lattice(p, mu=1.0):
    fs = p.fStar if p.fStar > 0 else p.MPl
    return A.Lattice(p.N, p.kIR, p.nflds, p.gsq, mu=mu, alpha=p.alpha, fs_over_mpl2=(fs / p.MPl) ** 2, vv=p.vv)


def _state0(oracle_mod, p):
    o = oracle_mod.Oracle(p)
    o.init_ic()
    f, pi, _, _ = o.state_k()
    bg = o.bg()
    H = p.N // 2 + 1
    shape = (p.nflds, p.N, p.N, H)
    return o, [f.reshape(shape), pi.reshape(shape), bg["a"], bg["ad"], bg["add"]]


@pytest.mark.parametrize("nf,vv,N,dt,nsteps", [(2, 4, 16, 0.005, 6), (1, 2, 16, 2e-4, 6)])
def test_forward_map_is_the_reference_step(oracle_mod, nf, vv, N, dt, nsteps):
    p = _params(nf, vv, N)
    o, st0 = _state0(oracle_mod, p)
    lat = _ref_lattice(p)
    st = list(st0)
    st[4] = lat.A(st[0], st[1], st[2])
    assert abs(st[4] - st0[4]) <= 1e-11 * abs(st0[4]) + 1e-300
    for _ in range(nsteps):
        st = lat.step(st, dt)
    o.step(dt, nsteps)
    f, pi, _, _ = o.state_k()
    bg = o.bg()
    assert rel(st[0].reshape(f.shape), f) < 1e-10
    assert rel(st[1].reshape(pi.shape), pi) < 1e-10
    assert abs(st[2] / bg["a"] - 1) < 1e-13
    assert abs(st[3] / bg["ad"] - 1) < 1e-11
    assert abs(st[4] / bg["add"] - 1) < 1e-9


@pytest.mark.parametrize("nf,vv,scale", [(2, 4, 1e-6), (1, 2, 1e-2)])
def test_gradients_against_central_differences(oracle_mod, nf, vv, scale):
    N = 8
    p = _params(nf, vv, N)
    _, st0 = _state0(oracle_mod, p)
    lat = _ref_lattice(p)
    dt, nsteps = (0.005, 5) if nf == 2 else (2e-4, 5)
    O, gf, gp, _, gb, gth = A.gradient(lat, st0, dt, nsteps)
    assert O > 0
    rng = np.random.default_rng(7)
    checks = []
    for name in ("f", "pi"):
        d = np.fft.rfftn(rng.standard_normal((nf, N, N, N)), axes=(-3, -2, -1))
        i = 0 if name == "f" else 1
        d *= scale * np.abs(st0[i]).mean() / np.abs(d).mean()

        def Of(e, d=d, i=i):
            s = list(st0)
            s[i] = st0[i] + e * d
            return A.run_O(lat, s, dt, nsteps)

        checks.append((name, Of, float(np.sum(np.real(np.conj(gf if i == 0 else gp) * d)))))
    hb = scale * abs(st0[3])

    def Ob(e):
        s = list(st0)
        s[3] = st0[3] + e * hb
        return A.run_O(lat, s, dt, nsteps)

    checks.append(("ad", Ob, gb * hb))
    for k, th in enumerate(("gsq", "mu")):
        base = getattr(lat.model, th)
        if base == 0:
            continue
        h = scale * base

        def Ot(e, th=th, base=base, h=h):
            m = A.Lattice.__new__(A.Lattice)
            m.__dict__.update(lat.__dict__)
            m.model = A.Model(lat.nf, lat.model.gsq, lat.model.mu)
            setattr(m.model, th, base + e * h)
            return A.run_O(m, st0, dt, nsteps)

        checks.append((th, Ot, gth[k] * h))
    for name, Of, pred in checks:
        fd = (Of(1.0) - Of(-1.0)) / 2
        assert abs(fd - pred) <= 1e-5 * abs(fd), (name, fd, pred)


def _gw_state(oracle_mod, N, zero_gw):
    p = Params.preheating(N=N, vv=2, spectral=0, with_gw=1)
    o = oracle_mod.Oracle(p)
    o.init_ic()
    f, pi, u, pu = o.state_k()
    bg = o.bg()
    sh, sg = (2, N, N, N // 2 + 1), (6, N, N, N // 2 + 1)
    z = 0.0 if zero_gw else 1.0
    st0 = [f.reshape(sh), pi.reshape(sh), bg["a"], bg["ad"], bg["add"], z * u.reshape(sg), z * pu.reshape(sg)]
    fs = p.fStar if p.fStar > 0 else p.MPl
    lat = A.Lattice(N, p.kIR, 2, p.gsq, alpha=p.alpha, fs_over_mpl2=(fs / p.MPl) ** 2, vv=2, gw=True)
    return p, o, st0, lat


def test_gw_forward_map_and_rho_gw_are_the_reference(oracle_mod):
    """u, pi_u after the real-space GW step and energy()'s rho_GW (output.cpp:1030-1060)."""
    p, o, st0, lat = _gw_state(oracle_mod, 16, False)
    st = list(st0)
    st[4] = lat.A(st[0], st[1], st[2])
    for _ in range(3):
        st = lat.step(st, 0.005)
    o.step(0.005, 3)
    f, pi, u, pu = o.state_k()
    assert rel(st[5].reshape(u.shape), u) < 1e-12
    assert rel(st[6].reshape(pu.shape), pu) < 1e-12
    assert abs(lat.rho_gw(st[6], st[2]) / o.energies()["rho_gw"] - 1) < 1e-12


def test_rho_gw_gradients_against_central_differences(oracle_mod):
    """rho_GW generated by the scalar source from u = pi_u = 0 (so it depends on the fields at
    O(1)); FD step 1e-3 of the fluctuation amplitude / 1e-6 of a scalar."""
    N, dt, nsteps = 8, 0.005, 4
    p, o, st0, lat = _gw_state(oracle_mod, N, True)
    O, gf, gp, _, gb, gth, gu, gpu = A.gradient(lat, st0, dt, nsteps, observable="rho_gw")
    assert O > 0
    rng = np.random.default_rng(5)
    checks = []
    for name, i, g in (("f", 0, gf), ("pi", 1, gp)):
        d = np.fft.rfftn(rng.standard_normal((2, N, N, N)), axes=(-3, -2, -1))
        fl = st0[i].copy()
        fl[:, 0, 0, 0] = 0
        d *= 1e-3 * np.abs(fl).mean() / np.abs(d).mean()

        def Of(e, d=d, i=i):
            s = list(st0)
            s[i] = st0[i] + e * d
            return A.run_O(lat, s, dt, nsteps, "rho_gw")

        checks.append((name, Of, float(np.sum(np.real(np.conj(g) * d)))))
    hb = 1e-6 * abs(st0[3])

    def Ob(e):
        s = list(st0)
        s[3] = st0[3] + e * hb
        return A.run_O(lat, s, dt, nsteps, "rho_gw")

    checks.append(("ad", Ob, gb * hb))
    for k, th in enumerate(("gsq", "mu")):
        base = getattr(lat.model, th)
        h = 1e-4 * base

        def Ot(e, th=th, base=base, h=h):
            m = A.Lattice.__new__(A.Lattice)
            m.__dict__.update(lat.__dict__)
            m.model = A.Model(lat.nf, lat.model.gsq, lat.model.mu)
            setattr(m.model, th, base + e * h)
            return A.run_O(m, st0, dt, nsteps, "rho_gw")

        checks.append((th, Ot, gth[k] * h))
    for name, Of, pred in checks:
        fd = (Of(1.0) - Of(-1.0)) / 2
        assert abs(fd - pred) <= 1e-5 * abs(fd), (name, fd, pred)
    # the GW tensors' own gradients: rho_GW is quadratic in pi_u(T), linear response in u(0), pi_u(0)
    _, _, st0g, _ = _gw_state(oracle_mod, N, False)
    O, gf, gp, _, gb, gth, gu, gpu = A.gradient(lat, st0g, dt, nsteps, observable="rho_gw")
    for name, i, g in (("u", 5, gu), ("pu", 6, gpu)):
        d = np.fft.rfftn(rng.standard_normal((6, N, N, N)), axes=(-3, -2, -1))
        d *= 1e-3 * np.abs(st0g[i]).mean() / np.abs(d).mean()

        def Og(e, d=d, i=i):
            s = list(st0g)
            s[i] = st0g[i] + e * d
            return A.run_O(lat, s, dt, nsteps, "rho_gw")

        fd = (Og(1.0) - Og(-1.0)) / 2
        pred = float(np.sum(np.real(np.conj(g) * d)))
        assert abs(fd - pred) <= 1e-7 * abs(fd), (name, fd, pred)
