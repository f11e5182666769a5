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
