"""The C ABI (include/psc.h) on the CPU: the library loads, exports every declared
entry point, validates configurations, and its host-side IC generator reproduces
the reference's initial conditions bit for bit. No GPU work is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

from golden_util import ALL_RUNS, load, params_for, rel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(psc_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_exports_every_declared_symbol(psc_lib):
    syms = declared_symbols()
    assert len(syms) >= 15
    for name in syms:
        assert hasattr(psc_lib, name), f"libpsc.so does not export {name}"


def test_params_struct_layout_matches_header(psc_lib):
    from pspectcosmo_gb300.params import Params

    p = Params()
    psc_lib.psc_default_params(ctypes.byref(p))
    ref = Params.reference_default()
    for name, _ in Params._fields_:
        a, b = getattr(p, name), getattr(ref, name)
        if name in ("initfield", "initderivs"):
            assert list(a) == list(b), name
        else:
            assert a == b, name


@pytest.mark.parametrize("bad", [dict(N=44), dict(N=15), dict(N=768), dict(N=2048), dict(N=4), dict(nflds=3),
                                 dict(vv=3), dict(precision=16), dict(with_gw=1, N_pad=32), dict(N=16, N_pad=44),
                                 dict(kIR=0.0), dict(model=1)])
def test_invalid_configurations_are_rejected(psc_lib, bad):
    from pspectcosmo_gb300.params import Params

    p = Params.reference_default(**bad)
    h = ctypes.c_void_p()
    rc = psc_lib.psc_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == -1, psc_lib.psc_last_error()
    assert h.value is None
    assert psc_lib.psc_strerror(rc) == b"unsupported configuration"


@pytest.mark.parametrize("ok", [dict(N=24), dict(N=20), dict(N=28), dict(N=96), dict(N=480), dict(N=1024),
                                dict(N=16, N_pad=24), dict(N=20, N_pad=30), dict(N=32, N_pad=64)])
def test_accepted_sizes_pass_validation(psc_lib, ok):
    """Even N up to 512 with prime factors 2, 3, 5, 7 (and such an N_pad above N) pass the
    parameter checks: psc_create fails only where no GPU is present (a CUDA error, not
    PSC_ERR_CONFIG)."""
    from pspectcosmo_gb300.params import Params

    p = Params.reference_default(**ok)
    h = ctypes.c_void_p()
    rc = psc_lib.psc_create(ctypes.byref(p), ctypes.byref(h))
    assert rc != -1, psc_lib.psc_last_error()
    if rc == 0:
        psc_lib.psc_destroy(h)


def test_null_arguments(psc_lib):
    h = ctypes.c_void_p()
    assert psc_lib.psc_create(None, ctypes.byref(h)) == -2
    assert psc_lib.psc_step(None, 0.1, 1) == -2


@pytest.mark.parametrize("run", ALL_RUNS)
def test_host_ic_generator_matches_reference(psc_lib, run):
    from pspectcosmo_gb300 import generate_ic

    g, meta = load(run)
    p = params_for(meta)
    f, pi, u, pu, info = generate_ic(p)
    n = g["ic_f_k"].shape[1]
    assert info["hubble_init"] == meta["ic_info"]["hubble_init"]
    assert info["ad"] == g["bg"][0, 3]
    if p.spectral:
        assert np.array_equal(f[:, :n], g["ic_f_k"])
        assert np.array_equal(pi[:, :n], g["ic_pi_k"])
    else:
        # the golden arrays are r2c(c2r(.)) of the generated ones
        assert rel(f[:, :n], g["ic_f_k"]) < 1e-14 and rel(pi[:, :n], g["ic_pi_k"]) < 1e-14
        m = g["ic_u_k"].shape[1]   # the modes the fixture keeps (a prefix at the larger sizes)
        assert rel(u[:, :m], g["ic_u_k"]) < 1e-14 and rel(pu[:, :m], g["ic_pi_u_k"]) < 1e-14


def test_host_ic_generator_equals_oracle(psc_lib, oracle_mod):
    """Same draws as the oracle restatement, including the Rayleigh branch
    (SIMULATE_INFLATION false) that the shipped reference cannot compile."""
    from pspectcosmo_gb300 import generate_ic
    from pspectcosmo_gb300.params import Params

    for p in (Params.reference_default(N=16, simulate_inflation=0),
              Params.preheating(N=16, spectral=0, with_gw=1, seed=7)):
        f, pi, u, pu, info = generate_ic(p)
        o = oracle_mod.Oracle(p)
        o.init_ic()
        if p.spectral:
            of, opi, _, _ = o.state_k()
            assert np.array_equal(f, of) and np.array_equal(pi, opi)
        else:
            of, opi, ou, opu = o.state_k()
            assert rel(f, of) < 1e-14 and rel(u, ou) < 1e-14 and rel(pu, opu) < 1e-14
