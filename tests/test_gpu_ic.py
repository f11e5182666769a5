"""Initial conditions generated on the device (one thread per mode, Park-Miller skip-ahead)
against the host generator, which reproduces the reference's initialize() /
initialize_GW() bit for bit (tests/test_oracle_golden.py).

The integer draws are the reference's exactly; the FP64 mode arithmetic uses the
device's sqrt/log/sin/cos, so FP64 states agree to 1e-13 relative (max norm), FP32
states to the FP32 rounding of the same values (1e-6)."""
import numpy as np
import pytest

from golden_util import rel

pytestmark = pytest.mark.gpu

CASES = {
    # name: Params factory, overrides (fixed-amplitude ICs: 1 draw per mode; Rayleigh: 4)
    "single_field_fixed_amplitude": ("default", dict(N=32)),
    "single_field_rayleigh_n16": ("default", dict(N=16, simulate_inflation=0, spectral=0)),
    "two_field_gw_fixed_amplitude": ("preheating", dict(N=32, spectral=0, with_gw=1)),
    "two_field_gw_rayleigh_n64": ("preheating", dict(N=64, spectral=0, with_gw=1, simulate_inflation=0, seed=7)),
    # a lattice size that is not a power of two (24 = 8 x 3)
    "two_field_gw_fixed_amplitude_n24": ("preheating", dict(N=24, spectral=0, with_gw=1)),
}


def _params(case, precision):
    from pspectcosmo_gb300.params import Params

    kind, kw = CASES[case]
    p = Params.preheating(**kw) if kind == "preheating" else Params.reference_default(**kw)
    p.precision = precision
    return p


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("case", list(CASES))
def test_device_ic_matches_host_generator(psc_lib, case, precision):
    from pspectcosmo_gb300 import Lattice, generate_ic

    p = _params(case, precision)
    f, pi, u, pu, info = generate_ic(p)
    tol = 1e-13 if precision == 64 else 1e-6
    with Lattice(p) as lat:
        lat.initialize()
        st = lat.get_state()
    assert rel(st["f_k"], f) < tol
    assert rel(st["pi_k"], pi) < tol
    # the fluctuation modes alone (the homogeneous mode dominates the max norm)
    for fld in range(p.nflds):
        a, b = st["f_k"][fld].copy(), f[fld].copy()
        a[0] = b[0] = 0
        assert rel(a, b) < 10 * tol
    if p.with_gw:
        assert rel(st["u_k"], u) < tol
        assert rel(st["pi_u_k"], pu) < tol
    assert st["a"] == info["a"] and st["ad"] == info["ad"]


def test_device_ic_is_deterministic_and_seeded(psc_lib):
    from pspectcosmo_gb300 import Lattice

    p = _params("single_field_fixed_amplitude", 64)
    with Lattice(p) as lat:
        lat.initialize()
        a = lat.get_state()["f_k"]
        lat.initialize()
        b = lat.get_state()["f_k"]
    assert np.array_equal(a, b)
    q = p.copy()
    q.seed = 2
    with Lattice(q) as lat:
        lat.initialize()
        c = lat.get_state()["f_k"]
    assert not np.allclose(a[0, 1:], c[0, 1:])
