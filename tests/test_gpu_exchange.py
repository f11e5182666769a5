"""State exchange through the C ABI (psc_set_state / psc_get_state) at the benchmark's size.

The FP32 upload copies the caller's FP64 arrays through a 16 Mi-double device scratch and
rounds on the device; the download copies in up to 16 chunks and widens on the host cores.
Page-locked host buffers mapped into the device (cudaHostAlloc, torch's pin_memory) are read
and written by the rounding and widening kernels directly, in one pass over the link.
At 256^3 with GWs every array group spans several chunks of both. A round trip must give
exactly the FP32 rounding of the input (round to nearest even, as a host cast), except the
fields' homogeneous modes f_k(0), pi_k(0), which the device keeps in FP64 and returns
unchanged; an FP64 lattice must return its input unchanged."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _random_state(p, rng):
    def c(n):
        return (rng.standard_normal((n, p.modes)) + 1j * rng.standard_normal((n, p.modes))) * 10.0 ** rng.uniform(
            -30, 30, (n, p.modes))
    return dict(f_k=c(p.nflds), pi_k=c(p.nflds), u_k=c(6), pi_u_k=c(6))


@pytest.mark.parametrize("N,precision", [(256, 32), (64, 64)])
def test_round_trip_is_the_fp32_rounding(N, precision):
    from pspectcosmo_gb300 import Lattice, Params

    p = Params.preheating(N=N, spectral=0, with_gw=1, vv=4, precision=precision)
    rng = np.random.default_rng(7)
    st = _random_state(p, rng)
    # edge values: zeros, FP32 subnormal results, a halfway case, the top of the FP32 range
    st["f_k"].flat[:6] = [0.0, 1e-40 + 1e-44j, 1.0 + 2.0 ** -24, 3.0e38 + 3.4028235e38j, -0.0, 2.0 ** -149 * 0.75]
    lat = Lattice(p)
    lat.set_state(st["f_k"], st["pi_k"], 1.25, 0.5, -0.125, st["u_k"], st["pi_u_k"])
    got = lat.get_state()
    assert (got["a"], got["ad"], got["add"]) == (1.25, 0.5, -0.125)
    for k in ("f_k", "pi_k", "u_k", "pi_u_k"):
        want = st[k] if precision == 64 else st[k].astype(np.complex64).astype(np.complex128)
        if k in ("f_k", "pi_k"):
            want[:, 0] = st[k][:, 0]   # the homogeneous modes: FP64 on the device
        g, w = got[k].view(np.float64), want.view(np.float64)
        assert np.array_equal(g, w, equal_nan=True), k
    # into caller-owned buffers (get_state(out=...)): the same values, the same arrays back
    out = {k: np.full_like(got[k], np.nan) for k in ("f_k", "pi_k", "u_k", "pi_u_k")}
    got2 = lat.get_state(out=out)
    for k in out:
        assert got2[k] is out[k]
        assert np.array_equal(out[k].view(np.float64), got[k].view(np.float64), equal_nan=True), k
    with pytest.raises(ValueError):
        lat.get_state(out=dict(out, f_k=np.empty((p.nflds, p.modes), np.complex64)))
    # page-locked buffers (widened on the device, copied straight in) and a page-locked
    # source: the same values
    import torch

    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    outp = {k: pin(np.full_like(got[k], np.nan)) for k in out}
    lat.get_state(out=outp)
    for k in outp:
        assert np.array_equal(outp[k].view(np.float64), got[k].view(np.float64), equal_nan=True), k
    src = {k: pin(st[k]) for k in st}
    lat.set_state(src["f_k"], src["pi_k"], 1.25, 0.5, -0.125, src["u_k"], src["pi_u_k"])
    lat.get_state(out=outp)
    for k in outp:
        assert np.array_equal(outp[k].view(np.float64), got[k].view(np.float64), equal_nan=True), k
