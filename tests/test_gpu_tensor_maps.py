"""Tile staging by tensor maps (TMA). The X passes (X inverse in FP32, X forward + kick; above
N = 256 a tile is N/256 boxes along x) and,
in FP32 at N = 128 .. 1024, the Y forward pass (persistent and pipelined; the GW Y inverse pass
in the same form at 1024, or on request) stage their tiles in shared memory by tiled tensor
copies; with the maps switched off (psc_set_tensor_maps) every
thread loads its own elements.
The staging only changes where a value is read from, so every form must give the same bits:
fields, GW tensors and background after a few steps, from the same state, with the same tile
shapes. The Y passes' tensor-map forms also walk their tiles in another order (TL consecutive
kz of one x plane, then the kz = N/2 column), which must not change a bit either.
Each pass's bounded waits are driven to run out (the test hook plants bytes that no copy
delivers; every copy lands in valid memory): psc_step returns PSC_ERR_TIMEOUT and the handle
then evolves exactly as a fresh one."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

X, Y, YI = 1, 2, 4
PSC_ERR_CONFIG = -1
PSC_ERR_TIMEOUT = -5
KEYS = ("f_k", "pi_k", "u_k", "pi_u_k")


def _params(N, precision, gw):
    from pspectcosmo_gb300 import Params

    return Params.preheating(N=N, vv=4, spectral=0, with_gw=gw, precision=precision)


def _same(a, b, gw):
    for k in KEYS[:4 if gw else 2]:
        assert np.array_equal(a[k].view(np.float64), b[k].view(np.float64)), k
    assert (a["a"], a["ad"], a["add"]) == (b["a"], b["ad"], b["add"])


@pytest.mark.parametrize("N,precision,gw,want", [(256, 32, 1, X | Y), (128, 64, 1, X), (128, 32, 0, X | Y),
                                                  (64, 32, 1, X), (16, 32, 1, 0), (512, 32, 1, X | Y), (24, 32, 1, 0)])
def test_groups_in_use(N, precision, gw, want):
    from pspectcosmo_gb300 import Lattice

    lat = Lattice(_params(N, precision, gw))
    assert lat.tensor_maps == want
    lat.tensor_maps = X
    assert lat.tensor_maps == want & X
    lat.tensor_maps = 0
    assert lat.tensor_maps == 0
    lat.tensor_maps = X | Y
    assert lat.tensor_maps == want
    L = lat._L
    assert L.psc_set_tensor_maps(lat._h, 8) != 0   # an unknown group
    if want & Y and gw:   # the pipelined GW Y inverse pass on request
        lat.tensor_maps = X | Y | YI
        assert lat.tensor_maps == X | Y | YI
    lat.close()


@pytest.mark.parametrize("N,precision,gw,shift", [(256, 32, 1, -1), (128, 32, 1, -1), (128, 64, 1, -1),
                                                  (256, 64, 0, -1), (128, 32, 0, -1), (256, 32, 1, 2),
                                                  (512, 32, 1, -1), (512, 64, 1, -1)])
def test_every_form_gives_the_same_bits(N, precision, gw, shift):
    from pspectcosmo_gb300 import Lattice

    lat = Lattice(_params(N, precision, gw))
    if shift >= 0:   # a narrower tile than the default (4 lines): still staged by tensor maps
        lat.shapes = (shift, -1, 0)
        assert lat.shapes[0] == shift
    lat.initialize()
    s0 = lat.get_state()
    out = {}
    for mask in (X | Y | YI, X | Y, Y, X, 0):
        lat.tensor_maps = mask
        lat.set_state(s0["f_k"], s0["pi_k"], s0["a"], s0["ad"], s0["add"], s0.get("u_k"), s0.get("pi_u_k"))
        lat.evolve(0.005, 3)
        out[mask] = lat.get_state()
    lat.close()
    for mask in (X | Y | YI, X | Y, Y, X):
        _same(out[mask], out[0], gw)


def test_batch_realizations_with_tensor_maps_equal_single_lattices():
    """Two 128^3 GW realizations in one batch group (the realization is a coordinate of every
    tensor map) equal the same lattices advanced alone, bit for bit."""
    from pspectcosmo_gb300 import Ensemble, Lattice, Params

    ps = [Params.preheating(N=128, vv=4, spectral=0, with_gw=1, seed=3 + i, precision=32) for i in range(2)]
    ens = Ensemble(ps)
    assert ens.groups == 1
    ens.initialize()
    ens.evolve(0.005, 3)
    for idx, p in enumerate(ps):
        lat = Lattice(p)
        assert lat.tensor_maps == X | Y
        lat.initialize()
        lat.evolve(0.005, 3)
        _same(ens.get_state(idx), lat.get_state(), 1)
        lat.close()
    ens.close()


@pytest.mark.parametrize("pas", [0, 1, 2, 3, 4], ids=["x_inverse", "y_inverse", "zpass", "y_forward", "x_forward"])
def test_each_staged_wait_runs_out_and_the_handle_recovers(pas):
    from pspectcosmo_gb300 import Lattice, PscError

    p = _params(128, 32, 1)
    ref = Lattice(p)
    ref.initialize()
    s0 = ref.get_state()
    ref.evolve(0.005, 2)
    want = ref.get_state()
    ref.close()

    lat = Lattice(p)
    L = lat._L
    lat.tensor_maps = X | Y | YI   # the Y inverse pass pipelined at this size too
    lat.set_state(s0["f_k"], s0["pi_k"], s0["a"], s0["ad"], s0["add"], s0["u_k"], s0["pi_u_k"])
    assert L.psc_test_wait_hook_pass(lat._h, ctypes.c_double(20.0), 16, pas) == 0
    with pytest.raises(PscError) as ei:
        lat.evolve(0.005, 2)
    assert ei.value.code == PSC_ERR_TIMEOUT
    assert L.psc_test_wait_hook_pass(lat._h, ctypes.c_double(1000.0), 0, pas) == 0
    lat.set_state(s0["f_k"], s0["pi_k"], s0["a"], s0["ad"], s0["add"], s0["u_k"], s0["pi_u_k"])
    lat.evolve(0.005, 2)
    _same(lat.get_state(), want, 1)
    # without tensor maps the hook has nothing to act on (the Z pass stages by bulk copies)
    lat.tensor_maps = 0
    rc = L.psc_test_wait_hook_pass(lat._h, ctypes.c_double(20.0), 16, pas)
    assert rc == (0 if pas == 2 else PSC_ERR_CONFIG)
    L.psc_test_wait_hook_pass(lat._h, ctypes.c_double(1000.0), 0, pas)
    lat.close()
