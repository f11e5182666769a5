"""Checkpoint / resume (psc_checkpoint_write / psc_checkpoint_read): a run continued from a
checkpoint file repeats the uninterrupted run bit for bit (FP32 and FP64, with GWs), the file
holds the state in psc_get_state's layout, and a lattice of another shape is refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [32, 64])
def test_resume_is_bit_exact(tmp_path, precision):
    from pspectcosmo_gb300 import Lattice, Params
    from pspectcosmo_gb300.lattice import h5_read

    p = Params.preheating(N=32, spectral=0, with_gw=1, vv=4, precision=precision)
    a = Lattice(p)
    a.initialize()
    a.evolve(0.005, 5)
    path = str(tmp_path / "ck.h5")
    a.checkpoint(path)
    st = a.get_state()
    t = a.t
    assert np.array_equal(h5_read(path, "f_k"), st["f_k"].view(np.float64).reshape(2, -1, 2))
    assert np.array_equal(h5_read(path, "pi_u_k"), st["pi_u_k"].view(np.float64).reshape(6, -1, 2))
    assert list(h5_read(path, "background")) == [t, st["a"], st["ad"], st["add"]]
    assert list(h5_read(path, "lattice")) == [32, 2, 1, 0, 0, 4, 1, precision]
    a.evolve(0.005, 5)
    want = a.get_state()

    b = Lattice(p)
    b.restore(path)
    assert b.t == t
    b.evolve(0.005, 5)
    got = b.get_state()
    for k in ("f_k", "pi_k", "u_k", "pi_u_k", "a", "ad", "add"):
        assert np.array_equal(np.asarray(got[k]), np.asarray(want[k])), k


def test_restore_refuses_other_lattice(tmp_path):
    from pspectcosmo_gb300 import Lattice, Params
    from pspectcosmo_gb300.lattice import PscError

    a = Lattice(Params.preheating(N=32, spectral=1, with_gw=0))
    a.initialize()
    path = str(tmp_path / "ck.h5")
    a.checkpoint(path)
    for q in (Params.preheating(N=64, spectral=1, with_gw=0), Params.preheating(N=32, spectral=0, with_gw=1),
              Params.reference_default(N=32)):
        with pytest.raises(PscError):
            Lattice(q).restore(path)
    with pytest.raises(PscError):
        Lattice(Params.preheating(N=32, spectral=1, with_gw=0)).restore(str(tmp_path / "missing.h5"))
