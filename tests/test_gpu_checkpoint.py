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


@pytest.mark.parametrize("gw,precision", [(1, 32), (1, 64), (0, 32)])
def test_step_calls_reuse_the_kept_force(gw, precision):
    """n single-step calls = one n-step call, bit for bit (the opening half kick of a call
    reuses the force the previous call's last kick kept); the same after set_state, which
    drops the kept force, and in a padded lattice."""
    from pspectcosmo_gb300 import Lattice, Params

    p = Params.preheating(N=32, spectral=1 - gw, with_gw=gw, vv=4, precision=precision)
    runs = []
    for split in (False, True):
        lat = Lattice(p)
        lat.initialize()
        if split:
            for _ in range(4):
                lat.evolve(0.005, 1)
        else:
            lat.evolve(0.005, 1)
            lat.evolve(0.005, 3)
        s = lat.get_state()
        lat.set_state(s["f_k"], s["pi_k"], s["a"], s["ad"], s["add"], s["u_k"], s["pi_u_k"])
        lat.evolve(0.005, 2)
        runs.append(lat.get_state())
    for k in ("f_k", "pi_k", "a", "ad", "add") + (("u_k", "pi_u_k") if gw else ()):
        assert np.array_equal(np.asarray(runs[0][k]), np.asarray(runs[1][k])), k


def test_kept_force_matches_evaluation():
    """A call after a call (kept force) equals a call after set_state (force evaluated)."""
    from pspectcosmo_gb300 import Lattice, Params

    p = Params.preheating(N=64, spectral=0, with_gw=1, vv=4, precision=32)
    a = Lattice(p)
    a.initialize()
    a.evolve(0.005, 2)
    s = a.get_state()
    a.evolve(0.005, 2)           # opening kick from the kept force
    b = Lattice(p)
    b.set_state(s["f_k"], s["pi_k"], s["a"], s["ad"], s["add"], s["u_k"], s["pi_u_k"])
    b.evolve(0.005, 2)           # opening kick from a force evaluation
    sa, sb = a.get_state(), b.get_state()
    for k in ("f_k", "pi_k", "u_k", "pi_u_k", "a", "ad", "add"):
        assert np.array_equal(np.asarray(sa[k]), np.asarray(sb[k])), k
