"""Batched ensembles: realizations of uneven lattice sizes advanced together (one graph per
step; on the register engine one launch per pass for all size groups, otherwise one launch
per pass per group) must give exactly what each realization gives on its own, and match the
oracle."""
import numpy as np
import pytest

from golden_util import rel

pytestmark = pytest.mark.gpu


def _params(precision):
    from pspectcosmo_gb300.params import Params

    rng = np.random.default_rng(12345)
    ps = []
    for N, count in ((16, 3), (32, 3), (64, 2)):
        for r in range(count):
            ps.append(Params.reference_default(N=N, vv=4, seed=1 + len(ps), precision=precision,
                                               initfield=[float(rng.uniform(10, 12)), 0.0]))
    return ps


@pytest.mark.parametrize("precision", [64, 32])
def test_batch_equals_individual_lattices(precision):
    from pspectcosmo_gb300 import Ensemble, Lattice

    ps = _params(precision)
    ens = Ensemble(ps)
    assert len(ens) == len(ps) and ens.groups == 3
    ens.initialize()
    ens.evolve(1e-4, 7)
    for idx, p in enumerate(ps):
        lat = Lattice(p)
        lat.initialize()
        lat.evolve(1e-4, 7)
        a, b = ens.get_state(idx), lat.get_state()
        assert rel(a["f_k"], b["f_k"]) == 0.0 and rel(a["pi_k"], b["pi_k"]) == 0.0, idx
        assert a["a"] == b["a"] and a["ad"] == b["ad"] and a["add"] == b["add"], idx
        sa, sb = ens.spectra_raw(idx), lat.spectra_raw()
        assert np.array_equal(sa["numpoints"], sb["numpoints"])
        assert rel(sa["f2"], sb["f2"]) < 1e-12
        ea, eb = ens.energies(idx), lat.energies()
        assert rel(ea["K"], eb["K"]) < 1e-14 and rel(ea["V"], eb["V"]) < 1e-14


def test_batch_fp64_matches_oracle(oracle_mod):
    from pspectcosmo_gb300 import Ensemble

    ps = _params(64)
    ens = Ensemble(ps)
    ens.initialize()
    ens.evolve(1e-4, 5)
    for idx in (0, 4, 7):
        o = oracle_mod.Oracle(ps[idx])
        o.init_ic()
        o.step(1e-4, 5)
        f, pi, _, _ = o.state_k()
        st = ens.get_state(idx)
        assert rel(st["f_k"], f) < 1e-10 and rel(st["pi_k"], pi) < 1e-10
        assert rel(st["a"], o.bg()["a"]) < 1e-12


@pytest.mark.parametrize("precision", [64, 32])
def test_batch_with_gw_equals_individual_lattices(precision):
    """Two-field preheating with GWs on the register engine (32^3 and 64^3 groups, the GW
    Z pass with realizations on blockIdx.z): each realization of the batch equals the same
    lattice advanced alone, bit for bit."""
    from pspectcosmo_gb300 import Ensemble, Lattice
    from pspectcosmo_gb300.params import Params

    ps = [Params.preheating(N=N, vv=4, spectral=0, with_gw=1, seed=1 + i, precision=precision)
          for i, N in enumerate((32, 32, 32, 64, 64))]
    ens = Ensemble(ps)
    assert ens.groups == 2
    assert ens.launch_mode(per_group=False)   # one launch per pass for both groups
    ens.initialize()
    ens.evolve(0.005, 4)
    for idx, p in enumerate(ps):
        lat = Lattice(p)
        lat.initialize()
        lat.evolve(0.005, 4)
        a, b = ens.get_state(idx), lat.get_state()
        for k in ("f_k", "pi_k", "u_k", "pi_u_k"):
            assert np.array_equal(a[k], b[k]), (idx, k)
        assert a["a"] == b["a"] and a["ad"] == b["ad"] and a["add"] == b["add"], idx
        lat.close()


def _mixed(precision):
    from pspectcosmo_gb300.params import Params

    rng = np.random.default_rng(7)
    ps = []
    for N, count in ((32, 4), (64, 3), (128, 1), (256, 1)):
        for _ in range(count):
            ps.append(Params.reference_default(N=N, vv=4, seed=1 + len(ps), precision=precision,
                                               initfield=[float(rng.uniform(10, 12)), 0.0]))
    return ps


@pytest.mark.parametrize("precision", [64, 32])
def test_one_launch_per_pass_equals_individual_lattices(precision):
    """Four size groups (32^3 .. 256^3) in one launch per pass: every realization equals the
    lattice advanced alone, bit for bit, and the per-group launches give the same bits."""
    from pspectcosmo_gb300 import Ensemble, Lattice

    ps = _mixed(precision)
    ens = Ensemble(ps)
    assert ens.groups == 4 and not ens.launch_mode() and ens.launch_mode(per_group=False)
    ens.initialize()
    ens.evolve(1e-4, 5)
    states = [ens.get_state(i) for i in range(len(ps))]
    for idx in (0, 3, 4, 7, 8):
        lat = Lattice(ps[idx])
        lat.initialize()
        lat.evolve(1e-4, 5)
        a, b = states[idx], lat.get_state()
        assert np.array_equal(a["f_k"], b["f_k"]) and np.array_equal(a["pi_k"], b["pi_k"]), idx
        assert a["a"] == b["a"] and a["ad"] == b["ad"] and a["add"] == b["add"], idx
        lat.close()
    ens.close()
    per = Ensemble(ps)
    assert not per.launch_mode(per_group=True)
    per.initialize()
    per.evolve(1e-4, 5)
    for idx in (1, 5, 8):
        b = per.get_state(idx)
        assert np.array_equal(states[idx]["f_k"], b["f_k"]) and states[idx]["a"] == b["a"], idx
    per.close()


@pytest.mark.parametrize("precision", [64, 32])
def test_mixed_radix_group_equals_individual_lattices(precision):
    """A batch with a group at a size that is not a power of two (24^3: the generic engine's
    radix 3) beside a register-engine group (32^3), GWs on: every realization equals the
    same lattice advanced alone, bit for bit."""
    from pspectcosmo_gb300 import Ensemble, Lattice
    from pspectcosmo_gb300.params import Params

    ps = [Params.preheating(N=N, vv=4, spectral=0, with_gw=1, seed=1 + i, precision=precision)
          for i, N in enumerate((24, 24, 32))]
    ens = Ensemble(ps)
    assert ens.groups == 2
    ens.initialize()
    ens.evolve(0.005, 3)
    for idx, p in enumerate(ps):
        lat = Lattice(p)
        lat.initialize()
        lat.evolve(0.005, 3)
        a, b = ens.get_state(idx), lat.get_state()
        for k in ("f_k", "pi_k", "u_k", "pi_u_k"):
            assert np.array_equal(a[k], b[k]), (idx, k)
        assert a["a"] == b["a"] and a["ad"] == b["ad"] and a["add"] == b["add"], idx
        lat.close()
    ens.close()
