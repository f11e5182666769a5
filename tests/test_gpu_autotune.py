"""The FFT tile / grid autotuner (psc_autotune) and every shape it can choose.

Each candidate shape of the register-engine passes (X/Y lines per tile, Z lines per tile,
Z blocks per SM) must compute the step: FP64 runs of the 64^3 two-field + GW lattice in every
candidate shape agree with the default shapes to 1e-12 (only the order of the K, G, <V>
partial sums differs), and an autotuned 128^3 FP32 lattice with the default one to FP32
rounding. The choice is cached per configuration, in the process and, through
PSC_TUNE_CACHE, across processes.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from golden_util import rel

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _pair_state(p, nsteps=3):
    from pspectcosmo_gb300 import Lattice

    lat = Lattice(p)
    lat.initialize()
    return lat


def _candidates(default):
    xy, z, k = default
    for s in range(xy, max(xy - 2, 2) - 1, -1):
        yield (s, z, k)
    for s in range(z, max(z - 2, 0) - 1, -1):
        for kk in range(k, 0, -1):
            yield (xy, s, kk)


@pytest.mark.parametrize("with_gw", [1, 0])
def test_every_candidate_shape_computes_the_step(with_gw):
    from pspectcosmo_gb300 import Params

    p = Params.preheating(N=64, vv=4, spectral=0 if with_gw else 1, with_gw=with_gw, precision=64)
    ref = _pair_state(p)
    s0 = ref.get_state()
    default = ref.shapes
    assert all(x >= 0 for x in default)
    ref.evolve(0.005, 3)
    sref = ref.get_state()
    ref.close()
    seen = 0
    for shape in _candidates(default):
        lat = _pair_state(p)
        lat.set_state(s0["f_k"], s0["pi_k"], s0["a"], s0["ad"], s0["add"], s0["u_k"], s0["pi_u_k"])
        lat.shapes = shape
        assert lat.shapes == shape
        lat.evolve(0.005, 3)
        st = lat.get_state()
        for k in ("f_k", "pi_k") + (("u_k", "pi_u_k") if with_gw else ()):
            assert rel(st[k], sref[k]) < 1e-12, (shape, k)
        assert rel(st["a"], sref["a"]) < 1e-14, shape
        lat.close()
        seen += 1
    assert seen >= 3


def test_autotuned_lattice_matches_default_fp32():
    from pspectcosmo_gb300 import Lattice, Params

    p = Params.preheating(N=128, vv=4, spectral=0, with_gw=1, precision=32)
    a = Lattice(p)
    a.initialize()
    s0 = a.get_state()
    res = a.autotune(reps=2)
    assert len(res["shape"]) == 3 and all(x >= 0 for x in res["shape"])
    assert a.shapes == res["shape"]
    a.evolve(0.005, 4)
    sa = a.get_state()
    b = Lattice(p)
    b.set_state(s0["f_k"], s0["pi_k"], s0["a"], s0["ad"], s0["add"], s0["u_k"], s0["pi_u_k"])
    b.evolve(0.005, 4)
    sb = b.get_state()
    for k in ("f_k", "pi_k", "u_k", "pi_u_k"):
        assert rel(sa[k], sb[k]) < 1e-5, k
    # same configuration: the cached choice, without timing
    c = Lattice(p)
    c.initialize()
    r2 = c.autotune()
    assert r2["from_cache"] and r2["shape"] == res["shape"]
    for x in (a, b, c):
        x.close()


def test_small_lattices_have_nothing_to_tune():
    from pspectcosmo_gb300 import Lattice, Params

    lat = Lattice(Params.preheating(N=16, precision=64))
    lat.initialize()
    assert lat.autotune()["shape"] == (-1, -1, -1)
    lat.close()


def test_tune_cache_file_across_processes(tmp_path):
    cache = tmp_path / "tune.txt"
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from pspectcosmo_gb300 import Lattice, Params\n"
            "lat = Lattice(Params.preheating(N=64, vv=2, spectral=1, with_gw=0, precision=32))\n"
            "lat.initialize()\n"
            "r = lat.autotune(reps=1)\n"
            "print(int(r['from_cache']), *r['shape'])\n") % ROOT
    env = dict(os.environ, PSC_TUNE_CACHE=str(cache))
    out1 = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True).stdout
    assert cache.exists() and cache.read_text().strip()
    out2 = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True).stdout
    a, b = out1.split(), out2.split()
    assert a[0] == "0" and b[0] == "1" and a[1:] == b[1:]


def test_batch_autotune_matches_lone_lattices():
    """A batch group tuned as a whole advances each realization as the lone lattice does (to
    FP32 rounding: the tuned shapes order the reductions differently)."""
    from pspectcosmo_gb300 import Ensemble, Lattice, Params

    ps = [Params.reference_default(N=32, vv=4, precision=32, seed=s + 1) for s in range(4)]
    ens = Ensemble(ps)
    ens.initialize()
    ens.autotune(reps=1)
    ens.evolve(1e-4, 3)
    st = ens.get_state(2)
    ens.close()
    lat = Lattice(ps[2])
    lat.initialize()
    lat.evolve(1e-4, 3)
    sl = lat.get_state()
    assert rel(st["f_k"], sl["f_k"]) < 1e-5 and rel(st["pi_k"], sl["pi_k"]) < 1e-5
    lat.close()
