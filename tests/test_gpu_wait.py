"""Failure detection of the device-side waits. The GW Z pass waits for its bulk copies (TMA)
on an mbarrier for a bounded time.

* The self-test entry point runs that wait on an mbarrier whose transactions never arrive
  (nothing sets it) and checks that the kernel gives up with PSC_ERR_TIMEOUT within its
  limit; the GPU context stays usable for a step that takes the bulk-copy path.
* The real path: a test hook makes every tile of the GW Z pass expect 16 bytes more than its
  copies deliver, with a 20 ms limit. The copies land, the wait runs out, the block counts
  the planted bytes itself and leaves, and psc_step returns PSC_ERR_TIMEOUT. With the hook
  off, the same handle then evolves the oracle's initial state and matches the oracle.
No GPU fault is used: every copy targets valid memory and every wait is bounded."""
import ctypes
import time

import numpy as np
import pytest

from golden_util import rel

pytestmark = pytest.mark.gpu

PSC_ERR_CONFIG = -1
PSC_ERR_TIMEOUT = -5


def test_bounded_bulk_wait_runs_out_and_the_context_survives():
    from pspectcosmo_gb300 import Lattice, Params, load_library

    L = load_library()
    status = ctypes.c_int(0)
    t0 = time.perf_counter()
    rc = L.psc_selftest_bulk_wait(ctypes.c_double(50.0), ctypes.byref(status))
    elapsed = time.perf_counter() - t0
    assert rc == 0
    assert status.value == PSC_ERR_TIMEOUT
    assert elapsed < 5.0

    lat = Lattice(Params.preheating(N=32, vv=2, spectral=0, with_gw=1, precision=32))
    lat.initialize()
    lat.evolve(0.005, 2)   # the FP32 GW Z pass stages by bulk copies at this size (TL even)
    bg = lat.background()
    assert np.isfinite(bg["a"]) and np.isfinite(bg["add"])


def test_zpass_wait_runs_out_on_the_real_path_and_the_handle_recovers(oracle_mod):
    from pspectcosmo_gb300 import Lattice, Params, PscError, load_library

    L = load_library()
    N = 32
    p = Params.preheating(N=N, vv=4, spectral=0, with_gw=1, precision=32)
    # the GW Z pass of this handle stages by bulk copies: 256 threads over nf x 4 input lines
    # of N/32 threads give TL = 32 lines per tile, and TL x (N/2 + 1) complex FP32 values
    # (4352 bytes) is a multiple of 16 bytes
    tl = 256 // (p.nflds * 4 * max(1, N // 32))
    assert (tl * (N // 2 + 1) * 8) % 16 == 0
    q = p.copy()
    q.precision = 64
    o = oracle_mod.Oracle(q)
    o.init_ic()
    f0, pi0, u0, pu0 = o.state_k()
    bg0 = o.bg()
    lat = Lattice(p)
    lat.set_state(f0, pi0, bg0["a"], bg0["ad"], bg0["add"], u0, pu0)

    assert L.psc_test_wait_hook(lat._h, ctypes.c_double(20.0), 16) == 0
    t0 = time.perf_counter()
    with pytest.raises(PscError) as ei:
        lat.evolve(0.005, 3)
    elapsed = time.perf_counter() - t0
    assert ei.value.code == PSC_ERR_TIMEOUT
    assert elapsed < 10.0   # one limit per block wave; the rest of the call does no work

    # hook off: the handle evolves the same initial state and matches the oracle
    assert L.psc_test_wait_hook(lat._h, ctypes.c_double(1000.0), 0) == 0
    lat.set_state(f0, pi0, bg0["a"], bg0["ad"], bg0["add"], u0, pu0)
    lat.evolve(0.005, 3)
    o.step(0.005, 3)
    st = lat.get_state()
    of, opi, ou, opu = o.state_k()
    for name, x, y in (("f_k", st["f_k"], of), ("pi_k", st["pi_k"], opi), ("u_k", st["u_k"], ou),
                       ("pi_u_k", st["pi_u_k"], opu)):
        assert rel(x, y) < 2e-4, name
    assert rel(st["a"], o.bg()["a"]) < 1e-6
    lat.close()

    # the hook refuses a handle whose Z pass does not stage by bulk copies (FP64 GW)
    lat64 = Lattice(q)
    assert L.psc_test_wait_hook(lat64._h, ctypes.c_double(20.0), 16) == PSC_ERR_CONFIG
    lat64.close()
