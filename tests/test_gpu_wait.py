"""Failure detection of the device-side waits. The GW Z pass waits for its bulk copies (TMA)
on an mbarrier for a bounded time; the self-test entry point runs that wait on an mbarrier
whose transactions never arrive (nothing sets it), checks that the kernel gives up with
PSC_ERR_TIMEOUT within its limit, and the GPU context stays usable for a step that takes
the bulk-copy path."""
import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

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
