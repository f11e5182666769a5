"""psc_spectra_noalloc: the scalar spectrum for callers that cannot allocate device memory.

Such a caller (an application whose own pool owns the GPU memory, or code that must not
allocate while it runs) passes its own device arrays; the entry point keeps its bin
accumulators in a fixed array inside the library and calls no cudaMalloc. This test gives
it device copies of a lattice's state (made here with torch, as such a caller would
provide them), calls it twice in a row through the C ABI, and checks both results
against the handle-based psc_spectra: bin counts exactly, per-bin means to 1e-12 relative
(the two differ only in the order of floating-point atomic additions). The second call
must leave the device's free memory unchanged (cudaMemGetInfo before and after): it
allocates nothing. Sizes 16^3 to 64^3, FP64 and FP32, on the default stream and on a
stream of the caller's.

This file sorts last so that a run stopping at its first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    f = lib.psc_spectra_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.mark.parametrize("N,precision,own_stream", [(32, 64, False), (32, 32, False), (16, 64, True),
                                                    (64, 32, True)])
def test_noalloc_spectra_match_handle_spectra(N, precision, own_stream):
    torch = pytest.importorskip("torch")
    from pspectcosmo_gb300 import Lattice, load_library
    from pspectcosmo_gb300.params import Params

    lib = load_library()
    fn = _noalloc(lib)
    p = Params.preheating(N=N, precision=precision)
    lat = Lattice(p)
    lat.initialize()
    lat.evolve(0.005, 4)
    ref = lat.spectra_raw()
    st = lat.get_state()

    cdt = torch.complex64 if precision == 32 else torch.complex128
    dev = torch.device("cuda:0")
    f_k = torch.from_numpy(st["f_k"]).to(cdt).to(dev).contiguous()
    pi_k = torch.from_numpy(st["pi_k"]).to(cdt).to(dev).contiguous()
    stream = torch.cuda.Stream(device=dev) if own_stream else None
    handle = ctypes.c_void_p(stream.cuda_stream) if own_stream else None
    nb = p.maxnumbins
    for call in range(2):
        numpoints = torch.full((p.nflds, nb), -1, dtype=torch.int32, device=dev)
        f2 = torch.full((p.nflds, nb), np.nan, dtype=torch.float64, device=dev)
        pi2 = torch.full_like(f2, np.nan)
        n2 = torch.full_like(f2, np.nan)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc = fn(ctypes.byref(p), st["a"], st["ad"], f_k.data_ptr(), pi_k.data_ptr(), numpoints.data_ptr(),
                f2.data_ptr(), pi2.data_ptr(), n2.data_ptr(), handle)
        assert rc == 0, lib.psc_last_error()
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(dev)[0]
        if call == 1:   # the first call may load the library's device code into the context
            assert free_after == free_before, f"device free memory changed by {free_before - free_after} bytes"
        assert np.array_equal(numpoints.cpu().numpy(), ref["numpoints"]), f"bin counts, call {call}"
        for name, got in (("f2", f2), ("pi2", pi2), ("n2", n2)):
            g = got.cpu().numpy()
            r = ref[name]
            assert np.all(np.isfinite(g)), name
            err = np.abs(g - r).max() / np.abs(r).max()
            assert err < 1e-12, f"{name} differs by {err:.3e} on call {call}"
    lat.close()


def test_noalloc_rejects_sizes_beyond_its_limit():
    from pspectcosmo_gb300 import load_library
    from pspectcosmo_gb300.params import Params

    lib = load_library()
    fn = _noalloc(lib)
    p = Params.reference_default(N=2048)
    dummy = ctypes.c_void_p(16)
    assert fn(ctypes.byref(p), 1.0, 1.0, dummy, dummy, None, None, None, None, None) == -1
    assert b"PSC_NOALLOC_MAX_N" in lib.psc_last_error()
