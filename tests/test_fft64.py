"""The oracle's FP64 FFT (the FFTW stand-in) against numpy.fft and a direct DFT: power-of-two
lengths (radix 2) and the mixed-radix lengths of other lattice sizes (factors 2, 3, 5, 7)."""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def fft(oracle_mod):
    L = ctypes.CDLL(oracle_mod.build())
    D = ctypes.POINTER(ctypes.c_double)
    L.fft64_r2c_3d.argtypes = [ctypes.c_int] * 3 + [D, D]
    L.fft64_c2r_3d.argtypes = [ctypes.c_int] * 3 + [D, D]
    L.fft64_c2c_line.argtypes = [D, ctypes.c_int, ctypes.c_long, ctypes.c_int]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@pytest.mark.parametrize("n", [2, 4, 8, 16, 64, 256, 1024, 3, 6, 12, 20, 24, 28, 30, 42, 49, 96, 210, 480])
def test_line_vs_direct_dft(fft, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    k = np.arange(n)
    ref = np.exp(-2j * np.pi * np.outer(k, k) / n) @ x
    y = x.copy()
    fft.fft64_c2c_line(_p(y.view(np.float64)), n, 1, -1)
    assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max() * max(1, np.log2(n))
    z = x.copy()
    fft.fft64_c2c_line(_p(z.view(np.float64)), n, 1, +1)
    assert np.allclose(z, np.fft.ifft(x) * n, rtol=0, atol=1e-12 * np.abs(x).sum())


@pytest.mark.parametrize("shape", [(8, 8, 8), (16, 16, 16), (32, 32, 32), (8, 16, 32), (12, 12, 12), (20, 20, 20),
                                   (24, 24, 24), (28, 28, 28), (30, 12, 42)])
def test_3d_real_transforms_match_numpy(fft, shape):
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape)
    out = np.zeros(shape[:2] + (shape[2] // 2 + 1,), np.complex128)
    fft.fft64_r2c_3d(*shape, _p(x), _p(out.view(np.float64)))
    ref = np.fft.rfftn(x)
    assert np.abs(out - ref).max() < 1e-12 * np.abs(ref).max()
    back = np.zeros(shape)
    fft.fft64_c2r_3d(*shape, _p(out.view(np.float64)), _p(back))
    assert np.abs(back / np.prod(shape) - x).max() < 1e-13


def test_c2r_ignores_imaginary_dc_and_nyquist(fft):
    """FFTW's c2r reads only X[0..N/2] and drops Im X[0], Im X[N/2]."""
    n = 8
    rng = np.random.default_rng(3)
    X = rng.standard_normal((n, n, n // 2 + 1)) + 1j * rng.standard_normal((n, n, n // 2 + 1))
    X2 = X.copy()
    X2[:, :, 0] = X[:, :, 0]  # same
    out1 = np.zeros((n, n, n))
    fft.fft64_c2r_3d(n, n, n, _p(X.view(np.float64)), _p(out1))
    ref = np.fft.irfftn(X, s=(n, n, n), axes=(0, 1, 2)) * n ** 3
    assert np.abs(out1 - ref).max() < 1e-11
