"""The reference's spectral zero-padding (padding / extract_padding, evolution.cpp:1271-1609):
the loop restatement in oracle/pad_ref.py against the closed-form index map the device
kernels use (pspectcosmo_gb300/csrc/psc_pad.cu), on the CPU."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import pad_ref  # noqa: E402


def scatter_map(src, Ns, Nd, scale=1.0):
    """k_pad_scatter: each source mode to its 1, 2 or 4 images, 1/2 per Nyquist axis."""
    h, Hd = Ns // 2, Nd // 2 + 1
    dst = np.zeros((Nd, Nd, Hd), dtype=src.dtype)
    s = src.reshape(Ns, Ns, h + 1)
    for i in range(Ns):
        for j in range(Ns):
            for kz in range(h + 1):
                f = scale * (0.5 if i == h else 1) * (0.5 if j == h else 1) * (0.5 if kz == h else 1)
                v = s[i, j, kz] * f
                I0 = i if i <= h else Nd - (Ns - i)
                J0 = j if j <= h else Nd - (Ns - j)
                Is = [I0] + ([Nd - h] if i == h else [])
                Js = [J0] + ([Nd - h] if j == h else [])
                for I in Is:
                    for J in Js:
                        assert 0 <= I < Nd and 0 <= J < Nd and kz < Hd
                        assert dst[I, J, kz] == 0
                        dst[I, J, kz] = v
    return dst


def extract_map(pad, N, Np):
    """k_pad_kick's read of V'_k_pad: the +N/2 image, x 2 per Nyquist axis, / (Np/N)^3 (a
    division, as evolution.cpp:1602: exact for power-of-two ratios, rounded as the reference
    rounds for the others)."""
    h = N // 2
    p = pad.reshape(Np, Np, Np // 2 + 1)
    out = np.zeros((N, N, h + 1), dtype=p.dtype)
    for i in range(N):
        for j in range(N):
            for kz in range(h + 1):
                I = i if i <= h else Np - (N - i)
                J = j if j <= h else Np - (N - j)
                g = (2 if i == h else 1) * (2 if j == h else 1) * (2 if kz == h else 1)
                out[i, j, kz] = p[I, J, kz] * g / (Np / N) ** 3
    return out


@pytest.mark.parametrize("N,Np", [(4, 8), (8, 16), (8, 32), (16, 32), (8, 12), (12, 20), (16, 24)])
def test_scatter_map_is_padding(N, Np):
    rng = np.random.default_rng(N * Np)
    fk = rng.standard_normal((N, N, N // 2 + 1)) + 1j * rng.standard_normal((N, N, N // 2 + 1))
    assert np.array_equal(scatter_map(fk, N, Np), pad_ref.padding(fk, N, Np))


@pytest.mark.parametrize("N,Np", [(4, 8), (8, 16), (8, 32), (16, 32), (8, 12), (12, 20), (16, 24)])
def test_extract_map_is_extract_padding(N, Np):
    rng = np.random.default_rng(N + Np)
    fkp = rng.standard_normal((Np, Np, Np // 2 + 1)) + 1j * rng.standard_normal((Np, Np, Np // 2 + 1))
    assert np.array_equal(extract_map(fkp, N, Np), pad_ref.extract_padding(fkp, N, Np))


def test_padding_interpolates_real_fields():
    rng = np.random.default_rng(3)
    N, Np = 8, 16
    f = rng.standard_normal((N, N, N))
    fk = np.fft.rfftn(f)
    fp = np.fft.irfftn(pad_ref.padding(fk, N, Np), s=(Np, Np, Np), axes=(0, 1, 2)) * (Np / N) ** 3
    assert np.abs(fp[::2, ::2, ::2] - f).max() < 1e-14
    # extract(padding(x)) = x (Np/N)^-3
    assert np.abs(pad_ref.extract_padding(pad_ref.padding(fk, N, Np), N, Np) * 8 - fk).max() < 1e-13
