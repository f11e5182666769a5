"""CPU restatement of the reference's spectral zero-padding (test infrastructure only).

padding()          evolution.cpp:1271-1443  half spectrum of an N lattice -> an N_pad one
extract_padding()  evolution.cpp:1446-1609  half spectrum of an N_pad lattice -> an N one

Loop-for-loop over the reference's index sets (numpy arrays [x][y][kz], kz fastest,
H = N/2 + 1). The product's device kernels (pspectcosmo_gb300/csrc/psc_pad.cu) compute
each output element from a closed-form index map; these loops check that map.
"""
from __future__ import annotations

import numpy as np


def padding(fk: np.ndarray, N: int, Np: int) -> np.ndarray:
    """f_k [N][N][N/2+1] -> f_k_pad [Np][Np][Np/2+1] (evolution.cpp:1271-1443)."""
    h = N // 2
    src = fk.reshape(N, N, h + 1)
    pad = np.zeros((Np, Np, Np // 2 + 1), dtype=src.dtype)

    def plane(k, scale):
        pad[0, 0, k] = src[0, 0, k] * scale if scale != 1 else src[0, 0, k]
        for j in range(1, h + 1):
            jp = Np - j
            for i in range(1, h + 1):
                ip = Np - i
                pad[i, j, k] = src[i, j, k] * scale
                pad[ip, j, k] = src[N - i, j, k] * scale
                pad[i, jp, k] = src[i, N - j, k] * scale
                pad[ip, jp, k] = src[N - i, N - j, k] * scale
        for i in range(1, h + 1):
            pad[i, 0, k] = src[i, 0, k] * scale
            pad[Np - i, 0, k] = src[N - i, 0, k] * scale
        for j in range(1, h + 1):
            pad[0, j, k] = src[0, j, k] * scale
            pad[0, Np - j, k] = src[0, N - j, k] * scale
        # Nyquist lines halved (corners twice)
        for j in range(1, h + 1):
            for (a, b) in ((h, j), (Np - h, j), (h, Np - j), (Np - h, Np - j)):
                pad[a, b, k] /= 2
        for i in range(1, h + 1):
            for (a, b) in ((i, h), (Np - i, h), (i, Np - h), (Np - i, Np - h)):
                pad[a, b, k] /= 2
        pad[h, 0, k] /= 2
        pad[Np - h, 0, k] /= 2
        pad[0, h, k] /= 2
        pad[0, Np - h, k] /= 2

    for k in range(h):
        plane(k, 1)
    # kz = N/2: copied with / 2 (src / 2 written, then the same line halvings)
    k = h
    pad[0, 0, k] = src[0, 0, k] / 2
    for j in range(1, h + 1):
        jp = Np - j
        for i in range(1, h + 1):
            ip = Np - i
            pad[i, j, k] = src[i, j, k] / 2
            pad[ip, j, k] = src[N - i, j, k] / 2
            pad[i, jp, k] = src[i, N - j, k] / 2
            pad[ip, jp, k] = src[N - i, N - j, k] / 2
    for i in range(1, h + 1):
        pad[i, 0, k] = src[i, 0, k] / 2
        pad[Np - i, 0, k] = src[N - i, 0, k] / 2
    for j in range(1, h + 1):
        pad[0, j, k] = src[0, j, k] / 2
        pad[0, Np - j, k] = src[0, N - j, k] / 2
    for j in range(1, h + 1):
        for (a, b) in ((h, j), (Np - h, j), (h, Np - j), (Np - h, Np - j)):
            pad[a, b, k] /= 2
    for i in range(1, h + 1):
        for (a, b) in ((i, h), (Np - i, h), (i, Np - h), (Np - i, Np - h)):
            pad[a, b, k] /= 2
    pad[h, 0, k] /= 2
    pad[Np - h, 0, k] /= 2
    pad[0, h, k] /= 2
    pad[0, Np - h, k] /= 2
    return pad


def extract_padding(fkp: np.ndarray, N: int, Np: int) -> np.ndarray:
    """V'_k_pad [Np][Np][Np/2+1] -> V'_k [N][N][N/2+1] (evolution.cpp:1446-1609)."""
    h = N // 2
    pad = fkp.reshape(Np, Np, Np // 2 + 1)
    out = np.zeros((N, N, h + 1), dtype=pad.dtype)

    def plane(k, mult):
        for j in range(1, h):
            jp = Np - j
            for i in range(1, h):
                ip = Np - i
                out[i, j, k] = pad[i, j, k] * mult
                out[N - i, j, k] = pad[ip, j, k] * mult
                out[i, N - j, k] = pad[i, jp, k] * mult
                out[N - i, N - j, k] = pad[ip, jp, k] * mult
        for j in (0, h):
            for i in range(1, h):
                out[i, j, k] = pad[i, j, k] * mult
                out[N - i, j, k] = pad[Np - i, j, k] * mult
        for i in (0, h):
            for j in range(1, h):
                out[i, j, k] = pad[i, j, k] * mult
                out[i, N - j, k] = pad[i, Np - j, k] * mult
        for i in (0, h):
            for j in (0, h):
                out[i, j, k] = pad[i, j, k] * mult
        out[:, h, k] *= 2
        out[h, :, k] *= 2

    for k in range(h):
        plane(k, 1)
    plane(h, 2)
    return out / (float(Np) / N) ** 3
