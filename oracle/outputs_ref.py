"""CPU restatement of the reference's output-step quantities of the real-space fields.

Test infrastructure only (the oracle): the product computes these on the device
(pspectcosmo_gb300/csrc/psc_outputs.cu). Pinned against the reference's own outputs
(tests/golden/snap2_n16_vv4.npz: its histogram files and the raw snapshot datasets).

  histograms()              output.cpp:1193-1297
  kinetic_energy_lattice    evolution.cpp:7-19
  gradient_energy_lattice   evolution.cpp:23-138
  snapshot energies         output.cpp:1614-1627
"""
from __future__ import annotations

import numpy as np


def _c_int_cast(q: np.ndarray) -> np.ndarray:
    """(int)q of a C double on x86-64: truncation toward zero; NaN and values outside
    the int range give INT_MIN."""
    out = np.full(q.shape, np.iinfo(np.int32).min, dtype=np.int64)
    ok = np.isfinite(q) & (q > -2147483649.0) & (q < 2147483648.0)
    out[ok] = np.trunc(q[ok]).astype(np.int64)
    return out


def histogram(f: np.ndarray, nbins: int = 256, hmin: float = 0.0, hmax: float = 0.0):
    """One field's histogram (output.cpp:1244-1279): (binfreq[nbins], bmin, df)."""
    x = np.asarray(f, dtype=np.float64).ravel()
    if hmax == hmin:
        bmin, bmax = float(x.min()), float(x.max())
    else:
        bmin, bmax = float(hmin), float(hmax)
    df = (bmax - bmin) / float(nbins)
    with np.errstate(divide="ignore", invalid="ignore"):
        binnum = _c_int_cast((x - bmin) / df)
    binnum[x == bmax] = nbins - 1
    keep = (binnum >= 0) & (binnum < nbins)
    counts = np.bincount(binnum[keep], minlength=nbins).astype(np.float64)
    numpts = float(keep.sum())
    with np.errstate(divide="ignore", invalid="ignore"):
        return counts / numpts, bmin, df


def histograms(f_all: np.ndarray, nbins: int = 256, hmin: float = 0.0, hmax: float = 0.0):
    """All fields: binfreq [nflds][nbins], bmin [nflds], df [nflds]."""
    res = [histogram(f, nbins, hmin, hmax) for f in f_all]
    return (np.array([r[0] for r in res]), np.array([r[1] for r in res]), np.array([r[2] for r in res]))


def derivative(f: np.ndarray, axis: int, kIR: float) -> np.ndarray:
    """1-D spectral derivative along `axis` (evolution.cpp:34-63): r2c, multiply by
    i kIR k (k = 0 .. N/2-1), Nyquist bin zeroed, c2r, / N."""
    N = f.shape[axis]
    F = np.fft.rfft(f, axis=axis)
    k = np.arange(N // 2 + 1, dtype=np.float64) * kIR
    k[N // 2] = 0.0
    shape = [1] * f.ndim
    shape[axis] = N // 2 + 1
    return np.fft.irfft(F * (1j * k.reshape(shape)), n=N, axis=axis)


def potential_density(f_all: np.ndarray, model: int, gsq: float) -> np.ndarray:
    """Sum over the model's terms of potential_energy(term, f(x)) (output.cpp:1618-1625;
    model.h:35-72 for phi^2, the two-field phi^2 chi^2 model for model 1)."""
    phi = f_all[0]
    v = 0.0 + 0.5 * (phi * phi)
    if model == 1:
        chi = f_all[1]
        v = v + 0.5 * gsq * (phi * phi) * (chi * chi)
    return v


def lattice_energies(f_all: np.ndarray, pi_all: np.ndarray, a: float, kIR: float, model: int, gsq: float) -> dict:
    """The SNAPSHOTS_ENERGY datasets: pot, kin (a^6/2 sum pi^2), grad (a^2/2 sum over
    fields and axes of (d_i f)^2) and tot = pot + kin + grad."""
    pot = potential_density(f_all, model, gsq)
    kin = np.zeros_like(pot)
    for p in pi_all:
        kin = kin + p * p
    kin = kin * (a ** 6 / 2.0)
    grad = np.zeros_like(pot)
    for f in f_all:
        for ax in range(3):
            d = derivative(f, ax, kIR)
            grad = grad + d * d
    grad = grad * (a * a / 2.0)
    return dict(pot=pot, kin=kin, grad=grad, tot=pot + kin + grad)
