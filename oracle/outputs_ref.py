"""CPU restatement of the reference's output-step quantities of the real-space fields.

Test infrastructure only (the oracle): the product computes these on the device
(pspectcosmo_gb300/csrc/psc_outputs.cu). Pinned against the reference's own outputs
(tests/golden/snap2_n16_vv4.npz: its histogram files and the raw snapshot datasets).

  histograms()              output.cpp:1193-1297
  histograms_2d()           output.cpp:1300-1413
  slices()                  output.cpp:1415-1539
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


def histogram_2d(f1: np.ndarray, f2: np.ndarray, nbins0: int = 10, nbins1: int = 10, hmin: float = 0.0,
                 hmax: float = 0.0):
    """One field pair (output.cpp:1369-1410): binfreq [nbins0][nbins1] (counts / N^3, not /
    the points binned), bmin [2], df [2]."""
    x, y = np.asarray(f1, np.float64).ravel(), np.asarray(f2, np.float64).ravel()
    if hmax == hmin:
        bmin = [float(x.min()), float(y.min())]
        bmax = [float(x.max()), float(y.max())]
    else:
        bmin, bmax = [float(hmin)] * 2, [float(hmax)] * 2
    df = [(bmax[0] - bmin[0]) / float(nbins0), (bmax[1] - bmin[1]) / float(nbins1)]
    with np.errstate(divide="ignore", invalid="ignore"):
        b0 = _c_int_cast((x - bmin[0]) / df[0])
        b1 = _c_int_cast((y - bmin[1]) / df[1])
    b0[x == bmax[0]] = nbins0 - 1
    b1[y == bmax[1]] = nbins1 - 1
    keep = (b0 >= 0) & (b0 < nbins0) & (b1 >= 0) & (b1 < nbins1)
    counts = np.bincount(b0[keep] * nbins1 + b1[keep], minlength=nbins0 * nbins1).astype(np.float64)
    return (counts / float(x.size)).reshape(nbins0, nbins1), np.array(bmin), np.array(df)


def slices(f: np.ndarray, slicedim: int = 1, slicelength: int | None = None, sliceskip: int = 1,
           sliceaverage: int = 1) -> np.ndarray:
    """One field's slice values in output order (output.cpp:1456-1534): the first slicedim
    axes from the origin (x = y = 0 for a line, x = 0 for a plane), every sliceskip-th point
    up to slicelength * sliceskip (at most N), each optionally the mean of its skip block
    (the 3-D case multiplies by 1/numpts, the others divide)."""
    N = f.shape[0]
    slicelength = N if slicelength is None else slicelength
    dim = min(slicedim, 3)
    final = min(slicelength * sliceskip, N)
    out = []
    starts = range(0, final, sliceskip)
    if dim == 1:
        for k in starts:
            if sliceaverage == 1:
                v, n = 0.0, 0
                for z in range(k, min(k + sliceskip, N)):
                    v += f[0, 0, z]
                    n += 1
                out.append(v / float(n))
            else:
                out.append(f[0, 0, k])
    elif dim == 2:
        for j in starts:
            for k in starts:
                if sliceaverage == 1:
                    v, n = 0.0, 0
                    for y in range(j, min(j + sliceskip, N)):
                        for z in range(k, min(k + sliceskip, N)):
                            v += f[0, y, z]
                            n += 1
                    out.append(v / float(n))
                else:
                    out.append(f[0, j, k])
    else:
        for i in starts:
            for j in starts:
                for k in starts:
                    if sliceaverage == 1:
                        v, n = 0.0, 0
                        for x in range(i, min(i + sliceskip, N)):
                            for y in range(j, min(j + sliceskip, N)):
                                for z in range(k, min(k + sliceskip, N)):
                                    v += f[x, y, z]
                                    n += 1
                        out.append(v * (1 / float(n)))
                    else:
                        out.append(f[i, j, k])
    return np.array(out)
