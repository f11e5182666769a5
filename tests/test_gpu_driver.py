"""The run loop (pspectcosmo_gb300.driver.run: calculate_dt, output cadence, save(),
save_Freq(), save_Infreq()) against the reference's own main() run to t = 0.02 on the
shipped configuration at 16^3 (golden drive1_n16: its text files at 17 digits).

The files written here carry the reference's 6-digit formatting, so values compare at
5e-6 relative (or half a unit of the last printed fixed digit); the rms columns of
average_scalar (sqrt(<f^2> - <f>^2) of a field with mean 11: cancellation) and the Friedmann
violation (a ratio of ~1e-12 differences) compare in absolute terms."""
import os

import numpy as np
import pytest

from golden_util import load

pytestmark = pytest.mark.gpu


def rows(path):
    with open(path) as fh:
        return np.array([[float(x) for x in ln.split()] for ln in fh if ln.strip()])


def blocks(path):
    out, cur = [], []
    with open(path) as fh:
        for ln in fh:
            if not ln.strip():
                if cur:
                    out.append(cur)
                    cur = []
                continue
            cur.append([float(x) for x in ln.split()])
    if cur:
        out.append(cur)
    return np.array(out)


def close(a, b, rtol=5e-6, atol=0.0):
    return np.all(np.abs(a - b) <= rtol * np.abs(b) + atol)


def test_run_loop_matches_reference_main(tmp_path):
    from pspectcosmo_gb300 import Params
    from pspectcosmo_gb300.driver import run

    g, meta = load("drive1_n16")
    d = str(tmp_path / "output")
    p = Params.reference_default(N=16)
    run(p, tf=0.02, tOutputFreq=0.001, tOutputInfreq=0.005, dir_=d)
    o = lambda name: os.path.join(d, name + ".txt")

    sc = rows(o("average_scalar_0"))
    ref = g["average_scalar_0"]
    assert sc.shape == ref.shape   # same cadence: 21 frequent outputs
    assert np.array_equal(np.round(sc[:, 0], 3), np.round(ref[:, 0], 3))
    assert close(sc[:, 1:5], ref[:, 1:5])
    assert close(sc[:, 5:], ref[:, 5:], rtol=0, atol=1e-6)
    sf = rows(o("average_scale_factor"))
    assert sf.shape == g["average_scale_factor"].shape
    assert close(sf, g["average_scale_factor"], atol=5e-7)
    en = rows(o("average_energies"))
    assert close(en[:, 1:], g["average_energies"][:, 1:], atol=1e-12)
    ec = rows(o("average_energy_conservation"))
    assert close(ec[:, 2:], g["average_energy_conservation"][:, 2:], atol=5e-7)
    assert np.all(np.abs(ec[:, 1] - g["average_energy_conservation"][:, 1]) < 1e-8)

    # 5 infrequent outputs; the times as the reference prints them (fixed, Infreq_prec = 2)
    with open(o("average_spectra_times")) as fh:
        st = [ln.strip() for ln in fh if ln.strip()]
    assert st == [f"{x:.2f}" for x in g["average_spectra_times"].ravel()]
    sp = blocks(o("spectra_scalar_0"))
    assert sp.shape == g["spectra_scalar_0"].shape
    assert np.array_equal(sp[..., 4], g["spectra_scalar_0"][..., 4])
    assert close(sp[..., :4], g["spectra_scalar_0"][..., :4], rtol=1e-5, atol=1e-30)
    ht = rows(o("histogramtimes"))
    assert close(ht, g["histogramtimes"], atol=5e-7)
    hb = blocks(o("histogram0"))[..., 0]
    assert hb.shape == g["histogram0"].shape
    npts = 16 ** 3
    moved = np.abs(np.rint(hb * npts) - np.rint(g["histogram0"] * npts)).sum(axis=1)
    assert np.all(moved <= 4)
    # info.txt (output_parameters) up to its clock lines, character for character
    with open(o("info")) as fh:
        info = fh.read()
    assert info.split("\nRun began at")[0] == meta["info"]
    assert "Run ended at" in info and " took " in info

