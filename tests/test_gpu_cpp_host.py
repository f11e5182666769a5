"""The C++ host (pspectcosmo_gb300/host/psc_run.cpp) compiled with g++ against libpsc.so and
run as a program, against the reference's own outputs:

* fixed step: 16^3 two-field preheating with GWs, Yoshida-4, FP64, 10 steps of 0.005 from
  the library's initial conditions; the final state it writes, taken to real space, equals
  the reference's final f, pi_f, u, pi_u (golden gw2_n16_vv4) to 1e-10 relative and its
  scale factor to 1e-12;
* the run loop: the shipped configuration at 16^3 to t = 0.02 with the reference's adaptive
  dt and output cadence; its text files equal those of the reference's own main()
  (golden drive1_n16) at the printed precision, as the Python run loop's do
  (tests/test_gpu_driver.py)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from golden_util import load, rel

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def psc_run(tmp_path_factory, psc_lib):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("host") / "psc_run")
    libdir = os.path.join(ROOT, "pspectcosmo_gb300")
    cmd = [gxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           os.path.join(libdir, "host", "psc_run.cpp"), "-L", libdir, "-lpsc", f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def read_state(path):
    raw = open(path, "rb").read()
    hdr = np.frombuffer(raw, np.int32, 4)
    assert hdr[0] == 0x53435350
    N, nf, gw = (int(x) for x in hdr[1:])
    modes = N * N * (N // 2 + 1)
    bg = np.frombuffer(raw, np.float64, 4, 16)
    off = 48
    out = {"t": bg[0], "a": bg[1], "ad": bg[2], "add": bg[3], "N": N}
    for name, n in (("f_k", nf), ("pi_k", nf)) + ((("u_k", 6), ("pi_u_k", 6)) if gw else ()):
        out[name] = np.frombuffer(raw, np.complex128, n * modes, off).reshape(n, N, N, N // 2 + 1)
        off += 16 * n * modes
    assert off == len(raw)
    return out


def test_cpp_host_fixed_step_matches_reference(psc_run, tmp_path):
    g, meta = load("gw2_n16_vv4")
    state = str(tmp_path / "state.bin")
    r = subprocess.run([psc_run, "preset=preheating", "N=16", "vv=4", "spectral=0", "with_gw=1", "precision=64",
                        "nsteps=10", "dt=0.005", f"state={state}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    st = read_state(state)
    N = st["N"]
    real = lambda k: np.fft.irfftn(k, s=(N, N, N), axes=(1, 2, 3))
    assert rel(real(st["f_k"]), g["fin_f"]) < 1e-10
    assert rel(real(st["pi_k"]), g["fin_pi_f"]) < 1e-10
    assert rel(real(st["u_k"]), g["fin_u"]) < 1e-10
    assert rel(real(st["pi_u_k"]), g["fin_pi_u"]) < 1e-10
    assert abs(st["t"] - 0.05) < 1e-12
    assert rel(st["a"], g["bg"][-1, 2]) < 1e-12


def test_cpp_host_run_loop_matches_reference_main(psc_run, tmp_path):
    from test_gpu_driver import blocks, close, rows

    g, meta = load("drive1_n16")
    d = str(tmp_path / "output")
    r = subprocess.run([psc_run, "N=16", "tf=0.02", "tOutputFreq=0.001", "tOutputInfreq=0.005", f"out={d}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    o = lambda name: os.path.join(d, name + ".txt")
    sc = rows(o("average_scalar_0"))
    ref = g["average_scalar_0"]
    assert sc.shape == ref.shape   # the same cadence: 21 frequent outputs
    assert np.array_equal(np.round(sc[:, 0], 3), np.round(ref[:, 0], 3))
    assert close(sc[:, 1:5], ref[:, 1:5])
    assert close(sc[:, 5:], ref[:, 5:], rtol=0, atol=1e-6)
    assert close(rows(o("average_scale_factor")), g["average_scale_factor"], atol=5e-7)
    assert close(rows(o("average_energies"))[:, 1:], g["average_energies"][:, 1:], atol=1e-12)
    ec = rows(o("average_energy_conservation"))
    assert close(ec[:, 2:], g["average_energy_conservation"][:, 2:], atol=5e-7)
    with open(o("average_spectra_times")) as fh:
        st = [ln.strip() for ln in fh if ln.strip()]
    assert st == [f"{x:.2f}" for x in g["average_spectra_times"].ravel()]
    sp = blocks(o("spectra_scalar_0"))
    assert sp.shape == g["spectra_scalar_0"].shape
    assert np.array_equal(sp[..., 4], g["spectra_scalar_0"][..., 4])
    assert close(sp[..., :4], g["spectra_scalar_0"][..., :4], rtol=1e-5, atol=1e-30)
