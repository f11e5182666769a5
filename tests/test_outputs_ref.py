"""Output-step oracle (histograms, lattice energy densities) pinned to the reference's own
outputs, and the HDF5 snapshot writer checked structurally (CPU only).

The golden run snap2_n16_vv4 is the reference's code (two-field preheating, 16^3,
Yoshida-4, spectral step) with snapshots on: its histogram files and the raw datasets
its snapshots() wrote at step 20."""
import os

import numpy as np
import pytest

import h5read
from golden_util import load, rel

SCIPY_H5 = None
try:
    import scipy

    _p = os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data", "testhdf5_7.4_GLNX86.mat")
    SCIPY_H5 = _p if os.path.exists(_p) else None
except ImportError:
    pass


@pytest.fixture(scope="module")
def snap():
    g, meta = load("snap2_n16_vv4")
    return g, meta


def _outputs_ref():
    import importlib
    import sys

    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(here, "oracle"))
    return importlib.import_module("outputs_ref")


def test_histograms_bit_exact_with_reference(snap):
    g, meta = snap
    o = _outputs_ref()
    f = np.stack([g["snap_ScalarField_0"], g["snap_ScalarField_1"]])
    freq, bmin, df = o.histograms(f, 256)
    times = g["histogramtimes"][-1]
    for fld in range(2):
        assert np.array_equal(freq[fld], g[f"histogram_{fld}"][-1])
        assert bmin[fld] == times[1 + 2 * fld] and df[fld] == times[2 + 2 * fld]


def test_histogram_edge_cases():
    o = _outputs_ref()
    x = np.array([0.0, 0.25, 0.5, 0.75, 1.0, 1.0])
    freq, bmin, df = o.histogram(x, 4)
    assert (bmin, df) == (0.0, 0.25)
    assert np.array_equal(freq * 6, [1, 1, 1, 3])   # the maximum goes to the top bin
    # explicit limits: (int) truncates toward zero, so values less than one bin below
    # hmin land in bin 0; values at or beyond hmax + df are dropped
    freq, _, _ = o.histogram(np.array([-0.1, 0.0, 0.5, 2.0, 5.0]), 2, hmin=0.0, hmax=1.0)
    assert np.array_equal(freq * 3, [2, 1])
    # constant field: (x - bmin) / 0 is NaN, every point equals bmax -> top bin
    freq, _, df = o.histogram(np.full(8, 3.0), 4)
    assert df == 0.0 and np.array_equal(freq, [0, 0, 0, 1])


def test_lattice_energies_match_reference(snap):
    g, meta = snap
    o = _outputs_ref()
    N = meta["N"]
    H = N // 2 + 1
    f = np.stack([g["snap_ScalarField_0"], g["snap_ScalarField_1"]])
    # pi(x) = c2r(pi_k) / N^3 of the final state (the reference's isChanged block)
    pi = np.stack([np.fft.irfftn(g["fin_pi_k"][i].reshape(N, N, H), s=(N, N, N), axes=(0, 1, 2)) for i in range(2)])
    a = g["bg"][-1][2]
    from pspectcosmo_gb300.params import Params

    p = Params.preheating(N=N)
    e = o.lattice_energies(f, pi, a, p.kIR, 1, p.gsq)
    assert rel(e["pot"], g["snap_PotentialEnergy"]) < 1e-15
    assert rel(e["kin"], g["snap_KineticEnergy"]) < 1e-12
    assert rel(e["grad"], g["snap_GradientEnergy"]) < 1e-12
    assert rel(e["tot"], g["snap_TotalEnergy"]) < 1e-12


@pytest.mark.skipif(SCIPY_H5 is None, reason="SciPy's HDF5 test file is not installed")
def test_reader_reads_a_libhdf5_file():
    # a file written by libhdf5 (MATLAB 7.3 format, 512-byte user block)
    f = h5read.File(SCIPY_H5)
    assert f.keys() == ["testdouble"]
    x = f.read("testdouble").ravel()
    assert np.allclose(x, np.arange(9) * np.pi / 4, rtol=0, atol=1e-15)


def test_writer_round_trip(tmp_path, psc_lib):
    from pspectcosmo_gb300.lattice import h5_write

    rng = np.random.default_rng(7)
    # more names than one symbol table node holds, unsorted, with leading '/'
    names = [f"/ScalarField_{i}" for i in (3, 0, 10, 1, 2, 9, 4, 5, 6, 7, 8)] + ["/TotalEnergy", "/PotentialEnergy"]
    data = {n: rng.standard_normal((4, 8, 16)) for n in names}
    path = str(tmp_path / "data_7_snapshot.h5")
    h5_write(path, data)
    f = h5read.File(path)
    assert f.keys() == sorted(n[1:] for n in names)
    assert f.eof == os.path.getsize(path)
    for n, v in data.items():
        info = f.dataset_info(n)
        assert info["shape"] == (4, 8, 16) and info["dtype"] == np.dtype("<f8")
        assert np.array_equal(f.read(n), v)
    if SCIPY_H5:
        # datatype bit field and fill value message as libhdf5 writes them
        ref = h5read.File(SCIPY_H5).dataset_info("testdouble")
        assert info["type_bits"] == ref["type_bits"]
        assert info["fill"] == ref["fill"]


def test_writer_rejects_bad_input(tmp_path, psc_lib):
    from pspectcosmo_gb300.lattice import PscError, h5_write

    with pytest.raises(PscError):
        h5_write(str(tmp_path / "x.h5"), {"/a": np.zeros(4), "a": np.zeros(4)})   # duplicate
    with pytest.raises(PscError):
        h5_write(str(tmp_path / "x.h5"), {"/g/a": np.zeros(4)})                    # not in the root group
    with pytest.raises(PscError):
        h5_write(str(tmp_path / "no_such_dir" / "x.h5"), {"a": np.zeros(4)})


def test_reader_round_trip(tmp_path, psc_lib):
    """The library's reader on the library's files (host only)."""
    from pspectcosmo_gb300.lattice import h5_read, h5_write

    rng = np.random.default_rng(9)
    data = {"/a": rng.standard_normal((3, 5)), "/b": rng.standard_normal((3, 5))}
    path = str(tmp_path / "x.h5")
    h5_write(path, data)
    for k, v in data.items():
        assert np.array_equal(h5_read(path, k), v)
        assert np.array_equal(h5_read(path, k.lstrip("/")), v)


def test_reader_refuses_other_layouts(psc_lib):
    from pspectcosmo_gb300.lattice import PscError, h5_read

    if SCIPY_H5 is None:
        pytest.skip("SciPy's HDF5 test file is not installed")
    with pytest.raises(PscError):
        h5_read(SCIPY_H5, "testdouble")   # user block + layout version 2: not this library's layout


def test_calculate_dt():
    """calculate_dt (pspectcosmo.cpp:213-233): 2 / (k / a) / 10, host arithmetic."""
    from pspectcosmo_gb300.driver import calculate_dt

    k = 25 * 16 * 3 ** 0.5 / 2
    assert calculate_dt(k, 1.0) == 2.0 / (k / 1.0) / 10
    assert calculate_dt(k, 2.0) == 2 * calculate_dt(k, 1.0)


def test_info_file_matches_reference(tmp_path):
    """info.txt (output_parameters, output.cpp:1750-1794) up to its clock lines, against the
    reference's own file from its main() run (golden drive1_n16)."""
    import json

    from pspectcosmo_gb300 import Params
    from pspectcosmo_gb300.outputs import TextWriter

    g, meta = load("drive1_n16")
    w = TextWriter(Params.reference_default(N=16), str(tmp_path))
    w.info_begin(0.0)
    w.info_end(0.0, 0.02)
    text = (tmp_path / "info.txt").read_text()
    assert text.split("\nRun began at")[0] == meta["info"]
    assert text.rstrip().endswith("took less than 1 second")
    assert TextWriter.readable_time(90061) == "1 days, 1 hours, 1 minutes, 1 seconds\n"


def test_histogram_2d_and_slices_match_reference():
    """histograms_2d() and slices() (output.cpp:1300-1539) of the reference's own save() at
    t = 0 (golden out2_n16_vv4: field pair 0, 1 in 10 x 10 bins; 2-D slices, skip 2, averaged)."""
    g, meta = load("out2_n16_vv4")
    o = _outputs_ref()
    f = g["ic_f_real"]
    freq, bmin, df = o.histogram_2d(f[0], f[1], 10, 10)
    assert np.array_equal(freq.ravel(), g["histogram2d0_1"][0])
    row = g["histogram2dtimes"][0]
    assert list(row[1:]) == [bmin[0], df[0], bmin[1], df[1]]
    for fld in range(2):
        assert np.array_equal(o.slices(f[fld], slicedim=2, sliceskip=2), g[f"slices_{fld}"][0])
