"""The model surface: model.h files written in the reference's model interface compile into
the library (pspectcosmo_gb300/model_adapter.py) and evaluate as the original file does.

Each model file is compiled twice on the host with g++: as written, against the helpers
of the reference's pspectcosmo.h (pw2, FIELD, LOOP, DECLARE_INDICES, N3, nflds and the
parameters.h constants; pspectcosmo.h:27, 184-192), and through the adapter's generated
header. dvdf, potential_energy and effective_mass at random field points must agree: bit for
bit in FP64 (-ffp-contract=off on both), and in FP32 to single-precision rounding. The
library's own compilation (psc_model_eval on the host) is compared with the original file
too. The reference's shipped model.h is checked where the reference checkout exists.
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from pspectcosmo_gb300 import model_adapter  # noqa: E402

MODELS = os.path.join(ROOT, "pspectcosmo_gb300", "models")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402  (the oracle's recipe names the reference checkout)

REF_MODEL = os.path.join(build_ref.REF, "model.h")
NPTS = 64

CASES = [("phi2", os.path.join(MODELS, "phi2.h"), 1), ("phi2chi2", os.path.join(MODELS, "phi2chi2.h"), 2),
         ("three_field", os.path.join(MODELS, "three_field.h"), 3), ("four_field", os.path.join(MODELS, "four_field.h"), 4)]

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstddef>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
namespace raw {
const int N = 2;
const int nflds = NFLDS;
const double N3 = 8.0;
const double MPl = 1.0, m_in_MPl = 1.0e-6, fStar = 1.0, omegaStar = 1.0e-6;
double f[nflds][N][N][N];
inline double pw2(double x) { return x * x; }
#define FIELD(fld) f[fld][i][j][k]
#define LOOP for (i = 0; i < N; i++) for (j = 0; j < N; j++) for (k = 0; k < N; k++)
#define DECLARE_INDICES int i, j, k;
#include MODEL_FILE
#undef FIELD
#undef LOOP
#undef DECLARE_INDICES
}  // namespace raw
#include "gen.cuh"

int main() {
    unsigned long long s = 12345;
    auto draw = [&]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return ((double)(s >> 11) / 9007199254740992.0 - 0.5) * 0.6;
    };
    const int nt = raw::num_potential_terms;
    std::printf("%d\n", nt);
    for (int n = 0; n < NPTS; ++n) {
        double v[raw::nflds];
        float vf[raw::nflds];
        for (int q = 0; q < raw::nflds; ++q) { v[q] = draw(); vf[q] = (float)v[q]; }
        double m[raw::nflds], mg[raw::nflds];
        float mf[raw::nflds];
        raw::effective_mass(m, v);
        psc::um_MODEL_f64::effective_mass(mg, v);
        psc::um_MODEL_f32::effective_mass(mf, vf);
        for (int q = 0; q < raw::nflds; ++q)
            std::printf("P %.17g D %.17g %.17g %.9g M %.17g %.17g %.9g\n", v[q], raw::dvdf(q, v),
                        psc::um_MODEL_f64::dvdf(q, v), (double)psc::um_MODEL_f32::dvdf(q, vf), m[q], mg[q],
                        (double)mf[q]);
        for (int t = 0; t < nt; ++t)
            std::printf("T %.17g %.17g %.9g\n", raw::potential_energy(t, v), psc::um_MODEL_f64::potential_energy(t, v),
                        (double)psc::um_MODEL_f32::potential_energy(t, vf));
    }
    return 0;
}
"""


def _run(tmp_path, name: str, path: str, nflds: int):
    gen = tmp_path / "gen.cuh"
    gen.write_text(model_adapter.generate([path]))
    src = tmp_path / "h.cpp"
    src.write_text(HARNESS.replace("MODEL_FILE", f'"{path}"').replace("NFLDS", str(nflds))
                   .replace("NPTS", str(NPTS)).replace("um_MODEL", f"um_{model_adapter.model_name(path)}"))
    exe = tmp_path / "h"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w", "-I", str(tmp_path), str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    nt = int(out[0])
    pts, d, t = [], [], []
    for ln in out[1:]:
        w = ln.split()
        if not w:
            continue
        if w[0] == "P":
            pts.append(float(w[1]))
            d.append([float(x) for x in (w[3], w[4], w[5], w[7], w[8], w[9])])
        elif w[0] == "T":
            t.append([float(x) for x in w[1:4]])
    return nt, np.array(pts).reshape(NPTS, nflds), np.array(d).reshape(NPTS, nflds, 6), np.array(t).reshape(NPTS, nt, 3)


def _compare(d, t):
    # FP64: the adapter's compilation is the original, bit for bit
    assert np.array_equal(d[..., 0], d[..., 1]), "dvdf differs in FP64"
    assert np.array_equal(d[..., 3], d[..., 4]), "effective_mass differs"
    assert np.array_equal(t[..., 0], t[..., 1]), "potential_energy differs in FP64"
    # FP32: the same formulas in single precision
    scale_d = np.abs(d[..., 0]).max() + 1e-30
    assert np.abs(d[..., 2] - d[..., 0]).max() <= 2e-6 * scale_d
    assert np.abs(d[..., 5] - d[..., 3]).max() <= 2e-6 * (np.abs(d[..., 3]).max() + 1e-30)
    assert np.abs(t[..., 2] - t[..., 0]).max() <= 2e-6 * (np.abs(t[..., 0]).max() + 1e-30)


@pytest.mark.parametrize("name,path,nflds", CASES, ids=[c[0] for c in CASES])
def test_adapter_matches_model_file(tmp_path, name, path, nflds):
    nt, pts, d, t = _run(tmp_path, name, path, nflds)
    _compare(d, t)


@pytest.mark.skipif(not os.path.exists(REF_MODEL), reason="the reference checkout is not here")
def test_adapter_matches_reference_model_h(tmp_path):
    """The reference's shipped model.h (single-field phi^2), unchanged, through the adapter."""
    nt, pts, d, t = _run(tmp_path, "model", REF_MODEL, 1)
    assert nt == 1
    _compare(d, t)


@pytest.mark.parametrize("name,path,nflds", CASES, ids=[c[0] for c in CASES])
def test_library_model_matches_model_file(tmp_path, name, path, nflds):
    """The library's compilation of each model (psc_model_eval on the host, FP64) equals the
    original file compiled as written."""
    from pspectcosmo_gb300 import Params
    from pspectcosmo_gb300.lattice import model_eval, model_id, load_library

    load_library()
    nt, pts, d, t = _run(tmp_path, name, path, nflds)
    p = Params.user_model(name, nflds)
    assert p.model == model_id(name)
    r = model_eval(p, pts, on_device=False)
    assert np.array_equal(r["dvdf"], d[..., 0])
    assert np.array_equal(r["mass_sq"], d[..., 3])
    assert np.array_equal(r["terms"], t[..., 0])
    p.precision = 32
    r32 = model_eval(p, pts, on_device=False)
    # (the FP32 values pass through 9-digit text: equal as FP32 numbers)
    f32 = np.float32
    assert np.array_equal(r32["dvdf"].astype(f32), d[..., 2].astype(f32))
    assert np.array_equal(r32["terms"].astype(f32), t[..., 2].astype(f32))


def test_process_drops_host_only_parts():
    text = model_adapter.process(open(os.path.join(MODELS, "three_field.h")).read())
    for name in model_adapter.HOST_ONLY:
        assert name not in text
    assert "throw" not in text and "double" not in text
    assert "__host__ __device__ inline psc_real dvdf(" in text


def test_user_model_ids_and_limits():
    from pspectcosmo_gb300.lattice import load_library, model_names

    L = load_library()
    names = model_names()
    assert names[0] == "builtin:phi2" and names[1] == "builtin:phi2chi2"
    assert {"phi2", "phi2chi2", "three_field", "four_field"} <= set(names.values())
    for mid, nm in names.items():
        assert L.psc_model_nterms(mid) == {"builtin:phi2": 1, "builtin:phi2chi2": 2, "phi2": 1, "phi2chi2": 2,
                                           "three_field": 3, "four_field": 4}.get(nm, L.psc_model_nterms(mid))
    assert L.psc_model_nterms(99) == 0


@pytest.mark.parametrize("run", ["spec3_n16_vv4", "gw3_n16_vv4", "spec3_n32_vv2", "gw3_n32_vv4", "gw4_n16_vv2",
                                 "gw4_n32_vv2", "pad3_n16_vv4"])
def test_user_model_initial_conditions_match_reference(run):
    """initialize() of the reference built with three_field.h (nflds = 3) or four_field.h (4) against the
    library's host generator with the same model compiled in: the scalar modes use the model's
    effective_mass (initialize.cpp:644), the background its potential_energy (:654)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from golden_util import load, params_for, rel
    from pspectcosmo_gb300.lattice import generate_ic

    g, meta = load(run)
    p = params_for(meta)
    f, pi, u, pu, info = generate_ic(p)
    n = g["ic_f_k"].shape[1]
    if p.spectral:
        assert np.array_equal(f[:, :n], g["ic_f_k"]) and np.array_equal(pi[:, :n], g["ic_pi_k"])
    else:
        # the reference's k-space view is the r2c of its c2r'd initial arrays
        assert rel(f[:, :n], g["ic_f_k"]) < 1e-14 and rel(pi[:, :n], g["ic_pi_k"]) < 1e-14
        m = g["ic_u_k"].shape[1]
        assert rel(u[:, :m], g["ic_u_k"]) < 1e-14 and rel(pu[:, :m], g["ic_pi_u_k"]) < 1e-14
    assert info["hubble_init"] == meta["ic_info"]["hubble_init"]
