"""Helpers shared by the tests: golden fixtures and parameter sets."""
from __future__ import annotations

import json
import re
import os

import numpy as np

from pspectcosmo_gb300.outputs import spectra_rows
from pspectcosmo_gb300.params import Params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

ALL_RUNS = ["spec1_n16", "spec1_n16_vv6", "spec1_n16_vv8", "spec1_n16_vv10", "spec1_n32_vv4", "spec1_n64_dt1e-4",
            "spec1_n64_dt2e-3", "spec2_n16_vv4", "spec2_n32_vv2", "gw2_n16_vv4", "gw1_n16_vv2", "specgw2_n16_vv4",
            "spec1_n24_vv4", "spec2_n20_vv2", "gw2_n24_vv4", "gw1_n28_vv2"]


def load(run: str):
    g = np.load(os.path.join(GOLDEN, f"{run}.npz"))
    meta = json.loads(str(g["meta"]))
    return g, meta


def params_for(meta: dict, precision: int = 64) -> Params:
    c = meta["config"]
    if c.startswith(("spec1", "gw1", "pad1", "anal1")):
        p = Params.reference_default(N=meta["N"])
    elif c.startswith("gw4"):
        p = Params.user_model("four_field", 4, initfield=(0.193, 0.0, 0.0, 0.0),
                              initderivs=(-0.142e-6, 0.0, 0.0, 0.0), N=meta["N"])
    elif c.startswith(("spec3", "gw3", "pad3")):
        # the three-field model file (pspectcosmo_gb300/models/three_field.h) compiled in
        p = Params.user_model("three_field", 3, initfield=(0.193, 0.0, 0.01), initderivs=(-0.142e-6, 0.0, 0.0),
                              N=meta["N"])
    else:
        p = Params.preheating(N=meta["N"])
    m = re.search(r"vv(\d+)", c)
    p.vv = int(m.group(1)) if m else 2
    p.spectral = meta["spectral"]
    p.with_gw = meta["gw"]
    p.precision = precision
    return p


def rel(a, b) -> float:
    a, b = np.asarray(a), np.asarray(b)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def output_rows(engine, p: Params) -> dict:
    """Reference output rows (spectra, energies, means, scale) from an engine that
    offers spectra()/spectra_raw(), energies(), means(), bg()/background()."""
    bg = engine.bg() if hasattr(engine, "bg") else engine.background()
    raw = engine.spectra_raw() if hasattr(engine, "spectra_raw") else engine.spectra()
    en = engine.energies()
    means = engine.means()
    mass_sq = engine.mass_sq_av() if p.model not in (0, 1) else None
    rows = spectra_rows(p, bg, raw, en["total"], means, mass_sq)
    rows["energies"] = en
    rows["means"] = means
    rows["bg"] = bg
    rows["raw"] = raw
    return rows
