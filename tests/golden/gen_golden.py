"""Generate the golden fixtures in tests/golden/ from the reference's OWN code.

Runs the oracle/_ref harnesses (the reference's sources compiled against the FFT shim by
oracle/build_ref.py) with fixed dt and stores what they write, at full FP64 precision,
as compressed .npz files. This needs the reference checkout and is run only where it
exists; the committed .npz files are what the tests read everywhere else.

Usage: python tests/golden/gen_golden.py [run ...]
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# run name -> (build config, nsteps, dt, output every, keep full state arrays)
RUNS = {
    "spec1_n16": ("spec1_n16", 20, 0.002, 10, True),
    "spec1_n16_vv6": ("spec1_n16_vv6", 10, 0.002, 5, True),
    "spec1_n16_vv8": ("spec1_n16_vv8", 10, 0.002, 5, True),
    "spec1_n16_vv10": ("spec1_n16_vv10", 10, 0.002, 5, True),
    "specgw2_n16_vv4": ("specgw2_n16_vv4", 10, 0.005, 5, True),
    "spec1_n32_vv4": ("spec1_n32_vv4", 20, 0.001, 10, False),
    "spec1_n64_dt2e-3": ("spec1_n64", 1000, 0.002, 50, False),
    "spec1_n64_dt1e-4": ("spec1_n64", 200, 0.0001, 50, False),
    "spec2_n16_vv4": ("spec2_n16_vv4", 20, 0.005, 10, True),
    "spec2_n32_vv2": ("spec2_n32_vv2", 40, 0.005, 20, False),
    "snap2_n16_vv4": ("snap2_n16_vv4", 20, 0.005, 10, True),
    "out2_n16_vv4": ("out2_n16_vv4", 0, 0.005, 1, True),
    "pad1_n16": ("pad1_n16", 20, 0.002, 10, True),
    "pad2_n16_vv4": ("pad2_n16_vv4", 20, 0.005, 10, True),
    "gw2_n16_vv4": ("gw2_n16_vv4", 10, 0.005, 5, True),
    "gw1_n16_vv2": ("gw1_n16_vv2", 10, 0.002, 5, True),
    "spec3_n16_vv4": ("spec3_n16_vv4", 20, 0.005, 10, True),
    "gw3_n16_vv4": ("gw3_n16_vv4", 10, 0.005, 5, True),
    "spec3_n32_vv2": ("spec3_n32_vv2", 40, 0.005, 20, False),
    "gw3_n32_vv4": ("gw3_n32_vv4", 10, 0.005, 5, False),
    "gw4_n16_vv2": ("gw4_n16_vv2", 10, 0.005, 5, True),
    "pad3_n16_vv4": ("pad3_n16_vv4", 20, 0.005, 10, True),
    "gw4_n32_vv2": ("gw4_n32_vv2", 10, 0.005, 5, False),
    "spec1_n24_vv4": ("spec1_n24_vv4", 20, 0.002, 10, True),
    "spec2_n20_vv2": ("spec2_n20_vv2", 20, 0.005, 10, True),
    "gw2_n24_vv4": ("gw2_n24_vv4", 10, 0.005, 5, True),
    "gw1_n28_vv2": ("gw1_n28_vv2", 10, 0.002, 5, False),
    "pad1_n16_np24": ("pad1_n16_np24", 20, 0.002, 10, True),
    "pad2_n20_vv4_np30": ("pad2_n20_vv4_np30", 20, 0.005, 10, True),
}


SYM6 = [0, 1, 2, 4, 5, 8]  # flat 3x3 indices of the independent u_ij


def read_state(path: str) -> dict:
    with open(path, "rb") as fh:
        raw = fh.read()
    hdr = np.frombuffer(raw, dtype=np.int32, count=6)
    assert hdr[0] == 0x44435350, "bad state magic"
    N, nflds, spectral, gw = (int(x) for x in hdr[2:6])
    off = 24
    bg = np.frombuffer(raw, dtype=np.float64, count=4, offset=off)
    off += 32
    modes = N * N * (N // 2 + 1)
    sites = N ** 3

    def take(count, dtype=np.float64):
        nonlocal off
        arr = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += arr.nbytes
        return arr

    st = {"N": N, "nflds": nflds, "spectral": spectral, "gw": gw,
          "t": bg[0], "a": bg[1], "ad": bg[2], "add": bg[3]}
    st["f_k"] = take(2 * modes * nflds).view(np.complex128).reshape(nflds, modes).copy()
    st["pi_k"] = take(2 * modes * nflds).view(np.complex128).reshape(nflds, modes).copy()
    st["f"] = take(sites * nflds).reshape(nflds, N, N, N).copy()
    st["pi_f"] = take(sites * nflds).reshape(nflds, N, N, N).copy()
    if gw:
        st["u"] = take(sites * 9).reshape(9, N, N, N).copy()
        st["pi_u"] = take(sites * 9).reshape(9, N, N, N).copy()
        st["u_k"] = take(2 * modes * 9).view(np.complex128).reshape(9, modes).copy()
        st["pi_u_k"] = take(2 * modes * 9).view(np.complex128).reshape(9, modes).copy()
    assert off == len(raw), "trailing bytes in state dump"
    return st


_NUM = re.compile(r"[-+]?(?:\d+\.\d{17}(?:e[-+]\d{2})?|nan|inf)")


def split_numbers(line: str) -> list[float]:
    """The reference pads with setw(15); at 17 significant digits adjacent fields touch,
    so each whitespace chunk is split on the fixed 17-digit fraction width."""
    vals = []
    for chunk in line.split():
        try:
            vals.append(float(chunk))
        except ValueError:
            parts = _NUM.findall(chunk)
            if "".join(parts) != chunk:
                raise ValueError(f"cannot tokenise {chunk!r}")
            vals.extend(float(x) for x in parts)
    return vals


def read_blocks(path: str) -> np.ndarray:
    """Blank-line separated blocks of numeric rows -> (nblocks, rows, cols)."""
    blocks, cur = [], []
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if not line:
                if cur:
                    blocks.append(cur)
                    cur = []
                continue
            cur.append(split_numbers(line))
    if cur:
        blocks.append(cur)
    return np.array(blocks, dtype=np.float64)


def read_rows(path: str) -> np.ndarray:
    rows = []
    with open(path) as fh:
        for line in fh:
            if line.strip():
                rows.append(split_numbers(line))
    return np.array(rows, dtype=np.float64)


def generate(run: str) -> str:
    cfg, nsteps, dt, every, full = RUNS[run]
    exe = os.path.join(ROOT, "oracle", "_ref", cfg, "harness")
    if not os.path.exists(exe):
        import build_ref  # noqa: E402

        exe = build_ref.build(cfg)
    with tempfile.TemporaryDirectory() as tmp:
        res = subprocess.run([exe, str(nsteps), repr(dt), str(every)], cwd=tmp, stdin=subprocess.DEVNULL,
                             capture_output=True, text=True)
        if res.returncode != 0:
            raise SystemExit(f"{run}: harness failed\n{res.stderr}")
        out = {}
        meta = {"run": run, "config": cfg, "nsteps": nsteps, "dt": dt, "every": every, "stdout": res.stdout}
        ic = read_state(os.path.join(tmp, "state_000000.bin"))
        fin = read_state(os.path.join(tmp, f"state_{nsteps:06d}.bin"))
        meta.update({k: ic[k] for k in ("N", "nflds", "spectral", "gw")})
        with open(os.path.join(tmp, "ic_info.txt")) as fh:
            meta["ic_info"] = {ln.split()[0]: float(ln.split()[1]) for ln in fh if ln.strip()}
        out["bg"] = read_rows(os.path.join(tmp, "bg.txt"))
        o = os.path.join(tmp, "output")
        for fld in range(ic["nflds"]):
            out[f"spectra_scalar_{fld}"] = read_blocks(os.path.join(o, f"spectra_scalar_{fld}.txt"))
            out[f"average_scalar_{fld}"] = read_rows(os.path.join(o, f"average_scalar_{fld}.txt"))
        out["average_energies"] = read_rows(os.path.join(o, "average_energies.txt"))
        out["average_energy_conservation"] = read_rows(os.path.join(o, "average_energy_conservation.txt"))
        out["average_scale_factor"] = read_rows(os.path.join(o, "average_scale_factor.txt"))
        if ic["gw"]:
            out["spectra_gws"] = read_blocks(os.path.join(o, "spectra_gws.txt"))
            out["energy_gws"] = read_rows(os.path.join(o, "energy_gws.txt"))
        # with snapshots on: the histograms (histograms(), output.cpp:1193-1297, one block
        # per output call) and the raw snapshot datasets of the last step
        # (output.cpp:1541-1648, written through the HDF5 shim)
        snap = os.path.join(o, "Snapshots")
        if os.path.isdir(snap) and os.listdir(snap):
            for fld in range(ic["nflds"]):
                out[f"histogram_{fld}"] = read_blocks(os.path.join(o, f"histogram{fld}.txt"))[..., 0]
            out["histogramtimes"] = read_rows(os.path.join(o, "histogramtimes.txt"))
            N = ic["N"]
            names = [f"ScalarField_{fld}" for fld in range(ic["nflds"])]
            names += ["PotentialEnergy", "KineticEnergy", "GradientEnergy", "TotalEnergy"]
            for name in names:
                raw = np.fromfile(os.path.join(snap, f"data_{nsteps}_snapshot.h5._{name}.bin"), dtype=np.float64)
                out[f"snap_{name}"] = raw.reshape(N, N, N)
        # with shistograms2d / sslices on: save()'s 2-D histograms and slices at t = 0
        if os.path.exists(os.path.join(o, "histogram2d0_1.txt")):
            out["histogram2d0_1"] = read_blocks(os.path.join(o, "histogram2d0_1.txt"))[..., 0]
            out["histogram2dtimes"] = read_rows(os.path.join(o, "histogram2dtimes.txt"))
            out["ic_f_real"] = ic["f"]   # the real-space fields save() binned and sliced
        if os.path.exists(os.path.join(o, "slices0.txt")):
            for fld in range(ic["nflds"]):
                out[f"slices_{fld}"] = read_blocks(os.path.join(o, f"slices{fld}.txt"))[..., 0]
            out["slicetimes"] = read_rows(os.path.join(o, "slicetimes.txt"))
        # initial state in k-space (what both paths start from)
        out["ic_f_k"] = ic["f_k"]
        out["ic_pi_k"] = ic["pi_k"]
        if ic["gw"]:
            # u_ij is symmetric: keep the six components 00, 01, 02, 11, 12, 22
            out["ic_u_k"] = ic["u_k"][SYM6]
            out["ic_pi_u_k"] = ic["pi_u_k"][SYM6]
        if full:
            if ic["spectral"]:
                out["fin_f_k"] = fin["f_k"]
                out["fin_pi_k"] = fin["pi_k"]
            else:
                out["fin_f"] = fin["f"]
                out["fin_pi_f"] = fin["pi_f"]
                if ic["gw"]:
                    out["fin_u"] = fin["u"][SYM6]
                    out["fin_pi_u"] = fin["pi_u"][SYM6]
        else:
            out["ic_f_k"] = ic["f_k"][:, :4096]
            out["ic_pi_k"] = ic["pi_k"][:, :4096]
            if ic["gw"]:
                out["ic_u_k"] = out["ic_u_k"][:, :4096]
                out["ic_pi_u_k"] = out["ic_pi_u_k"][:, :4096]
        out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, f"{run}.npz")
    np.savez_compressed(path, **out)
    return path


# the analytic pre-lattice phase (ANALYTIC_EVOLUTION builds): NA analytic steps of DTA with a
# dump every EVERYA, initialize_lattice(), NSTEPS lattice steps of DT with a dump every EVERY
ANALYTIC_RUNS = {
    "anal1_n16": ("anal1_n16", 10, 0.001, 5, 4, 0.002, 2),
    "anal2_n16_vv4": ("anal2_n16_vv4", 10, 0.002, 5, 4, 0.005, 2),
}


def read_analytic(path: str) -> dict:
    with open(path, "rb") as fh:
        raw = fh.read()
    hdr = np.frombuffer(raw, dtype=np.int32, count=4)
    assert hdr[0] == 0x41435350, "bad analytic dump magic"
    na, nf = int(hdr[1]), int(hdr[2])
    bg = np.frombuffer(raw, dtype=np.float64, count=4, offset=16)
    k2 = np.frombuffer(raw, dtype=np.int32, count=na, offset=48)
    off = 48 + 4 * na
    modes = np.frombuffer(raw, dtype=np.complex128, count=4 * nf * na, offset=off).reshape(4, nf, na).copy()
    assert off + modes.nbytes == len(raw), "trailing bytes in analytic dump"
    return {"t": bg[0], "a": bg[1], "ad": bg[2], "add": bg[3], "k2": k2.copy(), "modes": modes}


def generate_analytic(run: str) -> str:
    cfg, na, dta, everya, nsteps, dt, every = ANALYTIC_RUNS[run]
    exe = os.path.join(ROOT, "oracle", "_ref", cfg, "harness")
    if not os.path.exists(exe):
        import build_ref  # noqa: E402

        exe = build_ref.build(cfg)
    with tempfile.TemporaryDirectory() as tmp:
        args = [exe, "analytic", str(na), repr(dta), str(everya), str(nsteps), repr(dt), str(every)]
        res = subprocess.run(args, cwd=tmp, stdin=subprocess.DEVNULL, capture_output=True, text=True)
        if res.returncode != 0:
            raise SystemExit(f"{run}: harness failed\n{res.stderr}")
        out = {}
        for s in range(0, na + 1, everya):
            d = read_analytic(os.path.join(tmp, f"analytic_{s:06d}.bin"))
            out[f"ana_{s}_bg"] = np.array([d["t"], d["a"], d["ad"], d["add"]])
            out[f"ana_{s}_modes"] = d["modes"]
            out["k2"] = d["k2"]
        ic = read_state(os.path.join(tmp, "state_000000.bin"))
        fin = read_state(os.path.join(tmp, f"state_{nsteps:06d}.bin"))
        out["lat_ic_bg"] = np.array([ic["t"], ic["a"], ic["ad"], ic["add"]])
        out["lat_ic_f_k"] = ic["f_k"]
        out["lat_ic_pi_k"] = ic["pi_k"]
        out["lat_fin_bg"] = np.array([fin["t"], fin["a"], fin["ad"], fin["add"]])
        out["lat_fin_f_k"] = fin["f_k"]
        out["lat_fin_pi_k"] = fin["pi_k"]
        meta = {"run": run, "config": cfg, "N": ic["N"], "nflds": ic["nflds"], "spectral": ic["spectral"],
                "gw": ic["gw"], "na_steps": na, "dta": dta, "everya": everya, "nsteps": nsteps, "dt": dt,
                "every": every}
        out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, f"{run}.npz")
    np.savez_compressed(path, **out)
    return path


# runs of the reference's own main() (its adaptive-dt driver loop and output cadence)
MAIN_RUNS = {"drive1_n16": "drive1_n16"}


def generate_main(run: str) -> str:
    cfg = MAIN_RUNS[run]
    exe = os.path.join(ROOT, "oracle", "_ref", cfg, "harness")
    if not os.path.exists(exe):
        import build_ref  # noqa: E402

        exe = build_ref.build(cfg)
    with tempfile.TemporaryDirectory() as tmp:
        res = subprocess.run([exe, "main"], cwd=tmp, stdin=subprocess.DEVNULL, capture_output=True, text=True)
        if res.returncode != 0:
            raise SystemExit(f"{run}: reference main failed\n{res.stderr}")
        o = os.path.join(tmp, "output")
        out = {}
        for name in ("average_scalar_0", "average_scale_factor", "average_energies", "average_energy_conservation",
                     "average_spectra_times", "histogramtimes"):
            out[name] = read_rows(os.path.join(o, name + ".txt"))
        out["spectra_scalar_0"] = read_blocks(os.path.join(o, "spectra_scalar_0.txt"))
        out["histogram0"] = read_blocks(os.path.join(o, "histogram0.txt"))[..., 0]
        # info.txt up to its clock lines (output_parameters, output.cpp:1750-1786)
        with open(os.path.join(o, "info.txt")) as fh:
            info = fh.read().split("\nRun began at")[0]
        out["meta"] = np.array(json.dumps({"run": run, "config": cfg, "mode": "reference main()", "info": info}))
    path = os.path.join(HERE, f"{run}.npz")
    np.savez_compressed(path, **out)
    return path


def main(argv):
    for run in (argv or list(RUNS) + list(MAIN_RUNS) + list(ANALYTIC_RUNS)):
        if run in MAIN_RUNS:
            p = generate_main(run)
        elif run in ANALYTIC_RUNS:
            p = generate_analytic(run)
        else:
            p = generate(run)
        print(f"{p}  {os.path.getsize(p) / 1024:.0f} KiB")


if __name__ == "__main__":
    main(sys.argv[1:])
