"""Build recipe for oracle/_ref: the reference's OWN sources compiled as the CPU oracle.

Test infrastructure only. The reference (JieJiang-Cosmology/PSpectCosmo) is configured
at compile time through parameters.h and model.h, so each configuration is a separate
build:

  1. the four reference .cpp files and pspectcosmo.h are copied, unchanged, from the
     reference checkout into oracle/_ref/<config>/ (git-ignored). They must sit next to
     the per-config headers because pspectcosmo.h:24 includes "parameters.h" with quotes;
  2. parameters.h is the reference's own file with the named constants/macros replaced
     (regex on `const <type> NAME = ...;` and `#define NAME ...`);
  3. model.h is the reference's own (single-field phi^2) or one of the model files of the
     library's model surface, pspectcosmo_gb300/models/*.h (the two-field model the benchmark
     configurations need, a three-field model; written in the same API);
  4. g++ compiles them against oracle/shim (FFTW/HDF5 API shims over oracle/fft64.c),
     with pspectcosmo.cpp's main renamed and oracle/ref_harness.cpp as the driver.

Nothing here is run on the GPU machine: the reference checkout exists only where the
fixtures are generated. Usage: python oracle/build_ref.py [config ...]
"""
from __future__ import annotations

import os
import platform
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout this recipe reads (PSC_REFERENCE_DIR overrides the default)
REF = os.environ.get("PSC_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
MODELS = os.path.join(os.path.dirname(HERE), "pspectcosmo_gb300", "models")


def reference_available() -> bool:
    """True where the reference checkout exists (never on the GPU machine)."""
    return os.path.isdir(REF)

# name -> (model, overrides). Values are C++ source text.
CONFIGS: dict[str, tuple[str, dict[str, str]]] = {
    # shipped configuration (parameters.h as is) at N=16 and N=64
    "spec1_n16": ("phi2", {"N": "16"}),
    "spec1_n32_vv4": ("phi2", {"N": "32", "VV": "4"}),
    "spec1_n16_vv6": ("phi2", {"N": "16", "VV": "6"}),
    "spec1_n16_vv8": ("phi2", {"N": "16", "VV": "8"}),
    "spec1_n16_vv10": ("phi2", {"N": "16", "VV": "10"}),
    "spec1_n64": ("phi2", {}),
    # two-field preheating (phi0 = 0.193 MPl, phidot0 = -0.142 m MPl, kIR = 1 m)
    "spec2_n16_vv4": ("phi2chi2", {
        "N": "16", "VV": "4", "nflds": "2", "kIR": "1",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    "spec2_n32_vv2": ("phi2chi2", {
        "N": "32", "VV": "2", "nflds": "2", "kIR": "1",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    # the same with snapshots on (HDF5 datasets through the shim: fields + lattice energies)
    "snap2_n16_vv4": ("phi2chi2", {
        "N": "16", "VV": "4", "nflds": "2", "kIR": "1", "ssnapshot": "true",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    # the reference's own main() (adaptive dt, output cadence) on the shipped model, to t = 0.02
    "drive1_n16": ("phi2", {"N": "16", "tf": "0.02", "tOutputInfreq": "0.005"}),
    # the optional outputs of save(): 2-D histograms (field pair 0, 1) and 2-D slices with
    # averaging over 2 x 2 blocks (output.cpp:1300-1539)
    "out2_n16_vv4": ("phi2chi2", {
        "N": "16", "VV": "4", "nflds": "2", "kIR": "1", "shistograms2d": "true", "sslices": "true",
        "slicedim": "2", "slicelength": "N, sliceskip = 2",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    # the analytic pre-lattice phase (ANALYTIC_EVOLUTION): linear modes on the distinct |k|^2,
    # then initialize_lattice(); shipped model and the two-field preheating model
    "anal1_n16": ("phi2", {"N": "16", "ANALYTIC_EVOLUTION": "true", "t_analytic": "0.01"}),
    "anal2_n16_vv4": ("phi2chi2", {
        "N": "16", "VV": "4", "nflds": "2", "kIR": "1", "ANALYTIC_EVOLUTION": "true", "t_analytic": "0.1",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    # the dealiased spectral step evolve_VV_k_pad (PAD_FLAG, V' on an N_pad = 2N grid)
    "pad1_n16": ("phi2", {"N": "16", "PAD_FLAG": "true", "N_pad": "32"}),
    "pad2_n16_vv4": ("phi2chi2", {
        "N": "16", "VV": "4", "nflds": "2", "kIR": "1", "PAD_FLAG": "true", "N_pad": "32",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    # the benchmark workload on the reference's own code (timed, not dumped): 256^3 two-field
    # preheating with GWs, Yoshida-4, real-space step
    "bench_gw2_n256_vv4": ("phi2chi2", {
        "N": "256", "VV": "4", "nflds": "2", "kIR": "1",
        "SPECTRAL_FLAG": "false", "WITH_GW": "true",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    # three fields (pspectcosmo_gb300/models/three_field.h: phi, chi, sigma), the spectral step
    # and the real-space step with GWs, at N = 16 (full state) and N = 32 (outputs)
    "spec3_n16_vv4": ("three_field", {
        "N": "16", "VV": "4", "nflds": "3", "kIR": "1",
        "initfield[]": "{0.193 * MPl, 0., 0.01 * MPl}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0., 0.}",
    }),
    "gw3_n16_vv4": ("three_field", {
        "N": "16", "VV": "4", "nflds": "3", "kIR": "1",
        "SPECTRAL_FLAG": "false", "WITH_GW": "true",
        "initfield[]": "{0.193 * MPl, 0., 0.01 * MPl}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0., 0.}",
    }),
    "gw3_n32_vv4": ("three_field", {
        "N": "32", "VV": "4", "nflds": "3", "kIR": "1",
        "SPECTRAL_FLAG": "false", "WITH_GW": "true",
        "initfield[]": "{0.193 * MPl, 0., 0.01 * MPl}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0., 0.}",
    }),
    "spec3_n32_vv2": ("three_field", {
        "N": "32", "VV": "2", "nflds": "3", "kIR": "1",
        "initfield[]": "{0.193 * MPl, 0., 0.01 * MPl}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0., 0.}",
    }),
    # the padded step with padded grids that are not powers of two (ratio 1.5), and both sizes
    # mixed-radix
    "pad1_n16_np24": ("phi2", {"N": "16", "PAD_FLAG": "true", "N_pad": "24"}),
    "pad2_n20_vv4_np30": ("phi2chi2", {
        "N": "20", "VV": "4", "nflds": "2", "kIR": "1", "PAD_FLAG": "true", "N_pad": "30",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    # three fields on the padded (dealiased) spectral step
    "pad3_n16_vv4": ("three_field", {
        "N": "16", "VV": "4", "nflds": "3", "kIR": "1", "PAD_FLAG": "true", "N_pad": "32",
        "initfield[]": "{0.193 * MPl, 0., 0.01 * MPl}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0., 0.}",
    }),
    # four fields (pspectcosmo_gb300/models/four_field.h), the real-space step with GWs
    "gw4_n16_vv2": ("four_field", {
        "N": "16", "VV": "2", "nflds": "4", "kIR": "1",
        "SPECTRAL_FLAG": "false", "WITH_GW": "true",
        "initfield[]": "{0.193 * MPl, 0., 0., 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0., 0., 0.}",
    }),
    "gw4_n32_vv2": ("four_field", {
        "N": "32", "VV": "2", "nflds": "4", "kIR": "1",
        "SPECTRAL_FLAG": "false", "WITH_GW": "true",
        "initfield[]": "{0.193 * MPl, 0., 0., 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0., 0., 0.}",
    }),
    # lattice sizes that are not powers of two (FFTW takes any N; here the generic engine's
    # mixed radices 3, 5, 7)
    "spec1_n24_vv4": ("phi2", {"N": "24", "VV": "4"}),
    "spec2_n20_vv2": ("phi2chi2", {
        "N": "20", "VV": "2", "nflds": "2", "kIR": "1",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    "gw2_n24_vv4": ("phi2chi2", {
        "N": "24", "VV": "4", "nflds": "2", "kIR": "1",
        "SPECTRAL_FLAG": "false", "WITH_GW": "true",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    "gw1_n28_vv2": ("phi2", {
        "N": "28", "VV": "2", "SPECTRAL_FLAG": "false", "WITH_GW": "true",
    }),
    # real-space pseudo-spectral path with gravitational waves (evolve_VV)
    "gw2_n16_vv4": ("phi2chi2", {
        "N": "16", "VV": "4", "nflds": "2", "kIR": "1",
        "SPECTRAL_FLAG": "false", "WITH_GW": "true",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
    "gw1_n16_vv2": ("phi2", {
        "N": "16", "VV": "2", "SPECTRAL_FLAG": "false", "WITH_GW": "true",
    }),
    # the spectral step with WITH_GW on: u_k is set by initialize_GW() and never evolved,
    # and spectra() still writes the GW spectra of those modes
    "specgw2_n16_vv4": ("phi2chi2", {
        "N": "16", "VV": "4", "nflds": "2", "kIR": "1",
        "SPECTRAL_FLAG": "true", "WITH_GW": "true",
        "initfield[]": "{0.193 * MPl, 0.}",
        "initderivs[]": "{-0.142e-6 * MPl * MPl, 0.}",
    }),
}

MACROS = {"VV", "SPECTRAL_FLAG", "PAD_FLAG", "WITH_GW", "SIMULATE_INFLATION", "SNAPSHOTS_ENERGY",
          "BIFURCATION", "ANALYTIC_EVOLUTION"}

SOURCES = ["pspectcosmo.cpp", "initialize.cpp", "evolution.cpp", "output.cpp"]


def make_parameters(text: str, overrides: dict[str, str]) -> str:
    for name, value in overrides.items():
        if name in MACROS:
            pat = re.compile(r"^(#define\s+%s\s+)\S+" % re.escape(name), re.M)
            text, n = pat.subn(lambda m: m.group(1) + value, text)
        else:
            pat = re.compile(r"^(const\s+[\w:]+\s+%s\s*=\s*)[^;]*;" % re.escape(name), re.M)
            text, n = pat.subn(lambda m: m.group(1) + value + ";", text)
        if n != 1:
            raise SystemExit(f"parameters.h: could not override {name!r} ({n} matches)")
    return text


def prepared(name: str) -> bool:
    """True when oracle/_ref/<name> holds the copied sources and headers (they travel with
    the repository's working tree to a machine without the reference checkout)."""
    d = os.path.join(OUT, name)
    return all(os.path.exists(os.path.join(d, f)) for f in SOURCES + ["pspectcosmo.h", "parameters.h", "model.h"])


def prepare(name: str) -> str:
    """Steps 1-3: the reference's sources and the per-config headers into oracle/_ref/<name>."""
    model, overrides = CONFIGS[name]
    d = os.path.join(OUT, name)
    os.makedirs(d, exist_ok=True)
    for s in SOURCES + ["pspectcosmo.h"]:
        shutil.copyfile(os.path.join(REF, s), os.path.join(d, s))
    with open(os.path.join(REF, "parameters.h")) as fh:
        params = make_parameters(fh.read(), overrides)
    with open(os.path.join(d, "parameters.h"), "w") as fh:
        fh.write(params)
    if model == "phi2":
        shutil.copyfile(os.path.join(REF, "model.h"), os.path.join(d, "model.h"))
    else:
        shutil.copyfile(os.path.join(MODELS, f"{model}.h"), os.path.join(d, "model.h"))
    return d


def build(name: str) -> str:
    """Steps 1-4: prepare (where the reference checkout exists) and compile; returns the
    harness path. Without the checkout, compiles what prepare() left in oracle/_ref/<name>."""
    d = os.path.join(OUT, name)
    if reference_available():
        prepare(name)
    elif not prepared(name):
        raise SystemExit(f"{d}: neither the reference checkout nor prepared sources")

    shim = os.path.join(HERE, "shim")
    cxx = ["g++", "-O2", "-std=c++17", "-fopenmp", "-w", "-I", d, "-I", shim,
           "-include", os.path.join(shim, "prec_override.h")]
    link_extra, model_flags = [], []
    if int(CONFIGS[name][1].get("N", "64")) >= 128:
        # the reference's static N^3 arrays exceed the small code model's 2-4 GB of data; on
        # aarch64 the large model exists only for position-dependent code. Every object of the
        # program needs it (the shims' own statics end up beyond the arrays)
        if platform.machine() in ("aarch64", "arm64"):
            model_flags = ["-fno-pic", "-mcmodel=large"]
            link_extra = ["-no-pie"]
        else:
            model_flags = ["-mcmodel=medium"]
    cxx += model_flags
    objs = []
    jobs = []
    for s in SOURCES:
        extra = ["-Dmain=reference_main"] if s == "pspectcosmo.cpp" else []
        o = os.path.join(d, s.replace(".cpp", ".o"))
        jobs.append(cxx + extra + ["-c", os.path.join(d, s), "-o", o])
        objs.append(o)
    o = os.path.join(d, "ref_harness.o")
    jobs.append(cxx + ["-c", os.path.join(HERE, "ref_harness.cpp"), "-o", o])
    objs.append(o)
    for src in (os.path.join(shim, "shim_fftw.c"), os.path.join(HERE, "fft64.c")):
        o = os.path.join(d, os.path.basename(src).replace(".c", ".o"))
        jobs.append(["gcc", "-O2", "-std=c11", "-fopenmp"] + model_flags + ["-I", shim, "-c", src, "-o", o])
        objs.append(o)
    with ThreadPoolExecutor(max_workers=os.cpu_count()) as ex:
        for r in ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs):
            if r.returncode != 0:
                raise SystemExit(f"compile failed:\n{' '.join(r.args)}\n{r.stderr}")
    exe = os.path.join(d, "harness")
    r = subprocess.run(["g++", "-fopenmp"] + link_extra + ["-o", exe] + objs + ["-lm", "-lpthread"], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise SystemExit(f"link failed:\n{r.stderr}")
    return exe


def main(argv: list[str]) -> None:
    if not os.path.isdir(REF):
        print(f"reference checkout not found at {REF}; nothing to build")
        return
    names = argv or list(CONFIGS)
    with ThreadPoolExecutor(max_workers=4) as ex:
        for exe in ex.map(build, names):
            print(exe)


if __name__ == "__main__":
    main(sys.argv[1:])
