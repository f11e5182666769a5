"""Build libpsc.so (the CUDA path and its C ABI) in-tree for sm_103a.

The model.h files of the model surface (PSC_MODEL_H, default pspectcosmo_gb300/models/*.h)
are first turned into _build/psc_user_models.cuh by model_adapter.py. The translation units
compile in parallel with nvcc (the IC generator and the HDF5 writer with the host compiler
through nvcc) and link into pspectcosmo_gb300/libpsc.so. Rebuilds only when a source, a
model file or the generated header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpsc.so")
SOURCES = ["psc_kernels.cu", "psc_reg_f32.cu", "psc_reg_f64.cu", "psc_reg_user_f32.cu", "psc_reg_user_f64.cu",
           "psc_batch_f32.cu", "psc_batch_f64.cu",
           "psc_api.cu", "psc_noalloc.cu", "psc_adjoint.cu",
           "psc_ic_gpu.cu", "psc_outputs.cu", "psc_pad.cu", "psc_analytic.cu",
           "psc_ic.cpp", "psc_h5.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


USER_MODELS_H = os.path.join(BUILD, "psc_user_models.cuh")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "psc.h"), USER_MODELS_H]
    return [f for f in files if os.path.isfile(f)]


def build(force: bool = False, verbose: bool = False) -> str:
    sys.path.insert(0, HERE)
    import model_adapter  # noqa: E402

    sys.path.remove(HERE)
    model_adapter.write(USER_MODELS_H)   # rewritten (newer) only when the model list or a model changed
    newest = max(os.path.getmtime(f) for f in _deps() + [os.path.abspath(__file__)])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-I", CSRC, "-I", BUILD, "-I", os.path.join(ROOT, "include")]
    jobs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        path = os.path.join(CSRC, src)
        if src.endswith(".cu"):
            cmd = [cc] + ARCH + common + ["-lineinfo", "-Xptxas", "-O3", "-c", path, "-o", obj]
            if verbose:
                cmd += ["-Xptxas", "-v"]
        else:
            cmd = [cc] + common + ["-x", "c++", "-c", path, "-o", obj]
        jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for r in results:
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(r.args)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
    tmp = LIB + ".tmp"
    r = subprocess.run([cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
