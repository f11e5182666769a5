"""ctypes binding of the CPU oracle (oracle/port/psc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline arm, never by the product. `build()` compiles the shared library with gcc.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libpsc_oracle.so")
SRC = [os.path.join(HERE, "psc_oracle.c"), os.path.join(os.path.dirname(HERE), "fft64.c")]


def build(force: bool = False) -> str:
    # psc_oracle.h includes the library's psc.h for the psc_params layout
    deps = SRC + [os.path.join(HERE, "psc_oracle.h"), os.path.join(HERE, "..", "..", "include", "psc.h")]
    newest = max(os.path.getmtime(s) for s in deps)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-shared", "-fPIC"] + SRC + ["-o", LIB, "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        from pspectcosmo_gb300.params import Params  # noqa: F401  (struct layout)

        L = ctypes.CDLL(build())
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        I = ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = P
        L.orc_create.argtypes = [P]
        L.orc_destroy.argtypes = [P]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_init_ic.restype = ctypes.c_double
        L.orc_init_ic.argtypes = [P]
        L.orc_hubble_init.restype = ctypes.c_double
        L.orc_hubble_init.argtypes = [P]
        L.orc_step.argtypes = [P, ctypes.c_double]
        L.orc_step_stages.argtypes = [P, ctypes.c_double, ctypes.c_int]
        L.orc_stages.argtypes = [P]
        L.orc_stages.restype = ctypes.c_int
        L.orc_get_bg.argtypes = [P, D, D, D, D]
        L.orc_set_bg.argtypes = [P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_get_state_k.argtypes = [P, D, D, D, D]
        L.orc_set_state_k.argtypes = [P, D, D, D, D]
        L.orc_get_fields_real.argtypes = [P, D, D]
        L.orc_get_gw_real.argtypes = [P, D, D]
        L.orc_kernel_a.restype = ctypes.c_double
        L.orc_kernel_a.argtypes = [P]
        L.orc_maxnumbins.restype = ctypes.c_int
        L.orc_maxnumbins.argtypes = [ctypes.c_int]
        L.orc_spectra.argtypes = [P, I, D, D, D, I, D, D, D]
        L.orc_energies.argtypes = [P, D, D, D, D, D, D]
        L.orc_means.argtypes = [P, D]
        L.orc_rand_stream.argtypes = [ctypes.c_int, ctypes.c_int, D]
        _lib = L
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def rand_stream(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count)
    lib().orc_rand_stream(seed, count, _dp(out))
    return out


class Oracle:
    """FP64 CPU restatement of the reference path for one lattice."""

    def __init__(self, params, threads: int | None = None):
        self.p = params.copy()
        if threads:
            lib().orc_set_threads(threads)
        self._h = lib().orc_create(ctypes.byref(self.p))

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_ic(self) -> float:
        """initialize() (+ initialize_GW()); returns the printed pre-lattice a''."""
        return lib().orc_init_ic(self._h)

    @property
    def hubble_init(self) -> float:
        return lib().orc_hubble_init(self._h)

    def step(self, dt: float, nsteps: int = 1):
        for _ in range(nsteps):
            lib().orc_step(self._h, dt)

    def step_stages(self, dt: float, nstages: int):
        """Timing sample: the first nstages stages of one step."""
        lib().orc_step_stages(self._h, dt, nstages)

    @property
    def stages(self) -> int:
        return lib().orc_stages(self._h)

    def bg(self) -> dict:
        v = [ctypes.c_double() for _ in range(4)]
        lib().orc_get_bg(self._h, *[ctypes.byref(x) for x in v])
        return dict(zip(("t", "a", "ad", "add"), (x.value for x in v)))

    def set_bg(self, t, a, ad, add):
        lib().orc_set_bg(self._h, t, a, ad, add)

    def state_k(self):
        p = self.p
        f = np.zeros((p.nflds, p.modes), np.complex128)
        pi = np.zeros((p.nflds, p.modes), np.complex128)
        u = np.zeros((6, p.modes), np.complex128) if p.with_gw else None
        pu = np.zeros((6, p.modes), np.complex128) if p.with_gw else None
        lib().orc_get_state_k(self._h, _dp(f), _dp(pi), _dp(u), _dp(pu))
        return f, pi, u, pu

    def set_state_k(self, f_k, pi_k, u_k=None, pi_u_k=None):
        c = lambda a: None if a is None else np.ascontiguousarray(a, np.complex128)
        f_k, pi_k, u_k, pi_u_k = c(f_k), c(pi_k), c(u_k), c(pi_u_k)
        lib().orc_set_state_k(self._h, _dp(f_k), _dp(pi_k), _dp(u_k), _dp(pi_u_k))

    def fields_real(self):
        p = self.p
        f = np.zeros((p.nflds, p.N, p.N, p.N))
        pi = np.zeros((p.nflds, p.N, p.N, p.N))
        lib().orc_get_fields_real(self._h, _dp(f), _dp(pi))
        return f, pi

    def gw_real(self):
        p = self.p
        u = np.zeros((6, p.N, p.N, p.N))
        pu = np.zeros((6, p.N, p.N, p.N))
        lib().orc_get_gw_real(self._h, _dp(u), _dp(pu))
        return u, pu

    def kernel_a(self) -> float:
        return lib().orc_kernel_a(self._h)

    def spectra(self) -> dict:
        p = self.p
        nb = p.maxnumbins
        out = dict(numpoints=np.zeros((p.nflds, nb), np.int32), f2=np.zeros((p.nflds, nb)),
                   pi2=np.zeros((p.nflds, nb)), n2=np.zeros((p.nflds, nb)))
        if p.with_gw:
            out.update(gw_numpoints=np.zeros(nb, np.int32), h2=np.zeros(nb), hdot2=np.zeros(nb))
        hz = ctypes.c_double(0.0)
        lib().orc_spectra(self._h, _ip(out["numpoints"]), _dp(out["f2"]), _dp(out["pi2"]), _dp(out["n2"]),
                          _ip(out.get("gw_numpoints")), _dp(out.get("h2")), _dp(out.get("hdot2")),
                          ctypes.byref(hz))
        out["hdot2_zero"] = hz.value
        return out

    def energies(self) -> dict:
        p = self.p
        K = np.zeros(p.nflds)
        G = np.zeros(p.nflds)
        V = np.zeros(p.num_potential_terms)
        tot, fv, rho = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        lib().orc_energies(self._h, _dp(K), _dp(G), _dp(V), ctypes.byref(tot), ctypes.byref(fv), ctypes.byref(rho))
        return dict(K=K, G=G, V=V, total=tot.value, friedmann_violation=fv.value, rho_gw=rho.value)

    def means(self) -> np.ndarray:
        out = np.zeros((self.p.nflds, 6))
        lib().orc_means(self._h, _dp(out))
        return out
