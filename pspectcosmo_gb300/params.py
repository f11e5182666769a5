"""Run configuration: the reference's compile-time parameters.h / model.h surface.

`Params` is the ctypes mirror of `psc_params` in include/psc.h. Field names follow
parameters.h (N, nflds, kIR, a0, MPl, m_in_MPl, fStar, epsilon, seed, initfield,
initderivs, kcutoff, ...); the compile-time macros VV, SPECTRAL_FLAG, WITH_GW and
SIMULATE_INFLATION become the run-time ints vv, spectral, with_gw and
simulate_inflation. `Params.reference_default()` is the shipped parameters.h
(N = 64, one field, phi^2 model, kIR = 25, phi0 = 11, velocity Verlet).
"""
from __future__ import annotations

import ctypes
import math

MODEL_PHI2 = 0
MODEL_PHI2CHI2 = 1
MODEL_USER = 16      # model id of the first model.h compiled into the library (psc_model_find)
MAX_FIELDS = 4


class Params(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int),
        ("nflds", ctypes.c_int),
        ("vv", ctypes.c_int),
        ("alpha", ctypes.c_int),
        ("expansion", ctypes.c_int),
        ("simulate_inflation", ctypes.c_int),
        ("spectral", ctypes.c_int),
        ("with_gw", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("model", ctypes.c_int),
        ("seed", ctypes.c_int),
        ("N_pad", ctypes.c_int),       # PAD_FLAG / N_pad: 0 = off
        ("kIR", ctypes.c_double),
        ("a0", ctypes.c_double),
        ("MPl", ctypes.c_double),
        ("m_in_MPl", ctypes.c_double),
        ("fStar", ctypes.c_double),
        ("epsilon", ctypes.c_double),
        ("gsq", ctypes.c_double),
        ("initfield", ctypes.c_double * MAX_FIELDS),
        ("initderivs", ctypes.c_double * MAX_FIELDS),
        ("kcutoff", ctypes.c_double),
    ]

    @classmethod
    def reference_default(cls, **overrides) -> "Params":
        """parameters.h / model.h as shipped (parameters.h:10-133, model.h)."""
        p = cls()
        p.N = 64
        p.nflds = 1
        p.vv = 2
        p.alpha = 0
        p.expansion = 2
        p.simulate_inflation = 1
        p.spectral = 1
        p.with_gw = 0
        p.precision = 64
        p.model = MODEL_PHI2
        p.seed = 1
        p.kIR = 25.0
        p.a0 = 1.0
        p.MPl = 1.0
        p.m_in_MPl = 1.0e-6
        p.fStar = 1.0
        p.epsilon = 1.0e-3
        p.gsq = 0.0
        p.initfield[0] = 11.0 * p.MPl
        p.initfield[1] = 0.0
        p.initderivs[0] = -0.815284e-6 * p.MPl * p.MPl
        p.initderivs[1] = 0.0
        p.kcutoff = 0.0
        return p.update(**overrides)

    @classmethod
    def preheating(cls, **overrides) -> "Params":
        """Two-field preheating V = m^2 phi^2/2 + g^2 phi^2 chi^2/2, g^2 = 2.5e5 m^2/MPl^2,
        phi0 = 0.193 MPl, phidot0 = -0.142 m MPl, chi0 = 0, kIR = 1 m, Yoshida-4."""
        p = cls.reference_default()
        p.nflds = 2
        p.model = MODEL_PHI2CHI2
        p.gsq = 2.5e5
        p.kIR = 1.0
        p.vv = 4
        p.initfield[0] = 0.193 * p.MPl
        p.initfield[1] = 0.0
        p.initderivs[0] = -0.142e-6 * p.MPl * p.MPl
        p.initderivs[1] = 0.0
        return p.update(**overrides)

    @classmethod
    def user_model(cls, name: str, nflds: int, initfield=(), initderivs=(), **overrides) -> "Params":
        """A run of the model.h file `name` (its file stem) compiled into the library: the
        two-field preheating setup with that model, nflds fields and the given homogeneous
        initial values (the rest zero)."""
        from .lattice import model_id

        p = cls.preheating()
        p.model = model_id(name)
        p.nflds = nflds
        for i in range(MAX_FIELDS):
            p.initfield[i] = initfield[i] if i < len(initfield) else 0.0
            p.initderivs[i] = initderivs[i] if i < len(initderivs) else 0.0
        if not initfield:
            p.initfield[0] = 0.193 * p.MPl
        if not initderivs:
            p.initderivs[0] = -0.142e-6 * p.MPl * p.MPl
        return p.update(**overrides)

    def update(self, **overrides) -> "Params":
        for k, v in overrides.items():
            if k in ("initfield", "initderivs"):
                arr = getattr(self, k)
                for i, x in enumerate(v):
                    arr[i] = x
            elif not hasattr(self, k):
                raise AttributeError(f"unknown parameter {k!r}")
            else:
                setattr(self, k, v)
        return self

    def copy(self) -> "Params":
        q = Params()
        ctypes.pointer(q)[0] = self
        return q

    # derived quantities (parameters.h:25-32, 127-133)
    @property
    def H(self) -> int:
        return self.N // 2 + 1

    @property
    def modes(self) -> int:
        return self.N * self.N * self.H

    @property
    def sites(self) -> int:
        return self.N ** 3

    @property
    def maxnumbins(self) -> int:
        return int(math.sqrt(3.0) * (self.N // 2)) + 2

    @property
    def L(self) -> float:
        return 2 * math.pi / self.kIR

    @property
    def dx(self) -> float:
        return self.L / self.N

    @property
    def f_star(self) -> float:
        return self.fStar if self.fStar > 0 else self.MPl

    @property
    def omegaStar(self) -> float:
        return self.m_in_MPl * self.f_star

    @property
    def num_potential_terms(self) -> int:
        if self.model == MODEL_PHI2:
            return 1
        if self.model == MODEL_PHI2CHI2:
            return 2
        from .lattice import load_library

        return int(load_library().psc_model_nterms(self.model))

    @property
    def stages(self) -> int:
        return {2: 1, 4: 3, 6: 7, 8: 15, 10: 31}[self.vv]

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if name in ("initfield", "initderivs") else v
        return d
