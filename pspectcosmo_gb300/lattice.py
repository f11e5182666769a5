"""Python mirror of the reference's evolution interface over the C ABI (libpsc.so).

The reference drives its path through free functions on global arrays
(pspectcosmo.h:203-272): initialize(), evolve_VV_k_nopad(dt) / evolve_VV(dt),
kernel_a_k_nopad(), and the output routines spectra(), energy(), meansvars(),
scale(). `Lattice` exposes the same operations on one device-resident lattice:

    lat = Lattice(Params.reference_default())
    lat.initialize()                 # initialize() [+ initialize_GW()]
    lat.evolve(dt, nsteps)           # nsteps x evolve_VV_k_nopad(dt) / evolve_VV(dt)
    lat.spectra(), lat.energy(), lat.meansvars(), lat.scale()

Errors from the library raise PscError (the reference exits instead,
output.cpp:450-454). The CUDA library is required: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .params import Params

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpsc.so")

PSC_OK = 0
PSC_ERR_CONFIG = -1
PSC_ERR_ARG = -2
PSC_ERR_CUDA = -3
PSC_ERR_NONFINITE = -4
PSC_ERR_TIMEOUT = -5
PSC_ERR_STATE = -6
PSC_ERR_NOMEM = -7
PSC_ERR_IO = -8
PSC_ERR_DEVICE = -9

_lib = None


class PscError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        msg = _lib.psc_last_error().decode() if _lib else ""
        name = _lib.psc_strerror(code).decode() if _lib else str(code)
        super().__init__(f"{where}: {name} ({code}): {msg}")


def load_library(path: str | None = None):
    """Load libpsc.so (built by pspectcosmo_gb300.build). Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m pspectcosmo_gb300.build` "
                           "(the CUDA path has no CPU fallback)")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    D = ctypes.POINTER(ctypes.c_double)
    I32 = ctypes.POINTER(ctypes.c_int32)
    PP = ctypes.POINTER(Params)
    L.psc_default_params.argtypes = [PP]
    L.psc_default_params.restype = None
    L.psc_create.argtypes = [PP, ctypes.POINTER(P)]
    L.psc_destroy.argtypes = [P]
    L.psc_destroy.restype = None
    L.psc_init_ic.argtypes = [P]
    L.psc_generate_ic.argtypes = [PP, D, D, D, D, D]
    L.psc_set_state.argtypes = [P, D, D, ctypes.c_double, ctypes.c_double, ctypes.c_double, D, D]
    L.psc_get_state.argtypes = [P, D, D, D, D, D, D, D]
    L.psc_get_time.argtypes = [P, D]
    L.psc_set_time.argtypes = [P, ctypes.c_double]
    L.psc_step.argtypes = [P, ctypes.c_double, ctypes.c_int]
    L.psc_get_fields_real.argtypes = [P, D, D]
    L.psc_maxnumbins.argtypes = [ctypes.c_int]
    L.psc_spectra.argtypes = [P, I32, D, D, D, I32, D, D, D]
    L.psc_energies.argtypes = [P, D, D, D, D, D, D]
    L.psc_means.argtypes = [P, D]
    L.psc_last_step_ms.argtypes = [P, ctypes.POINTER(ctypes.c_float)]
    L.psc_time_passes.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
    L.psc_pass_bytes.argtypes = [P, D]
    L.psc_batch_create.argtypes = [PP, ctypes.c_int, ctypes.POINTER(P)]
    L.psc_batch_destroy.argtypes = [P]
    L.psc_batch_destroy.restype = None
    L.psc_batch_size.argtypes = [P]
    L.psc_batch_groups.argtypes = [P]
    L.psc_batch_init_ic.argtypes = [P]
    L.psc_batch_step.argtypes = [P, ctypes.c_double, ctypes.c_int]
    L.psc_batch_last_step_ms.argtypes = [P, ctypes.POINTER(ctypes.c_float)]
    L.psc_batch_set_state.argtypes = [P, ctypes.c_int, D, D, ctypes.c_double, ctypes.c_double, ctypes.c_double, D, D]
    L.psc_batch_get_state.argtypes = [P, ctypes.c_int, D, D, D, D, D, D, D]
    L.psc_batch_spectra.argtypes = [P, ctypes.c_int, I32, D, D, D, I32, D, D, D]
    L.psc_batch_energies.argtypes = [P, ctypes.c_int, D, D, D, D, D, D]
    L.psc_batch_means.argtypes = [P, ctypes.c_int, D]
    L.psc_adjoint_chi2.argtypes = [P, ctypes.c_double, ctypes.c_int, ctypes.c_int, D, D, D, D, D]
    L.psc_adjoint_forward_chi2.argtypes = [P, ctypes.c_double, ctypes.c_int, D]
    L.psc_adjoint.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, D, D, D, D, D, D, D]
    L.psc_adjoint_forward.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, D]
    L.psc_histograms.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_double, D, D, D]
    L.psc_snapshot_arrays.argtypes = [P, D, D, D, D, D]
    L.psc_write_snapshot.argtypes = [P, ctypes.c_char_p, ctypes.c_int]
    L.psc_h5_write_f64.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                   ctypes.POINTER(D), ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
    L.psc_batch_histograms.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, D, D, D]
    L.psc_batch_write_snapshot.argtypes = [P, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
    L.psc_time_c2r.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
    L.psc_set_state_padded.argtypes = [P, ctypes.c_int, D, D, ctypes.c_double, ctypes.c_double, ctypes.c_double, D,
                                       D]
    L.psc_checkpoint_write.argtypes = [P, ctypes.c_char_p]
    L.psc_checkpoint_read.argtypes = [P, ctypes.c_char_p]
    L.psc_h5_dataset_shape.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.psc_h5_read_f64.argtypes = [ctypes.c_char_p, ctypes.c_char_p, D, ctypes.c_uint64]
    L.psc_analytic_begin.argtypes = [P]
    L.psc_analytic_step.argtypes = [P, ctypes.c_double]
    L.psc_analytic_background.argtypes = [P, D, D, D, D, D, D]
    L.psc_analytic_modes.argtypes = [P, ctypes.POINTER(ctypes.c_int), I32, D]
    L.psc_analytic_to_lattice.argtypes = [P]
    L.psc_histograms_2d.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double, D, D, D]
    L.psc_slices.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, D,
                             ctypes.POINTER(ctypes.c_longlong)]
    L.psc_selftest_bulk_wait.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
    L.psc_test_wait_hook.argtypes = [P, ctypes.c_double, ctypes.c_int]
    L.psc_test_wait_hook_pass.argtypes = [P, ctypes.c_double, ctypes.c_int, ctypes.c_int]
    I3 = ctypes.POINTER(ctypes.c_int)
    L.psc_autotune.argtypes = [P, ctypes.c_int, I3, I3]
    L.psc_get_shapes.argtypes = [P, I3]
    L.psc_set_shapes.argtypes = [P, I3]
    L.psc_set_tensor_maps.argtypes = [P, ctypes.c_int]
    L.psc_get_tensor_maps.argtypes = [P, I3]
    L.psc_batch_autotune.argtypes = [P, ctypes.c_int]
    L.psc_batch_launch_mode.argtypes = [P, ctypes.c_int, I3]
    L.psc_model_count.argtypes = []
    L.psc_model_name.argtypes = [ctypes.c_int]
    L.psc_model_name.restype = ctypes.c_char_p
    L.psc_model_find.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
    L.psc_model_nterms.argtypes = [ctypes.c_int]
    L.psc_model_eval.argtypes = [PP, ctypes.c_int, ctypes.c_longlong, D, D, D, D]
    L.psc_mass_sq_av.argtypes = [P, D]
    L.psc_strerror.argtypes = [ctypes.c_int]
    L.psc_strerror.restype = ctypes.c_char_p
    L.psc_last_error.argtypes = []
    L.psc_last_error.restype = ctypes.c_char_p
    for name in ("psc_create", "psc_init_ic", "psc_generate_ic", "psc_set_state", "psc_get_state", "psc_get_time",
                 "psc_set_time", "psc_step", "psc_get_fields_real", "psc_maxnumbins", "psc_spectra", "psc_energies",
                 "psc_means", "psc_last_step_ms", "psc_time_passes", "psc_pass_bytes", "psc_batch_create",
                 "psc_batch_size", "psc_batch_groups", "psc_batch_init_ic", "psc_batch_step", "psc_batch_last_step_ms",
                 "psc_batch_set_state", "psc_batch_get_state", "psc_batch_spectra", "psc_batch_energies",
                 "psc_batch_means", "psc_adjoint_chi2", "psc_adjoint_forward_chi2", "psc_adjoint", "psc_adjoint_forward",
                 "psc_histograms", "psc_snapshot_arrays", "psc_write_snapshot", "psc_h5_write_f64",
                 "psc_batch_histograms", "psc_batch_write_snapshot", "psc_time_c2r",
                 "psc_set_state_padded", "psc_checkpoint_write", "psc_checkpoint_read",
                 "psc_h5_dataset_shape", "psc_h5_read_f64", "psc_analytic_begin", "psc_analytic_step",
                 "psc_analytic_background", "psc_analytic_modes", "psc_analytic_to_lattice",
                 "psc_histograms_2d", "psc_slices", "psc_selftest_bulk_wait", "psc_test_wait_hook", "psc_test_wait_hook_pass",
                 "psc_model_count", "psc_model_find", "psc_model_nterms", "psc_model_eval", "psc_mass_sq_av",
                 "psc_autotune", "psc_get_shapes", "psc_set_shapes", "psc_batch_autotune", "psc_batch_launch_mode",
                 "psc_set_tensor_maps", "psc_get_tensor_maps"):
        getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _check(rc: int, where: str):
    if rc != PSC_OK:
        raise PscError(rc, where)


def h5_write(path: str, datasets: dict) -> None:
    """Write FP64 arrays of one shape as root-group datasets of an HDF5 file with the
    library's own writer (the layout of psc_write_snapshot)."""
    L = load_library()
    arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in datasets.values()]
    shape = arrs[0].shape
    if any(x.shape != shape for x in arrs):
        raise ValueError("all datasets must have the same shape")
    names = (ctypes.c_char_p * len(arrs))(*[k.encode() for k in datasets])
    ptrs = (ctypes.POINTER(ctypes.c_double) * len(arrs))(*[_dp(x) for x in arrs])
    dims = (ctypes.c_uint64 * len(shape))(*shape)
    _check(L.psc_h5_write_f64(os.fsencode(path), len(arrs), names, ptrs, len(shape), dims), "psc_h5_write_f64")


def h5_read(path: str, name: str) -> np.ndarray:
    """One FP64 dataset of a file in the library's HDF5 layout (snapshots, checkpoints)."""
    L = load_library()
    dims = (ctypes.c_uint64 * 32)()
    rank = ctypes.c_int()
    _check(L.psc_h5_dataset_shape(os.fsencode(path), name.encode(), dims, 32, ctypes.byref(rank)),
           "psc_h5_dataset_shape")
    shape = tuple(int(dims[i]) for i in range(rank.value))
    out = np.empty(shape, dtype=np.float64)
    _check(L.psc_h5_read_f64(os.fsencode(path), name.encode(), _dp(out), out.size), "psc_h5_read_f64")
    return out


def model_id(name: str) -> int:
    """The model id of a model.h compiled into the library (its file stem) or of a built-in
    model ("builtin:phi2", "builtin:phi2chi2")."""
    L = load_library()
    mid = ctypes.c_int()
    _check(L.psc_model_find(name.encode(), ctypes.byref(mid)), "psc_model_find")
    return mid.value


def model_names() -> dict:
    """{id: name} of every model of this build."""
    L = load_library()
    ids = [0, 1] + [16 + i for i in range(L.psc_model_count())]
    return {i: L.psc_model_name(i).decode() for i in ids}


def model_eval(params: Params, fields, on_device: bool = True) -> dict:
    """dvdf, the potential terms and effective_mass of params' model at the field points
    fields[n][nflds] (psc_model_eval): in the lattice's arithmetic, on the GPU or the host."""
    L = load_library()
    x = np.ascontiguousarray(fields, np.float64).reshape(-1, params.nflds)
    n = x.shape[0]
    nt = L.psc_model_nterms(params.model)
    d = np.zeros((n, params.nflds))
    t = np.zeros((n, nt))
    m = np.zeros((n, params.nflds))
    _check(L.psc_model_eval(ctypes.byref(params), int(on_device), n, _dp(x), _dp(d), _dp(t), _dp(m)), "psc_model_eval")
    return dict(dvdf=d, terms=t, mass_sq=m)


def generate_ic(params: Params):
    """Host-only initial conditions (initialize() / initialize_GW()) as numpy arrays."""
    L = load_library()
    p = params
    f = np.zeros((p.nflds, p.modes), np.complex128)
    pi = np.zeros((p.nflds, p.modes), np.complex128)
    u = np.zeros((6, p.modes), np.complex128) if p.with_gw else None
    pu = np.zeros((6, p.modes), np.complex128) if p.with_gw else None
    info = np.zeros(6)
    _check(L.psc_generate_ic(ctypes.byref(p), _dp(f), _dp(pi), _dp(u), _dp(pu), _dp(info)), "psc_generate_ic")
    keys = ("hubble_init", "a", "ad", "add_printed", "kinetic", "potential")
    return f, pi, u, pu, dict(zip(keys, info.tolist()))


class Lattice:
    """One lattice on the current CUDA device (a psc_handle)."""

    def __init__(self, params: Params):
        self.p = params.copy()
        self._L = load_library()
        h = ctypes.c_void_p()
        _check(self._L.psc_create(ctypes.byref(self.p), ctypes.byref(h)), "psc_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.psc_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- initialize() / state -------------------------------------------------
    def initialize(self):
        """initialize() (initialize.cpp:562) and, with GWs, initialize_GW() (initialize.cpp:341)."""
        _check(self._L.psc_init_ic(self._h), "psc_init_ic")

    def set_state(self, f_k, pi_k, a, ad, add, u_k=None, pi_u_k=None):
        c = lambda x: None if x is None else np.ascontiguousarray(x, np.complex128)
        f_k, pi_k, u_k, pi_u_k = c(f_k), c(pi_k), c(u_k), c(pi_u_k)
        _check(self._L.psc_set_state(self._h, _dp(f_k), _dp(pi_k), a, ad, add, _dp(u_k), _dp(pi_u_k)),
               "psc_set_state")

    def set_state_padded(self, Nsrc: int, f_k, pi_k, a, ad, add, u_k=None, pi_u_k=None):
        """State of a coarser Nsrc lattice, spectrally interpolated to this N (padding(),
        evolution.cpp:1271-1443, amplitudes x (N/Nsrc)^3)."""
        c = lambda x: None if x is None else np.ascontiguousarray(x, np.complex128)
        f_k, pi_k, u_k, pi_u_k = c(f_k), c(pi_k), c(u_k), c(pi_u_k)
        _check(self._L.psc_set_state_padded(self._h, int(Nsrc), _dp(f_k), _dp(pi_k), a, ad, add, _dp(u_k),
                                            _dp(pi_u_k)), "psc_set_state_padded")

    def get_state(self, out: dict | None = None):
        """The state (psc_get_state). `out` (optional): caller-owned arrays f_k, pi_k and,
        with GWs, u_k, pi_u_k, C-contiguous complex128 of the returned shapes (e.g. in
        pinned host memory, reused across calls); they are filled and returned."""
        p = self.p
        shapes = dict(f_k=(p.nflds, p.modes), pi_k=(p.nflds, p.modes), u_k=(6, p.modes), pi_u_k=(6, p.modes))
        if out is not None:
            for k in ("f_k", "pi_k") + (("u_k", "pi_u_k") if p.with_gw else ()):
                x = out[k]
                if (not isinstance(x, np.ndarray) or x.dtype != np.complex128 or x.shape != shapes[k]
                        or not x.flags.c_contiguous or not x.flags.writeable):
                    raise ValueError(f"out[{k!r}] must be a writeable C-contiguous complex128 array of shape "
                                     f"{shapes[k]}")
            f, pi = out["f_k"], out["pi_k"]
            u, pu = (out["u_k"], out["pi_u_k"]) if p.with_gw else (None, None)
        else:
            # psc_get_state writes every element (no zero fill needed)
            f = np.empty(shapes["f_k"], np.complex128)
            pi = np.empty(shapes["pi_k"], np.complex128)
            u = np.empty(shapes["u_k"], np.complex128) if p.with_gw else None
            pu = np.empty(shapes["pi_u_k"], np.complex128) if p.with_gw else None
        a, ad, add = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(self._L.psc_get_state(self._h, _dp(f), _dp(pi), ctypes.byref(a), ctypes.byref(ad), ctypes.byref(add),
                                     _dp(u), _dp(pu)), "psc_get_state")
        return dict(f_k=f, pi_k=pi, u_k=u, pi_u_k=pu, a=a.value, ad=ad.value, add=add.value)

    @property
    def t(self) -> float:
        v = ctypes.c_double()
        _check(self._L.psc_get_time(self._h, ctypes.byref(v)), "psc_get_time")
        return v.value

    @t.setter
    def t(self, value: float):
        _check(self._L.psc_set_time(self._h, float(value)), "psc_set_time")

    def background(self) -> dict:
        st = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(self._L.psc_get_state(self._h, None, None, *(ctypes.byref(x) for x in st), None, None), "psc_get_state")
        return dict(t=self.t, a=st[0].value, ad=st[1].value, add=st[2].value)

    # -- evolution ------------------------------------------------------------
    def evolve(self, dt: float, nsteps: int = 1):
        """nsteps calls of evolve_VV_k_nopad(dt) (spectral) or evolve_VV(dt) (real space)."""
        _check(self._L.psc_step(self._h, float(dt), int(nsteps)), "psc_step")

    def last_step_ms(self) -> float:
        v = ctypes.c_float()
        _check(self._L.psc_last_step_ms(self._h, ctypes.byref(v)), "psc_last_step_ms")
        return v.value

    # -- FFT tile / grid shapes -----------------------------------------------
    def autotune(self, reps: int = 3) -> dict:
        """Time the candidate tile and grid shapes of the passes on the current state and keep
        the fastest (psc_autotune). Returns shape = (log2 X/Y lines per tile, log2 Z lines per
        tile, Z blocks per SM) and from_cache."""
        sh = (ctypes.c_int * 3)()
        fc = ctypes.c_int()
        _check(self._L.psc_autotune(self._h, int(reps), sh, ctypes.byref(fc)), "psc_autotune")
        return dict(shape=tuple(sh), from_cache=bool(fc.value))

    @property
    def shapes(self) -> tuple:
        sh = (ctypes.c_int * 3)()
        _check(self._L.psc_get_shapes(self._h, sh), "psc_get_shapes")
        return tuple(sh)

    @shapes.setter
    def shapes(self, value):
        sh = (ctypes.c_int * 3)(*[int(x) for x in value])
        _check(self._L.psc_set_shapes(self._h, sh), "psc_set_shapes")

    TMAP_X, TMAP_Y, TMAP_YINV = 1, 2, 4

    @property
    def tensor_maps(self) -> int:
        """The pass groups that stage their tiles by tensor maps (TMAP_X | TMAP_Y | TMAP_YINV bits)."""
        m = ctypes.c_int()
        _check(self._L.psc_get_tensor_maps(self._h, ctypes.byref(m)), "psc_get_tensor_maps")
        return m.value

    @tensor_maps.setter
    def tensor_maps(self, mask: int):
        _check(self._L.psc_set_tensor_maps(self._h, int(mask)), "psc_set_tensor_maps")

    # -- adjoint --------------------------------------------------------------
    def adjoint_chi2(self, dt: float, nsteps: int, every: int = 0, fields: bool = True) -> dict:
        """O = <chi^2> after nsteps and its gradient with respect to the current state.

        Returns O, grad_f_k / grad_pi_k (dO/dRe + i dO/dIm per stored mode, shaped like the
        state; None when fields is False), grad_ad0 (dO/da' at fixed a) and grad_theta =
        (dO/dgsq, dO/dmu). The lattice is left at the final state; last_step_ms() gives the
        device time of the computation.
        """
        p = self.p
        O, gad = ctypes.c_double(), ctypes.c_double()
        gf = np.zeros((p.nflds, p.modes), np.complex128) if fields else None
        gp = np.zeros((p.nflds, p.modes), np.complex128) if fields else None
        gth = np.zeros(2)
        _check(self._L.psc_adjoint_chi2(self._h, float(dt), int(nsteps), int(every), ctypes.byref(O), _dp(gf), _dp(gp),
                                        ctypes.byref(gad), _dp(gth)), "psc_adjoint_chi2")
        return dict(O=O.value, grad_f_k=gf, grad_pi_k=gp, grad_ad0=gad.value, grad_theta=gth)

    OBSERVABLES = {"chi2": 0, "rho_gw": 1}

    def adjoint(self, observable: str, dt: float, nsteps: int, every: int = 0, fields: bool = True) -> dict:
        """O (observable "chi2" = <chi^2> or "rho_gw" = the GW energy density) after nsteps and
        its gradient with respect to the current state: grad_f_k, grad_pi_k and, on a GW lattice,
        grad_u_k, grad_pi_u_k (dO/dRe + i dO/dIm per stored mode), grad_ad0, grad_theta =
        (dO/dgsq, dO/dmu). The lattice is left at the final state."""
        p = self.p
        O, gad = ctypes.c_double(), ctypes.c_double()
        gf = np.zeros((p.nflds, p.modes), np.complex128) if fields else None
        gp = np.zeros((p.nflds, p.modes), np.complex128) if fields else None
        gu = np.zeros((6, p.modes), np.complex128) if (fields and p.with_gw) else None
        gpu = np.zeros((6, p.modes), np.complex128) if (fields and p.with_gw) else None
        gth = np.zeros(2)
        _check(self._L.psc_adjoint(self._h, self.OBSERVABLES[observable], float(dt), int(nsteps), int(every),
                                   ctypes.byref(O), _dp(gf), _dp(gp), _dp(gu), _dp(gpu), ctypes.byref(gad), _dp(gth)),
               "psc_adjoint")
        return dict(O=O.value, grad_f_k=gf, grad_pi_k=gp, grad_u_k=gu, grad_pi_u_k=gpu, grad_ad0=gad.value,
                    grad_theta=gth)

    def adjoint_forward(self, observable: str, dt: float, nsteps: int) -> float:
        """O after nsteps of the product step from a''(0) = A(state(0)) (no gradient)."""
        O = ctypes.c_double()
        _check(self._L.psc_adjoint_forward(self._h, self.OBSERVABLES[observable], float(dt), int(nsteps),
                                           ctypes.byref(O)), "psc_adjoint_forward")
        return O.value

    def adjoint_forward_chi2(self, dt: float, nsteps: int) -> float:
        """O = <chi^2> after nsteps of the adjoint's own (unfused) forward map."""
        O = ctypes.c_double()
        _check(self._L.psc_adjoint_forward_chi2(self._h, float(dt), int(nsteps), ctypes.byref(O)),
               "psc_adjoint_forward_chi2")
        return O.value

    PASS_NAMES = ("ifft_x", "ifft_y", "zpass", "fft_y", "fft_x_kick", "background")

    def time_passes(self, reps: int = 5) -> dict:
        """Average device ms of each pass of one stage (CUDA events on the lattice's stream)."""
        ms = (ctypes.c_float * 6)()
        _check(self._L.psc_time_passes(self._h, int(reps), ms), "psc_time_passes")
        return dict(zip(self.PASS_NAMES, [float(x) for x in ms]))

    def time_c2r(self, reps: int = 10) -> float:
        """Device ms of one c2r of the field arrays to real space (the library's 3-D c2r)."""
        v = ctypes.c_float()
        _check(self._L.psc_time_c2r(self._h, int(reps), ctypes.byref(v)), "psc_time_c2r")
        return v.value

    def pass_bytes(self) -> dict:
        """Compulsory HBM bytes per launch of each pass."""
        b = np.zeros(6)
        _check(self._L.psc_pass_bytes(self._h, _dp(b)), "psc_pass_bytes")
        return dict(zip(self.PASS_NAMES, b.tolist()))

    # -- outputs --------------------------------------------------------------
    def fields_real(self):
        p = self.p
        f = np.zeros((p.nflds, p.N, p.N, p.N))
        pi = np.zeros((p.nflds, p.N, p.N, p.N))
        _check(self._L.psc_get_fields_real(self._h, _dp(f), _dp(pi)), "psc_get_fields_real")
        return f, pi

    def spectra_raw(self) -> dict:
        p = self.p
        nb = p.maxnumbins
        out = dict(numpoints=np.zeros((p.nflds, nb), np.int32), f2=np.zeros((p.nflds, nb)),
                   pi2=np.zeros((p.nflds, nb)), n2=np.zeros((p.nflds, nb)))
        if p.with_gw:
            out.update(gw_numpoints=np.zeros(nb, np.int32), h2=np.zeros(nb), hdot2=np.zeros(nb))
        hz = ctypes.c_double(0.0)
        _check(self._L.psc_spectra(self._h, _ip(out["numpoints"]), _dp(out["f2"]), _dp(out["pi2"]), _dp(out["n2"]),
                                   _ip(out.get("gw_numpoints")), _dp(out.get("h2")), _dp(out.get("hdot2")),
                                   ctypes.byref(hz)), "psc_spectra")
        out["hdot2_zero"] = hz.value
        return out

    def energies(self) -> dict:
        p = self.p
        K, G, V = np.zeros(p.nflds), np.zeros(p.nflds), np.zeros(p.num_potential_terms)
        tot, fv, rho = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(self._L.psc_energies(self._h, _dp(K), _dp(G), _dp(V), ctypes.byref(tot), ctypes.byref(fv),
                                    ctypes.byref(rho)), "psc_energies")
        return dict(K=K, G=G, V=V, total=tot.value, friedmann_violation=fv.value, rho_gw=rho.value)

    def means(self) -> np.ndarray:
        out = np.zeros((self.p.nflds, 6))
        _check(self._L.psc_means(self._h, _dp(out)), "psc_means")
        return out

    def mass_sq_av(self) -> np.ndarray:
        """<effective_mass(f(x))> over the lattice ([nflds]), the mass_sq_av of spectra()
        (output.cpp:566-580)."""
        out = np.zeros(self.p.nflds)
        _check(self._L.psc_mass_sq_av(self._h, _dp(out)), "psc_mass_sq_av")
        return out

    def histograms(self, nbins: int = 256, hmin: float = 0.0, hmax: float = 0.0) -> dict:
        """histograms() (output.cpp:1193-1297): binfreq [nflds][nbins], bmin, df [nflds]."""
        p = self.p
        freq, bmin, df = np.zeros((p.nflds, nbins)), np.zeros(p.nflds), np.zeros(p.nflds)
        _check(self._L.psc_histograms(self._h, int(nbins), float(hmin), float(hmax), _dp(freq), _dp(bmin), _dp(df)),
               "psc_histograms")
        return dict(binfreq=freq, bmin=bmin, df=df)

    def histograms_2d(self, fld1: int = 0, fld2: int = 1, nbins0: int = 10, nbins1: int = 10, hmin: float = 0.0,
                      hmax: float = 0.0) -> dict:
        """histograms_2d() (output.cpp:1300-1413): binfreq [nbins0][nbins1], bmin [2], df [2]."""
        freq, bmin, df = np.zeros((nbins0, nbins1)), np.zeros(2), np.zeros(2)
        _check(self._L.psc_histograms_2d(self._h, fld1, fld2, nbins0, nbins1, float(hmin), float(hmax), _dp(freq),
                                         _dp(bmin), _dp(df)), "psc_histograms_2d")
        return dict(binfreq=freq, bmin=bmin, df=df)

    def slices(self, slicedim: int = 1, slicelength: int | None = None, sliceskip: int = 1,
               sliceaverage: int = 1) -> np.ndarray:
        """slices() (output.cpp:1415-1539): [nflds][count] values in output order."""
        length = self.p.N if slicelength is None else slicelength
        cnt = ctypes.c_longlong()
        _check(self._L.psc_slices(self._h, slicedim, length, sliceskip, sliceaverage, None, ctypes.byref(cnt)),
               "psc_slices")
        out = np.zeros((self.p.nflds, cnt.value))
        _check(self._L.psc_slices(self._h, slicedim, length, sliceskip, sliceaverage, _dp(out), ctypes.byref(cnt)),
               "psc_slices")
        return out

    def snapshot_arrays(self, fields: bool = True, energy: bool = True) -> dict:
        """The datasets of snapshots() (output.cpp:1541-1648) as [N][N][N] arrays."""
        p = self.p
        sh = (p.N, p.N, p.N)
        out = {}
        if fields:
            out["f"] = np.zeros((p.nflds,) + sh)
        if energy:
            for k in ("pot", "kin", "grad", "tot"):
                out[k] = np.zeros(sh)
        _check(self._L.psc_snapshot_arrays(self._h, _dp(out.get("f")), _dp(out.get("pot")), _dp(out.get("kin")),
                                           _dp(out.get("grad")), _dp(out.get("tot"))), "psc_snapshot_arrays")
        return out

    # -- analytic pre-lattice phase (ANALYTIC_EVOLUTION) ---------------------------------
    def analytic_begin(self):
        """k_square_initialize + initialize_analytic_perturbation (initialize.cpp:815-958)."""
        _check(self._L.psc_analytic_begin(self._h), "psc_analytic_begin")

    def analytic_step(self, dt: float):
        """evolve_VV_analytic_perturbation(dt) (evolution.cpp:167-336)."""
        _check(self._L.psc_analytic_step(self._h, float(dt)), "psc_analytic_step")

    def analytic_background(self) -> dict:
        nf = self.p.nflds
        t, a, ad, add = (ctypes.c_double() for _ in range(4))
        f, pi = np.zeros(nf), np.zeros(nf)
        _check(self._L.psc_analytic_background(self._h, ctypes.byref(t), ctypes.byref(a), ctypes.byref(ad),
                                               ctypes.byref(add), _dp(f), _dp(pi)), "psc_analytic_background")
        return dict(t=t.value, a=a.value, ad=ad.value, add=add.value, f=f, pi=pi)

    def analytic_modes(self):
        """(k2 [nk], modes [4][nflds][nk] complex: f_left, pi_left, f_right, pi_right)."""
        nk = ctypes.c_int()
        _check(self._L.psc_analytic_modes(self._h, ctypes.byref(nk), None, None), "psc_analytic_modes")
        k2 = np.zeros(nk.value, np.int32)
        modes = np.zeros((4, self.p.nflds, nk.value), np.complex128)
        _check(self._L.psc_analytic_modes(self._h, ctypes.byref(nk), _ip(k2), _dp(modes)), "psc_analytic_modes")
        return k2, modes

    def analytic_to_lattice(self):
        """initialize_lattice() (initialize.cpp:961-1097)."""
        _check(self._L.psc_analytic_to_lattice(self._h), "psc_analytic_to_lattice")

    def checkpoint(self, path: str) -> None:
        """Full state, background and time to an HDF5 checkpoint file."""
        _check(self._L.psc_checkpoint_write(self._h, os.fsencode(path)), "psc_checkpoint_write")

    def restore(self, path: str) -> None:
        """Resume from a checkpoint file of a lattice with the same N, nflds, with_gw."""
        _check(self._L.psc_checkpoint_read(self._h, os.fsencode(path)), "psc_checkpoint_read")

    def write_snapshot(self, path: str, with_energy: bool = True) -> None:
        """The reference's data_<step>_snapshot.h5 (output.cpp:1541-1648) at `path`."""
        _check(self._L.psc_write_snapshot(self._h, os.fsencode(path), int(bool(with_energy))), "psc_write_snapshot")

    # reference-named output rows (the columns the reference writes)
    def spectra(self) -> dict:
        from .outputs import spectra_rows

        return spectra_rows(self.p, self.background(), self.spectra_raw(), self.energies()["total"])

    def energy(self) -> dict:
        from .outputs import energy_rows

        return energy_rows(self.p, self.background(), self.energies())

    def meansvars(self) -> np.ndarray:
        return self.means()

    def scale(self) -> list:
        from .outputs import scale_row

        return scale_row(self.p, self.background())


class Ensemble:
    """Independent realizations (possibly of different lattice sizes) advanced together:
    one launch per pass per same-configuration group, one CUDA graph per step."""

    def __init__(self, params_list):
        self.params = [q.copy() for q in params_list]
        self._L = load_library()
        arr = (Params * len(self.params))(*self.params)
        h = ctypes.c_void_p()
        _check(self._L.psc_batch_create(arr, len(self.params), ctypes.byref(h)), "psc_batch_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.psc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return self._L.psc_batch_size(self._h)

    @property
    def groups(self) -> int:
        return self._L.psc_batch_groups(self._h)

    def initialize(self):
        _check(self._L.psc_batch_init_ic(self._h), "psc_batch_init_ic")

    def evolve(self, dt: float, nsteps: int = 1):
        _check(self._L.psc_batch_step(self._h, float(dt), int(nsteps)), "psc_batch_step")

    def autotune(self, reps: int = 3):
        """psc_autotune for every same-configuration group (psc_batch_autotune)."""
        _check(self._L.psc_batch_autotune(self._h, int(reps)), "psc_batch_autotune")

    def launch_mode(self, per_group: bool | None = None) -> bool:
        """True when the batch advances with one launch per pass for all its groups
        (psc_batch_launch_mode); per_group=True asks for the per-group launches, False for the
        default, None leaves the choice."""
        v = ctypes.c_int()
        _check(self._L.psc_batch_launch_mode(self._h, -1 if per_group is None else int(per_group), ctypes.byref(v)),
               "psc_batch_launch_mode")
        return bool(v.value)

    def last_step_ms(self) -> float:
        v = ctypes.c_float()
        _check(self._L.psc_batch_last_step_ms(self._h, ctypes.byref(v)), "psc_batch_last_step_ms")
        return v.value

    def get_state(self, idx: int):
        p = self.params[idx]
        f = np.empty((p.nflds, p.modes), np.complex128)
        pi = np.empty((p.nflds, p.modes), np.complex128)
        u = np.empty((6, p.modes), np.complex128) if p.with_gw else None
        pu = np.empty((6, p.modes), np.complex128) if p.with_gw else None
        a, ad, add = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(self._L.psc_batch_get_state(self._h, idx, _dp(f), _dp(pi), ctypes.byref(a), ctypes.byref(ad),
                                           ctypes.byref(add), _dp(u), _dp(pu)), "psc_batch_get_state")
        return dict(f_k=f, pi_k=pi, u_k=u, pi_u_k=pu, a=a.value, ad=ad.value, add=add.value)

    def spectra_raw(self, idx: int) -> dict:
        p = self.params[idx]
        nb = p.maxnumbins
        out = dict(numpoints=np.zeros((p.nflds, nb), np.int32), f2=np.zeros((p.nflds, nb)),
                   pi2=np.zeros((p.nflds, nb)), n2=np.zeros((p.nflds, nb)))
        hz = ctypes.c_double(0.0)
        _check(self._L.psc_batch_spectra(self._h, idx, _ip(out["numpoints"]), _dp(out["f2"]), _dp(out["pi2"]),
                                         _dp(out["n2"]), None, None, None, ctypes.byref(hz)), "psc_batch_spectra")
        return out

    def histograms(self, idx: int, nbins: int = 256, hmin: float = 0.0, hmax: float = 0.0) -> dict:
        p = self.params[idx]
        freq, bmin, df = np.zeros((p.nflds, nbins)), np.zeros(p.nflds), np.zeros(p.nflds)
        _check(self._L.psc_batch_histograms(self._h, idx, int(nbins), float(hmin), float(hmax), _dp(freq), _dp(bmin),
                                            _dp(df)), "psc_batch_histograms")
        return dict(binfreq=freq, bmin=bmin, df=df)

    def write_snapshot(self, idx: int, path: str, with_energy: bool = True) -> None:
        _check(self._L.psc_batch_write_snapshot(self._h, idx, os.fsencode(path), int(bool(with_energy))),
               "psc_batch_write_snapshot")

    def energies(self, idx: int) -> dict:
        p = self.params[idx]
        K, G, V = np.zeros(p.nflds), np.zeros(p.nflds), np.zeros(p.num_potential_terms)
        tot, fv, rho = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(self._L.psc_batch_energies(self._h, idx, _dp(K), _dp(G), _dp(V), ctypes.byref(tot), ctypes.byref(fv),
                                          ctypes.byref(rho)), "psc_batch_energies")
        return dict(K=K, G=G, V=V, total=tot.value, friedmann_violation=fv.value, rho_gw=rho.value)
