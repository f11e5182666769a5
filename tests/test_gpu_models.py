"""The model surface on the GPU: model.h files compiled into the library (user models).

* The device compilation of every user model equals its host compilation (psc_model_eval)
  to FP64 / FP32 rounding (the device fuses multiply-adds).
* Three and four fields (pspectcosmo_gb300/models/three_field.h, four_field.h) against the
  reference's own code built with that model.h and nflds = 3 or 4 (golden fixtures): the spectral step and the real-space step
  with GWs at 16^3 (the generic engine; full final state) and at 32^3 (the register engine's
  user-model Z passes; outputs at every output step). FP64 at the bars of the two-field runs:
  states 1e-10, spectra 1e-10 (spectral) or 1e-7 (real space, the reference's rounding floor
  of phi0 + dphi in real space), bin counts exact; n_k at 1e-9. FP32 against FP64 at 128^3.
* A model.h restating a built-in model (phi2chi2.h, phi2.h) runs the user-model path and
  matches the built-in path: the 256^3 benchmark lattice (GW Z pass staged by bulk copies) and
  the spectral step.
"""
import numpy as np
import pytest

from golden_util import load, output_rows, params_for, rel

pytestmark = pytest.mark.gpu

REALSPACE_SPEC_TOL = 1e-7
# the occupation number n_k of the third field (sigma, with a large homogeneous value) cancels
# in |a^(alpha-3) pi + H f|^2 and in its effective-mass mean: measured 1.7e-10 on GB300
THREE_FIELD_NK_TOL = 1e-9


def _lattice(p):
    from pspectcosmo_gb300 import Lattice

    return Lattice(p)


@pytest.mark.parametrize("name,nf", [("phi2", 1), ("phi2chi2", 2), ("three_field", 3), ("four_field", 4)])
@pytest.mark.parametrize("precision", [64, 32])
def test_device_model_equals_host_model(name, nf, precision):
    from pspectcosmo_gb300 import Params
    from pspectcosmo_gb300.lattice import model_eval

    p = Params.user_model(name, nf, precision=precision)
    rng = np.random.default_rng(7)
    x = rng.uniform(-0.3, 0.3, size=(4096, nf))
    dev = model_eval(p, x, on_device=True)
    host = model_eval(p, x, on_device=False)
    tol = 1e-14 if precision == 64 else 1e-6
    for k in ("dvdf", "terms", "mass_sq"):
        assert rel(dev[k], host[k]) < (1e-14 if k == "mass_sq" else tol), k


def _compare_rows(rows, g, blk, p, tol, tol_nk, tol_e):
    for f in range(p.nflds):
        ref = g[f"spectra_scalar_{f}"][blk]
        got = rows[f"spectra_scalar_{f}"]
        assert np.array_equal(got[:, 4].astype(int), ref[:, 4].astype(int)), "bin counts"
        for c in (1, 2):
            assert rel(got[:, c], ref[:, c]) < tol, f"field {f} spectra column {c}"
        assert rel(got[:, 3], ref[:, 3]) < tol_nk, f"field {f} n_k"
    en = rows["energies"]
    vals = []
    for f in range(p.nflds):
        vals += [en["K"][f], en["G"][f]]
    vals += list(en["V"]) + [en["total"]]
    assert rel(vals, g["average_energies"][blk][1:]) < tol_e, "energies"
    if p.with_gw:
        ref = g["spectra_gws"][blk]
        got = rows["spectra_gws"]
        assert np.array_equal(got[:, 4].astype(int), ref[:, 4].astype(int))
        for c in (1, 2):
            assert rel(got[:, c], ref[:, c]) < tol, f"GW spectra column {c}"


@pytest.mark.parametrize("run", ["spec3_n16_vv4", "gw3_n16_vv4", "gw4_n16_vv2"])
def test_user_models_fp64_match_reference_16(run):
    """Three or four fields, 16^3, from the device initial conditions: ICs, final state and outputs
    against the reference's own run."""
    g, meta = load(run)
    p = params_for(meta, 64)
    lat = _lattice(p)
    lat.initialize()
    st = lat.get_state()
    n = g["ic_f_k"].shape[1]
    assert rel(st["f_k"][:, :n], g["ic_f_k"]) < 1e-13 and rel(st["pi_k"][:, :n], g["ic_pi_k"]) < 1e-13
    lat.evolve(meta["dt"], meta["nsteps"])
    st = lat.get_state()
    ref = g["bg"][-1]
    assert rel(st["a"], ref[2]) < 1e-12 and rel(st["ad"], ref[3]) < 1e-12 and rel(st["add"], ref[4]) < 1e-10
    N = p.N
    if p.spectral:
        assert rel(st["f_k"], g["fin_f_k"]) < 1e-10 and rel(st["pi_k"], g["fin_pi_k"]) < 1e-10
        tol = 1e-10
    else:
        fr, pr = lat.fields_real()
        assert rel(fr.reshape(p.nflds, N, N, N), g["fin_f"]) < 1e-10
        assert rel(pr.reshape(p.nflds, N, N, N), g["fin_pi_f"]) < 1e-10
        uk = np.fft.rfftn(g["fin_u"], axes=(1, 2, 3)).reshape(6, -1)
        puk = np.fft.rfftn(g["fin_pi_u"], axes=(1, 2, 3)).reshape(6, -1)
        assert rel(st["u_k"], uk) < 1e-10 and rel(st["pi_u_k"], puk) < 1e-10
        tol = REALSPACE_SPEC_TOL
    _compare_rows(output_rows(lat, p), g, -1, p, tol, max(tol, THREE_FIELD_NK_TOL), 1e-11)
    lat.close()


@pytest.mark.parametrize("run", ["spec3_n32_vv2", "gw3_n32_vv4", "gw4_n32_vv2"])
def test_user_models_fp64_match_reference_32(run):
    """Three or four fields, 32^3 (register engine, user-model Z passes), FP64: outputs at every output
    step of the reference's run."""
    g, meta = load(run)
    p = params_for(meta, 64)
    lat = _lattice(p)
    lat.initialize()
    st = lat.get_state()
    n = g["ic_f_k"].shape[1]
    assert rel(st["f_k"][:, :n], g["ic_f_k"]) < 1e-13 and rel(st["pi_k"][:, :n], g["ic_pi_k"]) < 1e-13
    tol = 1e-10 if p.spectral else REALSPACE_SPEC_TOL
    every = meta["every"]
    for blk in range(1, meta["nsteps"] // every + 1):
        lat.evolve(meta["dt"], every)
        bg = lat.background()
        ref = g["bg"][blk * every]
        assert rel(bg["a"], ref[2]) < 1e-12 and rel(bg["ad"], ref[3]) < 1e-12
        _compare_rows(output_rows(lat, p), g, blk, p, tol, max(tol, THREE_FIELD_NK_TOL), 1e-11)
    lat.close()


def test_three_fields_fp32_against_fp64_128():
    """Three fields with GWs at 128^3 (Yoshida-4, dt 0.005, 40 steps), FP32 against the FP64
    path from the same initial state, sigma starting at 0: the errors of the two-field model
    at this size (measured on GB300: P_f, P_pi of phi 2.6e-4, 1.9e-4, as the built-in
    two-field model's; chi, sigma and the GW spectra <= 6e-7). A field with a large homogeneous
    value (sigma0 = 0.01) has fluctuations near FP32 resolution per site: its FP32 spectrum is
    off by 1e-1 after 40 steps, the limitation the homogeneous FP64 modes do not lift."""
    from pspectcosmo_gb300 import Params

    p64 = Params.user_model("three_field", 3, initfield=(0.193, 0.0, 0.0), initderivs=(-0.142e-6, 0.0, 0.0),
                            N=128, vv=4, spectral=0, with_gw=1, precision=64)
    p32 = p64.copy()
    p32.precision = 32
    a, b = _lattice(p64), _lattice(p32)
    a.initialize()
    s0 = a.get_state()
    b.set_state(s0["f_k"], s0["pi_k"], s0["a"], s0["ad"], s0["add"], s0["u_k"], s0["pi_u_k"])
    a.evolve(0.005, 40)
    b.evolve(0.005, 40)
    ra, rb = output_rows(a, p64), output_rows(b, p32)
    for f, tol in ((0, 1e-3), (1, 1e-5), (2, 1e-5)):
        for c in (1, 2):
            assert rel(rb[f"spectra_scalar_{f}"][:, c], ra[f"spectra_scalar_{f}"][:, c]) < tol, (f, c)
    for c in (1, 2):
        assert rel(rb["spectra_gws"][:, c], ra["spectra_gws"][:, c]) < 1e-5, c
    assert rel(b.background()["a"], a.background()["a"]) < 1e-7
    a.close()
    b.close()


@pytest.mark.parametrize("precision", [64, 32])
def test_user_phi2chi2_matches_builtin_at_benchmark_lattice(precision):
    """phi2chi2.h through the user-model path against the built-in two-field model on the
    256^3 two-field + GW lattice (Yoshida-4, dt 0.005, 2 steps from the same state): the
    same formulas, so FP64 agrees to rounding and FP32 to FP32 rounding."""
    from pspectcosmo_gb300 import Params

    pb = Params.preheating(N=256, vv=4, spectral=0, with_gw=1, precision=precision)
    pu = Params.user_model("phi2chi2", 2, N=256, vv=4, spectral=0, with_gw=1, precision=precision)
    a = _lattice(pb)
    a.initialize()
    s0 = a.get_state()
    a.evolve(0.005, 2)
    sa = a.get_state()
    a.close()
    b = _lattice(pu)
    b.set_state(s0["f_k"], s0["pi_k"], s0["a"], s0["ad"], s0["add"], s0["u_k"], s0["pi_u_k"])
    b.evolve(0.005, 2)
    sb = b.get_state()
    b.close()
    tol = 1e-12 if precision == 64 else 2e-5
    for k in ("f_k", "pi_k", "u_k", "pi_u_k"):
        assert rel(sb[k], sa[k]) < tol, k
    assert rel(sb["a"], sa["a"]) < (1e-14 if precision == 64 else 1e-9)


def test_user_phi2_matches_builtin_spectral():
    """phi2.h (the shipped model restated) on the spectral step at 64^3, FP64."""
    from pspectcosmo_gb300 import Params
    from pspectcosmo_gb300.lattice import model_id

    pb = Params.reference_default(N=64)
    pu = Params.reference_default(N=64)
    pu.model = model_id("phi2")
    a, b = _lattice(pb), _lattice(pu)
    a.initialize()
    b.initialize()
    a.evolve(1e-4, 20)
    b.evolve(1e-4, 20)
    sa, sb = a.get_state(), b.get_state()
    assert rel(sb["f_k"], sa["f_k"]) < 1e-13 and rel(sb["pi_k"], sa["pi_k"]) < 1e-13
    ra, rb = output_rows(a, pb), output_rows(b, pu)
    assert rel(rb["spectra_scalar_0"][:, 3], ra["spectra_scalar_0"][:, 3]) < 1e-12
    a.close()
    b.close()


def test_user_model_limits():
    from pspectcosmo_gb300 import Params
    from pspectcosmo_gb300.lattice import PSC_ERR_CONFIG, PscError

    p = Params.user_model("three_field", 3, N=1024, spectral=0, with_gw=1)
    with pytest.raises(PscError) as e:
        _lattice(p)
    assert e.value.code == PSC_ERR_CONFIG
    p = Params.user_model("three_field", 3, N=32, spectral=0, with_gw=0, simulate_inflation=0)
    lat = _lattice(p)
    lat.initialize()
    with pytest.raises(PscError) as e:
        lat.adjoint_chi2(0.005, 2)
    assert e.value.code == PSC_ERR_CONFIG
    lat.close()


def test_user_model_batch_equals_individual_lattices():
    """Realizations of a model.h compiled in (three fields, GW, 32^3 and 64^3 groups) advanced
    as a batch equal the lattices advanced alone, bit for bit."""
    from pspectcosmo_gb300 import Ensemble, Lattice, Params

    ps = [Params.user_model("three_field", 3, initfield=(0.193, 0.0, 0.01), initderivs=(-0.142e-6, 0.0, 0.0),
                            N=N, vv=4, spectral=0, with_gw=1, seed=1 + i, precision=32)
          for i, N in enumerate((32, 32, 64))]
    ens = Ensemble(ps)
    assert ens.groups == 2
    ens.initialize()
    ens.evolve(0.005, 3)
    for idx, p in enumerate(ps):
        lat = _lattice(p)
        lat.initialize()
        lat.evolve(0.005, 3)
        a, b = ens.get_state(idx), lat.get_state()
        for k in ("f_k", "pi_k", "u_k", "pi_u_k"):
            assert np.array_equal(a[k], b[k]), (idx, k)
        assert a["a"] == b["a"], idx
        lat.close()
    ens.close()
