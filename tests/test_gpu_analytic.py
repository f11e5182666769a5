"""The analytic pre-lattice phase (ANALYTIC_EVOLUTION) against the reference's own code
(golden anal1_n16: shipped phi^2 model, velocity Verlet; anal2_n16_vv4: two-field
preheating, Yoshida-4), FP64:

* initialize_analytic_perturbation: the background and every mode function at t = 0 to
  1e-14 of their largest value;
* evolve_VV_analytic_perturbation: background and modes after 5 and 10 steps to 1e-12
  (the modes advance on the device with the reference's operation order, each product and
  sum rounded on its own);
* initialize_lattice: the lattice state (4 random draws per mode in the reference's order)
  to 1e-12, a, a', a'' and t exactly as the phase left them;
* 4 lattice steps from there to 1e-10, as every FP64 lattice run."""
import numpy as np
import pytest

from golden_util import load, params_for, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("run", ["anal1_n16", "anal2_n16_vv4"])
def test_analytic_phase_matches_reference(run):
    from pspectcosmo_gb300 import Lattice

    g, meta = load(run)
    p = params_for(meta, 64)
    lat = Lattice(p)
    lat.analytic_begin()
    k2, modes = lat.analytic_modes()
    assert np.array_equal(k2, g["k2"])
    bg = lat.analytic_background()
    ref = g["ana_0_bg"]
    assert [bg["t"], bg["a"], bg["ad"]] == list(ref[:3]) and rel(bg["add"], ref[3]) < 1e-14
    assert rel(modes, g["ana_0_modes"]) < 1e-14
    for s in range(1, meta["na_steps"] + 1):
        lat.analytic_step(meta["dta"])
        if s % meta["everya"] == 0:
            bg = lat.analytic_background()
            ref = g[f"ana_{s}_bg"]
            for i, k in enumerate(("t", "a", "ad", "add")):
                assert rel(bg[k], ref[i]) < 1e-12, (s, k)
            _, modes = lat.analytic_modes()
            want = g[f"ana_{s}_modes"]
            for w in range(4):
                assert rel(modes[w], want[w]) < 1e-12, (s, w)
    lat.analytic_to_lattice()
    st = lat.get_state()
    ref = g["lat_ic_bg"]
    assert lat.t == pytest.approx(ref[0], rel=1e-14)
    assert rel(st["a"], ref[1]) < 1e-12 and rel(st["ad"], ref[2]) < 1e-12 and rel(st["add"], ref[3]) < 1e-12
    assert rel(st["f_k"], g["lat_ic_f_k"]) < 1e-12
    assert rel(st["pi_k"], g["lat_ic_pi_k"]) < 1e-12
    lat.evolve(meta["dt"], meta["nsteps"])
    st = lat.get_state()
    assert rel(st["f_k"], g["lat_fin_f_k"]) < 1e-10
    assert rel(st["pi_k"], g["lat_fin_pi_k"]) < 1e-10
    ref = g["lat_fin_bg"]
    assert rel(st["a"], ref[1]) < 1e-12 and rel(st["ad"], ref[2]) < 1e-11


def test_analytic_driver_runs(tmp_path):
    """driver.run with t_analytic: the analytic phase, its output files, the lattice after it."""
    from pspectcosmo_gb300 import Params
    from pspectcosmo_gb300.driver import run

    p = Params.reference_default(N=16)
    d = str(tmp_path / "out")
    lat = run(p, tf=0.01, tOutputFreq=0.001, tOutputInfreq=0.005, dir_=d, t_analytic=0.004)
    assert lat.t == pytest.approx(0.01, abs=1e-9)
    rows = [ln for ln in open(f"{d}/average_scalar_0.txt") if ln.strip()]
    assert len(rows) == 11   # t = 0 .. 0.01 every 0.001: 5 analytic rows, 6 lattice rows
    assert rows[0].split()[-1] == "0" and rows[-1].split()[-1] != "0"
    spec = open(f"{d}/spectra_scalar_0.txt").read().strip().split("\n\n")
    assert len(spec) == 3    # t = 0 (analytic save), 0.005, 0.01


def test_analytic_errors():
    from pspectcosmo_gb300 import Lattice, Params
    from pspectcosmo_gb300.lattice import PscError

    lat = Lattice(Params.reference_default(N=16))
    with pytest.raises(PscError):
        lat.analytic_step(1e-3)   # before analytic_begin
    with pytest.raises(PscError):
        lat.analytic_to_lattice()
