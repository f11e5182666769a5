"""Reference output rows and text files computed from the device reductions.

The column formulas follow the reference's writers:
  spectra_scalar_<f>.txt   output.cpp:671-690   (p, P_f, P_pi, n_k, numpoints)
  spectra_gws.txt          output.cpp:1041-1052 (p, P_h, dP_rhoGW, reference line, numpoints)
  energy_gws.txt           output.cpp:1055-1060 (t, rho_GW / rho, rho_GW)
  average_energies.txt     output.cpp:1163-1168 (t, K_0, G_0, [K_1, G_1], V_terms..., total)
  average_energy_conservation.txt  output.cpp:1171-1185
  average_scale_factor.txt output.cpp:467-486
  average_scalar_<f>.txt   output.cpp:430-461
Numbers are written with the reference's 6 significant digits (std::scientific,
setprecision(6)) so existing post-processing scripts read the files unchanged.
"""
from __future__ import annotations

import math
import os

import numpy as np

from .params import MODEL_PHI2, MODEL_PHI2CHI2, Params


def mass_sq_av(p: Params, means: np.ndarray) -> np.ndarray:
    """<effective_mass(f(x))> over the lattice (output.cpp:571-580) for the built-in models:
    their effective masses are linear in the squared fields, so <f^2> suffices. A user model
    (model.h compiled in) takes it from Lattice.mass_sq_av(), evaluated at every site."""
    if p.model == MODEL_PHI2:
        return np.array([1.0])
    phi2, chi2 = means[0, 2], means[1, 2]
    return np.array([1.0 + p.gsq * chi2, p.gsq * phi2])


def spectra_rows(p: Params, bg: dict, raw: dict, total: float, means: np.ndarray | None = None,
                 mass_sq: np.ndarray | None = None) -> dict:
    """The rows of spectra_scalar_<fld> and spectra_gws (output.cpp:690-705, 1040-1062); the
    occupation numbers use mass_sq (the lattice mean of effective_mass) when given, else the
    built-in models' mean from `means`."""
    a, ad, al = bg["a"], bg["ad"], p.alpha
    n3 = float(p.sites)
    nb = p.maxnumbins
    a_of_pi = a ** (al - 3)
    out = {}
    if mass_sq is not None:
        m2 = np.asarray(mass_sq)
    elif p.model in (MODEL_PHI2, MODEL_PHI2CHI2):
        m2 = mass_sq_av(p, means) if means is not None else (np.array([1.0]) if p.model == MODEL_PHI2 else None)
    else:
        m2 = None
    for f in range(p.nflds):
        rows = []
        for i in range(1, nb):
            pk = p.kIR * i
            npt = int(raw["numpoints"][f, i])
            f2, pi2, n2 = raw["f2"][f, i], raw["pi2"][f, i], raw["n2"][f, i]
            nd = 0.0
            if m2 is not None:
                om2 = abs(pk * pk + a * a * m2[f])
                if om2 > 0:
                    om = math.sqrt(om2)
                    nd = (a * a * p.L ** 3 / 2.0 / n3 ** 2 * (p.f_star / p.omegaStar) ** 2
                          * (om * f2 + a ** (2 * (1 - al)) / om * n2))
            rows.append((pk, i / n3 ** 2 * npt * f2, i / n3 ** 2 * npt * a_of_pi ** 2 * pi2, nd, npt))
        out[f"spectra_scalar_{f}"] = np.array(rows)
    if p.with_gw:
        rows = []
        for i in range(1, nb):
            npt = int(raw["gw_numpoints"][i])
            rows.append((p.kIR * i, i / n3 ** 2 * npt * raw["h2"][i],
                         i / n3 ** 2 / 4.0 / a ** 6 * (p.f_star / p.MPl) ** 2 / total * npt * raw["hdot2"][i],
                         (p.MPl * p.omegaStar) ** 2 / p.f_star ** 4 * 2 / math.pi ** 2 * ad ** 2 / a ** (2 * al + 2),
                         npt))
        out["spectra_gws"] = np.array(rows)
    return out


def energy_rows(p: Params, bg: dict, en: dict) -> dict:
    vals = []
    for f in range(p.nflds):
        vals += [en["K"][f], en["G"][f]]
    vals += list(en["V"])
    vals.append(en["total"])
    return dict(average_energies=np.array([bg["t"]] + vals),
                average_energy_conservation=np.array([bg["t"], en["friedmann_violation"]]),
                energy_gws=np.array([bg["t"], en["rho_gw"] / en["total"] if en["total"] else 0.0, en["rho_gw"]]))


def scale_row(p: Params, bg: dict) -> list:
    a, ad, add, al = bg["a"], bg["ad"], bg["add"], p.alpha
    return [bg["t"], a, ad, ad / a, add, 1 / (a ** (-al) * ad), 1 + al - a * add / ad ** 2]


class TextWriter:
    """Appends the reference's text outputs (output.cpp) in directory `dir_`."""

    def __init__(self, p: Params, dir_: str = "output", ext: str = ".txt", shistograms: bool = True,
                 nbins: int = 256, histogram_min: float = 0.0, histogram_max: float = 0.0,
                 snapshots_energy: bool = True, shistograms2d: bool = False, nbins2d: tuple = (10, 10),
                 histogram2d_min: float = 0.0, histogram2d_max: float = 0.0, hist2dflds: tuple = (0, 1),
                 sslices: bool = False, slicedim: int = 1, slicelength: int | None = None, sliceskip: int = 1,
                 sliceaverage: int = 1):
        self.p, self.dir, self.ext = p, dir_, ext
        os.makedirs(os.path.join(dir_, "Snapshots"), exist_ok=True)
        self._first_spectra = True
        # parameters.h:90-93 (histograms) and :14 (SNAPSHOTS_ENERGY)
        self.shistograms, self.nbins = shistograms, nbins
        self.histogram_min, self.histogram_max = histogram_min, histogram_max
        self.snapshots_energy = snapshots_energy
        # parameters.h:95-105 (2-D histograms, slices)
        self.shistograms2d, self.nbins2d = shistograms2d, tuple(nbins2d)
        self.histogram2d_min, self.histogram2d_max = histogram2d_min, histogram2d_max
        self.hist2dflds = tuple(hist2dflds)
        self.sslices, self.slicedim, self.sliceskip, self.sliceaverage = sslices, slicedim, sliceskip, sliceaverage
        self.slicelength = p.N if slicelength is None else slicelength

    def _open(self, name):
        return open(os.path.join(self.dir, name + self.ext), "a")

    @staticmethod
    def _e(x):
        return f"{x:15.6e}"

    @staticmethod
    def _g(x) -> str:
        """A double as an ostream prints it by default (6 significant digits, %g)."""
        return f"{x:g}"

    @staticmethod
    def readable_time(t: int) -> str:
        """readable_time (output.cpp:1708-1744)."""
        if t == 0:
            return "less than 1 second\n"
        parts = []
        for unit, name in ((86400, "days"), (3600, "hours"), (60, "minutes")):
            if t > unit:
                parts.append(f"{t // unit} {name}")
                t %= unit
        if t > 0:
            parts.append(f"{t} seconds")
        return ", ".join(parts) + "\n"

    def info_begin(self, dt: float = 0.0):
        """output_parameters() at the start of a run (output.cpp:1750-1786): info.txt with the
        model and program information and the start time."""
        import time

        p, g = self.p, self._g
        omega = p.m_in_MPl * p.f_star
        lines = ["--------------------------\n", "Model Specific Information\n", "--------------------------\n"]
        if p.model == 1:
            lines += ["two-field phi^2 + g^2 phi^2 chi^2 Model\n", "V = 1/2 m^2 PHI^2 + 1/2 g^2 PHI^2 CHI^2\n\n",
                      f"m_in_MPl = {g(p.m_in_MPl)}\n", f"g^2 (program units) = {g(p.gsq)}\n"]
        else:
            lines += ["single phi^2 Model\n", "V = 1/2 * m_in_MPl^2 * PHI^2 \n\n", f"m_in_MPl = {g(p.m_in_MPl)}\n"]
        lines += [f"fStar = {g(p.f_star)}\n", f"omegaStar = {g(omega)}\n"]
        lines += ["\n--------------------------\n", "General Program Information\n", "-----------------------------\n",
                  f"Grid size={p.N}^3\n", f"Number of fields={p.nflds}\n", f"L={g(p.L)}\n", f"kIR={g(p.kIR)}\n",
                  f"dt={g(dt)}, dt/dx={g(dt / (p.L / p.N))}\n",
                  {0: "No expansion\n", 1: "Fixed background expansion\n",
                   2: "Expansion calculated self-consistently\n"}.get(p.expansion, "")]
        self._t_start = time.time()
        lines.append("\nRun began at " + time.ctime(self._t_start) + "\n")
        with open(os.path.join(self.dir, "info" + self.ext), "w") as fh:
            fh.write("".join(lines))

    def info_end(self, t0: float, t: float):
        """output_parameters() at the end of a run: end time and elapsed wall time."""
        import time

        now = time.time()
        took = int(now - getattr(self, "_t_start", now))
        with open(os.path.join(self.dir, "info" + self.ext), "a") as fh:
            fh.write("Run ended at " + time.ctime(now) + "\n")
            fh.write(f"\nRun from t={self._g(t0)} to t={self._g(t)} took " + self.readable_time(took) + "\n")

    # analytic pre-lattice phase (output.cpp:117-375): the same files from the background
    # and the mode functions
    def save_freq_analytic(self, lat):
        """save_Freq_analytic(): meansvars_analytic, scale_analytic, energy_analytic."""
        p = self.p
        bg = lat.analytic_background()
        t, a = bg["t"], bg["a"]
        aop = a ** (p.alpha - 3)
        for f in range(p.nflds):
            vals = [bg["f"][f], bg["pi"][f] * aop, bg["f"][f] ** 2, (bg["pi"][f] * aop) ** 2]
            with self._open(f"average_scalar_{f}") as fh:
                fh.write(f"{t:.3f}" + "".join(self._e(v) for v in vals) + f"{0:15d}{0:15d}\n")
        if p.expansion == 2:
            r = scale_row(p, bg)
            with self._open("average_scale_factor") as fh:
                fh.write(f"{r[0]:.6f} {r[1]:.6f} {r[2]:.6f} {r[3]:.6f} {r[4]:.6f} {r[5]:15.6e} {r[6]:.6f}\n")
        total, cols = 0.0, []
        for f in range(p.nflds):
            k = bg["pi"][f] ** 2 / a ** 6 / 2.0
            total += k
            cols += [k, 0.0]
        fv = list(bg["f"]) + [0.0] * (2 - p.nflds)
        for term in range(p.num_potential_terms):
            v = 0.5 * fv[0] ** 2 if term == 0 else 0.5 * p.gsq * fv[0] ** 2 * fv[1] ** 2
            total += v
            cols.append(v)
        with self._open("average_energies") as fh:
            fh.write(f"{t:.3f}" + "".join(f" {v:.6e}" for v in cols) + f" {total:.6e}\n")
        if p.expansion != 1:
            lhs = bg["ad"] ** 2
            rhs = (p.f_star / p.MPl) ** 2 * a ** (2 * (p.alpha + 1)) * total / 3.0
            with self._open("average_energy_conservation") as fh:
                fh.write(f"{t:.3f} {abs(lhs - rhs) / abs(lhs + rhs):.8e} {lhs:.6f} {rhs:.6f}\n")

    def save_infreq_analytic(self, lat):
        """save_Infreq_analytic() -> spectra_analytic_discrete() (output.cpp:164-258): per
        l = 1 .. maxnumbins-1 the mode of k^2 = l^2: k, k^3/(2 pi^2) |f_k|^2,
        a^(2(alpha-3)) k^3/(2 pi^2) |pi_k|^2 (left-moving solution), 0, 0."""
        import math

        p = self.p
        bg = lat.analytic_background()
        k2, modes = lat.analytic_modes()
        aop = bg["a"] ** (p.alpha - 3)
        pos = {int(v): i for i, v in enumerate(k2)}
        for f in range(p.nflds):
            with self._open(f"spectra_scalar_{f}") as fh:
                for l in range(1, p.maxnumbins):
                    q = pos[l * l]
                    km = math.sqrt(k2[q]) * p.kIR
                    s1 = km ** 3 / (2 * math.pi ** 2) * abs(modes[0, f, q]) ** 2
                    s2 = aop ** 2 * km ** 3 / (2 * math.pi ** 2) * abs(modes[1, f, q]) ** 2
                    fh.write(f"{km:.1f} {s1:15.6e} {s2:15.6e} 0 0\n")
                fh.write("\n")
        with self._open("average_spectra_times") as fh:
            fh.write(f"{bg['t']:.2f}\n")

    def save_analytic(self, lat):
        """save_analytic() (output.cpp:1855-1873): the frequent and infrequent outputs."""
        self.save_freq_analytic(lat)
        self.save_infreq_analytic(lat)

    def save(self, lat, numsteps: int = 0, ssnapshot: bool = False):
        """save() (output.cpp:1796-1829): meansvars, scale, energy, histograms, the 2-D
        histograms and slices when on, the snapshot when ssnapshot, spectra."""
        self.save_freq(lat)
        if self.shistograms:
            self.histograms(lat)
        if self.shistograms2d:
            self.histograms_2d(lat)
        if self.sslices:
            self.slices(lat)
        if ssnapshot:
            self.snapshot(lat, numsteps)
        self.spectra(lat)

    def save_freq(self, lat):
        """save_Freq(): meansvars, scale, energy (output.cpp:1831-1840)."""
        p = self.p
        bg = lat.background()
        means = lat.means()
        for f in range(p.nflds):
            with self._open(f"average_scalar_{f}") as fh:
                m = means[f]
                fh.write(f"{bg['t']:.3f}" + "".join(self._e(v) for v in m) + "\n")
        if p.expansion == 2:
            r = scale_row(p, bg)
            with self._open("average_scale_factor") as fh:
                fh.write(f"{r[0]:.6f} {r[1]:.6f} {r[2]:.6f} {r[3]:.6f} {r[4]:.6f} {r[5]:15.6e} {r[6]:.6f}\n")
        en = lat.energies()
        er = energy_rows(p, bg, en)
        with self._open("average_energies") as fh:
            fh.write(f"{bg['t']:.3f}" + "".join(f" {v:.6e}" for v in er["average_energies"][1:]) + "\n")
        if p.expansion != 1:
            lhs = bg["ad"] ** 2
            rhs = (p.f_star / p.MPl) ** 2 * bg["a"] ** (2 * (p.alpha + 1)) * en["total"] / 3.0
            with self._open("average_energy_conservation") as fh:
                fh.write(f"{bg['t']:.3f} {en['friedmann_violation']:.8e} {lhs:.6f} {rhs:.6f}\n")

    def histograms(self, lat):
        """histograms() (output.cpp:1193-1297): histogram<f>.txt, one frequency per line and
        a blank line per call; histogramtimes.txt: t, then bmin and df of each field."""
        p = self.p
        h = lat.histograms(self.nbins, self.histogram_min, self.histogram_max)
        for f in range(p.nflds):
            with self._open(f"histogram{f}") as fh:
                fh.write("".join(f"{v:.6e}\n" for v in h["binfreq"][f]) + "\n")
        with self._open("histogramtimes") as fh:
            t = lat.background()["t"]
            fh.write(f"{t:.6f}" + "".join(f" {h['bmin'][f]:.6e} {h['df'][f]:.6e}" for f in range(p.nflds)) + "\n")

    def histograms_2d(self, lat):
        """histograms_2d() (output.cpp:1300-1413): histogram2d<f1>_<f2>.txt per field pair,
        the nbins0 x nbins1 frequencies one per line and a blank line per call;
        histogram2dtimes.txt: t, then bmin and df of both fields of each pair."""
        t = lat.background()["t"]
        times = f"{t:.6f}"
        for q in range(len(self.hist2dflds) // 2):
            f1, f2 = self.hist2dflds[2 * q], self.hist2dflds[2 * q + 1]
            h = lat.histograms_2d(f1, f2, self.nbins2d[0], self.nbins2d[1], self.histogram2d_min, self.histogram2d_max)
            with self._open(f"histogram2d{f1}_{f2}") as fh:
                fh.write("".join(f"{v:.6e}\n" for v in h["binfreq"].ravel()) + "\n")
            times += f" {h['bmin'][0]:.6e} {h['df'][0]:.6e} {h['bmin'][1]:.6e} {h['df'][1]:.6e}"
        with self._open("histogram2dtimes") as fh:
            fh.write(times + "\n")

    def slices(self, lat):
        """slices() (output.cpp:1415-1539): slices<f>.txt, one value per line and a blank line
        per call; slicetimes.txt: t."""
        v = lat.slices(self.slicedim, self.slicelength, self.sliceskip, self.sliceaverage)
        for f in range(self.p.nflds):
            with self._open(f"slices{f}") as fh:
                fh.write("".join(f"{x:.6e}\n" for x in v[f]) + "\n")
        with self._open("slicetimes") as fh:
            fh.write(f"{lat.background()['t']:.6f}\n")

    def snapshot(self, lat, step: int) -> str:
        """save_Snap(step) -> snapshots() (output.cpp:1541-1648): <dir>/Snapshots/
        data_<step>_snapshot.h5 with the fields and, with SNAPSHOTS_ENERGY, the lattice
        energy densities. Returns the path."""
        path = os.path.join(self.dir, "Snapshots", f"data_{int(step)}_snapshot.h5")
        lat.write_snapshot(path, self.snapshots_energy)
        return path

    def save_infreq(self, lat):
        """save_Infreq() (output.cpp:1842-1848): histograms() when shistograms, then
        spectra() (output.cpp:490-1062)."""
        if self.shistograms:
            self.histograms(lat)
        self.spectra(lat)

    def spectra(self, lat):
        """spectra() (output.cpp:490-1062): spectra_scalar_<f>.txt, average_spectra_times.txt
        and with GWs spectra_gws.txt, energy_gws.txt."""
        p = self.p
        bg = lat.background()
        en = lat.energies()
        user = p.model not in (MODEL_PHI2, MODEL_PHI2CHI2)
        rows = spectra_rows(p, bg, lat.spectra_raw(), en["total"], lat.means(), lat.mass_sq_av() if user else None)
        for f in range(p.nflds):
            with self._open(f"spectra_scalar_{f}") as fh:
                for r in rows[f"spectra_scalar_{f}"]:
                    fh.write(f"{r[0]:.1f} {r[1]:15.6e} {r[2]:15.6e} {r[3]:15.6e} {int(r[4])}\n")
                fh.write("\n")
        with self._open("average_spectra_times") as fh:
            fh.write(f"{bg['t']:.2f}\n")
        if p.with_gw:
            with self._open("spectra_gws") as fh:
                for r in rows["spectra_gws"]:
                    fh.write(f"{r[0]:.1f} {r[1]:15.6e} {r[2]:15.6e} {r[3]:15.6e} {int(r[4])}\n")
                fh.write("\n")
            with self._open("energy_gws") as fh:
                rho = en["rho_gw"]
                fh.write(f"{bg['t']:.2f} {rho / en['total']:.6e} {rho:.6e}\n")
