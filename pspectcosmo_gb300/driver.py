"""The reference's run loop over the C ABI: adaptive time step and output cadence.

The reference's main() (pspectcosmo.cpp:600-697) advances the lattice with

    dt = calculate_dt(kIR * N * sqrt(3) / 2, a)       # pspectcosmo.cpp:213-233: 0.2 a / k
    dt = min(dt, tOutputFreq)
    if t + dt passes the next frequent or infrequent output time: dt = the time left to it
    evolve(dt)
    at an output time (|t - next| < 1e-10): save_Freq() / save_Infreq() / save_Snap()

after initialize() and an initial save() (output.cpp:1796-1829). `run` is that loop on a
`Lattice` with `TextWriter` producing the reference's output files; each step is one
`psc_step` call, whose opening half kick reuses the force the previous call kept.
"""
from __future__ import annotations

import math

from .lattice import Lattice
from .outputs import TextWriter
from .params import Params


def calculate_dt(k: float, a: float) -> float:
    """calculate_dt (pspectcosmo.cpp:213-233): 2 / (k / a) / 10."""
    factor = 10
    return 2.0 / (k / a) / factor


def run(p: Params, tf: float, tOutputFreq: float, tOutputInfreq: float, tSnapFreq: float = 0.05,
        ssnapshot: bool = False, dir_: str = "output", writer: TextWriter | None = None,
        lattice: Lattice | None = None, t_analytic: float | None = None) -> Lattice:
    """initialize(), save(), then the main loop to tf (pspectcosmo.cpp:600-697). Returns the
    lattice at the final time; the reference's text files (and snapshots) are in dir_.

    With t_analytic (ANALYTIC_EVOLUTION, pspectcosmo.cpp:370-447) the run starts with the
    analytic phase to t_analytic (the same adaptive dt on a_k and output cadence, its own
    output functions), then initialize_lattice() and the lattice loop from there."""
    lat = lattice if lattice is not None else Lattice(p)
    w = writer if writer is not None else TextWriter(p, dir_)
    kmax = p.kIR * p.N * math.sqrt(3) / 2.0
    next_freq, next_infreq = tOutputFreq, tOutputInfreq
    numsteps = 0
    if t_analytic is not None:
        lat.analytic_begin()
        t0 = 0.0
        w.info_begin(0.0)
        w.save_analytic(lat)   # initialize_analytic_perturbation ends with save_analytic()
        t = 0.0
        while t < t_analytic:
            dt = calculate_dt(kmax, lat.analytic_background()["a"])
            dt = min(dt, tOutputFreq)
            if t + dt > next_freq or t + dt > next_infreq:
                dt = min(next_freq - t, next_infreq - t)
            lat.analytic_step(dt)
            t = lat.analytic_background()["t"]
            if abs(t - next_freq) < 1e-10:
                next_freq += tOutputFreq
                w.save_freq_analytic(lat)
            if abs(t - next_infreq) < 1e-10:
                next_infreq += tOutputInfreq
                w.save_infreq_analytic(lat)
        lat.analytic_to_lattice()
        t = lat.t
        next_snap = t_analytic + tSnapFreq
    else:
        lat.initialize()
        t0 = lat.t
        w.info_begin(0.0)   # initialize() ends with output_parameters() (initialize.cpp:803); dt is not set yet
        w.save(lat, numsteps, ssnapshot)
        t = lat.t
        next_snap = t + tSnapFreq
    while t < tf:
        dt = calculate_dt(kmax, lat.background()["a"])
        dt = min(dt, tOutputFreq)
        if t + dt > next_freq or t + dt > next_infreq:
            dt = min(next_freq - t, next_infreq - t)
        lat.evolve(dt, 1)
        t = lat.t
        if abs(t - next_freq) < 1e-10:
            next_freq += tOutputFreq
            w.save_freq(lat)
        if abs(t - next_infreq) < 1e-10:
            next_infreq += tOutputInfreq
            w.save_infreq(lat)
        if abs(t - next_snap) < 1e-10:
            next_snap += tSnapFreq
            numsteps += 1
            if ssnapshot:
                w.snapshot(lat, numsteps)
    w.info_end(t0, t)   # output_parameters() after the loop (pspectcosmo.cpp:699)
    return lat
