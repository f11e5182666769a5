"""Benchmark: site-steps/s of the pseudo-spectral lattice step on GB300.

Workload (the configuration the headline metric is quoted on): 256^3 two-field
preheating, V = m^2 phi^2/2 + g^2 phi^2 chi^2/2 with g^2 = 2.5e5, gravitational waves on
(six u_ij, evolve_VV semantics), Yoshida-4, dt = 0.005, FP32 fields with FP64
background and reductions. Synthetic data: the reference's own seeded initial
conditions (seed 1), generated on the host. Every array is larger than the 129 MB L2
(2 GB resident), so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config preheat_gw_256|preheat_gw_1024|preheat_256|inflation_64|ensemble_mixed|
                            adjoint_128]
                  [--precision 32|64]

One JSON line (rank 0). `value` is device-timed whole-job site-steps/s (inputs resident
in HBM); `e2e` is the same metric through the C ABI with host buffers in pinned memory,
the state copied host->device before the steps and device->host after them, and the
background read back after every step (`pageable_host_value`: the same from ordinary
numpy arrays). `--impl reference` times the CPU restatement of the reference's
FP64 path (oracle/port) on this machine's host cores.
Multi-GPU: independent replicas, one lattice per rank (the path does not shard); the
timed region is bracketed by barriers and the max over ranks is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: (Params factory kwargs, dt, description)
    "preheat_gw_256": (dict(kind="preheating", N=256, spectral=0, with_gw=1, vv=4), 0.005,
                       "256^3 two-field preheating + GW, Yoshida-4"),
    # the 1024^3 configuration (~90 GB resident): the stated dt = 0.01 breaks the Yoshida-4
    # stability bound (omega_max dt ~ 8.9 with omega_max = kIR N sqrt(3)/2 ~ 887), so it runs
    # at the reference's own adaptive rule dt = 0.2 a / (kIR N sqrt(3)/2) at a = 1
    "preheat_gw_1024": (dict(kind="preheating", N=1024, spectral=0, with_gw=1, vv=4), 0.2 / (1024 * 3 ** 0.5 / 2),
                        "1024^3 two-field preheating + GW, Yoshida-4"),
    "preheat_256": (dict(kind="preheating", N=256, spectral=1, with_gw=0, vv=4), 0.005,
                    "256^3 two-field preheating (spectral path, no GW), Yoshida-4"),
    "inflation_64": (dict(kind="default", N=64, vv=2), 0.002, "64^3 single-field inflation, velocity Verlet"),
    # 256 x 32^3 + 64 x 64^3 + 8 x 128^3 single-field realizations, per-realization seed and
    # phi0 ~ U[10, 12] (host RNG seed 12345), Yoshida-4, one graph per step for all of them
    "ensemble_mixed": (dict(kind="ensemble"), 1e-4,
                       "ensemble: 256 x 32^3 + 64 x 64^3 + 8 x 128^3 single-field inflation, Yoshida-4"),
    # one timed step = the gradients of <chi^2> and of rho_GW after ADJ_STEPS model steps of the
    # two-field + GW lattice (checkpoints every ADJ_EVERY steps, each segment recomputed once),
    # FP32 fields / FP64 background
    "adjoint_128": (dict(kind="preheating", N=128, spectral=0, with_gw=1, vv=2), 0.005,
                    "adjoint of <chi^2> and rho_GW after 2000 steps: 128^3 two-field preheating + GW, "
                    "velocity Verlet, checkpoints every 100 steps"),
    # the 1024^3 configuration's own check: FP32 1024^3 + GW from the 256^3 initial state
    # prolonged spectrally (psc_set_state_padded), against the FP64 256^3 run on the same modes
    # (bins |k| < 128 kIR, inside the 256^3 lattice), GW energy spectrum every 100 steps
    "gw_modes_1024": (dict(kind="preheating", N=1024, spectral=0, with_gw=1, vv=4), 0.2 / (1024 * 3 ** 0.5 / 2),
                      "1024^3 two-field preheating + GW (FP32) vs FP64 256^3 on the same modes, Yoshida-4"),
}
ADJ_STEPS, ADJ_EVERY = 2000, 100
MODES_EVERY, MODES_OUTPUTS = 100, 2


def ensemble_params(precision: int):
    import numpy as np
    from pspectcosmo_gb300.params import Params

    rng = np.random.default_rng(12345)
    ps = []
    for N, count in ((32, 256), (64, 64), (128, 8)):
        for _ in range(count):
            ps.append(Params.reference_default(N=N, vv=4, seed=1 + len(ps), precision=precision,
                                               initfield=[float(rng.uniform(10.0, 12.0)), 0.0]))
    return ps

# algorithmic HBM bytes per site-step of the fused dataflow: per stage and field 9C + 2R,
# GW 36C + 12R (C = P (1 + 2/N) per site for a half-spectrum complex array, R = P)
def algorithmic_bytes_per_site_step(p) -> float:
    P = 4 if p.precision == 32 else 8
    C = P * (1 + 2 / p.N)
    R = P
    per_stage = p.nflds * (9 * C + 2 * R) + (36 * C + 12 * R if p.with_gw else 0)
    return p.stages * per_stage


def make_params(name: str, precision: int):
    from pspectcosmo_gb300.params import Params

    kw, dt, desc = CONFIGS[name]
    kw = dict(kw)
    kind = kw.pop("kind")
    p = Params.preheating(**kw) if kind == "preheating" else Params.reference_default(**kw)
    p.precision = precision
    return p, dt, desc


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region: start() returns
    once the sampler is producing (so the region is covered from its first step), and only the
    samples taken after that count (the last earlier one when the region is shorter than the
    sampling interval)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, interval_ms: int = 10):
        self.idx = gpu_index
        self.interval_ms = interval_ms
        self.proc = None
        self.lines = []
        self.mark = 0
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.005)
        self.mark = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[self.mark:] or self.lines[-1:]:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "interval_ms": self.interval_ms}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return world, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, value: float) -> float:
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], device="cuda" if torch.cuda.is_available() else "cpu", dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(p, dt, budget_s: float = 20.0, threads: int | None = None) -> dict:
    """The CPU restatement of the reference's FP64 path (oracle/port) on this host:
    as many Yoshida stages of the same lattice as fit in ~budget_s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
    import oracle

    oracle.build()
    q = p.copy()
    q.precision = 64
    threads = threads or os.cpu_count()
    o = oracle.Oracle(q, threads=threads)
    o.init_ic()
    s = o.stages
    o.step_stages(dt, 1)  # warm-up (page faults, twiddles)
    done, t0 = 0, time.perf_counter()
    while True:
        o.step_stages(dt, 1)
        done += 1
        el = time.perf_counter() - t0
        if el > budget_s or done >= 3 * s:
            break
    per_step = el / done * s
    return {"value": p.sites / per_step, "unit": "site-steps/s", "cores": threads, "kind": "port",
            "stages_timed": done,
            "sample": f"{done} Yoshida stage(s) of the {p.N}^3 lattice ({s} per step) in {el:.1f} s, FP64 "
                      f"restatement (oracle/port) with {threads} threads"}


REF_BENCH_CONFIG = "bench_gw2_n256_vv4"   # oracle/build_ref.py: the headline workload on the reference's code


def reference_sample(p, dt, nsteps: int = 1) -> dict | None:
    """The reference's OWN evolve_VV (its sources, prepared in oracle/_ref by
    oracle/build_ref.py and compiled here against the FFTW API shim) timed for `nsteps` steps
    of the headline workload on this host's cores: initial conditions, then the steps on the
    wall clock. None when the prepared sources are absent or the build fails."""
    if (p.N, p.nflds, p.with_gw, p.spectral, p.vv) != (256, 2, 1, 0, 4):
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    try:
        import build_ref

        if not build_ref.prepared(REF_BENCH_CONFIG) and not build_ref.reference_available():
            return None
        exe = os.path.join(build_ref.OUT, REF_BENCH_CONFIG, "harness")
        if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(
                os.path.join(build_ref.OUT, REF_BENCH_CONFIG, "parameters.h")):
            exe = build_ref.build(REF_BENCH_CONFIG)
        import tempfile

        with tempfile.TemporaryDirectory() as tmp:
            env = dict(os.environ, PSC_HARNESS_STACK_GB="16")
            # initialize() waits for a key press (initialize.cpp:681): give it one
            r = subprocess.run([exe, "time", str(nsteps), repr(dt)], cwd=tmp, env=env, input="\n",
                               capture_output=True, text=True, timeout=900)
        line = [ln for ln in r.stdout.splitlines() if ln.startswith("steps ")]
        if r.returncode != 0 or not line:
            print(f"reference harness failed (rc {r.returncode}): {r.stderr[-500:]}", file=sys.stderr)
            return None
        f = line[-1].split()
        sps, threads = float(f[5]), int(f[7])
    except (Exception, SystemExit) as e:
        print(f"reference harness unavailable: {e!r}"[:800], file=sys.stderr)
        return None
    return {"value": p.sites / sps, "unit": "site-steps/s", "cores": threads, "kind": "reference",
            "steps_timed": nsteps,
            "sample": f"{nsteps} step(s) ({p.stages} Yoshida stages each) of the {p.N}^3 lattice in {sps * nsteps:.1f} s: "
                      f"the reference's own evolve_VV (evolution.cpp:607-694) and initialize(), compiled with "
                      f"g++ -O2 against the FFTW API shim (FFTW is not installed); FFTs on {threads} threads, "
                      f"the rest single-threaded as in the reference"}


def run_reference(args):
    world, rank, local, dist = dist_setup()
    if rank != 0:
        return
    p, dt, desc = make_params(args.config, args.precision)
    cs = reference_sample(p, dt, 1)
    if cs is None:   # no prepared reference sources for this workload: the C restatement
        budget = max(5.0, min(120.0, 8.0 * args.steps))
        cs = cpu_sample(p, dt, budget_s=budget)
    timed_steps = cs.get("steps_timed", cs.get("stages_timed", 0) / max(1, p.stages))
    line = {"impl": "reference", "metric": "site-steps/s", "value": cs["value"], "unit": "site-steps/s",
            "n_gpus": args.gpus, "steps": timed_steps, "steps_requested": args.steps, "warmup": 0,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (reference seeded ICs)",
            "config": {"workload": desc, "N": p.N, "nflds": p.nflds, "gw": bool(p.with_gw), "vv": p.vv,
                       "dt": dt, "parallelism": "cpu threads"},
            "cpu_baseline": cs,
            "e2e": {"value": cs["value"], "unit": "site-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ensemble(args):
    world, rank, local, dist = dist_setup()
    from pspectcosmo_gb300 import Ensemble, build

    build.build()
    _, dt, desc = CONFIGS[args.config]
    ps = ensemble_params(args.precision)
    sites = sum(p.sites for p in ps)
    ens = Ensemble(ps)
    ens.initialize()
    if not args.no_autotune:
        ens.autotune(reps=2)
    one_launch = ens.launch_mode(per_group=False if args.one_launch else None)
    ens.evolve(dt, args.warmup)
    clocks = ClockSampler(local)
    barrier(dist)
    clocks.start()
    barrier(dist)
    ens.evolve(dt, args.steps)
    barrier(dist)
    ms = max_over_ranks(dist, ens.last_step_ms())
    clk = clocks.stop()
    value = world * sites * args.steps / (ms / 1e3)
    if rank == 0:
        line = {"metric": "site-steps/s", "value": value, "unit": "site-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == 32 else "f64",
                "data": "synthetic (reference seeded initial conditions per realization)",
                "config": {"workload": desc, "realizations": len(ps), "groups": ens.groups, "sites": sites,
                           "dt": dt, "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                           "fft_shapes": "default" if args.no_autotune else "autotuned per group",
                           "launches": "one per pass for all groups" if one_launch else "one per pass per group"},
                "clocks": clk,
                "gpu_launches": (1 if one_launch else ens.groups) * 6 * ps[0].stages * args.steps}
        print(json.dumps(line), flush=True)
    ens.close()
    if dist is not None:
        dist.destroy_process_group()


def run_modes_check(args):
    """GW energy spectrum of the 1024^3 FP32 lattice against an FP64 256^3 run on the same modes:
    the 256^3 initial state (the reference's initialize() + initialize_GW()) is the 1024^3 state
    by spectral prolongation (zero modes above the 256^3 band), both evolve with the 1024^3
    step's dt, and the spectra_gws columns of the bins |k| < 128 kIR (every mode of the bin lies
    in both lattices) are compared every MODES_EVERY steps, with rho_GW and a(t)."""
    world, rank, local, dist = dist_setup()
    import numpy as np
    from pspectcosmo_gb300 import Lattice, build
    from pspectcosmo_gb300.outputs import spectra_rows

    build.build()
    p, dt, desc = make_params(args.config, 32)
    q = p.copy()
    q.N, q.precision = 256, 64
    small = Lattice(q)
    small.initialize()
    st = small.get_state()
    big = Lattice(p)
    big.set_state_padded(256, st["f_k"], st["pi_k"], st["a"], st["ad"], st["add"], st["u_k"], st["pi_u_k"])
    del st
    if not args.no_autotune:
        big.autotune(reps=2)

    def rows(lat, pp):
        en = lat.energies()
        return spectra_rows(pp, lat.background(), lat.spectra_raw(), en["total"]), en

    points, big_ms = [], 0.0
    clocks = ClockSampler(local)
    clocks.start()
    for k in range(1, MODES_OUTPUTS + 1):
        big.evolve(dt, MODES_EVERY)
        big_ms += big.last_step_ms()
        small.evolve(dt, MODES_EVERY)
        (rb, eb), (rs, es) = rows(big, p), rows(small, q)
        # bin i (|k| in [i, i+1) kIR) is row i - 1 of both lattices' spectra; bins below 128 kIR
        def inside(x):
            return x[x[:, 0] < 128 * q.kIR]

        gb, gs = inside(rb["spectra_gws"]), inside(rs["spectra_gws"])
        pt = {"step": k * MODES_EVERY, "t": big.background()["t"]}
        for c, name in ((1, "h2"), (2, "hdot2")):
            d = np.abs(gb[:, c] - gs[:, c]).max() / np.abs(gs[:, c]).max()
            pt[f"gw_{name}_rel_err"] = float(d)
        for f in range(p.nflds):
            a_, b_ = inside(rb[f"spectra_scalar_{f}"]), inside(rs[f"spectra_scalar_{f}"])
            pt[f"P_f{f}_rel_err"] = float(np.abs(a_[:, 1] - b_[:, 1]).max() / np.abs(b_[:, 1]).max())
        pt["rho_gw_rel_err"] = abs(eb["rho_gw"] - es["rho_gw"]) / abs(es["rho_gw"])
        pt["a_rel_err"] = abs(big.background()["a"] - small.background()["a"]) / small.background()["a"]
        points.append(pt)
    clk = clocks.stop()
    steps = MODES_EVERY * MODES_OUTPUTS
    if rank == 0:
        line = {"metric": "site-steps/s", "value": p.sites * steps / (big_ms / 1e3), "unit": "site-steps/s",
                "n_gpus": 1, "steps": steps, "warmup": 0, "ms_per_step": big_ms / steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (reference seeded 256^3 initial conditions, prolonged)",
                "config": {"workload": desc, "N": p.N, "nflds": p.nflds, "gw": True, "vv": p.vv, "dt": dt,
                           "compared_bins": "|k| < 128 kIR", "output_every": MODES_EVERY},
                "gw_spectrum_vs_fp64_256": points, "clocks": clk}
        print(json.dumps(line), flush=True)
    big.close()
    small.close()


def adjoint_check(lat, p, dt, st0, ndir):
    """Accuracy of the FP32 adjoint at this configuration: directional derivatives of <chi^2> and
    rho_GW along ndir random directions of (f_k, pi_k, u_k, pi_u_k, gsq) at t = 0, from the FP32
    and FP64 adjoint gradients, against FP64 central differences of the product's forward map
    (h = 1e-6 relative: each array's perturbation has mean modulus 1e-6 of the array's, gsq
    moves by 1e-6 gsq times a standard normal)."""
    import numpy as np
    from pspectcosmo_gb300 import Lattice

    q = p.copy()
    q.precision = 64
    keys = ("f_k", "pi_k", "u_k", "pi_u_k")
    cur = [None]

    def set64(st, gsq=None):
        # an FP64 lattice holding st (a new one per coupling value: gsq is a run parameter)
        if cur[0] is not None:
            cur[0].close()
        qq = q.copy()
        if gsq is not None:
            qq.gsq = gsq
        cur[0] = Lattice(qq)
        cur[0].set_state(*(st[k] for k in ("f_k", "pi_k", "a", "ad", "add", "u_k", "pi_u_k")))
        return cur[0]

    def reset32():
        lat.set_state(*(st0[k] for k in ("f_k", "pi_k", "a", "ad", "add", "u_k", "pi_u_k")))

    grads = {}
    for name in ("chi2", "rho_gw"):
        reset32()
        g32 = lat.adjoint(name, dt, ADJ_STEPS, ADJ_EVERY)
        g64 = set64(st0).adjoint(name, dt, ADJ_STEPS, ADJ_EVERY)
        grads[name] = (g32, g64)
    # rho_GW of the forward map's final state: the energies after a forward run equal the
    # adjoint's rho_GW observable (checked on the unperturbed state)
    l64 = set64(st0)
    o_chi = l64.adjoint_forward("chi2", dt, ADJ_STEPS)
    o_rho_e = l64.energies()["rho_gw"]
    o_rho = set64(st0).adjoint_forward("rho_gw", dt, ADJ_STEPS)
    rng = np.random.default_rng(2026)
    N = p.N
    dirs = []
    for d in range(ndir):
        v = {}
        for k in keys:
            base = st0[k]
            x = np.fft.rfftn(rng.standard_normal((base.shape[0], N, N, N)), axes=(-3, -2, -1)).reshape(base.shape)
            v[k] = x * (1e-6 * np.abs(base).mean() / np.abs(x).mean())
        dg = 1e-6 * p.gsq * float(rng.standard_normal())
        fd = {}
        for sign in (1, -1):
            st = dict(st0)
            for k in keys:
                st[k] = st0[k] + sign * v[k]
            l64 = set64(st, gsq=p.gsq + sign * dg)
            oc = l64.adjoint_forward("chi2", dt, ADJ_STEPS)
            orho = l64.energies()["rho_gw"]
            fd.setdefault("chi2", []).append(oc)
            fd.setdefault("rho_gw", []).append(orho)
        row = {"direction": d}
        for name in ("chi2", "rho_gw"):
            fdv = (fd[name][0] - fd[name][1]) / 2
            for tag, g in zip(("fp32", "fp64"), grads[name]):
                pred = sum(float(np.sum(np.real(np.conj(g["grad_" + k]) * v[k]))) for k in keys
                           if g.get("grad_" + k) is not None) + float(g["grad_theta"][0]) * dg
                row[f"{name}_{tag}_rel_err"] = abs(pred - fdv) / abs(fdv)
            row[f"{name}_fd"] = fdv
        dirs.append(row)
    cur[0].close()
    worst = {k: max(r[k] for r in dirs) for k in dirs[0] if k.endswith("rel_err")}
    return {"directions": ndir, "h": "1e-6 relative", "O_chi2": o_chi, "O_rho_gw": o_rho,
            "rho_gw_energies_vs_observable": abs(o_rho_e - o_rho) / abs(o_rho), "worst": worst,
            "per_direction": dirs, "stated_tolerance": 1e-3}


def run_adjoint(args):
    world, rank, local, dist = dist_setup()
    from pspectcosmo_gb300 import Lattice, build

    build.build()
    p, dt, desc = make_params(args.config, args.precision)
    lat = Lattice(p)
    lat.initialize()
    st0 = lat.get_state()

    def reset():
        lat.set_state(st0["f_k"], st0["pi_k"], st0["a"], st0["ad"], st0["add"], st0["u_k"], st0["pi_u_k"])

    # forward alone on the product's captured step, the same ADJ_STEPS steps
    reset()
    lat.evolve(dt, ADJ_STEPS)
    reset()
    lat.evolve(dt, ADJ_STEPS)
    fwd_ms = lat.last_step_ms()
    for _ in range(args.warmup):
        reset()
        lat.adjoint("rho_gw", dt, ADJ_STEPS, ADJ_EVERY, fields=False)
    clocks = ClockSampler(local)
    barrier(dist)
    clocks.start()
    barrier(dist)
    # one step: both gradients (<chi^2> and rho_GW) from the same initial state
    dev_ms, ms_obs = 0.0, {"chi2": 0.0, "rho_gw": 0.0}
    obs = {}
    for _ in range(args.steps):
        for name in ("chi2", "rho_gw"):
            reset()
            g = lat.adjoint(name, dt, ADJ_STEPS, ADJ_EVERY, fields=False)
            dev_ms += lat.last_step_ms()
            ms_obs[name] += lat.last_step_ms()
            obs[name] = g
    barrier(dist)
    ms = max_over_ranks(dist, dev_ms)
    clk = clocks.stop()
    value = world * p.sites * ADJ_STEPS * args.steps / (ms / 1e3)
    # end to end: host state in, every gradient array out
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for name in ("chi2", "rho_gw"):
            reset()
            lat.adjoint(name, dt, ADJ_STEPS, ADJ_EVERY)
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    state_bytes = (2 * p.nflds + 12) * p.modes * 16
    check = adjoint_check(lat, p, dt, st0, args.adj_check) if (args.adj_check > 0 and rank == 0) else None
    if rank == 0:
        line = {"metric": "site-steps/s", "value": value, "unit": "site-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32" if p.precision == 32 else "f64",
                "data": "synthetic (reference seeded initial conditions, seed 1)",
                "config": {"workload": desc, "N": p.N, "nflds": p.nflds, "vv": p.vv, "dt": dt,
                           "model_steps_per_gradient": ADJ_STEPS, "checkpoint_every": ADJ_EVERY,
                           "precision": f"fp{p.precision} fields, fp64 background/reductions/adjoint scalars",
                           "parallelism": f"replicas x{world}" if world > 1 else "single lattice",
                           "l2": "arrays > 129 MB L2 (no flush needed)"},
                "adjoint_over_forward": {k: (v / args.steps) / fwd_ms for k, v in ms_obs.items()},
                "forward_ms": fwd_ms,
                "adjoint_ms": {k: v / args.steps for k, v in ms_obs.items()},
                "observables": {k: {"O": v["O"], "grad_theta": list(map(float, v["grad_theta"])),
                                    "grad_ad0": v["grad_ad0"]} for k, v in obs.items()},
                "e2e": {"value": world * p.sites * ADJ_STEPS * args.steps / e2e_s, "unit": "site-steps/s",
                        "h2d_bytes_per_step": 2 * (state_bytes + 24),
                        "d2h_bytes_per_step": 2 * (state_bytes + 32)},
                "roofline": None,
                "cpu_baseline": None,
                "clocks": clk,
                "gradient_check": check,
                "gpu_launches": int(ADJ_STEPS * p.stages * (2 * (2 * 6 + 11) + 13) + 32)}
        print(json.dumps(line), flush=True)
    lat.close()
    if dist is not None:
        dist.destroy_process_group()


def pinned_state(st):
    """Copies of the host state's arrays in pinned (page-locked) host memory, and pinned
    output arrays of the same shapes for get_state(out=...); (None, None) without CUDA."""
    import numpy as np
    import torch

    if not torch.cuda.is_available():
        return None, None
    keys = [k for k in ("f_k", "pi_k", "u_k", "pi_u_k") if st[k] is not None]
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    src = dict(st)
    out = {}
    for k in keys:
        src[k] = pin(st[k])
        out[k] = pin(np.empty_like(st[k]))
    return src, out


def fft_yardstick(lat, p, reps: int = 10):
    """The library's 3-D c2r (X, Y inverse passes and the Z c2r pass) of the field arrays
    beside cuFFT's (torch.fft.irfftn, complex64 -> float32) on the same half spectra: device
    ms per field, the achieved GB/s against the compulsory bytes of a c2r (read the half
    spectrum, write the real array) and the max-norm relative difference of the outputs."""
    import ctypes

    import numpy as np
    import torch

    if p.precision != 32 or not torch.cuda.is_available():
        return None
    N, H = p.N, p.N // 2 + 1
    ours_ms = lat.time_c2r(reps) / p.nflds
    f0 = np.zeros((p.nflds, N, N, N))
    rc = lat._L.psc_get_fields_real(lat._h, f0.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    if rc != 0:
        return None
    # the last field: with two fields chi has zero mean, so the comparison sees its
    # fluctuations (phi's sit below FP32 resolution next to phi0 ~ 0.19)
    last = p.nflds - 1
    fk = lat.get_state()["f_k"][last].reshape(N, N, H).astype(np.complex64)
    x = torch.from_numpy(fk).cuda()
    for _ in range(3):
        y = torch.fft.irfftn(x, s=(N, N, N))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    for _ in range(reps):
        y = torch.fft.irfftn(x, s=(N, N, N))
    ev1.record()
    torch.cuda.synchronize()
    cufft_ms = ev0.elapsed_time(ev1) / reps
    yc = y.cpu().numpy().astype(np.float64)
    diff = float(np.abs(f0[last] - yc).max() / max(np.abs(yc).max(), 1e-300))
    nbytes = 8 * N * N * H + 4 * N ** 3
    del x, y
    torch.cuda.empty_cache()
    return {"transform": f"3-D c2r {N}^3 fp32 (one field)", "ours_ms": ours_ms, "cufft_ms": cufft_ms,
            "ours_over_cufft_time": ours_ms / cufft_ms, "compulsory_bytes": nbytes,
            "ours_gbs": nbytes / (ours_ms / 1e3) / 1e9, "cufft_gbs": nbytes / (cufft_ms / 1e3) / 1e9,
            "max_rel_diff": diff, "compared_field": last, "library": "cuFFT via torch.fft (yardstick only, not on the product path)"}


def run_ours(args):
    if args.config == "ensemble_mixed":
        return run_ensemble(args)
    if args.config == "adjoint_128":
        return run_adjoint(args)
    if args.config == "gw_modes_1024":
        return run_modes_check(args)
    world, rank, local, dist = dist_setup()
    from pspectcosmo_gb300 import Lattice, build
    from pspectcosmo_gb300.params import Params  # noqa: F401

    build.build()
    p, dt, desc = make_params(args.config, args.precision)
    lat = Lattice(p)
    lat.tensor_maps = args.tensor_maps
    lat.initialize()
    # FFT tile / grid shapes: the planner's defaults, then the autotuner's choice (timed on
    # this state, before the warm-up)
    shapes = {"default": list(lat.shapes)}
    if not args.no_autotune:
        tune = lat.autotune(reps=3)
        shapes.update(chosen=list(tune["shape"]), from_cache=tune["from_cache"])
    # host copy of the initial state (the e2e input); at 1024^3 the FP64 host state would be
    # ~140 GB, so that size has no e2e leg and restarts from the device generator instead
    big = p.N >= 1024
    st0 = None if big else lat.get_state()
    # warm-up (graph build, first launches)
    lat.evolve(dt, args.warmup)
    if big:
        lat.initialize()
    else:
        lat.set_state(st0["f_k"], st0["pi_k"], st0["a"], st0["ad"], st0["add"], st0["u_k"], st0["pi_u_k"])

    clocks = ClockSampler(local)
    barrier(dist)
    clocks.start()
    barrier(dist)
    lat.evolve(dt, args.steps)     # device-timed with CUDA events on the lattice's stream
    barrier(dist)
    ms = max_over_ranks(dist, lat.last_step_ms())
    clk = clocks.stop()
    value = world * p.sites * args.steps / (ms / 1e3)

    # end to end through the C ABI with host buffers
    import numpy as np  # noqa: F401

    e2e = None
    if not big:
        # the host state in pinned memory (input and output buffers, allocated once), and
        # for comparison in ordinary pageable numpy arrays with fresh output arrays per call;
        # each the median of three repetitions (the host side varies by +-20 % run to run)
        def e2e_run(src, out=None):
            reps = []
            for _ in range(3):
                barrier(dist)
                t0 = time.perf_counter()
                lat.set_state(src["f_k"], src["pi_k"], src["a"], src["ad"], src["add"], src["u_k"], src["pi_u_k"])
                for _ in range(args.steps):
                    lat.evolve(dt, 1)
                    lat.background()
                res = lat.get_state(out=out)
                reps.append(max_over_ranks(dist, time.perf_counter() - t0))
                del res
            return sorted(reps)[1], reps

        pinned, pinned_out = pinned_state(st0)
        e2e_s, reps = e2e_run(pinned if pinned is not None else st0, pinned_out)
        e2e_pg, reps_pg = e2e_run(st0)
        state_arrays = 2 * p.nflds + (12 if p.with_gw else 0)
        state_bytes_host = state_arrays * p.modes * 16   # host buffers are FP64 complex
        e2e = {"value": world * p.sites * args.steps / e2e_s, "unit": "site-steps/s",
               "h2d_bytes_per_step": state_bytes_host / args.steps + 8,
               "d2h_bytes_per_step": state_bytes_host / args.steps + 3 * 8 + 4 + 8,
               "host_buffers": "pinned" if pinned is not None else "pageable (pinning unavailable)",
               "timing": "median of 3 repetitions", "repetitions_s": reps,
               "pageable_host_value": world * p.sites * args.steps / e2e_pg, "pageable_repetitions_s": reps_pg}

    # per-pass device times and roofline of the dominant pass
    passes = lat.time_passes(reps=10)
    pbytes = lat.pass_bytes()
    peak, peak_kind = measured_peaks()
    dom = max((k for k in passes if k != "background"), key=lambda k: passes[k])
    achieved = pbytes[dom] / (passes[dom] / 1e3) / 1e9
    step_alg = algorithmic_bytes_per_site_step(p) * p.sites
    step_achieved = step_alg / (ms / 1e3 / args.steps) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as fh:
                traffic = json.load(fh).get(f"{args.config}:{dom}")
        except Exception:
            traffic = None

    launches_per_stage = 6
    gpu_launches = 1 + 7 + p.stages * launches_per_stage * args.steps

    # the same K steps in FP64 (the plain method): its rate and the FP32 spectrum error
    # against it (spectra() bins, max-norm relative over bins; GW h^2, hdot^2 when on)
    fp_cmp = None
    if p.precision == 32 and rank == 0 and not args.no_fp64 and not big:
        q = p.copy()
        q.precision = 64
        lat64 = Lattice(q)
        lat64.initialize()
        lat64.evolve(dt, args.steps)
        ms64 = lat64.last_step_ms()
        s32, s64 = lat.spectra_raw(), lat64.spectra_raw()
        lat64.close()

        def relmax(a, b):
            d = float(np.abs(b).max())
            return float(np.abs(a - b).max() / d) if d > 0 else 0.0

        err = {k: relmax(s32[k], s64[k]) for k in ("f2", "pi2", "n2") + (("h2", "hdot2") if p.with_gw else ())}
        fp_cmp = {"fp64_value": p.sites * args.steps / (ms64 / 1e3), "fp64_ms_per_step": ms64 / args.steps,
                  "fp32_over_fp64": (ms64 / args.steps) / (ms / args.steps),
                  "spectrum_rel_err": err, "stated_tolerance": {"f2": 1e-4, "pi2": 1e-4, "n2": 1e-4, "h2": 1e-4,
                                                                  "hdot2": 1e-4},
                  "after_steps": args.steps}

    # a long FP32 and FP64 trajectory side by side (--fp64-steps S): the spectrum, a and rho_GW
    # errors of the FP32 path against the FP64 one and both Friedmann violations along the way
    traj = None
    if p.precision == 32 and rank == 0 and args.fp64_steps > 0 and not big:
        q = p.copy()
        q.precision = 64
        lat32, lat64 = Lattice(p), Lattice(q)
        lat32.initialize()
        lat64.initialize()
        points, done = [], 0
        chunk = max(1, args.fp64_steps // 8)
        while done < args.fp64_steps:
            n = min(chunk, args.fp64_steps - done)
            lat32.evolve(dt, n)
            lat64.evolve(dt, n)
            done += n
            s32, s64 = lat32.spectra_raw(), lat64.spectra_raw()
            e32, e64 = lat32.energies(), lat64.energies()
            b32, b64 = lat32.background(), lat64.background()

            def relmax(a, b):
                d = float(np.abs(b).max())
                return float(np.abs(a - b).max() / d) if d > 0 else 0.0

            pt = {"step": done, "t": b64["t"], "a": b64["a"], "a_rel_err": abs(b32["a"] - b64["a"]) / abs(b64["a"]),
                  "friedmann_violation_fp32": e32["friedmann_violation"],
                  "friedmann_violation_fp64": e64["friedmann_violation"]}
            pt.update({f"{k}_rel_err": relmax(s32[k], s64[k])
                       for k in ("f2", "pi2", "n2") + (("h2", "hdot2") if p.with_gw else ())})
            if p.with_gw:
                pt["rho_gw_rel_err"] = abs(e32["rho_gw"] - e64["rho_gw"]) / abs(e64["rho_gw"])
            points.append(pt)
        lat32.close()
        lat64.close()
        keys = [k for k in points[0] if k.endswith("_rel_err")] + ["friedmann_violation_fp32"]
        traj = {"steps": args.fp64_steps, "dt": dt, "points": points,
                "worst": {k: max(pt[k] for pt in points) for k in keys},
                "stated_tolerance": {"spectra_and_rho_gw_rel_err": 1e-4, "friedmann_violation_fp32": 1e-5}}

    if rank == 0:
        yard = None if big else fft_yardstick(lat, p)
        cpu = cpu_sample(p, dt, budget_s=20.0) if (world == 1 and not args.no_cpu and not big) else None
        cpu_ref = reference_sample(p, dt, 1) if (world == 1 and not args.no_cpu and not big) else None
        line = {
            "metric": "site-steps/s", "value": value, "unit": "site-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if p.precision == 32 else "f64",
            "data": "synthetic (reference seeded initial conditions, seed 1)",
            "config": {"workload": desc, "N": p.N, "nflds": p.nflds, "gw": bool(p.with_gw), "vv": p.vv, "dt": dt,
                       "precision": f"fp{p.precision} fields, fp64 background/reductions",
                       "parallelism": f"replicas x{world}" if world > 1 else "single lattice",
                       "l2": "arrays > 129 MB L2 (no flush needed)",
                       "fft_shapes": shapes,
                       "tensor_map_staging": {"x_passes": bool(lat.tensor_maps & 1), "y_forward": bool(lat.tensor_maps & 2),
                                              "y_inverse": bool(lat.tensor_maps & 4)}},
            "e2e": e2e,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "bytes_per_launch": pbytes[dom], "ms_per_launch": passes[dom],
                         "step": {"algorithmic_bytes_per_site_step": algorithmic_bytes_per_site_step(p),
                                  "achieved": step_achieved, "frac": step_achieved / peak}},
            "passes_ms": passes,
            "fp32_vs_fp64": fp_cmp,
            "fft_yardstick": yard,
            "fp32_vs_fp64_trajectory": traj,
            "cpu_baseline": cpu,
            "cpu_baseline_reference": cpu_ref,
            "clocks": clk,
            "gpu_launches": gpu_launches,
        }
        print(json.dumps(line), flush=True)
    lat.close()
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="preheat_gw_256", choices=sorted(CONFIGS))
    ap.add_argument("--precision", type=int, default=32, choices=[32, 64])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-autotune", action="store_true", help="keep the planner's default FFT tile shapes")
    ap.add_argument("--tensor-maps", type=int, default=3, choices=range(8),
                    help="pass groups that stage their tiles by tensor maps: 1 X passes, 2 Y passes (default both), "
                         "4 the pipelined GW Y inverse pass below N = 1024")
    ap.add_argument("--one-launch", action="store_true",
                    help="ensemble_mixed: one launch per pass for all size groups (default: per-group launches)")
    ap.add_argument("--adj-check", type=int, default=0,
                    help="adjoint_128: also check the FP32 and FP64 gradients against FP64 central differences "
                         "on this many random directions")
    ap.add_argument("--fp64-steps", type=int, default=None,
                    help="also run FP32 and FP64 lattices this many steps side by side and report the errors "
                         "(default: 1000 for preheat_gw_256, 0 otherwise)")
    args = ap.parse_args()
    if args.fp64_steps is None:
        args.fp64_steps = 1000 if args.config == "preheat_gw_256" else 0
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
