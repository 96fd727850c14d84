#!/usr/bin/env python
"""Throughput of the kagome VMC hot path on GB300: accepted moves per second.

Workload (the headline configuration): 6x6 doubled kagome cells (N=216,
n_up = n_down = 108), pi-flux parton orbitals, the reference's acceptance
rule, 2048 independent walkers from seeded random starts.  One step = every
walker makes `--moves` accepted exchange moves (kvmc_advance; local energy
every 108 proposals), with W refreshed in FP64 every R accepted moves (mixed
form) or every 108 proposals (plain FP64 form).  The mixed form's settings
(where W lives, delayed-update depth k, R, threads per walker) are the
autotuner's choice for this workload on a GB300 (kagomevmc/tuned.json);
flags override them.  The walkers' FP32 W state (2048 x 186.6 KB = 382 MB,
and 191 MB for the non-trivial rows the one-warp sweep works on during a
call) is larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  The reference arm times the reference
algorithm's CPU restatement (complex double, one chain per host thread).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "kagomedsl.jl_gb300"))

CELLS = (6, 6)          # doubled cells -> DoubleKagome(1.0, 12, 6)
N_SITES = 216
METRIC = "accepted moves/sec at N=216, mixed-prec batched vs plain FP64, at |dE/N|<=1e-4"
UNIT = "accepted_moves/s"


def args_():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--walkers", type=int, default=2048)
    p.add_argument("--moves", type=int, default=1024, help="accepted moves per walker per step")
    p.add_argument("--refresh", type=int, default=None, help="mixed form: accepted moves between FP64 refreshes")
    p.add_argument("--delay-k", type=int, default=None)
    p.add_argument("--placement", default=None, choices=["auto", "chip", "hbm"])
    p.add_argument("--threads", type=int, default=None, help="threads per walker with W in HBM")
    p.add_argument("--warp", type=int, default=None, help="walkers per CTA with one warp per walker (0: one CTA each)")
    p.add_argument("--guard", default=None, help="accuracy guard hi,lo of the one-warp sweep (0,0: off)")
    p.add_argument("--refresh32", type=int, default=None,
                   help="the periodic refresh's form: 0 FP64, 1 one thread per row, 2 tiled, 3 tensor cores")
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--skip-plain", action="store_true")
    p.add_argument("--skip-cpu", action="store_true")
    p.add_argument("--skip-gate", action="store_true")
    p.add_argument("--gate-walkers", type=int, default=512, help="walkers of the energy gate")
    p.add_argument("--gate-calls", type=int, default=None,
                   help="advance calls of the energy gate (default: two refresh intervals, at least 8)")
    p.add_argument("--skip-e2e", action="store_true")
    p.add_argument("--no-peaks", action="store_true")
    p.add_argument("--skip-grad", action="store_true")
    p.add_argument("--skip-uneven", action="store_true")
    p.add_argument("--skip-large", action="store_true")
    p.add_argument("--large-walkers", type=int, default=512, help="walkers of the N=864 leg")
    p.add_argument("--skip-field", action="store_true")
    p.add_argument("--skip-batched", action="store_true")
    p.add_argument("--skip-plugin", action="store_true")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def model():
    import kagomevmc as kv

    lat = kv.DoubleKagome(1.0, 2 * CELLS[0], CELLS[1], (True, True), (False, True))
    return kv.Hamiltonian.build(N_SITES // 2, N_SITES // 2, lat)


# ---------------------------------------------------------------------------
# CPU restatement (oracle port): the cpu_baseline and the reference arm
# ---------------------------------------------------------------------------

def oracle_model():
    """The headline lattice built by the oracle alone (numpy restatement of
    Hmat, orbitals and get_nn): the CPU legs map no library of this repo."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import kagome_oracle as o

    lat = o.double_kagome(1.0, 2 * CELLS[0], CELLS[1], (True, True), (False, True))
    h = o.hamiltonian(N_SITES // 2, N_SITES // 2, lat)
    return h.U_up, h.U_down, [(i - 1, j - 1) for i, j in h.nn]


def cpu_port_run(model_, chains, proposals, seed, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import kagome_oracle as o
    import oracle_c

    U_up, U_down, bonds = model_
    m = oracle_c.OracleModel(U_up, U_down, bonds, "cplx")
    starts = [o.seeded_start(seed, w, U_up, U_down)[:2] for w in range(chains)]
    n = N_SITES // 2
    sec, ch = oracle_c.run_chains(m, starts, seed, proposals, n, n, 0, threads)
    acc = sum(c.c.accepted for c in ch)
    return acc, sec


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_arm(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    om = oracle_model()
    threads = cpu_threads()
    proposals = 5400  # fifty reference refresh intervals per chain per step (about a second of host time)
    vals = []
    for s in range(a.warmup + a.steps):
        acc, sec = cpu_port_run(om, threads, proposals, a.seed + 7919 * s, threads)
        if s >= a.warmup:
            vals.append((acc, sec))
    acc = sum(v[0] for v in vals)
    sec = sum(v[1] for v in vals)
    value = acc / sec
    sample = f"{threads} chains x {proposals} proposals per step, N=216, complex double, refresh and E_L every 108 proposals"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * sec / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded random starts)",
            "config": {"workload": "kagome VMC, 6x6 doubled cells (N=216), reference acceptance rule",
                       "walkers": threads, "proposals_per_walker_per_step": proposals},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def measure_peaks(device):
    """FP64 and FP32 (no TF32) GEMM throughput of this GPU, measured in-run
    with cuBLAS through torch (the denominators for FP64/FP32-pipe kernels)."""
    out = {}
    try:
        import torch

        torch.backends.cuda.matmul.allow_tf32 = False
        dev = torch.device("cuda", device)
        for name, dt, n in (("fp64_tflops", torch.float64, 4096), ("fp32_tflops", torch.float32, 8192)):
            a = torch.randn(n, n, device=dev, dtype=dt)
            b = torch.randn(n, n, device=dev, dtype=dt)
            best = math.inf
            for _ in range(4):
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize(dev)
                s.record()
                torch.matmul(a, b)
                e.record()
                torch.cuda.synchronize(dev)
                best = min(best, s.elapsed_time(e))
            out[name] = 2 * n ** 3 / (best * 1e-3) / 1e12
            del a, b
        torch.cuda.empty_cache()
    except Exception as exc:  # torch missing: peaks stay unknown
        out["error"] = str(exc)
    return out


def run_steps(eng, steps, moves):
    tot = {"accepted": 0, "proposals": 0, "launches": 0, "refreshes": 0, "measurements": 0, "sum_energy": 0.0,
           "max_drift": 0.0, "bad_walkers": 0}
    for _ in range(steps):
        st = eng.advance(moves)
        for k in ("accepted", "proposals", "launches", "refreshes", "measurements", "sum_energy", "bad_walkers"):
            tot[k] += st[k]
        tot["max_drift"] = max(tot["max_drift"], st["max_drift"])
    return tot


def mixed_choice(kv, ham, a):
    """The autotuner's cached choice for this workload, with flag overrides."""
    from kagomevmc import autotune

    ch = autotune.lookup(ham, a.walkers) or autotune.Choice(delay_k=0, refresh_interval=1024, placement="auto")
    if a.refresh is not None:
        ch.refresh_interval = a.refresh
    if a.delay_k is not None:
        ch.delay_k = a.delay_k
    if a.placement is not None:
        ch.placement = a.placement
    if a.threads is not None:
        ch.threads = a.threads
    if a.warp is not None:
        ch.warp = a.warp
    if a.guard is not None:
        ch.guard_hi, ch.guard_lo = (int(x) for x in a.guard.split(","))
    if a.refresh32 is not None:
        ch.refresh32 = a.refresh32
    ch.trials = []
    return ch


def energy_gate(ham, kv, walkers, calls, moves, choice, seed, therm=1):
    """Both forms on identical walkers and proposal streams, driven the way the
    bench drives the mixed form: `therm` kvmc_advance calls of `moves`
    accepted moves per walker to leave the random starts behind (their
    samples are discarded, as the bench's warm-up steps are), then `calls`
    calls whose local energies are compared.  The worst relative W drift
    seen at a refresh is reported for both phases."""
    import numpy as np

    from kagomevmc import autotune

    res = {}
    for prec in ("plain", "mixed"):
        if prec == "mixed":
            eng = autotune.make_engine(ham, walkers, choice, seed=seed)
        else:
            eng = kv.Engine(ham, walkers, precision="plain", seed=seed)
        eng.init()
        drift_therm = 0.0
        for _ in range(therm):
            drift_therm = max(drift_therm, eng.advance(moves)["max_drift"])
        eng.reset_stats()
        drift = 0.0
        for _ in range(calls):
            drift = max(drift, eng.advance(moves)["max_drift"])
        ws = eng.walker_stats()
        res[prec] = (ws["sum_e"], ws["n_meas"], eng.get_state()[0], (drift, drift_therm), ws["proposals"])
        eng.close()
    (ep, np_, kp, _, pp), (em, nm, km, (drift, drift_therm), pm) = res["plain"], res["mixed"]
    same = np.array([np.array_equal(kp[w], km[w]) for w in range(walkers)])
    dE_same = abs(ep[same].sum() / np_[same].sum() - em[same].sum() / nm[same].sum()) / N_SITES
    # all walkers: the difference of the two forms' per-walker means, with the
    # standard error of that difference across walkers (chains share starts
    # and streams, so the difference is paired).  The gate passes when the
    # paired mean difference plus two standard errors is within 1e-4.
    d = (em / nm - ep / np_) / N_SITES
    dE = float(abs(d.mean()))
    se = float(d.std(ddof=1) / np.sqrt(walkers))
    return {"dE_per_site": dE, "se_dE_per_site": se, "bound": dE + 2 * se, "walkers": walkers, "calls": calls,
            "accepted_moves_per_call": moves, "proposals_per_walker": float(np.mean(pm)),
            "identical_chains": int(same.sum()), "dE_per_site_identical_chains": float(dE_same),
            "worst_walker_dE_per_site": float(np.abs(d).max()),
            "thermalization_calls": therm, "max_w_drift_at_refresh": float(drift),
            "max_w_drift_at_refresh_thermalization": float(drift_therm), "pass": bool(dE + 2 * se <= 1e-4)}


def adjoint_run(kv, seed, device, walkers=1024, sweeps=20):
    """The differentiation workload: 4x4 doubled cells (N=96), the pi-flux
    ansatz extended by (t2, m, theta) drawn from `seed`, 1024 chains (complex
    FP32 W, reference acceptance rule), one adjoint evaluation of dE/da and the
    3x3 SR matrix per 48-proposal sweep.  Reports the adjoint kernel's time
    against the sweep (and refresh) kernels' time per sweep."""
    import numpy as np

    alpha = kv.ansatz.draw_alpha(seed)
    A = kv.Ansatz.build(kv.DoubleKagome(1.0, 8, 4, (True, True), (False, True)), 48, 48, *alpha)
    eng = kv.Engine(A.ham, walkers, precision="mixed", seed=seed, refresh_interval=64, device=device)
    eng.set_log_derivatives(A.dU_up, A.dU_down)
    eng.init()
    eng.sweep(960)
    eng.reset_stats()
    eng.enable_timing(True)
    eng.region_start()
    for _ in range(sweeps):
        eng.sweep(48)
        eng.measure_grad()
    wall = eng.region_stop()
    k0, _ = eng.kernel_time(0)
    k1, _ = eng.kernel_time(1)
    k2, n2 = eng.kernel_time(2)
    res = kv.estimate(eng.grad_sums(), 3)
    eng.close()
    return {"workload": "kagome VMC, 4x4 doubled cells (N=96), extended ansatz (t2, m, theta) drawn from seed "
                        f"{seed}, {walkers} chains, mixed complex FP32 W, 48 proposals + 1 adjoint per sweep",
            "alpha": list(alpha), "sweeps": sweeps,
            "sweep_ms_per_sweep": (k0 + k1) / sweeps, "adjoint_ms_per_sweep": k2 / sweeps,
            "adjoint_over_sweep": k2 / (k0 + k1) if k0 + k1 > 0 else None, "target_ratio": 2.0,
            "wall_ms": wall, "E_per_site": res["E"] / 96, "grad_per_site": (res["grad"] / 96).tolist(),
            "se_grad_per_site": (np.asarray(res["se_grad"]) / 96).tolist(), "S": res["S"].tolist()}


def plugin_run(kv, seed, device, walkers=2048, sweeps=200, warm=20):
    """The reference-shaped plugin surface end to end: MC / init_ / sweep_ /
    measure_ (the Carlo.jl callbacks, kagomevmc/montecarlo.py) at the headline
    workload, one fused sweep_ of min(N_up, N_down) = 108 proposals per walker
    per Carlo sweep (the reference's refresh and measurement interval), the
    autotuner's settings, host buffers: every call returns its statistics to
    the host, and measure_ pushes the batch mean of the call's E_L samples.
    Host wall clock around `sweeps` calls."""
    params = dict(n1=2 * CELLS[0], n2=CELLS[1], PBC=(True, True), antiPBC=(False, True), N_up=N_SITES // 2,
                  N_down=N_SITES // 2, walkers=walkers, precision="mixed", proposals_per_sweep=N_SITES // 2,
                  seed=seed, device=device, tuned=True)
    mc = kv.MC(params)
    ctx = kv.MCContext()
    kv.init_(mc, ctx, params)
    for _ in range(warm):
        kv.sweep_(mc, ctx)
        ctx.sweeps += 1
        kv.measure_(mc, ctx)
    acc = 0
    t0 = time.perf_counter()
    for _ in range(sweeps):
        kv.sweep_(mc, ctx)
        ctx.sweeps += 1
        kv.measure_(mc, ctx)
        acc += mc.last_stats["accepted"]
    sec = time.perf_counter() - t0
    ev = kv.Evaluator()
    kv.register_evaluables(kv.MC, ev, params)
    energy = ev.run({"OL": ctx.observables["OL"][warm:]})["energy"]
    cfg = mc.engine.config()
    mc.engine.close()
    # per call: the per-walker counters and sums read before and after (5 x 8 B
    # each), the status words and drift (4 B each), two refresh counters
    d2h = walkers * (2 * 5 * 8 + 4 + 4) + 16
    return {"value": acc / sec, "unit": UNIT, "sweeps": sweeps, "proposals_per_sweep": N_SITES // 2,
            "accepted_per_sweep": acc / sweeps, "ms_per_sweep": 1e3 * sec / sweeps, "h2d_bytes_per_step": 0,
            "d2h_bytes_per_step": d2h, "energy_per_site": float(energy), "delay_k": cfg["delay_k"],
            "path": "MC -> init_ -> (sweep_ -> measure_) x sweeps: kvmc_sweep(h, 108) per Carlo sweep, host wall clock"}


def uneven_run(kv, seed, device, moves=512, steps=3):
    """The uneven batch: 1024 chains at 3x3 doubled cells (N=54), 768 at 6x6
    (N=216) and 256 at 8x8 (N=384), each class with the autotuner's settings,
    advanced together by one captured CUDA graph per step (kvmc_group), and
    the same three classes advanced one after another for comparison."""
    from kagomevmc import autotune

    cells = {54: (3, 3), 216: (6, 6), 384: (8, 8)}
    classes = [(54, 1024), (216, 768), (384, 256)]
    res = {}
    for mode in ("graph", "sequential"):
        engines, choices = [], []
        for N, walkers in classes:
            a_, b_ = cells[N]
            ham = kv.Hamiltonian.build(N // 2, N // 2, kv.DoubleKagome(1.0, 2 * a_, b_, (True, True), (False, True)))
            ch = autotune.lookup(ham, walkers) or autotune.Choice(delay_k=0, refresh_interval=1024, placement="auto")
            eng = autotune.make_engine(ham, walkers, ch, seed=seed + N, device=device)
            eng.init()
            engines.append(eng)
            choices.append(dict(N=N, walkers=walkers, delay_k=eng.config()["delay_k"],
                                refresh_interval=ch.refresh_interval, placement=ch.placement, threads=ch.threads))
        acc, ms_tot = 0, 0.0
        if mode == "graph":
            g = kv.Group(engines)
            g.advance(moves)  # warm-up, captures the graph
            for _ in range(steps):
                st, ms = g.advance(moves)
                acc += sum(x["accepted"] for x in st)
                ms_tot += ms
            g.close()
        else:
            for e in engines:
                e.advance(moves)
            engines[0].region_start()
            for _ in range(steps):
                for e in engines:
                    acc += e.advance(moves)["accepted"]
            ms_tot = engines[0].region_stop()
        for e in engines:
            e.close()
        res[mode] = {"value": acc / (ms_tot * 1e-3), "ms": ms_tot, "accepted": acc}
    return {"workload": "1024 x N=54 + 768 x N=216 + 256 x N=384 walkers, reference rule, "
                        f"{moves} accepted moves per walker per step, {steps} steps", "unit": UNIT,
            "classes": choices, "graph": res["graph"], "sequential": res["sequential"],
            "graph_over_sequential": res["graph"]["value"] / res["sequential"]["value"]}


def batched_run(kv, seed, device, walkers=4096, moves=1024):
    """Batched walkers at 4x4 doubled cells (N=96): 4096 chains from seeded
    random starts, once with the settings the workload names (delayed depth
    16, FP64-quality refresh every 64 accepted moves) and once with the
    autotuner's choice for this batch."""
    import numpy as np

    from kagomevmc import autotune

    ham = kv.Hamiltonian.build(48, 48, kv.DoubleKagome(1.0, 8, 4, (True, True), (False, True)))
    named = autotune.Choice(delay_k=16, refresh_interval=64, placement="hbm", threads=128)
    tuned = autotune.lookup(ham, walkers) or named
    out = {}
    for label, ch in (("k16_R64", named), ("tuned", tuned)):
        eng = autotune.make_engine(ham, walkers, ch, seed=seed, device=device)
        eng.init()
        eng.advance(256)
        eng.region_start()
        st = eng.advance(moves)
        ms = eng.region_stop()
        out[label] = {"value": st["accepted"] / (ms * 1e-3), "unit": UNIT, "delay_k": eng.config()["delay_k"],
                      "refresh_interval": ch.refresh_interval, "placement": ch.placement, "threads": ch.threads}
        eng.close()
    # as the workload is written: 500 warm-up and 2000 measured sweeps (one
    # proposal each) per chain, E/N of the FMA and the 3xTF32 flush against
    # the plain FP64 form on the same starts and proposal streams
    energies, rates = {}, {}
    for label in ("plain", "fma", "3xtf32"):
        if label == "plain":
            eng = kv.Engine(ham, walkers, precision="plain", seed=seed, device=device)
        else:
            eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, device=device, delay_k=16,
                            refresh_interval=64, w_placement="hbm")
            eng.set_stream_threads(128)
            eng.set_tc_flush(label == "3xtf32")
        eng.init()
        eng.sweep(500)
        eng.reset_stats()
        eng.region_start()
        st = eng.sweep(2000)
        ms = eng.region_stop()
        ws = eng.walker_stats()
        energies[label] = ws["sum_e"] / ws["n_meas"] / 96
        rates[label] = st["accepted"] / (ms * 1e-3)
        eng.close()
    sweeps = {}
    for label, e in energies.items():
        row = {"E_per_site": float(e.mean()), "se": float(e.std(ddof=1) / np.sqrt(walkers)),
               "accepted_moves_per_s": rates[label]}
        if label != "plain":
            d = e - energies["plain"]
            row["dE_per_site_vs_plain"] = float(d.mean())
            row["se_dE"] = float(d.std(ddof=1) / np.sqrt(walkers))
            row["gate_pass"] = bool(abs(d.mean()) + 2 * row["se_dE"] <= 1e-4)
        sweeps[label] = row
    return {"workload": f"kagome VMC, 4x4 doubled cells (N=96), {walkers} walkers, {moves} accepted moves per walker",
            **out, "as_written_500_2000_sweeps": sweeps}


def field_run(kv, seed, device, walkers=2048, moves=256):
    """The field workload of scripts/LL.jl: 8x8 doubled cells (N=192), B =
    imbalance * pi / S with imbalance 4 (N_up = 98, N_down = 94), complex
    orbitals; the mixed complex form (delayed updates, W in HBM) against the
    plain complex FP64 form on the same walkers."""
    import math

    lat = kv.DoubleKagome(1.0, 8, 8, (True, True), (False, True))
    H = kv.Hmat(lat, B=4 * math.pi / (64 * 2 * math.sqrt(3)))
    Uu, Ud = kv.orbitals(H, 98, 94)
    ham = kv.Hamiltonian(98, 94, Uu, Ud, H, kv.get_nn(H))
    from kagomevmc import autotune

    # the mixed form with the autotuner's settings for this workload, over two
    # of its refresh intervals
    ch = autotune.lookup(ham, walkers) or autotune.Choice(delay_k=8, refresh_interval=512, placement="hbm")
    out = {}
    for prec, R, mv in (("mixed", ch.refresh_interval, max(4 * moves, 2 * ch.refresh_interval)),
                        ("plain", 0, moves // 4)):
        if prec == "mixed":
            eng = autotune.make_engine(ham, walkers, ch, seed=seed, device=device)
        else:
            eng = kv.Engine(ham, walkers, precision=prec, seed=seed, refresh_interval=R, device=device)
        eng.init()
        eng.advance(32)
        eng.region_start()
        st = eng.advance(mv)
        ms = eng.region_stop()
        out[prec] = {"value": st["accepted"] / (ms * 1e-3), "unit": UNIT, "moves_per_walker": mv,
                     "delay_k": eng.config()["delay_k"], "refresh_interval": eng.config()["refresh_interval"],
                     "walker_refreshes": st["refreshes"]}
        eng.close()
    return {"workload": f"kagome VMC in a field, 8x8 doubled cells (N=192), imbalance 4, {walkers} walkers, "
                        "complex orbitals", **out, "mixed_over_plain": out["mixed"]["value"] / out["plain"]["value"]}


def large_run(kv, seed, device, walkers=512, moves=128, steps=2):
    """The large lattice: 12x12 doubled cells (N=864, 432 orbitals per spin),
    512 walkers, W (2 x 864 x 432 FP32 = 2.99 MB per walker, 1.53 GB in all)
    in HBM with rank-16 delayed updates, a refresh every 128 accepted moves
    by the FP32 refinement with its residual on the tensor cores (FP64 for
    the walkers it hands back); the same with the tiled FP32 refinement on
    the CUDA cores and with the FP64 refresh; and the plain FP64 form on the
    same walkers."""
    from kagomevmc import autotune

    ham = kv.Hamiltonian.build(432, 432, kv.DoubleKagome(1.0, 24, 12, (True, True), (False, True)))
    ch = autotune.Choice(delay_k=16, refresh_interval=128, placement="hbm", threads=256)

    def run(refresh32):
        eng = autotune.make_engine(ham, walkers, ch, seed=seed, device=device)
        eng.set_drift_tolerance(1e-2)
        eng.set_refresh32(refresh32)
        eng.init()
        eng.advance(moves)
        eng.enable_timing(True)
        eng.region_start()
        acc = redos = 0
        for _ in range(steps):
            st = eng.advance(moves)
            acc += st["accepted"]
            redos += st["fp64_redos"]
        ms = eng.region_stop()
        k0, _ = eng.kernel_time(0)
        k1, _ = eng.kernel_time(1)
        eng.close()
        return acc, ms, k0, k1, redos

    acc, ms, k0, k1, redos = run(3)
    acc2, ms2, _, k1_2, redos2 = run(2)
    acc64, ms64, _, k1_64, _ = run(0)
    w_bytes = 2 * 864 * 432 * 4
    flush_bytes = 2 * w_bytes / 16 * acc          # W read + written once per 16 accepted moves
    pe = kv.Engine(ham, walkers, precision="plain", seed=seed, device=device)
    pe.init()
    pe.advance(8)
    pe.region_start()
    pst = pe.advance(128)   # spans several of its refreshes (every 432 proposals)
    pms = pe.region_stop()
    pacc = pst["accepted"]
    pe.close()
    return {"workload": f"kagome VMC, 12x12 doubled cells (N=864), {walkers} walkers, W in HBM, delayed k=16, "
                        f"FP32 refinement refresh every 128 accepted moves with its residual on the tensor cores "
                        f"(exact bf16 digit products), {steps} x {moves} accepted moves per walker",
            "value": acc / (ms * 1e-3), "unit": UNIT, "ms": ms, "sweep_ms": k0, "refresh_ms": k1,
            "refreshes_redone_fp64": redos,
            "sweep_only_moves_per_s": acc / (k0 * 1e-3) if k0 else None,
            "flush_hbm_gbs_in_sweep": flush_bytes / (k0 * 1e-3) / 1e9 if k0 else None,
            "tiled_fp32_refresh": {"value": acc2 / (ms2 * 1e-3), "unit": UNIT, "refresh_ms": k1_2,
                                   "refreshes_redone_fp64": redos2},
            "fp64_refresh": {"value": acc64 / (ms64 * 1e-3), "unit": UNIT, "refresh_ms": k1_64},
            "plain_fp64": {"value": pacc / (pms * 1e-3), "unit": UNIT, "moves_per_walker": 128,
                           "walker_refreshes": pst["refreshes"]},
            "note": "refresh-bound. One walker refresh (both spins): FP64 LU and solves 2*((2/3)n^3 + 2(N-n)n^2) "
                    "= 0.43 GFLOP; the FP32 forms run the LU, G = M^-1 and V = B G, then per refinement pass the "
                    "residual B - V M (tensor cores: 22 bf16 MMAs per k-step of 16 into seven exact weight classes; "
                    "tiled: 6 FP32 operations per product) and V += R G"}


def gpu_arm(a):
    import numpy as np

    import kagomevmc as kv

    rank, world, local = dist_env()
    torch = None
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    ham = model()
    n = N_SITES // 2
    peaks = measure_peaks(local) if (rank == 0 and not a.no_peaks) else {}
    from kagomevmc import replicas

    from kagomevmc import autotune

    choice = mixed_choice(kv, ham, a)
    eng = autotune.make_engine(ham, a.walkers, choice, seed=replicas.replica_seed(a.seed, rank), device=local)
    cfg = eng.config()
    eng.init()
    run_steps(eng, a.warmup, a.moves)
    eng.enable_timing(True)
    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    eng.region_start()
    tot = run_steps(eng, a.steps, a.moves)
    ms = eng.region_stop()
    clk = clocks.stop()
    barrier()
    sweep_ms, sweep_n = eng.kernel_time(0)
    ref_ms, ref_n = eng.kernel_time(1)
    eng.enable_timing(False)
    import numpy as np
    dr = eng.walker_drift()
    drift = {"p50": float(np.percentile(dr, 50)), "p99": float(np.percentile(dr, 99)), "max": float(dr.max()),
             "walker_refreshes_per_step": tot["refreshes"] / a.steps / a.walkers,
             "what": "relative W drift max|W32 - W64|/(1+|W64|) per walker at its last refresh of the last step"}
    def allreduce(values, op):
        t = torch.tensor(values, dtype=torch.float64, device=f"cuda:{local}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX if op == "max" else torch.distributed.ReduceOp.SUM)
        return t.tolist()

    ms, red = replicas.reduce_run(ms, {"accepted": tot["accepted"]}, allreduce if world > 1 else None)
    accepted = red["accepted"]
    value = accepted / (ms * 1e-3)

    # end to end through the public API with host buffers: the walkers'
    # configurations and stream counters go host -> device, the step runs,
    # configurations, counters and per-walker statistics come back.
    ku, kd, ct = eng.get_state()
    e2e_steps = 0 if a.skip_e2e else min(a.steps, 4)
    e2e_acc = 0
    eng.region_start()
    for _ in range(e2e_steps):
        eng.set_state(ku, kd, ct)
        st = eng.advance(a.moves)
        ku, kd, ct = eng.get_state()
        ws = eng.walker_stats()
        e2e_acc += st["accepted"]
    e2e_ms = eng.region_stop()
    Wk = a.walkers
    h2d = ku.nbytes + kd.nbytes + ct.nbytes
    d2h = ku.nbytes + kd.nbytes + ct.nbytes + (sum(v.nbytes for v in ws.values()) if e2e_steps else 0)
    e2e = {"value": e2e_acc / (e2e_ms * 1e-3) if e2e_steps else None, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
           "path": "kvmc_set_state (H2D + W rebuild by FP32 refinement, FP64 per flagged walker) -> kvmc_advance -> "
                   "kvmc_get_state + kvmc_walker_stats (D2H)"}
    eng.close()
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # plain FP64 form on the same walkers (the denominator of the headline speed-up)
    plain = None
    if not a.skip_plain:
        pe = kv.Engine(ham, a.walkers, precision="plain", seed=a.seed, device=local)
        pe.init()
        run_steps(pe, 1, 16)
        pe.region_start()
        ptot = run_steps(pe, 2, 64)
        pms = pe.region_stop()
        pe.close()
        plain = {"value": ptot["accepted"] / (pms * 1e-3), "unit": UNIT, "ms": pms,
                 "moves_per_walker": 128, "accepted": ptot["accepted"]}
    # long enough for every walker to pass two of the mixed form's periodic refreshes
    # (acceptance ~0.127 at N=216)
    # two of the mixed form's refresh intervals, in calls of the bench's step size
    gate_calls = a.gate_calls or max(8, -(-2 * cfg["refresh_interval"] // a.moves))
    gate = None if a.skip_gate else energy_gate(ham, kv, a.gate_walkers, gate_calls, a.moves, choice, a.seed + 1)
    adjoint = None if a.skip_grad else adjoint_run(kv, 4, local)
    uneven = None if a.skip_uneven else uneven_run(kv, a.seed, local)
    large = None if a.skip_large else large_run(kv, a.seed, local, walkers=a.large_walkers)
    field = None if a.skip_field else field_run(kv, a.seed, local)
    batched = None if a.skip_batched else batched_run(kv, a.seed, local)
    plugin = None if a.skip_plugin else plugin_run(kv, a.seed, local, walkers=a.walkers)

    # roofline of the dominant kernel
    refreshes = tot["refreshes"]
    f_refresh = 2 * ((2.0 / 3.0) * n ** 3 + 2.0 * (N_SITES - n) * n ** 2)   # FP64 flop per walker refresh
    f_move = 2.0 * N_SITES * N_SITES                                        # FP32 flop per accepted move
    warp = getattr(choice, "warp", 0)
    kern = {
        "sweep_mixed": {"ms": sweep_ms, "launches": sweep_n, "flop": tot["accepted"] * f_move,
                        "unit_work": "2*N^2 FP32 flop per accepted move (both spins' rank-1 update of N x n W)",
                        **({"kernel": "sweep_warp_kernel or sweep_warp_wide_kernel (one warp per walker)",
                            "executed_flop_per_move": N_SITES * N_SITES,
                            "executed_note": "the label-indexed blocks hold W's non-trivial rows only: "
                                             "2 spins x 2 flop x n_up x n_down = N^2 per accepted move"}
                           if warp else {})},
        "refresh": {"ms": ref_ms, "launches": ref_n, "flop": refreshes * f_refresh,
                    "unit_work": "2*((2/3)n^3 + 2(N-n)n^2) flop per walker refresh (the FP64 algorithm's count)",
                    "arithmetic": ("FP32 iterative refinement, one thread per row (FP32 LU and solves, "
                                   "exact-product compensated residual), FP64 fallback per walker" if n < 96 else
                                   "tiled FP32 iterative refinement (FP32 LU, explicit inverse, GEMM-shaped solves, "
                                   "residual summed exactly on a fixed grid), FP64 fallback per walker")},
    }
    for k in kern.values():
        k["achieved_tflops"] = k["flop"] / (k["ms"] * 1e-3) / 1e12 if k["ms"] > 0 else None
    dom = max(kern, key=lambda k: kern[k]["ms"])
    peak_key = "fp64_tflops" if (dom == "refresh" and n > 128) else "fp32_tflops"
    peak = peaks.get(peak_key)
    # DRAM bytes per launch from the ncu captures summarised in profiles/,
    # scaled from the captured launch to this run's launches by the units
    # each processes (walkers per sweep launch, walker-spins per refresh)
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        tj = json.load(open(tfile))
        if dom == "sweep_mixed" and kern[dom]["launches"]:
            key = "sweep_warp" if warp else ("sweep_mixed" if cfg["w_on_chip"] else "sweep_mixed_hbm")
            if key in tj:
                # bytes per accepted move of the captured launch, times this run's moves per launch
                if "bytes_per_accepted_move" in tj[key]:
                    traffic = tj[key]["bytes_per_accepted_move"] * tot["accepted"] / kern[dom]["launches"]
                else:
                    traffic = tj[key]["bytes_per_walker_launch"] * a.walkers * a.steps / kern[dom]["launches"]
        elif dom == "refresh" and kern[dom]["launches"]:
            traffic = tj["refresh_fp64"]["bytes_per_walker_spin"] * 2 * refreshes / kern[dom]["launches"]
    ach = kern[dom]["achieved_tflops"]
    roof = {"bound": "fp64" if peak_key == "fp64_tflops" else "fp32", "kernel": dom,
            "achieved": ach, "peak": peak, "unit": "TFLOP/s",
            "frac": (ach / peak) if (ach and peak) else None, "traffic": traffic,
            "peak_source": f"cuBLAS {peak_key[:4].upper()} GEMM via torch.matmul, measured in this run",
            "per_launch_flop": kern[dom]["flop"] / max(kern[dom]["launches"], 1),
            "kernels": kern}

    cpu = None
    if not a.skip_cpu:
        threads = cpu_threads()
        acc, sec = cpu_port_run(oracle_model(), threads, 64800, a.seed, threads)
        cpu = {"value": acc / sec, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{threads} chains x 64800 proposals, N=216, complex double (oracle port), "
                         f"refresh and E_L every 108 proposals, {sec:.1f} s wall"}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (W, ratios, rank-1) + f64 (refresh, energy sums)", "data": "synthetic (seeded random starts)",
            "config": {"workload": "kagome VMC, 6x6 doubled cells (N=216), pi-flux partons, reference acceptance rule",
                       "walkers_per_gpu": a.walkers, "accepted_moves_per_walker_per_step": a.moves,
                       "refresh_every_accepted": cfg["refresh_interval"], "measure_every_proposals": n,
                       "delay_k": cfg["delay_k"], "w_on_chip": cfg["w_on_chip"],
                       "threads_per_walker": (32 if warp else choice.threads if not cfg["w_on_chip"] else 512),
                       **({"kernel": "one warp per walker, W's non-trivial rows indexed by labels",
                           "walkers_per_cta": warp, "accuracy_guard": [choice.guard_hi, choice.guard_lo]}
                          if warp else {}),
                       "settings_from": "autotuner cache kagomevmc/tuned.json (GB300), flags override",
                       "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (W state 382 MB per GPU)",
                       # the accuracy gate of the metric, as flat keys next to the workload it qualifies
                       **({"gate_dE_per_site_all_walkers": gate["dE_per_site"],
                           "gate_se_dE_per_site": gate["se_dE_per_site"], "gate_pass": gate["pass"],
                           "gate_walkers": gate["walkers"], "gate_worst_walker_dE": gate["worst_walker_dE_per_site"],
                           "gate_max_w_drift_at_refresh": gate["max_w_drift_at_refresh"]} if gate else {})},
            "proposals_per_step": tot["proposals"] / a.steps * world, "acceptance": tot["accepted"] / tot["proposals"],
            "gpu_launches": tot["launches"], "e2e": e2e, "roofline": roof, "cpu_baseline": cpu,
            "plain_fp64": plain, "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
            "energy_gate": gate, "adjoint": adjoint, "uneven_batch": uneven, "large_lattice": large,
            "field_workload": field, "batched_n96": batched, "plugin_e2e": plugin,
            "drift": drift, "clocks": clk, "peaks_measured": peaks}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    a = args_()
    if a.impl == "reference":
        reference_arm(a)
    else:
        gpu_arm(a)


if __name__ == "__main__":
    main()
