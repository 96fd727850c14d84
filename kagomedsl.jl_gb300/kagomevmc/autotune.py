"""Autotuner for the mixed form: where W lives, the launch shape, the
delayed-update depth k and the refresh interval R.

For a model and batch size it times short trials over the candidates on the
actual GPU and keeps the fastest one whose measured W drift stays within a
bound.  Drift is measured at each FP64 refresh as
max |W_fp32 - W_fp64| / (1 + |W_fp64|) per walker (the refresh kernel
records it), so a longer interval is accepted only when the FP32 state it
leaves behind is still accurate.

Candidates:
  placement  "chip" (W staged in shared memory, one walker per SM; only when
             it fits) or "hbm" (W in HBM, delayed factors on chip, two or four
             walkers per SM)
  threads    128 or 256 threads per walker with W in HBM
  warp       W in HBM with one warp per walker (label-indexed W blocks), 4 to
             14 walkers per CTA, with the accuracy guard GUARD
  k          1 (rank-1), 4, 8, 12, 16
  R          accepted moves between FP64 refreshes

Results are cached per (sites, orbitals, walkers, acceptance rule, device
name) in a JSON file so a production run tunes once; ``tuned.json`` next to
this module holds the choices measured on a GB300 for the shipped workloads.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time
from dataclasses import asdict, dataclass, field

import numpy as np

from . import _lib

DELAYS = (1, 4, 8, 12, 16)
REFRESH = (128, 256, 512, 1024, 2048, 4096, 8192)
PLACEMENTS = ("chip", "hbm")
THREADS = (128, 256)
WARPS = (4, 7, 10, 14)   # walkers per CTA for one warp per walker
GUARD = (200, 20)        # the one-warp sweep's accuracy guard (kvmc.h KVMC_TUNE_COND_HI / _LO)
DRIFT_BOUND = 1e-2  # on the 99.9th percentile of per-walker relative drift
SHIPPED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned.json")


@dataclass
class Choice:
    delay_k: int
    refresh_interval: int
    placement: str = "chip"
    threads: int = 256
    moves_per_s: float = 0.0
    max_drift: float = 0.0
    trials: list = field(default_factory=list)
    warp: int = 0            # > 0: one warp per walker, this many walkers per CTA
    guard_hi: int = 0
    guard_lo: int = 0
    refresh32: int = -1      # the periodic refresh's form (KVMC_TUNE_REFRESH32); -1: the library's default

    def engine_kwargs(self) -> dict:
        return dict(precision="mixed", delay_k=self.delay_k, refresh_interval=self.refresh_interval,
                    w_placement=self.placement)


def _device_name(device: int) -> str:
    """The chip the choice was measured on ("GB300" for any GB300 board)."""
    buf = C.create_string_buffer(256)
    try:
        rc = _lib.load().kvmc_device_name(int(device), buf, len(buf), None)
    except OSError:
        return "GB300"
    if rc != _lib.KVMC_OK:
        return "GB300"
    name = buf.value.decode(errors="replace")
    return "GB300" if "GB300" in name else name


def cache_key(ham, walkers, accept="reference", device_name=None):
    return (f"N{ham.U_up.shape[0]}_nu{ham.U_up.shape[1]}_nd{ham.U_down.shape[1]}_W{walkers}_{accept}"
            f"_{'c' if np.iscomplexobj(ham.U_up) else 'r'}_{device_name or 'GB300'}")


def lookup(ham, walkers, accept="reference", device_name=None, path: str | None = None) -> Choice | None:
    """The cached choice for this workload, from `path` or the shipped table."""
    for p in ([path] if path else []) + [SHIPPED]:
        if p and os.path.exists(p):
            cache = json.load(open(p))
            key = cache_key(ham, walkers, accept, device_name)
            if key in cache:
                return Choice(**cache[key])
    return None


def make_engine(ham, walkers, choice: Choice, **kw):
    """An Engine configured with `choice` (kw: accept, seed, device, ...)."""
    from .montecarlo import Engine

    eng = Engine(ham, walkers, **choice.engine_kwargs(), **kw)
    if choice.refresh32 >= 0:
        eng.set_refresh32(choice.refresh32)
    if choice.warp > 0:
        eng.set_warp_walkers(choice.warp)
        eng.set_accuracy_guard(choice.guard_hi, choice.guard_lo)
    elif choice.placement == "hbm" and choice.delay_k > 1:
        eng.set_stream_threads(choice.threads)
    return eng


def tune(ham, walkers: int, *, device: int = 0, seed: int = 1, accept: str = "reference",
         warmup: int = 512, delays=DELAYS, refresh=REFRESH, placements=PLACEMENTS, threads=THREADS,
         warps=WARPS, guard=GUARD, drift_bound: float = DRIFT_BOUND, cache_path: str | None = None,
         verbose: bool = False) -> Choice:
    """Times the candidates for this model on `walkers` walkers and returns the best.

    Each trial: fresh engine, seeded random starts, a warm-up of
    max(R, warmup) accepted moves per walker (past the transient after the
    random starts), then a timed 2R accepted moves per walker (CUDA events
    on the handle's stream), so each walker's FP64 refreshes fall inside the
    timed window.  Candidates that do not fit on chip are skipped.
    """
    from .montecarlo import Engine

    dev_name = _device_name(device)
    key = cache_key(ham, walkers, accept, dev_name)
    if cache_path and os.path.exists(cache_path):
        cache = json.load(open(cache_path))
        if key in cache:
            return Choice(**cache[key])
    trials = []
    best = None
    # (placement, threads, walkers per CTA for one warp per walker or 0)
    shapes = []
    for place in placements:
        shapes += [(place, th, 0) for th in (threads if place == "hbm" else (256,))]
        if place == "hbm":
            shapes += [(place, 256, wp) for wp in warps]
    for place, th, wp in shapes:
        for k in delays:
            if (th != 256 or wp) and k <= 1:
                continue
            for R in refresh:
                try:
                    eng = Engine(ham, walkers, precision="mixed", accept=accept, seed=seed, refresh_interval=R,
                                 device=device, delay_k=k, w_placement=place)
                    if wp:
                        eng.set_warp_walkers(wp)
                        eng.set_accuracy_guard(*guard)
                    elif place == "hbm" and k > 1:
                        eng.set_stream_threads(th)
                except _lib.KvmcError:
                    continue  # does not fit for this model
                try:
                    if eng.config()["delay_k"] != k:
                        continue
                    eng.init()
                    eng.advance(max(R, warmup))
                    eng.region_start()
                    st = eng.advance(2 * R)
                    ms = eng.region_stop()
                    drift = float(np.percentile(eng.walker_drift(), 99.9))
                finally:
                    eng.close()
                rate = st["accepted"] / (ms * 1e-3)
                row = dict(placement=place, threads=th, warp=wp, delay_k=k, refresh_interval=R, moves_per_s=rate,
                           max_drift=drift, refreshes=st["refreshes"])
                trials.append(row)
                if verbose:
                    print(row, flush=True)
                if drift <= drift_bound and (best is None or rate > best["moves_per_s"]):
                    best = row
    if not trials:
        raise _lib.KvmcError(_lib.KVMC_ERR_UNSUPPORTED, "no candidate configuration could be created")
    if best is None:  # nothing met the bound: the most frequent refresh of the fastest candidate
        best = min(trials, key=lambda r: (r["refresh_interval"], -r["moves_per_s"]))
    choice = Choice(best["delay_k"], best["refresh_interval"], best["placement"], best["threads"],
                    best["moves_per_s"], best["max_drift"], trials, best.get("warp", 0),
                    guard[0] if best.get("warp", 0) else 0, guard[1] if best.get("warp", 0) else 0)
    if cache_path:
        cache = json.load(open(cache_path)) if os.path.exists(cache_path) else {}
        cache[key] = asdict(choice)
        tmp = f"{cache_path}.{os.getpid()}.{int(time.time())}"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, cache_path)
    return choice
