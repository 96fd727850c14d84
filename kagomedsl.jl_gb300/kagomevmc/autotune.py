"""Autotuner for the mixed form: delayed-update depth k and refresh interval R.

For a model and batch size it times short trials over the candidate
(k, R) pairs on the actual GPU and keeps the fastest pair whose measured W
drift stays within a bound.  Drift is measured at each FP64 refresh as
max |W_fp32 - W_fp64| / (1 + |W_fp64|) over all walkers (the refresh
kernel records it), so a longer interval is accepted only when the FP32
state it leaves behind is still accurate.

Results are cached per (sites, orbitals, walkers, device name) in a JSON
file so a production run tunes once.
"""
from __future__ import annotations

import json
import os
import time
from dataclasses import asdict, dataclass

import numpy as np

from . import _lib

DELAYS = (1, 4, 8, 12, 16)
REFRESH = (32, 64, 128, 256, 512, 1024, 2048)
DRIFT_BOUND = 1e-2  # on the 99.9th percentile of per-walker relative drift


@dataclass
class Choice:
    delay_k: int
    refresh_interval: int
    moves_per_s: float
    max_drift: float
    trials: list


def _device_name(device: int) -> str:
    try:
        import torch

        return torch.cuda.get_device_name(device)
    except Exception:
        return f"device{device}"


def _cache_key(ham, walkers, device):
    return f"N{ham.U_up.shape[0]}_nu{ham.U_up.shape[1]}_nd{ham.U_down.shape[1]}_W{walkers}_{_device_name(device)}"


def tune(ham, walkers: int, *, device: int = 0, seed: int = 1, accept: str = "reference",
         proposals: int = 1024, delays=DELAYS, refresh=REFRESH, drift_bound: float = DRIFT_BOUND,
         cache_path: str | None = None, verbose: bool = False) -> Choice:
    """Times (k, R) candidates for this model on `walkers` walkers and returns the best.

    Each trial: fresh engine, seeded random starts, a warm-up of
    max(R, proposals/8) accepted moves per walker, then a timed 2R accepted
    moves per walker (CUDA events on the handle's stream), so each walker's
    FP64 refreshes fall inside the timed window.  Candidates whose depth
    does not fit in shared memory for this model are skipped.
    """
    from .montecarlo import Engine

    key = _cache_key(ham, walkers, device)
    if cache_path and os.path.exists(cache_path):
        cache = json.load(open(cache_path))
        if key in cache:
            return Choice(**cache[key])
    trials = []
    best = None
    for k in delays:
        for R in refresh:
            try:
                eng = Engine(ham, walkers, precision="mixed", accept=accept, seed=seed, refresh_interval=R,
                             device=device, delay_k=k)
            except _lib.KvmcError:
                break  # this depth does not fit for this model
            try:
                # warm up, then time 2R accepted moves per walker so that every
                # walker pays for its FP64 refreshes inside the timed window
                eng.init()
                eng.advance(max(R, proposals))  # past the transient after the random starts
                eng.region_start()
                st = eng.advance(2 * R)
                ms = eng.region_stop()
                drift_p999 = float(np.percentile(eng.walker_drift(), 99.9))
            finally:
                eng.close()
            rate = st["accepted"] / (ms * 1e-3)
            row = dict(delay_k=k, refresh_interval=R, moves_per_s=rate, max_drift=drift_p999,
                       refreshes=st["refreshes"])
            trials.append(row)
            if verbose:
                print(row, flush=True)
            ok = st["max_drift"] <= drift_bound
            if ok and (best is None or rate > best["moves_per_s"]):
                best = row
    if best is None:  # nothing met the bound: the most frequent refresh of the fastest depth
        best = min(trials, key=lambda r: (r["refresh_interval"], -r["moves_per_s"]))
    choice = Choice(best["delay_k"], best["refresh_interval"], best["moves_per_s"], best["max_drift"], trials)
    if cache_path:
        cache = json.load(open(cache_path)) if os.path.exists(cache_path) else {}
        cache[key] = asdict(choice)
        tmp = f"{cache_path}.{os.getpid()}.{int(time.time())}"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, cache_path)
    return choice
