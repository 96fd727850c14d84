"""Tunes the shipped workloads on the local GPU and writes kagomevmc/tuned.json.

    python -m kagomevmc.tune_shipped            # from kagomedsl.jl_gb300/

Workloads (doubled-cell kagome, pi-flux partons, half filling, reference
acceptance rule):
  N=216 x 2048 walkers   the headline batch
  N=96  x 4096           batched walkers
  N=54  x 1024, N=216 x 768, N=384 x 256   the classes of the uneven batch
  N=864 x 512            the large lattice (W in HBM)
  N=192 x 2048, complex  the field workload (8x8 doubled cells, imbalance 4)
"""
from __future__ import annotations

import json
import math
import os
import sys

from . import autotune
from .lattice import DoubleKagome, Hamiltonian

CELLS = {54: (3, 3), 96: (4, 4), 216: (6, 6), 384: (8, 8), 864: (12, 12)}
WORKLOADS = [(216, 2048, {}), (96, 4096, {}), (54, 1024, {}), (216, 768, {}), (384, 256, {}),
             (864, 512, dict(delays=(8, 16), refresh=(128, 256), threads=(256,), placements=("hbm",), warps=(2,),
                             warmup=128))]
# Candidates beyond the default refresh list are left out at N=864, where one
# FP64 refresh of 512 walkers takes ~0.5 s.


def model(N):
    a, b = CELLS[N]
    return Hamiltonian.build(N // 2, N // 2, DoubleKagome(1.0, 2 * a, b, (True, True), (False, True)))


def field_model():
    """8x8 doubled cells (N=192) in the field B = 4 pi / S of imbalance 4
    (N_up = 98, N_down = 94): complex orbitals."""
    from .lattice import Hmat, get_nn, orbitals

    lat = DoubleKagome(1.0, 8, 8, (True, True), (False, True))
    H = Hmat(lat, B=4 * math.pi / (64 * 2 * math.sqrt(3)))
    Uu, Ud = orbitals(H, 98, 94)
    return Hamiltonian(98, 94, Uu, Ud, H, get_nn(H))


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    only = None
    if "--only" in argv:
        i = argv.index("--only")
        only = {int(x) for x in argv[i + 1].split(",")}
        argv = argv[:i] + argv[i + 2:]
    out = argv[0] if argv else autotune.SHIPPED
    cache = json.load(open(out)) if os.path.exists(out) else {}
    jobs = [(model(N), walkers, kw) for N, walkers, kw in WORKLOADS if only is None or N in only]
    # complex W: delayed depths 4 and 8, W in HBM
    if only is None or 192 in only:
        jobs.append((field_model(), 2048, dict(delays=(4, 8), placements=("hbm",), threads=(256,), warps=())))
    for ham, walkers, kw in jobs:
        key = autotune.cache_key(ham, walkers, "reference", autotune._device_name(0))
        ch = autotune.tune(ham, walkers, **kw)
        row = dict(delay_k=ch.delay_k, refresh_interval=ch.refresh_interval, placement=ch.placement,
                   threads=ch.threads, moves_per_s=ch.moves_per_s, max_drift=ch.max_drift, trials=ch.trials,
                   warp=ch.warp, guard_hi=ch.guard_hi, guard_lo=ch.guard_lo)
        cache[key] = row
        print(key, {k: v for k, v in row.items() if k != "trials"}, flush=True)
        with open(out, "w") as f:
            json.dump(cache, f, indent=1)


if __name__ == "__main__":
    main()
