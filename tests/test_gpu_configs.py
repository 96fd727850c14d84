"""The workloads the hot path is specified on, run as written.

Small plain: 2x2 doubled cells (N=24), the pi-flux parton state, one Markov
chain in FP64 from the reference's pivoted-QR start, seed 0, 1000 warm-up
and 10000 measured sweeps (a sweep of src/MonteCarlo.jl:538-607 is one
proposal; the energy is sampled every 12), against the exact FP64
enumeration of all C(24,12) placements of the up spins (golden fixture)
within two standard errors, the error bar from 25 block means.  The same chain
through the C oracle is identical proposal by proposal.

Batched: 4x4 doubled cells (N=96), 4096 chains from seeded random starts,
FP32 ratios with rank-16 delayed updates, the flush as FP32 FMA or as 3xTF32
on the tensor cores, a refresh every 64 accepted moves, 500 warm-up and 2000
measured sweeps per chain; E/N of each against the plain FP64 form on the
same starts and proposal streams: the paired per-walker difference
satisfies |mean| + 2 se <= 1e-4 per site.
"""
import json
import os

import numpy as np
import pytest

import oracle_c

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def kv(built):
    import kagomevmc

    return kagomevmc


def ham24(kv):
    """N=24 with the orbital choice the enumeration fixture was made with
    (the pi-flux spectrum is degenerate at half filling)."""
    ham = kv.Hamiltonian.build(12, 12, kv.DoubleKagome(1.0, 4, 2, (True, True), (False, True)))
    U = np.load(os.path.join(GOLD, "u_N24.npy"))
    return kv.Hamiltonian(12, 12, U, U.copy(), ham.H_mat, ham.nn)


def test_single_chain_n24_against_exact_enumeration(kv):
    golden = json.load(open(os.path.join(GOLD, "golden.json")))
    exact = golden["enum_N24"]["E_per_site_reference_rule"]
    ham = ham24(kv)
    ku, kd = kv.init_conf_qr(ham.U_up, ham.U_down, 24, 12)
    eng = kv.Engine(ham, 1, precision="plain", seed=0)
    eng.init(ku, kd)
    eng.sweep(1000)
    eng.reset_stats()
    blocks, prev_s, prev_n = [], 0.0, 0
    for _ in range(25):
        eng.sweep(400)
        ws = eng.walker_stats()
        s, n = float(ws["sum_e"][0]), int(ws["n_meas"][0])
        blocks.append((s - prev_s) / (n - prev_n))
        prev_s, prev_n = s, n
    ku1, kd1, _ = eng.get_state()
    acc = int(eng.walker_stats()["accepted"][0])
    eng.close()
    blocks = np.array(blocks) / 24
    e, se = blocks.mean(), blocks.std(ddof=1) / np.sqrt(len(blocks))
    assert abs(e - exact) <= 2 * se, (e, exact, se)
    # the same chain through the oracle, proposal by proposal
    ch = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn).new_chain(ku, kd)
    ch.run(0, 0, 1000, 12, 12, 0, record=False)
    a0, s0, n0 = ch.c.accepted, ch.c.sum_e, ch.c.n_meas
    ch.run(0, 0, 10000, 12, 12, 0, record=False)
    assert np.array_equal(ch.ku, ku1[0]) and np.array_equal(ch.kd, kd1[0])
    assert ch.c.accepted - a0 == acc and ch.c.n_meas - n0 == prev_n
    assert abs((ch.c.sum_e - s0) - prev_s) <= 1e-9 * max(1.0, abs(prev_s))


@pytest.mark.parametrize("flush", ["fma", "3xtf32"])
def test_batched_n96_against_plain(kv, flush):
    ham = kv.Hamiltonian.build(48, 48, kv.DoubleKagome(1.0, 8, 4, (True, True), (False, True)))
    walkers, seed = 4096, 31
    out = {}
    for prec in ("plain", "mixed"):
        if prec == "plain":
            eng = kv.Engine(ham, walkers, precision="plain", seed=seed)
        else:
            eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, delay_k=16, refresh_interval=64,
                            w_placement="hbm")
            eng.set_stream_threads(128)
            if flush == "3xtf32":
                eng.set_tc_flush(True)
        eng.init()
        eng.sweep(500)
        eng.reset_stats()
        st = eng.sweep(2000)
        assert st["bad_walkers"] == 0
        ws = eng.walker_stats()
        out[prec] = ws["sum_e"] / ws["n_meas"] / 96
        eng.close()
    d = out["mixed"] - out["plain"]
    assert abs(d.mean()) + 2 * d.std(ddof=1) / np.sqrt(walkers) <= 1e-4, (d.mean(), d.std(ddof=1))
