"""GPU parity of the one-warp-per-walker sweep (label-indexed W blocks).

Every chain is compared with the C oracle on the same Philox stream: same
final configuration, same accepted-move count, energy sums within 1e-4
relative (FP32 W); an FP32 rounding may flip a decision that sits within
~1e-6 of its threshold, so at most one walker of a batch may diverge.  W
after the call is compared with the oracle's reevaluateW at 1e-3 relative to
max(1, |W|) (the FP32 state after 2000+ proposals).
"""
import numpy as np
import pytest

import kagome_oracle as o
import oracle_c

pytestmark = pytest.mark.gpu

CELLS = {54: (3, 3), 96: (4, 4), 216: (6, 6), 384: (8, 8)}


@pytest.fixture(scope="module")
def kv(built):
    import kagomevmc

    return kagomevmc


def ham_for(kv, N):
    a, b = CELLS[N]
    return kv.Hamiltonian.build(N // 2, N // 2, kv.DoubleKagome(1.0, 2 * a, b, (True, True), (False, True)))


def close(a, b, rel):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.all(np.abs(a - b) <= rel * max(1.0, np.abs(b).max()))


def run_against_oracle(ham, eng, seed, proposals, walkers):
    n_up, n_dn = ham.U_up.shape[1], ham.U_down.shape[1]
    ku0, kd0, _ = eng.get_state()
    st = eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    meas = min(n_up, n_dn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, meas, meas, 0)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            assert ws["n_meas"][w] == proposals // meas
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= 1e-4 * max(1.0, abs(ch.c.sum_e)), w
    assert match >= walkers - 1, match
    assert st["bad_walkers"] == 0
    Wu, Wd = eng.get_w()
    for w in range(walkers):
        assert close(Wu[w], o.reevaluateW(ham.U_up, ku1[w]), 1e-3), w
        assert close(Wd[w], o.reevaluateW(ham.U_down, kd1[w]), 1e-3), w
    return st


@pytest.mark.parametrize("N,delay_k,wpb", [(54, 4, 14), (96, 8, 14), (96, 16, 4), (216, 8, 14), (216, 12, 7),
                                           (216, 4, 3), (384, 8, 8)])
def test_warp_chains_match_c_oracle(kv, N, delay_k, wpb):
    walkers, proposals, seed = 10, 2400, 71
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=96, delay_k=delay_k,
                    w_placement="hbm")
    eng.set_warp_walkers(wpb)
    eng.init()
    run_against_oracle(ham, eng, seed, proposals, walkers)
    # advance: exact move counts
    before = eng.walker_stats()["accepted"].copy()
    eng.advance(77)
    assert np.all(eng.walker_stats()["accepted"] == before + 77)
    eng.close()


@pytest.mark.parametrize("rule", ["reference", "metropolis"])
def test_warp_unequal_spin_counts(kv, rule):
    """N_up != N_down: the two blocks are n_down x n_up and n_up x n_down."""
    N, n_up, seed, walkers, proposals = 54, 30, 23, 8, 1500
    lat = kv.DoubleKagome(1.0, 6, 3, (True, True), (False, True))
    H = kv.Hmat(lat)
    Uu, Ud = kv.orbitals(H, n_up, N - n_up)
    ham = kv.Hamiltonian(n_up, N - n_up, Uu, Ud, H, kv.get_nn(H))
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, delay_k=8, w_placement="hbm", accept=rule,
                    refresh_interval=64)
    eng.set_warp_walkers(8)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(Uu, Ud, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, 24, 24, 0 if rule == "reference" else 1)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= 1e-4 * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - 1
    eng.close()


def test_warp_matches_cta_kernel_walker_by_walker(kv):
    """The same walkers through the one-CTA-per-walker pipelined kernel and the
    one-warp kernel: same chains (up to FP32 decision flips), same energy sums."""
    N, walkers, seed = 216, 32, 5
    ham = ham_for(kv, N)
    out = []
    for warp in (0, 14):
        eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=512, delay_k=8,
                        w_placement="hbm")
        if warp:
            eng.set_warp_walkers(warp)
        eng.init()
        eng.advance(600)
        ws = eng.walker_stats()
        out.append((eng.get_state(), ws["sum_e"].copy(), ws["accepted"].copy()))
        eng.close()
    (s0, e0, a0), (s1, e1, a1) = out
    same = [w for w in range(walkers) if np.array_equal(s0[0][w], s1[0][w])]
    assert len(same) >= walkers - 2
    assert np.all(a0 == a1)
    for w in same:
        assert abs(e0[w] - e1[w]) <= 1e-4 * max(1.0, abs(e0[w]))


@pytest.mark.parametrize("segment,refresh32", [(0, 1), (16, 1), (16, 2)])
def test_warp_accuracy_guard_refreshes_and_keeps_chains(kv, segment, refresh32):
    """A guard every walker trips at almost every move (hi 1, lo 1000: some
    entry above 1 has always been seen, and a move's entries stay below
    1000).  The refresh it asks for waits for the end of the call, or of its
    segment of 16 moves: one refresh per walker per call or segment, exact
    move counts, chains still the oracle's, W at the end the oracle's.  The
    refreshes inside the call write the label-indexed rows, by the FP32
    refresh one thread per row (1) or in tiles (2)."""
    N, walkers, seed, A = 96, 8, 43, 300
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=4096, delay_k=8,
                    w_placement="hbm")
    eng.set_refresh32(refresh32)
    eng.set_warp_walkers(8)
    eng.set_accuracy_guard(1, 1000)
    eng.set_segment(segment)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.advance(A)
    assert st["accepted"] == walkers * A
    per_walker = 1 if segment == 0 else -(-A // segment)
    # an FP32 refresh that does not converge is redone in FP64 (counted once more)
    assert walkers * per_walker <= st["refreshes"] <= walkers * per_walker + walkers, st["refreshes"]
    ku1, kd1, ct = eng.get_state()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, int(ct[w]), N // 2, N // 2)
        match += int(np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]))
    assert match >= walkers - 1
    Wu, Wd = eng.get_w()
    for w in range(walkers):
        # right after the refresh at the end of the call
        assert close(Wu[w], o.reevaluateW(ham.U_up, ku1[w]), 1e-5), w
        assert close(Wd[w], o.reevaluateW(ham.U_down, kd1[w]), 1e-5), w
    eng.close()


def test_warp_walkers_refused_off_its_path(kv):
    ham = ham_for(kv, 96)
    eng = kv.Engine(ham, 2, precision="plain")
    with pytest.raises(kv.KvmcError):
        eng.set_warp_walkers(8)
    eng.close()
    eng = kv.Engine(ham, 2, precision="mixed", delay_k=1)
    with pytest.raises(kv.KvmcError):
        eng.set_warp_walkers(8)
    eng.close()


def test_headline_energy_gate_and_drift_bound(kv):
    """N=216 with the shipped one-warp settings of the headline batch (k, R,
    walkers per CTA, accuracy guard) on 256 walkers, against the plain FP64
    form on the same starts and proposal streams: after one thermalization
    call of 1024 accepted moves, four more calls.  The paired difference of
    the per-walker mean energies over every walker satisfies
    |mean| + 2 se <= 1e-4 per site, and no refresh in the measured calls sees
    a relative W drift above 1e-2."""
    from kagomevmc import autotune

    ham = ham_for(kv, 216)
    choice = autotune.lookup(ham, 2048)
    assert choice is not None and choice.warp > 0 and choice.guard_hi > 0
    walkers, seed, moves = 256, 2025, 1024
    out = {}
    for prec in ("plain", "mixed"):
        eng = (autotune.make_engine(ham, walkers, choice, seed=seed) if prec == "mixed"
               else kv.Engine(ham, walkers, precision="plain", seed=seed))
        eng.init()
        eng.advance(moves)
        eng.reset_stats()
        drift = 0.0
        for _ in range(4):
            drift = max(drift, eng.advance(moves)["max_drift"])
        ws = eng.walker_stats()
        out[prec] = (ws["sum_e"] / ws["n_meas"], drift)
        eng.close()
    d = (out["mixed"][0] - out["plain"][0]) / 216
    assert abs(d.mean()) + 2 * d.std(ddof=1) / np.sqrt(walkers) <= 1e-4, (d.mean(), d.std())
    assert out["mixed"][1] <= 1e-2, out["mixed"][1]


def test_warp_blocks_stay_the_state_across_calls_and_w_reads(kv):
    """One-warp mode keeps W's label-indexed blocks as the state from one
    sweep call to the next and converts back only for a call that reads the
    site-indexed W.  Two calls of 120 accepted moves per walker with kvmc_get_w
    and kvmc_measure between them end in exactly the configurations, counts and
    energy sums of one call of 240 from the same starts (120 is a multiple of
    the delay depth 12, so both runs flush the same moves together; no refresh
    due in either run, guard off), and the W read in between is the oracle's
    to 1e-2 relative (the FP32 state 120 moves after its last rebuild)."""
    ham = ham_for(kv, 216)
    walkers, seed = 14, 41
    runs = []
    for split in (True, False):
        eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=4096, delay_k=12,
                        w_placement="hbm")
        eng.set_warp_walkers(7)
        eng.set_drift_tolerance(1e9)
        eng.init()
        if split:
            eng.advance(120)
            Wu, Wd = eng.get_w()
            ku, kd, _ = eng.get_state()
            for w in range(walkers):
                # FP32 W after 120 moves without a refresh (guard off): a
                # conversion fault would show as O(1) errors
                assert close(Wu[w], o.reevaluateW(ham.U_up, ku[w]), 1e-2), w
                assert close(Wd[w], o.reevaluateW(ham.U_down, kd[w]), 1e-2), w
            e = eng.measure()
            assert np.all(np.isfinite(e))
            eng.advance(120)
        else:
            eng.advance(240)
        ku, kd, ct = eng.get_state()
        stats = eng.walker_stats()
        runs.append((ku, kd, ct, stats))
        eng.close()
    (ka, kda, ca, sa), (kb, kdb, cb, sb) = runs
    assert np.array_equal(ka, kb) and np.array_equal(kda, kdb) and np.array_equal(ca, cb)
    assert np.array_equal(sa["accepted"], sb["accepted"])
    assert np.array_equal(sa["sum_e"], sb["sum_e"])
