"""GPU parity: libkvmc (through its C ABI) against the oracle and the golden fixtures.

Tolerances (stated per result):
  plain FP64 form: W, ratios, local energies within 1e-10 relative to the
  oracle; chains follow the oracle's trajectory exactly.
  mixed FP32 form: W within 1e-6 relative to max(1, |W|) after a refresh;
  ratios and local energies within 1e-5 relative; chains follow the
  oracle's trajectory (an FP32 rounding may flip a decision that sits within
  ~1e-6 of its threshold, so at most one walker of a batch may diverge).
"""
import json
import os

import numpy as np
import pytest

import kagome_oracle as o
import oracle_c

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CELLS = {24: (2, 2), 54: (3, 3), 96: (4, 4), 216: (6, 6), 384: (8, 8), 864: (12, 12)}


@pytest.fixture(scope="module")
def kv(built):
    import kagomevmc

    return kagomevmc


@pytest.fixture(scope="module")
def golden():
    return json.load(open(os.path.join(GOLD, "golden.json")))


def ham_for(kv, N):
    a, b = CELLS[N]
    ham = kv.Hamiltonian.build(N // 2, N // 2, kv.DoubleKagome(1.0, 2 * a, b, (True, True), (False, True)))
    if N == 24:
        U = np.load(os.path.join(GOLD, "u_N24.npy"))
        ham = kv.Hamiltonian(12, 12, U, U.copy(), ham.H_mat, ham.nn)
    return ham


def oracle_ham(ham):
    return o.Hamiltonian(ham.N_up, ham.N_down, ham.U_up, ham.U_down, ham.H_mat, [(i + 1, j + 1) for i, j in ham.nn])


def close(a, b, rel):
    """Elementwise |a - b| <= rel * max(1, max|b|): the error of a solve with
    tilde_U scales with the largest entry of W (cond(tilde_U) reaches ~1e4 at
    N=216, while both sides stay backward stable to ~1e-12)."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.all(np.abs(a - b) <= rel * max(1.0, np.abs(b).max()))


@pytest.mark.parametrize("precision", ["plain", "mixed"])
@pytest.mark.parametrize("N", [24, 54, 96, 216, 384, 864])
def test_refresh_matches_oracle(kv, N, precision):
    """N <= 320 factorises tilde_U in shared memory; N = 384 and 864 (192 and
    432 orbitals per spin) take the blocked LU in HBM."""
    ham = ham_for(kv, N)
    U = ham.U_up
    nw = 4 if N <= 384 else 2
    starts = [o.seeded_start(13, w, U, U)[:2] for w in range(nw)]
    eng = kv.Engine(ham, nw, precision=precision, seed=13)
    eng.init(np.stack([s[0] for s in starts]), np.stack([s[1] for s in starts]))
    Wu, Wd = eng.get_w()
    tol = 1e-10 if precision == "plain" else 1e-6
    for w, (ku, kd) in enumerate(starts):
        assert close(Wu[w], o.reevaluateW(U, ku), tol), (N, w)
        assert close(Wd[w], o.reevaluateW(U, kd), tol), (N, w)
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
@pytest.mark.parametrize("N", [24, 54, 96])
def test_ratios_and_local_energy_match_golden(kv, golden, N, precision):
    ham = ham_for(kv, N)
    cases = golden["configs"][str(N)]
    eng = kv.Engine(ham, len(cases), precision=precision)
    eng.init(np.array([c["kappa_up"] for c in cases]), np.array([c["kappa_down"] for c in cases]))
    tol = 1e-10 if precision == "plain" else 1e-5
    E = eng.measure()
    for w, c in enumerate(cases):
        assert abs(E[w] - c["local_energy"]) <= tol * max(1.0, abs(c["local_energy"])), (N, w, E[w])
    nm = min(len(c["moves"]) for c in cases)
    moves = np.array([c["moves"][:nm] for c in cases])
    R = eng.eval_ratios(moves)
    for w, c in enumerate(cases):
        np.testing.assert_allclose(R[w], c["ratios"][:nm], rtol=tol, atol=tol)
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
@pytest.mark.parametrize("N", [24, 54])
def test_chain_matches_golden(kv, golden, N, precision):
    """Same Philox stream as the oracle: same accepted moves, same final configuration."""
    g = golden["chains"][str(N)]
    ham = ham_for(kv, N)
    W = len(g["walkers"])
    eng = kv.Engine(ham, W, precision=precision, seed=g["seed"], measure_interval=g["measure_every"])
    eng.init(np.array([c["start_up"] for c in g["walkers"]]), np.array([c["start_down"] for c in g["walkers"]]))
    st = eng.sweep(g["proposals"])
    ku, kd, ct = eng.get_state()
    ws = eng.walker_stats()
    assert np.all(ct == g["proposals"])
    match = 0
    for w, c in enumerate(g["walkers"]):
        if ku[w].tolist() == c["final_up"] and kd[w].tolist() == c["final_down"]:
            match += 1
            assert ws["accepted"][w] == c["accepted"]
            assert ws["n_meas"][w] == len(c["energies"])
            tol = 1e-9 if precision == "plain" else 1e-4
            assert abs(ws["sum_e"][w] - sum(c["energies"])) <= tol * max(1.0, abs(sum(c["energies"])))
    assert match >= W - (0 if precision == "plain" else 1)
    assert st["bad_walkers"] == 0
    eng.close()


@pytest.mark.parametrize("precision,delay_k", [("plain", 0), ("mixed", 1), ("mixed", 4), ("mixed", 8), ("mixed", 16)])
@pytest.mark.parametrize("accept", ["reference", "metropolis"])
def test_long_chains_match_c_oracle(kv, precision, delay_k, accept):
    """Plain form and the mixed form with rank-1 or delayed (depth 4/8/16) updates."""
    N, walkers, proposals, seed = 96, 12, 3000, 21
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision=precision, accept=accept, seed=seed,
                    refresh_interval=(64 if precision == "mixed" else 0), delay_k=delay_k)
    if precision == "mixed":
        assert eng.config()["delay_k"] == max(delay_k, 1)
        eng.set_pipeline(False)   # the sequential scan / column-write kernel; the pipelined one is the default
    eng.init()
    ku0, kd0, _ = eng.get_state()
    eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    rule = 0 if accept == "reference" else 1
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, 48, 48, rule)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            tol = 1e-8 if precision == "plain" else 1e-4
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= tol * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - (0 if precision == "plain" else 1)
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_seeded_starts_match_oracle(kv, precision):
    N, seed = 54, 77
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, 6, precision=precision, seed=seed)
    att = eng.init()
    ku, kd, ct = eng.get_state()
    for w in range(6):
        oku, okd, a = o.seeded_start(seed, w, ham.U_up, ham.U_down)
        assert ku[w].tolist() == oku.tolist() and kd[w].tolist() == okd.tolist()
        assert att[w] == a + 1
    assert np.all(ct == 0)
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_apply_moves_match_oracle(kv, precision):
    """update_configurations! with update_W! (src/MonteCarlo.jl:497-511, 279-292)."""
    N = 54
    ham = ham_for(kv, N)
    U = ham.U_up
    ku, kd, _ = o.seeded_start(5, 0, U, U)
    st = o.ChainState(ku.copy(), kd.copy(), o.reevaluateW(U, ku), o.reevaluateW(U, kd))
    eng = kv.Engine(ham, 1, precision=precision)
    eng.init(ku, kd)
    rng = np.random.default_rng(0)
    nn = ham.nn
    for step in range(6):
        while True:   # an exchange whose target configuration is not near-singular
            i, site = nn[rng.integers(len(nn))]
            f1 = st.kappa_up[i] != 0 and st.kappa_down[site] != 0
            f2 = st.kappa_up[site] != 0 and st.kappa_down[i] != 0
            if not (f1 or f2):
                continue
            flag = 1 if f1 else 2
            l_up = int(st.kappa_up[i] if flag == 1 else st.kappa_up[site])
            l_dn = int(st.kappa_down[site] if flag == 1 else st.kappa_down[i])
            Ku, Kd = (site, i) if flag == 1 else (i, site)
            if abs(st.W_up[Ku, l_up - 1]) > 0.05 and abs(st.W_down[Kd, l_dn - 1]) > 0.05:
                break
        o.update_configurations(st, flag, i + 1, site + 1, l_up, l_dn)
        eng.apply_moves([flag, i, site, l_up, l_dn])
    gku, gkd, _ = eng.get_state()
    assert gku[0].tolist() == st.kappa_up.tolist() and gkd[0].tolist() == st.kappa_down.tolist()
    Wu, Wd = eng.get_w()
    tol = 1e-9 if precision == "plain" else 1e-4
    assert close(Wu[0], st.W_up, tol) and close(Wd[0], st.W_down, tol)
    eng.close()


def test_invalid_and_singular_configurations(kv):
    ham = ham_for(kv, 24)
    eng = kv.Engine(ham, 1)
    ku, kd, _ = o.seeded_start(1, 0, ham.U_up, ham.U_down)
    bad = kd.copy()
    bad[np.argmax(ku > 0)] = 5   # doubly occupied
    with pytest.raises(kv.ArgumentError):
        eng.init(ku, bad)
    bad = ku.copy()
    bad[np.argmax(ku > 0)] = 99
    with pytest.raises(kv.BoundsError):
        eng.init(bad, kd)
    eng.close()
    # identical rows make every tilde_U singular (test/test-MonteCarlo.jl:429-477)
    rng = np.random.default_rng(3)
    Us = np.repeat(rng.random((1, 12)), 24, axis=0)
    sing = kv.Hamiltonian(12, 12, Us, rng.random((24, 12)), ham.H_mat, ham.nn)
    eng = kv.Engine(sing, 1)
    with pytest.raises(kv.SingularException):
        eng.init(ku, kd)
    eng.close()


def test_set_state_rejects_a_bad_walker_and_keeps_every_state(kv):
    """The labels of set_state are checked on the device: an invalid walker
    among valid ones fails the call, the error names the first invalid
    walker and its site, and no walker's configuration or counter changes,
    not even one whose new labels were valid."""
    ham = ham_for(kv, 96)
    walkers = 9
    eng = kv.Engine(ham, walkers)
    eng.init()
    eng.advance(16)
    ku0, kd0, ct0 = eng.get_state()
    ku, kd = ku0.copy(), kd0.copy()
    a, b = int(np.argmax(ku[0] > 0)), int(np.argmax(kd[0] > 0))   # walker 0: a valid exchange
    ku[0, a], kd[0, a], ku[0, b], kd[0, b] = 0, kd0[0, b], ku0[0, a], 0
    s5 = int(np.argmax(ku[5] > 0))
    kd[5, s5] = 1                                                   # walker 5: doubly occupied
    ku[7, int(np.argmax(ku[7] > 0))] = 999                          # walker 7: label out of range
    with pytest.raises(kv.ArgumentError, match=f"walker 5 site {s5} is doubly occupied"):
        eng.set_state(ku, kd, ct0)
    ku[5], kd[5] = ku0[5], kd0[5]
    with pytest.raises(kv.BoundsError, match="walker 7 site"):
        eng.set_state(ku, kd, ct0)
    ku1, kd1, ct1 = eng.get_state()
    assert np.array_equal(ku1, ku0) and np.array_equal(kd1, kd0) and np.array_equal(ct1, ct0)
    ku[7] = ku0[7]
    eng.set_state(ku, kd, ct0)                                      # only walker 0 changed
    ku2, kd2, _ = eng.get_state()
    assert np.array_equal(ku2, ku) and np.array_equal(kd2, kd)
    eng.close()


def test_carlo_callbacks_and_checkpoint(kv):
    params = dict(n1=4, n2=2, PBC=(True, True), antiPBC=(False, True), N_up=12, N_down=12, walkers=8,
                  precision="mixed", proposals_per_sweep=12, seed=3)
    mc = kv.MC(params)
    ctx = kv.MCContext()
    kv.init_(mc, ctx, params)
    for _ in range(20):
        kv.sweep_(mc, ctx)
        ctx.sweeps += 1
        kv.measure_(mc, ctx)
    ev = kv.Evaluator()
    kv.register_evaluables(kv.MC, ev, params)
    res = ev.run(ctx.observables)
    assert np.isfinite(res["energy"]) and -1.0 < res["energy"] < 0.0
    assert len(ctx.observables["acc"]) == 20 and len(ctx.observables["OL"]) == 20
    ck = {}
    kv.write_checkpoint(mc, ck)
    mc2 = kv.MC(params)
    kv.read_checkpoint_(mc2, ck)
    a, b = mc.engine.get_state(), mc2.engine.get_state()
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    np.testing.assert_allclose(mc.engine.measure(), mc2.engine.measure(), rtol=1e-5, atol=1e-5)
    mc.engine.sweep(200)
    mc2.engine.sweep(200)
    a, b = mc.engine.get_state(), mc2.engine.get_state()
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_qr_start_singular_message(kv):
    """The reference's singular-start error (src/MonteCarlo.jl:401-408) through the product."""
    params = dict(n1=2, n2=2, PBC=(False, False), N_up=6, N_down=6, walkers=1)
    mc = kv.MC(params)
    rng = np.random.default_rng(3)
    Us = np.repeat(rng.random((1, 6)), 12, axis=0)
    mc.Ham = kv.Hamiltonian(6, 6, Us, rng.random((12, 6)), mc.Ham.H_mat, mc.Ham.nn)
    mc.engine = kv.Engine(mc.Ham, 1)
    with pytest.raises(RuntimeError, match="QR-based configuration is singular"):
        kv.init_(mc, kv.MCContext(), params)


@pytest.mark.parametrize("precision", ["plain", "mixed"])
@pytest.mark.parametrize("accept,key", [("reference", "E_per_site_reference_rule"), ("metropolis", "E_per_site_psi2")])
def test_energy_matches_exact_enumeration(kv, golden, precision, accept, key):
    """N=24: E/N within 2 standard errors of the exact value for the rule's stationary law."""
    ham = ham_for(kv, 24)
    walkers = 2048
    eng = kv.Engine(ham, walkers, precision=precision, accept=accept, seed=99)
    eng.init()
    eng.sweep(600)
    eng.reset_stats()
    eng.sweep(3600)
    ws = eng.walker_stats()
    m = ws["sum_e"] / ws["n_meas"]
    e = m.mean() / 24
    se = m.std(ddof=1) / np.sqrt(walkers) / 24
    exact = golden["enum_N24"][key]
    assert abs(e - exact) <= 2 * se, (e, exact, se)
    eng.close()


def test_mixed_vs_plain_energy_gate(kv):
    """|dE/N| <= 1e-4 between the two forms on identical walkers and proposal
    streams, over every walker: the paired difference of the per-walker mean
    energies satisfies |mean| + 2 se <= 1e-4 per site."""
    ham = ham_for(kv, 96)
    walkers, seed = 256, 5
    out = {}
    for precision in ("plain", "mixed"):
        eng = kv.Engine(ham, walkers, precision=precision, seed=seed, refresh_interval=(256 if precision == "mixed" else 0))
        eng.init()
        eng.sweep(2400)
        ws = eng.walker_stats()
        out[precision] = (ws["sum_e"].copy(), ws["n_meas"].copy(), eng.get_state())
        eng.close()
    (ep, npm, sp), (em, nmm, sm) = out["plain"], out["mixed"]
    same = np.array([np.array_equal(sp[0][w], sm[0][w]) for w in range(walkers)])
    assert same.mean() > 0.95
    d = (em / nmm - ep / npm) / 96
    assert abs(d.mean()) + 2 * d.std(ddof=1) / np.sqrt(walkers) <= 1e-4, (d.mean(), d.std())


@pytest.mark.parametrize("delay_k", [1, 12])
def test_n216_mixed_chain_matches_c_oracle(kv, delay_k):
    """The headline size: FP32 W on chip (delayed depth 12 fits next to it)."""
    N, walkers, proposals, seed = 216, 8, 2000, 31
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=128, delay_k=delay_k)
    cfg = eng.config()
    assert cfg["w_on_chip"] and cfg["delay_k"] == delay_k
    eng.init()
    ku0, kd0, _ = eng.get_state()
    eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, 108, 108, 0)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= 1e-4 * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - 1
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_advance_makes_exactly_the_asked_moves(kv, precision):
    """kvmc_advance: every walker makes exactly A more accepted moves; the chain is the oracle's."""
    N, walkers, seed, A = 54, 10, 17, 60
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision=precision, seed=seed, refresh_interval=(32 if precision == "mixed" else 0))
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.advance(A)
    ku1, kd1, ct = eng.get_state()
    ws = eng.walker_stats()
    assert np.all(ws["accepted"] == A) and st["accepted"] == walkers * A
    assert np.all(ws["proposals"] == ct)
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, int(ct[w]), 27, 27)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == A
    assert match >= walkers - (0 if precision == "plain" else 1)
    eng.close()


def test_severe_drift_refreshes_at_once_within_the_call(kv):
    """The severe branch of the drift trigger: with the severe threshold set
    to the tolerance itself, every check past the tolerance refreshes the
    walker at once, so each walker is refreshed several times inside one
    call; the move counts stay exact and the chains stay the oracle's."""
    N, walkers, seed, A = 96, 8, 29, 200
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=1024, delay_k=8, w_placement="hbm")
    eng.set_drift_tolerance(1e-12)
    eng.set_drift_severe(1)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.advance(A)
    assert st["accepted"] == walkers * A
    # checks on every fourth flush of 8 moves: about A / 32 per walker
    assert st["refreshes"] >= 3 * walkers, st["refreshes"]
    ku1, kd1, ct = eng.get_state()
    ws = eng.walker_stats()
    assert np.all(ws["accepted"] == A)
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, int(ct[w]), N // 2, N // 2)
        match += int(np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]))
    assert match >= walkers - 1
    with pytest.raises(kv.KvmcError):
        eng.set_drift_severe(-1)
    eng.close()


def test_drift_triggered_refresh_waits_for_the_end_of_the_call(kv):
    """A drift tolerance every check exceeds: within a kvmc_advance call whose
    moves fit in the refresh interval the walkers do not stop, each is
    refreshed once at the end of the call, the move counts are exact and the
    chains are still the oracle's."""
    N, walkers, seed, A = 96, 8, 29, 200
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=1024, delay_k=8, w_placement="hbm")
    eng.set_drift_tolerance(1e-12)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    for call in range(3):
        st = eng.advance(A)
        assert st["accepted"] == walkers * A
        # one refresh per walker (and an FP64 redo of a walker the FP32 refresh
        # flags, should there be one); a refresh at the trigger would give one
        # per checked flush, several per call
        assert walkers <= st["refreshes"] <= walkers + walkers // 4, (call, st["refreshes"])
    ku1, kd1, ct = eng.get_state()
    ws = eng.walker_stats()
    assert np.all(ws["accepted"] == 3 * A)
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, int(ct[w]), N // 2, N // 2)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
    assert match >= walkers - 1
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_advance_stops_a_walker_that_cannot_move(kv, precision):
    """Four sites, one bond (0, 1).  Walker 0 holds both up spins on the bond:
    Z_mu = 0, every proposal is rejected, and kvmc_advance stops it after its
    allowance of 65536 proposals per requested move with an error; walker 1
    (opposite spins on the bond) makes its moves."""
    rng = np.random.default_rng(4)
    U = rng.normal(size=(4, 2))
    H = np.zeros((4, 4))
    H[0, 1] = H[1, 0] = -1.0
    ham = kv.Hamiltonian(2, 2, U, U.copy(), H, [(0, 1)])
    eng = kv.Engine(ham, 2, precision=precision, seed=1, refresh_interval=64, measure_interval=64)
    eng.init(np.array([[1, 2, 0, 0], [1, 0, 2, 0]]), np.array([[0, 0, 1, 2], [0, 1, 0, 2]]))
    with pytest.raises(kv.KvmcError, match="fewer than 3 accepted moves"):
        eng.advance(3)
    ws = eng.walker_stats()
    assert ws["accepted"][0] == 0 and ws["proposals"][0] == 3 * 65536
    assert ws["accepted"][1] == 3
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_unequal_spin_counts(kv, precision):
    """N_up != N_down (src/MonteCarlo.jl:165-185 takes both): two W widths."""
    N, n_up, seed, walkers, proposals = 54, 30, 23, 8, 1500
    lat = kv.DoubleKagome(1.0, 6, 3, (True, True), (False, True))
    H = kv.Hmat(lat)
    Uu, Ud = kv.orbitals(H, n_up, N - n_up)
    ham = kv.Hamiltonian(n_up, N - n_up, Uu, Ud, H, kv.get_nn(H))
    eng = kv.Engine(ham, walkers, precision=precision, seed=seed)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    assert np.all((ku0 != 0).sum(1) == n_up) and np.all((kd0 != 0).sum(1) == N - n_up)
    eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(Uu, Ud, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, 24, 24)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            tol = 1e-8 if precision == "plain" else 1e-4
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= tol * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - (0 if precision == "plain" else 1)
    Wu, Wd = eng.get_w()
    assert Wu.shape[2] == n_up and Wd.shape[2] == N - n_up
    eng.close()


def test_custom_link_tables(kv):
    """Zero-flux links (all amplitudes +1, as scripts/zero_flux.jl builds) through the whole path."""
    lin = {k: 1.0 for k in kv.PI_LINK_IN}
    lint = {k: 1.0 for k in kv.PI_LINK_INTER}
    lat = kv.DoubleKagome(1.0, 6, 3, (True, True), (False, True))
    Lo = o.double_kagome(1.0, 6, 3, (True, True), (False, True))
    H = kv.Hmat(lat, lin, lint)
    assert np.array_equal(H, o.hmat(Lo, lin, lint))
    Uu, Ud = kv.orbitals(H, 27, 27)
    ham = kv.Hamiltonian(27, 27, Uu, Ud, H, kv.get_nn(H))
    seed, walkers, proposals = 29, 6, 1200
    eng = kv.Engine(ham, walkers, precision="plain", seed=seed)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    m = oracle_c.OracleModel(Uu, Ud, ham.nn)
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, 27, 27)
        assert np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w])
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_large_lattice_chain(kv, precision):
    """N=384 (8x8 doubled cells): blocked-LU refresh and W streamed from HBM."""
    N, walkers, proposals, seed = 384, 4, 800, 41
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision=precision, seed=seed, refresh_interval=(64 if precision == "mixed" else 0))
    assert not eng.config()["w_on_chip"]
    eng.init()
    ku0, kd0, _ = eng.get_state()
    eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, 192, 192)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            tol = 1e-8 if precision == "plain" else 1e-4
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= tol * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - (0 if precision == "plain" else 1)
    eng.close()


@pytest.mark.parametrize("N,delay_k", [(96, 4), (96, 16), (216, 12), (216, 16)])
def test_hbm_streaming_chains_match_c_oracle(kv, N, delay_k):
    """Mixed form with W kept in HBM and only the delayed factors on chip."""
    walkers, proposals, seed = 8, 2000, 37
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=128, delay_k=delay_k,
                    w_placement="hbm")
    cfg = eng.config()
    assert not cfg["w_on_chip"] and cfg["delay_k"] == delay_k
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, N // 2, N // 2, 0)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= 1e-4 * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - 1
    assert st["bad_walkers"] == 0
    # the state left in HBM is the W of the final configuration
    Wu, Wd = eng.get_w()
    for w in range(walkers):
        assert close(Wu[w], o.reevaluateW(ham.U_up, ku1[w]), 1e-3)
    eng.close()


def test_placement_on_chip_is_refused_when_w_does_not_fit(kv):
    ham = ham_for(kv, 384)
    with pytest.raises(kv.KvmcError):
        kv.Engine(ham, 2, precision="mixed", w_placement="chip")


@pytest.mark.parametrize("N,delay_k,placement", [(96, 4, "chip"), (96, 16, "chip"), (96, 8, "hbm"), (216, 12, "hbm"),
                                                 (216, 12, "chip"), (384, 8, "hbm")])
def test_pipelined_scan_chains_match_c_oracle(kv, N, delay_k, placement):
    """The scan for the next move overlapping the factor-column write of the last one."""
    walkers, proposals, seed = 8, 2400, 53
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=96, delay_k=delay_k,
                    w_placement=placement)
    eng.set_pipeline(True)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, N // 2, N // 2, 0)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            assert ws["n_meas"][w] == proposals // (N // 2)
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= 1e-4 * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - 1
    assert st["bad_walkers"] == 0
    Wu, Wd = eng.get_w()
    for w in range(walkers):
        assert close(Wu[w], o.reevaluateW(ham.U_up, ku1[w]), 1e-3)
    # advance: exact move counts with the pipelined scan
    st = eng.advance(77)
    assert np.all(eng.walker_stats()["accepted"] == ws["accepted"] + 77)
    eng.close()


@pytest.mark.parametrize("N,delay_k,threads", [(96, 8, 256), (96, 16, 128), (216, 12, 256), (216, 4, 256),
                                               (384, 8, 256)])
def test_tensor_core_flush_chains_match_c_oracle(kv, N, delay_k, threads):
    """W in HBM with the rank-k flush on the tensor cores (tcgen05, 3xTF32)."""
    walkers, proposals, seed = 8, 2400, 59
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=96, delay_k=delay_k,
                    w_placement="hbm")
    eng.set_stream_threads(threads)
    eng.set_tc_flush(True)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, N // 2, N // 2, 0)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= 1e-4 * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - 1
    assert st["bad_walkers"] == 0
    Wu, Wd = eng.get_w()
    for w in range(walkers):
        assert close(Wu[w], o.reevaluateW(ham.U_up, ku1[w]), 1e-3)
        assert close(Wd[w], o.reevaluateW(ham.U_down, kd1[w]), 1e-3)
    eng.close()


def test_tensor_core_flush_refused_off_its_path(kv):
    ham = ham_for(kv, 96)
    eng = kv.Engine(ham, 2, precision="mixed", delay_k=8, w_placement="chip")
    with pytest.raises(kv.KvmcError):
        eng.set_tc_flush(True)
    eng.close()


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("N,placement", [(96, "hbm"), (216, "hbm"), (216, "chip"), (384, "hbm"), (864, "hbm")])
def test_fp32_refinement_refresh(kv, N, placement, mode):
    """The periodic refresh by FP32 iterative refinement, one thread per row (1),
    in tiles of 32 rows (2), or tiled with the residual on the tensor cores (3):
    W right after it within 5e-6 of the FP64 rebuild (relative to max(1, |W|)),
    and chains that follow the oracle.  The tiled forms converge on their own:
    at most a quarter of their refreshes are redone in FP64."""
    walkers, seed, R = (8, 61, 64) if N < 864 else (4, 61, 32)
    ham = ham_for(kv, N)
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=R, w_placement=placement)
    eng.set_refresh32(mode)
    eng.set_drift_tolerance(1e9)        # no early refreshes: every walker refreshes exactly every R moves
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.advance(2 * R)             # ends right after a refresh of every walker
    assert st["refreshes"] >= 2 * walkers and st["bad_walkers"] == 0
    if mode >= 2:
        assert 4 * st["fp64_redos"] <= st["refreshes"], st
    ku1, kd1, ct = eng.get_state()
    Wu, Wd = eng.get_w()
    for w in range(walkers):
        assert close(Wu[w], o.reevaluateW(ham.U_up, ku1[w]), 5e-6), w
        assert close(Wd[w], o.reevaluateW(ham.U_down, kd1[w]), 5e-6), w
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, int(ct[w]), N // 2, N // 2, 0)
        match += int(np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]))
    assert match >= walkers - 1
    eng.close()


def test_tensor_core_refresh_ragged_large(kv):
    """The refresh on the tensor cores at N = 576 with 290 + 286 orbitals:
    partial 64-column tiles in the residual, two 160-column tiles in the
    correction, 128-row groups cut at 286 and 290 rows, and unequal spins.
    W right after a refresh of every walker against the oracle's FP64
    reevaluateW (5e-6 relative to max(1, |W|)), the chains against the
    oracle, and no more than a quarter of the refreshes redone in FP64."""
    lat = kv.DoubleKagome(1.0, 16, 12, (True, True), (False, True))
    H = kv.Hmat(lat)
    N = H.shape[0]
    assert N == 576
    Uu, Ud = kv.orbitals(H, 290, N - 290)
    ham = kv.Hamiltonian(290, N - 290, Uu, Ud, H, kv.get_nn(H))
    walkers, seed, R = 4, 23, 48
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=R, w_placement="hbm")
    eng.set_refresh32("tc")
    eng.set_drift_tolerance(1e9)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.advance(2 * R)
    assert st["refreshes"] >= 2 * walkers and st["bad_walkers"] == 0
    assert 4 * st["fp64_redos"] <= st["refreshes"], st
    ku1, kd1, ct = eng.get_state()
    Wu, Wd = eng.get_w()
    for w in range(walkers):
        assert close(Wu[w], o.reevaluateW(Uu, ku1[w]), 5e-6), w
        assert close(Wd[w], o.reevaluateW(Ud, kd1[w]), 5e-6), w
    m = oracle_c.OracleModel(Uu, Ud, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, int(ct[w]), N - 290, N - 290, 0)
        match += int(np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]))
    assert match >= walkers - 1
    eng.close()


@pytest.mark.parametrize("mode", ["tiled", "tc"])
@pytest.mark.parametrize("n1,n2,n_up", [(10, 5, 75), (10, 5, 77), (6, 3, 30), (4, 2, 12)])
def test_tiled_refresh_ragged_sizes(kv, n1, n2, n_up, mode):
    """The tiled FP32 refresh where neither spin's orbital count nor the other
    spin's row count is a multiple of 4 or 32 (N = 150 with 75 + 75 and
    77 + 73 orbitals, N = 54 with 30 + 24, N = 24): W after a refresh of every
    walker against the FP64 rebuild, and the chains against the oracle."""
    lat = kv.DoubleKagome(1.0, n1, n2, (True, True), (False, True))
    H = kv.Hmat(lat)
    N = H.shape[0]
    Uu, Ud = kv.orbitals(H, n_up, N - n_up)
    ham = kv.Hamiltonian(n_up, N - n_up, Uu, Ud, H, kv.get_nn(H))
    walkers, seed, R = 6, 17, 48
    eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=R, w_placement="hbm")
    eng.set_refresh32(mode)
    eng.set_drift_tolerance(1e9)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.advance(2 * R)
    assert st["refreshes"] >= 2 * walkers and st["bad_walkers"] == 0
    ku1, kd1, ct = eng.get_state()
    Wu, Wd = eng.get_w()
    for w in range(walkers):
        assert close(Wu[w], o.reevaluateW(Uu, ku1[w]), 5e-6), w
        assert close(Wd[w], o.reevaluateW(Ud, kd1[w]), 5e-6), w
    m = oracle_c.OracleModel(Uu, Ud, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, int(ct[w]), min(n_up, N - n_up), min(n_up, N - n_up), 0)
        match += int(np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]))
    assert match >= walkers - 1
    eng.close()


@pytest.mark.parametrize("N,ctas", [(96, 2), (216, 2), (216, 4), (384, 4)])
def test_cluster_sweep_matches_oracle_and_the_one_cta_kernel(kv, N, ctas):
    """W split over a thread-block cluster (rows by site blocks in each CTA's
    shared memory, read by the others over DSMEM), rank-1 updates: chains
    against the oracle, and against the one-CTA rank-1 kernel on the same
    walkers, which does the same FP32 operations (identical chains, energy
    sums within 1e-5: only the order of the energy reduction differs)."""
    walkers, proposals, seed = 8, 2000, 37
    ham = ham_for(kv, N)
    out = []
    for ct in (0, ctas):
        eng = kv.Engine(ham, walkers, precision="mixed", seed=seed, refresh_interval=96, delay_k=1,
                        w_placement="hbm")
        if ct:
            eng.set_cluster(ct)
        eng.init()
        ku0, kd0, _ = eng.get_state()
        st = eng.sweep(proposals)
        assert st["bad_walkers"] == 0
        ku1, kd1, ct_ = eng.get_state()
        ws = eng.walker_stats()
        Wu, Wd = eng.get_w()
        out.append((ku0, kd0, ku1, kd1, ws["sum_e"].copy(), ws["accepted"].copy(), Wu, Wd))
        eng.close()
    (a0, b0, a1, b1, e0, n0, _, _), (c0, d0, c1, d1, e1, n1, Wu, Wd) = out
    assert np.array_equal(a1, c1) and np.array_equal(b1, d1) and np.array_equal(n0, n1)
    assert np.all(np.abs(e0 - e1) <= 1e-5 * np.maximum(1.0, np.abs(e0)))
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(c0[w], d0[w])
        ch.run(seed, w, proposals, N // 2, N // 2, 0)
        match += int(np.array_equal(ch.ku, c1[w]) and np.array_equal(ch.kd, d1[w]))
    assert match >= walkers - 1
    for w in range(walkers):
        assert close(Wu[w], o.reevaluateW(ham.U_up, c1[w]), 1e-3), w
        assert close(Wd[w], o.reevaluateW(ham.U_down, d1[w]), 1e-3), w


def test_cluster_sweep_refused_off_its_path(kv):
    ham = ham_for(kv, 96)
    eng = kv.Engine(ham, 2, precision="mixed", delay_k=8, w_placement="hbm")
    with pytest.raises(kv.KvmcError):
        eng.set_cluster(4)
    eng.close()
    eng = kv.Engine(ham, 2, precision="mixed", delay_k=1, w_placement="hbm")
    with pytest.raises(kv.KvmcError):
        eng.set_cluster(3)
    eng.close()
