"""GPU parity for complex orbitals (B != 0): libkvmc through its C ABI against
the numpy oracle and the complex C oracle.

The field workloads follow scripts/LL.jl:11-25: B = imbalance * pi / S with
S = n1 * n2 * 2 sqrt(3), N_up = N/2 + imbalance/2, N_down = N/2 - imbalance/2.

Tolerances, as for the real path:
  plain FP64 form: W, ratios, local energies within 1e-10 relative to
  max(1, |W|); chains follow the oracle's trajectory exactly.
  mixed FP32 form: W within 1e-6 relative after a refresh, ratios and local
  energies within 1e-5; at most one walker of a batch may leave the oracle's
  trajectory (an FP32 rounding flipping a decision within ~1e-6 of its
  threshold).
"""
import math

import numpy as np
import pytest

import kagome_oracle as o
import oracle_c

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def kv(built):
    import kagomevmc

    return kagomevmc


def field_ham(kv, n1, n2, imbalance):
    lat = kv.DoubleKagome(1.0, n1, n2, (True, True), (False, True))
    B = imbalance * math.pi / (n1 * n2 * 2 * math.sqrt(3))
    H = kv.Hmat(lat, B=B)
    N = H.shape[0]
    n_up, n_dn = N // 2 + imbalance // 2, N // 2 - imbalance // 2
    Uu, Ud = kv.orbitals(H, n_up, n_dn)
    assert np.iscomplexobj(Uu) and np.abs(Uu.imag).max() > 1e-3
    return kv.Hamiltonian(n_up, n_dn, Uu, Ud, H, kv.get_nn(H))


def close(a, b, rel):
    a, b = np.asarray(a), np.asarray(b)
    return np.all(np.abs(a - b) <= rel * max(1.0, np.abs(b).max()))


@pytest.mark.parametrize("precision", ["plain", "mixed"])
@pytest.mark.parametrize("cells", [(6, 3, 2), (8, 4, 4), (8, 8, 4), (8, 10, 4), (12, 10, 2)])
def test_complex_refresh_matches_oracle(kv, cells, precision):
    """W = U tilde_U^{-1} in complex FP64 (N = 54, 96, 192; and N = 240, 360
    with 122 and 181 orbitals, where tilde_U is factorised in HBM)."""
    ham = field_ham(kv, *cells)
    nw = 4
    starts = [o.seeded_start(13, w, ham.U_up, ham.U_down)[:2] for w in range(nw)]
    eng = kv.Engine(ham, nw, precision=precision, seed=13)
    assert eng.complex
    eng.init(np.stack([s[0] for s in starts]), np.stack([s[1] for s in starts]))
    Wu, Wd = eng.get_w()
    assert Wu.dtype == np.complex128
    tol = 1e-10 if precision == "plain" else 1e-6
    for w, (ku, kd) in enumerate(starts):
        assert close(Wu[w], o.reevaluateW(ham.U_up, ku), tol), (cells, w)
        assert close(Wd[w], o.reevaluateW(ham.U_down, kd), tol), (cells, w)
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_complex_ratios_and_local_energy(kv, precision):
    """Ratios W_up[K,l] W_down[K',l'] and E_L = Re getOL (src/Hamiltonian.jl:762-778)."""
    ham = field_ham(kv, 8, 4, 4)
    oh = o.Hamiltonian(ham.N_up, ham.N_down, ham.U_up, ham.U_down, ham.H_mat, [(i + 1, j + 1) for i, j in ham.nn])
    nw = 5
    starts = [o.seeded_start(8, w, ham.U_up, ham.U_down)[:2] for w in range(nw)]
    eng = kv.Engine(ham, nw, precision=precision)
    eng.init(np.stack([s[0] for s in starts]), np.stack([s[1] for s in starts]))
    E = eng.measure()
    tol = 1e-10 if precision == "plain" else 1e-5
    rng = np.random.default_rng(2)
    N = ham.U_up.shape[0]
    moves = np.zeros((nw, 16, 4), dtype=np.int32)
    want = np.zeros((nw, 16), dtype=complex)
    for w, (ku, kd) in enumerate(starts):
        Wu, Wd = o.reevaluateW(ham.U_up, ku), o.reevaluateW(ham.U_down, kd)
        e = o.getOL(oh, Wu, Wd, ku, kd)
        assert abs(E[w] - e) <= tol * max(1.0, abs(e)), (w, E[w], e)
        for k in range(16):
            Ku, Kd = rng.integers(N), rng.integers(N)
            lu, ld = rng.integers(1, ham.N_up + 1), rng.integers(1, ham.N_down + 1)
            moves[w, k] = (Ku, lu, Kd, ld)
            want[w, k] = Wu[Ku, lu - 1] * Wd[Kd, ld - 1]
    R = eng.eval_ratios(moves)
    assert R.dtype == np.complex128
    assert np.all(np.abs(R - want) <= tol * np.maximum(1.0, np.abs(want)))
    eng.close()


@pytest.mark.parametrize("precision,delay_k,pipeline", [("plain", 0, True), ("mixed", 1, True), ("mixed", 4, True),
                                                     ("mixed", 8, True), ("mixed", 8, False)])
@pytest.mark.parametrize("accept", ["reference", "metropolis"])
def test_complex_chains_match_c_oracle(kv, precision, delay_k, pipeline, accept):
    """Delayed depths 4 and 8 run the pipelined complex kernel (scan overlapping
    the factor-column write) unless the pipeline is switched off."""
    n1, n2, imbalance = 8, 4, 4
    ham = field_ham(kv, n1, n2, imbalance)
    walkers, proposals, seed = 10, 3000, 19
    eng = kv.Engine(ham, walkers, precision=precision, accept=accept, seed=seed,
                    refresh_interval=(64 if precision == "mixed" else 0), delay_k=delay_k)
    if precision == "mixed":
        assert eng.config()["delay_k"] == delay_k
        eng.set_pipeline(pipeline)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    for w in range(walkers):   # the seeded starts are the oracle's
        oku, okd, _ = o.seeded_start(seed, w, ham.U_up, ham.U_down)
        assert ku0[w].tolist() == oku.tolist() and kd0[w].tolist() == okd.tolist()
    st = eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn, "cplx")
    rule = 0 if accept == "reference" else 1
    n_occ = min(ham.N_up, ham.N_down)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, n_occ, n_occ, rule)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            tol = 1e-8 if precision == "plain" else 1e-4
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= tol * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - (0 if precision == "plain" else 1)
    assert st["bad_walkers"] == 0 and st["accepted"] > 0
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_complex_lattice_of_the_field_scan(kv, precision):
    """8x8 cells, N = 192, imbalance 4 (N_up 98, N_down 94): one point of the field scan."""
    ham = field_ham(kv, 8, 8, 4)
    walkers, proposals, seed = 4, 1200, 43
    eng = kv.Engine(ham, walkers, precision=precision, seed=seed, refresh_interval=(64 if precision == "mixed" else 0))
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.sweep(proposals)
    assert st["bad_walkers"] == 0
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn, "cplx")
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, 94, 94)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            tol = 1e-8 if precision == "plain" else 1e-4
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= tol * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - (0 if precision == "plain" else 1)
    eng.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_complex_apply_moves_match_oracle(kv, precision):
    """update_configurations! with the complex update_W! (src/MonteCarlo.jl:497-511, 279-292)."""
    ham = field_ham(kv, 6, 3, 2)
    ku, kd, _ = o.seeded_start(5, 0, ham.U_up, ham.U_down)
    st = o.ChainState(ku.copy(), kd.copy(), o.reevaluateW(ham.U_up, ku), o.reevaluateW(ham.U_down, kd))
    eng = kv.Engine(ham, 1, precision=precision)
    eng.init(ku, kd)
    rng = np.random.default_rng(0)
    nn = ham.nn
    for _ in range(6):
        while True:
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


def test_complex_handle_at_zero_field_equals_real_handle(kv):
    """Real orbitals passed with a zero imaginary part take the complex kernels
    and make the same moves as the real kernels."""
    lat = kv.DoubleKagome(1.0, 8, 4, (True, True), (False, True))
    H = kv.Hmat(lat)
    Uu, Ud = kv.orbitals(H, 48, 48)
    real = kv.Hamiltonian(48, 48, Uu, Ud, H, kv.get_nn(H))
    cplx = kv.Hamiltonian(48, 48, Uu.astype(complex), Ud.astype(complex), H, kv.get_nn(H))
    out = []
    for ham in (real, cplx):
        eng = kv.Engine(ham, 8, precision="plain", seed=3)
        eng.init()
        eng.sweep(1500)
        out.append((eng.get_state(), eng.walker_stats()))
        eng.close()
    (sa, wa), (sb, wb) = out
    assert all(np.array_equal(x, y) for x, y in zip(sa, sb))
    assert np.array_equal(wa["accepted"], wb["accepted"])
    np.testing.assert_allclose(wa["sum_e"], wb["sum_e"], rtol=1e-9, atol=1e-9)


def test_complex_delay_depths(kv):
    """Complex W takes rank-1 or delayed updates of depth 4 or 8 (W in HBM); 8 by default."""
    ham = field_ham(kv, 6, 3, 2)
    with pytest.raises(kv.KvmcError):
        kv.Engine(ham, 2, precision="mixed", delay_k=12)
    eng = kv.Engine(ham, 2, precision="mixed", delay_k=0)
    assert eng.config()["delay_k"] == 8 and not eng.config()["w_on_chip"]
    eng.close()


@pytest.mark.parametrize("precision,delay_k", [("plain", 0), ("mixed", 4)])
def test_complex_chains_beyond_the_shared_memory_refresh(kv, precision, delay_k):
    """N = 240 in a field (122 + 118 orbitals, more than the 112 the
    shared-memory complex refresh holds): chains against the complex C
    oracle, with the blocked HBM refresh every 64 accepted moves (mixed) or
    every n proposals (plain)."""
    ham = field_ham(kv, 8, 10, 4)
    walkers, proposals, seed = 6, 1500, 29
    eng = kv.Engine(ham, walkers, precision=precision, seed=seed,
                    refresh_interval=(64 if precision == "mixed" else 0), delay_k=delay_k)
    eng.init()
    ku0, kd0, _ = eng.get_state()
    st = eng.sweep(proposals)
    ku1, kd1, _ = eng.get_state()
    ws = eng.walker_stats()
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, ham.nn, "cplx")
    n_occ = min(ham.N_up, ham.N_down)
    match = 0
    for w in range(walkers):
        ch = m.new_chain(ku0[w], kd0[w])
        ch.run(seed, w, proposals, n_occ, n_occ, 0)
        if np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]):
            match += 1
            assert ch.c.accepted == ws["accepted"][w]
            tol = 1e-8 if precision == "plain" else 1e-4
            assert abs(ch.c.sum_e - ws["sum_e"][w]) <= tol * max(1.0, abs(ch.c.sum_e))
    assert match >= walkers - (0 if precision == "plain" else 1)
    assert st["bad_walkers"] == 0 and st["accepted"] > 0
    Wu, Wd = eng.get_w()
    tol = 1e-8 if precision == "plain" else 1e-3
    for w in range(walkers):
        assert close(Wu[w], o.reevaluateW(ham.U_up, ku1[w]), tol), w
        assert close(Wd[w], o.reevaluateW(ham.U_down, kd1[w]), tol), w
    eng.close()
