"""The C oracle against the numpy oracle and the golden fixtures (no GPU)."""
import json
import os

import numpy as np
import pytest

import kagome_oracle as o
import oracle_c

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def golden():
    return json.load(open(os.path.join(GOLD, "golden.json")))


def model(N):
    a, b = {24: (2, 2), 54: (3, 3), 96: (4, 4), 216: (6, 6)}[N]
    ham = o.hamiltonian(N // 2, N // 2, o.double_kagome(1.0, 2 * a, b, (True, True), (False, True)))
    U = np.load(os.path.join(GOLD, "u_N24.npy")) if N == 24 else ham.U_up.real.copy()
    return ham, U


@pytest.mark.parametrize("N", [24, 54, 96])
def test_configs_match_golden(golden, N):
    ham, U = model(N)
    for case in golden["configs"][str(N)]:
        ku, kd = np.array(case["kappa_up"]), np.array(case["kappa_down"])
        Wu, Wd = o.reevaluateW(U, ku), o.reevaluateW(U, kd)
        assert o.getOL(ham, Wu, Wd, ku, kd) == pytest.approx(case["local_energy"], rel=1e-10, abs=1e-10)
        for mv, r in zip(case["moves"], case["ratios"]):
            assert Wu[mv[0], mv[1] - 1] * Wd[mv[2], mv[3] - 1] == pytest.approx(r, rel=1e-9, abs=1e-12)
        # C oracle refresh and energy
        m = oracle_c.OracleModel(U, U, [(i - 1, j - 1) for i, j in ham.nn])
        ch = m.new_chain(ku, kd)
        assert np.abs(ch.Wu - Wu).max() <= 1e-10 * max(1.0, np.abs(Wu).max())
        assert ch.local_energy() == pytest.approx(case["local_energy"], rel=1e-10, abs=1e-10)


@pytest.mark.parametrize("N", [24, 54])
def test_seeded_starts_match_golden(golden, N):
    ham, U = model(N)
    for case in golden["configs"][str(N)]:
        ku, kd, _ = o.seeded_start(3, case["walker"], U, U)
        assert ku.tolist() == case["kappa_up"] and kd.tolist() == case["kappa_down"]


@pytest.mark.parametrize("N", [24, 54])
def test_c_chain_matches_golden_chain(golden, N):
    ham, U = model(N)
    g = golden["chains"][str(N)]
    m = oracle_c.OracleModel(U, U, [(i - 1, j - 1) for i, j in ham.nn])
    for wc in g["walkers"]:
        ch = m.new_chain(wc["start_up"], wc["start_down"])
        _, e = ch.run(g["seed"], wc["walker"], g["proposals"], g["refresh_every"], g["measure_every"])
        assert ch.ku.tolist() == wc["final_up"] and ch.kd.tolist() == wc["final_down"]
        assert ch.c.accepted == wc["accepted"]
        np.testing.assert_allclose(e[:len(wc["energies"])], wc["energies"], rtol=1e-9, atol=1e-9)


def test_complex_oracle_equals_real_at_zero_field():
    ham, U = model(54)
    bonds = [(i - 1, j - 1) for i, j in ham.nn]
    mr, mc = oracle_c.OracleModel(U, U, bonds, "real"), oracle_c.OracleModel(U, U, bonds, "cplx")
    ku, kd, _ = o.seeded_start(9, 0, U, U)
    a, b = mr.new_chain(ku, kd), mc.new_chain(ku, kd)
    _, ea = a.run(9, 0, 800, 27, 27)
    _, eb = b.run(9, 0, 800, 27, 27)
    assert np.array_equal(a.ku, b.ku) and a.c.accepted == b.c.accepted
    np.testing.assert_allclose(ea, eb, rtol=1e-10, atol=1e-10)


def test_complex_oracle_matches_numpy_chain_in_field():
    """B != 0 with N_up != N_down (scripts/LL.jl:21-25 shape, 6x3 cells): the
    complex C oracle follows the numpy restatement's trajectory and energies."""
    import math

    n1, n2, imbalance = 6, 3, 2
    L = o.double_kagome(1.0, n1, n2, (True, True), (False, True))
    B = imbalance * math.pi / (n1 * n2 * 2 * math.sqrt(3))
    N = n1 * n2 * 3
    ham = o.hamiltonian(N // 2 + imbalance // 2, N // 2 - imbalance // 2, L, B=B)
    assert np.iscomplexobj(ham.U_up) and np.abs(ham.U_up.imag).max() > 1e-3
    bonds = [(i - 1, j - 1) for i, j in ham.nn]
    m = oracle_c.OracleModel(ham.U_up, ham.U_down, bonds, "cplx")
    for walker in range(2):
        ku, kd, _ = o.seeded_start(4, walker, ham.U_up, ham.U_down)
        st = o.ChainState(ku.copy(), kd.copy(), o.reevaluateW(ham.U_up, ku), o.reevaluateW(ham.U_down, kd))
        o.run_chain(ham.nn, ham.U_up, ham.U_down, st, 4, walker, 400, 26, 26, ham=ham)
        ch = m.new_chain(ku, kd)
        _, e = ch.run(4, walker, 400, 26, 26)
        assert ch.ku.tolist() == st.kappa_up.tolist() and ch.kd.tolist() == st.kappa_down.tolist()
        assert ch.c.accepted == st.accepted and st.accepted > 0
        np.testing.assert_allclose(e[:len(st.energies)], st.energies, rtol=1e-9, atol=1e-9)


def test_threaded_chains_equal_serial():
    ham, U = model(24)
    m = oracle_c.OracleModel(U, U, [(i - 1, j - 1) for i, j in ham.nn])
    starts = [o.seeded_start(4, w, U, U)[:2] for w in range(6)]
    _, chains = oracle_c.run_chains(m, starts, 4, 500, 12, 12, 0, 3)
    for w, (ku, kd) in enumerate(starts):
        ch = m.new_chain(ku, kd)
        ch.run(4, w, 500, 12, 12)
        assert chains[w].c.accepted == ch.c.accepted and chains[w].c.sum_e == pytest.approx(ch.c.sum_e, rel=1e-12)


@pytest.mark.slow
def test_enumeration_reproduces_golden(golden):
    """Exact N=24 energies (about a minute of numpy)."""
    ham, U = model(24)
    e_psi2, e_ref = o.enumerate_energy(U, ham.nn, chunk=200000)
    assert e_psi2 == pytest.approx(golden["enum_N24"]["E_per_site_psi2"], abs=1e-12)
    assert e_ref == pytest.approx(golden["enum_N24"]["E_per_site_reference_rule"], abs=1e-12)
