"""The oracle against the literal values of the reference's own test-suite.

Each test restates one reference testset (file:line in the KagomeDSL.jl tree)
with the reference's 1-based site numbers; the oracle functions take them
as-is.  No GPU.
"""
import math

import numpy as np
import pytest

import kagome_oracle as o


def lat(n1, n2, pbc, anti=(False, False)):
    return o.double_kagome(1.0, n1, n2, pbc, anti)


def H1(H, i, j):  # 1-based access like the Julia tests
    return H[i - 1, j - 1]


# ---- test/test-Lattice.jl ---------------------------------------------------

def test_doublekagome_lattice_jl_1_8():
    with pytest.raises(AssertionError):
        o.double_kagome(1.0, 3, 3, (False, False))
    assert o.ns(lat(4, 3, (False, False))) == 36


def test_nearest_neighbor_lattice_jl_10_45():
    H1m = o.hmat(lat(4, 4, (True, False)))
    assert H1m.shape[0] == 48
    nn = o.get_nn(H1m)
    assert all(i < j for i, j in nn)
    assert (1, 2) in nn and (1, 3) in nn and (2, 3) in nn and (1, 4) not in nn
    H2m = o.hmat(lat(4, 4, (True, True), (True, True)))
    nn2 = o.get_nn(H2m)
    assert len(nn) != len(nn2)
    assert all(p in nn2 for p in nn)
    assert all(H1(H1m, i, j) != 0 for i, j in nn)
    assert all(H1(H2m, i, j) != 0 for i, j in nn2)


# ---- test/test-Hamiltonian.jl -------------------------------------------------

def test_hamiltonian_obc_pbc_hamiltonian_jl_4_27():
    H = o.hmat(lat(4, 3, (False, False)))
    assert np.allclose(H, H.conj().T)
    assert H1(H, 1, 1) == 0 and H1(H, 1, 2) == -1 and H1(H, 1, 3) == -1
    assert all(abs(H1(H, 1, i)) < 1e-14 for i in range(4, 37))
    assert abs(H1(H, 3, 13) - 1) < 1e-14
    H2 = o.hmat(lat(4, 3, (True, False)))
    assert np.allclose(H2, H2.conj().T)
    assert H1(H2, 1, 2) == -1 and H1(H2, 1, 3) == -1
    assert H1(H2, 1, 11) == -1      # horizontal PBC
    assert H1(H2, 1, 3 * 4 + 1) == 0  # vertical OBC


def test_antiperiodic_hamiltonian_jl_30_61():
    H = o.hmat(lat(4, 3, (True, False), (True, False)))
    assert np.allclose(H, H.conj().T)
    assert H1(H, 1, 2) == -1 and H1(H, 1, 3) == -1 and H1(H, 5, 7) == -1 and H1(H, 1, 11) == 1
    H = o.hmat(lat(4, 3, (True, True), (False, True)))
    assert H1(H, 1, 11) == -1 and H1(H, 1, 3 + 4 * 6) == -1
    H = o.hmat(lat(4, 3, (True, True), (True, True)))
    assert H1(H, 1, 11) == 1 and H1(H, 1, 27) == -1 and H1(H, 11, 27) == 1
    H = o.hmat(lat(4, 3, (True, True), (True, False)))
    assert H1(H, 1, 11) == 1 and H1(H, 1, 3 + 4 * 6) == 1


def test_bc_errors_hamiltonian_jl_64_80():
    with pytest.raises(ValueError):
        lat(4, 3, (False, False), (True, False))
    with pytest.raises(ValueError):
        lat(4, 3, (False, False), (False, True))


def test_orbitals_hamiltonian_jl_84_95():
    ham = o.hamiltonian(18, 18, lat(4, 3, (True, False)))
    assert ham.U_up.shape == (36, 18) and ham.U_down.shape == (36, 18)


def test_getxprime_hamiltonian_jl_97_135():
    ham = o.hamiltonian(1, 0, lat(4, 3, (False, False)))
    ku = np.array([1] + [0] * 35)
    kd = np.array([0] + list(range(1, 36)))
    xp = o.getxprime(ham, ku, kd)
    assert len(xp) == 3
    assert xp[(-1, -1, -1, -1)] == (len(ham.nn) - 2) * 0.25 + 2 * (-0.25)
    assert xp[(2, 1, 1, 1)] == -0.5
    assert xp[(3, 1, 1, 2)] == -0.5


def test_getol_nonzero_hamiltonian_jl_137_146():
    params = dict(n1=2, n2=2, PBC=(False, False), N_up=6, N_down=6)
    ham = o.hamiltonian(6, 6, lat(params["n1"], params["n2"], params["PBC"]))
    ku = np.array([1, 0, 2, 3, 4, 5, 6, 0, 0, 0, 0, 0])
    kd = np.array([0, 1, 0, 0, 0, 0, 0, 2, 3, 4, 5, 6])
    W = np.zeros((12, 6))  # MC(params) allocates zero W (src/MonteCarlo.jl:181-182)
    # with zero W only the diagonal survives, which is nonzero here
    assert o.getOL(ham, W, W, ku, kd) != 0.0


def test_sz_hamiltonian_jl_148_235():
    assert o.Sz(1, [1, 0, 2], [0, 2, 0]) == 0.5
    assert o.Sz(2, [1, 0, 2], [0, 2, 0]) == -0.5
    with pytest.raises(o.ArgumentError):
        o.Sz(2, [1, 2, 0], [0, 2, 1])
    with pytest.raises(IndexError):
        o.Sz(4, [1, 2, 0], [0, 2, 1])
    with pytest.raises(IndexError):
        o.Sz(0, [1, 2, 0], [0, 2, 1])
    with pytest.raises(ValueError):
        o.Sz(1, [1, 2, 0, 1], [0, 2, 1])
    assert o.Sz(1, [1], [0]) == 0.5 and o.Sz(1, [0], [1]) == -0.5
    with pytest.raises(o.ArgumentError):
        o.Sz(1, [0], [0])
    with pytest.raises(o.ArgumentError):
        o.Sz(1, [1], [1])
    n = 1000
    ku, kd = np.zeros(n, int), np.zeros(n, int)
    ku[0] = 1
    kd[-1] = 1
    assert o.Sz(1, ku, kd) == 0.5 and o.Sz(n, ku, kd) == -0.5
    with pytest.raises(o.ArgumentError):
        o.Sz(2, ku, kd)
    rng = np.random.default_rng(42)
    sites = rng.permutation(100) + 1
    ku, kd = np.zeros(100, int), np.zeros(100, int)
    for i, s in enumerate(sites[:50]):
        ku[s - 1] = i + 1
    for i, s in enumerate(sites[50:]):
        kd[s - 1] = i + 1
    for s in sites:
        assert o.Sz(int(s), ku, kd) == (0.5 if ku[s - 1] else -0.5)


def test_spin_interaction_hamiltonian_jl_237_331():
    ku, kd = [1, 0, 2], [0, 1, 0]
    xp = {}
    o.spinInteraction(xp, ku, kd, 2, 1)
    assert xp[(2, 1, 1, 1)] == pytest.approx(-0.5)
    xp = {}
    o.spinInteraction(xp, ku, kd, 1, 2)
    assert xp[(2, 1, 1, 1)] == pytest.approx(-0.5)
    xp = {}
    o.spinInteraction(xp, ku, kd, 1, 3)
    assert xp == {}
    o.spinInteraction(xp, ku, kd, 2, 3)
    assert xp[(2, 2, 3, 1)] == -0.5
    xp = {}
    o.spinInteraction(xp, ku, kd, 1, 2)
    o.spinInteraction(xp, ku, kd, 1, 2)
    assert xp[(2, 1, 1, 1)] == pytest.approx(-1.0)
    xp = {}
    o.spinInteraction(xp, [1], [0], 1, 1)
    assert xp == {}
    with pytest.raises(IndexError):
        o.spinInteraction({}, [], [], 1, 1)
    ku, kd = np.zeros(1000, int), np.zeros(1000, int)
    ku[0], kd[1] = 1, 1
    xp = {}
    o.spinInteraction(xp, ku, kd, 1, 2)
    assert xp[(2, 1, 1, 1)] == pytest.approx(-0.5)
    xp = {(2, 1, 1, 1): 0.25}
    o.spinInteraction(xp, [1, 0, 2], [0, 1, 0], 1, 2)
    assert xp[(2, 1, 1, 1)] == pytest.approx(-0.25)


def _abc(pbc, anti, link_inter, s1, s2, B=0.0, n1=4, n2=3):
    L = lat(n1, n2, pbc, anti)
    N = n1 * n2 * 3 * 2
    T = np.zeros((N, N), complex)
    o.apply_boundary_conditions(T, L, s1, s2, link_inter, B)
    return T[s1 - 1, s2 - 1]


def test_apply_boundary_conditions_hamiltonian_jl_332_438():
    li = {(1, 5, -1, 0): 1.0, (5, 1, 1, 0): 1.0}
    assert _abc((True, True), (False, False), li, 1, 11) == pytest.approx(1.0)
    assert _abc((True, True), (False, False), li, 11, 1) == pytest.approx(1.0)
    assert _abc((True, True), (True, False), li, 1, 11) == pytest.approx(-1.0)
    assert _abc((True, True), (True, False), li, 11, 1) == pytest.approx(-1.0)
    ly = {(3, 6, 0, -1): 1.0, (6, 3, 0, 1): 1.0}
    assert _abc((True, True), (False, True), ly, 3, 3 * 2 * 4 + 6) == pytest.approx(-1.0)
    assert _abc((True, True), (False, True), ly, 3 * 2 * 4 + 6, 3) == pytest.approx(-1.0)
    # diagonal crossing: signs cancel (ns = 36 here)
    L = lat(4, 3, (True, True), (True, True))
    T = np.zeros((36, 36), complex)
    o.apply_boundary_conditions(T, L, 1, 36, {(1, 6, -1, -1): 1.0}, 0.0)
    assert T[0, 35] == pytest.approx(1.0)
    T = np.zeros((36, 36), complex)
    o.apply_boundary_conditions(T, L, 1, 7, {(1, 5, 1, 0): 1.0}, 0.0)
    assert T[0, 6] == pytest.approx(0.0)
    L = lat(4, 3, (True, True))
    with pytest.raises(AssertionError):
        o.apply_boundary_conditions(np.zeros((36, 36), complex), L, 1, 2, {(1, 5, -1, 0): 1.0}, 0.0)
    with pytest.raises(AssertionError):
        o.apply_boundary_conditions(np.zeros((36, 36), complex), L, 0, 1, {(1, 5, -1, 0): 1.0}, 0.0)
    with pytest.raises(AssertionError):
        o.apply_boundary_conditions(np.zeros((37, 37), complex), L, 1, 37, {(1, 5, -1, 0): 1.0}, 0.0)


def test_doublekagome_bc_hamiltonian_jl_440_465():
    li = {(1, 5, -1, 0): 1.0, (5, 1, 1, 0): 1.0}
    assert _abc((True, True), (True, False), li, 1, 11) == pytest.approx(-1.0 * li[(1, 5, -1, 0)])


def test_unitcell_coord_hamiltonian_jl_467_504():
    L = lat(4, 2, (False, False))
    m = 2
    assert np.allclose(o.unitcell_coord(L, 1), [0, 0]) and np.allclose(o.unitcell_coord(L, 6), [0, 0])
    assert np.allclose(o.unitcell_coord(L, 7), L.a1)
    assert np.allclose(o.unitcell_coord(L, m * 2 * 6), (m - 1) * L.a1 + 1 * L.a2)
    assert np.allclose(o.unitcell_coord(L, 6 * m), (m - 1) * L.a1)
    assert np.allclose(o.unitcell_coord(L, 6 * m + 1), L.a2)
    with pytest.raises(AssertionError):
        o.unitcell_coord(L, 0)
    with pytest.raises(AssertionError):
        o.unitcell_coord(L, m * 2 * 6 + 1)
    assert o.unitcell_coord(L, 7)[0] - o.unitcell_coord(L, 1)[0] == pytest.approx(4.0)
    assert o.unitcell_coord(L, 6 * m + 1)[1] - o.unitcell_coord(L, 1)[1] == pytest.approx(math.sqrt(3))


def test_unitcell_diff_hamiltonian_jl_506_604():
    L = lat(4, 3, (False, False))
    a1, a2 = L.a1, L.a2
    z = np.zeros(2)
    assert o.unitcell_diff(L, a1, z) == (1, 0)
    assert o.unitcell_diff(L, a2, z) == (0, 1)
    assert o.unitcell_diff(L, a1 + a2, z) == (1, 1)
    for eps in (-0.1, 0.1):
        assert o.unitcell_diff(L, a1 + eps, z) == (1, 0)
        assert o.unitcell_diff(L, a2 + eps, z) == (0, 1)
    assert o.unitcell_diff(L, z, a1) == (-1, 0)
    assert o.unitcell_diff(L, z, a2) == (0, -1)
    assert o.unitcell_diff(L, 2 * a1, z) == (2, 0)
    assert o.unitcell_diff(L, 2 * a2, z) == (0, 2)
    assert o.unitcell_diff(L, 2 * a1 + 2 * a2, z) == (2, 2)
    assert o.unitcell_diff(L, z, z) == (0, 0)
    assert o.unitcell_diff(L, [0.1, 0.1], z) == (0, 0)
    s3 = math.sqrt(3.0)
    for c1, c2, ex in (([0, 0], [4, 0], (-1, 0)), ([4, 0], [0, 0], (1, 0)), ([0, 0], [1, s3], (0, -1)),
                       ([1, s3], [0, 0], (0, 1)), ([5, s3], [0, 0], (1, 1))):
        assert o.unitcell_diff(L, c1, c2) == ex


def test_get_boundary_shifts_hamiltonian_jl_606_701():
    L = lat(4, 3, (True, True))
    with pytest.raises(AssertionError):
        o.get_boundary_shifts(L, 3, 3)
    assert (1, 0, 1.0) in o.get_boundary_shifts(L, 3, 9)
    sh = o.get_boundary_shifts(L, 3, 6 * (2 - 1) + 3)
    assert (-(2 - 1), 0, 1.0) in sh and (2 + 1, 0, 1.0) in sh
    assert o.get_boundary_shifts(lat(4, 3, (False, False)), 3, 9) == [(1, 0, 1.0)]
    sh = o.get_boundary_shifts(lat(4, 3, (True, False)), 3, 9)
    assert len(sh) > 1 and all(s[1] == 0 for s in sh)
    sh = o.get_boundary_shifts(lat(4, 3, (True, False), (True, False)), 3, 6 * (2 - 1) + 3)
    assert any(s[2] == -1.0 for s in sh)
    with pytest.raises(AssertionError):
        o.get_boundary_shifts(L, 0, 1)
    with pytest.raises(AssertionError):
        o.get_boundary_shifts(L, 1, 4 * 3 * 6 + 1)
    sh = o.get_boundary_shifts(L, 3, 6 * 4 // 2 + 9)
    assert any(s[0] != 0 and s[1] != 0 for s in sh)
    sh = o.get_boundary_shifts(lat(4, 3, (True, True), (True, True)), 3, 6 * 4 // 2 + 9)
    by = {}
    for dx, dy, sg in sh:
        by.setdefault((dx, dy), set()).add(sg)
    assert all(len(v) == 1 for v in by.values())
    assert (1, 0, 1.0) in o.get_boundary_shifts(L, 3, 9)
    assert any(abs(s[0]) == 2 + 1 for s in o.get_boundary_shifts(L, 3, 6 * (2 - 1) + 3))


def test_get_site_coord_hamiltonian_jl_703_720():
    L = lat(4, 3, (False, False))
    assert np.array_equal(o.get_site_coord(L, 1), [0.0, 0.0])
    assert np.array_equal(o.get_site_coord(L, 2), [1.0, 0.0])
    assert np.array_equal(o.get_site_coord(L, 3), [0.5, 0.5 * math.sqrt(3.0)])
    assert np.array_equal(o.get_site_coord(L, 7), [4.0, 0.0])
    assert np.array_equal(o.get_site_coord(L, 13), [1.0, math.sqrt(3.0)])


def test_magnetic_field_hamiltonian_jl_722_774():
    L = lat(4, 3, (False, False))
    B = 0.1
    HB, H0 = o.hmat(L, B=B), o.hmat(L, B=0.0)
    assert np.allclose(HB, HB.conj().T)
    assert np.array_equal(H0, o.hmat(L))

    def ph(Lx, s1, s2, r2=None):
        r1 = o.get_site_coord(Lx, s1)
        r2 = o.get_site_coord(Lx, s2) if r2 is None else r2
        return (B / 2) * (r1[0] + r2[0]) * (r2[1] - r1[1])

    assert H1(HB, 1, 3) == -complex(math.cos(ph(L, 1, 3)), math.sin(ph(L, 1, 3)))
    assert ph(L, 1, 2) == 0.0 and H1(HB, 1, 2) == -1.0
    p = ph(L, 3, 13)
    assert H1(HB, 3, 13) == -o.PI_LINK_INTER[(3, 1, 0, 1)] * complex(math.cos(p), math.sin(p))
    Lp = lat(4, 3, (True, True))
    HBp = o.hmat(Lp, B=B)
    r2 = o.get_site_coord(Lp, 11) + (-(Lp.n1 // 2)) * Lp.a1
    p = ph(Lp, 1, 11, r2)
    assert H1(HBp, 1, 11) == -o.PI_LINK_INTER[(1, 5, -1, 0)] * complex(math.cos(p), math.sin(p))


# ---- test/test-MonteCarlo.jl --------------------------------------------------

def test_init_conf_qr_montecarlo_jl_14_52():
    rng = np.random.default_rng(0)
    ns_, Nu = 12, 6
    Uu, Ud = rng.random((ns_, Nu)), rng.random((ns_, ns_ - Nu))
    ku, kd = o.init_conf_qr(Uu, Ud, ns_, Nu)
    assert np.count_nonzero(ku) == Nu and np.count_nonzero(kd) == ns_ - Nu
    assert set(ku[ku != 0]) <= set(range(1, Nu + 1)) and set(kd[kd != 0]) <= set(range(1, ns_ - Nu + 1))
    assert all((ku[i] != 0) ^ (kd[i] != 0) for i in range(ns_))
    assert abs(np.linalg.det(o.tilde_U(Uu, ku))) > np.finfo(float).eps
    assert abs(np.linalg.det(o.tilde_U(Ud, kd))) > np.finfo(float).eps


def test_tilde_u_montecarlo_jl_54_173():
    U = np.array([[1.0, 2, 3], [4, 5, 6], [7, 8, 9]])
    r = o.tilde_U(U, [2, 3, 1])
    assert r.shape == (3, 3)
    assert np.array_equal(r[0], U[2]) and np.array_equal(r[1], U[0]) and np.array_equal(r[2], U[1])
    with pytest.raises(o.ArgumentError):
        o.tilde_U(np.array([[1.0, 2], [3, 4]]), [0, 0])
    U = np.array([[1.0, 2], [3, 4], [5, 6]])
    r = o.tilde_U(U, [1, 0, 2])
    assert r.shape == (2, 2) and np.array_equal(r[0], U[0]) and np.array_equal(r[1], U[2])
    U = np.array([[1 + 1j, 2 + 2j], [3 + 3j, 4 + 4j]])
    r = o.tilde_U(U, [2, 1])
    assert np.array_equal(r[0], U[1]) and np.array_equal(r[1], U[0])
    assert o.tilde_U(np.zeros((0, 0)), []).shape == (0, 0)
    assert np.array_equal(o.tilde_U(np.array([[1.0]]), [1]), [[1.0]])
    U = np.array([[1.0, 2], [3, 4]])
    U0 = U.copy()
    k = [1, 2]
    o.tilde_U(U, k)
    assert np.array_equal(U, U0) and k == [1, 2]
    with pytest.raises(IndexError):
        o.tilde_U(U, [3, 1])
    with pytest.raises(ValueError):
        o.tilde_U(U, [1, 2, 3])
    assert o.tilde_U(U, [1, 2]).dtype == U.dtype
    assert o.tilde_U(np.array([[1, 2], [3, 4]]), [1, 2]).dtype == np.array([[1, 2]]).dtype


def test_z_montecarlo_jl_175_183():
    assert o.Z([(1, 2), (2, 3), (1, 3)], [0, 1, 0], [1, 0, 2]) == 2


def test_reevaluate_w_montecarlo_jl_185_231():
    Uu = np.array([[1.0, 0.2], [0.2, 1.0]])
    Ud = np.array([[1.0, 0.3], [0.3, 1.0]])
    Wu = o.reevaluateW(Uu, [1, 2])
    Wd = o.reevaluateW(Ud, [2, 1])
    assert np.allclose(Wu, Uu @ np.linalg.inv(o.tilde_U(Uu, [1, 2])), atol=1e-10)
    assert np.allclose(Wd, Ud @ np.linalg.inv(o.tilde_U(Ud, [2, 1])), atol=1e-10)
    rng = np.random.default_rng(1)
    n = 4
    Uu = np.eye(n) + 0.1 * rng.random((n, n))
    Uu = (Uu + Uu.T) / 2
    W = o.reevaluateW(Uu, [1, 2, 3, 4])
    assert W.shape == (n, n) and np.allclose(W, W.T, atol=1e-10)


def test_update_w_montecarlo_jl_235_341():
    W = np.array([[1.0, 0.2], [0.2, 1.0]])
    W0 = W.copy()
    o.update_W(W, 1, 2)
    factor = W[0, 0] / W[1, 0]
    assert W[0, 0] == pytest.approx(W0[0, 0] - factor * (W0[1, 0] - 1.0))
    assert W[0, 1] == pytest.approx(W0[0, 1] - factor * W0[1, 1])
    assert not np.array_equal(W, W0)
    rng = np.random.default_rng(2)
    n = 4
    W = (np.eye(n) + 0.1 * rng.random((n, n))).astype(complex)
    W = (W + W.conj().T) / 2
    o.update_W(W, 1, 3)
    assert np.all(np.isfinite(W))
    W = np.array([[1.0, 1e-10], [1e-10, 1.0]])
    o.update_W(W, 1, 2)
    assert np.all(np.isfinite(W))
    W = np.eye(5) + 1e-10 * rng.random((5, 5))
    o.update_W(W, 2, 4)
    assert np.all(np.isfinite(W))


def test_is_occupied_montecarlo_jl_344_351():
    k = [1, 0, 2, 0]
    assert [o.is_occupied(k, i) for i in (1, 2, 3, 4)] == [True, False, True, False]
    with pytest.raises(IndexError):
        o.is_occupied(k, 5)


def test_update_configurations_montecarlo_jl_354_406():
    class S:
        pass

    for flag, args in ((1, (2, 1, 1, 1)), (2, (1, 2, 1, 1))):
        s = S()
        s.kappa_up, s.kappa_down = np.array([1, 0, 2, 0]), np.array([0, 1, 0, 2])
        s.W_up, s.W_down = np.ones((4, 2)), np.ones((4, 2))
        o.update_configurations(s, flag, *args)
        assert s.kappa_up[0] == 1 and s.kappa_up[1] == 0
        assert s.kappa_down[0] == 0 and s.kappa_down[1] == 1


def test_carlo_init_montecarlo_jl_408_427():
    ham = o.hamiltonian(6, 6, lat(2, 2, (False, False)))
    ku, kd, Wu, Wd = o.find_initial_configuration(ham.U_up, ham.U_down, 12, 6)
    assert abs(np.linalg.det(o.tilde_U(ham.U_up, ku))) != 0.0
    assert abs(np.linalg.det(o.tilde_U(ham.U_down, kd))) != 0.0


def test_carlo_init_singular_montecarlo_jl_429_477():
    rng = np.random.default_rng(3)
    Uu = np.repeat(rng.random((1, 6)), 12, axis=0)
    with pytest.raises(RuntimeError, match="QR-based configuration is singular"):
        o.find_initial_configuration(Uu, rng.random((12, 6)), 12, 6)


# ---- the shared random stream -------------------------------------------------

def test_philox_known_answers():
    """Random123's published Philox4x32-10 known-answer vectors."""
    assert o.philox4x32_10((0, 0, 0, 0), (0, 0)) == (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    assert o.philox4x32_10((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2) == (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)
    assert o.philox4x32_10((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0)) == (
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)
