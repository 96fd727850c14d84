"""Host side of the extended ansatz (no GPU): kvmc_ansatz_hopping against the
oracle's independent construction, dH against finite differences, the flux
it puts through each triangle, and the orbital derivatives against finite
differences of log|det tilde_U| (the gauge-invariant part of O_a)."""
import numpy as np
import pytest

import kagome_oracle as o

CASES = [(4, 2, 0.0), (6, 3, 0.0), (8, 4, 0.0), (8, 4, 0.2), (4, 3, 0.0)]
ALPHA_N24 = (-0.2515, 0.1215, -0.0494)


@pytest.fixture(scope="module")
def kv(built):
    import kagomevmc

    return kagomevmc


@pytest.mark.parametrize("n1,n2,B", CASES)
def test_ansatz_matrix_matches_oracle(kv, n1, n2, B):
    rng = np.random.default_rng(n1 * 10 + n2)
    par = (rng.uniform(-0.3, 0.3), rng.uniform(0, 0.2), rng.uniform(-0.2, 0.2))
    lat = kv.DoubleKagome(1.0, n1, n2, (True, True), (False, True))
    H, dH = kv.ansatz_hmat(lat, *par, B=B)
    Ho, dHo = o.ansatz_hmat(o.double_kagome(1.0, n1, n2, (True, True), (False, True)), par, B=B)
    assert np.abs(H - Ho).max() <= 1e-14
    assert all(np.abs(a - b).max() <= 1e-14 for a, b in zip(dH, dHo))
    assert np.abs(H - H.conj().T).max() == 0.0
    # four second neighbours per site, each hop once per direction
    assert np.count_nonzero(dH[0]) == 4 * H.shape[0]
    h = 1e-6
    for q in range(3):
        pp, pm = list(par), list(par)
        pp[q] += h
        pm[q] -= h
        fd = (kv.ansatz_hmat(lat, *pp, B=B)[0] - kv.ansatz_hmat(lat, *pm, B=B)[0]) / (2 * h)
        assert np.abs(fd - dH[q]).max() <= 1e-8, q


def test_zero_parameters_give_the_pi_flux_matrix(kv):
    lat = kv.DoubleKagome(1.0, 6, 3, (True, True), (False, True))
    H, _ = kv.ansatz_hmat(lat, 0.0, 0.0, 0.0, B=0.1)
    assert np.array_equal(H, kv.Hmat(lat, B=0.1))


def test_triangle_flux_is_theta(kv):
    lat = kv.DoubleKagome(1.0, 6, 3, (True, True), (False, True))
    theta = 0.15
    H, _ = kv.ansatz_hmat(lat, 0.0, 0.0, theta)
    H0 = kv.Hmat(lat)
    N = H.shape[0]
    adj = [set(np.nonzero(H0[i])[0]) - {i} for i in range(N)]
    flux = []
    for i in range(N):
        for j in adj[i]:
            for k in adj[i] & adj[j]:
                if i < j < k:
                    r = H[i, j] * H[j, k] * H[k, i] / (H0[i, j] * H0[j, k] * H0[k, i])
                    flux.append(abs(np.angle(r)))
    assert len(flux) == 2 * N // 3
    np.testing.assert_allclose(flux, theta, atol=1e-13)


def test_log_derivative_matches_finite_differences(kv):
    """Re O_a = d log|det tilde_U| / d a, which does not depend on the eigenvector gauge."""
    lat = kv.DoubleKagome(1.0, 4, 2, (True, True), (False, True))
    par = np.array(ALPHA_N24)
    A = kv.Ansatz.build(lat, 12, 12, *par)
    U, D = A.ham.U_up, A.dU_up
    Uo, _, Do, _ = o.orbital_derivatives(*o.ansatz_hmat(o.double_kagome(1.0, 4, 2, (True, True), (False, True)), par),
                                         12, 12)
    assert np.abs(Uo - U).max() <= 1e-12 and np.abs(Do - D).max() <= 1e-10
    h = 1e-5
    for w in range(3):
        ku, kd, _ = o.seeded_start(1, w, A.ham.U_up, A.ham.U_down)
        O = o.log_derivative(A.ham.U_up, A.dU_up, ku) + o.log_derivative(A.ham.U_down, A.dU_down, kd)
        for q in range(3):
            pp, pm = par.copy(), par.copy()
            pp[q] += h
            pm[q] -= h
            Ap, Am = kv.Ansatz.build(lat, 12, 12, *pp), kv.Ansatz.build(lat, 12, 12, *pm)
            lp = o.logabsdet(Ap.ham.U_up, ku) + o.logabsdet(Ap.ham.U_down, kd)
            lm = o.logabsdet(Am.ham.U_up, ku) + o.logabsdet(Am.ham.U_down, kd)
            assert abs(O[q].real - (lp - lm) / (2 * h)) <= 1e-7 * max(1.0, abs(O[q].real)), (w, q)


def test_degenerate_fermi_level_is_rejected(kv):
    """The pi-flux state at 2x2 doubled cells has a degenerate shell at half filling."""
    lat = kv.DoubleKagome(1.0, 4, 2, (True, True), (False, True))
    with pytest.raises(kv.ArgumentError, match="degenerate Fermi level"):
        kv.Ansatz.build(lat, 12, 12, 0.0, 0.0, 0.0)


def test_estimate_from_sums_matches_direct_formula(kv):
    """The host reduction of the per-walker sums (layout of kvmc_grad_sums)."""
    rng = np.random.default_rng(0)
    P, Wk, S = 3, 5, 40
    E = rng.normal(size=(Wk, S)) + 0.1j * rng.normal(size=(Wk, S))
    O = rng.normal(size=(Wk, S, P)) + 1j * rng.normal(size=(Wk, S, P))
    wt = rng.integers(10, 30, size=(Wk, S)).astype(float)
    L = 3 + 4 * P + 2 * P * P
    sums = np.zeros((Wk, L))
    for w in range(Wk):
        sums[w, 0] = wt[w].sum()
        se = (wt[w] * E[w]).sum()
        sums[w, 1:3] = se.real, se.imag
        so = (wt[w, :, None] * O[w]).sum(0)
        soe = (wt[w, :, None] * O[w].conj() * E[w][:, None]).sum(0)
        soo = np.einsum("s,sa,sb->ab", wt[w], O[w].conj(), O[w]).ravel()
        for k, v in enumerate(so):
            sums[w, 3 + 2 * k:5 + 2 * k] = v.real, v.imag
        for k, v in enumerate(soe):
            sums[w, 3 + 2 * P + 2 * k:5 + 2 * P + 2 * k] = v.real, v.imag
        for k, v in enumerate(soo):
            sums[w, 3 + 4 * P + 2 * k:5 + 4 * P + 2 * k] = v.real, v.imag
    r = kv.estimate(sums, P)
    wf, Ef, Of = wt.ravel(), E.ravel(), O.reshape(-1, P)
    mE = (wf * Ef).sum() / wf.sum()
    mO = (wf[:, None] * Of).sum(0) / wf.sum()
    mOE = (wf[:, None] * Of.conj() * Ef[:, None]).sum(0) / wf.sum()
    mOO = np.einsum("s,sa,sb->ab", wf, Of.conj(), Of) / wf.sum()
    np.testing.assert_allclose(r["E"], mE.real, rtol=1e-12)
    np.testing.assert_allclose(r["grad"], 2 * np.real(mOE - mO.conj() * mE), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(r["S"], np.real(mOO - np.outer(mO.conj(), mO)), rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("n1,n2,pbc", [(2, 2, (True, True)), (4, 1, (True, False)), (2, 3, (True, True))])
def test_oracle_gradient_matches_finite_differences_of_exact_energy(n1, n2, pbc):
    """Pins the oracle's exact gradient (used for the N=24 fixture): central
    differences of the enumerated energy on 12- and 18-site lattices."""
    lat = o.double_kagome(1.0, n1, n2, pbc, (False, pbc[1]))
    N = o.ns(lat)
    n = N // 2
    par = np.array([0.21, 0.13, -0.11])
    nn = o.get_nn(o.hmat(lat))
    Uu, Ud, Du, Dd = o.orbital_derivatives(*o.ansatz_hmat(lat, par), n, n)
    r = o.enumerate_gradient(Uu, Ud, Du, Dd, nn)
    assert np.allclose(r["S"], r["S"].T) and np.linalg.eigvalsh(r["S"]).min() > -1e-12
    h = 1e-4
    for q in range(3):
        E = []
        for s in (1, -1):
            pp = par.copy()
            pp[q] += s * h
            a, b, c, d = o.orbital_derivatives(*o.ansatz_hmat(lat, pp), n, n)
            E.append(o.enumerate_gradient(a, b, c[:0], d[:0], nn)["E"])
        assert abs((E[0] - E[1]) / (2 * h) - r["grad"][q]) <= 1e-6 * max(1.0, abs(r["grad"][q])), q
