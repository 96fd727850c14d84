"""GPU parity of the adjoint gradient estimator (kvmc_measure_grad).

  * per configuration, E_L (complex) and O_a = d ln psi / d a against the
    oracle (tilde_U^{-1} tilde_dU_a traces and the complex local energy):
    1e-9 relative in the plain FP64 form, 2e-4 in the mixed FP32 form;
  * at N=24, the Monte Carlo E, dE/da and SR matrix against the exact FP64
    values from enumerating all C(24,12) configurations (golden fixture,
    within 4 standard errors), under both acceptance rules (the reference
    rule's samples are reweighted by Z_mu);
  * correlated-sampling central finite differences (h = 1e-4) on the same
    samples agree with the adjoint estimate.
"""
import json
import os

import numpy as np
import pytest

import kagome_oracle as o

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def kv(built):
    import kagomevmc

    return kagomevmc


@pytest.fixture(scope="module")
def golden():
    return json.load(open(os.path.join(GOLD, "golden.json")))


def lat24(kv):
    return kv.DoubleKagome(1.0, 4, 2, (True, True), (False, True))


def engine(kv, A, walkers, precision, accept="metropolis", seed=7):
    eng = kv.Engine(A.ham, walkers, precision=precision, accept=accept, seed=seed,
                    refresh_interval=(64 if precision == "mixed" else 0))
    eng.set_log_derivatives(A.dU_up, A.dU_down)
    return eng


@pytest.mark.parametrize("precision", ["plain", "mixed"])
@pytest.mark.parametrize("N", [24, 96])
def test_adjoint_per_configuration_matches_oracle(kv, golden, N, precision):
    if N == 24:
        A = kv.Ansatz.build(lat24(kv), 12, 12, *golden["grad_N24"]["alpha"])
    else:
        A = kv.Ansatz.build(kv.DoubleKagome(1.0, 8, 4, (True, True), (False, True)), 48, 48,
                            *kv.ansatz.draw_alpha(4))
    assert np.iscomplexobj(A.ham.U_up)
    nw = 4
    starts = [o.seeded_start(11, w, A.ham.U_up, A.ham.U_down)[:2] for w in range(nw)]
    eng = engine(kv, A, nw, precision, accept="reference")
    eng.init(np.stack([s[0] for s in starts]), np.stack([s[1] for s in starts]))
    nn1 = [(i + 1, j + 1) for i, j in A.ham.nn]
    E, O = eng.measure_grad(want=True)
    eng.measure_grad()
    tol = 1e-9 if precision == "plain" else 2e-4
    want_E, want_O, Z = [], [], []
    for w, (ku, kd) in enumerate(starts):
        Wu, Wd = o.reevaluateW(A.ham.U_up, ku), o.reevaluateW(A.ham.U_down, kd)
        e = o.local_energy_complex(nn1, Wu, Wd, ku, kd)
        Ow = o.log_derivative(A.ham.U_up, A.dU_up, ku) + o.log_derivative(A.ham.U_down, A.dU_down, kd)
        assert abs(E[w] - e) <= tol * max(1.0, abs(e)), (w, E[w], e)
        assert np.all(np.abs(O[w] - Ow) <= tol * np.maximum(1.0, np.abs(Ow))), (w, O[w], Ow)
        want_E.append(e)
        want_O.append(Ow)
        Z.append(o.Z(nn1, ku, kd))
    # two evaluations at the same configurations, weight Z_mu (reference rule)
    sums = eng.grad_sums()
    lay = kv.ansatz.sum_layout(3)
    for w in range(nw):
        assert sums[w, 0] == 2 * Z[w]
        np.testing.assert_allclose(sums[w, 1] + 1j * sums[w, 2], 2 * Z[w] * want_E[w], rtol=tol, atol=tol)
        so = sums[w, lay["O"]]
        np.testing.assert_allclose(so[0::2] + 1j * so[1::2], 2 * Z[w] * want_O[w], rtol=tol, atol=tol * Z[w])
    eng.close()


@pytest.mark.parametrize("precision,accept", [("plain", "metropolis"), ("mixed", "metropolis"),
                                              ("mixed", "reference")])
def test_gradient_matches_exact_enumeration(kv, golden, precision, accept):
    g = golden["grad_N24"]
    A = kv.Ansatz.build(lat24(kv), 12, 12, *g["alpha"])
    eng = engine(kv, A, 2048, precision, accept=accept, seed=13)
    eng.init()
    res = kv.energy_and_gradient(eng, n_sweeps=600, thermalize=600)
    E, se_E = res["E"] / 24, res["se_E"] / 24
    grad, se_g = res["grad"] / 24, res["se_grad"] / 24
    assert abs(E - g["E_per_site"]) <= 2 * se_E, (E, g["E_per_site"], se_E)
    assert np.all(np.abs(grad - g["grad_per_site"]) <= 2 * se_g), (grad, g["grad_per_site"], se_g)
    S = np.array(g["S"])
    assert np.allclose(res["S"], res["S"].T, atol=1e-12)
    assert np.abs(res["S"] - S).max() <= 0.03 + 0.05 * np.abs(S).max(), (res["S"], S)
    eng.close()


def test_correlated_finite_differences_agree_with_adjoint(kv, golden):
    """Central differences (h = 1e-4) of the reweighted energy
    E(a') = sum r E_L(a') / sum r, r = |psi_a'(x) / psi_a(x)|^2, over the samples
    of one chain batch at a, against the adjoint estimate on the same samples.
    The two differ by the sample mean of d Re E_L / d a, which has zero
    expectation; a jackknife over walker groups gives its error bar."""
    g = golden["grad_N24"]
    alpha = np.array(g["alpha"])
    lat = lat24(kv)
    A = kv.Ansatz.build(lat, 12, 12, *alpha)
    walkers, points, h = 1024, 40, 1e-4
    eng = engine(kv, A, walkers, "plain", seed=17)
    eng.init()
    eng.sweep(600)
    shifted = []
    for q in range(3):
        for sgn in (1, -1):
            a2 = alpha.copy()
            a2[q] += sgn * h
            shifted.append(kv.Engine(kv.Ansatz.build(lat, 12, 12, *a2).ham, walkers, precision="plain"))
    base = kv.Engine(A.ham, walkers, precision="plain")
    E_s, O_s, r_s, Ep_s = [], [], [], []
    for _ in range(points):
        eng.sweep(12)
        E, O = eng.measure_grad(want=True)
        ku, kd, _ = eng.get_state()
        base.set_state(ku, kd)
        l0 = base.walker_logdet().sum(1)
        rs, eps = [], []
        for e2 in shifted:
            e2.set_state(ku, kd)
            rs.append(np.exp(2 * (e2.walker_logdet().sum(1) - l0)))
            eps.append(e2.measure())
        E_s.append(E)
        O_s.append(O)
        r_s.append(np.array(rs))
        Ep_s.append(np.array(eps))
    E_s, O_s = np.array(E_s), np.array(O_s)            # [points][W], [points][W][3]
    r_s, Ep_s = np.array(r_s), np.array(Ep_s)          # [points][6][W]

    def both(mask):
        e, oo = E_s[:, mask].ravel(), O_s[:, mask].reshape(-1, 3)
        adj = 2 * np.real((oo.conj() * e[:, None]).mean(0) - oo.conj().mean(0) * e.mean())
        fd = np.zeros(3)
        for q in range(3):
            val = []
            for k in (2 * q, 2 * q + 1):
                r, ep = r_s[:, k][:, mask].ravel(), Ep_s[:, k][:, mask].ravel()
                val.append((r * ep).sum() / r.sum())
            fd[q] = (val[0] - val[1]) / (2 * h)
        return adj, fd

    adj, fd = both(np.ones(walkers, bool))
    groups = 32
    jk = []
    for k in range(groups):
        m = np.ones(walkers, bool)
        m[k::groups] = False
        a_k, f_k = both(m)
        jk.append(f_k - a_k)
    jk = np.array(jk)
    se = np.sqrt((groups - 1) / groups * ((jk - jk.mean(0)) ** 2).sum(0))
    assert np.all(np.abs(fd - adj) <= 2 * se), (fd / 24, adj / 24, se / 24)
    exact = np.array(g["grad_per_site"]) * 24
    se_adj = np.std([both(np.arange(walkers) % groups == k)[0] for k in range(groups)], axis=0, ddof=1) / np.sqrt(groups)
    assert np.all(np.abs(adj - exact) <= 2 * se_adj), (adj / 24, exact / 24, se_adj / 24)
    for e2 in shifted + [base, eng]:
        e2.close()


def test_differentiation_workload_forms_agree(kv):
    """N=96, parameters drawn from a seed, 256 chains: the mixed complex FP32
    form and the plain complex FP64 form give the same E and dE/da within
    their statistical errors on identical proposal streams."""
    A = kv.Ansatz.build(kv.DoubleKagome(1.0, 8, 4, (True, True), (False, True)), 48, 48, *kv.ansatz.draw_alpha(4))
    out = {}
    for precision in ("plain", "mixed"):
        eng = engine(kv, A, 256, precision, accept="reference", seed=3)
        eng.init()
        out[precision] = kv.energy_and_gradient(eng, n_sweeps=30, thermalize=960)
        eng.close()
    p, m = out["plain"], out["mixed"]
    assert abs(p["E"] - m["E"]) / 96 <= 1e-4
    assert np.all(np.abs(p["grad"] - m["grad"]) <= 0.25 * p["se_grad"] + 1e-6), (p["grad"], m["grad"], p["se_grad"])
    w = np.linalg.eigvalsh(m["S"])
    assert w.min() >= -1e-9
