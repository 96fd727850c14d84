"""Generates the golden fixtures in this directory from the oracle.

    python tests/golden/make_golden.py

Writes
  u_N24.npy      the N=24 orbitals (2x2 doubled cells, PBC, antiperiodic
                 along a2).  Its Fermi shell is open (4 states, 2 filled), so
                 the orbitals are shipped as data: every N=24 test uses this
                 exact basis choice.
  golden.json    exact N=24 energies by enumeration; per-configuration local
                 energies and determinant ratios at N=24/54/96 on seeded
                 configurations; short seeded chains at N=24/54; the exact
                 N=24 energy, gradient and SR matrix of the extended ansatz
                 at one parameter point (key grad_N24).

    python tests/golden/make_golden.py grad_N24     # rebuilds that key only

The oracle itself is pinned separately against the literal values of the
reference's test-suite (tests/test_oracle_pins.py).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import kagome_oracle as o  # noqa: E402

# "a x b doubled cells": DoubleKagome(1.0, 2a, b, (true,true); antiPBC=(false,true))
CELLS = {24: (2, 2), 54: (3, 3), 96: (4, 4), 216: (6, 6)}


def model(N):
    a, b = CELLS[N]
    lat = o.double_kagome(1.0, 2 * a, b, (True, True), (False, True))
    ham = o.hamiltonian(N // 2, N // 2, lat)
    U = ham.U_up.real.copy()
    if N == 24 and os.path.exists(os.path.join(HERE, "u_N24.npy")):
        U = np.load(os.path.join(HERE, "u_N24.npy"))
    return ham, U


def config_cases(N, U, ham, seed=3, walkers=3, n_ratios=8):
    out = []
    for w in range(walkers):
        ku, kd, _ = o.seeded_start(seed, w, U, U)
        Wu, Wd = o.reevaluateW(U, ku), o.reevaluateW(U, kd)
        E = o.getOL(ham, Wu, Wd, ku, kd)
        moves, ratios = [], []
        for (i, j) in ham.nn:
            if len(moves) >= n_ratios:
                break
            for (a, b) in ((j, i), (i, j)):    # up at a, down at b: up moves a -> b
                if ku[a - 1] != 0 and kd[b - 1] != 0:
                    K_up, l_up, K_dn, l_dn = b, int(ku[a - 1]), a, int(kd[b - 1])
                    moves.append([K_up - 1, l_up, K_dn - 1, l_dn])
                    ratios.append(float(Wu[K_up - 1, l_up - 1] * Wd[K_dn - 1, l_dn - 1]))
        out.append(dict(walker=w, kappa_up=ku.tolist(), kappa_down=kd.tolist(), local_energy=E,
                        moves=moves, ratios=ratios,
                        logdet=[o.logabsdet(U, ku), o.logabsdet(U, kd)]))
    return out


def chain_case(N, U, ham, seed=5, walkers=4, proposals=1500):
    out = []
    n = N // 2
    for w in range(walkers):
        ku, kd, _ = o.seeded_start(seed, w, U, U)
        st = o.ChainState(ku.copy(), kd.copy(), o.reevaluateW(U, ku), o.reevaluateW(U, kd))
        o.run_chain(ham.nn, U, U, st, seed, w, proposals, refresh_every=n, measure_every=n, ham=ham)
        out.append(dict(walker=w, start_up=ku.tolist(), start_down=kd.tolist(), final_up=st.kappa_up.tolist(),
                        final_down=st.kappa_down.tolist(), accepted=st.accepted, energies=st.energies))
    return dict(seed=seed, proposals=proposals, refresh_every=n, measure_every=n, walkers=out)


# A parameter point of the extended ansatz (t2, m, theta) with an open gap
# at half filling on 2x2 doubled cells (the pi-flux shell there is degenerate).
ALPHA_N24 = (-0.2515, 0.1215, -0.0494)


def grad_case():
    lat = o.double_kagome(1.0, 4, 2, (True, True), (False, True))
    H, dH = o.ansatz_hmat(lat, ALPHA_N24)
    Uu, Ud, Du, Dd = o.orbital_derivatives(H, dH, 12, 12)
    nn = o.get_nn(o.hmat(lat))
    r = o.enumerate_gradient(Uu, Ud, Du, Dd, nn)
    return dict(alpha=list(ALPHA_N24), E_per_site=r["E"] / 24, grad_per_site=(r["grad"] / 24).tolist(),
                S=r["S"].tolist())


def main():
    if sys.argv[1:] == ["grad_N24"]:
        path = os.path.join(HERE, "golden.json")
        g = json.load(open(path))
        g["grad_N24"] = grad_case()
        with open(path, "w") as f:
            json.dump(g, f)
        print("updated grad_N24 in", path)
        return
    ham24, U24 = model(24)
    if not os.path.exists(os.path.join(HERE, "u_N24.npy")):
        np.save(os.path.join(HERE, "u_N24.npy"), U24)
    g = {"cells": {str(k): v for k, v in CELLS.items()}}
    e_psi2, e_ref = o.enumerate_energy(U24, ham24.nn, chunk=200000)
    g["enum_N24"] = {"E_per_site_psi2": e_psi2, "E_per_site_reference_rule": e_ref}
    g["configs"] = {}
    for N in (24, 54, 96):
        ham, U = model(N)
        g["configs"][str(N)] = config_cases(N, U, ham)
    g["chains"] = {}
    for N in (24, 54):
        ham, U = model(N)
        g["chains"][str(N)] = chain_case(N, U, ham)
    g["grad_N24"] = grad_case()
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(g, f)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
