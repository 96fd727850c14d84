"""Extended mean-field ansatz and the adjoint energy gradient.

No reference counterpart: KagomeDSL.jl evaluates the energy of the pi-flux
state only.  This module adds three real variational parameters on top of
the reference's hopping matrix (src/Hamiltonian.jl:308-354) and the host
side of the gradient estimator:

* ``ansatz_hmat`` -- H(t2, m, theta) and dH/d(t2, m, theta) from
  ``kvmc_ansatz_hopping`` (the parameterisation is stated in include/kvmc.h);
* ``orbital_derivatives`` -- U and dU/da by first-order eigenvector
  perturbation of the host FP64 diagonalisation (the same ``eigh`` that
  builds the orbitals, src/Hamiltonian.jl:382-393);
* ``Ansatz`` -- the model bundle at one parameter point;
* ``estimate`` -- dE/da and the stochastic-reconfiguration matrix from the
  per-walker sums that ``Engine.measure_grad`` accumulates on the GPU;
  ``julia/KagomeVMCChainRules.jl`` wraps the same estimate as a
  ChainRulesCore ``rrule`` on the Julia side.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import ArgumentError
from .lattice import PI_LINK_IN, PI_LINK_INTER, DoubleKagome, Hamiltonian, Hmat, _links, get_nn, ns

PARAMS = ("t2", "m", "theta")
# the ranges the parameters are drawn from: t2 in [-0.3, 0.3], m in [0, 0.2], theta in [-0.2, 0.2] rad
RANGES = ((-0.3, 0.3), (0.0, 0.2), (-0.2, 0.2))


def draw_alpha(seed: int) -> tuple:
    """(t2, m, theta) drawn uniformly from RANGES with numpy's PCG64 stream of `seed`."""
    rng = np.random.default_rng(seed)
    return tuple(float(rng.uniform(lo, hi)) for lo, hi in RANGES)


def ansatz_hmat(lat: DoubleKagome, t2: float, m: float, theta: float, B: float = 0.0,
                link_in=PI_LINK_IN, link_inter=PI_LINK_INTER):
    """(H, [dH/dt2, dH/dm, dH/dtheta]), complex N x N each."""
    N = ns(lat)
    lin, nin = _links(link_in, False)
    lint, nint = _links(link_inter, True)
    H = np.zeros(2 * N * N)
    dH = np.zeros(6 * N * N)
    par = np.array([t2, m, theta], dtype=np.float64)
    _lib.check(_lib.load().kvmc_ansatz_hopping(C.byref(lat.desc()), lin, nin, lint, nint, float(B), _lib.ptr(par),
                                               _lib.ptr(H), _lib.ptr(dH)))

    def unpack(v):
        return (v[0::2] + 1j * v[1::2]).reshape((N, N), order="F")

    return unpack(H), [unpack(dH[2 * q * N * N:2 * (q + 1) * N * N]) for q in range(3)]


def orbital_derivatives(H: np.ndarray, dHs, N_up: int, N_down: int, min_gap: float = 1e-8):
    """U_up, U_down (lowest eigenvectors of H) and dU_up, dU_down ([P][N][n]).

    dU[:, c] = sum over unoccupied m of v_m (v_m^H dH v_c) / (e_c - e_m).  The
    occupied-occupied part of the perturbation is left out: it only rotates U
    inside its span, which changes every determinant by one common factor and
    no expectation value.  Raises when the level above the last occupied one
    is closer than ``min_gap`` (the derivative of the orbitals is then
    undefined).
    """
    H = np.asarray(H)
    cplx = bool(np.any(H.imag != 0) or any(np.any(np.asarray(d).imag != 0) for d in dHs))
    w, V = np.linalg.eigh(H if cplx else H.real)
    p = np.argsort(w, kind="stable")
    w, V = w[p], V[:, p]
    res = []
    for n in (N_up, N_down):
        if n < len(w) and w[n] - w[n - 1] <= min_gap:
            raise ArgumentError(_lib.KVMC_ERR_ARGUMENT,
                                f"degenerate Fermi level at {n} orbitals (gap {w[n] - w[n - 1]:.3g})")
        U, Vu = V[:, :n], V[:, n:]
        den = w[:n][None, :] - w[n:][:, None]
        D = np.stack([Vu @ ((Vu.conj().T @ (np.asarray(dH) if cplx else np.asarray(dH).real) @ U) / den)
                      for dH in dHs])
        res.append((np.ascontiguousarray(U), D))
    (Uu, Du), (Ud, Dd) = res
    return Uu, Ud, Du, Dd


@dataclass
class Ansatz:
    """The model at one parameter point: Hamiltonian bundle plus dU/da."""
    ham: Hamiltonian
    dU_up: np.ndarray
    dU_down: np.ndarray
    params: tuple

    @classmethod
    def build(cls, lat: DoubleKagome, N_up: int, N_down: int, t2=0.0, m=0.0, theta=0.0, B=0.0,
              link_in=PI_LINK_IN, link_inter=PI_LINK_INTER):
        H, dH = ansatz_hmat(lat, t2, m, theta, B, link_in, link_inter)
        Uu, Ud, Du, Dd = orbital_derivatives(H, dH, N_up, N_down)
        # the Heisenberg bonds are the nearest-neighbour ones of the pi-flux H
        nn = get_nn(Hmat(lat, link_in, link_inter, B))
        return cls(Hamiltonian(N_up, N_down, Uu, Ud, H, nn), Du, Dd, (t2, m, theta))


def sum_layout(P: int):
    """Slices of one walker's row of kvmc_grad_sums."""
    o = 3
    return dict(w=0, E=slice(1, 3), O=slice(o, o + 2 * P), OE=slice(o + 2 * P, o + 4 * P),
                OO=slice(o + 4 * P, o + 4 * P + 2 * P * P))


def _cx(v):
    return v[..., 0::2] + 1j * v[..., 1::2]


def estimate(sums: np.ndarray, P: int) -> dict:
    """E, dE/da, S from per-walker sums [W][L], with standard errors of E
    and dE/da from the spread over walkers (each walker one independent chain).

    E and its gradient are totals (divide by N for per site).
    """
    lay = sum_layout(P)
    w = sums[:, lay["w"]]
    tot = sums.sum(0)
    W = tot[0]
    E = complex(tot[1], tot[2]) / W
    O = _cx(tot[lay["O"]]) / W
    OE = _cx(tot[lay["OE"]]) / W
    OO = _cx(tot[lay["OO"]]).reshape(P, P) / W
    grad = 2 * np.real(OE - np.conj(O) * E)
    S = np.real(OO - np.outer(np.conj(O), O))
    # per-walker estimates for error bars
    ok = w > 0
    ww = w[ok]
    Ew = (sums[ok, 1] + 1j * sums[ok, 2]) / ww
    Ow = _cx(sums[ok][:, lay["O"]]) / ww[:, None]
    OEw = _cx(sums[ok][:, lay["OE"]]) / ww[:, None]
    gw = 2 * np.real(OEw - np.conj(Ow) * Ew[:, None])
    nw = int(ok.sum())
    se_E = float(np.std(Ew.real, ddof=1) / np.sqrt(nw)) if nw > 1 else float("nan")
    se_g = np.std(gw, axis=0, ddof=1) / np.sqrt(nw) if nw > 1 else np.full(P, np.nan)
    return dict(E=float(E.real), E_imag=float(E.imag), grad=grad, S=S, O=O, se_E=se_E, se_grad=se_g,
                walkers=nw)


def energy_and_gradient(engine, n_sweeps: int, proposals_per_sweep: int | None = None, thermalize: int = 0) -> dict:
    """Runs n_sweeps sweeps of `proposals_per_sweep` proposals per walker
    (default min(N_up, N_down), the reference's sweep), one adjoint
    evaluation after each, and returns ``estimate`` of the sums."""
    nps = proposals_per_sweep or min(engine.n_up, engine.n_down)
    if thermalize:
        engine.sweep(thermalize)
    engine.reset_stats()
    for _ in range(n_sweeps):
        engine.sweep(nps)
        engine.measure_grad()
    return estimate(engine.grad_sums(), engine.n_params)
