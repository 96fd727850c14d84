"""Lattice and mean-field model constructors (host, FP64).

Mirrors the constructor surface of KagomeDSL.jl: ``DoubleKagome``
(src/Lattice.jl:17-97), ``Hmat`` (src/Hamiltonian.jl:308-354), ``orbitals``
(:382-393), ``get_nn`` (:447-451) and ``Hamiltonian`` (:420-492).  The
hopping matrix and the bond list come from libkvmc; the diagonalisation is
numpy's LAPACK ``eigh``.  Site indices are 0-based (Python), configuration
values keep the reference meaning (0 empty, 1..n label).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import ArgumentError

# The reference's pi-flux tables, src/Hamiltonian.jl:219-235 and :250-261.
PI_LINK_IN = {
    (1, 2): 1, (1, 3): 1, (2, 3): 1, (2, 4): -1, (4, 6): 1, (4, 5): 1, (5, 6): 1,
    (2, 1): 1, (3, 1): 1, (3, 2): 1, (4, 2): -1, (6, 4): 1, (5, 4): 1, (6, 5): 1,
}
PI_LINK_INTER = {
    (3, 5, -1, 1): -1, (3, 1, 0, 1): -1, (6, 2, 0, 1): -1, (6, 4, 0, 1): 1, (5, 1, 1, 0): 1,
    (1, 5, -1, 0): 1, (1, 3, 0, -1): -1, (2, 6, 0, -1): -1, (4, 6, 0, -1): 1, (5, 3, 1, -1): -1,
}


@dataclass(frozen=True)
class DoubleKagome:
    """Doubled-cell kagome lattice, 6 sites per cell, n1*n2*3 sites (src/Lattice.jl:17-97)."""
    t: float
    n1: int
    n2: int
    PBC: tuple
    antiPBC: tuple = (False, False)

    def __post_init__(self):
        for i, (p, a) in enumerate(zip(self.PBC, self.antiPBC)):
            if a and not p:
                d = "first" if i == 0 else "second"
                raise ArgumentError(_lib.KVMC_ERR_ARGUMENT,
                                    f"Invalid boundary conditions in {d} direction: Cannot have antiperiodic "
                                    "boundary conditions without periodic boundary conditions")
        if self.n1 % 2 != 0:
            raise ArgumentError(_lib.KVMC_ERR_ARGUMENT, "n1 must be even in DoubleKagome")

    @property
    def a1(self):
        return np.array([4 * self.t, 0.0])

    @property
    def a2(self):
        return np.array([self.t, math.sqrt(3) * self.t])

    def desc(self) -> _lib.LatticeDesc:
        d = _lib.LatticeDesc()
        d.n1, d.n2 = self.n1, self.n2
        d.pbc[0], d.pbc[1] = int(bool(self.PBC[0])), int(bool(self.PBC[1]))
        d.antipbc[0], d.antipbc[1] = int(bool(self.antiPBC[0])), int(bool(self.antiPBC[1]))
        d.t = float(self.t)
        return d


def ns(lat: DoubleKagome) -> int:
    """Number of sites (src/Lattice.jl:97)."""
    n = C.c_int32()
    _lib.check(_lib.load().kvmc_lattice_sites(C.byref(lat.desc()), C.byref(n)))
    return n.value


def _links(table, inter):
    arr = (_lib.Link * len(table))()
    for k, (key, amp) in enumerate(table.items()):
        arr[k].label1, arr[k].label2 = key[0], key[1]
        arr[k].dx, arr[k].dy = (key[2], key[3]) if inter else (0, 0)
        arr[k].amplitude = float(amp)
    return arr, len(table)


def Hmat(lat: DoubleKagome, link_in=PI_LINK_IN, link_inter=PI_LINK_INTER, B: float = 0.0) -> np.ndarray:
    """Spinon hopping matrix -(T + T^dagger), complex N x N (src/Hamiltonian.jl:308-354)."""
    N = ns(lat)
    lin, nin = _links(link_in, False)
    lint, nint = _links(link_inter, True)
    H = np.zeros(2 * N * N, dtype=np.float64)
    _lib.check(_lib.load().kvmc_hopping_matrix(C.byref(lat.desc()), lin, nin, lint, nint, float(B), _lib.ptr(H)))
    Hc = H[0::2] + 1j * H[1::2]
    return Hc.reshape((N, N), order="F")


def get_nn(H: np.ndarray) -> list:
    """Bonds (i, j), i < j, 0-based, in the reference's column-major order (src/Hamiltonian.jl:447-451)."""
    N = H.shape[0]
    buf = np.empty(2 * N * N, dtype=np.float64)
    Hf = np.asfortranarray(H, dtype=complex)
    buf[0::2] = Hf.real.ravel(order="F")
    buf[1::2] = Hf.imag.ravel(order="F")
    nb = C.c_int32()
    lib = _lib.load()
    _lib.check(lib.kvmc_bonds_from_hopping(N, _lib.ptr(buf), C.byref(nb), None))
    bonds = np.empty(2 * nb.value, dtype=np.int32)
    _lib.check(lib.kvmc_bonds_from_hopping(N, _lib.ptr(buf), C.byref(nb), _lib.ptr(bonds)))
    return [(int(bonds[2 * k]), int(bonds[2 * k + 1])) for k in range(nb.value)]


def orbitals(H: np.ndarray, N_up: int, N_down: int):
    """Lowest N_up / N_down eigenvectors of H, the same basis for both spins (src/Hamiltonian.jl:382-393).

    Inside a degenerate Fermi shell the reference keeps whatever LAPACK
    returns; here the real symmetric H (B = 0) is diagonalised as a real
    matrix by numpy's ``eigh`` so that the orbitals are real, and a complex
    Hermitian H (B != 0) gives complex orbitals.
    """
    H = np.asarray(H)
    if np.iscomplexobj(H) and np.any(H.imag != 0):
        w, V = np.linalg.eigh(H)
    else:
        w, V = np.linalg.eigh(np.real(H))
    p = np.argsort(w, kind="stable")
    V = V[:, p]
    return np.ascontiguousarray(V[:, :N_up]), np.ascontiguousarray(V[:, :N_down])


@dataclass
class Hamiltonian:
    """Mean-field model bundle (src/Hamiltonian.jl:420-427)."""
    N_up: int
    N_down: int
    U_up: np.ndarray
    U_down: np.ndarray
    H_mat: np.ndarray
    nn: list

    @classmethod
    def build(cls, N_up, N_down, lat, link_in=PI_LINK_IN, link_inter=PI_LINK_INTER, B=0.0):
        """src/Hamiltonian.jl:480-492."""
        H = Hmat(lat, link_in=link_in, link_inter=link_inter, B=B)
        U_up, U_down = orbitals(H, N_up, N_down)
        return cls(N_up, N_down, U_up, U_down, H, get_nn(H))
