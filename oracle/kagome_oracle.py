"""CPU oracle for the KagomeDSL.jl variational Monte Carlo hot path.

TEST INFRASTRUCTURE ONLY.  This module is a plain numpy / pure-Python
restatement of the reference algorithm.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it, and only as the checker.  The product
(``kagomedsl.jl_gb300``) never imports or calls anything in ``oracle/``.

Every function cites the reference file and lines it restates
(paths relative to the KagomeDSL.jl project root).  Indexing follows the
reference: site numbers passed to the functions below are 1-based, arrays are
0-based numpy arrays, and configuration vectors ``kappa`` hold 0 for an empty
site and the 1-based orbital label otherwise (src/MonteCarlo.jl:92-115).

Pinning: the functions here are checked against every literal value in the
reference's own test-suite (test/test-Lattice.jl, test/test-Hamiltonian.jl,
test/test-MonteCarlo.jl), restated with their literal values in ``tests/test_oracle_pins.py``.
The Monte Carlo chain itself is parity-unpinned against the reference (its
RNG stream belongs to the third-party Carlo.jl / StatsBase packages); the
chain here draws from the Philox4x32-10 counter stream defined below, which
the GPU path shares, so chain-level parity is tested against this oracle and,
statistically, against exact enumeration (``enumerate_energy``).
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------------------
# Lattice: src/Lattice.jl
# ---------------------------------------------------------------------------


def validate_boundary_conditions(PBC, antiPBC):
    """src/Lattice.jl:3-15 -- antiperiodic requires periodic in that direction."""
    for i, (pbc, apbc) in enumerate(zip(PBC, antiPBC)):
        if apbc and not pbc:
            d = "first" if i == 0 else "second"
            raise ValueError(
                f"Invalid boundary conditions in {d} direction: Cannot have "
                "antiperiodic boundary conditions without periodic boundary conditions")


@dataclass
class DoubleKagome:
    """src/Lattice.jl:17-31 (struct) and :68-92 (constructor)."""
    n1: int
    n2: int
    t: float
    a1: np.ndarray
    a2: np.ndarray
    r: list
    PBC: tuple
    antiPBC: tuple


def double_kagome(t, n1, n2, PBC, antiPBC=(False, False)):
    """src/Lattice.jl:68-92."""
    validate_boundary_conditions(PBC, antiPBC)
    if n1 % 2 != 0:
        raise AssertionError("n1 must be even in DoubleKagome")
    a = 2 * t
    a1 = np.array([2 * a, 0.0])
    a2 = np.array([0.5 * a, 0.5 * math.sqrt(3) * a])
    r1 = np.array([0.0, 0.0])
    r2 = 0.25 * a1
    r3 = 0.5 * a2
    r4 = 0.5 * a1
    r5 = 0.75 * a1
    r6 = np.array([2.5 * t, 0.5 * math.sqrt(3) * t])
    return DoubleKagome(n1, n2, t, a1, a2, [r1, r2, r3, r4, r5, r6],
                        tuple(PBC), tuple(antiPBC))


def ns(lat):
    """src/Lattice.jl:97."""
    return lat.n1 * lat.n2 * 3


# ---------------------------------------------------------------------------
# Hopping matrix: src/Hamiltonian.jl:28-354
# ---------------------------------------------------------------------------

# src/Hamiltonian.jl:219-235
PI_LINK_IN = {
    (1, 2): 1, (1, 3): 1, (2, 3): 1, (2, 4): -1, (4, 6): 1, (4, 5): 1, (5, 6): 1,
    (2, 1): 1, (3, 1): 1, (3, 2): 1, (4, 2): -1, (6, 4): 1, (5, 4): 1, (6, 5): 1,
}
# src/Hamiltonian.jl:250-261
PI_LINK_INTER = {
    (3, 5, -1, 1): -1, (3, 1, 0, 1): -1, (6, 2, 0, 1): -1, (6, 4, 0, 1): 1,
    (5, 1, 1, 0): 1, (1, 5, -1, 0): 1, (1, 3, 0, -1): -1, (2, 6, 0, -1): -1,
    (4, 6, 0, -1): 1, (5, 3, 1, -1): -1,
}


def unitcell_coord(lat, s):
    """src/Hamiltonian.jl:28-38 (s is 1-based)."""
    n1 = lat.n1 // 2
    n2 = lat.n2
    nsites = n1 * n2 * 6
    if not (1 <= s <= nsites):
        raise AssertionError(f"s should be in the range of 1 to ns, got: {s}")
    u = (s - 1) // 6
    return (u % n1) * lat.a1 + (u // n1) * lat.a2


def unitcell_diff(lat, c1, c2):
    """src/Hamiltonian.jl:56-76 -- integer (dx, dy) with c1-c2 = dx*a1+dy*a2."""
    diff = np.asarray(c1, dtype=float) - np.asarray(c2, dtype=float)
    a1, a2 = lat.a1, lat.a2
    det = a1[0] * a2[1] - a1[1] * a2[0]
    # Julia round(Int, x) rounds half to even, as does Python's round().
    dx = round((a2[1] * diff[0] - a2[0] * diff[1]) / det)
    dy = round((-a1[1] * diff[0] + a1[0] * diff[1]) / det)
    return int(dx), int(dy)


def get_boundary_shifts(lat, s1, s2):
    """src/Hamiltonian.jl:99-153 -- image shifts (dx, dy, sign), order kept."""
    if s1 == s2:
        raise AssertionError(f"s1 and s2 should not be the same, got: {s1} and {s2}")
    PBC1, PBC2 = lat.PBC
    anti1, anti2 = lat.antiPBC
    n1 = lat.n1 // 2
    n2 = lat.n2
    nsites = n1 * n2 * 6
    if not (1 <= s1 <= nsites):
        raise AssertionError("s1 out of range")
    if not (1 <= s2 <= nsites):
        raise AssertionError("s2 out of range")
    u1 = unitcell_coord(lat, s1)
    u2 = unitcell_coord(lat, s2)
    dx, dy = unitcell_diff(lat, u2, u1)
    if tuple(lat.PBC) == (False, False):
        return [(dx, dy, 1.0)]
    shifts = [(dx, dy, 1.0)]
    shifts_x = [-n1, 0, n1] if PBC1 else [0]
    shifts_y = [-n2, 0, n2] if PBC2 else [0]
    for sh1 in shifts_x:          # Julia `for a in A, b in B`: b runs fastest
        for sh2 in shifts_y:
            if sh1 == 0 and sh2 == 0:
                continue
            sign = 1.0
            if anti1 and sh1 != 0:
                sign *= -1.0
            if anti2 and sh2 != 0:
                sign *= -1.0
            shifts.append((dx + sh1, dy + sh2, sign))
    out = []
    for s in shifts:              # unique(), first occurrence kept
        if s not in out:
            out.append(s)
    return out


def get_site_coord(lat, s):
    """src/Hamiltonian.jl:279-283."""
    label = (s - 1) % 6
    return unitcell_coord(lat, s) + lat.r[label]


def _peierls(B, r1, r2):
    """The phase expression of src/Hamiltonian.jl:201-202 and :325-326."""
    phase = (B / 2) * (r1[0] + r2[0]) * (r2[1] - r1[1])
    return complex(math.cos(phase), math.sin(phase))


def apply_boundary_conditions(T, lat, s1, s2, link_inter, B):
    """src/Hamiltonian.jl:177-207 -- adds every image hop s1->s2 into T (0-based array)."""
    cell1 = (s1 - 1) // 6 + 1
    cell2 = (s2 - 1) // 6 + 1
    if cell1 == cell2:
        raise AssertionError("s1 and s2 should not be in the same cell")
    label1 = (s1 - 1) % 6 + 1
    label2 = (s2 - 1) % 6 + 1
    shifts = get_boundary_shifts(lat, s1, s2)
    r1 = get_site_coord(lat, s1)
    r_uc_1 = unitcell_coord(lat, s1)
    dr_2 = get_site_coord(lat, s2) - unitcell_coord(lat, s2)
    for dx, dy, sign in shifts:
        key = (label1, label2, dx, dy)
        if key in link_inter:
            r_uc_2_real = r_uc_1 + dx * lat.a1 + dy * lat.a2
            r2_real = r_uc_2_real + dr_2
            T[s1 - 1, s2 - 1] += sign * link_inter[key] * _peierls(B, r1, r2_real)


def hmat(lat, link_in=PI_LINK_IN, link_inter=PI_LINK_INTER, B=0.0):
    """src/Hamiltonian.jl:308-354 -- H = -(T + T^dagger), complex N x N."""
    n1, n2 = lat.n1, lat.n2
    nsites = n1 * n2 * 3
    T = np.zeros((nsites, nsites), dtype=complex)
    ncell = n1 * n2 // 2
    for c1 in range(1, ncell + 1):
        sites = range((c1 - 1) * 6 + 1, c1 * 6 + 1)
        for s1 in sites:
            for s2 in sites:
                if s1 >= s2:
                    continue
                key = ((s1 - 1) % 6 + 1, (s2 - 1) % 6 + 1)
                if key in link_in:
                    r1 = get_site_coord(lat, s1)
                    r2 = get_site_coord(lat, s2)
                    T[s1 - 1, s2 - 1] = link_in[key] * _peierls(B, r1, r2)
    for c1 in range(1, ncell + 1):
        sites1 = range((c1 - 1) * 6 + 1, c1 * 6 + 1)
        for c2 in range(1, ncell + 1):
            if c1 == c2:
                continue
            sites2 = range((c2 - 1) * 6 + 1, c2 * 6 + 1)
            for s1 in sites1:
                for s2 in sites2:
                    if s1 >= s2:
                        continue
                    apply_boundary_conditions(T, lat, s1, s2, link_inter, B)
    if np.any(np.tril(T, -1) != 0):
        raise RuntimeError("tunneling matrix must be upper triangular")
    return -(T + T.conj().T)


def orbitals(H, N_up, N_down):
    """src/Hamiltonian.jl:382-393 -- lowest-N columns of eigh(H), shared by both spins.

    The reference takes whatever LAPACK returns inside a degenerate shell; this
    restatement takes numpy's ``eigh`` basis (LAPACK ``*heevd``) and, for a
    real symmetric H, diagonalises the real matrix so that U is real.
    """
    Hh = np.asarray(H)
    if np.all(Hh.imag == 0):
        w, V = np.linalg.eigh(Hh.real)
    else:
        w, V = np.linalg.eigh(Hh)
    p = np.argsort(w, kind="stable")
    V = V[:, p]
    return V[:, :N_up].copy(), V[:, :N_down].copy()


def get_nn(H):
    """src/Hamiltonian.jl:447-451 -- upper-triangular nonzeros, Julia column-major order, 1-based."""
    H = np.asarray(H)
    n = H.shape[0]
    out = []
    for j in range(n):
        for i in range(j + 1):
            if H[i, j] != 0:
                out.append((i + 1, j + 1))
    return out


@dataclass
class Hamiltonian:
    """src/Hamiltonian.jl:420-427."""
    N_up: int
    N_down: int
    U_up: np.ndarray
    U_down: np.ndarray
    H_mat: np.ndarray
    nn: list


def hamiltonian(N_up, N_down, lat, link_in=PI_LINK_IN, link_inter=PI_LINK_INTER, B=0.0):
    """src/Hamiltonian.jl:480-492."""
    H = hmat(lat, link_in=link_in, link_inter=link_inter, B=B)
    U_up, U_down = orbitals(H, N_up, N_down)
    return Hamiltonian(N_up, N_down, U_up, U_down, H, get_nn(H))


# ---------------------------------------------------------------------------
# Local energy: src/Hamiltonian.jl:531-778
# ---------------------------------------------------------------------------


def is_occupied(kappa, l):
    """src/MonteCarlo.jl:132-135 (l is 1-based)."""
    if not (1 <= l <= len(kappa)):
        raise IndexError(f"BoundsError: index {l} out of 1..{len(kappa)}")
    return kappa[l - 1] != 0


def Sz(i, kappa_up, kappa_down):
    """src/Hamiltonian.jl:531-565."""
    n = len(kappa_up)
    if not (1 <= i <= n):
        raise IndexError(f"BoundsError: index {i}")
    if len(kappa_down) != n:
        raise ValueError("DimensionMismatch: kappa_up and kappa_down must have same length")
    up = is_occupied(kappa_up, i)
    dn = is_occupied(kappa_down, i)
    if up and not dn:
        return 0.5
    if dn and not up:
        return -0.5
    if up and dn:
        raise ArgumentError(f"Site {i} is doubly occupied")
    raise ArgumentError(f"Site {i} is unoccupied")


class ArgumentError(ValueError):
    """Julia's ArgumentError."""


DIAG_KEY = (-1, -1, -1, -1)


def SzInteraction(xprime, kappa_up, kappa_down, i, j):
    """src/Hamiltonian.jl:593-604."""
    xprime[DIAG_KEY] = xprime.get(DIAG_KEY, 0.0) + Sz(i, kappa_up, kappa_down) * Sz(j, kappa_up, kappa_down)


def spinInteraction(xprime, kappa_up, kappa_down, i, j):
    """src/Hamiltonian.jl:636-672 -- keys (K_up, l_up, K_down, l_down), 1-based."""
    if not (1 <= i <= len(kappa_up)) or not (1 <= j <= len(kappa_up)):
        raise IndexError("BoundsError")
    i_up, j_up = kappa_up[i - 1], kappa_up[j - 1]
    i_dn, j_dn = kappa_down[i - 1], kappa_down[j - 1]
    if j_up != 0 and i_dn != 0:
        k = (i, int(j_up), j, int(i_dn))
        xprime[k] = xprime.get(k, 0.0) - 0.5
    if i_up != 0 and j_dn != 0:
        k = (j, int(i_up), i, int(j_dn))
        xprime[k] = xprime.get(k, 0.0) - 0.5


def getxprime(ham, kappa_up, kappa_down):
    """src/Hamiltonian.jl:711-720."""
    xprime = {}
    for (i, j) in ham.nn:
        spinInteraction(xprime, kappa_up, kappa_down, i, j)
        SzInteraction(xprime, kappa_up, kappa_down, i, j)
    return xprime


def getOL(ham, W_up, W_down, kappa_up, kappa_down):
    """src/Hamiltonian.jl:762-778 -- E_L = diag + sum coeff*W_up[K,l]*W_down[K',l'], real part."""
    if len(kappa_up) != len(kappa_down):
        raise AssertionError("length mismatch")
    OL = 0.0
    for conf, coff in getxprime(ham, kappa_up, kappa_down).items():
        if conf == DIAG_KEY:
            OL += coff
        else:
            OL += coff * W_up[conf[0] - 1, conf[1] - 1] * W_down[conf[2] - 1, conf[3] - 1]
    return float(np.real(OL))


# ---------------------------------------------------------------------------
# W algebra: src/MonteCarlo.jl
# ---------------------------------------------------------------------------


def tilde_U(U, kappa):
    """src/MonteCarlo.jl:92-115 -- row l of the result is U[R,:] for kappa[R] == l."""
    U = np.asarray(U)
    n, m = U.shape
    kappa = list(kappa)
    if len(kappa) != n:
        raise ValueError(f"DimensionMismatch: Length of kappa ({len(kappa)}) must match number of rows in U ({n})")
    if sum(1 for x in kappa if x != 0) != m:
        raise ArgumentError(f"kappa ({kappa}) is not valid")
    out = np.zeros((m, m), dtype=U.dtype)
    for R, l in enumerate(kappa):
        if l != 0:
            if not (1 <= l <= m):
                raise IndexError("BoundsError")
            out[l - 1, :] = U[R, :]
    return out


def reevaluateW(U, kappa):
    """src/MonteCarlo.jl:55-66 -- W = U * (tilde_U \\ I)."""
    tU = tilde_U(U, kappa)
    return np.asarray(U) @ np.linalg.solve(tU, np.eye(tU.shape[0], dtype=tU.dtype))


def update_W(W, l, K):
    """src/MonteCarlo.jl:279-292 -- in-place Sherman-Morrison rank-1, l and K 1-based."""
    row = W[K - 1, :].copy()
    row[l - 1] -= 1.0
    col = W[:, l - 1].copy()
    alpha = -1.0 / W[K - 1, l - 1]
    W += np.outer(col, alpha * row)


def update_W_matrices(W_up, W_down, K_up, K_down, l_up, l_down):
    """src/MonteCarlo.jl:255-258."""
    update_W(W_up, l_up, K_up)
    update_W(W_down, l_down, K_down)


def Z(nn, kappa_up, kappa_down):
    """src/MonteCarlo.jl:460-474 -- number of antiparallel (exchangeable) bonds."""
    c = 0
    for (s1, s2) in nn:
        if kappa_up[s1 - 1] != 0 and kappa_down[s2 - 1] != 0:
            c += 1
        elif kappa_up[s2 - 1] != 0 and kappa_down[s1 - 1] != 0:
            c += 1
    return c


def update_configurations(st, flag, i, site, l_up, l_down):
    """src/MonteCarlo.jl:497-511 (st has kappa_up, kappa_down, W_up, W_down)."""
    if flag == 1:
        if st.W_up is not None:
            update_W_matrices(st.W_up, st.W_down, site, i, l_up, l_down)
        st.kappa_up[i - 1], st.kappa_up[site - 1] = 0, l_up
        st.kappa_down[i - 1], st.kappa_down[site - 1] = l_down, 0
    else:
        if st.W_up is not None:
            update_W_matrices(st.W_up, st.W_down, i, site, l_up, l_down)
        st.kappa_up[i - 1], st.kappa_up[site - 1] = l_up, 0
        st.kappa_down[i - 1], st.kappa_down[site - 1] = 0, l_down


def init_conf_qr(U_up, U_down, nsites, N_up):
    """src/MonteCarlo.jl:326-357 -- pivoted-QR start; N_down = ns - N_up (reference quirk at :339)."""
    import scipy.linalg as sla
    _, _, p_up = sla.qr(np.asarray(U_up).conj().T, mode="economic", pivoting=True)
    sites_up = [int(p) + 1 for p in p_up[:N_up]]
    kappa_up = np.zeros(nsites, dtype=np.int64)
    for i, s in enumerate(sites_up):
        kappa_up[s - 1] = i + 1
    N_down = nsites - N_up
    kappa_down = np.zeros(nsites, dtype=np.int64)
    if N_down > 0:
        avail = [s for s in range(1, nsites + 1) if s not in set(sites_up)]
        sub = np.asarray(U_down)[[a - 1 for a in avail], :]
        _, _, p_dn = sla.qr(sub.conj().T, mode="economic", pivoting=True)
        for i, idx in enumerate(p_dn[:N_down]):
            kappa_down[avail[int(idx)] - 1] = i + 1
    return kappa_up, kappa_down


def find_initial_configuration(U_up, U_down, nsites, N_up):
    """src/MonteCarlo.jl:382-410 -- raises on a singular QR start."""
    ku, kd = init_conf_qr(U_up, U_down, nsites, N_up)
    try:
        tu = tilde_U(U_up, ku)
        if abs(np.linalg.det(tu)) == 0.0:
            raise np.linalg.LinAlgError
        W_up = np.asarray(U_up) @ np.linalg.solve(tu, np.eye(len(tu)))
        W_down = None
        if nsites - N_up > 0:
            td = tilde_U(U_down, kd)
            if abs(np.linalg.det(td)) == 0.0:
                raise np.linalg.LinAlgError
            W_down = np.asarray(U_down) @ np.linalg.solve(td, np.eye(len(td)))
    except np.linalg.LinAlgError:
        raise RuntimeError("QR-based configuration is singular. The Hamiltonian may be rank-deficient.")
    return ku, kd, W_up, W_down


# ---------------------------------------------------------------------------
# Counter-based random stream shared with the GPU path (Philox4x32-10,
# Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as easy as 1, 2, 3",
# SC'11).  The reference draws from Carlo.jl's Xoshiro; that stream is
# third-party and not reproducible here, so both sides of every chain-level
# parity test draw from this one instead.
# ---------------------------------------------------------------------------

_M0, _M1 = 0xD2511F53, 0xCD9E8D57
_W0, _W1 = 0x9E3779B9, 0xBB67AE85
_MASK = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    for rnd in range(10):
        p0 = _M0 * c0
        p1 = _M1 * c2
        hi0, lo0 = (p0 >> 32) & _MASK, p0 & _MASK
        hi1, lo1 = (p1 >> 32) & _MASK, p1 & _MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        if rnd < 9:
            k0 = (k0 + _W0) & _MASK
            k1 = (k1 + _W1) & _MASK
    return c0, c1, c2, c3


STREAM_SWEEP = 0
STREAM_INIT = 1


def proposal_draw(seed, walker, t, n_bonds):
    """The draw for proposal t of a walker: (r in [0,1) with 53 bits, bond index 0-based)."""
    x = philox4x32_10((t & _MASK, (t >> 32) & _MASK, walker & _MASK, STREAM_SWEEP),
                      (seed & _MASK, (seed >> 32) & _MASK))
    u53 = ((x[0] >> 5) << 26) | (x[1] >> 6)
    r = u53 * (1.0 / 9007199254740992.0)
    b = (x[2] * n_bonds) >> 32
    return r, b


# ---------------------------------------------------------------------------
# One chain: src/MonteCarlo.jl:538-634
# ---------------------------------------------------------------------------

ACCEPT_REFERENCE = 0   # the reference's rule: stationary law |psi|^2 / Z_mu
ACCEPT_METROPOLIS = 1  # plain Metropolis on a uniform bond: stationary law |psi|^2


@dataclass
class ChainState:
    kappa_up: np.ndarray
    kappa_down: np.ndarray
    W_up: np.ndarray | None = None
    W_down: np.ndarray | None = None
    t: int = 0
    accepted: int = 0
    energies: list = field(default_factory=list)


def propose(st, nn, seed, walker, mode=ACCEPT_REFERENCE):
    """One Carlo.sweep! call (src/MonteCarlo.jl:538-591) with the Philox draw for proposal st.t.

    Returns (accepted, move) where move = (flag, i, site, l_up, l_down) or None.
    The reference draws r, then (only if r <= Z_mu/Z_max) a uniform bond, then a
    flag among the valid orientations; at most one orientation is valid when every
    site holds exactly one spin, so the flag draw carries no randomness here.
    """
    nb = len(nn)
    r, b = proposal_draw(seed, walker, st.t, nb)
    st.t += 1
    if mode == ACCEPT_REFERENCE:
        thr = Z(nn, st.kappa_up, st.kappa_down) / nb
        if r > thr:
            return False, None
    else:
        thr = 1.0
    i, site = nn[b]
    f1 = st.kappa_up[i - 1] != 0 and st.kappa_down[site - 1] != 0
    f2 = st.kappa_up[site - 1] != 0 and st.kappa_down[i - 1] != 0
    if not (f1 or f2):
        return False, None
    flag = 1 if f1 else 2
    l_up = int(st.kappa_up[i - 1] if flag == 1 else st.kappa_up[site - 1])
    l_down = int(st.kappa_down[site - 1] if flag == 1 else st.kappa_down[i - 1])
    if flag == 1:
        ratio = st.W_up[site - 1, l_up - 1] * st.W_down[i - 1, l_down - 1]
    else:
        ratio = st.W_up[i - 1, l_up - 1] * st.W_down[site - 1, l_down - 1]
    acc = float(np.real(ratio * np.conj(ratio)))
    move = (flag, i, site, l_up, l_down)
    if mode == ACCEPT_REFERENCE:
        ok = (acc >= 1 and r < thr) or (acc < 1 and r < thr * acc)
    else:
        ok = acc >= 1 or r < acc
    if ok:
        update_configurations(st, flag, i, site, l_up, l_down)
        st.accepted += 1
    return ok, move


def run_chain(ham_nn, U_up, U_down, st, seed, walker, n_proposals,
              refresh_every=None, measure_every=None, mode=ACCEPT_REFERENCE, ham=None):
    """Runs n_proposals proposals; after proposal t (0-based) it refreshes W when
    (t+1) % refresh_every == 0 (src/MonteCarlo.jl:594-604) and records E_L when
    (t+1) % measure_every == 0 (src/MonteCarlo.jl:628-634)."""
    n_occ = min(int(np.count_nonzero(st.kappa_up)), int(np.count_nonzero(st.kappa_down)))
    refresh_every = refresh_every or n_occ
    measure_every = measure_every or n_occ
    for _ in range(n_proposals):
        propose(st, ham_nn, seed, walker, mode)
        if st.t % refresh_every == 0:
            st.W_up = reevaluateW(U_up, st.kappa_up)
            st.W_down = reevaluateW(U_down, st.kappa_down)
        if ham is not None and st.t % measure_every == 0:
            st.energies.append(getOL(ham, st.W_up, st.W_down, st.kappa_up, st.kappa_down))
    return st


# ---------------------------------------------------------------------------
# Seeded random starts (the batched path's walker initialisation)
# ---------------------------------------------------------------------------

LOGDET_MIN = -25.0        # enumeration cut-off at N=24 (weights below exp(-50))
PIVOT_RATIO_MIN = 1e-8     # a start is usable when min|u_kk|/max|u_kk| of the pivoted LU exceeds this


def random_configuration(seed, walker, nsites, n_up, attempt=0):
    """Seeded uniformly random configuration with n_up up spins.

    Fisher-Yates over sites driven by the Philox stream (stream id 1, counter
    (attempt, walker)); up spins take labels 1..n_up and down spins labels
    1..n_down, both in increasing site order.
    """
    perm = list(range(nsites))
    ctr = 0
    words = []
    for k in range(nsites - 1, 0, -1):
        if not words:
            x = philox4x32_10((ctr & _MASK, attempt & _MASK, walker & _MASK, STREAM_INIT),
                              (seed & _MASK, (seed >> 32) & _MASK))
            words = list(x)
            ctr += 1
        u = words.pop(0)
        j = (u * (k + 1)) >> 32
        perm[k], perm[j] = perm[j], perm[k]
    up_sites = sorted(perm[:n_up])
    kup = np.zeros(nsites, dtype=np.int64)
    kdn = np.zeros(nsites, dtype=np.int64)
    for lab, s in enumerate(up_sites):
        kup[s] = lab + 1
    lab = 0
    for s in range(nsites):
        if kup[s] == 0:
            lab += 1
            kdn[s] = lab
    return kup, kdn


def logabsdet(U, kappa):
    return float(np.linalg.slogdet(tilde_U(U, kappa))[1])


def pivot_ratio(U, kappa):
    """min|u_kk| / max|u_kk| of the partially pivoted LU of tilde_U (LAPACK getrf)."""
    import scipy.linalg as sla
    d = np.abs(np.diag(sla.lu_factor(tilde_U(U, kappa), check_finite=False)[0]))
    return float(d.min() / d.max()) if d.max() > 0 else 0.0


def seeded_start(seed, walker, U_up, U_down, max_attempts=256):
    """Draw configurations until tilde_U is regular for both spins.

    Random half-filled configurations are either regular (pivot ratio
    1e-3..1e-1 at N=24..216) or exactly singular by symmetry (1e-14..1e-16),
    so the cut at PIVOT_RATIO_MIN separates them without depending on N.
    """
    N, n_up = np.asarray(U_up).shape
    for a in range(max_attempts):
        ku, kd = random_configuration(seed, walker, N, n_up, a)
        if pivot_ratio(U_up, ku) > PIVOT_RATIO_MIN and pivot_ratio(U_down, kd) > PIVOT_RATIO_MIN:
            return ku, kd, a
    raise RuntimeError("no non-singular configuration found")


# ---------------------------------------------------------------------------
# Exact enumeration (oracle addition, no reference counterpart)
# ---------------------------------------------------------------------------


def enumerate_energy(U, nn, chunk=100000):
    """Exact <E_L> over all C(N, N/2) configurations for a real U shared by both spins.

    Returns (E/N under |psi|^2, E/N under |psi|^2/Z_mu) -- the second is the
    stationary law of the reference sampler (src/MonteCarlo.jl:544-591).
    Configurations with log|det| < LOGDET_MIN in either spin carry weight
    below exp(-50) relative and are skipped.
    """
    U = np.asarray(U, dtype=float)
    N, h = U.shape
    nn0 = np.asarray(nn, dtype=np.int64) - 1
    combos = np.array(list(itertools.combinations(range(N), h)), dtype=np.int16)
    num = den = numz = denz = 0.0
    ref = None
    for s in range(0, len(combos), chunk):
        A = combos[s:s + chunk]
        c = len(A)
        up = np.zeros((c, N), bool)
        up[np.arange(c)[:, None], A] = True
        dn = ~up
        Bd = np.nonzero(dn)[1].reshape(c, N - h)
        Uu, Ud = U[A], U[Bd]
        _, lu = np.linalg.slogdet(Uu)
        _, ld = np.linalg.slogdet(Ud)
        ok = (lu > LOGDET_MIN) & (ld > LOGDET_MIN)
        A, Bd, Uu, Ud, lu, ld, up, dn = A[ok], Bd[ok], Uu[ok], Ud[ok], lu[ok], ld[ok], up[ok], dn[ok]
        c = len(A)
        rku = np.cumsum(up, 1) - 1
        rkd = np.cumsum(dn, 1) - 1
        Wu = U[None] @ np.linalg.inv(Uu)
        Wd = U[None] @ np.linalg.inv(Ud)
        ar = np.arange(c)
        sz = np.where(up, 0.5, -0.5)
        EL = np.zeros(c)
        Zm = np.zeros(c)
        for i, j in nn0:
            EL += sz[:, i] * sz[:, j]
            for a, b in ((j, i), (i, j)):
                m = up[:, a] & dn[:, b]
                EL += np.where(m, -0.5 * Wu[ar, b, rku[:, a]] * Wd[ar, a, rkd[:, b]], 0.0)
                Zm += m
        L = 2 * (lu + ld)
        if ref is None:
            ref = L.max()
        p = np.exp(L - ref)
        num += (p * EL).sum()
        den += p.sum()
        numz += (p / Zm * EL).sum()
        denz += (p / Zm).sum()
    return num / den / N, numz / denz / N


# ---------------------------------------------------------------------------
# Extended ansatz and its energy gradient (oracle addition, no reference
# counterpart).  The reference has the pi-flux hopping only; the family
# below adds a triangle flux theta and second-neighbour hops t2 + i*m*nu, and
# the gradient of E(t2, m, theta) is computed exactly (enumeration) from the
# log-derivatives O_a(x) = d ln psi(x) / d a.
# ---------------------------------------------------------------------------


def _min_image(lat, i, j, want):
    """Displacements r_j - r_i (0-based sites) over the periodic images whose
    squared length equals `want` to 1e-9 t^2."""
    ri, rj = get_site_coord(lat, i + 1), get_site_coord(lat, j + 1)
    L1, L2 = (lat.n1 // 2) * lat.a1, lat.n2 * lat.a2
    out = []
    for p in ((-1, 0, 1) if lat.PBC[0] else (0,)):
        for q in ((-1, 0, 1) if lat.PBC[1] else (0,)):
            d = rj - ri + p * L1 + q * L2
            if abs(d @ d - want) <= 1e-9 * lat.t ** 2:
                out.append(d)
    return out


def ansatz_hmat(lat, params, B=0.0, link_in=PI_LINK_IN, link_inter=PI_LINK_INTER):
    """H(t2, m, theta) and [dH/dt2, dH/dm, dH/dtheta].

    Triangles are found as mutually adjacent triples of the pi-flux H and
    oriented by the sign of their area; each directed edge i->j of a
    triangle gets exp(i theta s/3) with s = +1 counter-clockwise.  Second
    neighbours are the pairs at sqrt(3) t through a common neighbour j;
    H_ik += -(t2 + i m nu) g with g = sign(H0_ij H0_jk) and nu = +1 for a left
    turn at j.
    """
    t2, m, theta = (float(x) for x in params)
    H0 = hmat(lat, link_in, link_inter, B)
    Hp = hmat(lat, link_in, link_inter, 0.0)
    N = H0.shape[0]
    t = lat.t
    adj = [set(np.nonzero(Hp[i])[0]) - {i} for i in range(N)]
    disp = {}
    for i in range(N):
        for j in adj[i]:
            d = _min_image(lat, i, j, t * t)
            if len(d) != 1:
                raise ValueError(f"lattice too small for the extended ansatz ({i}, {j})")
            disp[i, j] = d[0]
    H = H0.astype(complex).copy()
    dT, dM, dTh = (np.zeros((N, N), complex) for _ in range(3))
    s_edge = {}
    for i in range(N):
        for j in adj[i]:
            for k in adj[i] & adj[j]:
                if i < j < k:
                    a = disp[i, j]
                    b = disp[i, k]
                    ccw = (a[0] * b[1] - a[1] * b[0]) > 0
                    order = (i, j, k) if ccw else (i, k, j)
                    for x, y in zip(order, order[1:] + order[:1]):
                        s_edge[x, y] = 1.0
                        s_edge[y, x] = -1.0
    for (i, j), s in s_edge.items():
        ph = complex(math.cos(theta * s / 3.0), math.sin(theta * s / 3.0))
        H[i, j] = H0[i, j] * ph
        dTh[i, j] = H[i, j] * complex(0.0, s / 3.0)
    for j in range(N):
        for i in adj[j]:
            for k in adj[j]:
                if i == k or k in adj[i]:
                    continue
                d = disp[i, j] + disp[j, k]
                if abs(d @ d - 3 * t * t) > 1e-9 * t * t:
                    continue
                g = 1.0 if Hp[i, j].real * Hp[j, k].real > 0 else -1.0
                cr = disp[i, j][0] * disp[j, k][1] - disp[i, j][1] * disp[j, k][0]
                nu = 1.0 if cr > 0 else -1.0
                H[i, k] += -complex(t2, m * nu) * g
                dT[i, k] += -g
                dM[i, k] += complex(0.0, -nu * g)
    return H, [dT, dM, dTh]


def orbital_derivatives(H, dHs, N_up, N_down):
    """U_sigma = lowest-N_sigma eigenvectors of H (as ``orbitals``) and their
    first-order derivatives dU[:, c] = sum_{m unoccupied} v_m (v_m^H dH v_c) / (e_c - e_m).

    Occupied-occupied mixing is left out: it rotates U inside its own span,
    which multiplies every determinant by one constant and so drops out of
    every expectation value.  Requires a gap above the last occupied level.
    """
    Hh = np.asarray(H)
    cplx = np.any(Hh.imag != 0) or any(np.any(np.asarray(d).imag != 0) for d in dHs)
    w, V = np.linalg.eigh(Hh if cplx else Hh.real)
    p = np.argsort(w, kind="stable")
    w, V = w[p], V[:, p]
    out = []
    for n in (N_up, N_down):
        if w[n] - w[n - 1] <= 1e-10:
            raise ValueError(f"no gap above level {n}: {w[n - 1]} {w[n]}")
        U, Vu = V[:, :n], V[:, n:]
        den = w[:n][None, :] - w[n:][:, None]          # (N - n) x n: e_c - e_m
        D = []
        for dH in dHs:
            dH = np.asarray(dH) if cplx else np.asarray(dH).real
            Bm = (Vu.conj().T @ dH @ U) / den
            D.append(Vu @ Bm)
        out.append((U.copy(), np.array(D)))
    return out[0][0], out[1][0], out[0][1], out[1][1]


def log_derivative(U, D, kappa):
    """O_a = tr(tilde_U^{-1} tilde_D_a) for one spin: d ln det tilde_U / d a."""
    tU = tilde_U(U, kappa)
    inv = np.linalg.inv(tU)
    return np.array([np.trace(inv @ tilde_U(Da, kappa)) for Da in D])


def local_energy_complex(nn, W_up, W_down, kappa_up, kappa_down):
    """E_L with its imaginary part kept (src/Hamiltonian.jl:762-778 before the real part is taken)."""
    E = 0.0 + 0.0j
    for (i, j) in nn:
        a, b = i - 1, j - 1
        E += 0.25 if (kappa_up[a] != 0) == (kappa_up[b] != 0) else -0.25
        for x, y in ((b, a), (a, b)):
            if kappa_up[x] != 0 and kappa_down[y] != 0:
                E -= 0.5 * W_up[y, kappa_up[x] - 1] * W_down[x, kappa_down[y] - 1]
    return E


def enumerate_gradient(U_up, U_down, D_up, D_down, nn, chunk=50000):
    """Exact E, dE/da and the SR matrix over all configurations with
    sum(kappa_up != 0) = N_up under |psi|^2 (oracle addition).

    Returns a dict with E (total energy), grad (dE/da), S (Re <O*_a O_b> -
    Re <O*_a><O_b>) and O (<O_a>).  Configurations with log|det| below
    LOGDET_MIN for either spin carry weight below exp(-50) relative and are
    skipped.
    """
    U_up, U_down = np.asarray(U_up, complex), np.asarray(U_down, complex)
    D_up, D_down = np.asarray(D_up, complex), np.asarray(D_down, complex)
    N, nu = U_up.shape
    nd = U_down.shape[1]
    A_ = len(D_up)
    nn0 = np.asarray(nn, dtype=np.int64) - 1
    combos = np.array(list(itertools.combinations(range(N), nu)), dtype=np.int16)
    ref = None
    acc = dict(w=0.0, E=0j, O=np.zeros(A_, complex), OE=np.zeros(A_, complex), OO=np.zeros((A_, A_), complex))
    for s in range(0, len(combos), chunk):
        A = combos[s:s + chunk]
        c = len(A)
        up = np.zeros((c, N), bool)
        up[np.arange(c)[:, None], A] = True
        dn = ~up
        Bd = np.nonzero(dn)[1].reshape(c, nd)
        Uu, Ud = U_up[A], U_down[Bd]
        _, lu = np.linalg.slogdet(Uu)
        _, ld = np.linalg.slogdet(Ud)
        ok = (lu > LOGDET_MIN) & (ld > LOGDET_MIN)
        A, Bd, Uu, Ud, lu, ld, up, dn = A[ok], Bd[ok], Uu[ok], Ud[ok], lu[ok], ld[ok], up[ok], dn[ok]
        c = len(A)
        iu, idn = np.linalg.inv(Uu), np.linalg.inv(Ud)
        Wu, Wd = U_up[None] @ iu, U_down[None] @ idn
        rku = np.cumsum(up, 1) - 1
        rkd = np.cumsum(dn, 1) - 1
        ar = np.arange(c)
        sz = np.where(up, 0.5, -0.5)
        EL = np.zeros(c, complex)
        for i, j in nn0:
            EL += sz[:, i] * sz[:, j]
            for a, b in ((j, i), (i, j)):
                msk = up[:, a] & dn[:, b]
                EL += np.where(msk, -0.5 * Wu[ar, b, rku[:, a]] * Wd[ar, a, rkd[:, b]], 0.0)
        O = np.zeros((c, A_), complex)
        for k in range(A_):
            O[:, k] = np.einsum("cij,cji->c", iu, D_up[k][A]) + np.einsum("cij,cji->c", idn, D_down[k][Bd])
        L = 2 * (lu + ld)
        if ref is None:
            ref = L.max()
        p = np.exp(L - ref)
        acc["w"] += p.sum()
        acc["E"] += (p * EL).sum()
        acc["O"] += (p[:, None] * O).sum(0)
        acc["OE"] += (p[:, None] * O.conj() * EL[:, None]).sum(0)
        acc["OO"] += np.einsum("c,ca,cb->ab", p, O.conj(), O)
    w = acc["w"]
    E, O, OE, OO = acc["E"] / w, acc["O"] / w, acc["OE"] / w, acc["OO"] / w
    grad = 2 * np.real(OE - O.conj() * E)
    S = np.real(OO - np.outer(O.conj(), O))
    return dict(E=float(E.real), E_imag=float(E.imag), grad=grad, S=S, O=O)
