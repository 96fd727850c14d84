"""Host side of the library without a GPU: the C ABI loads and exports every
declared symbol, the FP64 hopping-matrix builder and bond list match the
oracle bit for bit, and argument errors carry the reference's error classes."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import kagome_oracle as o

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "kvmc.h")).read()
    return sorted(set(re.findall(r"KVMC_API\s+int\s+(kvmc_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(built):
    import kagomevmc as kv

    lib = kv.load()
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(kv.EXPORTS)


def test_version(built):
    import kagomevmc as kv

    abi, arch = C.c_int32(), C.c_int32()
    assert kv.load().kvmc_version(C.byref(abi), C.byref(arch)) == 0
    assert abi.value == 4 and arch.value == 1030


@pytest.mark.parametrize("n1,n2,pbc,anti,B", [
    (4, 3, (False, False), (False, False), 0.0), (4, 3, (True, False), (False, False), 0.0),
    (4, 3, (True, True), (True, True), 0.0), (4, 3, (True, True), (True, False), 0.1),
    (4, 2, (True, True), (False, True), 0.0), (6, 3, (True, True), (False, True), 0.0),
    (8, 4, (True, True), (False, True), 0.3), (2, 2, (False, False), (False, False), 0.0),
    (12, 6, (True, True), (False, True), 0.0)])
def test_hopping_matrix_and_bonds_match_oracle_exactly(built, n1, n2, pbc, anti, B):
    import kagomevmc as kv

    Ho = o.hmat(o.double_kagome(1.0, n1, n2, pbc, anti), B=B)
    Hk = kv.Hmat(kv.DoubleKagome(1.0, n1, n2, pbc, anti), B=B)
    assert np.array_equal(Ho, Hk)
    assert kv.get_nn(Hk) == [(i - 1, j - 1) for i, j in o.get_nn(Ho)]


def test_custom_links_zero_flux_shape(built):
    """Custom link tables (the reference's link_in / link_inter keywords)."""
    import kagomevmc as kv

    lin = {k: abs(v) for k, v in kv.PI_LINK_IN.items()}
    lint = {k: abs(v) for k, v in kv.PI_LINK_INTER.items()}
    L = kv.DoubleKagome(1.0, 4, 2, (True, True), (False, True))
    Lo = o.double_kagome(1.0, 4, 2, (True, True), (False, True))
    assert np.array_equal(kv.Hmat(L, lin, lint), o.hmat(Lo, lin, lint))


@pytest.mark.parametrize("n1,n2,pbc,anti,B", [(6, 3, (True, True), (True, True), 0.2),
                                              (8, 2, (True, False), (True, False), 0.05),
                                              (4, 4, (False, True), (False, True), 0.0)])
def test_hopping_builder_with_wide_and_wrapping_links(built, n1, n2, pbc, anti, B):
    """Inter-cell keys two cells away and keys that only an image reaches: the
    builder that visits (cell, link, image) triples gives the oracle's
    cell-pair loop (src/Hamiltonian.jl:333-343) bit for bit, accumulation
    order included."""
    import kagomevmc as kv

    lint = dict(kv.PI_LINK_INTER)
    lint.update({(1, 2, 2, 0): 0.5, (4, 3, -2, 1): -0.25, (6, 1, 1, 2): 0.75, (2, 5, 0, -3): 0.3})
    L = kv.DoubleKagome(1.0, n1, n2, pbc, anti)
    Lo = o.double_kagome(1.0, n1, n2, pbc, anti)
    assert np.array_equal(kv.Hmat(L, kv.PI_LINK_IN, lint, B=B), o.hmat(Lo, kv.PI_LINK_IN, lint, B=B))


def test_hopping_builder_scales_linearly(built):
    """12 x 12 doubled cells (N=864): the couplings take O(N) work, so the
    whole dense build (an N x N output) takes well under a second."""
    import time

    import kagomevmc as kv

    L = kv.DoubleKagome(1.0, 24, 12, (True, True), (False, True))
    t0 = time.perf_counter()
    H = kv.Hmat(L)
    assert time.perf_counter() - t0 < 1.0
    # 4-regular, |t| = 1: 2N bonds
    assert len(kv.get_nn(H)) == 2 * 864 and np.allclose(np.abs(H[np.abs(H) > 0]), 1.0)


def test_lattice_errors(built):
    import kagomevmc as kv

    with pytest.raises(kv.ArgumentError):
        kv.DoubleKagome(1.0, 3, 3, (False, False))
    with pytest.raises(kv.ArgumentError):
        kv.DoubleKagome(1.0, 4, 3, (False, False), (True, False))
    assert kv.ns(kv.DoubleKagome(1.0, 4, 3, (False, False))) == 36


def test_bad_link_table_is_rejected(built):
    import kagomevmc as kv

    with pytest.raises(kv.ArgumentError):
        kv.Hmat(kv.DoubleKagome(1.0, 4, 2, (True, True)), {(1, 7): 1.0})


def test_create_validates_before_touching_a_device(built):
    import kagomevmc as kv

    L = kv.DoubleKagome(1.0, 4, 2, (True, True), (False, True))
    ham = kv.Hamiltonian.build(12, 12, L)
    bad = kv.Hamiltonian(12, 11, ham.U_up, ham.U_down[:, :11], ham.H_mat, ham.nn)
    with pytest.raises(kv.ArgumentError):
        kv.Engine(bad, 2)
    bad = kv.Hamiltonian(12, 12, ham.U_up, ham.U_down, ham.H_mat, [(0, 99)])
    with pytest.raises(kv.BoundsError):
        kv.Engine(bad, 2)
    # a bond given twice (in either orientation) is refused
    i, j = ham.nn[0]
    bad = kv.Hamiltonian(12, 12, ham.U_up, ham.U_down, ham.H_mat, list(ham.nn) + [(j, i)])
    with pytest.raises(kv.ArgumentError, match="more than once"):
        kv.Engine(bad, 2)


def test_complex_orbitals_beyond_the_shared_memory_refresh_are_accepted(built):
    """A field at 8x10 cells (240 sites, 120 orbitals per spin) exceeds the
    shared-memory complex refresh (112 orbitals); kvmc_create accepts it (the
    refresh then factorises tilde_U in HBM) and, without a GPU, stops at the
    device check, not at the model's size."""
    import math

    import kagomevmc as kv

    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = kv.DoubleKagome(1.0, 8, 10, (True, True), (False, True))
    H = kv.Hmat(L, B=math.pi / (8 * 10 * 2 * math.sqrt(3)))
    Uu, Ud = kv.orbitals(H, 120, 120)
    assert np.iscomplexobj(Uu)
    with pytest.raises(kv.DeviceError):
        kv.Engine(kv.Hamiltonian(120, 120, Uu, Ud, H, kv.get_nn(H)), 2)


def test_no_device_is_a_clean_error_on_cpu(built):
    import kagomevmc as kv

    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = kv.DoubleKagome(1.0, 4, 2, (True, True), (False, True))
    with pytest.raises(kv.DeviceError):
        kv.Engine(kv.Hamiltonian.build(12, 12, L), 2)


def test_carlo_context_and_evaluator_host_logic(built):
    """The measurement sink and evaluables of the Carlo-facing surface (no GPU)."""
    import kagomevmc as kv

    ctx = kv.MCContext()
    for v in (1.0, 2.0, 3.0):
        ctx.measure("OL", v)
    assert ctx.observables["OL"] == [1.0, 2.0, 3.0] and ctx.sweeps == 0
    ev = kv.Evaluator()
    kv.register_evaluables(kv.MC, ev, dict(n1=4, n2=2))
    res = ev.run(ctx.observables)
    assert res["energy"] == pytest.approx(2.0 / 24)
