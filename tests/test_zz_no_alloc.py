"""kvmc_refresh_static -- the refresh entry point that allocates nothing.

It serves callers that cannot allocate device memory themselves, such as
Monte Carlo code whose GPU memory belongs to another allocator (a Julia
CUDA.jl pool, a framework's caching allocator), or code that must not hit
cudaMalloc's device synchronisation mid-loop.  It solves in a fixed array
compiled into the library and writes into the caller's own buffers.

The test drives it through the C ABI.  It makes two calls in a row with
different configurations, so the second call cannot pass on what the first
left in the shared array.  Each call is checked against W from the existing
entry point (kvmc_init with given configurations, then kvmc_get_w, plain FP64
form) and against the oracle's reevaluateW, at the tolerance of the other
FP64 parity tests: 1e-10 relative to max|W|.  Items whose configuration is
singular or has the wrong number of occupied sites leave their W untouched.
This file sorts last so that a run stopping at its first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C
import os

import numpy as np
import pytest

import kagome_oracle as o

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CELLS = {54: (3, 3), 216: (6, 6)}


@pytest.fixture(scope="module")
def kv(built):
    import kagomevmc

    return kagomevmc


def _ham(kv, N):
    a, b = CELLS[N]
    return kv.Hamiltonian.build(N // 2, N // 2, kv.DoubleKagome(1.0, 2 * a, b, (True, True), (False, True)))


def _existing_entry(kv, ham, ku):
    """W_up from the handle API (kvmc_create, kvmc_init, kvmc_get_w), plain FP64."""
    N = ham.U_up.shape[0]
    eng = kv.Engine(ham, len(ku), precision="plain")
    # the handle wants full configurations: down spins on the sites the up spins leave empty
    kd = np.zeros_like(ku)
    for w in range(len(ku)):
        empty = np.nonzero(ku[w] == 0)[0]
        kd[w, empty] = np.arange(1, len(empty) + 1)
    eng.init(ku, kd)
    Wu, _ = eng.get_w()
    eng.close()
    assert Wu.shape == (len(ku), N, ham.U_up.shape[1])
    return Wu


@pytest.mark.parametrize("N", [54, 216])
def test_static_refresh_matches_existing_entry_on_two_calls(kv, N):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    ham = _ham(kv, N)
    n = ham.U_up.shape[1]
    lib = kv.load()
    dev = torch.device("cuda", 0)
    U = torch.tensor(np.ascontiguousarray(ham.U_up), dtype=torch.float64, device=dev)    # row-major [N][n]
    batch = 6
    for call, seed in enumerate((101, 202)):
        ku = np.stack([o.seeded_start(seed, w, ham.U_up, ham.U_down)[0] for w in range(batch)]).astype(np.int32)
        kappa = torch.tensor(ku, dtype=torch.int32, device=dev)
        W = torch.full((batch, N, n), float("nan"), dtype=torch.float64, device=dev)
        logdet = torch.zeros(batch, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = lib.kvmc_refresh_static(N, n, batch, C.c_void_p(U.data_ptr()), C.c_void_p(kappa.data_ptr()),
                                     C.c_void_p(W.data_ptr()), C.c_void_p(logdet.data_ptr()), None)
        assert rc == 0, (call, rc)
        torch.cuda.synchronize()
        got = W.cpu().numpy()
        want = _existing_entry(kv, ham, ku)
        for w in range(batch):
            tol = 1e-10 * max(1.0, np.abs(want[w]).max())
            assert np.abs(got[w] - want[w]).max() <= tol, (call, w)
            # and against the oracle's reevaluateW directly
            exact = o.reevaluateW(ham.U_up, ku[w])
            assert np.abs(got[w] - exact).max() <= 1e-10 * max(1.0, np.abs(exact).max()), (call, w)
            assert np.isfinite(logdet[w].item())
            assert logdet[w].item() == pytest.approx(o.logabsdet(ham.U_up, ku[w]), abs=1e-9)


def test_static_refresh_leaves_bad_items_untouched(kv):
    """One item with a repeated label (tilde_U then has a zero row: logdet
    -inf) and one with a site too few occupied (logdet NaN) between two good
    items: the bad items' W keep their NaN fill, the good ones match the
    oracle's reevaluateW."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    ham = _ham(kv, 54)
    N, n = ham.U_up.shape
    lib = kv.load()
    dev = torch.device("cuda", 0)
    ku = np.stack([o.seeded_start(303, w, ham.U_up, ham.U_down)[0] for w in range(4)]).astype(np.int32)
    occ = np.nonzero(ku[1])[0]
    ku[1, occ[1]] = ku[1, occ[0]]            # label repeated, another label missing
    ku[2, np.nonzero(ku[2])[0][0]] = 0        # n - 1 occupied sites
    U = torch.tensor(np.ascontiguousarray(ham.U_up), dtype=torch.float64, device=dev)
    kappa = torch.tensor(ku, dtype=torch.int32, device=dev)
    W = torch.full((4, N, n), float("nan"), dtype=torch.float64, device=dev)
    logdet = torch.zeros(4, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = lib.kvmc_refresh_static(N, n, 4, C.c_void_p(U.data_ptr()), C.c_void_p(kappa.data_ptr()),
                                 C.c_void_p(W.data_ptr()), C.c_void_p(logdet.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    got, ld = W.cpu().numpy(), logdet.cpu().numpy()
    assert ld[1] == -np.inf and np.isnan(ld[2])
    assert np.all(np.isnan(got[1])) and np.all(np.isnan(got[2]))
    for w in (0, 3):
        exact = o.reevaluateW(ham.U_up, ku[w])
        assert np.abs(got[w] - exact).max() <= 1e-10 * max(1.0, np.abs(exact).max()), w
        assert ld[w] == pytest.approx(o.logabsdet(ham.U_up, ku[w]), abs=1e-9)


def test_static_refresh_rejects_batches_beyond_its_array(kv):
    """216 sites, 108 orbitals: 108 * 108 * 8 B per item, so 90 items exceed the 8 MiB array."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = kv.load()
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    assert lib.kvmc_refresh_static(216, 108, 90, p, p, p, None, None) == 1   # KVMC_ERR_ARGUMENT
    assert lib.kvmc_refresh_static(400, 200, 1, p, p, p, None, None) == 7    # more than 160 orbitals
