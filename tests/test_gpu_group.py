"""Groups of handles advanced by one captured CUDA graph (kvmc_group_*):
walkers of three lattice sizes (N = 54, 216, 384) with their own delayed-update
depths, refresh intervals and W placements.  Every walker must make exactly
the asked accepted moves and follow the same chain as when its handle is
advanced on its own (bit for bit: the same kernels act on each walker in the
same order), and the chains follow the C oracle."""
import numpy as np
import pytest

import kagome_oracle as o
import oracle_c

pytestmark = pytest.mark.gpu

CELLS = {54: (3, 3), 216: (6, 6), 384: (8, 8)}
CLASSES = [(54, 24, dict(delay_k=8, refresh_interval=64)),
           (216, 12, dict(delay_k=12, refresh_interval=128, w_placement="hbm")),
           (384, 6, dict(delay_k=8, refresh_interval=256))]


@pytest.fixture(scope="module")
def kv(built):
    import kagomevmc

    return kagomevmc


def hams(kv):
    out = {}
    for N, _, _ in CLASSES:
        a, b = CELLS[N]
        out[N] = kv.Hamiltonian.build(N // 2, N // 2, kv.DoubleKagome(1.0, 2 * a, b, (True, True), (False, True)))
    return out


def engines(kv, H, seed):
    es = []
    for N, walkers, kw in CLASSES:
        e = kv.Engine(H[N], walkers, precision="mixed", seed=seed + N, **kw)
        e.init()
        es.append(e)
    return es


def test_group_matches_handles_advanced_alone(kv):
    H = hams(kv)
    A = 150
    grouped = engines(kv, H, 5)
    alone = engines(kv, H, 5)
    g = kv.Group(grouped)
    for _ in range(2):
        stats, ms = g.advance(A)
        assert ms > 0
        for e, st in zip(alone, stats):
            e.advance(A)
    for (N, walkers, _), eg, ea, st in zip(CLASSES, grouped, alone, stats):
        ws = eg.walker_stats()
        assert np.all(ws["accepted"] == 2 * A), N
        assert st["accepted"] == walkers * A and st["bad_walkers"] == 0
        sg, sa = eg.get_state(), ea.get_state()
        assert all(np.array_equal(x, y) for x, y in zip(sg, sa)), N
        np.testing.assert_array_equal(ws["sum_e"], ea.walker_stats()["sum_e"])
    g.close()
    for e in grouped + alone:
        e.close()


def test_group_chains_follow_the_oracle(kv):
    H = hams(kv)
    es = engines(kv, H, 9)
    starts = [e.get_state() for e in es]
    g = kv.Group(es)
    g.advance(120)
    for (N, walkers, kw), e, (ku0, kd0, _) in zip(CLASSES, es, starts):
        ku1, kd1, ct = e.get_state()
        m = oracle_c.OracleModel(H[N].U_up, H[N].U_down, H[N].nn)
        match = 0
        for w in range(walkers):
            ch = m.new_chain(ku0[w], kd0[w])
            ch.run(9 + N, w, int(ct[w]), N // 2, N // 2, 0)
            match += int(np.array_equal(ch.ku, ku1[w]) and np.array_equal(ch.kd, kd1[w]))
        assert match >= walkers - 1, (N, match)
    g.close()
    for e in es:
        e.close()


def test_group_rejects_mixed_devices_and_duplicates(kv):
    H = hams(kv)
    e = kv.Engine(H[54], 4, precision="mixed")
    with pytest.raises(kv.KvmcError):
        kv.Group([e, e])
    e.close()
