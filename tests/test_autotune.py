"""The autotuner's selection and cache logic on the CPU, with a stand-in
engine whose speed and drift depend on the candidate: the fastest candidate
within the drift bound wins, candidates that do not fit are skipped, the
choice round-trips through the cache, and the shipped table holds the
workloads the bench reads."""
import json

import numpy as np
import pytest


@pytest.fixture(scope="module")
def kv(built):
    import kagomevmc

    return kagomevmc


class FakeEngine:
    """Rate = f(placement, threads, k, R); drift grows with R; chip does not fit at k=16."""

    def __init__(self, ham, walkers, precision="mixed", accept="reference", seed=0, refresh_interval=0, device=0,
                 delay_k=0, w_placement="auto", **kw):
        import kagomevmc

        if w_placement == "chip" and delay_k == 16:
            raise kagomevmc.KvmcError(7, "does not fit")
        self.k, self.R, self.place, self.walkers, self.threads = delay_k, refresh_interval, w_placement, walkers, 256
        self.warp = 0

    def set_stream_threads(self, th):
        self.threads = th

    def set_warp_walkers(self, wp):
        self.warp = wp

    def set_accuracy_guard(self, hi, lo):
        self.guard = (hi, lo)

    def config(self):
        return dict(delay_k=self.k, refresh_interval=self.R, measure_interval=1, w_on_chip=self.place == "chip")

    def init(self):
        pass

    def advance(self, moves):
        return dict(accepted=moves * self.walkers, refreshes=self.walkers)

    def region_start(self):
        pass

    def region_stop(self):
        speed = 1.0 + 0.1 * self.k + (0.5 if self.place == "hbm" else 0.0) + (0.2 if self.threads == 128 else 0.0)
        speed += 0.05 * self.warp
        speed *= 1.0 + np.log2(self.R) / 10
        return 1000.0 / speed

    def walker_drift(self):
        return np.full(self.walkers, 1e-6 * self.R * (1 + self.k / 4))

    def close(self):
        pass


def test_tuner_picks_fastest_within_drift_bound(kv, monkeypatch, tmp_path):
    from kagomevmc import autotune, montecarlo

    monkeypatch.setattr(montecarlo, "Engine", FakeEngine)
    ham = kv.Hamiltonian(2, 2, np.eye(4)[:, :2], np.eye(4)[:, 2:], np.zeros((4, 4)), [(0, 1)])
    cache = str(tmp_path / "tuned.json")
    ch = autotune.tune(ham, 64, cache_path=cache, drift_bound=5e-3)
    # the largest R whose drift 1e-6 R (1 + k/4) stays within 5e-3, at the fastest (k, placement, threads)
    for row in ch.trials:
        assert not (row["placement"] == "chip" and row["delay_k"] == 16)
    ok = [r for r in ch.trials if r["max_drift"] <= 5e-3]
    best = max(ok, key=lambda r: r["moves_per_s"])
    assert (ch.delay_k, ch.refresh_interval, ch.placement, ch.threads, ch.warp) == (
        best["delay_k"], best["refresh_interval"], best["placement"], best["threads"], best["warp"])
    assert ch.warp == 14 and (ch.guard_hi, ch.guard_lo) == autotune.GUARD   # the fastest shape of the stand-in
    assert ch.max_drift <= 5e-3
    # cached: a second call returns the same choice without trials
    ch2 = autotune.tune(ham, 64, cache_path=cache)
    assert (ch2.delay_k, ch2.refresh_interval, ch2.placement) == (ch.delay_k, ch.refresh_interval, ch.placement)
    assert autotune.lookup(ham, 64, path=cache).refresh_interval == ch.refresh_interval
    assert autotune.lookup(ham, 65, path=cache) is None   # another batch size is another workload


def test_shipped_table_covers_the_bench_workloads(kv):
    from kagomevmc import autotune

    table = json.load(open(autotune.SHIPPED))
    for key in ("N216_nu108_nd108_W2048_reference_r_GB300", "N96_nu48_nd48_W4096_reference_r_GB300",
                "N54_nu27_nd27_W1024_reference_r_GB300", "N216_nu108_nd108_W768_reference_r_GB300",
                "N384_nu192_nd192_W256_reference_r_GB300", "N192_nu98_nd94_W2048_reference_c_GB300"):
        row = table[key]
        assert row["placement"] in ("chip", "hbm") and row["delay_k"] in (1, 4, 8, 12, 16)
        assert row["refresh_interval"] > 0 and row["threads"] in (128, 256)
        assert row.get("warp", 0) in (0, 2, 4, 7, 10, 14)


def test_tuner_without_a_candidate_inside_the_bound(kv, monkeypatch):
    """When every candidate drifts past the bound (as at N=864), the tuner
    takes the most frequent refresh, and the fastest candidate at it."""
    from kagomevmc import autotune, montecarlo

    monkeypatch.setattr(montecarlo, "Engine", FakeEngine)
    ham = kv.Hamiltonian(2, 2, np.eye(4)[:, :2], np.eye(4)[:, 2:], np.zeros((4, 4)), [(0, 1)])
    ch = autotune.tune(ham, 64, drift_bound=1e-12)
    assert all(r["max_drift"] > 1e-12 for r in ch.trials)
    r_min = min(r["refresh_interval"] for r in ch.trials)
    fastest = max((r for r in ch.trials if r["refresh_interval"] == r_min), key=lambda r: r["moves_per_s"])
    assert ch.refresh_interval == r_min
    assert (ch.delay_k, ch.placement, ch.threads) == (fastest["delay_k"], fastest["placement"], fastest["threads"])


def test_field_workload_is_in_the_shipped_table(kv):
    """The complex field workload the bench runs (8x8 doubled cells, imbalance
    4) resolves to its row of the shipped table."""
    from kagomevmc import autotune
    from kagomevmc.tune_shipped import field_model

    ham = field_model()
    assert np.iscomplexobj(ham.U_up) and ham.U_up.shape == (192, 98) and ham.U_down.shape == (192, 94)
    ch = autotune.lookup(ham, 2048)
    assert ch is not None and ch.placement == "hbm" and ch.delay_k in (4, 8) and ch.refresh_interval > 0
