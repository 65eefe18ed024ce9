"""Runtime features around the kernels: CUDA-graph replay, the autotuner, status words."""
import os

import numpy as np
import pytest

from helpers import BIN_KEYS, ising_spins, lj_configs

pytestmark = pytest.mark.gpu


def lj_batch(gpu, oracle, W=16, n=31, seed=4, lpw=0):
    R = 2.5
    confs = lj_configs(oracle, n, R, range(60, 60 + W))
    cfg = gpu.make_config(gpu.LJ, W, n, energy_bin=0.134, max_allowed=0.0, e_lo=-140, e_hi=1,
                          target_rate=0.5, translation_scale=0.1, seed=seed, lanes_per_walker=lpw)
    b = gpu.Batch(cfg, [(n, R, (0, 0, 0))] * W)
    b.upload(confs)
    b.initialize()
    return b


def snapshot(b):
    return [(b.bins(w), b.scalars(w), b.state(w)) for w in range(b.W)]


def assert_same(s1, s2):
    for (b1, c1, p1), (b2, c2, p2) in zip(s1, s2):
        assert b1["min"] == b2["min"]
        for k in BIN_KEYS:
            assert np.array_equal(b1[k], b2[k]), k
        assert c1 == c2
        assert np.array_equal(p1, p2)


@pytest.mark.parametrize("lpw", [8, 1])
def test_graph_replay_equals_direct_launches(gpu, oracle, monkeypatch, lpw):
    a = lj_batch(gpu, oracle, lpw=lpw)
    for _ in range(3):
        a.run(3000)  # captured once, replayed twice
    monkeypatch.setenv("SADMC_NO_GRAPHS", "1")
    b = lj_batch(gpu, oracle, lpw=lpw)
    b.run(9000)
    assert_same(snapshot(a), snapshot(b))


def test_autotune_restores_state_and_picks_a_candidate(gpu, oracle, tmp_path, monkeypatch):
    monkeypatch.setenv("SADMC_TUNE_CACHE", str(tmp_path / "tune.txt"))
    b = lj_batch(gpu, oracle, W=64)
    b.run(500)
    before = snapshot(b)
    lpw, ms = b.autotune(moves=512)
    assert lpw in (1, 2, 4, 8, 16, 32) and ms > 0
    assert b.lanes_per_walker() == lpw
    assert_same(before, snapshot(b))
    line = open(tmp_path / "tune.txt").read().split()
    assert int(line[1]) == lpw
    # a new handle of the same shape picks the recorded result
    c = lj_batch(gpu, oracle, W=64)
    assert c.lanes_per_walker() == lpw


@pytest.mark.parametrize("lpw", [1, 2, 4, 8, 16, 32])
def test_lanes_per_walker_variants_agree(gpu, oracle, lpw):
    """Every lane layout runs the same Markov chain: decisions depend on binary32 sums
    whose order changes with the layout, so compare statistics, not bits."""
    b = lj_batch(gpu, oracle, W=32, lpw=lpw)
    b.run(4000)
    m, a = b.counters()
    assert m == 32 * 4000
    assert 0.2 < a / m < 0.9
    assert not b.status().any()


def test_bin_range_is_flagged_not_faulted(gpu):
    """A proposal beyond the preallocated bins is rejected and flagged (the reference
    would grow its vectors)."""
    L, W = 8, 4
    cfg = gpu.make_config(gpu.ISING, W, L, e_lo=-16, e_hi=16, seed=1)  # far narrower than [-128, 128]
    spins = [ising_spins(L, 5 + w) for w in range(W)]
    b = gpu.Batch(cfg, [(L, 0.0, (0, 0, 0))] * W)
    b.upload(spins)
    b.initialize()
    b.run(20000)
    st = b.status()
    assert (st & gpu.ST_BIN_RANGE).any()
    assert not (st & ~np.uint32(gpu.ST_BIN_RANGE)).any()
    E = b.energies()
    # the planes hold the configured range plus two guard bins on each side
    assert np.all(E >= -16 - 2 * 4) and np.all(E <= 16 + 2 * 4)
    np.testing.assert_array_equal(E, b.compute_energies())
