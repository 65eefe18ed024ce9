"""Delayed-acceptance LJ moves screened by the learned surrogate.

With a constant surrogate the first stage always accepts without drawing, so the chain
must be the plain chain bit for bit; with a trained surrogate the screen rejects moves
before the exact evaluation while the sampled energies stay those of the plain chain."""
import numpy as np
import pytest

from helpers import BIN_KEYS, lj_configs

pytestmark = pytest.mark.gpu


def lj_batch(gpu, oracle, n, W, R, seed, lpw=32):
    confs = lj_configs(oracle, n, R, range(500, 500 + W))
    cfg = gpu.make_config(gpu.LJ, W, n, energy_bin=0.1, max_allowed=0.0, e_lo=-80, e_hi=1,
                          min_T=0.1, target_rate=0.5, translation_scale=0.1, seed=seed,
                          lanes_per_walker=lpw)
    b = gpu.Batch(cfg, [(n, R, (0, 0, 0))] * W)
    b.upload(confs)
    b.initialize()
    return b


def test_constant_surrogate_reproduces_the_plain_chain(gpu, oracle):
    n, W, R, moves = 13, 8, 2.5, 6000
    plain = lj_batch(gpu, oracle, n, W, R, seed=9)
    plain.run(moves)
    da = lj_batch(gpu, oracle, n, W, R, seed=9)
    da.surrogate_init(seed=1)
    da.surrogate_set_params(np.zeros(da.SG_NPARAM, np.float32))
    stats = da.run_da(moves)
    assert (stats[:, 0] == 0).all() and (stats[:, 1] == moves).all()
    for w in range(W):
        x, y = plain.bins(w), da.bins(w)
        assert x["min"] == y["min"]
        for k in BIN_KEYS:
            assert np.array_equal(x[k], y[k]), (w, k)
        assert plain.scalars(w) == da.scalars(w)
        assert np.array_equal(plain.state(w), da.state(w))


def test_trained_surrogate_screens_and_keeps_the_distribution(gpu, oracle):
    n, W, R = 13, 64, 2.5
    da = lj_batch(gpu, oracle, n, W, R, seed=3)
    da.surrogate_init(seed=2, ring_capacity=8192)
    for _ in range(40):
        da.run(400)
        da.surrogate_collect()
    loss = da.surrogate_train(600, batch=256, lr=2e-3, seed=4)
    assert loss < 5.0, loss   # mean squared configuration-energy error (epsilon^2)
    stats = da.run_da(20000)
    screened = stats[:, 0].sum() / (stats.sum())
    assert 0.02 < screened < 0.9, screened
    plain = lj_batch(gpu, oracle, n, W, R, seed=3)
    plain.run(16000 + 20000)
    # both ensembles visit the same energies: compare walker-averaged mean energy per
    # bin-weighted histogram over the last stretch through the bins' energy sums
    def mean_energy(b):
        tot, cnt = 0.0, 0
        for w in range(b.W):
            bb = b.bins(w)
            tot += bb["sumE"].sum()
            cnt += int(bb["hist"].sum())
        return tot / cnt
    a, p = mean_energy(da), mean_energy(plain)
    assert abs(a - p) < 0.05 * abs(p), (a, p)
