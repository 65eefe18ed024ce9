"""Delayed-acceptance LJ moves screened by the learned surrogate.

With a constant surrogate the first stage always accepts without drawing, so the chain
must be the plain chain bit for bit; with a trained surrogate the screen rejects moves
before the exact evaluation while the sampled energies stay those of the plain chain."""
import numpy as np
import pytest

from helpers import BIN_KEYS, assert_bins_equal, assert_scalars_equal, lj_configs, sphere_configs

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


def _production_hist(b, before):
    """Per-walker histograms accumulated since `before` (walker -> {bin centre: count})."""
    out = []
    for w in range(b.W):
        bb = b.bins(w)
        centres = bb["min"] + bb["width"] * (np.arange(len(bb["hist"])) + 0.5)
        h = {round(float(c), 6): int(x) for c, x in zip(centres, bb["hist"])}
        out.append({c: x - before[w].get(c, 0) for c, x in h.items()})
    return out


def test_trained_surrogate_keeps_the_distribution_at_fixed_weights(gpu, oracle, tmp_path):
    """With ln w frozen (Wang-Landau production: gamma drops below min_gamma at the first
    flat histogram and is then 0) the plain chain samples P(E) ~ g(E) exp(-ln w(E)), and
    so must the delayed-acceptance chain, whatever its surrogate.  Both continue from one
    checkpoint; their walker-averaged mean production energies must agree within sampling
    noise (walker-to-walker spread), and their histograms closely."""
    n, W, R = 13, 64, 2.5
    confs = lj_configs(oracle, n, R, range(500, 500 + W))
    cfg = gpu.make_config(gpu.LJ, W, n, method=2, min_gamma=0.6, energy_bin=1.0,
                          min_allowed=-28.0, max_allowed=0.0, e_lo=-31, e_hi=2,
                          translation_scale=0.1, seed=3, lanes_per_walker=32)
    da = gpu.Batch(cfg, [(n, R, (0, 0, 0))] * W)
    da.upload(confs)
    da.initialize()
    da.surrogate_init(seed=2, ring_capacity=8192)
    for _ in range(200):
        da.run(2000)
        da.surrogate_collect()
        if all(da.scalars(w)["gamma"] == 0.0 for w in range(W)):
            break
    assert all(da.scalars(w)["gamma"] == 0.0 for w in range(W)), "not every walker in production"
    loss = da.surrogate_train(400, batch=256, lr=2e-3, seed=4)
    assert loss < 5.0, loss   # mean squared configuration-energy error (epsilon^2)
    da.checkpoint(str(tmp_path / "fork.ck"))
    plain = gpu.Batch.resume(str(tmp_path / "fork.ck"))
    before = _production_hist(da, [{}] * W)
    moves = 30000
    stats = da.run_da(moves)
    plain.run(moves)
    screened = stats[:, 0].sum() / stats.sum()
    assert 0.02 < screened < 0.9, screened
    hd, hp = _production_hist(da, before), _production_hist(plain, before)
    for h in hd + hp:
        assert sum(h.values()) == moves

    def walker_means(hs):
        return np.array([sum(c * x for c, x in h.items()) / moves for h in hs])
    md, mp = walker_means(hd), walker_means(hp)
    se = np.sqrt(md.var(ddof=1) / W + mp.var(ddof=1) / W)
    assert abs(md.mean() - mp.mean()) < 4 * se, (md.mean(), mp.mean(), se)
    # total variation distance between the pooled histograms
    keys = sorted(set().union(*hd, *hp))
    pd = np.array([sum(h.get(k, 0) for h in hd) for k in keys], float)
    pp = np.array([sum(h.get(k, 0) for h in hp) for k in keys], float)
    tv = 0.5 * np.abs(pd / pd.sum() - pp / pp.sum()).sum()
    assert tv < 0.05, tv


# (atoms, sphere radius, lowest energy bin): one atom slot per lane (13); two slots with
# the second one's few atoms spread over the lanes (38); two full slots (50)
CLUSTERS = {13: (2.5, -80.0), 38: (3.5, -180.0), 50: (4.0, -250.0)}


@pytest.mark.parametrize("method,n", [(0, 13), (2, 13), (0, 38)])
def test_da_trace_replay(gpu, oracle, method, n):
    """A traced run (plain moves, surrogate training, then delayed-acceptance moves)
    replayed by the FP64 oracle from the GPU's proposed energies and surrogate changes dS:
    the oracle takes both stages' decisions itself (the screen from its own ln w, the
    second stage with the reverse screen), so every screen, acceptance, bin and counter
    must be the GPU's."""
    W, seed, plain_moves, da_moves = 8, 6, 3000, 6000
    R, e_lo = CLUSTERS[n]
    confs = lj_configs(oracle, n, R, range(700, 700 + W))
    kw = dict(method=method, min_T=0.1, energy_bin=0.1, max_allowed=0.0, target_rate=0.5,
              translation_scale=0.1, seed=seed)
    b = gpu.Batch(gpu.make_config(gpu.LJ, W, n, e_lo=e_lo, e_hi=1, lanes_per_walker=32, **kw),
                  [(n, R, (0, 0, 0))] * W)
    b.upload(confs)
    b.initialize()
    E0 = b.energies()
    total = plain_moves + da_moves
    b.set_trace(total)
    b.surrogate_init(seed=2, ring_capacity=8192)
    for _ in range(6):
        b.run(plain_moves // 6)
        b.surrogate_collect()
    b.surrogate_train(200, batch=128, lr=2e-3, seed=4)
    stats = b.run_da(da_moves)
    screened = stats[:, 0].sum() / stats.sum()
    assert 0.02 < screened < 0.95, screened
    for w in range(W):
        e1, e2 = b.trace(w, total)
        ds = b.trace_ds(w, total)
        assert len(e1) == total and len(ds) == total
        assert not ds[:plain_moves].any()
        ow = oracle.Walker(oracle.make_config(oracle.LJ, n, radius=R, walker=w, e0=float(E0[w]),
                                              **kw), confs[w])
        d1, m1 = ow.run_override(e1[:plain_moves], e2[:plain_moves])
        d2, m2 = ow.run_override_da(e1[plain_moves:], e2[plain_moves:], ds[plain_moves:])
        assert m1 == 0 and m2 == 0, (w, m1, m2)
        assert max(d1, d2) < 2e-5, (w, d1, d2)
        label = f"da method {method} n {n} walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_allclose(b.state(w), ow.state(), atol=1e-11)


@pytest.mark.parametrize("n", [38, 50])
def test_da_screen_matches_the_mlp_statement(gpu, oracle, n):
    """The screen's surrogate change dS of every accepted delayed-acceptance move against the
    FP64 statement of the MLP (BF16 rounding emulated) on fresh descriptors of the
    configurations before and after the move, which the oracle replays from the trace.  The
    kernel keeps descriptors incrementally and per-atom energies of the current
    configuration, so this checks every row and column of the incremental update, the moved
    atom's row and the MLP on all row tiles: 38 atoms take the second atom slot's few rows
    spread over the lanes, 50 atoms a lane per row.  Tolerance per move 0.02 (the tanh form
    of SiLU, about 2^-11 per unit, and BF16 roundings it flips; observed below 0.005), and
    the errors may not add up (their sum within 0.05)."""
    import mlp_oracle as M
    W, seed, plain_moves, da_moves = 2, 3, 2000, 1500
    R, e_lo = CLUSTERS[n]
    confs = lj_configs(oracle, n, R, range(900, 900 + W))
    kw = dict(method=0, min_T=0.1, energy_bin=0.2, max_allowed=0.0, target_rate=0.5,
              translation_scale=0.1, seed=seed)
    b = gpu.Batch(gpu.make_config(gpu.LJ, W, n, e_lo=e_lo, e_hi=1, lanes_per_walker=32, **kw),
                  [(n, R, (0, 0, 0))] * W)
    b.upload(confs)
    b.initialize()
    E0 = b.energies()
    total = plain_moves + da_moves
    b.set_trace(total)
    b.surrogate_init(seed=2, ring_capacity=8192)
    for _ in range(4):
        b.run(plain_moves // 4)
        b.surrogate_collect()
    b.surrogate_train(200, batch=128, lr=2e-3, seed=4)
    p = gpu.unpack_params(b.surrogate_params())
    es = lambda pos: float(M.forward(M.descriptors(pos), p, emulate_bf16=True)[0].sum())
    x_before = [b.state(w) for w in range(W)]
    b.run_da(da_moves, refresh_interval=1 << 30)  # one launch: descriptors built once
    for w in range(W):
        e1, e2 = b.trace(w, total)
        ds = b.trace_ds(w, total).astype(np.float64)
        ow = oracle.Walker(oracle.make_config(oracle.LJ, n, radius=R, walker=w, e0=float(E0[w]),
                                              **kw), confs[w])
        ow.run_override(e1[:plain_moves], e2[:plain_moves])
        np.testing.assert_allclose(x_before[w], ow.state(), atol=1e-11)
        err = []
        for t in range(plain_moves, total):
            x0 = ow.state().copy()
            ow.run_override_da(e1[t:t + 1], e2[t:t + 1], ds[t:t + 1])
            x1 = ow.state()
            if np.any(x1 != x0):
                err.append(ds[t] - (es(x1) - es(x0)))
        err = np.array(err)
        assert len(err) > da_moves // 10, len(err)
        assert np.abs(err).max() < 0.02, (w, np.abs(err).max())
        assert abs(err.sum()) < 0.05, (w, err.sum())
        np.testing.assert_allclose(b.state(w), ow.state(), atol=1e-11)


def test_da_trace_replay_at_c4_launch_geometry(gpu, oracle):
    """Delayed acceptance at the LJ38 workload's own launch geometry (8192 walkers, R = 3.5,
    SAD min_T 0.05, bins of 0.2): plain moves with online collection, training, then
    delayed-acceptance moves with online retraining, all traced; walkers from the first,
    middle and last blocks are replayed through the FP64 oracle, which takes both stages'
    decisions itself."""
    n, W, R, seed = 38, 8192, 3.5, 8
    plain_moves, da_moves = 1500, 3000
    confs = sphere_configs(n, R, W, seed=5000)
    kw = dict(method=0, min_T=0.05, energy_bin=0.2, max_allowed=0.0, target_rate=0.5,
              translation_scale=0.1, seed=seed)
    b = gpu.Batch(gpu.make_config(gpu.LJ, W, n, e_lo=-180.0, e_hi=1.0, lanes_per_walker=32, **kw),
                  [(n, R, (0, 0, 0))] * W)
    b.upload(confs)
    b.initialize()
    E0 = b.energies()
    total = plain_moves + da_moves
    b.set_trace(total)
    b.surrogate_init(seed=2, ring_capacity=1 << 15)
    b.run_online(plain_moves, False, collect_interval=500, retrain_interval=1500, train_steps=100,
                 batch=256, lr=2e-3, seed=4)
    stats = b.run_online(da_moves, True, collect_interval=1000, retrain_interval=1500, train_steps=20,
                         batch=256, lr=1e-3, seed=5)
    screened = stats[:, 0].sum() / stats.sum()
    assert 0.02 < screened < 0.95, screened
    for w in (0, 1, 3, 4, 4096, 4099, 8188, 8191):
        e1, e2 = b.trace(w, total)
        ds = b.trace_ds(w, total)
        assert not ds[:plain_moves].any()
        ow = oracle.Walker(oracle.make_config(oracle.LJ, n, radius=R, walker=w, e0=float(E0[w]), **kw),
                           confs[w])
        d1, m1 = ow.run_override(e1[:plain_moves], e2[:plain_moves])
        d2, m2 = ow.run_override_da(e1[plain_moves:], e2[plain_moves:], ds[plain_moves:])
        assert m1 == 0 and m2 == 0, (w, m1, m2)
        assert max(d1, d2) < 2e-5, (w, d1, d2)
        label = f"da C4 launch walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_allclose(b.state(w), ow.state(), atol=1e-11)
    assert not b.status().any()
