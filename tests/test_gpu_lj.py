"""GPU LJ-cluster kernel against the FP64 oracle.

Pair energies run in binary32 on the GPU, so the oracle replays each GPU trajectory with
the GPU's proposed energies substituted (trace replay): the oracle's own FP64 proposals
must agree within the binary32 tolerance below, and with the same energies every
flat-histogram decision and bin must be bit-identical.
"""
import numpy as np
import pytest

from helpers import assert_bins_equal, assert_scalars_equal, lj_configs, sphere_configs

pytestmark = pytest.mark.gpu

# Binary32 pair terms on positions rounded to binary32: 4 (s^6 - s^3) cancels near
# r = sigma, so the rounding error scales with the gross magnitude 4 s^6 + 4 s^3 of each
# term.  Injected proposals: |e2_gpu - e2_fp64| <= DE_ABS + DE_REL * |e2 - E|.  Trace
# replay: the oracle reports max |e2_gpu - e2_fp64| / (1e-3 + sum of 4 s^6 + 4 s^3 over
# the proposal's pair terms), bounded by REPLAY_REL.
DE_ABS, DE_REL = 2e-4, 2e-5
REPLAY_REL = 2e-5


def make_batch(gpu, n, W, radius, moves_bins, method=0, seed=3, target_rate=0.5, lpw=0,
               energy_bin=0.05, e_lo=-140.0):
    cfg = gpu.make_config(gpu.LJ, W, n, method=method, min_T=0.1, energy_bin=energy_bin,
                          max_allowed=0.0, e_lo=e_lo, e_hi=1.0, target_rate=target_rate,
                          translation_scale=0.1, seed=seed, lanes_per_walker=lpw, t0=200.0)
    return gpu.Batch(cfg, [(n, radius, (0, 0, 0))] * W), cfg


@pytest.mark.parametrize("n,lpw", [(13, 8), (31, 8), (31, 4), (31, 32), (38, 8), (38, 16), (13, 1),
                                   (31, 1), (31, 2), (38, 1), (38, 2)])
def test_lj_trace_replay(gpu, oracle, n, lpw):
    W, moves, radius, seed = 12, 6000, 2.5 if n < 35 else 3.5, 5
    confs = lj_configs(oracle, n, radius, range(100, 100 + W))
    b, cfg = make_batch(gpu, n, W, radius, moves, seed=seed, lpw=lpw)
    b.upload(confs)
    b.initialize()
    E0 = b.energies()
    b.set_trace(moves)
    b.run(moves // 2)
    b.run(moves - moves // 2)
    for w in range(W):
        e1, e2 = b.trace(w, moves)
        assert len(e1) == moves
        ow = oracle.Walker(oracle.make_config(oracle.LJ, n, radius=radius, method=0, min_T=0.1,
                                              energy_bin=0.05, max_allowed=0.0, target_rate=0.5,
                                              translation_scale=0.1, seed=seed, walker=w,
                                              e0=float(E0[w])), confs[w])
        disc, mismatch = ow.run_override(e1, e2)
        assert mismatch == 0, f"walker {w}: possibility differs on {mismatch} moves"
        assert disc < REPLAY_REL, f"walker {w}: max relative |de| {disc} at {ow.override_worst()}"
        label = f"n{n} lpw{lpw} walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_allclose(b.state(w), ow.state(), atol=1e-11)
    assert not b.status().any()
    drift = max(b.scalars(w)["drift"] for w in range(W))
    assert drift < 1e-2, drift  # |E_incremental - E_fp64| at the periodic FP64 re-sums
    # incremental energy vs FP64 re-sum of the final configuration
    np.testing.assert_allclose(b.energies(), b.compute_energies(), atol=1e-3)


def test_lj_injected_proposals(gpu, oracle):
    """plan_move with injected proposals: binary32 GPU dE vs FP64 oracle dE."""
    n, W, radius = 31, 6, 2.5
    confs = lj_configs(oracle, n, radius, range(7, 7 + W))
    b, _ = make_batch(gpu, n, W, radius, 0)
    b.upload(confs)
    E_gpu = b.compute_energies()
    rng = np.random.default_rng(0)
    worst = 0.0
    for w in range(W):
        ow = oracle.Walker(oracle.make_config(oracle.LJ, n, radius=radius), confs[w])
        assert E_gpu[w] == pytest.approx(ow.compute_energy(), rel=1e-12, abs=1e-12)
        for k in range(150):
            which = int(rng.integers(n))
            g = rng.standard_normal(3).astype(np.float32).astype(np.float64)
            scale = float(rng.choice([0.05, 0.1, 0.3, 1.0]))
            eg = b.plan_move(w, which, g, scale)
            eo = ow.plan_move(which, g, scale=scale)
            assert (eg is None) == (eo is None)
            if eg is None:
                continue
            de = abs(eg - eo)
            worst = max(worst, de / (DE_ABS + DE_REL * abs(eo - E_gpu[w])))
            assert de <= DE_ABS + DE_REL * abs(eo - E_gpu[w]), (w, which, eg, eo)
    assert worst <= 1.0


def test_lj_descent_reaches_max_allowed(gpu, oracle):
    """from_params descent (energy.rs:840-851) from configurations with E > 0."""
    n, W, radius = 31, 8, 2.5
    rng = np.random.default_rng(4)
    confs = []
    for _ in range(W):
        p = rng.normal(size=(n, 3))
        p *= (rng.random(n) ** (1 / 3) * 2.4 / np.linalg.norm(p, axis=1))[:, None]
        confs.append(p)
    b, _ = make_batch(gpu, n, W, radius, 0)
    b.upload(confs)
    assert (b.compute_energies() > 0).all()
    b.initialize()
    E = b.energies()
    assert (E < 0).all()
    assert not (b.status() & gpu.ST_DESCENT_FAILED).any()
    np.testing.assert_allclose(E, b.compute_energies(), rtol=1e-12)


def test_heat_capacity_gpu_vs_oracle(gpu, oracle):
    rng = np.random.default_rng(2)
    E = np.sort(rng.uniform(-134, 0, 1000))
    S = rng.uniform(0, 80, 1000)
    T = np.linspace(0.05, 0.5, 64)
    np.testing.assert_allclose(gpu.heat_capacity(T, E, S), oracle.heat_capacity(T, E, S),
                               rtol=1e-10)


@pytest.mark.parametrize("lpw", [8, 1])
def test_lj_c2_launch_geometry_trace_replay(gpu, oracle, lpw):
    """The headline workload's own launch: 4096 LJ31 walkers (R = 2.5, SAD min_T 0.2, 1000
    bins of 0.134 over [-134, 0], max_allowed_energy 0, step 0.1 adapted to 50 %) at its
    default shape, one run traced; walkers from the first, middle and last warps and blocks
    are replayed through the FP64 oracle: every decision and bin must be the GPU's."""
    n, W, radius, seed, moves = 31, 4096, 2.5, 17, 3000
    width = 0.134
    confs = sphere_configs(n, radius, W, seed=2000)
    cfg = gpu.make_config(gpu.LJ, W, n, method=0, min_T=0.2, energy_bin=width, max_allowed=0.0,
                          e_lo=-134.0 - 2 * width, e_hi=2 * width, target_rate=0.5,
                          translation_scale=0.1, seed=seed, lanes_per_walker=lpw)
    b = gpu.Batch(cfg, [(n, radius, (0, 0, 0))] * W)
    b.upload(confs)
    b.initialize()
    E0 = b.energies()
    b.set_trace(moves)
    b.run(moves)
    for w in (0, 1, 3, 4, 127, 2048, 2051, 4092, 4095):
        e1, e2 = b.trace(w, moves)
        ow = oracle.Walker(oracle.make_config(oracle.LJ, n, radius=radius, method=0, min_T=0.2,
                                              energy_bin=width, max_allowed=0.0, target_rate=0.5,
                                              translation_scale=0.1, seed=seed, walker=w,
                                              e0=float(E0[w])), confs[w])
        disc, mismatch = ow.run_override(e1, e2)
        assert mismatch == 0 and disc < REPLAY_REL, (w, mismatch, disc)
        label = f"C2 launch lpw{lpw} walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_allclose(b.state(w), ow.state(), atol=1e-11)
    assert not b.status().any()
