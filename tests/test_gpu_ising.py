"""GPU Ising kernel against the FP64 oracle: integer energies, so the whole flat-histogram
chain (spins, bins, SAD/WL/SAMC state) must be bit-identical on the same Philox stream."""
import numpy as np
import pytest

from helpers import METHOD_KW, assert_bins_equal, assert_scalars_equal, ising_spins

pytestmark = pytest.mark.gpu


def run_pair(gpu, oracle, L, W, moves, method, seed=17, lpw=0, chunks=1, extra=None):
    kw = dict(METHOD_KW[method], **(extra or {}))
    N = L * L
    cfg = gpu.make_config(gpu.ISING, W, L, e_lo=-2.0 * N - 4, e_hi=2.0 * N + 4, seed=seed,
                          lanes_per_walker=lpw, **kw)
    b = gpu.Batch(cfg, [(L, 0.0, (0, 0, 0))] * W)
    spins = [ising_spins(L, 1000 + w) for w in range(W)]
    b.upload(spins)
    b.initialize()
    for _ in range(chunks):
        b.run(moves // chunks)
    walkers = []
    okw = {k: v for k, v in kw.items()}
    for w in range(W):
        ow = oracle.Walker(oracle.make_config(oracle.ISING, L, seed=seed, walker=w, **okw), spins[w])
        ow.run(moves)
        walkers.append(ow)
    return b, walkers


@pytest.mark.parametrize("method", ["sad", "wl", "inv_t_wl", "samc", "canonical"])
@pytest.mark.parametrize("lpw", [0, 32])
def test_ising_batch_bit_exact(gpu, oracle, method, lpw):
    """lpw 32: one walker per warp, run as a serial chain on one lane with its bins and spins
    in shared memory and the warp filling draw and gamma tables 32 moves ahead, for each of
    the three launches (SAD specialised; Wang-Landau, 1/t-WL switching to SAMC, SAMC and
    canonical through the generic bookkeeping)."""
    b, ws = run_pair(gpu, oracle, L=8, W=40, moves=30000, method=method, chunks=3, lpw=lpw)
    for w in range(b.W):
        label = f"{method} walker {w}"
        assert_bins_equal(b.bins(w), ws[w].bins(), label=label)
        assert_scalars_equal(b.scalars(w), ws[w].scalars(), label=label)
        np.testing.assert_array_equal(b.state(w), ws[w].state())
        if method in ("wl", "inv_t_wl"):
            gh, gme = b.wl_hist(w)
            oh, ome = ws[w].wl_hist()
            if ws[w].scalars()["method_kind"] == 2:
                np.testing.assert_array_equal(gh, oh)
                assert gme == ome
    assert not b.status().any()


def test_ising_single_walker_32x32(gpu, oracle):
    """The one-walker 32x32 SAD chain (the C1 shape), over launches whose move counts are
    not multiples of the 32-move table batches."""
    b, ws = run_pair(gpu, oracle, L=32, W=1, moves=200001, method="sad", lpw=32, chunks=3)
    assert_bins_equal(b.bins(0), ws[0].bins(), label="L32")
    assert_scalars_equal(b.scalars(0), ws[0].scalars(), label="L32")
    np.testing.assert_array_equal(b.state(0), ws[0].state())


def test_ising_single_walker_steady_state(gpu, oracle):
    """Two million moves of the C1 walker: after the discovery phase nearly every move takes
    the integer fast path of the pipelined SAD chain."""
    b, ws = run_pair(gpu, oracle, L=32, W=1, moves=2_000_000, method="sad", lpw=32, chunks=2,
                     seed=23)
    assert_bins_equal(b.bins(0), ws[0].bins(), label="L32 steady")
    assert_scalars_equal(b.scalars(0), ws[0].scalars(), label="L32 steady")
    np.testing.assert_array_equal(b.state(0), ws[0].state())


@pytest.mark.parametrize("energy_bin,bounds,target_rate", [
    (1.0, None, None),                  # half-integer bin centres: non-integer window edges
    (2.0, (-400.0, 300.0), None),       # both energy bounds
    (8.0, None, None),                  # two energy levels per bin
    (3.0, (-450.0, 420.0), None),       # not a power of two: the generic bookkeeping throughout
    (4.0, (-500.0, -100.0), None),      # initial descent below max_allowed, then the chain
    (4.0, None, 0.3),                   # acceptance-rate mode: translation scale on tF changes
])
def test_ising_single_walker_chain_bins_and_bounds(gpu, oracle, energy_bin, bounds, target_rate):
    """The pipelined SAD chain with other bin widths, with min/max_allowed_energy and with
    the acceptance-rate mode (whose translation-scale updates the replay warp applies),
    three walkers of 16x16 over launches of uneven length."""
    extra = {"energy_bin": energy_bin}
    if bounds is not None:
        extra.update(min_allowed=bounds[0], max_allowed=bounds[1])
    if target_rate is not None:
        extra.update(target_rate=target_rate)
    b, ws = run_pair(gpu, oracle, L=16, W=3, moves=150_003, method="sad", lpw=32, chunks=3,
                     seed=29, extra=extra)
    for w in range(b.W):
        label = f"bin {energy_bin} bounds {bounds} rate {target_rate} walker {w}"
        assert_bins_equal(b.bins(w), ws[w].bins(), label=label)
        assert_scalars_equal(b.scalars(w), ws[w].scalars(), label=label)
        np.testing.assert_array_equal(b.state(w), ws[w].state())
    assert not b.status().any()


def test_ising_single_walker_unstaged(gpu, oracle):
    """64x64: the bins and spins (about 266 KB) exceed the shared memory of a block, so the
    lone walker runs on its planes in global memory (the warp-per-walker kernel)."""
    b, ws = run_pair(gpu, oracle, L=64, W=1, moves=60000, method="sad", lpw=32, chunks=2)
    assert_bins_equal(b.bins(0), ws[0].bins(), label="L64")
    assert_scalars_equal(b.scalars(0), ws[0].scalars(), label="L64")
    np.testing.assert_array_equal(b.state(0), ws[0].state())


def test_ising_energy_matches_compute_energy(gpu, oracle):
    b, ws = run_pair(gpu, oracle, L=16, W=8, moves=5000, method="sad")
    np.testing.assert_array_equal(b.energies(), b.compute_energies())
    np.testing.assert_array_equal(b.energies(), [w.compute_energy() for w in ws])


@pytest.mark.parametrize("system,n", [(0, 8), (0, 32), (1, 31), (1, 1024), (3, 38)])
def test_device_draws_match_oracle(gpu, oracle, system, n):
    """The kernels' Philox draws (index, three binary32 normals, 53-bit uniform) equal the
    oracle's bit for bit."""
    seed, walker, t0, count = 2**33 + 7, 11, 1, 4000
    gi, gg, gu = gpu.draws(system, n, seed, walker, t0, count)
    for k in range(0, count, 7):
        idx, g, u = oracle.draws(system, n, seed, walker, t0 + k)
        assert np.array_equal(idx, gi[k]) and np.array_equal(g, gg[k]) and u == gu[k], k


def test_ising_initial_descent_bit_exact(gpu, oracle):
    """from_params descent (energy.rs:840-851) on the descent stream: walkers starting above
    max_allowed_energy flip downhill until below it (each makes at least one proposal), then
    run; spins, energies and bins equal the oracle's."""
    L, W, moves, seed = 12, 16, 20000, 31
    N = L * L
    kw = dict(method=0, min_T=0.2)
    cfg = gpu.make_config(gpu.ISING, W, L, e_lo=-2.0 * N - 4, e_hi=2.0 * N + 4, seed=seed,
                          max_allowed=-100.0, **kw)
    b = gpu.Batch(cfg, [(L, 0.0, (0, 0, 0))] * W)
    spins = [ising_spins(L, 700 + w) for w in range(W)]
    b.upload(spins)
    b.initialize()
    E0 = b.energies()
    assert (E0 < -100.0).all()
    b.run(moves)
    for w in range(W):
        ow = oracle.Walker(oracle.make_config(oracle.ISING, L, seed=seed, walker=w,
                                              max_allowed=-100.0, **kw), spins[w])
        assert ow.energy() == E0[w]
        ow.run(moves)
        label = f"descent walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_array_equal(b.state(w), ow.state())
    assert not b.status().any()
