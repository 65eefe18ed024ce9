"""GPU periodic-cell kernels against the FP64 oracle.

Square well with a hard core (the contact-count "hard sphere" system): overlap and
contact decisions are FP64-exact, energies are integers, so the whole run on the same
Philox stream must be bit-identical.  WCA: binary32 pair energies, checked by trace
replay like the LJ cluster.
"""
import numpy as np
import pytest

from helpers import assert_bins_equal, assert_scalars_equal

pytestmark = pytest.mark.gpu


def sw_walkers(oracle, n, ffs, seed0):
    out = []
    for k, ff in enumerate(ffs):
        pos, box = oracle.init_sw_fcc(n, ff, 1.3, seed0 + k)
        out.append((pos, box))
    return out


@pytest.mark.parametrize("method,lpw", [("wl", 8), ("sad", 8), ("wl", 32), ("wl", 4), ("samc", 16)])
def test_square_well_bit_exact(gpu, oracle, method, lpw):
    n, moves, seed = 108, 20000, 9
    ffs = [0.30, 0.35, 0.40, 0.45, 0.50, 0.32, 0.38, 0.47]
    ws = sw_walkers(oracle, n, ffs, 40)
    W = len(ws)
    kw = {"wl": dict(method=2), "sad": dict(method=0, min_T=0.5), "samc": dict(method=1, t0=1000.0)}[method]
    cfg = gpu.make_config(gpu.SW, W, n, e_lo=-6.0 * n - 2, e_hi=2.0, well_width=1.3, seed=seed,
                          translation_scale=0.05, lanes_per_walker=lpw, **kw)
    b = gpu.Batch(cfg, [(n, 0.0, box) for _, box in ws])
    b.upload([p for p, _ in ws])
    E0 = b.compute_energies()
    b.initialize()
    b.run(moves // 2)
    b.run(moves - moves // 2)
    for w, (pos, box) in enumerate(ws):
        ow = oracle.Walker(oracle.make_config(oracle.SW, n, box=box, well_width=1.3, seed=seed,
                                              walker=w, translation_scale=0.05, **kw), pos)
        assert ow.energy() == E0[w]
        ow.run(moves)
        label = f"sw {method} lpw{lpw} walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_array_equal(b.state(w), ow.state())
    np.testing.assert_array_equal(b.energies(), b.compute_energies())
    assert not b.status().any()


def test_square_well_rejects_small_boxes(gpu):
    cfg = gpu.make_config(gpu.SW, 1, 8, e_lo=-50, e_hi=2, well_width=1.3)
    with pytest.raises(gpu.SadmcError):
        gpu.Batch(cfg, [(8, 0.0, (3.0, 3.0, 3.0))])  # floor(3/1.3) = 2 subcells


def wca_config(n, rho, seed):
    """Random subset of a jittered simple-cubic lattice filling the box."""
    L = (n / rho) ** (1 / 3)
    m = int(np.ceil(n ** (1 / 3)))
    rng = np.random.default_rng(seed)
    g = np.array([(i, j, k) for i in range(m) for j in range(m) for k in range(m)], float)
    g = g[rng.permutation(len(g))[:n]]
    pos = (g + 0.5 + rng.uniform(-0.05, 0.05, g.shape)) * (L / m)
    return np.mod(pos, L), (L, L, L)


@pytest.mark.parametrize("lpw", [4, 16])
def test_wca_pressure_channel(gpu, oracle, lpw):
    """The binned "pressure" datum (wca.rs:202-218, every N^2 moves): counts bit-exact,
    totals to FP64 summation order, on small fluids that collect several samples."""
    specs = [(32, 0.6), (27, 0.7), (40, 0.8), (48, 0.8)]
    moves, seed, w_bin = 8000, 9, 0.5
    confs = [wca_config(n, rho, 30 + k) for k, (n, rho) in enumerate(specs)]
    cfg = gpu.make_config(gpu.WCA, len(specs), max(n for n, _ in specs), method=1, t0=500.0,
                          energy_bin=w_bin, e_lo=-2 * w_bin, e_hi=2100.0, max_allowed=2000.0,
                          translation_scale=0.1, seed=seed, lanes_per_walker=lpw,
                          resum_interval=1500)
    b = gpu.Batch(cfg, [(n, 0.0, box) for (n, _), (_, box) in zip(specs, confs)])
    b.upload([p for p, _ in confs])
    b.initialize()
    E0 = b.energies()
    b.set_trace(moves)
    b.run(moves)
    for w, ((n, rho), (pos, box)) in enumerate(zip(specs, confs)):
        e1, e2 = b.trace(w, moves)
        ow = oracle.Walker(oracle.make_config(oracle.WCA, n, box=box, method=1, t0=500.0,
                                              energy_bin=w_bin, max_allowed=2000.0,
                                              translation_scale=0.1, seed=seed, walker=w,
                                              e0=float(E0[w])), pos)
        disc, mismatch = ow.run_override(e1, e2)
        assert mismatch == 0 and disc < 5e-6, (w, mismatch, disc, ow.override_worst())
        gc, gt = b.extra(w)
        oc, ot = ow.extra()
        assert int(gc.sum()) == moves // (n * n), (w, gc.sum())
        np.testing.assert_array_equal(gc, oc, err_msg=f"walker {w}")
        np.testing.assert_allclose(gt, ot, rtol=1e-12, atol=0, err_msg=f"walker {w}")
    # the square well collects no data
    (pos, box), = sw_walkers(oracle, 108, [0.3], 7)
    sw = gpu.Batch(gpu.make_config(gpu.SW, 1, 108, e_lo=-650.0, e_hi=2.0, well_width=1.3),
                   [(108, 0.0, box)])
    sw.upload([pos])
    sw.initialize()
    sw.run(10)
    with pytest.raises(gpu.SadmcError, match="collects no data"):
        sw.extra(0)


@pytest.mark.parametrize("lpw", [8, 32])
def test_wca_uneven_trace_replay(gpu, oracle, lpw):
    specs = [(64, 0.6), (64, 0.9), (128, 0.7), (128, 0.8), (96, 0.75), (64, 0.85)]
    moves, seed, w_bin = 8000, 4, 0.5
    confs = [wca_config(n, rho, 10 + k) for k, (n, rho) in enumerate(specs)]
    W = len(specs)
    cfg = gpu.make_config(gpu.WCA, W, max(n for n, _ in specs), method=1, t0=500.0,
                          energy_bin=w_bin, e_lo=-2 * w_bin, e_hi=2100.0, max_allowed=2000.0,
                          translation_scale=0.1, seed=seed, lanes_per_walker=lpw,
                          resum_interval=1500)  # no re-sum on the last move
    b = gpu.Batch(cfg, [(n, 0.0, box) for (n, _), (_, box) in zip(specs, confs)])
    b.upload([p for p, _ in confs])
    b.initialize()
    E0 = b.energies()
    b.set_trace(moves)
    b.run(moves)
    for w, ((n, rho), (pos, box)) in enumerate(zip(specs, confs)):
        e1, e2 = b.trace(w, moves)
        ow = oracle.Walker(oracle.make_config(oracle.WCA, n, box=box, method=1, t0=500.0,
                                              energy_bin=w_bin, max_allowed=2000.0,
                                              translation_scale=0.1, seed=seed, walker=w,
                                              e0=float(E0[w])), pos)
        disc, mismatch = ow.run_override(e1, e2)
        assert mismatch == 0, (w, mismatch)
        # double-single pair differences: measured gaps about 1.4e-6 of the gross magnitude
        assert disc < 5e-6, (w, disc)
        label = f"wca lpw{lpw} walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_allclose(b.state(w), ow.state(), atol=1e-12)
    # incremental binary32 dE since the last FP64 re-sum (500 moves) vs the FP64 re-sum
    np.testing.assert_allclose(b.energies(), b.compute_energies(), atol=1e-3, rtol=2e-6)
    assert not (b.status() & ~np.uint32(gpu.ST_DESCENT_FAILED)).any()


def test_square_well_initial_descent_bit_exact(gpu, oracle):
    """The descent of energy.rs:840-851 on the square well: walkers start above
    max_allowed_energy and gain contacts downhill; states and bins equal the oracle's."""
    n, moves, seed = 108, 6000, 13
    ws = sw_walkers(oracle, n, [0.30, 0.40, 0.45, 0.35], 90)
    E_start = np.array([oracle.Walker(oracle.make_config(oracle.SW, n, box=box), p).energy()
                        for p, box in ws])
    max_allowed = float(E_start.max() - 15.0)
    kw = dict(method=0, min_T=0.5)
    cfg = gpu.make_config(gpu.SW, len(ws), n, e_lo=-6.0 * n - 2, e_hi=2.0, well_width=1.3,
                          seed=seed, translation_scale=0.05, max_allowed=max_allowed,
                          lanes_per_walker=8, **kw)
    b = gpu.Batch(cfg, [(n, 0.0, box) for _, box in ws])
    b.upload([p for p, _ in ws])
    b.initialize()
    E0 = b.energies()
    assert (E0 < max_allowed).all()
    b.run(moves)
    for w, (pos, box) in enumerate(ws):
        ow = oracle.Walker(oracle.make_config(oracle.SW, n, box=box, well_width=1.3, seed=seed,
                                              walker=w, translation_scale=0.05,
                                              max_allowed=max_allowed, **kw), pos)
        assert ow.energy() == E0[w]
        ow.run(moves)
        label = f"sw descent walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_array_equal(b.state(w), ow.state())
    assert not b.status().any()


@pytest.mark.parametrize("lpw", [32, 16])
def test_square_well_c5_shape_bit_exact(gpu, oracle, lpw):
    """The hard-sphere workload's own shape: N = 1024 square-well atoms (lambda 1.3) at
    packing fractions 0.30 and 0.50 (9 and 7 subcells per axis) and between, Wang-Landau
    on contact bins, a few thousand moves; bins, scalars and configurations bit-identical
    to the oracle's (optsquare.rs:74-95, 273-322)."""
    n, moves, seed = 1024, 3000, 11
    ws = sw_walkers(oracle, n, [0.30, 0.50, 0.40, 0.45], 60)
    ncs = [int(np.floor(box[0] / 1.3)) for _, box in ws]
    assert ncs[0] == 9 and ncs[1] == 7, ncs
    cfg = gpu.make_config(gpu.SW, len(ws), n, method=2, e_lo=-6.0 * n - 2, e_hi=2.0, well_width=1.3,
                          seed=seed, translation_scale=0.05, lanes_per_walker=lpw)
    b = gpu.Batch(cfg, [(n, 0.0, box) for _, box in ws])
    b.upload([p for p, _ in ws])
    E0 = b.compute_energies()
    b.initialize()
    b.run(moves)
    for w, (pos, box) in enumerate(ws):
        ow = oracle.Walker(oracle.make_config(oracle.SW, n, box=box, well_width=1.3, method=2, seed=seed,
                                              walker=w, translation_scale=0.05), pos)
        assert ow.energy() == E0[w]
        ow.run(moves)
        label = f"sw C5 shape lpw{lpw} walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_array_equal(b.state(w), ow.state())
    np.testing.assert_array_equal(b.energies(), b.compute_energies())
    assert not b.status().any()


def test_wca_c3_shape_trace_replay(gpu, oracle):
    """The uneven WCA workload's largest walkers: N = 512 at density 0.6 (8 subcells per
    axis) and N = 256 at 0.9 (5), beside N = 512 at 0.75 and N = 256 at 0.6, SAMC, traced
    and replayed by the FP64 oracle (wca.rs:119-140)."""
    specs = [(512, 0.6), (256, 0.9), (512, 0.75), (256, 0.6)]
    moves, seed, w_bin = 4000, 21, 0.5
    confs = [wca_config(n, rho, 70 + k) for k, (n, rho) in enumerate(specs)]
    assert int(np.floor(confs[0][1][0] / 2 ** (1 / 6))) == 8
    cfg = gpu.make_config(gpu.WCA, len(specs), 512, method=1, t0=1e4, energy_bin=w_bin, e_lo=-2 * w_bin,
                          e_hi=4100.0, max_allowed=4000.0, translation_scale=0.1, seed=seed,
                          lanes_per_walker=16, resum_interval=1500)
    b = gpu.Batch(cfg, [(n, 0.0, box) for (n, _), (_, box) in zip(specs, confs)])
    b.upload([p for p, _ in confs])
    b.initialize()
    E0 = b.energies()
    b.set_trace(moves)
    b.run(moves)
    for w, ((n, rho), (pos, box)) in enumerate(zip(specs, confs)):
        e1, e2 = b.trace(w, moves)
        ow = oracle.Walker(oracle.make_config(oracle.WCA, n, box=box, method=1, t0=1e4,
                                              energy_bin=w_bin, max_allowed=4000.0,
                                              translation_scale=0.1, seed=seed, walker=w,
                                              e0=float(E0[w])), pos)
        disc, mismatch = ow.run_override(e1, e2)
        assert mismatch == 0 and disc < 5e-6, (w, mismatch, disc)
        label = f"wca C3 shape walker {w}"
        assert_bins_equal(b.bins(w), ow.bins(), label=label)
        assert_scalars_equal(b.scalars(w), ow.scalars(), label=label)
        np.testing.assert_allclose(b.state(w), ow.state(), atol=1e-12)
    assert not (b.status() & ~np.uint32(gpu.ST_DESCENT_FAILED)).any()
