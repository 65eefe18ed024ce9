"""Grand-canonical LJ cluster with the energy-number method (src/mc/energy_number.rs,
src/system/lj.rs:291-319) against the FP64 oracle by trace replay: with the GPU's proposed
energies substituted, every decision, every (E, N) bin, the counters and the configuration
are the oracle's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SAME = ("moves", "accepted", "addremove_probability", "N", "num_states", "t_last", "gamma",
        "lowest_hist", "highest_hist", "total_hist", "max_S", "max_S_index", "min", "width",
        "max_N", "num_E", "addremove_attempts", "addremove_accepted")


@pytest.mark.parametrize("method,target,lanes,max_N", [
    ("samc", None, 8, 13), ("wl", None, 8, 13), ("samc", 0.5, 8, 13), ("samc", None, 32, 13),
    ("wl", None, 4, 13), ("samc", None, 16, 40), ("wl", 0.5, 8, 40)])
def test_grand_trace_replay(gpu, oracle, method, target, lanes, max_N):
    """Walker groups of `lanes` lanes; 7 walkers leave the last warp partly empty."""
    W, moves, R, seed = 7, 20000, 2.5, 3
    m = gpu.SAMC if method == "samc" else gpu.WL
    common = dict(t0=1000.0, energy_bin=0.5, max_allowed=10.0, translation_scale=0.1,
                  addremove_probability=0.1, target_rate=target, seed=seed)
    b = gpu.GrandBatch(gpu.make_grand_config(W, max_N, R, method=m, e_lo=-200.0, e_hi=12.0,
                                             lanes_per_walker=lanes, **common))
    b.set_trace(moves)
    b.run(moves)
    for w in range(W):
        e1, e2 = b.trace(w, moves)
        assert len(e1) == moves
        ow = oracle.GrandWalker(oracle.make_grand_config(R, method=m, max_N=max_N, walker=w, **common))
        disc, mismatch = ow.run_override(e1, e2)
        assert mismatch == 0 and disc < 1e-5, (w, mismatch, disc, ow.worst())
        gb, ob = b.bins(w), ow.bins()
        for k in ("lnw", "hist", "visited", "round_trips"):
            np.testing.assert_array_equal(gb[k], ob[k], err_msg=f"walker {w} {k}")
        if method == "wl":
            np.testing.assert_array_equal(gb["wl_hist"], ob["wl_hist"], err_msg=f"walker {w}")
        gs, os_ = b.scalars(w), ow.scalars()
        for k in SAME:
            assert gs[k] == os_[k], (w, k, gs[k], os_[k])
        assert gs["status"] == 0
        ga, gc = b.translation_counts(w)
        oa, oc = ow.translation_counts()
        np.testing.assert_array_equal(ga, oa)
        np.testing.assert_array_equal(gc, oc)
        np.testing.assert_allclose(b.state(w), ow.state(), atol=1e-11)
        assert gs["energy"] == pytest.approx(ow.compute_energy(), abs=1e-3)


@pytest.mark.parametrize("method,lanes", [("samc", 32), ("wl", 32), ("samc", 16), ("wl", 8)])
def test_grand_wca_trace_replay(gpu, oracle, method, lanes):
    """The WCA fluid's grand moves (wca.rs:307-323): adds at a uniform point of the box,
    removals by swap_remove out of the subcell lists (optcell.rs:177-193)."""
    W, moves, max_N, L, seed = 6, 20000, 40, 4.5, 5
    m = gpu.SAMC if method == "samc" else gpu.WL
    common = dict(t0=1000.0, energy_bin=0.5, max_allowed=20.0, translation_scale=0.1,
                  addremove_probability=0.2, seed=seed)
    b = gpu.GrandBatch(gpu.make_grand_config(W, max_N, box=(L, L, L), method=m, e_lo=-1.0,
                                             e_hi=25.0, lanes_per_walker=lanes, **common))
    b.set_trace(moves)
    b.run(moves)
    for w in range(W):
        e1, e2 = b.trace(w, moves)
        ow = oracle.GrandWalker(oracle.make_grand_config(box=(L, L, L), method=m, max_N=max_N,
                                                         walker=w, **common))
        disc, mismatch = ow.run_override(e1, e2)
        assert mismatch == 0 and disc < 5e-6, (w, mismatch, disc, ow.worst())
        gb, ob = b.bins(w), ow.bins()
        for k in ("lnw", "hist", "visited", "round_trips"):
            np.testing.assert_array_equal(gb[k], ob[k], err_msg=f"walker {w} {k}")
        if method == "wl":
            np.testing.assert_array_equal(gb["wl_hist"], ob["wl_hist"], err_msg=f"walker {w}")
        gs, os_ = b.scalars(w), ow.scalars()
        for k in SAME:
            assert gs[k] == os_[k], (w, k, gs[k], os_[k])
        assert gs["status"] == 0
        np.testing.assert_array_equal(b.state(w), ow.state())
        assert gs["energy"] == pytest.approx(ow.compute_energy(), abs=1e-3)
