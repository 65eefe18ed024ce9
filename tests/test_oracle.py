"""CPU tests of the FP64 oracle: the reference's own invariant tests re-run on the
restatement, the published Philox known answers, and the golden fixtures."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for philox4x32-10
    assert [int(x) for x in oracle.philox([0, 0, 0, 0], [0, 0])] == \
        [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert [int(x) for x in oracle.philox([0xffffffff] * 4, [0xffffffff] * 2)] == \
        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert [int(x) for x in oracle.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                          [0xa4093822, 0x299f31d0])] == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_normals_are_standard(oracle):
    rng = np.random.default_rng(0)
    a = rng.integers(0, 2**32, 200000, dtype=np.uint32)
    b = rng.integers(0, 2**32, 200000, dtype=np.uint32)
    z0, z1 = oracle.normal_pairs(a, b)
    z = np.concatenate([z0, z1]).astype(np.float64)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1) < 0.01
    assert abs(((z - z.mean()) ** 4).mean() / z.var() ** 2 - 3.0) < 0.05
    assert abs(np.corrcoef(z0, z1)[0, 1]) < 0.01


@pytest.mark.parametrize("L", [2, 3, 10, 15, 137, 150])
def test_ising_energy_works(oracle, L):
    """ising.rs:125-147: energy() == compute_energy() after each of 1e4 flips."""
    assert oracle.selftest_ising(L, 10000) == 0


@pytest.mark.parametrize("n", [3, 50, 100])
def test_lj_energy_is_right(oracle, n):
    """lj.rs:380-427: incremental energy passes verify_energy after each move."""
    radius = 5 * 2 * n ** (1 / 3)
    pos, ok = oracle.init_lj(n, radius, 1)
    assert ok
    w = oracle.Walker(oracle.make_config(oracle.LJ, n, radius=radius), pos)
    assert w.energy() == w.compute_energy()
    assert oracle.selftest_moves(w, 1000, 1.0) == 0


@pytest.mark.parametrize("n,ff", [(3, 0.1), (50, 0.3), (100, 0.3), (200, 0.3)])
def test_square_well_energy_is_right(oracle, n, ff):
    """optsquare.rs:585-618: E == compute_energy exactly after every move."""
    pos, box = oracle.init_sw_fcc(n, ff, 1.3, 0)
    w = oracle.Walker(oracle.make_config(oracle.SW, n, box=box), pos)
    assert w.verify_energy()
    assert oracle.selftest_moves(w, 1000, 1.0) == 0


@pytest.mark.parametrize("n", [100, 200])
def test_square_well_minimum_images(oracle, n):
    """optsquare.rs:438-521: closest-distance variants agree; candidates are minimum images."""
    pos, box = oracle.init_sw_fcc(n, 0.3, 1.3, 0)
    w = oracle.Walker(oracle.make_config(oracle.SW, n, box=box), pos)
    assert oracle.selftest_cell(w) == 0
    oracle.selftest_moves(w, 100000, 1.0)
    assert oracle.selftest_cell(w) == 0


@pytest.mark.parametrize("n,rho", [(50, 0.3), (50, 1.0), (100, 0.3)])
def test_wca_energy_is_right(oracle, n, rho):
    """wca.rs:647-694 (including the dense rho = 1.0 case)."""
    L = (n / rho) ** (1 / 3)
    pos = np.random.default_rng(n).uniform(0, L, (n, 3))
    w = oracle.Walker(oracle.make_config(oracle.WCA, n, box=(L, L, L)), pos)
    assert oracle.selftest_moves(w, 1000, 1.0) == 0


def test_wca_pressure_datum(oracle):
    """wca.rs:202-218: every N^2 moves the bin of the current energy receives
    sum_pairs 12 (2 s^6 - s^3) / (3 V) (s = 1/r^2, r < 2^(1/6)), computed here with numpy
    minimum images on the final state after exactly N^2 moves."""
    n, rho = 32, 0.6
    L = (n / rho) ** (1 / 3)
    m = 4
    g = np.array([(i, j, k) for i in range(m) for j in range(m) for k in range(m)], float)
    g = g[np.random.default_rng(5).permutation(len(g))[:n]]
    pos = np.mod((g + 0.5) * (L / m), L)
    w = oracle.Walker(oracle.make_config(oracle.WCA, n, box=(L, L, L), method=1, t0=500.0,
                                         energy_bin=0.5, max_allowed=2000.0), pos)
    w.run(n * n - 1)
    c, t = w.extra()
    assert len(c) == 0  # nothing collected before move N^2 (the BinCounts is created lazily)
    w.run(1)
    c, t = w.extra()
    assert int(c.sum()) == 1 and len(c) == len(w.bins()["lnw"])
    x = w.state()
    d = x[:, None, :] - x[None, :, :]
    d -= L * np.round(d / L)
    r2 = (d ** 2).sum(-1)
    np.fill_diagonal(r2, np.inf)
    s = np.where(r2 < 2 ** (1 / 3), 1.0 / r2, 0.0)
    p = (12.0 * (2 * s ** 6 - s ** 3)).sum() / (3 * L ** 3)
    assert p > 0
    np.testing.assert_allclose(t.sum(), p, rtol=1e-12)
    b = w.bins()
    assert int(np.nonzero(c)[0][0]) == int((w.energy() - b["min"]) / b["width"])


@pytest.mark.parametrize("method", ["samc", "wl"])
def test_grand_energy_number_invariants(oracle, method):
    """The energy-number walker (src/mc/energy_number.rs) on the grand-canonical LJ
    cluster (lj.rs:291-319): the incremental energy equals compute_energy, N stays within
    max_N, every move is counted once, the histogram holds every visit."""
    m = oracle.M_SAMC if method == "samc" else oracle.M_WL
    w = oracle.GrandWalker(oracle.make_grand_config(2.5, method=m, t0=500.0, energy_bin=0.5,
                                                    max_N=10, max_allowed=5.0, seed=4,
                                                    translation_scale=0.1,
                                                    addremove_probability=0.2))
    moves = 60000
    w.run(moves)
    s = w.scalars()
    assert 0 <= s["N"] <= 10 and s["max_N"] <= 10
    assert s["energy"] == pytest.approx(w.compute_energy(), rel=1e-9, abs=1e-9)
    assert len(w.state()) == s["N"]
    b = w.bins()
    assert int(b["hist"].sum()) == moves + 1            # the initial bin starts at 1
    att, acc = w.translation_counts()
    assert int(att.sum()) + s["addremove_attempts"] == moves
    assert int(acc.sum()) + s["addremove_accepted"] == s["accepted"]
    assert (b["lnw"][b["hist"] > 0] > 0).all()
    assert (b["lnw"][b["hist"] == 0] == 0).all()


@pytest.mark.parametrize("method", ["samc", "wl"])
def test_grand_wca_invariants(oracle, method):
    """The WCA fluid's grand moves (wca.rs:307-323): adds, swap_remove with the subcell
    renaming of optcell.rs:177-193; the lists always equal a rebuild from the positions
    and the incremental energy equals compute_energy."""
    m = oracle.M_SAMC if method == "samc" else oracle.M_WL
    L = 4.5
    w = oracle.GrandWalker(oracle.make_grand_config(box=(L, L, L), method=m, t0=500.0,
                                                    energy_bin=0.5, max_N=40, max_allowed=20.0,
                                                    translation_scale=0.1,
                                                    addremove_probability=0.3, seed=6))
    for _ in range(10):
        w.run(5000)
        assert w.check_cells() == 0
    s = w.scalars()
    assert 0 <= s["N"] <= 40 and s["addremove_accepted"] > 100
    assert s["energy"] == pytest.approx(w.compute_energy(), rel=1e-9, abs=1e-9)
    x = w.state()
    assert len(x) == s["N"] and ((x >= 0) & (x < L)).all()


def test_max_balls_within(oracle):
    # optsquare.rs:290-322 counts lattice points of its own construction
    assert oracle.max_balls_within(1.3) == 6


def test_golden_fixtures(oracle):
    """Values pinned in tests/golden (see make_golden.py)."""
    with open(os.path.join(GOLDEN, "golden.json")) as fh:
        g = json.load(fh)
    for (r2, v) in g["lj_potential"]:
        assert oracle.lib().orc_lj_potential(r2) == v
    for (r2, v) in g["wca_potential"]:
        assert oracle.lib().orc_wca_potential(r2) == v
    for rec in g["draws"]:
        idx, gg, u = oracle.draws(rec["system"], rec["n"], rec["seed"], rec["walker"], rec["t"])
        assert [int(x) for x in idx] == rec["idx"]
        assert [float(x) for x in gg] == rec["g"]
        assert u == rec["u"]
    T = np.array(g["cv"]["T"])
    C = oracle.heat_capacity(T, np.array(g["cv"]["E"]), np.array(g["cv"]["S"]))
    np.testing.assert_allclose(C, np.array(g["cv"]["C"]), rtol=1e-12)


def test_ising_sad_converges_to_exact_dos(oracle):
    """Known answer from mathematics: SAD's ln w of a 4x4 Ising lattice approaches the
    exact ln g(E) (2^16-state enumeration) up to a constant."""
    with open(os.path.join(GOLDEN, "golden.json")) as fh:
        g = json.load(fh)["ising4_exact"]
    E = np.array(g["E"])
    lng = np.array(g["lng"])
    spins = np.where(np.random.default_rng(3).random(16) < 0.5, -1.0, 1.0)
    w = oracle.Walker(oracle.make_config(oracle.ISING, 4, method=oracle.M_WL, seed=5), spins)
    w.run(3_000_000)
    b = w.bins()
    centers = b["min"] + (np.arange(len(b["lnw"])) + 0.5) * b["width"]
    got = {}
    for c, l, h in zip(centers, b["lnw"], b["hist"]):
        if h > 0:
            got[int(round(c))] = l
    common = [e for e in E if int(e) in got]
    assert len(common) == len(E)
    d = np.array([got[int(e)] for e in common]) - lng
    assert np.max(np.abs(d - d.mean())) < 0.15


def test_heat_capacity_matches_numpy(oracle):
    rng = np.random.default_rng(1)
    E = np.sort(rng.uniform(-100, 0, 300))
    S = rng.uniform(0, 50, 300)
    T = np.linspace(0.05, 0.5, 40)
    C = oracle.heat_capacity(T, E, S)
    for t, c in zip(T, C):  # plotting/final_heat_capacity.py:79-88 stated in numpy
        b = S - E / t
        P = np.exp(b - b.max())
        P = P / P.sum()
        U = (E * P).sum()
        assert c == pytest.approx(((E - U) ** 2 * P).sum() / t ** 2, rel=1e-10)


def test_mlp_oracle_gradients_by_finite_differences():
    """The FP64 surrogate oracle's analytic gradients (no bf16 emulation) against central
    differences."""
    import mlp_oracle as M
    rng = np.random.default_rng(0)
    n, C = 6, 3
    pos = rng.uniform(-1.2, 1.2, (C, n, 3))
    G = np.concatenate([M.descriptors(p) for p in pos])
    target = rng.uniform(-10, 0, C)
    p = M.init_params(1)
    p["b1"] = rng.normal(0, 0.1, 64)
    p["b3"] = np.array([0.3])
    loss, g = M.loss_and_grads(G, n, target, p, emulate_bf16=False)
    for name in p:
        flat = p[name].ravel()
        for k in rng.choice(flat.size, size=min(6, flat.size), replace=False):
            old = flat[k]
            flat[k] = old + 1e-6
            lp, _ = M.loss_and_grads(G, n, target, p, emulate_bf16=False)
            flat[k] = old - 1e-6
            lm, _ = M.loss_and_grads(G, n, target, p, emulate_bf16=False)
            flat[k] = old
            fd = (lp - lm) / 2e-6
            assert fd == pytest.approx(g[name].ravel()[k], rel=1e-5, abs=1e-8), (name, k)


def test_bf16_rounding_is_nearest_even():
    import mlp_oracle as M
    x = np.array([1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, 1.0 + 3 * 2 ** -8, -3.14159])
    r = M.bf16(x)
    assert r[0] == 1.0                      # midpoint, ties to even (down)
    assert r[1] == 1.0                      # below the midpoint
    assert r[2] == 1.0 + 2 ** -7            # above the midpoint
    assert r[3] == 1.0 + 2 ** -6            # midpoint, ties to even (up)
    assert r[4] == -3.140625


def test_native_build_is_the_checker(oracle):
    """The host-tuned build of the oracle that the CPU baseline times (-mcpu/-march=native,
    still without contraction) runs the same chains as the checker build, move for move."""
    from helpers import sphere_configs
    confs = sphere_configs(31, 2.5, 4, 5)
    cfgs = [oracle.make_config(oracle.LJ, 31, radius=2.5, method=oracle.M_SAD, min_T=0.2,
                               energy_bin=0.134, max_allowed=0.0, target_rate=0.5,
                               translation_scale=0.1, seed=3, walker=w) for w in range(4)]
    states = [c.reshape(-1) for c in confs]
    _, m0, a0 = oracle.bench(cfgs, states, 50_000, 4)
    _, m1, a1 = oracle.bench(cfgs, states, 50_000, 4, native=True)
    assert (m0, a0) == (m1, a1)
