"""CPU tests of the export to the reference's save and analysis formats, on oracle
walkers (the GPU batch goes through the same functions in test_gpu_export.py)."""
import os

import numpy as np
import pytest

import export
from helpers import OracleView, read_flow_yaml


def plugin_frames(movie_time, max_moves):
    """The movie plugin's state machine (plugin.rs:447-477) stepped move by move."""
    period, which, out = 1, 0, []
    for moves in range(1, max_moves + 1):
        if moves == period:
            which += 1
            nxt = int(movie_time ** which + 0.5)
            while nxt <= moves:
                which += 1
                nxt = int(movie_time ** which + 0.5)
            period = nxt
            out.append(moves)
    return out


def test_movie_times():
    assert export.movie_times(2.0, 100) == [1, 2, 4, 8, 16, 32, 64]
    assert export.movie_times(10 ** 0.25, 1000) == [1, 2, 3, 6, 10, 18, 32, 56, 100, 178, 316, 562, 1000]
    for t in (1.05, 1.3, 1.5, 2.7, 10.0):
        assert export.movie_times(t, 20000) == plugin_frames(t, 20000), t
    assert export.movie_times(None, 100) == []


def wca_walker(oracle, method, moves):
    n, rho = 32, 0.6
    L = (n / rho) ** (1 / 3)
    m = 4
    g = np.array([(i, j, k) for i in range(m) for j in range(m) for k in range(m)], float)
    g = g[np.random.default_rng(2).permutation(len(g))[:n]]
    pos = np.mod((g + 0.5) * (L / m), L)
    kw = {"sad": dict(method=oracle.M_SAD, min_T=0.5), "samc": dict(method=1, t0=500.0)}[method]
    w = oracle.Walker(oracle.make_config(oracle.WCA, n, box=(L, L, L), energy_bin=0.5,
                                         max_allowed=2000.0, seed=3, **kw), pos)
    w.run(moves)
    return w


def test_document_round_trip(oracle, tmp_path):
    w = wca_walker(oracle, "sad", 6000)
    doc = export.document(OracleView(w))
    p = str(tmp_path / "wca.yaml")
    export.write_yaml(doc, p)
    back = read_flow_yaml(p)
    assert back == doc
    b = w.bins()
    assert doc["moves"] == 6000
    assert doc["bins"]["histogram"] == [int(x) for x in b["hist"]]
    assert doc["bins"]["lnw"] == [float(x) for x in b["lnw"]]
    sad = doc["method"]["Sad"]
    assert sad["min_T"] == 0.5 and sad["too_lo"] <= sad["too_hi"]
    cell = doc["system"]["Wca"]["cell"]
    assert len(cell["positions"]) == 32
    np.testing.assert_array_equal([[p["x"], p["y"], p["z"]] for p in cell["positions"]], w.state())
    count, total = w.extra()
    assert doc["bins"]["extra"]["pressure"]["count"] == [int(x) for x in count]
    assert sum(doc["bins"]["extra"]["pressure"]["count"]) == 6000 // (32 * 32)


def test_yaml_floats():
    assert export._yaml(1e-05) == "1.0e-05"
    assert export._yaml(-2.5e+300) == "-2.5e+300"
    assert export._yaml(float("inf")) == ".inf" and export._yaml(float("-inf")) == "-.inf"
    assert export._yaml({"a": [1, 2.0, None, True, "x"]}) == '{"a": [1, 2.0, null, true, "x"]}'


def test_dat_files(oracle, tmp_path):
    """The parse-binning.py:176-190 files: padding, orientation and the SAD entropy."""
    w = wca_walker(oracle, "sad", 6000)
    doc = export.document(OracleView(w))
    base = str(tmp_path / "wca")
    export.write_dat(doc, base)
    n = len(doc["bins"]["lnw"])
    eb = np.loadtxt(base + "-energy-boundaries.dat")
    assert len(eb) == n + 1 and eb[0] == doc["bins"]["min"]
    np.testing.assert_allclose(np.diff(eb), doc["bins"]["width"])
    me = np.loadtxt(base + "-mean-energy.dat")
    assert len(me) == n + 2 and np.isnan(me[0]) and np.isnan(me[-1])
    h = np.array(doc["bins"]["histogram"], float)
    vis = h > 0
    np.testing.assert_allclose(me[1:-1][vis], np.array(doc["bins"]["energy_total"])[vis] / h[vis])
    # each visited bin's mean energy lies in the bin
    assert np.all(me[1:-1][vis] >= eb[:-1][vis] - 1e-9) and np.all(me[1:-1][vis] < eb[1:][vis] + 1e-9)
    hist = np.loadtxt(base + "-histogram.dat")
    assert hist[0] == 0 and hist[-1] == 0 and np.array_equal(hist[1:-1], h)
    lnw = np.loadtxt(base + "-lnw.dat")
    assert len(lnw) == n + 2 and lnw[0] == -np.inf and lnw[-1] == -np.inf
    assert abs(np.log(np.exp(lnw[1:-1]).sum())) < 1e-12  # normalised
    # inside the SAD window the entropy is ln w itself, up to the normalising constant
    sad = doc["method"]["Sad"]
    E = doc["bins"]["min"] + (np.arange(n) + 0.5) * doc["bins"]["width"]
    win = (E >= sad["too_lo"]) & (E <= sad["too_hi"])
    raw = np.array(doc["bins"]["lnw"])
    d = lnw[1:-1][win] - raw[win]
    np.testing.assert_allclose(d, d[0], atol=1e-9)
    # below the window: slope 1/min_T plus ln(hist / mean window hist)
    s = export.excess_entropy(doc)
    i_lo = int(np.abs(E - sad["too_lo"]).argmin())
    i_hi = int(np.abs(E - sad["too_hi"]).argmin())
    mh = h[i_lo:i_hi + 1].mean()
    k = int(np.nonzero(win)[0][0])  # a bin the reconstruction leaves alone
    below = np.nonzero((E < sad["too_lo"]) & (h > 0))[0]
    assert len(below) > 0
    for i in below:
        want = raw[i_lo] + (E[i] - sad["too_lo"]) / 0.5 + np.log(h[i] / mh)
        assert s[i] - s[k] == pytest.approx(want - raw[k], abs=1e-9)
    p = np.loadtxt(base + "-pressure.dat")
    assert len(p) == n + 2 and p[0] == -np.inf and p[-1] == -np.inf
    c = np.array(doc["bins"]["extra"]["pressure"]["count"])
    t = np.array(doc["bins"]["extra"]["pressure"]["total"])
    k = int(np.nonzero(c)[0][0])
    assert p[::-1][1 + k] == pytest.approx(t[k] / c[k], rel=1e-15)  # written high energy first
    sysd = read_flow_yaml(base + "-system.dat")
    assert sysd["kind"] == "WCA" and sysd["N"] == 32
    assert sysd["density"] == pytest.approx(0.6, rel=1e-12)


def test_wl_production_entropy(oracle, tmp_path):
    """A Wang-Landau production run (gamma reported 0) adds ln of its histogram."""
    spins = np.where(np.random.default_rng(4).random(16) < 0.5, -1.0, 1.0)
    w = oracle.Walker(oracle.make_config(oracle.ISING, 4, method=oracle.M_WL, seed=2,
                                         min_gamma=1e-3), spins)
    w.run(200000)
    doc = export.document(OracleView(w))
    wl = doc["method"]["WL"]
    assert wl["min_gamma"] == 1e-3 and wl["inv_t"] is False
    on_bins = export.wl_hist_on_bins(doc)
    assert on_bins.sum() == sum(wl["hist"])
    doc["method"]["WL"]["gamma"] = 0.0
    s = export.excess_entropy(doc)
    raw = np.array(doc["bins"]["lnw"])
    pos = on_bins > 0
    want = raw.copy()
    want[pos] += np.log(on_bins[pos])
    np.testing.assert_allclose(s, want - want.max())
    base = str(tmp_path / "ising")
    export.write_dat(doc, base)
    assert not os.path.exists(base + "-pressure.dat")
    assert read_flow_yaml(base + "-system.dat") == {"kind": "unknown"}
