"""The CUDA path against the reference's own LJ31 numbers (tests/golden/
lj31_cv_reference.json): the headline workload's configuration (LJ31, R = 2.5, SAD min_T
0.2, 1000 bins of 0.134 over [-134, 0], step 0.1 adapted to 50 %) run long on the GPU;
each walker's heat capacity, reconstructed in FP64 on the device from its own bins,
follows the Rc = 2.5 reference curves (RESTMC, t-REM) from T = 0.25 through the melting
peak, and no walker visits an energy below the LJ31 ground state -133.586422
(big-lj-31.sh:16).  The per-walker reconstruction is first checked against its FP64
numpy statement (oracle/cv_oracle.py)."""
import json
import os

import numpy as np
import pytest

import cv_oracle as CV
from helpers import sphere_configs

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "lj31_cv_reference.json")
T_CHECK = np.array([0.25, 0.28, 0.30, 0.33, 0.36])


def c2_batch(gpu, oracle, W, seed, lpw=0):
    width = 0.134
    cfg = gpu.make_config(gpu.LJ, W, 31, method=gpu.SAD, min_T=0.2, energy_bin=width, max_allowed=0.0,
                          e_lo=-134.0 - 2 * width, e_hi=2 * width, target_rate=0.5,
                          translation_scale=0.1, seed=seed, lanes_per_walker=lpw)
    b = gpu.Batch(cfg, [(31, 2.5, (0, 0, 0))] * W)
    b.upload(sphere_configs(31, 2.5, W, seed=3000 + seed))
    b.initialize()
    return b


def test_walker_heat_capacity_matches_the_statement(gpu, oracle):
    """sadmc_walker_heat_capacity (FP64, from the bin planes) against the numpy statement
    on each walker's bins, for SAD (window extension), SAMC and Wang-Landau production."""
    T = np.linspace(0.2, 0.5, 13)
    b = c2_batch(gpu, oracle, 16, seed=3)
    b.run(200_000)
    C = b.heat_capacities(T)
    for w in range(b.W):
        want = CV.heat_capacity(T, *CV.walker_entropy(b.bins(w), b.scalars(w), min_T=0.2))
        np.testing.assert_allclose(C[w], want, rtol=1e-9, err_msg=f"SAD walker {w}")
    L, W = 4, 8
    for kw in (dict(method=1, t0=200.0), dict(method=2, min_gamma=0.02)):
        cfg = gpu.make_config(gpu.ISING, W, L, e_lo=-36, e_hi=36, seed=12, **kw)
        ib = gpu.Batch(cfg, [(L, 0.0, (0, 0, 0))] * W)
        ib.upload([np.where(np.random.default_rng(50 + w).random(L * L) < 0.5, -1.0, 1.0) for w in range(W)])
        ib.initialize()
        ib.run(300_000)
        Ti = np.linspace(1.0, 4.0, 7)
        Ci = ib.heat_capacities(Ti)
        for w in range(W):
            s = ib.scalars(w)
            wl = None
            if kw["method"] == 2 and s["gamma"] == 0.0:
                bb = ib.bins(w)
                h, emin = ib.wl_hist(w)  # the production histogram starts at its min_energy
                wl = np.zeros(len(bb["hist"]))
                off = int(round((emin - bb["min"]) / bb["width"]))
                for k, v in enumerate(h):
                    if 0 <= off + k < len(wl):
                        wl[off + k] = v
            want = CV.heat_capacity(Ti, *CV.walker_entropy(ib.bins(w), s, wl_hist=wl))
            np.testing.assert_allclose(Ci[w], want, rtol=1e-9, err_msg=f"{kw} walker {w}")


def test_gpu_lj31_heat_capacity_matches_the_reference(gpu, oracle):
    g = json.load(open(GOLDEN))
    ref = np.mean([np.interp(T_CHECK, g["curves"][k]["T"], g["curves"][k]["Cv"])
                   for k in ("RESTMC", "t-REM")], axis=0)
    W, moves = 512, 40_000_000
    b = c2_batch(gpu, oracle, W, seed=29)
    for _ in range(moves // 4_000_000):
        b.run(4_000_000)
    assert not b.status().any()
    C = b.heat_capacities(T_CHECK)
    med = np.median(C, axis=0)
    rel = np.abs(med - ref) / ref
    # 512 walkers x 4e7 moves: within 5 % of the reference at every T checked
    assert rel.max() < 0.05, (med, ref, rel)
    for w in range(W):
        bb = b.bins(w)
        lowest = bb["min"] + np.nonzero(np.asarray(bb["hist"]))[0][0] * bb["width"]
        assert lowest + bb["width"] > g["ground_state"], (w, lowest)
    assert (b.compute_energies() >= g["ground_state"] - 1e-9).all()
