"""The FP64 oracle pinned to the reference's own LJ31 numbers (tests/golden/
lj31_cv_reference.json, made by tests/golden/make_lj31_cv.py from the reference's CSV
curves): the LJ31 ground state -133.586422 (big-lj-31.sh:16) bounds every energy the
oracle visits, and the heat capacity of the LJ31 workload (R = 2.5, SAD min_T 0.2, bins
of 0.134) reconstructed from its walkers' ln w (plotting/final_heat_capacity.py:79-88,
entropy as plotting/parse-binning.py:136-160) follows the Rc = 2.5 reference curves
(RESTMC and t-REM) from T = 0.25 through the melting peak.  Below T = 0.25 the SAD window
of min_T 0.2 does not reach: the entropy there is the slope-1/min_T extension."""
import json
import os
import threading

import numpy as np

import cv_oracle as CV

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "lj31_cv_reference.json")
T_CHECK = np.array([0.25, 0.28, 0.30, 0.33, 0.36])


def reference():
    g = json.load(open(GOLDEN))
    curves = [g["curves"][k] for k in ("RESTMC", "t-REM")]
    ref = np.mean([np.interp(T_CHECK, c["T"], c["Cv"]) for c in curves], axis=0)
    return g, ref


def test_fixture_holds_the_reference_curves():
    g, ref = reference()
    assert g["ground_state"] == -133.586422
    assert set(g["curves"]) == {"REM", "RESTMC", "MCET", "EMC", "t-REM"}
    # every curve agrees within 10 % below T = 0.25; the Rc = 2.5 pair within 2 % throughout
    for t in (0.05, 0.1, 0.15, 0.2):
        vals = [np.interp(t, c["T"], c["Cv"]) for c in g["curves"].values()]
        assert (max(vals) - min(vals)) / min(vals) < 0.10, (t, vals)
    a, b = g["curves"]["RESTMC"], g["curves"]["t-REM"]
    for t in T_CHECK:
        x, y = np.interp(t, a["T"], a["Cv"]), np.interp(t, b["T"], b["Cv"])
        assert abs(x - y) / x < 0.02, (t, x, y)
    assert 115 < ref[3] < 125  # the melting peak near T = 0.33


def test_oracle_lj31_heat_capacity_matches_the_reference(oracle):
    g, ref = reference()
    W, moves, width, min_T = 24, 40_000_000, 0.134, 0.2
    ws = []
    for w in range(W):
        pos, ok = oracle.init_lj(31, 2.5, 100 + w)
        assert ok
        ws.append(oracle.Walker(oracle.make_config(oracle.LJ, 31, radius=2.5, method=oracle.M_SAD,
                                                   min_T=min_T, energy_bin=width, max_allowed=0.0,
                                                   target_rate=0.5, translation_scale=0.1, seed=5,
                                                   walker=w), pos))
    # ctypes releases the GIL: one host thread per walker slot
    slots = list(range(W))
    lock = threading.Lock()

    def worker():
        while True:
            with lock:
                if not slots:
                    return
                w = slots.pop()
            ws[w].run(moves)
    threads = [threading.Thread(target=worker) for _ in range(min(W, os.cpu_count() or 1))]
    [t.start() for t in threads]
    [t.join() for t in threads]
    C = []
    for wk in ws:
        b, s = wk.bins(), wk.scalars()
        # no visited bin lies wholly below the ground state, nor does the final energy
        lowest = b["min"] + np.nonzero(np.asarray(b["hist"]))[0][0] * b["width"]
        assert lowest + b["width"] > g["ground_state"], lowest
        assert wk.energy() >= g["ground_state"] - 1e-9
        C.append(CV.heat_capacity(T_CHECK, *CV.walker_entropy(b, s, min_T=min_T)))
    med = np.median(np.array(C), axis=0)
    rel = np.abs(med - ref) / ref
    # 24 walkers x 4e7 moves: within 4 % of the reference (7 % allowed)
    assert rel.max() < 0.07, (med, ref, rel)
