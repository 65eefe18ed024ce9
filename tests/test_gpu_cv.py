"""Heat capacity from GPU runs against answers known exactly: the 4x4 periodic Ising
lattice, whose density of states is enumerated in tests/golden (SAD and SAMC runs, Cv(T)
reconstructed in FP64 on the GPU, plotting/final_heat_capacity.py:79-88).  SAMC's ln w
error after t moves scales as sqrt(t0 / t); t0 = 200 suits 16 spins."""
import json
import os

import numpy as np
import pytest

from helpers import ising_spins

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.json")


def exact_cv(T):
    g = json.load(open(GOLDEN))["ising4_exact"]
    E, S = np.array(g["E"], float), np.array(g["lng"])
    out = []
    for t in T:
        b = S - E / t
        P = np.exp(b - b.max())
        P /= P.sum()
        U = (E * P).sum()
        out.append(((E - U) ** 2 * P).sum() / t ** 2)
    return np.array(out)


@pytest.mark.parametrize("method,kw", [("sad", dict(method=0, min_T=0.5)),
                                       ("samc", dict(method=1, t0=200.0))])
def test_ising4_cv_error(gpu, method, kw):
    L, W = 4, 64
    cfg = gpu.make_config(gpu.ISING, W, L, e_lo=-36, e_hi=36, seed=12, **kw)
    b = gpu.Batch(cfg, [(L, 0.0, (0, 0, 0))] * W)
    b.upload([ising_spins(L, 100 + w) for w in range(W)])
    b.initialize()
    b.run(400_000)
    T = np.linspace(1.0, 4.0, 31)
    ref = exact_cv(T)
    cvs = np.array([gpu.cv_from_bins(b.bins(w), T) for w in range(W)])
    mean = cvs.mean(axis=0)
    err = np.max(np.abs(mean - ref) / ref.max())
    assert err < 0.02, (method, err)
    # each walker's own estimate is unbiased within its spread
    spread = cvs.std(axis=0).max() / ref.max()
    assert spread < 0.1, spread
