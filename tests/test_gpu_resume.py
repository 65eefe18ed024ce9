"""Checkpoint / resume of a GPU batch, modelled on tests/resume-sad.rs:10-97: N moves
straight equals k moves, checkpoint, resume in a new handle, and N - k more moves."""
import os

import numpy as np
import pytest

from helpers import BIN_KEYS, ising_spins, lj_configs

pytestmark = pytest.mark.gpu


def same(b1, b2):
    assert b1.W == b2.W
    for w in range(b1.W):
        x, y = b1.bins(w), b2.bins(w)
        assert x["min"] == y["min"]
        for k in BIN_KEYS:
            assert np.array_equal(x[k], y[k]), k
        s1, s2 = b1.scalars(w), b2.scalars(w)
        assert s1 == s2
        assert np.array_equal(b1.state(w), b2.state(w))


@pytest.mark.parametrize("k", [1, 500, 999])
def test_resume_ising_bit_exact(gpu, tmp_path, k):
    L, W, N = 8, 16, 1000
    cfg = gpu.make_config(gpu.ISING, W, L, e_lo=-132, e_hi=132, seed=3)
    spins = [ising_spins(L, w) for w in range(W)]
    straight = gpu.Batch(cfg, [(L, 0.0, (0, 0, 0))] * W)
    straight.upload(spins); straight.initialize(); straight.run(N)
    part = gpu.Batch(cfg, [(L, 0.0, (0, 0, 0))] * W)
    part.upload(spins); part.initialize(); part.run(k)
    path = str(tmp_path / "ck.sadmc")
    part.checkpoint(path)
    assert os.path.exists(path) and not os.path.exists(path + ".tmp")
    part.close()
    resumed = gpu.Batch.resume(path)
    resumed.run(N - k)
    same(straight, resumed)


def test_resume_lj_and_square_well(gpu, oracle, tmp_path):
    n, W, R, N, k = 31, 8, 2.5, 3000, 1234
    confs = lj_configs(oracle, n, R, range(20, 20 + W))
    cfg = gpu.make_config(gpu.LJ, W, n, energy_bin=0.134, max_allowed=0.0, e_lo=-140, e_hi=1,
                          target_rate=0.5, translation_scale=0.1, seed=8, resum_interval=500)
    a = gpu.Batch(cfg, [(n, R, (0, 0, 0))] * W)
    a.upload(confs); a.initialize(); a.run(N)
    b = gpu.Batch(cfg, [(n, R, (0, 0, 0))] * W)
    b.upload(confs); b.initialize(); b.run(k)
    b.checkpoint(str(tmp_path / "lj.ck"))
    c = gpu.Batch.resume(str(tmp_path / "lj.ck"))
    c.run(N - k)
    same(a, c)
    pos, box = oracle.init_sw_fcc(108, 0.4, 1.3, 2)
    cfg = gpu.make_config(gpu.SW, 2, 108, method=2, e_lo=-6 * 108 - 2, e_hi=2, seed=1)
    a = gpu.Batch(cfg, [(108, 0.0, box)] * 2)
    a.upload([pos, pos]); a.initialize(); a.run(2000)
    b = gpu.Batch(cfg, [(108, 0.0, box)] * 2)
    b.upload([pos, pos]); b.initialize(); b.run(700)
    b.checkpoint(str(tmp_path / "sw.ck"))
    c = gpu.Batch.resume(str(tmp_path / "sw.ck"))
    c.run(1300)
    same(a, c)


def test_resume_rejects_garbage(gpu, tmp_path):
    p = tmp_path / "bad.ck"
    p.write_bytes(b"not a checkpoint")
    with pytest.raises(gpu.SadmcError):
        gpu.Batch.resume(str(p))
