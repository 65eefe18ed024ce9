"""The learned surrogate on the GPU against the FP64 oracle statement (oracle/mlp_oracle.py):
bf16 tensor-core forward, FP32 backward (gradients), and online training."""
import numpy as np
import pytest

import mlp_oracle as M
from helpers import lj_configs

pytestmark = pytest.mark.gpu


def batch_with_surrogate(gpu, oracle, n=38, W=16, seed=0):
    R = 3.5
    confs = lj_configs(oracle, n, R, range(300, 300 + W))
    cfg = gpu.make_config(gpu.LJ, W, n, energy_bin=0.134, max_allowed=0.0, e_lo=-180, e_hi=1,
                          target_rate=0.5, translation_scale=0.1, seed=seed)
    b = gpu.Batch(cfg, [(n, R, (0, 0, 0))] * W)
    b.upload(confs)
    b.initialize()
    b.surrogate_init(seed=5, ring_capacity=4096)
    return b, confs


def test_forward_matches_fp64_statement(gpu, oracle):
    b, confs = batch_with_surrogate(gpu, oracle)
    p = gpu.unpack_params(b.surrogate_params())
    p["b1"][:] = np.linspace(-0.2, 0.2, 64)
    p["b2"][:] = np.linspace(0.1, -0.1, 64)
    p["b3"][:] = 0.05
    b.surrogate_set_params(gpu.pack_params(p))
    p = gpu.unpack_params(b.surrogate_params())
    pos = np.array(confs, np.float32)
    got = b.surrogate_predict(pos)
    want = []
    for c in pos.astype(np.float64):
        G = M.descriptors(c)
        e, _ = M.forward(G, p, emulate_bf16=True)
        want.append(e.sum())
    want = np.array(want)
    # binary32 descriptors/accumulation vs FP64, bf16 rounding of h1 at different points
    np.testing.assert_allclose(got, want, rtol=2e-2, atol=2e-2 * np.abs(want).max())


def test_gradients_match_fp64_statement(gpu, oracle):
    b, confs = batch_with_surrogate(gpu, oracle)
    pos = np.array(confs, np.float32)
    n = pos.shape[1]
    target = np.array([oracle.Walker(oracle.make_config(oracle.LJ, n, radius=3.5), c).compute_energy()
                       for c in confs], np.float32)
    loss, g = b.surrogate_loss_grads(pos, target)
    p = gpu.unpack_params(b.surrogate_params())
    G = np.concatenate([M.descriptors(c) for c in pos.astype(np.float64)])
    loss_o, g_o = M.loss_and_grads(G, n, target.astype(np.float64), p, emulate_bf16=True)
    assert loss == pytest.approx(loss_o, rel=2e-2)
    gg = gpu.unpack_params(g)
    for name in g_o:
        a, o = gg[name].ravel(), np.asarray(g_o[name]).ravel()
        scale = np.abs(o).max() + 1e-12
        assert np.max(np.abs(a - o)) / scale < 3e-2, (name, np.max(np.abs(a - o)) / scale)


def test_online_training_reduces_the_error(gpu, oracle):
    b, _ = batch_with_surrogate(gpu, oracle, W=64)
    for _ in range(20):
        b.run(500)
        b.surrogate_collect()
    first = b.surrogate_train(1, batch=256, lr=2e-3, seed=1)
    last = b.surrogate_train(400, batch=256, lr=2e-3, seed=2)
    assert last < 0.2 * first, (first, last)
