"""sadmc_surrogate_loss_grads_noalloc through the C ABI: caller device buffers, the static
scratch, called twice in a row, against the allocating sadmc_surrogate_loss_grads; the
static scratch's limit of SADMC_SG_NOALLOC_MAX_ROWS = 4096 rows (configurations x atoms)
is accepted in full and a request one row above it is refused before anything launches."""
import numpy as np
import pytest

from helpers import sphere_configs

pytestmark = pytest.mark.gpu

MAX_ROWS = 4096


def _batch(gpu, oracle, n, W, R, seed=0):
    confs = sphere_configs(n, R, W, seed=300 + n)
    cfg = gpu.make_config(gpu.LJ, W, n, energy_bin=0.134, max_allowed=0.0, e_lo=-180, e_hi=1,
                          target_rate=0.5, translation_scale=0.1, seed=seed)
    b = gpu.Batch(cfg, [(n, R, (0, 0, 0))] * W)
    b.upload(confs)
    b.initialize()
    b.surrogate_init(seed=5, ring_capacity=4096)
    pos = np.array(confs, np.float32)
    target = np.array([oracle.Walker(oracle.make_config(oracle.LJ, n, radius=R), c).compute_energy()
                       for c in confs], np.float32)
    return b, pos, target


def _noalloc_twice(torch, b, pos, target):
    """Two calls in a row on poisoned outputs; both must match the allocating entry point."""
    loss_ref, g_ref = b.surrogate_loss_grads(pos, target)
    dev = torch.device("cuda:0")
    pos_d = torch.from_numpy(pos).to(dev)
    tgt_d = torch.from_numpy(target).to(dev)
    loss_d = torch.empty(1, dtype=torch.float64, device=dev)
    g_d = torch.empty(b.SG_NPARAM, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)  # an explicit stream: the entry point is stream-ordered
    for _ in range(2):
        loss_d.fill_(1e30)           # the entry point zeroes the loss before accumulating
        g_d.fill_(float("nan"))      # and overwrites every gradient
        torch.cuda.synchronize(dev)  # the fills ran on torch's own stream
        b.surrogate_loss_grads_noalloc(pos_d.data_ptr(), tgt_d.data_ptr(), len(target),
                                       loss_d.data_ptr(), g_d.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        loss = float(loss_d.cpu()[0])
        g = g_d.cpu().numpy()
        # the same kernels on the same inputs, tiles summed in a fixed order
        assert loss == pytest.approx(loss_ref, rel=1e-9)
        np.testing.assert_allclose(g, g_ref, rtol=1e-6, atol=1e-6 * np.abs(g_ref).max())
    return pos_d, tgt_d, loss_d, g_d, stream


def test_noalloc_loss_grads_match_the_allocating_entry_point(gpu, oracle):
    torch = pytest.importorskip("torch")
    n, W = 38, 16
    b, pos, target = _batch(gpu, oracle, n, W, 3.5)
    pos_d, tgt_d, loss_d, g_d, stream = _noalloc_twice(torch, b, pos, target)
    too_many = MAX_ROWS // n + 1     # configs x atoms above the static scratch
    with pytest.raises(gpu.SadmcError, match="static scratch"):
        b.surrogate_loss_grads_noalloc(pos_d.data_ptr(), tgt_d.data_ptr(), too_many,
                                       loss_d.data_ptr(), g_d.data_ptr(), stream.cuda_stream)


def test_noalloc_takes_the_whole_static_scratch(gpu, oracle):
    """32-atom configurations x 128 = exactly 4096 rows (the end of the scratch layout) are
    served; 17-atom configurations x 241 = 4097 rows are refused."""
    torch = pytest.importorskip("torch")
    n, W = 32, 128
    b, pos, target = _batch(gpu, oracle, n, W, 3.0)
    assert n * W == MAX_ROWS
    _noalloc_twice(torch, b, pos, target)
    n2, W2 = 17, 241
    assert n2 * W2 == MAX_ROWS + 1
    b2, pos2, target2 = _batch(gpu, oracle, n2, 4, 2.5)
    dev = torch.device("cuda:0")
    big = torch.zeros(W2 * n2 * 3, dtype=torch.float32, device=dev)
    tgt = torch.zeros(W2, dtype=torch.float32, device=dev)
    loss_d = torch.empty(1, dtype=torch.float64, device=dev)
    g_d = torch.empty(b2.SG_NPARAM, dtype=torch.float32, device=dev)
    with pytest.raises(gpu.SadmcError, match="static scratch"):
        b2.surrogate_loss_grads_noalloc(big.data_ptr(), tgt.data_ptr(), W2, loss_d.data_ptr(),
                                        g_d.data_ptr(), None)
