"""sadmc_surrogate_loss_grads_noalloc through the C ABI: caller device buffers, the static
scratch, called twice in a row, against the allocating sadmc_surrogate_loss_grads; a
request above the static scratch is refused before anything is launched."""
import numpy as np
import pytest

from helpers import lj_configs

pytestmark = pytest.mark.gpu


def test_noalloc_loss_grads_match_the_allocating_entry_point(gpu, oracle):
    torch = pytest.importorskip("torch")
    n, W, R = 38, 16, 3.5
    confs = lj_configs(oracle, n, R, range(300, 300 + W))
    cfg = gpu.make_config(gpu.LJ, W, n, energy_bin=0.134, max_allowed=0.0, e_lo=-180, e_hi=1,
                          target_rate=0.5, translation_scale=0.1, seed=0)
    b = gpu.Batch(cfg, [(n, R, (0, 0, 0))] * W)
    b.upload(confs)
    b.initialize()
    b.surrogate_init(seed=5, ring_capacity=4096)
    pos = np.array(confs, np.float32)
    target = np.array([oracle.Walker(oracle.make_config(oracle.LJ, n, radius=R), c).compute_energy()
                       for c in confs], np.float32)
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
        b.surrogate_loss_grads_noalloc(pos_d.data_ptr(), tgt_d.data_ptr(), W, loss_d.data_ptr(),
                                       g_d.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        loss = float(loss_d.cpu()[0])
        g = g_d.cpu().numpy()
        # same kernels on the same inputs; the loss is an FP64 atomic sum (order only)
        assert loss == pytest.approx(loss_ref, rel=1e-9)
        np.testing.assert_allclose(g, g_ref, rtol=1e-6, atol=1e-6 * np.abs(g_ref).max())

    too_many = 4096 // n + 1         # configs x atoms above SADMC_SG_NOALLOC_MAX_ROWS
    with pytest.raises(gpu.SadmcError, match="static scratch"):
        b.surrogate_loss_grads_noalloc(pos_d.data_ptr(), tgt_d.data_ptr(), too_many,
                                       loss_d.data_ptr(), g_d.data_ptr(), stream.cuda_stream)
