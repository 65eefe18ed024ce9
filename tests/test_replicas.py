"""Multi-GPU replica coordination, exercised with two gloo ranks on the CPU: disjoint
walker ranges and streams, max-over-ranks timing, host gather (no GPU involved)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "sad-monte-carlo_gb300"))
    import torch.distributed as dist
    import replicas as R
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    walkers = list(R.walker_range(rank, 4))
    t = R.max_over_ranks(1.0 + rank)
    s = R.sum_over_ranks(len(walkers))
    g = R.gather_to_rank0(np.arange(3, dtype=np.float64) + 10 * rank)
    seed = R.rank_seed(7, rank)
    np.save(os.path.join(out_dir, f"r{rank}.npy"),
            np.array([walkers[0], walkers[-1], t, s, seed % 1000003], dtype=np.float64))
    if rank == 0:
        np.save(os.path.join(out_dir, "gather.npy"), np.stack(g))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    r0, r1 = np.load(tmp_path / "r0.npy"), np.load(tmp_path / "r1.npy")
    assert (r0[0], r0[1], r1[0], r1[1]) == (0, 3, 4, 7)   # disjoint walker ranges
    assert r0[2] == r1[2] == 2.0                          # slowest rank's time everywhere
    assert r0[3] == r1[3] == 8                            # all walkers counted once
    assert r0[4] != r1[4]                                 # distinct streams
    g = np.load(tmp_path / "gather.npy")
    np.testing.assert_array_equal(g, [[0, 1, 2], [10, 11, 12]])
