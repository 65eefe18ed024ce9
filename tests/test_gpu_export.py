"""The export of GPU walkers to the reference's save format equals the export of the
oracle walkers on the same chain (Ising: bit-exact), movie frames included."""
import os

import numpy as np
import pytest

import export
from helpers import METHOD_KW, OracleView, ising_spins, read_flow_yaml

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["sad", "wl"])
def test_ising_documents_and_movie(gpu, oracle, method, tmp_path):
    L, W, moves, seed, movie_time = 6, 4, 20000, 23, 1.6
    kw = METHOD_KW[method]
    N = L * L
    cfg = gpu.make_config(gpu.ISING, W, L, e_lo=-2.0 * N - 4, e_hi=2.0 * N + 4, seed=seed, **kw)
    b = gpu.Batch(cfg, [(L, 0.0, (0, 0, 0))] * W)
    spins = [ising_spins(L, 500 + w) for w in range(W)]
    b.upload(spins)
    b.initialize()
    save_as = str(tmp_path / "ising-{walker}.yaml")
    frames = export.run_with_movie(b, moves, movie_time, save_as)
    assert frames == export.movie_times(movie_time, moves)
    for w in range(W):
        ow = oracle.Walker(oracle.make_config(oracle.ISING, L, seed=seed, walker=w, **kw), spins[w])
        done = 0
        d = export.movie_dir(save_as.format(walker=w))
        assert sorted(os.listdir(d)) == [f"{t:014d}.yaml" for t in frames]
        for t in frames[-3:]:
            ow.run(t - done)
            done = t
            got = read_flow_yaml(os.path.join(d, f"{t:014d}.yaml"))
            assert got == export.document(OracleView(ow)), (w, t)
        ow.run(moves - done)
        final = read_flow_yaml(save_as.format(walker=w))
        assert final == export.document(OracleView(ow)), w
        assert final["moves"] == moves
        base = str(tmp_path / f"ising-{w}")
        export.write_dat(final, base)
        lnw = np.loadtxt(base + "-lnw.dat")
        assert abs(np.log(np.exp(lnw[1:-1]).sum())) < 1e-12
