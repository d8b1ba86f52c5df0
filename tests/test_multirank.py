"""Shot sharding and the gradient sum over ranks, as world_size-2 gloo
processes on the CPU (the GPU path runs one rank per GPU the same way)."""
import os
import socket

import numpy as np
import pytest

from geophyinv_gb300 import shots


def test_sschunks_match_the_reference_split():
    # round.(range(0, nss, length = nworker + 1)), ties to even
    assert shots.sschunks(16, 3) == [(0, 5), (5, 11), (11, 16)]
    assert shots.sschunks(32, 8) == [(4 * i, 4 * i + 4) for i in range(8)]
    assert shots.sschunks(5, 2) == [(0, 2), (2, 5)]  # round(2.5) = 2
    assert shots.sschunks(3, 8) == [(0, 1), (1, 2), (2, 3)]  # no more workers than shots
    assert list(shots.my_shots(3, 5, 8)) == []
    for nss in range(1, 40):
        for w in range(1, 9):
            c = shots.sschunks(nss, w)
            assert c[0][0] == 0 and c[-1][1] == nss
            assert all(a[1] == b[0] for a, b in zip(c, c[1:]))


def _per_shot_gradient(iss, shape):
    rng = np.random.default_rng(100 + iss)
    return rng.standard_normal(shape).astype(np.float32)


def _worker(rank, world, port, nss, shape, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        g = np.zeros(shape, np.float32)
        for iss in shots.my_shots(nss, rank, world):
            g += _per_shot_gradient(iss, shape)
        shots.reduce_gradient(g)
        np.save(os.path.join(out, "g%d.npy" % rank), g)
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.mark.parametrize("nss", [1, 5, 16])
def test_gradient_sum_over_two_ranks(tmp_path, nss):
    import torch.multiprocessing as mp

    shape = (7, 9)
    mp.spawn(_worker, args=(2, _free_port(), nss, shape, str(tmp_path)), nprocs=2, join=True)
    want = sum(_per_shot_gradient(i, shape).astype(np.float64) for i in range(nss))
    for r in range(2):
        g = np.load(tmp_path / ("g%d.npy" % r))
        np.testing.assert_allclose(g, want, rtol=1e-5, atol=1e-5)
