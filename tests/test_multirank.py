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


def _illum_worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # an FP64 column-major stack (pac.illum_stack of a sharded run)
        a = np.asfortranarray(np.arange(24, dtype=np.float64).reshape(4, 6) * (rank + 1) + 0.25)
        shots.reduce_gradient(a)
        np.save(os.path.join(out, "i%d.npy" % rank), a)
        assert a.flags.f_contiguous
    finally:
        dist.destroy_process_group()


def test_fp64_column_major_stack_sums_over_two_ranks(tmp_path):
    import torch.multiprocessing as mp

    mp.spawn(_illum_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    want = np.arange(24, dtype=np.float64).reshape(4, 6) * 3 + 0.5
    for r in range(2):
        assert np.array_equal(np.load(tmp_path / ("i%d.npy" % r)), want)


@pytest.mark.parametrize("nss", [1, 5, 16])
def test_gradient_sum_over_two_ranks(tmp_path, nss):
    import torch.multiprocessing as mp

    shape = (7, 9)
    mp.spawn(_worker, args=(2, _free_port(), nss, shape, str(tmp_path)), nprocs=2, join=True)
    want = sum(_per_shot_gradient(i, shape).astype(np.float64) for i in range(nss))
    for r in range(2):
        g = np.load(tmp_path / ("g%d.npy" % r))
        np.testing.assert_allclose(g, want, rtol=1e-5, atol=1e-5)


def _fwi_workload():
    from geophyinv_gb300 import configs

    return configs.acoustic2d_fwi(nz=40, nx=70, nt=200, nshots=3, nrec=11, anomaly=False)


def _oracle_worker(rank, world, port, out):
    """One rank: the oracle gradient of its own supersources (the engine's
    shard split), summed over the ranks with the product's reduction."""
    import torch.distributed as dist

    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        wl = _fwi_workload()
        ex = wl.as_dict()
        mine = list(shots.my_shots(len(ex["shots"]), rank, world))
        ex["shots"] = [ex["shots"][i] for i in mine]
        nr = len(wl.shots[0][1])
        dobs = {f: np.zeros((len(mine), wl.nt, nr), np.float32) for f in wl.rfields}
        loss, g, _, _ = O.gradient(ex, dobs, nthreads=1)
        gv = np.concatenate([g["invK"].ravel(order="F"), g["rho"].ravel(order="F")]).astype(np.float32)
        shots.reduce_gradient(gv)
        J = shots.reduce_scalar(loss)
        np.save(os.path.join(out, "g%d.npy" % rank), gv)
        np.save(os.path.join(out, "J%d.npy" % rank), np.array([J]))
    finally:
        dist.destroy_process_group()


def test_sharded_oracle_gradients_sum_to_the_single_rank_gradient(tmp_path):
    """Two CPU ranks each compute real per-shot FWI gradients (the oracle's
    gradient! on their chunk of 3 supersources: 2 + 1); the reduced
    gradient and misfit equal one rank's gradient over all supersources."""
    import torch.multiprocessing as mp

    from oracle import oracle as O

    mp.spawn(_oracle_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    wl = _fwi_workload()
    nr = len(wl.shots[0][1])
    dobs = {f: np.zeros((len(wl.shots), wl.nt, nr), np.float32) for f in wl.rfields}
    loss, g, _, _ = O.gradient(wl.as_dict(), dobs, nthreads=1)
    want = np.concatenate([g["invK"].ravel(order="F"), g["rho"].ravel(order="F")])
    for r in range(2):
        got = np.load(tmp_path / ("g%d.npy" % r))
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-6
        assert abs(np.load(tmp_path / ("J%d.npy" % r))[0] - loss) <= 1e-6 * abs(loss)


def _engine_worker(rank, world, port, out):
    """One rank on the (shared) GPU: a sharded experiment's gradient! ."""
    import torch.distributed as dist

    from geophyinv_gb300 import L2DistLoss, Recs, get_modelvector, gradient

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        wl = _fwi_workload()
        pa = wl.expt(mode="forward_save", shard=True)
        assert pa.nss == len(shots.my_shots(len(wl.shots), rank, world))
        dobs = [Recs(len(s[1]), wl.tgrid, list(wl.rfields),
                     {f: np.zeros((wl.nt, len(s[1])), np.float32) for f in wl.rfields}) for s in wl.shots]
        m = get_modelvector(pa, ["invK", "rho"])
        g = np.zeros_like(m)
        J = gradient(g, m, L2DistLoss(), dobs, pa)
        np.save(os.path.join(out, "g%d.npy" % rank), g)
        np.save(os.path.join(out, "J%d.npy" % rank), np.array([J]))
        pa.close()
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_sharded_engine_gradient_equals_the_single_rank_gradient(tmp_path):
    """Two gloo ranks drive the engine on the same GPU, each on its chunk of
    the supersources (no kernel waits on the other rank: the only exchange
    is the host-side sum); gradient! on the sharded experiment equals the
    one-rank gradient! over all supersources."""
    import torch.multiprocessing as mp

    from geophyinv_gb300 import L2DistLoss, Recs, get_modelvector, gradient

    mp.spawn(_engine_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    wl = _fwi_workload()
    pa = wl.expt(mode="forward_save")
    dobs = [Recs(len(s[1]), wl.tgrid, list(wl.rfields),
                 {f: np.zeros((wl.nt, len(s[1])), np.float32) for f in wl.rfields}) for s in wl.shots]
    m = get_modelvector(pa, ["invK", "rho"])
    want = np.zeros_like(m)
    J = gradient(want, m, L2DistLoss(), dobs, pa)
    for r in range(2):
        got = np.load(tmp_path / ("g%d.npy" % r))
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5
        assert abs(np.load(tmp_path / ("J%d.npy" % r))[0] - J) <= 1e-6 * abs(J)
