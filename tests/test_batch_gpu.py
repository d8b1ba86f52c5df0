"""Batches (gpi_batch_*, update_batch): several forward experiments advanced
by the same launches -- one per tile class and time step over the tiles of
all of them -- give each experiment the records of its own update!(pa), bit
for bit: acoustic and elastic media, different grids, shot counts and step
counts (members leave the batch at different steps, step counts that are
not multiples of the 16-step graph)."""
import numpy as np
import pytest

from geophyinv_gb300 import configs, update, update_batch


def _acoustic(nz, nx, nt, nshots, seed):
    wl = configs.acoustic2d_layers(nz=nz, nx=nx, nt=nt, nrec=max(8, nx // 4), seed=seed, rfields=("p", "vz"))
    src, rec = wl.shots[0]
    xm = wl.grid[1].last
    wl.shots = [(np.array([[src[0, 0], x]]), rec) for x in np.linspace(0.0, xm, nshots + 2)[1:-1]]
    return wl


def _elastic(nz, nx, nt, nshots, seed):
    return configs.elastic2d_batch(nz=nz, nx=nx, nt=nt, nshots=nshots, nrec=max(8, nx // 4), seed=seed)


def _records(pa):
    return [{f: r.d[f].copy() for f in pa.rfields} for r in pa.data[0]]


def _check_batch(workloads):
    import torch

    stream = torch.cuda.Stream()
    alone = []
    for wl in workloads:
        pa = wl.expt(stream=stream.cuda_stream)
        update(pa)
        alone.append(_records(pa))
        pa.close()
    pas = [wl.expt(stream=stream.cuda_stream) for wl in workloads]
    update_batch(pas, max_steps=40)
    for k, pa in enumerate(pas):
        got = _records(pa)
        for s, (a, b) in enumerate(zip(alone[k], got)):
            for f in a:
                assert np.any(a[f] != 0), (k, s, f)
                assert np.array_equal(a[f], b[f]), (k, s, f, float(np.max(np.abs(a[f] - b[f]))))
        # a member keeps working as a plain experiment afterwards
        update(pa)
        again = _records(pa)
        for a, b in zip(alone[k], again):
            for f in a:
                assert np.array_equal(a[f], b[f]), (k, "after", f)
        pa.close()


@pytest.mark.gpu
def test_acoustic_batch_equals_runs_alone(engine):
    _check_batch([_acoustic(120, 200, 171, 2, 1), _acoustic(90, 310, 96, 1, 2), _acoustic(200, 140, 203, 3, 3),
                  _acoustic(64, 90, 37, 1, 4)])


@pytest.mark.gpu
def test_elastic_batch_equals_runs_alone(engine):
    _check_batch([_elastic(110, 190, 150, 2, 5), _elastic(140, 120, 83, 1, 6), _elastic(90, 260, 120, 3, 7)])


@pytest.mark.gpu
def test_batch_rejects_mixed_physics(engine):
    import torch

    from geophyinv_gb300 import _lib

    stream = torch.cuda.Stream()
    L = _lib.load()
    a = _acoustic(60, 80, 20, 1, 1).expt(stream=stream.cuda_stream)
    e = _elastic(60, 80, 20, 1, 1).expt(stream=stream.cuda_stream)
    import ctypes

    b = ctypes.c_void_p()
    assert L.gpi_batch_create(torch.cuda.current_device(), None, ctypes.byref(b)) == 0
    try:
        assert L.gpi_batch_add(b, a.plan) == 0
        assert L.gpi_batch_add(b, e.plan) == -1
        assert b"physics" in L.gpi_batch_error(b)
        assert L.gpi_batch_add(b, a.plan) == -1  # already a member
        active = ctypes.c_int32()
        while True:
            assert L.gpi_batch_advance(b, 64, ctypes.byref(active)) == 0
            if active.value == 0:
                break
        done = (ctypes.c_void_p * 4)()
        n = ctypes.c_int32()
        assert L.gpi_batch_finished(b, done, 4, ctypes.byref(n)) == 0
        assert n.value == 1 and done[0] == a.plan.value
    finally:
        L.gpi_batch_destroy(b)
    a.close()
    e.close()
