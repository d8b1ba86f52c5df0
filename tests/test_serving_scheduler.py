"""Host parts of the serving path (no GPU): the device bytes a request is
charged against the HBM budget (gpi_plan_estimate, computed without
allocating), the request arrays the client hands to the C server, and the
server's refusal to start without a device.  Admission, overlap and the
alone == mixed property run on the GPU (test_serving_gpu.py)."""
import ctypes
import os

import numpy as np
import pytest

from geophyinv_gb300 import _build, _lib, serving


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_build.LIB):
        _build.build()
    return _lib.load()


def _desc(npw=1, checkpoints=0, nz=300, nx=400, nshots=2, nt=100, order=4):
    d = _lib.PlanDesc()
    d.physics, d.ndim, d.order = 0, 2, order
    d.nz, d.ny, d.nx, d.npml, d.nbound, d.nt, d.nshots, d.npw = nz, 1, nx, 43, 3, nt, nshots, npw
    d.dt, d.dz, d.dx, d.dy = 5e-4, 5.0, 5.0, 1.0
    d.pml_faces = d.rigid_faces = 0x33
    d.checkpoints = checkpoints
    return d


def _estimate(lib, d):
    b = ctypes.c_size_t()
    assert lib.gpi_plan_estimate(ctypes.byref(d), ctypes.byref(b)) == 0, lib.gpi_last_error(None)
    return b.value


def test_plan_estimate_covers_the_layout_and_grows_with_the_work(lib):
    fwd = _estimate(lib, _desc())
    # at least both buffers of p, vx, vz for every shot on the padded grid
    assert fwd >= 2 * 3 * 2 * 300 * 400 * 4
    assert _estimate(lib, _desc(nshots=4)) > fwd
    grad = _estimate(lib, _desc(npw=2))
    assert grad > 2 * fwd * 0.9  # two wavefields and the boundary store
    c2, c4 = _estimate(lib, _desc(npw=2, checkpoints=2)), _estimate(lib, _desc(npw=2, checkpoints=4))
    assert c4 > c2 and (c4 - c2) % 2 == 0
    o2 = _estimate(lib, _desc(order=2))
    o8 = _estimate(lib, _desc(order=8))
    assert o8 > o2 > 0  # a wider padding at order 8
    bad = _desc(npw=2)
    bad.order = 2
    assert lib.gpi_plan_estimate(ctypes.byref(bad), ctypes.byref(ctypes.c_size_t())) == -4


def test_request_arrays_follow_the_workload(lib):
    req = serving.make_stream(1, rate=10.0, seed=5, sides=(60, 90), steps=(40, 60), shots=(2, 3))[0]
    rb = serving.RequestBuffers(req)
    wl = req.payload()
    d = rb.desc
    assert (d.nz, d.nx) == (len(wl.grid[0]) + 86, len(wl.grid[1]) + 86)
    assert d.nshots == len(wl.shots) and d.nt == wl.nt
    assert d.npw == (2 if req.kind == "acoustic_gradient" else 1)
    assert len(rb.pml) == (8 if wl.physics == "elastic" else 4) * 3 * 2 * 43
    assert rb.request.nrec == len(wl.shots) * len(wl.rfields)
    assert all(np.isfinite(m).all() for m in rb.mod)
    assert serving.request_bytes(req) > _estimate(lib, rb.desc)


def test_server_needs_a_device(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    d = _lib.ServerDesc()
    d.device, d.max_inflight, d.hbm_budget = 0, 2, 1 << 30
    h = ctypes.c_void_p()
    assert lib.gpi_server_create(ctypes.byref(d), ctypes.byref(h)) == -3
    assert b"device" in lib.gpi_server_message(None, 0)
    d.max_inflight = 0
    assert lib.gpi_server_create(ctypes.byref(d), ctypes.byref(h)) == -1
