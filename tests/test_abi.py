"""The C ABI library loads and exports every entry point include/gpi_fdtd.h
declares (no compute without a GPU)."""
import os
import re

import pytest

from geophyinv_gb300 import _build, _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def _declared():
    names = set()
    for fn in os.listdir(HEADER):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(HEADER, fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(gpi_[a-z_0-9]+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_build.LIB):
        _build.build()
    return _lib.load()


def test_header_matches_binding():
    assert _declared() == set(_lib.EXPORTS)


def test_library_exports_every_symbol(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_create_rejects_bad_descriptor(lib):
    import ctypes

    d = _lib.PlanDesc()
    d.physics, d.ndim, d.order = 0, 2, 2
    d.nz, d.ny, d.nx, d.npml, d.nbound, d.nt, d.nshots, d.npw = 200, 1, 200, 41, 3, 10, 1, 1
    d.dt, d.dz, d.dx, d.dy = 1e-3, 5.0, 5.0, 1.0
    plan = ctypes.c_void_p()
    d.order = 3
    rc = lib.gpi_plan_create(ctypes.byref(d), ctypes.byref(plan))
    assert rc == -1  # orders 2, 4, 6, 8 only
    assert b"order" in lib.gpi_last_error(None)
    d.order, d.npw = 2, 2
    rc = lib.gpi_plan_create(ctypes.byref(d), ctypes.byref(plan))
    assert rc == -4  # orders other than 4: forward runs only
    assert b"order" in lib.gpi_last_error(None)
    d.order, d.npw = 4, 1
    d.pml_faces = 0x3F  # CPML on every face
    d.nz = 60  # too small for two PML strips
    assert lib.gpi_plan_create(ctypes.byref(d), ctypes.byref(plan)) == -1


def test_create_rejects_bad_checkpoint_requests(lib):
    """A checkpointed adjoint needs npw = 2 and an acoustic medium (checked
    before any device call)."""
    import ctypes

    d = _lib.PlanDesc()
    d.physics, d.ndim, d.order = 0, 2, 4
    d.nz, d.ny, d.nx, d.npml, d.nbound, d.nt, d.nshots, d.npw = 200, 1, 200, 41, 3, 10, 1, 1
    d.dt, d.dz, d.dx, d.dy = 1e-3, 5.0, 5.0, 1.0
    d.pml_faces = 0x3F
    plan = ctypes.c_void_p()
    d.checkpoints = 4  # npw = 1: no adjoint to checkpoint
    assert lib.gpi_plan_create(ctypes.byref(d), ctypes.byref(plan)) == -1
    assert b"checkpoints" in lib.gpi_last_error(None)
    d.npw, d.physics = 2, 1  # elastic: no gradient
    assert lib.gpi_plan_create(ctypes.byref(d), ctypes.byref(plan)) == -4
    assert b"acoustic" in lib.gpi_last_error(None)
    d.checkpoints = -1
    assert lib.gpi_plan_create(ctypes.byref(d), ctypes.byref(plan)) == -1


def test_entry_points_reject_a_null_plan(lib):
    """Every plan entry point answers GPI_E_INVALID for a null plan, before
    touching a device."""
    import ctypes

    null = ctypes.c_void_p()
    assert lib.gpi_set_illum(null, 1) == -1
    assert lib.gpi_get_illum(null, None, 0) == -1
    assert lib.gpi_run(null, 0) == -1
    assert lib.gpi_set_graph(null, 1) == -1
    assert lib.gpi_set_snapshots(null, 0, 0, None) == -1
    out = ctypes.c_size_t()
    assert lib.gpi_plan_bytes(null, ctypes.byref(out)) == -1


def test_estimate_at_every_order(lib):
    """gpi_plan_estimate takes every order of the reference; stencil orders
    other than 4 need more than 65535 shots to be refused for their grid."""
    import ctypes

    d = _lib.PlanDesc()
    d.physics, d.ndim = 1, 3
    d.nz, d.ny, d.nx, d.nbound, d.nt, d.nshots, d.npw = 80, 80, 80, 3, 10, 1, 1
    d.dt, d.dz, d.dx, d.dy = 1e-3, 10.0, 10.0, 10.0
    d.pml_faces = 0x3F
    sizes = []
    for order in (2, 4, 6, 8):
        d.order, d.npml = order, 10 + order - 1
        b = ctypes.c_size_t()
        assert lib.gpi_plan_estimate(ctypes.byref(d), ctypes.byref(b)) == 0, lib.gpi_last_error(None)
        sizes.append(b.value)
    assert all(s > 0 for s in sizes)
    d.order, d.nshots = 2, 70000
    assert lib.gpi_plan_estimate(ctypes.byref(d), ctypes.byref(ctypes.c_size_t())) == -4
