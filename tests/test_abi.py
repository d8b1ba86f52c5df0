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
