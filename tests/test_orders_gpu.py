"""Stencil orders 2, 6 and 8 (the reference's set_preferences(order=...),
src/GeoPhyInv.jl:69-100, src/fdtd/diff2D.jl / diff3D.jl): the engine's
generic path against the CPU oracle at the same order -- records and the
final state after the extra velocity half step, 2-D and 3-D, acoustic and
elastic, PML and free-surface faces.  Tolerance: relative L2 1e-5 (FP32)."""
import numpy as np
import pytest

from geophyinv_gb300 import configs, update
from oracle import oracle as O

TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0)


def _run(wl, order, fields):
    d = wl.as_dict()
    d["order"] = order
    ref, orc = O.forward(d, return_oracle=True)
    pa = wl.expt(order=order)
    update(pa)
    last = len(wl.shots) - 1
    for iss in range(len(wl.shots)):
        for f in wl.rfields:
            assert np.linalg.norm(ref[f][iss]) > 0, (f, iss)
            e = rel(pa.data[0][iss].d[f], ref[f][iss])
            assert e < TOL, (order, f, iss, e)
    for f in fields:
        e = rel(pa.field(f, iss=last), orc.field(f))
        assert e < TOL, (order, f, e)
    orc.close()
    pa.close()


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 6, 8])
def test_acoustic2d_orders_match_oracle(engine, order):
    wl = configs.acoustic2d_layers(nz=81, nx=111, nt=300, nrec=31)
    _run(wl, order, ("p", "vx", "vz"))


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 6, 8])
@pytest.mark.parametrize("surface", ["pml", "free"])
def test_elastic2d_orders_match_oracle(engine, order, surface):
    wl = configs.elastic2d_batch(nz=90, nx=140, nt=250, nshots=2, nrec=21)
    if surface == "free":
        wl.pml_faces = ["zmax", "xmin", "xmax"]
        wl.stressfree_faces = ["zmin"]
        # without a top CPML pad the first rows are outside every velocity
        # update at order 8 (h = 7): receivers below them
        wl.shots = [(src, rec + [50.0, 0.0]) for src, rec in wl.shots]
    _run(wl, order, ("tauxx", "tauzz", "tauxz", "vx", "vz"))


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 8])
def test_acoustic3d_orders_match_oracle(engine, order):
    wl = configs.acoustic3d(nz=24, ny=20, nx=26, nt=200, dt=0.0005, npml=14, nrec_side=4, rfields=("p", "vz"))
    _run(wl, order, ("p", "vx", "vy", "vz"))


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 6])
def test_elastic3d_orders_match_oracle(engine, order):
    wl = configs.elastic3d(nz=24, ny=20, nx=26, nt=200, dt=0.0005, npml=14, nrec_side=4, rfields=("vx", "vz"))
    _run(wl, order, ("tauxx", "tauyy", "tauzz", "tauxy", "tauxz", "tauyz", "vx", "vy", "vz"))


@pytest.mark.gpu
@pytest.mark.parametrize("gkind", [1, 2])
def test_generic_order_graph_replays_equal_plain_runs(engine, gkind):
    wl = configs.elastic2d_batch(nz=80, nx=120, nt=100, nshots=2, nrec=15)
    plain = wl.expt(order=6)
    update(plain)
    pa = wl.expt(order=6)
    pa.set_graph(gkind)
    for _ in range(2):  # capture, then replay
        update(pa)
        for i in range(len(wl.shots)):
            for f in wl.rfields:
                assert np.array_equal(pa.data[0][i].d[f], plain.data[0][i].d[f]), (i, f)
    assert np.array_equal(pa.field("tauxz", iss=1), plain.field("tauxz", iss=1))
