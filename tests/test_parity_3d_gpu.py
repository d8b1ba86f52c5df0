"""3-D acoustic and elastic steps of the CUDA engine against the CPU oracle,
through the C ABI (Python host mirror), on reduced versions of the 3-D
workloads (a 10-cell CPML instead of 23 keeps the oracle quick).

Tolerance: relative L2 error 1e-5 in FP32, as for the 2-D kernels."""
import numpy as np
import pytest

from geophyinv_gb300 import configs, update
from oracle import oracle as O

TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0)


def _check(wl, fields):
    ref, orc = O.forward(wl.as_dict(), return_oracle=True)
    pa = wl.expt()
    update(pa)
    for iss in range(len(wl.shots)):
        for f in wl.rfields:
            e = rel(pa.data[0][iss].d[f], ref[f][iss])
            assert e < TOL, (f, iss, e)
    for f in fields:
        e = rel(pa.field(f, iss=len(wl.shots) - 1), orc.field(f))
        assert e < TOL, (f, e)
    orc.close()


@pytest.mark.gpu
def test_acoustic3d_matches_oracle(engine):
    wl = configs.acoustic3d(nz=24, ny=20, nx=28, nt=150, npml=10, nrec_side=5)
    _check(wl, ("p", "vx", "vy", "vz"))


@pytest.mark.gpu
@pytest.mark.parametrize("surface", ["pml", "free"])
def test_elastic3d_matches_oracle(engine, surface):
    wl = configs.elastic3d(nz=24, ny=20, nx=28, nt=150, npml=10, nrec_side=5, rfields=("vx", "vy", "vz"))
    if surface == "free":
        wl.pml_faces = ["zmax", "ymin", "ymax", "xmin", "xmax"]
        wl.stressfree_faces = ["zmin"]
    _check(wl, ("tauxx", "tauyy", "tauzz", "tauxy", "tauxz", "tauyz", "vx", "vy", "vz"))


@pytest.mark.gpu
def test_elastic3d_velocity_source_two_shots(engine):
    """A vy body-force source, two supersources batched in one launch."""
    wl = configs.elastic3d(nz=20, ny=22, nx=24, nt=120, npml=10, nrec_side=4, rfields=("vy", "vz"),
                           src_field="vy")
    src, rec = wl.shots[0]
    wl.shots = [(src, rec), (src + np.array([[0.0, -40.0, 30.0]]), rec)]
    _check(wl, ("vx", "vy", "vz", "tauxx"))


@pytest.mark.gpu
@pytest.mark.parametrize("surface", ["pml", "free"])
def test_elastic3d_mid_size_two_shots(engine, surface):
    """A mid-size grid (100 x 76 x 116 extended: several 32 x 8 tiles and
    columns beyond the CPML reach on every axis), two shots in one launch,
    every field at the end."""
    wl = configs.elastic3d(nz=80, ny=56, nx=96, nt=100, npml=10, nrec_side=5, rfields=("vx", "vy", "vz"))
    src, rec = wl.shots[0]
    wl.shots = [(src, rec), (src + np.array([[60.0, -50.0, 40.0]]), rec)]
    if surface == "free":
        wl.pml_faces = ["zmax", "ymin", "ymax", "xmin", "xmax"]
        wl.stressfree_faces = ["zmin"]
    _check(wl, ("tauxx", "tauyy", "tauzz", "tauxy", "tauxz", "tauyz", "vx", "vy", "vz"))


@pytest.mark.gpu
def test_elastic3d_velocity_source_mid_size(engine):
    """A vz body-force source on the mid-size grid."""
    wl = configs.elastic3d(nz=80, ny=56, nx=96, nt=100, npml=10, nrec_side=5, rfields=("vz",), src_field="vz")
    _check(wl, ("vx", "vy", "vz", "tauzz"))
