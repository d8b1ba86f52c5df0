"""CUDA engine against the CPU oracle, through the C ABI (Python host mirror).

Tolerance: relative L2 error 1e-5 in FP32 (the bound of the target);
the kernels keep the reference's operation order without FMA contraction,
so the observed error is at rounding level."""
import numpy as np
import pytest

from geophyinv_gb300 import configs, update
from oracle import oracle as O

TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0)


def _compare_records(pa, ref, wl):
    for iss in range(len(wl.shots)):
        for f in wl.rfields:
            e = rel(pa.data[0][iss].d[f], ref[f][iss])
            assert e < TOL, (f, iss, e)


@pytest.mark.gpu
def test_acoustic2d_small_matches_oracle(engine):
    wl = configs.acoustic2d_layers(nz=101, nx=131, nt=500, nrec=41)
    ref, orc = O.forward(wl.as_dict(), return_oracle=True)
    pa = wl.expt()
    update(pa)
    _compare_records(pa, ref, wl)
    # final state, including the extra velocity half step after the loop
    for f in ("p", "vx", "vz"):
        e = rel(pa.field(f), orc.field(f))
        assert e < TOL, (f, e)
    orc.close()


@pytest.mark.gpu
def test_acoustic2d_full_config_matches_oracle(engine):
    """201 x 301 at 5 m, 2000 steps, 101 receivers, p/vx/vz records."""
    wl = configs.acoustic2d_layers()
    ref = O.forward(wl.as_dict())
    pa = wl.expt()
    update(pa)
    _compare_records(pa, ref, wl)


@pytest.mark.gpu
@pytest.mark.parametrize("surface", ["pml", "free"])
def test_elastic2d_batch_matches_oracle(engine, surface):
    """Reduced 2-D elastic batch: 3 surface shots, explosive tauxx source,
    vx/vz records; with a PML top or a stress-free top (free_surface!)."""
    wl = configs.elastic2d_batch(nz=110, nx=190, nt=400, nshots=3, nrec=31)
    if surface == "free":
        wl.pml_faces = ["zmax", "xmin", "xmax"]
        wl.stressfree_faces = ["zmin"]
    ref, orc = O.forward(wl.as_dict(), return_oracle=True)
    pa = wl.expt()
    update(pa)
    _compare_records(pa, ref, wl)
    for f in ("tauxx", "tauzz", "tauxz", "vx", "vz"):
        e = rel(pa.field(f, iss=2), orc.field(f))
        assert e < TOL, (f, e)
    orc.close()


@pytest.mark.gpu
def test_elastic2d_interior_tiles(engine):
    """A grid large enough for tiles away from every strip and face, which
    take the kernel's straight-line interior path."""
    wl = configs.elastic2d_batch(nz=300, nx=420, nt=300, nshots=2, nrec=41)
    ref, orc = O.forward(wl.as_dict(), return_oracle=True)
    pa = wl.expt()
    update(pa)
    _compare_records(pa, ref, wl)
    for f in ("tauxx", "tauzz", "tauxz", "vx", "vz"):
        e = rel(pa.field(f, iss=1), orc.field(f))
        assert e < TOL, (f, e)
    orc.close()


@pytest.mark.gpu
def test_elastic2d_velocity_source(engine):
    wl = configs.elastic2d_batch(nz=100, nx=140, nt=300, nshots=2, nrec=19, src_field="vz")
    ref = O.forward(wl.as_dict())
    pa = wl.expt()
    update(pa)
    _compare_records(pa, ref, wl)


@pytest.mark.gpu
def test_acoustic2d_multishot_velocity_sources(engine):
    """Several supersources batched in one launch, vz sources, no PML on top
    (rigid faces = pml faces only), records of every shot."""
    wl = configs.acoustic2d_layers(nz=90, nx=120, nt=300, nrec=17, src_field="vz")
    rec = wl.shots[0][1]
    wl.shots = [(np.array([[30.0, x]]), rec) for x in (100.0, 300.0, 500.0)]
    wl.pml_faces = ["zmax", "xmin", "xmax"]
    ref = O.forward(wl.as_dict())
    pa = wl.expt()
    update(pa)
    _compare_records(pa, ref, wl)


@pytest.mark.gpu
@pytest.mark.parametrize("nz,nze", [(69, 112), (133, 176)])
def test_bottom_ghost_rows_at_warp_edges(engine, nz, nze):
    """Depths whose padded grids have 155 and 219 rows (PML on both z faces,
    or a free surface on top): with blocks of 124 rows the bottom ghost rows
    of vz (dirichletzmax!) fall on lanes 0 and 1 of a warp, away from the
    lanes of their mirror source rows."""
    wl = configs.acoustic2d_layers(nz=nz, nx=120, nt=300, nrec=17)
    ref, orc = O.forward(wl.as_dict(), return_oracle=True)
    pa = wl.expt()
    update(pa)
    _compare_records(pa, ref, wl)
    for f in ("p", "vx", "vz"):
        e = rel(pa.field(f), orc.field(f))
        assert e < TOL, (f, e)
    orc.close()
    wl = configs.elastic2d_batch(nz=nze, nx=130, nt=300, nshots=2, nrec=15)
    wl.pml_faces = ["zmax", "xmin", "xmax"]
    wl.stressfree_faces = ["zmin"]
    ref, orc = O.forward(wl.as_dict(), return_oracle=True)
    pa = wl.expt()
    update(pa)
    _compare_records(pa, ref, wl)
    for f in ("tauxx", "tauzz", "tauxz", "vx", "vz"):
        e = rel(pa.field(f, iss=1), orc.field(f))
        assert e < TOL, (f, e)
    orc.close()
