"""Snapshots (tsnaps / snaps_field, snaps_save!, src/fdtd/fdtd.jl:586-591):
the oracle keeps the field at the end of the requested steps (CPU), and the
engine's snapshots match the oracle's (GPU, relative L2 < 1e-5)."""
import numpy as np
import pytest

from geophyinv_gb300 import configs, update
from oracle import oracle as O

TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0)


def test_oracle_snapshot_at_the_last_step_is_the_final_pressure():
    wl = configs.acoustic2d_layers(nz=41, nx=51, nt=80, nrec=11)
    res, orc = O.forward(wl.as_dict(), return_oracle=True, snaps=("p", [40, 80]))
    # p is not touched by the extra velocity half step after the loop
    assert np.array_equal(res["snaps"][0][1], orc.field("p"))
    assert not np.array_equal(res["snaps"][0][0], res["snaps"][0][1])
    orc.close()


def _check(wl, field, ts):
    tg = wl.tgrid.values()
    its = [int(np.argmin(np.abs(tg - t))) + 1 for t in ts]
    res = O.forward(wl.as_dict(), snaps=(field, its))
    pa = wl.expt(tsnaps=ts, snaps_field=field)
    assert pa.itsnaps == its
    update(pa)
    for iss in range(len(wl.shots)):
        got = pa["snaps", iss]
        for k in range(len(its)):
            e = rel(got[k], res["snaps"][iss][k])
            assert e < TOL, (field, iss, k, e)


@pytest.mark.gpu
def test_acoustic2d_snapshots_match_oracle(engine):
    wl = configs.acoustic2d_layers(nz=101, nx=131, nt=300, nrec=21)
    t = wl.tgrid.values()
    _check(wl, "p", [t[99], t[250]])


@pytest.mark.gpu
def test_elastic2d_snapshots_match_oracle_two_shots(engine):
    wl = configs.elastic2d_batch(nz=110, nx=190, nt=200, nshots=2, nrec=31)
    t = wl.tgrid.values()
    _check(wl, "tauxx", [t[150]])
    _check(wl, "vz", [t[80], t[199]])


@pytest.mark.gpu
def test_acoustic3d_snapshots_match_oracle(engine):
    wl = configs.acoustic3d(nz=20, ny=18, nx=22, nt=80, npml=10, nrec_side=4, rfields=("vz",))
    t = wl.tgrid.values()
    _check(wl, "vx", [t[60]])
