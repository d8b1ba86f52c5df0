"""Error of every kind of result of the FP32 CUDA engine against an FP64 run
of the oracle (the reference's algorithm in double precision), on reduced
versions of the workloads.  Each case prints one line

    FP64 <case> <quantity> <relative L2 error>

(run with -s to see them) and checks it against a bound well above the
measured values: the engine computes in FP32, so these are FP32 rounding
levels accumulated over the time loop, not parity bounds (parity with the
FP32 oracle is 1e-5 elsewhere)."""
import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, Recs, configs, get_modelvector, gradient, update
from oracle import oracle as O

BOUND = 1e-4


def rel(a, b):
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0))


def _report(case, what, e):
    print("FP64 %-28s %-12s %.3e" % (case, what, e))
    assert e < BOUND, (case, what, e)


def _forward(case, wl):
    ref = O.forward(wl.as_dict(), dtype=np.float64)
    pa = wl.expt()
    update(pa)
    for f in wl.rfields:
        got = np.stack([pa.data[0][i].d[f] for i in range(len(wl.shots))])
        _report(case, "rec " + f, rel(got, ref[f]))


@pytest.mark.gpu
def test_fp64_error_forward_records(engine):
    _forward("acoustic2d 201x301 2000st", configs.acoustic2d_layers())
    _forward("elastic2d 110x190 3 shots", configs.elastic2d_batch(nz=110, nx=190, nt=400, nshots=3, nrec=31))
    _forward("acoustic3d 24x20x28", configs.acoustic3d(nz=24, ny=20, nx=28, nt=150, npml=10, nrec_side=5,
                                                      rfields=("p", "vz")))
    _forward("elastic3d 24x20x28", configs.elastic3d(nz=24, ny=20, nx=28, nt=150, npml=10, nrec_side=5,
                                                    rfields=("vx", "vy", "vz")))


def _grad(case, wl, checkpoints):
    nr = len(wl.shots[0][1])
    dobs_arr = {f: np.zeros((len(wl.shots), wl.nt, nr), np.float32) for f in wl.rfields}
    # the reference's gradient is time reversal; the checkpointed one is the
    # same imaging condition over the forward history
    _, _, _, raw = O.gradient(wl.as_dict(), dobs_arr, dtype=np.float64, history=checkpoints > 0)
    pa = wl.expt(mode="forward_save", checkpoints=checkpoints)
    dobs = [Recs(nr, pa.tgrid, list(wl.rfields), {f: dobs_arr[f][i] for f in wl.rfields})
            for i in range(len(wl.shots))]
    m = get_modelvector(pa, ["invK", "rho"])
    gradient(np.zeros_like(m), m, L2DistLoss(), dobs, pa)
    for k in ("invK", "rho"):
        _report(case, "grad " + k, rel(pa.gradients[k], raw[k]))


@pytest.mark.gpu
def test_fp64_error_gradients(engine):
    _grad("acoustic2d grad 90x160 2 shots", configs.acoustic2d_fwi(nz=90, nx=160, nt=600, nshots=2, nrec=53,
                                                                   anomaly=False), 0)
    _grad("acoustic2d ckpt 90x160 2 shots", configs.acoustic2d_fwi(nz=90, nx=160, nt=600, nshots=2, nrec=53,
                                                                   anomaly=False), 7)
    _grad("acoustic3d ckpt 20x18x22", configs.acoustic3d(nz=20, ny=18, nx=22, nt=100, npml=10, nrec_side=4,
                                                         rfields=("vz",), src_field="p"), 3)
