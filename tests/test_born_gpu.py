"""Born modelling on the GPU (gpi_set_born + gpi_run(GPI_BORN), through
update(pa, medium, medium_pert) and BornMap, the LinearMap(pa) of the
reference, src/fdtd/func_grad.jl:53-120):

  * the engine's Born records against the oracle's (GPO_BORN), relative
    L2 < 1e-5;
  * linearity, F (x1 + x2) = F x1 + F x2 (test/fwi/born_map.jl:23-30; in
    FP32 to rounding level);
  * the adjoint dot test <y, F x> = <F' y, x> with F' the checkpointed,
    finite-difference-consistent imaging gradient (born_map.jl:33-47,
    rtol 1e-5 there; FP32 here) and <x, F' F x> > 0.
"""
import numpy as np
import pytest

from geophyinv_gb300 import AcousticMedium, BornMap, FdtdAcousticBorn, SeisForwExpt, configs, update
from oracle import oracle as O

NPML = 43


def _expt(wl, checkpoints=0):
    return SeisForwExpt(FdtdAcousticBorn(), medium=wl.medium(), ageom=wl.ageom(), srcwav=wl.srcwav(), tgrid=wl.tgrid,
                        rfields=wl.rfields, pml_faces=wl.pml_faces, checkpoints=checkpoints, ref_compat_grad=False)


@pytest.mark.gpu
def test_born_records_match_oracle(engine):
    wl = configs.acoustic2d_layers(nz=80, nx=120, nt=500, nrec=31, rfields=("p", "vx", "vz"))
    rng = np.random.default_rng(11)
    m = wl.medium()
    pert = AcousticMedium(m.grid, m.vp * (1 + 0.03 * rng.standard_normal(m.vp.shape)).astype(np.float32),
                          m.rho * (1 + 0.03 * rng.standard_normal(m.rho.shape)).astype(np.float32))
    pa = _expt(wl)
    update(pa, m, pert)
    update(pa)
    prep = O.Prepared(wl.as_dict())
    vp = np.pad(pert.vp, NPML, mode="edge")
    rho = np.pad(pert.rho, NPML, mode="edge")
    dK = (np.float32(1) / ((vp * vp) * rho)).astype(np.float32) - prep.mod[0]
    dR = rho - prep.mod[1]
    ref = O.born(wl.as_dict(), dK, dR)
    for f in wl.rfields:
        got = pa.data[1][0].d[f]
        e = np.linalg.norm(got - ref[f][0]) / np.linalg.norm(ref[f][0])
        assert np.linalg.norm(ref[f][0]) > 0 and e < 1e-5, (f, e)


@pytest.mark.gpu
def test_born_map_is_linear_and_its_transpose_is_the_imaging_gradient(engine):
    nz, nx = 40, 70
    wl = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=300, nshots=2, nrec=23, anomaly=False)
    pa = _expt(wl, checkpoints=4)
    F = BornMap(pa)
    shape = [len(g) for g in pa.exgrid]
    rng = np.random.default_rng(12)

    def rand_x():
        x = np.zeros([2] + shape, np.float32)
        for k, name in enumerate(("invK", "rho")):
            x[k, NPML:NPML + nz, NPML:NPML + nx] = 0.01 * rng.standard_normal((nz, nx)) * \
                pa.mod[name][NPML:NPML + nz, NPML:NPML + nx]
        return np.concatenate([x[0].ravel(order="F"), x[1].ravel(order="F")])

    x1, x2 = rand_x(), rand_x()
    d1, d2, d12 = F.matvec(x1), F.matvec(x2), F.matvec(x1 + x2)
    e = np.linalg.norm(d12 - d1 - d2) / np.linalg.norm(d12)
    assert e < 1e-5, e
    y = rng.standard_normal(F.nd).astype(np.float32) * np.float32(np.abs(d1).max())
    a = float(np.dot(y.astype(np.float64), d1))
    b = float(np.dot(F.rmatvec(y).astype(np.float64), x1))
    print("adjoint test: %.8e %.8e" % (a, b))
    assert abs(a - b) <= 1e-4 * abs(a), (a, b)
    c = float(np.dot(x1.astype(np.float64), F.rmatvec(d1)))
    assert c > 0
