"""Born (linearised) modelling, CPU: the oracle's restatement
(GPO_BORN: wavefield 2 driven by the secondary sources of a medium
perturbation) against the oracle's own nonlinear forward runs and its
imaging gradient.  The reference pins its Born operator with a linearity
test and an adjoint dot test (test/fwi/born_map.jl:7-51); both are
restated here, plus the derivative test the reference cannot run (its
Born kernels, src/fdtd/born.jl:1-13, pass arguments its kernels do not
take)."""
import numpy as np

from geophyinv_gb300 import configs
from oracle import oracle as O

NPML = 43


def _setup(nz, nx, nt, seed, layers=True):
    wl = (configs.acoustic2d_layers(nz=nz, nx=nx, nt=nt, nrec=21, rfields=("p", "vz")) if layers else
          configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=1, nrec=23, anomaly=False))
    ex = wl.as_dict()
    prep = O.Prepared(ex, np.float64)
    inner = (slice(NPML, NPML + nz), slice(NPML, NPML + nx))
    rng = np.random.default_rng(seed)
    dKi = 0.02 * rng.standard_normal((nz, nx)) * prep.mod[0][inner]
    dRi = 0.02 * rng.standard_normal((nz, nx)) * prep.mod[1][inner]
    return wl, ex, prep, inner, dKi, dRi


def test_born_records_are_the_derivative_of_the_forward_records():
    """Born records of (dinvK, drho) against central differences of the
    nonlinear forward records, medium +- eps (dinvK, drho) (FP64; the
    perturbation padded into the PML as padarray! pads the medium)."""
    wl, ex, prep, inner, dKi, dRi = _setup(60, 90, 400, 5)
    b = O.born(ex, np.pad(dKi, NPML, mode="edge"), np.pad(dRi, NPML, mode="edge"), dtype=np.float64)

    def fwd(e):
        rho = ex["rho"].astype(np.float64) + e * dRi
        invK = prep.mod[0][inner] + e * dKi
        ee = dict(ex)
        ee["rho"], ee["vp"] = rho, np.sqrt(1.0 / (invK * rho))
        return O.forward(ee, dtype=np.float64)

    eps = 1e-2
    fp, fm = fwd(eps), fwd(-eps)
    for f in wl.rfields:
        fd = (fp[f] - fm[f]) / (2 * eps)
        e = np.linalg.norm(fd - b[f]) / np.linalg.norm(fd)
        assert e < 1e-3, (f, e)  # measured 1.7e-4 (second-order remainder)


def test_born_is_linear():
    """F (x1 + x2) = F x1 + F x2 (born_map.jl:23-30)."""
    wl, ex, prep, inner, dKi, dRi = _setup(40, 60, 250, 6)
    rng = np.random.default_rng(8)
    z = np.zeros(prep.shape)
    x1 = (z.copy(), z.copy())
    x2 = (z.copy(), z.copy())
    x1[0][inner], x1[1][inner] = dKi, dRi
    x2[0][inner] = 0.01 * rng.standard_normal(dKi.shape) * prep.mod[0][inner]
    x2[1][inner] = 0.01 * rng.standard_normal(dRi.shape) * prep.mod[1][inner]
    b1 = O.born(ex, *x1, dtype=np.float64)
    b2 = O.born(ex, *x2, dtype=np.float64)
    b12 = O.born(ex, x1[0] + x2[0], x1[1] + x2[1], dtype=np.float64)
    for f in wl.rfields:
        e = np.linalg.norm(b12[f] - b1[f] - b2[f]) ** 2 / np.linalg.norm(b12[f]) ** 2
        assert e < 1e-25, (f, e)


def test_born_adjoint_is_the_imaging_gradient():
    """<y, F x> = <F' y, x> with F' the imaging gradient of the discrete
    model (gpo_set_imaging 1) on the exact forward history (born_map.jl:
    33-47: rtol 1e-5); F' y = -raw accumulations for adjoint sources y
    (dobs = dcal + y / 2 makes L2's adjoint source 2 (dobs - dcal) = y)."""
    wl, ex, prep, inner, dKi, dRi = _setup(40, 70, 300, 7, layers=False)
    dK = np.zeros(prep.shape)
    dR = np.zeros(prep.shape)
    dK[inner], dR[inner] = dKi, dRi
    b = O.born(ex, dK, dR, dtype=np.float64)
    rng = np.random.default_rng(9)
    y = {f: rng.standard_normal(b[f].shape) for f in b}
    dcal = O.forward(ex, dtype=np.float64)
    _, _, _, raw = O.gradient(ex, {f: dcal[f] + 0.5 * y[f] for f in y}, dtype=np.float64, imaging=1, history=True)
    a = sum(float((b[f] * y[f]).sum()) for f in b)
    c = -float((raw["invK"] * dK).sum() + (raw["rho"] * dR).sum())
    assert abs(a - c) <= 1e-5 * abs(a), (a, c)  # measured 5e-9
