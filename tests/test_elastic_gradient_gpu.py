"""3-D elastic FWI gradient through the checkpointed adjoint (no
counterpart in the reference, which defines gradients for 2-D acoustic
media only, src/fdtd/gradient.jl:17-64; the imaging condition is the
engine's own: the gradient of the discrete scheme with respect to
invlambda, invmu and rho, see k_grad_e3 and the oracle's GPO_ADJOINT_HIST).

  * parity: raw accumulations against the CPU oracle's history mode,
    relative L2 < 1e-5 (explosive and velocity sources);
  * finite differences: dJ/dlog(m) on 20 random cells (seed 2) for each
    parameter against central differences (h = 1e-3) of the FP64 oracle's
    misfit;
  * directional derivative: <g, dm> for a random smooth dm of all three
    parameters against the central difference of the misfit along dm.
"""
import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, Recs, configs, get_modelvector, gradient
from oracle import oracle as O
from oracle import setup_ref as S

TOL = 1e-5
PARAMS = ["invlambda", "invmu", "rho"]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0)


def _workload(src_field="tauxx", nt=160):
    wl = configs.elastic3d(nz=16, ny=14, nx=18, nt=nt, npml=10, nrec_side=4, rfields=("vx", "vz"),
                           src_field=src_field)
    s, r = wl.shots[0]
    r = r.copy()
    r[:, 0] = 40.0  # receivers 4 cells below the surface
    wl.shots = [(s, r)]
    return wl


def _engine(wl, dobs_arr, slots=4):
    pa = wl.expt(mode="forward_save", checkpoints=slots)
    dobs = [Recs(len(s[1]), pa.tgrid, list(wl.rfields), {f: np.asarray(dobs_arr[f][i], np.float32) for f in wl.rfields})
            for i, s in enumerate(wl.shots)]
    m = get_modelvector(pa, PARAMS)
    g = np.zeros_like(m)
    J = gradient(g, m, L2DistLoss(), dobs, pa, PARAMS)
    return J, pa.gradients, g, pa


@pytest.mark.gpu
@pytest.mark.parametrize("src_field", ["tauxx", "vz"])
def test_elastic3d_gradient_matches_oracle(engine, src_field):
    wl = _workload(src_field)
    dobs = {f: np.zeros((1, wl.nt, len(wl.shots[0][1])), np.float32) for f in wl.rfields}
    loss_o, _, _, raw_o = O.gradient(wl.as_dict(), dobs, history=True)
    J, raw, g, _ = _engine(wl, dobs)
    assert abs(J - loss_o) <= TOL * abs(loss_o)
    for k in PARAMS:
        assert np.linalg.norm(raw_o[k]) > 0, k
        e = rel(raw[k], raw_o[k])
        assert e < TOL, (k, e)
    assert np.all(np.isfinite(g))


@pytest.mark.gpu
def test_elastic3d_gradient_mid_size_matches_oracle(engine):
    """The same parity on a mid-size grid (100 x 68 x 76 extended), five
    checkpoint slots."""
    wl = configs.elastic3d(nz=80, ny=48, nx=56, nt=60, npml=10, nrec_side=5, rfields=("vx", "vz"))
    dobs = {f: np.zeros((1, wl.nt, len(wl.shots[0][1])), np.float32) for f in wl.rfields}
    loss_o, _, _, raw_o = O.gradient(wl.as_dict(), dobs, history=True)
    J, raw, g, _ = _engine(wl, dobs, slots=5)
    assert abs(J - loss_o) <= TOL * abs(loss_o)
    for k in PARAMS:
        assert np.linalg.norm(raw_o[k]) > 0, k
        e = rel(raw[k], raw_o[k])
        assert e < TOL, (k, e)


def _fd_setup():
    wl = _workload("tauxx")
    ex = wl.as_dict()
    true = dict(ex)
    vp = ex["vp"].copy()
    vp[5:9, 4:8, 6:10] *= 1.05
    true["vp"] = vp
    dobs = O.forward(true, dtype=np.float64)
    return wl, ex, dobs


def _J(ex, dobs, scale):
    """FP64 misfit with the medium parameters of the inner (non-PML) cells
    scaled by `scale` (name -> factor array on the physical grid), the PML
    cells left as padded: the model vector's meaning (update!(pa, m,
    mparams) changes the inner cells only)."""
    prep = O.Prepared(ex)
    npml = prep.npml
    inner = tuple(slice(npml, n - npml) for n in prep.shape)
    mod = [m.astype(np.float64) for m in prep.mod]
    for i, k in enumerate(PARAMS):
        if k in scale:
            mod[i][inner] = mod[i][inner] * scale[k]
    r = O.forward(ex, dtype=np.float64, mod=mod)
    return sum(S.l2_value(dobs[f], r[f]) for f in ex["rfields"])


@pytest.mark.gpu
def test_elastic3d_gradient_matches_finite_differences_on_20_random_cells(engine):
    wl, ex, dobs = _fd_setup()
    _, _, g, pa = _engine(wl, dobs)
    shape = tuple(len(x) for x in wl.grid)
    n = int(np.prod(shape))
    rng = np.random.default_rng(2)
    cells = [tuple(int(rng.integers(0, s)) for s in shape) for _ in range(20)]
    h = 1e-3
    for ip, name in enumerate(PARAMS):
        gg = g[ip * n:(ip + 1) * n].reshape(shape, order="F")
        floor = 2e-5 * np.abs(gg).max()
        for cell in cells:
            vals = []
            for sg in (1, -1):
                f = np.ones(shape)
                f[cell] = np.exp(sg * h)
                vals.append(_J(ex, dobs, {name: f}))
            fd = (vals[0] - vals[1]) / (2 * h)
            adj = float(gg[cell])
            print("FD %-9s cell %s: fd %.5e adjoint %.5e" % (name, cell, fd, adj))
            assert abs(adj - fd) <= 5e-3 * abs(fd) + floor, (name, cell, fd, adj)


@pytest.mark.gpu
def test_elastic3d_gradient_directional_derivative(engine):
    wl, ex, dobs = _fd_setup()
    _, _, g, _ = _engine(wl, dobs)
    shape = tuple(len(x) for x in wl.grid)
    from geophyinv_gb300.configs import smooth_noise

    dm = {k: smooth_noise(shape, 2.0, 20 + i) for i, k in enumerate(PARAMS)}
    h = 1e-3
    Jp = _J(ex, dobs, {k: np.exp(h * v) for k, v in dm.items()})
    Jm = _J(ex, dobs, {k: np.exp(-h * v) for k, v in dm.items()})
    fd = (Jp - Jm) / (2 * h)
    adj = float(g.astype(np.float64) @ np.concatenate([dm[k].ravel(order="F") for k in PARAMS]))
    print("directional: fd %.8e adjoint %.8e" % (fd, adj))
    assert abs(adj - fd) <= 1e-3 * abs(fd), (fd, adj)
