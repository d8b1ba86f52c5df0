"""The finite-difference-consistent imaging condition (plans created with
ref_compat_grad=False, gpi_plan_desc.imaging = 1; no counterpart in the
reference).

The reference's rho term (src/fdtd/gradient.jl:31-56) averages the velocity
correlations four and five cells away from the velocity cells whose update
coefficients hold rho(r, c); the gradient of the discrete model takes them
at vx (r, c+2), (r, c+3) and vz (r+2, c), (r+3, c) instead (dt / avg(rho)
at vx cell c averages rho at c-3 and c-2, src/fdtd/medium.jl:191-221).

  * parity: the engine's raw accumulations against the CPU oracle in the
    same mode (gpo_set_imaging), 2-D time reversal and checkpointed, 3-D
    checkpointed, relative L2 < 1e-5;
  * finite differences: the FWI gradient of the 2-D acoustic workload's
    shape with respect to log(invK) and log(rho) on 20 random cells (seed
    2), against central differences (h = 1e-3) of the misfit computed by
    the FP64 oracle.
"""
import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, Recs, configs, get_modelvector, gradient
from oracle import oracle as O
from oracle import setup_ref as S

TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0)


def _engine(wl, dobs_arr, slots):
    pa = wl.expt(mode="forward_save", checkpoints=slots, ref_compat_grad=False)
    dobs = [Recs(len(s[1]), pa.tgrid, list(wl.rfields), {f: np.asarray(dobs_arr[f][i], np.float32) for f in wl.rfields})
            for i, s in enumerate(wl.shots)]
    m = get_modelvector(pa, ["invK", "rho"])
    g = np.zeros_like(m)
    loss = gradient(g, m, L2DistLoss(), dobs, pa)
    return loss, pa.gradients, g, pa


def _zero(wl):
    return {f: np.zeros((len(wl.shots), wl.nt, len(wl.shots[0][1])), np.float32) for f in wl.rfields}


@pytest.mark.gpu
@pytest.mark.parametrize("slots", [0, 5])
def test_consistent_imaging_2d_matches_oracle(engine, slots):
    wl = configs.acoustic2d_fwi(nz=60, nx=110, nt=500, nshots=2, nrec=37, anomaly=False)
    dobs = _zero(wl)
    _, _, _, raw_o = O.gradient(wl.as_dict(), dobs, imaging=1, history=slots > 0)
    _, raw, _, _ = _engine(wl, dobs, slots)
    for k in ("invK", "rho"):
        e = rel(raw[k], raw_o[k])
        assert e < TOL, (k, e)
    # the two rho terms differ (the reference's is offset by five cells)
    _, _, _, raw_ref = O.gradient(wl.as_dict(), dobs, history=slots > 0)
    assert rel(raw["rho"], raw_ref["rho"]) > 0.1


@pytest.mark.gpu
def test_consistent_imaging_3d_matches_oracle(engine):
    wl = configs.acoustic3d(nz=20, ny=18, nx=22, nt=120, npml=10, nrec_side=4, rfields=("vz",), src_field="p")
    dobs = _zero(wl)
    _, _, _, raw_o = O.gradient(wl.as_dict(), dobs, imaging=1, history=True)
    _, raw, _, _ = _engine(wl, dobs, 4)
    for k in ("invK", "rho"):
        e = rel(raw[k], raw_o[k])
        assert e < TOL, (k, e)


@pytest.mark.gpu
def test_gradient_matches_finite_differences_on_20_random_cells(engine):
    """dJ/dlog(invK) and dJ/dlog(rho) of the engine (checkpointed plan,
    consistent imaging) on 20 random inner cells against central
    differences of the FP64 oracle's misfit (h = 1e-3, relative).  Cells
    the wavefield has not reached (|g| below 2e-5 of the largest) only need
    to stay below that level."""
    nz, nx, nt = 50, 90, 400
    true = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=2, nrec=31, anomaly=True, radius=60.0)
    wl = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=2, nrec=31, anomaly=False)
    dobs = O.forward(true.as_dict(), dtype=np.float64)
    _, _, g, pa = _engine(wl, dobs, 5)
    n = nz * nx
    gk = g[:n].reshape(nz, nx, order="F")
    gr = g[n:].reshape(nz, nx, order="F")
    ex = wl.as_dict()

    prep = O.Prepared(ex)
    npml = prep.npml

    def J(name, z, x, f):
        # the inner cell's parameter scaled, the PML cells as padded (what
        # update!(pa, m, mparams) does)
        mod = [m.astype(np.float64) for m in prep.mod]
        mod[0 if name == "invK" else 1][npml + z, npml + x] *= f
        r = O.forward(ex, dtype=np.float64, mod=mod)
        return sum(S.l2_value(dobs[k], r[k]) for k in ex["rfields"])

    rng = np.random.default_rng(2)
    cells = [(int(rng.integers(0, nz)), int(rng.integers(0, nx))) for _ in range(20)]
    h = 1e-3
    for name, gg in (("invK", gk), ("rho", gr)):
        floor = 2e-5 * np.abs(gg).max()
        for z, x in cells:
            vals = [J(name, z, x, np.exp(sg * h)) for sg in (1, -1)]
            fd = (vals[0] - vals[1]) / (2 * h)
            adj = float(gg[z, x])
            print("FD %-4s cell (%2d, %2d): fd %.5e adjoint %.5e" % (name, z, x, fd, adj))
            assert abs(adj - fd) <= 5e-3 * abs(fd) + floor, (name, (z, x), fd, adj)
