"""Finite-difference check of the GPU FWI gradient (the reference's
gradient-accuracy test, test/fwi/gradient_accuracy.jl, restated on the
current API: central differences of lossvalue against gradient! on blocks
of the inner grid).

The invK part agrees to ~1e-3 or better.  The rho part is the reference's
imaging condition (src/fdtd/gradient.jl:31-56: g -= av(v_adj_prev (v - v_prev)
dtI), averaged one cell off and without a 1/rho factor); it is reproduced
exactly (tests/test_gradient_gpu.py) but is not the derivative of the
discrete misfit, so only its finiteness is checked here."""
import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, Recs, configs, get_modelvector, gradient, lossvalue


@pytest.mark.gpu
def test_invK_gradient_matches_finite_differences(engine):
    nz, nx, nt, nrec = 60, 100, 500, 33
    wl = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=1, nrec=nrec, anomaly=False)
    pa = wl.expt(mode="forward_save")
    dobs = [Recs(nrec, pa.tgrid, ["vz"], {"vz": np.zeros((nt, nrec), np.float32)})]
    m0 = get_modelvector(pa, ["invK", "rho"])
    g = np.zeros_like(m0)
    gradient(g, m0, L2DistLoss(), dobs, pa)
    assert np.all(np.isfinite(g))
    h = 1e-2
    for z0, x0 in ((20, 60), (35, 45), (10, 40)):
        e = np.zeros_like(m0)
        blk = np.zeros((nz, nx), np.float32)
        blk[z0:z0 + 8, x0:x0 + 8] = 1
        e[:nz * nx] = blk.ravel(order="F")
        fd = (lossvalue(m0 + h * e, L2DistLoss(), dobs, pa) - lossvalue(m0 - h * e, L2DistLoss(), dobs, pa)) / (2 * h)
        adj = float(g @ e)
        assert abs(fd - adj) <= 1e-2 * abs(adj), (z0, x0, fd, adj)
