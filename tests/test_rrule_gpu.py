"""rrule(lossvalue, ...) and the torch wrapper `misfit`: the primal is
lossvalue's number, the pullback gradient!'s (bit for bit), scaled by the
incoming cotangent; it runs once; a checkpointed 3-D plan works the same."""
import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, NoTangent, Recs, configs, get_modelvector, gradient, lossvalue, misfit, rrule


def _setup(wl, **kw):
    pa = wl.expt(mode="forward_save", **kw)
    dobs = [Recs(len(s[1]), pa.tgrid, list(wl.rfields),
                 {f: np.zeros((wl.nt, len(s[1])), np.float32) for f in wl.rfields}) for s in wl.shots]
    return pa, dobs, get_modelvector(pa, ["invK", "rho"])


@pytest.mark.gpu
@pytest.mark.parametrize("checkpoints", [0, 5])
def test_rrule_matches_lossvalue_and_gradient(engine, checkpoints):
    wl = configs.acoustic2d_fwi(nz=40, nx=64, nt=240, nshots=2, nrec=21, anomaly=False)
    pa, dobs, m = _setup(wl, checkpoints=checkpoints)
    m = m * np.float32(1.01)
    J0 = lossvalue(m, L2DistLoss(), dobs, pa)
    g0 = np.zeros_like(m)
    gradient(g0, m, L2DistLoss(), dobs, pa)
    J, pb = rrule(lossvalue, m, L2DistLoss(), dobs, pa)
    assert J == J0
    t = pb(2.5)
    assert t[0] is NoTangent and all(x is NoTangent for x in t[2:])
    np.testing.assert_allclose(t[1], np.float32(2.5) * g0, rtol=1e-6)
    with pytest.raises(RuntimeError):
        pb(1.0)
    _, pb = rrule(lossvalue, m, L2DistLoss(), dobs, pa)
    assert np.array_equal(pb(1.0)[1], g0)


@pytest.mark.gpu
def test_torch_misfit_backward_is_the_adjoint_gradient(engine):
    import torch

    wl = configs.acoustic2d_fwi(nz=40, nx=64, nt=240, nshots=1, nrec=21, anomaly=False)
    pa, dobs, m = _setup(wl, checkpoints=4)
    g0 = np.zeros_like(m)
    J0 = gradient(g0, m, L2DistLoss(), dobs, pa)
    mt = torch.from_numpy(m.copy()).requires_grad_(True)
    J = misfit(mt, L2DistLoss(), dobs, pa)
    assert float(J.detach()) == J0
    (3.0 * J).backward()
    np.testing.assert_allclose(mt.grad.numpy(), 3.0 * g0, rtol=1e-6)


@pytest.mark.gpu
def test_rrule_on_a_checkpointed_3d_plan(engine):
    wl = configs.acoustic3d(nz=20, ny=18, nx=22, nt=100, npml=10, nrec_side=4, rfields=("vz",), src_field="p")
    pa, dobs, m = _setup(wl, checkpoints=3)
    g0 = np.zeros_like(m)
    J0 = gradient(g0, m, L2DistLoss(), dobs, pa)
    J, pb = rrule(lossvalue, m, L2DistLoss(), dobs, pa)
    assert J == J0
    assert np.array_equal(pb(1.0)[1], g0)
