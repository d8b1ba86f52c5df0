"""The FWI driver on the GPU engine: the inversion-grid gradient matches
finite differences of the inversion-grid misfit along an invK direction,
and L-BFGS lowers the misfit of a small anomaly problem (the reference's
SeisInvExpt + update!(paw), src/fwi/fwi.jl)."""
import numpy as np
import pytest

from geophyinv_gb300 import Recs, configs, fwi, update


def _problem(nshots=2, nt=400):
    true = configs.acoustic2d_fwi(nz=50, nx=90, nt=nt, nshots=nshots, nrec=45, anomaly=True, radius=60.0)
    pt = true.expt()
    update(pt)
    dobs = [Recs(r.n, r.grid, r.fields, {f: r.d[f].copy() for f in r.fields}) for r in pt.data[0]]
    start = configs.acoustic2d_fwi(nz=50, nx=90, nt=nt, nshots=nshots, nrec=45, anomaly=False)
    return fwi.SeisInvExpt(start.expt(mode="forward_save", checkpoints=4), dobs, [8, 12])


@pytest.mark.gpu
def test_inversion_grid_gradient_matches_finite_differences(engine):
    paw = _problem()
    m0 = fwi.get_modelvector_inv(paw)
    g = np.zeros_like(m0)
    fwi.gradient_inv(g, m0, paw)
    rng = np.random.default_rng(1)
    d = np.zeros_like(m0)
    d[: m0.size // 2] = rng.standard_normal(m0.size // 2)  # invK part
    h = 1e-3
    fd = (fwi.lossvalue_inv(m0 + h * d, paw) - fwi.lossvalue_inv(m0 - h * d, paw)) / (2 * h)
    adj = float(g @ d)
    assert abs(fd - adj) <= 2e-2 * abs(adj), (fd, adj)


@pytest.mark.gpu
def test_lbfgs_lowers_the_misfit(engine):
    paw = _problem()
    res = fwi.update(paw, maxiter=4)
    assert np.isfinite(res.fun)
    assert paw.history[-1] < 0.8 * paw.history[0], paw.history


@pytest.mark.gpu
def test_inversion_grid_gradient_matches_oracle(engine):
    """gradient!(g, m, pa::SeisInvExpt) (src/fwi/func_grad.jl:42-62) of the
    engine against the oracle's restatement (oracle/fwi_ref.py: the model
    through the inversion matrices, update!(pa, m) on the inner cells, the
    oracle's gradient!, the transposed matrices) at a perturbed model."""
    from oracle import fwi_ref as R
    from oracle import oracle as O
    from oracle import setup_ref as S

    paw = _problem(nshots=2, nt=300)
    pa = paw.paf
    m0 = fwi.get_modelvector_inv(paw)
    m = (m0 + 0.02 * np.random.default_rng(4).standard_normal(m0.size)).astype(np.float32)
    g = np.zeros_like(m)
    J, _ = fwi.gradient_inv(g, m, paw)
    start = configs.acoustic2d_fwi(nz=50, nx=90, nt=300, nshots=2, nrec=45, anomaly=False)
    ex = start.as_dict()
    prep = O.Prepared(ex)
    P = R.inversion_matrices(paw.mmgrid, paw.migrid)
    ref = {k: S.bounds(prep.mod[i])[0] for i, k in enumerate(("invK", "rho"))}
    mfull = R.to_full(m, P, paw.mparams)
    mod = R.medium_from_modelvector(prep, mfull, paw.mparams, ref)
    dobs = {"vz": np.stack([d.d["vz"] for d in paw.dobs])}
    loss, go, _, _ = O.gradient(ex, dobs, mod=mod, history=True)  # the plan is checkpointed
    gfull = np.concatenate([go["invK"].ravel(order="F"), go["rho"].ravel(order="F")])
    want = R.to_inversion(gfull, P, paw.mparams)
    e = np.linalg.norm(g - want) / np.linalg.norm(want)
    assert e < 1e-5, e
    assert abs(J - loss) <= 1e-5 * abs(loss), (J, loss)
