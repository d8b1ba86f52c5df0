"""2-D acoustic FWI gradient (forward_save -> adjoint with boundary forcing
-> imaging condition) of the CUDA engine against the CPU oracle.

The observed data are zero, so the adjoint source is the whole modelled
record (-2 dcal) and the gradient is far above rounding level.  (With
observed data from a slightly different model the residual of these short
runs is close to FP32 rounding, and both sides then differentiate noise.)
Tolerance: relative L2 error 1e-5 on the raw per-cell accumulations."""
import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, Recs, configs, get_modelvector, gradient
from oracle import oracle as O

TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("nz,nx,nt,nshots", [(40, 70, 300, 1), (90, 160, 600, 2)])
def test_acoustic2d_gradient_matches_oracle(engine, nz, nx, nt, nshots):
    nrec = nx // 3
    start = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=nshots, nrec=nrec, anomaly=False)
    dobs_ref = {"vz": np.zeros((nshots, nt, nrec), np.float32)}
    loss_o, _, dcal_o, raw_o = O.gradient(start.as_dict(), dobs_ref)
    pa = start.expt(mode="forward_save")
    tg = pa.tgrid
    dobs = [Recs(len(s[1]), tg, ["vz"], {"vz": dobs_ref["vz"][i]}) for i, s in enumerate(start.shots)]
    m = get_modelvector(pa, ["invK", "rho"])
    g = np.zeros_like(m)
    loss = gradient(g, m, L2DistLoss(), dobs, pa)
    for i in range(nshots):
        e = rel(pa.data[0][i].d["vz"], dcal_o["vz"][i])
        assert e < 1e-5, ("dcal", i, e)
    assert abs(loss - loss_o) <= 1e-5 * abs(loss_o), (loss, loss_o)
    for k in ("invK", "rho"):
        e = rel(pa.gradients[k], raw_o[k])
        assert e < TOL, (k, e)
    assert np.all(np.isfinite(g)) and np.linalg.norm(g) > 0


class _HostL2(L2DistLoss):
    """L2DistLoss evaluated on the host (gradient! takes the device path for
    L2DistLoss itself only)."""


@pytest.mark.gpu
@pytest.mark.parametrize("checkpoints", [0, 6])
def test_device_adjoint_sources_equal_host_ones(engine, checkpoints):
    """gpi_set_adjoint_l2 (adjoint sources and misfit from the records on the
    device) gives the gradient of the host path bit for bit and its misfit
    within summation-order rounding, with observed data from another model."""
    nz, nx, nt, nshots = 60, 110, 400, 2
    true = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=nshots, nrec=nx // 2)
    pt = true.expt()
    from geophyinv_gb300 import update

    update(pt)
    dobs = [Recs(r.n, r.grid, r.fields, {f: r.d[f].copy() for f in r.fields}) for r in pt.data[0]]
    pt.close()
    start = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=nshots, nrec=nx // 2, anomaly=False)
    out = {}
    for name, loss in (("device", L2DistLoss()), ("host", _HostL2())):
        pa = start.expt(mode="forward_save", checkpoints=checkpoints)
        m = get_modelvector(pa, ["invK", "rho"])
        g = np.zeros_like(m)
        J = gradient(g, m, loss, dobs, pa)
        out[name] = (J, g.copy(), {k: v.copy() for k, v in pa.gradients.items()})
        pa.close()
    (Jd, gd, rd), (Jh, gh, rh) = out["device"], out["host"]
    assert Jd > 0 and abs(Jd - Jh) <= 1e-12 * Jh, (Jd, Jh)
    assert np.array_equal(gd, gh)
    for k in rd:
        assert np.array_equal(rd[k], rh[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [0, 2])
def test_gradient_with_copies_beside_the_runs_equals_the_plain_flow(engine, graph):
    """On a plan with its own stream gradient! uploads the observed data
    during the forward_save run and reads the records during the adjoint run;
    misfit, gradient and records equal those of the plan without a stream."""
    import torch

    from geophyinv_gb300 import update

    nz, nx, nt, nshots = 50, 90, 320, 3
    true = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=nshots, nrec=nx // 2)
    pt = true.expt()
    update(pt)
    dobs = [Recs(r.n, r.grid, r.fields, {f: np.array(r.d[f], order="F") for f in r.fields}) for r in pt.data[0]]
    start = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=nshots, nrec=nx // 2, anomaly=False)
    out = []
    for stream in (None, torch.cuda.Stream()):
        pa = start.expt(mode="forward_save", stream=None if stream is None else stream.cuda_stream)
        pa.set_graph(graph)
        m = get_modelvector(pa, ["invK", "rho"])
        g = np.zeros_like(m)
        J = gradient(g, m, L2DistLoss(), dobs, pa)
        J2 = gradient(g, m, L2DistLoss(), dobs, pa)  # a second call reuses the plan
        assert J2 == J
        out.append((J, g.copy(), [pa.data[0][i].d["vz"].copy() for i in range(nshots)]))
    (Ja, ga, ra), (Jb, gb, rb) = out
    assert Ja == Jb and Ja > 0
    assert np.array_equal(ga, gb)
    for a, b in zip(ra, rb):
        assert np.any(a != 0) and np.array_equal(a, b)
