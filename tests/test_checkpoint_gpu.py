"""Checkpointed adjoint (a plan created with `checkpoints` > 0; no
counterpart in the reference): forward_save keeps a few full states of the
forward wavefield, the adjoint run recomputes forward states from them on a
binomial schedule instead of rebuilding them by time reversal from the
boundary store.

Parity: the CPU oracle's history mode (GPO_FORWARD_HIST / GPO_ADJOINT_HIST)
computes the same imaging condition with wavefield 1 taken from the stored
forward history; the raw per-cell accumulations agree within a relative L2
error of 1e-5 (FP32).  Against the reference's own time-reversal gradient
(the oracle's default mode) they agree within 1e-5 away from the edge of
the inner grid: in the reference's 3-cell boundary strips and where the
rho averages reach into the PML, the time-reversed run correlates values it
left unforced there, so the two gradients differ in a 6-cell border."""
import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, Recs, configs, get_modelvector, gradient, lossvalue, update
from oracle import oracle as O

TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0)


def _gpu_gradient(wl, slots, dobs_arr, graph=False, reverse_sources=False):
    pa = wl.expt(mode="forward_save", checkpoints=slots)
    if graph:
        pa.set_graph(True)
    tg = pa.tgrid
    dobs = [Recs(len(s[1]), tg, list(wl.rfields), {f: dobs_arr[f][i] for f in wl.rfields})
            for i, s in enumerate(wl.shots)]
    m = get_modelvector(pa, ["invK", "rho"])
    g = np.zeros_like(m)
    if reverse_sources:
        # the reference's own flow (func_grad.jl:33): time-reversed sources
        # for wavefield 1; the checkpointed plan recomputes with the sources
        # of its forward_save run regardless
        pa.checkpoints_saved, pa.checkpoints = pa.checkpoints, 0
        try:
            loss = gradient(g, m, L2DistLoss(), dobs, pa)
        finally:
            pa.checkpoints = pa.checkpoints_saved
    else:
        loss = gradient(g, m, L2DistLoss(), dobs, pa)
    return loss, pa.gradients, g, pa


def _zero_dobs(wl):
    return {f: np.zeros((len(wl.shots), wl.nt, len(wl.shots[0][1])), np.float32) for f in wl.rfields}


@pytest.mark.gpu
@pytest.mark.parametrize("nz,nx,nt,nshots,slots", [(40, 70, 300, 1, 3), (90, 160, 600, 2, 7)])
def test_acoustic2d_checkpointed_gradient_matches_oracle(engine, nz, nx, nt, nshots, slots):
    wl = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=nshots, nrec=nx // 3, anomaly=False)
    dobs = _zero_dobs(wl)
    loss_h, _, _, raw_h = O.gradient(wl.as_dict(), dobs, history=True)
    loss, raw, _, _ = _gpu_gradient(wl, slots, dobs)
    assert abs(loss - loss_h) <= 1e-5 * abs(loss_h)
    for k in ("invK", "rho"):
        assert rel(raw[k], raw_h[k]) < TOL, (k, rel(raw[k], raw_h[k]))
    # the reference's time-reversal gradient, away from the border
    _, _, _, raw_r = O.gradient(wl.as_dict(), dobs)
    npml = 43
    inner = (slice(npml + 6, npml + nz - 6), slice(npml + 6, npml + nx - 6))
    for k in ("invK", "rho"):
        e = rel(raw[k][inner], raw_r[k][inner].astype(np.float64))
        assert e < TOL, (k, e)


@pytest.mark.gpu
def test_slot_count_does_not_change_the_gradient(engine):
    """The recomputed forward states are the forward run's own, bit for bit,
    whatever the schedule."""
    wl = configs.acoustic2d_fwi(nz=40, nx=60, nt=200, nshots=2, nrec=20, anomaly=False)
    dobs = _zero_dobs(wl)
    ref = _gpu_gradient(wl, 200, dobs)[1]
    for slots in (1, 2, 9):
        raw = _gpu_gradient(wl, slots, dobs)[1]
        for k in ("invK", "rho"):
            assert np.array_equal(raw[k], ref[k]), (slots, k)


@pytest.mark.gpu
def test_checkpointed_gradient_under_graphs_and_reference_flow(engine):
    wl = configs.acoustic2d_fwi(nz=40, nx=60, nt=200, nshots=1, nrec=20, anomaly=False)
    dobs = _zero_dobs(wl)
    ref = _gpu_gradient(wl, 4, dobs)[1]
    for kw in ({"graph": True}, {"reverse_sources": True}):
        raw = _gpu_gradient(wl, 4, dobs, **kw)[1]
        for k in ("invK", "rho"):
            assert np.array_equal(raw[k], ref[k]), (kw, k)


@pytest.mark.gpu
@pytest.mark.parametrize("src_field", ["p", "vz"])
def test_acoustic3d_checkpointed_gradient_matches_oracle(engine, src_field):
    wl = configs.acoustic3d(nz=20, ny=18, nx=22, nt=100, npml=10, nrec_side=4, rfields=("vz",), src_field=src_field)
    dobs = _zero_dobs(wl)
    loss_h, _, _, raw_h = O.gradient(wl.as_dict(), dobs, history=True)
    loss, raw, _, _ = _gpu_gradient(wl, 3, dobs)
    assert abs(loss - loss_h) <= 1e-5 * abs(loss_h)
    for k in ("invK", "rho"):
        assert rel(raw[k], raw_h[k]) < TOL, (k, rel(raw[k], raw_h[k]))


@pytest.mark.gpu
@pytest.mark.parametrize("npml", [43, 23, 10])
def test_acoustic3d_checkpointed_invK_gradient_matches_finite_differences(engine, npml):
    """Central differences of lossvalue on blocks of the inner grid (the
    reference's gradient-accuracy test, test/fwi/gradient_accuracy.jl, in
    3-D, which the reference cannot run), with the reference's 43-cell PML
    and with thin ones: measured on GB300, 1e-6 to 1e-4 on the blocks with
    a large gradient at every width (the third block's gradient is 40 times
    smaller, 5e-4 to 5e-3)."""
    nz, ny, nx, nt = 32, 28, 34, 220
    wl = configs.acoustic3d(nz=nz, ny=ny, nx=nx, nt=nt, npml=npml, nrec_side=5, rfields=("vz",), src_field="p")
    s, r = wl.shots[0]
    r = r.copy()
    r[:, 0] = 40.0  # receivers 4 cells below the surface
    wl.shots = [(s, r)]
    pa = wl.expt(mode="forward_save", checkpoints=6)
    nr = len(r)
    dobs = [Recs(nr, pa.tgrid, ["vz"], {"vz": np.zeros((nt, nr), np.float32)})]
    m0 = get_modelvector(pa, ["invK", "rho"])
    g = np.zeros_like(m0)
    gradient(g, m0, L2DistLoss(), dobs, pa)
    assert np.all(np.isfinite(g))
    h = 1e-2
    n = nz * ny * nx
    for z0, y0, x0 in ((12, 8, 10), (10, 10, 10), (14, 12, 16)):
        blk = np.zeros((nz, ny, nx), np.float32)
        blk[z0:z0 + 6, y0:y0 + 6, x0:x0 + 6] = 1
        e = np.zeros_like(m0)
        e[:n] = blk.ravel(order="F")
        fd = (lossvalue(m0 + h * e, L2DistLoss(), dobs, pa) - lossvalue(m0 - h * e, L2DistLoss(), dobs, pa)) / (2 * h)
        adj = float(g @ e)
        print("npml %d block %s: fd %.6e adjoint %.6e rel %.2e" % (npml, (z0, y0, x0), fd, adj, abs(fd - adj) / abs(adj)))
        assert abs(fd - adj) <= 1e-2 * abs(adj), ((z0, y0, x0), fd, adj)
