"""CUDA graphs (gpi_set_graph): a captured and replayed run (1: the whole
run; 2: replays of a captured 16-step chunk that reads the step from a
device counter, remainder steps plain) gives the same records, fields and
gradients as plain launches, bit for bit, and changing the sources drops
and re-captures the graph."""
import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, Recs, configs, get_modelvector, gradient, update


def _records(pa, wl):
    return [{f: pa.data[0][i].d[f].copy() for f in wl.rfields} for i in range(len(wl.shots))]


@pytest.mark.gpu
@pytest.mark.parametrize("gkind", [1, 2])
@pytest.mark.parametrize("kind", ["acoustic", "elastic", "acoustic3d"])
def test_graph_runs_match_plain_runs(engine, kind, gkind):
    if kind == "acoustic":
        wl = configs.acoustic2d_layers(nz=101, nx=131, nt=300, nrec=21)
    elif kind == "elastic":
        wl = configs.elastic2d_batch(nz=110, nx=190, nt=300, nshots=3, nrec=31)
    else:
        wl = configs.acoustic3d(nz=20, ny=18, nx=22, nt=75, npml=10, nrec_side=4, rfields=("p", "vz"))
    plain = wl.expt()
    update(plain)
    want = _records(plain, wl)
    pa = wl.expt()
    pa.set_graph(gkind)
    for _ in range(2):  # capture, then replay
        update(pa)
        got = _records(pa, wl)
        for a, b in zip(got, want):
            for f in wl.rfields:
                assert np.array_equal(a[f], b[f]), f
    f0 = "vz" if kind == "elastic" else "p"
    assert np.array_equal(pa.field(f0, iss=len(wl.shots) - 1), plain.field(f0, iss=len(wl.shots) - 1))
    # new wavelets: the graph is dropped and captured again
    sw = wl.srcwav()
    for s in sw:
        for f in s.fields:
            s.d[f] = (2.0 * s.d[f]).astype(np.float32)
    update(plain, sw, [1])
    update(plain)
    update(pa, sw, [1])
    update(pa)
    for a, b in zip(_records(pa, wl), _records(plain, wl)):
        for f in wl.rfields:
            assert np.array_equal(a[f], b[f]), f


@pytest.mark.gpu
def test_graph_gradient_matches_plain_gradient(engine):
    nz, nx, nt, nrec = 40, 70, 300, 23
    wl = configs.acoustic2d_fwi(nz=nz, nx=nx, nt=nt, nshots=2, nrec=nrec, anomaly=False)
    out = []
    for graph in (0, 1, 2):
        pa = wl.expt(mode="forward_save")
        pa.set_graph(graph)
        dobs = [Recs(nrec, pa.tgrid, ["vz"], {"vz": np.zeros((nt, nrec), np.float32)}) for _ in range(2)]
        m = get_modelvector(pa, ["invK", "rho"])
        g = np.zeros_like(m)
        loss = gradient(g, m, L2DistLoss(), dobs, pa)
        out.append((loss, g.copy()))
    for loss, g in out[1:]:
        assert loss == out[0][0]
        assert np.array_equal(g, out[0][1])
