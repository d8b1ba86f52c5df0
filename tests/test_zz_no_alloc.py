"""gpi_forward_acoustic2d_noalloc: the forward run for hosts that cannot call
cudaMalloc (a pre-reserved pool allocator owns their HBM, or their loop must
not hit cudaMalloc's device-wide synchronisation).  It must give the records
of the plan path (gpi_plan_create + gpi_run), call after call, although it
keeps all intermediates in one shared static device array.

This file is collected last so that a failure here cannot hide the other
GPU tests."""
import ctypes

import numpy as np
import pytest

from geophyinv_gb300 import configs, update

TOL = 1e-5  # relative L2, the tolerance of the other parity tests


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32).ravel(order="F"))).cuda()


def _noalloc(engine, torch, pa):
    """One gpi_forward_acoustic2d_noalloc call on the inputs of plan `pa`;
    returns {field: records nt x nr}."""
    invK = _dev(torch, pa.mod["invK"])
    rho = _dev(torch, pa.mod["rho"])
    pml = _dev(torch, np.concatenate([np.concatenate(x) for x in pa.pml]))
    sw = pa.srcwav[0][0]
    field = sw.fields[0]
    wav = _dev(torch, sw.d[field])
    scp, srv, snz = pa._proj(field, pa.ageom[0].points("s", 2))
    rf = pa.rfields
    fid = {"p": 0, "vx": 1, "vz": 3}
    nr = [pa.ageom[0].nr] * len(rf)
    cps = [pa._rproj[0][f][0] for f in rf]
    rvs = [pa._rproj[0][f][1] for f in rf]
    nzs = [pa._rproj[0][f][2] for f in rf]
    P = ctypes.c_void_p
    arrp = lambda xs: (P * len(xs))(*[x.ctypes.data for x in xs])  # noqa: E731
    stream = torch.cuda.current_stream().cuda_stream
    outs = [torch.full((pa.nt * n,), np.nan, device="cuda") for n in nr]
    rc = engine.gpi_forward_acoustic2d_noalloc(
        ctypes.byref(pa.desc), P(invK.data_ptr()), P(rho.data_ptr()), P(pml.data_ptr()), fid[field], sw.n,
        P(scp.ctypes.data), P(srv.ctypes.data), P(snz.ctypes.data), P(wav.data_ptr()), len(rf),
        (ctypes.c_int * len(rf))(*[fid[f] for f in rf]), (ctypes.c_int * len(rf))(*nr), arrp(cps), arrp(rvs),
        arrp(nzs), (P * len(rf))(*[o.data_ptr() for o in outs]), P(stream))
    assert rc == 0, engine.gpi_last_error(None)
    torch.cuda.synchronize()
    return {f: o.cpu().numpy().reshape(n, pa.nt).T for f, o, n in zip(rf, outs, nr)}


def _check(got, pa, what):
    for f in pa.rfields:
        ref = pa.data[0][0].d[f]
        e = np.linalg.norm(got[f] - ref) / np.linalg.norm(ref)
        assert e < TOL, (what, f, e)


@pytest.mark.gpu
def test_noalloc_forward_matches_plan_path(engine):
    """Two calls in a row on the same inputs both give the plan's records."""
    import torch

    wl = configs.acoustic2d_layers(nz=101, nx=131, nt=400, nrec=31)
    pa = wl.expt()
    update(pa)
    for call in range(2):
        _check(_noalloc(engine, torch, pa), pa, call)


@pytest.mark.gpu
def test_noalloc_larger_then_smaller_call_leaves_nothing_behind(engine):
    """A larger grid followed by a smaller one (the scratch layout shifts
    between them) and a velocity source in the second call: each call
    matches the plan path, and the second one also the CPU oracle."""
    import torch

    from oracle import oracle as O

    big = configs.acoustic2d_layers(nz=161, nx=221, nt=300, nrec=41)
    pb = big.expt()
    update(pb)
    _check(_noalloc(engine, torch, pb), pb, "big")
    small = configs.acoustic2d_layers(nz=97, nx=123, nt=350, nrec=29, src_field="vz")
    ps = small.expt()
    update(ps)
    got = _noalloc(engine, torch, ps)
    _check(got, ps, "small after big")
    ref = O.forward(small.as_dict())
    for f in small.rfields:
        e = np.linalg.norm(got[f] - ref[f][0]) / np.linalg.norm(ref[f][0])
        assert e < TOL, ("oracle", f, e)


@pytest.mark.gpu
def test_noalloc_rejects_problems_beyond_the_scratch(engine):
    wl = configs.acoustic2d_layers(nz=101, nx=131, nt=10, nrec=3)
    pa = wl.expt()
    d = pa.desc
    big = type(d)()
    ctypes.memmove(ctypes.byref(big), ctypes.byref(d), ctypes.sizeof(d))
    big.nz, big.nx = 4000, 4000  # about 0.7 GB of intermediates
    P = ctypes.c_void_p
    one = np.array([0, 1], np.int64)
    row = np.array([0], np.int64)
    w = np.array([1.0], np.float32)
    rc = engine.gpi_forward_acoustic2d_noalloc(ctypes.byref(big), P(1), P(1), P(1), 0, 1, P(one.ctypes.data),
                                               P(row.ctypes.data), P(w.ctypes.data), P(1), 0, None, None, None,
                                               None, None, None, None)
    assert rc == -1
    assert b"64 MiB" in engine.gpi_last_error(None)
