"""Parity at the sizes the benchmark times, against the CPU oracle.

  elastic 2-D batch   1000 x 3000 at 5 m (1086 x 3086 extended), 16 shots,
                      4000 steps, 601 vx / vz receivers, 16-step chunk graphs:
                      the whole batch on the GPU, shots 0 and 15 checked
  acoustic 2-D FWI    500 x 1500 at 10 m (586 x 1586), 3000 steps; observed
  gradient            data from the model with the anomaly, gradient! on the
                      model without it for shots 15 and 16 of the 32
  elastic 3-D         600^3 at 10 m with npml 23 (646^3 extended), the full
                      grid for 60 of its 2500 steps

Relative L2 tolerance 1e-5 against the FP32 oracle (the target's bound).
Each case also prints its error against an FP64 oracle run where the host
can hold one (the 3-D grid in FP64 would need about 70 GB of host memory;
its FP64 error is measured on reduced grids in test_fp64_error_gpu.py).
Run with -s to see the lines

    FULL <case> <quantity> fp32 <error> [fp64 <error>]
"""
import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, Recs, configs, get_modelvector, gradient, update
from oracle import oracle as O

TOL = 1e-5


def rel(a, b):
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0))


def _line(case, what, e32, e64=None):
    print("FULL %-34s %-10s fp32 %.3e%s" % (case, what, e32, "" if e64 is None else "  fp64 %.3e" % e64))


def _subset(ex, shots):
    ex = dict(ex)
    ex["shots"] = [ex["shots"][i] for i in shots]
    return ex


@pytest.mark.gpu
def test_elastic2d_batch_full_size_matches_oracle(engine):
    wl = configs.elastic2d_batch()
    assert len(wl.shots) == 16 and wl.nt == 4000
    pa = wl.expt()
    pa.set_graph(2)  # replays of a captured 16-step chunk, as timed
    update(pa)
    ex = wl.as_dict()
    for iss in (0, 15):
        ref = O.forward(_subset(ex, [iss]))
        ref64 = O.forward(_subset(ex, [iss]), dtype=np.float64) if iss == 0 else None
        for f in wl.rfields:
            got = pa.data[0][iss].d[f]
            e = rel(got, ref[f][0])
            _line("elastic2d 1086x3086 4000 st shot %d" % iss, "rec " + f, e,
                  None if ref64 is None else rel(got, ref64[f][0]))
            assert e < TOL, (iss, f, e)
    pa.close()


@pytest.mark.gpu
def test_acoustic2d_fwi_gradient_full_size_matches_oracle(engine):
    # two of the 32 shots above the anomaly (the outermost shots' records
    # do not reach it within 3 s, so their residual would be rounding noise)
    shots = [15, 16]
    true = configs.acoustic2d_fwi()
    assert len(true.shots) == 32 and true.nt == 3000
    true.shots = [true.shots[i] for i in shots]
    pt = true.expt()
    update(pt)
    dobs = [Recs(r.n, r.grid, r.fields, {f: r.d[f].copy() for f in r.fields}) for r in pt.data[0]]
    pt.close()
    wl = configs.acoustic2d_fwi(anomaly=False)
    wl.shots = [wl.shots[i] for i in shots]
    pa = wl.expt(mode="forward_save")
    pa.set_graph(2)
    m0 = get_modelvector(pa, ["invK", "rho"])
    g = np.zeros_like(m0)
    J = gradient(g, m0, L2DistLoss(), dobs, pa)
    od = {f: np.stack([d.d[f] for d in dobs]) for f in wl.rfields}
    loss, _, dcal, raw = O.gradient(wl.as_dict(), od)
    loss64, _, dcal64, raw64 = O.gradient(wl.as_dict(), od, dtype=np.float64)
    case = "acoustic2d grad 586x1586 3000 st"
    for i in range(len(shots)):
        e = rel(pa.data[0][i].d["vz"], dcal["vz"][i])
        _line(case + " shot %d" % shots[i], "rec vz", e, rel(pa.data[0][i].d["vz"], dcal64["vz"][i]))
        assert e < TOL, ("records", i, e)
    assert loss > 0 and np.linalg.norm(raw["rho"]) > 0
    for k in ("invK", "rho"):
        e = rel(pa.gradients[k], raw[k])
        _line(case, "grad " + k, e, rel(pa.gradients[k], raw64[k]))
        assert e < TOL, (k, e)
    assert abs(J - loss) <= TOL * abs(loss), (J, loss)
    pa.close()


@pytest.mark.gpu
def test_elastic3d_full_grid_matches_oracle(engine):
    nt = 60
    wl = configs.elastic3d(nt=nt, rfields=("vx", "vz"))
    assert wl.npml == 23 and [len(g) for g in wl.grid] == [600, 600, 600]
    pa = wl.expt()
    update(pa)
    got = {f: pa.data[0][0].d[f].copy() for f in wl.rfields}
    pa.close()
    ref = O.forward(wl.as_dict())
    for f in wl.rfields:
        e = rel(got[f], ref[f][0])
        _line("elastic3d 646^3 npml23 60 st", "rec " + f, e)
        assert np.linalg.norm(ref[f][0]) > 0, f
        assert e < TOL, (f, e)
