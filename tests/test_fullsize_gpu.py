"""Parity at the sizes the benchmark times, against the CPU oracle.

  elastic 2-D batch   1000 x 3000 at 5 m (1086 x 3086 extended), 16 shots,
                      4000 steps, 601 vx / vz receivers, 16-step chunk graphs:
                      the whole batch on the GPU, shots 0 and 15 checked
  acoustic 2-D FWI    500 x 1500 at 10 m (586 x 1586), 3000 steps,
  gradient            gradient! on the model without the anomaly for shots 15
                      and 16 of the 32 (zero observed data, and observed data
                      from the model with the anomaly)
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


def _grad_case(engine_dobs, oracle_dobs, shots, label):
    wl = configs.acoustic2d_fwi(anomaly=False)
    wl.shots = [wl.shots[i] for i in shots]
    pa = wl.expt(mode="forward_save")
    pa.set_graph(2)
    m0 = get_modelvector(pa, ["invK", "rho"])
    g = np.zeros_like(m0)
    J = gradient(g, m0, L2DistLoss(), engine_dobs, pa)
    loss, _, dcal, raw = O.gradient(wl.as_dict(), oracle_dobs)
    _, _, dcal64, raw64 = O.gradient(wl.as_dict(), oracle_dobs, dtype=np.float64)
    case = "acoustic2d grad 586x1586 3000 st " + label
    for i in range(len(shots)):
        _line(case + " shot %d" % shots[i], "rec vz", rel(pa.data[0][i].d["vz"], dcal["vz"][i]),
              rel(pa.data[0][i].d["vz"], dcal64["vz"][i]))
    e = {}
    for k in ("invK", "rho"):
        e[k] = (rel(pa.gradients[k], raw[k]), rel(pa.gradients[k], raw64[k]), rel(raw[k], raw64[k]))
        _line(case, "grad " + k, e[k][0], e[k][1])
    recs = [rel(pa.data[0][i].d["vz"], dcal["vz"][i]) for i in range(len(shots))]
    pa.close()
    return J, loss, e, recs


@pytest.mark.gpu
def test_acoustic2d_fwi_gradient_full_size_matches_oracle(engine):
    """The FWI gradient at full size (586 x 1586, 3000 steps) for shots 15
    and 16 of the 32, through the reference's time-reversal adjoint.

    With zero observed data the adjoint sources are the whole records and
    the gradient is well conditioned: engine and FP32 oracle agree within
    1e-5.  With observed data from the model with the anomaly (the
    benchmark's case) the residual is about 1e-5 of the records at these
    offsets, so any FP32 run of the gradient carries rounding at the
    percent level: the engine's distance from the FP64 gradient is then
    required to stay within twice the FP32 oracle's own distance from it."""
    shots = [15, 16]
    nt, nr = 3000, 1500
    zero_e = [Recs(nr, configs.acoustic2d_fwi().tgrid, ["vz"], {"vz": np.zeros((nt, nr), np.float32)})
              for _ in shots]
    zero_o = {"vz": np.zeros((len(shots), nt, nr), np.float32)}
    J, loss, e, recs = _grad_case(zero_e, zero_o, shots, "zero dobs")
    for r in recs:
        assert r < TOL, r
    for k in ("invK", "rho"):
        assert e[k][0] < TOL, (k, e[k])
    assert abs(J - loss) <= TOL * abs(loss), (J, loss)
    # observed data from the model with the anomaly
    true = configs.acoustic2d_fwi()
    assert len(true.shots) == 32 and true.nt == nt
    true.shots = [true.shots[i] for i in shots]
    pt = true.expt()
    update(pt)
    dobs = [Recs(r.n, r.grid, r.fields, {f: r.d[f].copy() for f in r.fields}) for r in pt.data[0]]
    pt.close()
    od = {f: np.stack([d.d[f] for d in dobs]) for f in ["vz"]}
    J, loss, e, recs = _grad_case(dobs, od, shots, "anomaly dobs")
    for k in ("invK", "rho"):
        print("FULL anomaly dobs grad %s: FP32 oracle vs FP64 oracle %.3e" % (k, e[k][2]))
        assert e[k][1] <= 2 * e[k][2] + TOL, (k, e[k])


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
