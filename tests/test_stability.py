"""check_stability (src/fdtd/stability.jl:8-60) and findfreq's max / min
(src/Utils/freq.jl:28-57), host only: the Courant and the spatial-sampling
warnings fire where the reference's would."""
import warnings

import numpy as np
import pytest

from geophyinv_gb300 import AcousticMedium, ElasticMedium, FdtdAcoustic, FdtdElastic, Grid, SeisForwExpt, ricker
from geophyinv_gb300 import setup as S


class _Expt:
    """The attributes check_stability reads, without a plan."""

    def __init__(self, attrib, medium, dt, fmax):
        self.attrib, self.medium, self.dt, self.freqmax = attrib, medium, dt, fmax
        self.ndim, self.order = len(medium.grid), 4


def _acoustic(d=5.0):
    g = [Grid(0.0, d, 30), Grid(0.0, d, 40)]
    vp = np.full((30, 40), 2000.0, np.float32)
    vp[15:] = 3000.0
    return AcousticMedium(g, vp, np.full((30, 40), 2000.0, np.float32))


def _check(e):
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        SeisForwExpt.check_stability(e)
    return [str(x.message) for x in w]


def test_courant_limit():
    m = _acoustic()
    lim = 5.0 / np.sqrt(2) / 3000.0  # 1.18e-3
    assert not _check(_Expt(FdtdAcoustic(), m, 1e-3, 20.0))
    msg = _check(_Expt(FdtdAcoustic(), m, 1.3e-3, 20.0))
    assert any("decrease time sampling" in x for x in msg), msg
    assert lim < 1.3e-3


def test_spatial_sampling_uses_the_slowest_velocity_and_fmax():
    m = _acoustic(d=5.0)
    # 2000 m/s / 5 points / 100 Hz = 4 m < 5 m
    msg = _check(_Expt(FdtdAcoustic(), m, 1e-4, 100.0))
    assert any("decrease maximum spatial sampling" in x for x in msg), msg
    assert not any("spatial" in x for x in _check(_Expt(FdtdAcoustic(), m, 1e-4, 50.0)))


def test_elastic_limits_use_vs_and_the_p_s_combination():
    g = [Grid(0.0, 5.0, 20), Grid(0.0, 5.0, 20)]
    vp = np.full((20, 20), 3000.0, np.float32)
    vs = np.full((20, 20), 1500.0, np.float32)
    m = ElasticMedium(g, vp, vs, np.full((20, 20), 2000.0, np.float32))
    # a homogeneous medium gets bounds of +-10 % (the reference's Medium
    # bounds): vmax = sqrt(3300^2 + 1650^2) = 3689 -> dt limit 9.58e-4
    assert any("time sampling" in x for x in _check(_Expt(FdtdElastic(), m, 1.0e-3, 10.0)))
    assert not any("time sampling" in x for x in _check(_Expt(FdtdElastic(), m, 9.0e-4, 10.0)))
    # vmin = vs = 1500: 1500 / 5 / 70 = 4.3 m < 5 m
    assert any("spatial" in x for x in _check(_Expt(FdtdElastic(), m, 1e-4, 70.0)))


def test_findfreq_max_and_min_bracket_the_peak():
    tg = Grid(0.0, 0.001, 1000)
    w = np.asarray(ricker(15.0, tg), np.float64)
    fpk = S.findfreq(w, 0.001, "peak")
    fmax = S.findfreq(w, 0.001, "max")
    fmin = S.findfreq(w, 0.001, "min")
    assert fmin < fpk < fmax
    assert abs(fpk - S.findfreq_peak(w, 0.001)) < 1e-9
    assert 13.0 < fpk < 17.0 and fmax > 2 * fpk
