"""Host-side setup of the product against the oracle's restatement:
padding, derived parameters, CPML profiles, projection matrices, wavelets."""
import numpy as np
import pytest

from geophyinv_gb300 import setup as P
from oracle import setup_ref as S


def test_padding_and_derived():
    rng = np.random.default_rng(3)
    vp = (2000 + 500 * rng.random((17, 23))).astype(np.float32)
    rho = (1800 + 300 * rng.random((17, 23))).astype(np.float32)
    for mask in (63, 63 & ~1, 16 | 2):
        a = P.padarray(vp, 43, mask)
        b = S.padarray(vp, 43, mask)
        assert np.array_equal(a, b)
        assert [(g.start, g.step, g.n) for g in P.padgrid([P.Grid(0, 5, 17), P.Grid(0, 5, 23)], 43, mask)] == \
            S.padmgrid([(0.0, 5.0, 17), (0.0, 5.0, 23)], 43, mask)
    assert np.array_equal(P.invK(vp, rho), S.derived_acoustic(vp, rho)[0])
    vs = (vp / 1.8).astype(np.float32)
    e = S.derived_elastic(vp, vs, rho)
    assert np.array_equal(P.invlambda(vp, vs, rho), e[0])
    assert np.array_equal(P.invmu(vs, rho), e[1])
    r1, b1 = P.ref_bounds(vp)
    r2, b2 = S.bounds(vp)
    assert r1 == r2 and np.array_equal(np.array(b1), b2)


@pytest.mark.parametrize("physics,ndim", [("acoustic", 2), ("elastic", 2), ("acoustic", 3), ("elastic", 3)])
def test_cpml_profiles(physics, ndim):
    grid = [P.Grid(0, 5, 31), P.Grid(0, 10, 21), P.Grid(0, 5, 41)][:ndim] if ndim == 3 else [P.Grid(0, 5, 31),
                                                                                            P.Grid(0, 5, 41)]
    mask = 63 & ~1
    dt, va, fp = np.float32(0.0005), np.float32(2745.5), np.float32(15.0)
    a = P.cpml_all(physics, ndim, 4, grid, mask, dt, va, fp, 43)
    b = S.pml_all(physics, ndim, 4, [(g.start, g.step, g.n) for g in grid], mask, dt, va, fp)
    assert len(a) == len(b) == len(P.DERIV[(physics, ndim)])
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            np.testing.assert_allclose(u, v, rtol=2e-7, atol=1e-12)


@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("ref_compat", [True, False])
def test_projection_matrices(ndim, ref_compat):
    rng = np.random.default_rng(7)
    if ndim == 2:
        grid = [P.Grid(-215, 5, 87), P.Grid(-215, 5, 101)]
        pts = np.stack([rng.uniform(-5, 220, 9), rng.uniform(-5, 290, 9)], 1)
        pts[0] = (0.0, 0.0)
        fields = ["p", "vx", "vz"]
    else:
        grid = [P.Grid(-100, 10, 31), P.Grid(-100, 10, 29), P.Grid(-100, 10, 33)]
        pts = np.stack([rng.uniform(0, 90, 6), rng.uniform(0, 70, 6), rng.uniform(0, 110, 6)], 1)
        fields = ["p", "vx", "vy", "vz", "tauxy", "tauxz", "tauyz"]
    sgrid = [(g.start, g.step, g.n) for g in grid]
    for f in fields:
        cp, rv, nz = P.projection(f, grid, pts, 4, ref_compat)
        cp2, rv2, nz2 = S.proj_matrix(f, sgrid, [tuple(p) for p in pts], ndim, 4, ref_compat)
        assert np.array_equal(cp, cp2)
        assert np.array_equal(rv, rv2)
        np.testing.assert_array_equal(nz, nz2)


def test_wavelets():
    g = P.Grid(0.0, 0.0005, 2000)
    np.testing.assert_allclose(P.ricker(15.0, g), S.ricker(15.0, 2000, 0.0005), rtol=0, atol=1e-15)
    w = P.ricker(15.0, g).astype(np.float32)
    assert P.findfreq_peak(w, 0.0005) == S.findfreq_peak(w, 0.0005) == 15.0
    w2 = np.stack([w, 2 * w], 1)
    np.testing.assert_array_equal(P.reverse_source(w2), S.source_reverse(w2))


def test_ormsby_wavelet():
    """ormsby (src/srcwav/wavelets.jl:75-142), with Julia's normalised sinc:
    unit peak at tpeak, symmetric about it, the pass band at pi [f1, f4],
    and the taper! of src/Utils/taper.jl:20-36 zeroing the end samples."""
    import math

    from geophyinv_gb300.setup import Grid, findfreq_peak, ormsby, taper

    tg = Grid(0.0, 0.001, 801)
    f = 5.0
    w = ormsby(f, tg)
    f1, f4 = f - 0.6 * f, f + 0.6 * f
    f2, f3 = 0.25 * f4 + 0.75 * f1, 0.25 * f1 + 0.75 * f4
    tpeak = 1.5 / (0.25 * (f1 + f4))
    ip = int(round(tpeak / 0.001))
    assert abs(np.max(np.abs(w)) - 1.0) < 1e-15 and abs(w[ip] - 1.0) < 1e-12
    assert np.allclose(w[ip - 100:ip], w[ip + 100:ip:-1], atol=1e-12)

    # one sample against the formula written out with sin (Julia's sinc(x) = sin(pi x) / (pi x))
    def S(fk, t):
        x = math.pi * fk * t
        return (math.sin(math.pi * x) / (math.pi * x)) ** 2

    pi = math.pi
    A43, A34 = (pi * f4) ** 2 / (pi * f4 - pi * f3), (pi * f3) ** 2 / (pi * f4 - pi * f3)
    A21, A12 = (pi * f2) ** 2 / (pi * f2 - pi * f1), (pi * f1) ** 2 / (pi * f2 - pi * f1)
    t = 0.037 - tpeak
    raw = (A43 * S(f4, t) - A34 * S(f3, t)) - (A21 * S(f2, t) - A12 * S(f1, t))
    t0 = 1e-9
    peak = (A43 * S(f4, t0) - A34 * S(f3, t0)) - (A21 * S(f2, t0) - A12 * S(f1, t0))
    assert abs(w[37] - raw / peak) < 1e-6
    fp = findfreq_peak(w, 0.001)
    assert pi * f1 <= fp <= pi * f4
    wt = ormsby(f, tg, tperc=10.0)
    assert wt[0] == 0.0 and wt[-1] == 0.0 and wt[ip] == w[ip]
    x = taper(np.ones(20), 25.0)  # 5 samples each end: sin(k pi / 9)
    assert np.allclose(x[:5], np.sin(np.arange(5) * math.pi / 9)) and np.allclose(x[5:15], 1.0)
    assert np.allclose(x[15:], np.sin((20 - np.arange(16, 21)) * math.pi / 9))
