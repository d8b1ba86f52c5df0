"""The engine against the 2-D Green's function (the reference's accuracy
test, test/fdtd/accuracy2D.jl:6-82): pressure of a point pressure source in
a homogeneous medium, FP32 on the GPU, against rho dA w / 4 H0^(2)(w r / c)
W(w) in absolute amplitude and phase (the reference asks a normalised
misfit below 1e-2), at every stencil order; and the 3-D one
(accuracy3D.jl), rho dV / (4 pi r) w'(t - r / c)."""
import numpy as np
import pytest
from scipy.special import hankel2

from geophyinv_gb300 import Grid, configs, ricker, update


@pytest.mark.gpu
@pytest.mark.parametrize("order,bound", [(4, 1e-4), (2, 5e-3), (6, 1e-4), (8, 1e-4)])
def test_green_function_on_the_engine(engine, order, bound):
    nz = nx = 161
    d, nt, dt = 5.0, 600, 0.0005
    vp, rho, f0 = 2000.0, 2000.0, 15.0
    sz = sx = 400.0
    offs = np.array([100.0, 150.0, 200.0])
    tgrid = Grid(0.0, dt, nt)
    w = ricker(f0, tgrid)
    wl = configs.Workload("homogeneous", "acoustic", [Grid(0.0, d, nz), Grid(0.0, d, nx)],
                          np.full((nz, nx), vp, np.float32), np.full((nz, nx), rho, np.float32),
                          shots=[(np.array([[sz, sx]]), np.array([[sz, sx + o] for o in offs]))],
                          tgrid=tgrid, wavelet=w, rfields=("p",), pml_faces=("zmin", "zmax", "xmin", "xmax"),
                          src_field="p")
    pa = wl.expt(order=order)
    update(pa)
    r = pa.data[0][0].d["p"].astype(np.float64)
    nf = 8 * nt
    om = 2 * np.pi * np.fft.rfftfreq(nf, dt)
    # the spray adds K dt w to one cell of area dA; the leapfrog places the
    # injected sample half a step late
    W = np.fft.rfft(np.asarray(w, np.float64), nf) * np.exp(-1j * om * 0.5 * dt)
    err = []
    for i, o in enumerate(offs):
        H = np.zeros_like(W)
        H[1:] = rho * d * d * om[1:] / 4.0 * hankel2(0, om[1:] * o / vp)
        p_an = np.fft.irfft(H * W, nf)[:nt]
        err.append(np.sum((r[:, i] - p_an) ** 2) / np.sum(p_an ** 2))
    assert max(err) < 1e-2, err  # the reference's bound
    assert max(err) < bound, err


@pytest.mark.gpu
@pytest.mark.parametrize("order,bound", [(4, 1e-4), (8, 1e-4)])
def test_green_function_3d_on_the_engine(engine, order, bound):
    n, d, nt, dt = 61, 10.0, 260, 0.001
    vp, rho, f0 = 2000.0, 2000.0, 12.0
    c0 = 0.5 * (n - 1) * d
    offs = np.array([100.0, 150.0, 200.0])
    tgrid = Grid(0.0, dt, nt)
    w = ricker(f0, tgrid)
    g = Grid(0.0, d, n)
    wl = configs.Workload("homogeneous3d", "acoustic", [g, g, g], np.full((n, n, n), vp, np.float32),
                          np.full((n, n, n), rho, np.float32),
                          shots=[(np.array([[c0, c0, c0]]), np.array([[c0, c0, c0 + o] for o in offs]))],
                          tgrid=tgrid, wavelet=w, rfields=("p",), src_field="p", npml=13 + order - 1)
    pa = wl.expt(order=order, ref_compat_proj=False)
    update(pa)
    r = pa.data[0][0].d["p"].astype(np.float64)
    nf = 8 * nt
    om = 2 * np.pi * np.fft.rfftfreq(nf, dt)
    W = np.fft.rfft(np.asarray(w, np.float64), nf) * np.exp(-1j * om * 0.5 * dt)
    err = []
    for i, o in enumerate(offs):
        P = rho * d ** 3 / (4 * np.pi * o) * (1j * om) * W * np.exp(-1j * om * o / vp)
        p_an = np.fft.irfft(P, nf)[:nt]
        err.append(np.sum((r[:, i] - p_an) ** 2) / np.sum(p_an ** 2))
    assert max(err) < 1e-2, err  # the reference's bound
    assert max(err) < bound, err


@pytest.mark.gpu
@pytest.mark.parametrize("order", [4, 2])
def test_engine_elastic_explosion_equals_the_acoustic_pressure_source(engine, order):
    """P waves only: the engine's elastic steps with an explosive source give
    the velocity records of its acoustic steps with a pressure source and
    K = lambda + 2 mu, with the opposite sign (FP32)."""
    nz = nx = 121
    d, nt, dt = 5.0, 500, 0.0004
    vp, vs, rho = 2500.0, 1400.0, 2000.0
    tgrid = Grid(0.0, dt, nt)
    w = ricker(15.0, tgrid)
    c = 0.5 * (nz - 1) * d
    rec = np.array([[c + 40.0, c + 60.0], [c - 80.0, c + 30.0], [c, c + 120.0], [c + 100.0, c - 100.0]])
    grid = [Grid(0.0, d, nz), Grid(0.0, d, nx)]
    faces = ("zmin", "zmax", "xmin", "xmax")
    full = lambda v: np.full((nz, nx), v, np.float32)  # noqa: E731
    el = configs.Workload("explosion", "elastic", grid, full(vp), full(rho), vs=full(vs),
                          shots=[(np.array([[c, c]]), rec)], tgrid=tgrid, wavelet=w, rfields=("vx", "vz"),
                          pml_faces=faces, src_field="tauxx")
    ac = configs.Workload("pressure", "acoustic", grid, full(vp), full(rho), shots=[(np.array([[c, c]]), rec)],
                          tgrid=tgrid, wavelet=w, rfields=("vx", "vz"), pml_faces=faces, src_field="p")
    pe, pa = el.expt(order=order), ac.expt(order=order)
    update(pe)
    update(pa)
    for f in ("vx", "vz"):
        a = pe.data[0][0].d[f].astype(np.float64)
        b = pa.data[0][0].d[f].astype(np.float64)
        assert np.abs(b).max() > 0.05
        assert np.linalg.norm(a + b) / np.linalg.norm(b) < 1e-5, f
