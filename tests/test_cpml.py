"""CPML profiles at any PML width, checked independently of both
restatements (the product's setup.cpml_all and the oracle's pml_all).

The reference computes the profiles with its constant _fd_npml = 40 + h
(src/fdtd/cpml.jl:29,88-99); a plan with npml = n + h must use npml for the
padding, the damping thickness (npml - 1) * step and the kept strips alike.
These tests derive the expected values from the Komatitsch-Martin formulas
in closed form (cell index -> distance into the PML), so an error shared by
the two restatements cannot hide here."""
import math

import numpy as np
import pytest

from geophyinv_gb300 import setup as P
from oracle import setup_ref as S

DT, VAVG, FPEAK = np.float32(0.0005), np.float32(2500.0), np.float32(15.0)

# staggering offset (in cells, relative to the extended grid's first point)
# and length change of each field kind along its axis at order 4 (h = 3)
OFFSET = {P.KF: (0.0, 0), P.KV: (-1.5, 3), P.KH: (1.5, -3), P.KI: (3.0, -6)}


def _closed_form(kind, n_phys, npml, step):
    """Expected (a, b) on the 2*npml kept points of a field of `kind` along
    an axis of n_phys physical cells with a PML of npml cells on both faces.
    Position of point i (0-based) relative to the first physical cell:
    (i - npml + off) * step; the PML starts 2 cells outside the physical
    grid on either side; s = distance into the PML (>= 0 inside)."""
    off, dn = OFFSET[kind]
    n = n_phys + 2 * npml + dn
    L = (npml - 1) * step
    d0 = -3.0 * float(VAVG) * math.log(1e-3) / (2.0 * L)
    amax = math.pi * float(FPEAK)
    a = np.zeros(n)
    b = np.zeros(n)
    for i in range(n):
        x = (i - npml + off) * step
        s = max(-2.0 * step - x, x - ((n_phys - 1) * step + 2.0 * step))
        if s >= 0.0:
            d = d0 * (s / L) ** 2
            al = max(amax * (1.0 - s / L) + 0.01 * amax, 0.0)
        else:
            d, al = 0.0, 0.0
        b[i] = math.exp(-(d + al) * float(DT))
        a[i] = d * (b[i] - 1.0) / (d + al) if abs(d) > 1e-6 else 0.0
    sel = np.r_[0:npml, n - npml:n]
    return a[sel], b[sel]


@pytest.mark.parametrize("npml", [10, 23, 43])
@pytest.mark.parametrize("physics,ndim", [("acoustic", 2), ("elastic", 2), ("elastic", 3)])
def test_profiles_follow_the_formulas_at_any_width(npml, physics, ndim):
    steps = [5.0, 10.0, 7.5][:ndim] if ndim == 3 else [5.0, 7.5]
    nphys = [37, 29, 41][:ndim] if ndim == 3 else [37, 41]
    grid = [P.Grid(0.0, s, n) for s, n in zip(steps, nphys)]
    prof = P.cpml_all(physics, ndim, 4, grid, 63, DT, VAVG, FPEAK, npml)
    oprof = S.pml_all(physics, ndim, 4, [(g.start, g.step, g.n) for g in grid], 63, DT, VAVG, FPEAK, npml)
    for q, (name, axis, kinds) in enumerate(P.DERIV[(physics, ndim)]):
        ia = axis if ndim == 3 else (0 if axis == 0 else 1)
        ea, eb = _closed_form(kinds[axis], nphys[ia], npml, steps[ia])
        for got in (prof[q], oprof[q]):
            a, b, kI = got
            assert len(a) == len(b) == len(kI) == 2 * npml, name
            np.testing.assert_allclose(a, ea, rtol=2e-6, atol=1e-9, err_msg=name)
            np.testing.assert_allclose(b, eb, rtol=2e-6, atol=1e-9, err_msg=name)
            assert np.all(kI == 1.0)


@pytest.mark.parametrize("npml", [10, 23])
def test_profiles_taper_to_the_interface_and_mirror(npml):
    """On a grid with both faces in the PML the max-face slots are the
    min-face slots reversed, and the damping falls to zero at the interface
    (the last min-face slots and the first max-face slots carry no d)."""
    grid = [P.Grid(0.0, 5.0, 51), P.Grid(0.0, 5.0, 63)]
    prof = P.cpml_all("elastic", 2, 4, grid, 63, DT, VAVG, FPEAK, npml)
    for q, (name, axis, kinds) in enumerate(P.DERIV[("elastic", 2)]):
        a, b, _ = prof[q]
        np.testing.assert_allclose(a[npml:][::-1], a[:npml], rtol=1e-5, atol=1e-9, err_msg=name)
        np.testing.assert_allclose(b[npml:][::-1], b[:npml], rtol=1e-6, atol=1e-9, err_msg=name)
        # outermost point: the strongest damping; the inner end: none
        assert a[0] < a[npml - 1] <= 0.0
        assert abs(a[npml - 1]) < 0.02 * abs(a[0]) and abs(a[npml]) < 0.02 * abs(a[0])
        assert np.all(np.diff(a[:npml]) >= 0.0)


def _homogeneous(npml, nt=700):
    """Homogeneous 2-D acoustic model, source mid-grid, a ring of receivers
    between the source and the PML: the records after the direct wave are
    reflections from the PML."""
    from geophyinv_gb300.setup import Grid, ricker

    nz, nx, d = 81, 81, 5.0
    tg = Grid(0.0, 0.0005, nt)
    w = ricker(25.0, tg).astype(np.float32)
    zc, xc = 200.0, 200.0
    ang = np.linspace(0, 2 * np.pi, 24, endpoint=False)
    rec = [(zc + 120 * math.sin(t), xc + 120 * math.cos(t)) for t in ang]
    return {"physics": "acoustic", "ndim": 2, "order": 4, "grid": [(0.0, d, nz), (0.0, d, nx)],
            "vp": np.full((nz, nx), 2000.0, np.float32), "rho": np.full((nz, nx), 2000.0, np.float32),
            "pml_faces": 63, "free_faces": 0, "dt": 0.0005, "nt": nt, "npml": npml,
            "shots": [{"src": {"p": ([(zc, xc)], w[:, None])}, "rec": rec}], "rfields": ["p"]}


def _run(ex, pml=None):
    from oracle import oracle as O

    prep = O.Prepared(ex)
    if pml is not None:
        prep.pml = pml
    orc = O.Oracle(prep)
    src, rec = O._shot_inputs(prep, ex["shots"][0])
    out = orc.shot(0, 0, src, rec)["p"]
    orc.close()
    return out.astype(np.float64)


def _reflected(thin, thick):
    """Energy of the thin-PML records relative to the thick-PML ones, over
    the window after the direct wave has passed the receivers."""
    late = slice(420, None)  # 0.21 s: direct wave gone, PML echoes arriving
    return np.linalg.norm(thin[late] - thick[late]) / np.linalg.norm(thick)


def test_thin_pml_absorbs_like_the_thick_one():
    """Reflection test: a 23-cell PML leaves echoes far below the direct
    wave, measured against a 43-cell PML on the same model.  The same
    comparison with the thin PML given the strips of a 43-cell profile
    (the failure mode of a profile computed for the wrong width) is two
    orders of magnitude worse, so the check can see that error."""
    thick = _run(_homogeneous(43))
    ex = _homogeneous(23)
    thin = _run(ex)
    e_ok = _reflected(thin, thick)
    assert e_ok < 5e-3, e_ok  # measured 2.9e-3
    # planted error, on the CPU oracle only: the 43-cell profile's first
    # 2*23 points as if they were the 23-cell strips
    wrong = []
    full = S.pml_all("acoustic", 2, 4, ex["grid"], 63, np.float32(ex["dt"]), np.float32(2000.0 * 1.0),
                     np.float32(25.0), 43)
    for a, b, k in full:
        wrong.append((a[:46].copy(), b[:46].copy(), k[:46].copy()))
    e_bad = _reflected(_run(ex, wrong), thick)
    assert e_bad > 30 * e_ok, (e_bad, e_ok)  # measured 0.28
