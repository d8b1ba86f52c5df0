"""Host-side setup of an FDTD experiment (the Julia host's job in the
reference): padding of the medium, derived parameters, CPML profiles,
sparse projection matrices, wavelets.  Vectorised numpy; the numbers follow
the reference's floating-point types (Float32 media and weights, Float64
PML profile from Float32 inputs).
"""
import math

import numpy as np

FACE_BITS = {"zmin": 1, "zmax": 2, "ymin": 4, "ymax": 8, "xmin": 16, "xmax": 32}
KF, KV, KH, KI = 0, 1, 2, 3
FIELD_KINDS = {
    "p": (KF, KF, KF), "vx": (KF, KF, KV), "vy": (KF, KV, KF), "vz": (KV, KF, KF),
    "tauxx": (KF, KF, KF), "tauyy": (KF, KF, KF), "tauzz": (KF, KF, KF),
    "tauxy": (KI, KH, KH), "tauxz": (KH, KI, KH), "tauyz": (KH, KH, KI),
}
# derivative fields in the engine's canonical order: (name, axis, kinds)
DERIV = {
    ("acoustic", 2): [("dpdx", 2, (KI, KF, KH)), ("dpdz", 0, (KH, KF, KI)),
                      ("dvxdx", 2, (KF, KF, KF)), ("dvzdz", 0, (KF, KF, KF))],
    ("elastic", 2): [("dtauxxdx", 2, (KI, KF, KH)), ("dtauxzdx", 2, (KH, KF, KI)),
                     ("dtauzzdz", 0, (KH, KF, KI)), ("dtauxzdz", 0, (KI, KF, KH)),
                     ("dvxdx", 2, (KF, KF, KF)), ("dvzdz", 0, (KF, KF, KF)),
                     ("dvxdz", 0, (KH, KF, KH)), ("dvzdx", 2, (KH, KF, KH))],
    ("acoustic", 3): [("dpdx", 2, (KI, KI, KH)), ("dpdy", 1, (KI, KH, KI)), ("dpdz", 0, (KH, KI, KI)),
                      ("dvxdx", 2, (KF, KF, KF)), ("dvydy", 1, (KF, KF, KF)), ("dvzdz", 0, (KF, KF, KF))],
    ("elastic", 3): [("dtauxxdx", 2, (KI, KI, KH)), ("dtauxydx", 2, (KI, KH, KI)),
                     ("dtauxzdx", 2, (KH, KI, KI)), ("dtauyydy", 1, (KI, KH, KI)),
                     ("dtauxydy", 1, (KI, KI, KH)), ("dtauyzdy", 1, (KH, KI, KI)),
                     ("dtauzzdz", 0, (KH, KI, KI)), ("dtauyzdz", 0, (KI, KH, KI)),
                     ("dtauxzdz", 0, (KI, KI, KH)), ("dvxdx", 2, (KF, KF, KF)),
                     ("dvydy", 1, (KF, KF, KF)), ("dvzdz", 0, (KF, KF, KF)),
                     ("dvxdy", 1, (KI, KH, KH)), ("dvxdz", 0, (KH, KI, KH)),
                     ("dvydx", 2, (KI, KH, KH)), ("dvydz", 0, (KH, KH, KI)),
                     ("dvzdx", 2, (KH, KI, KH)), ("dvzdy", 1, (KH, KH, KI))],
}


class Grid:
    """A uniform axis (Julia's StepRangeLen{Float64}): start, step, length."""

    def __init__(self, start, step, n):
        self.start, self.step, self.n = float(start), float(step), int(n)

    @classmethod
    def range(cls, start, stop, length):
        return cls(start, (stop - start) / (length - 1), length)

    def __len__(self):
        return self.n

    def values(self):
        return self.start + self.step * np.arange(self.n)

    @property
    def first(self):
        return self.start

    @property
    def last(self):
        return self.start + self.step * (self.n - 1)

    def __repr__(self):
        return "Grid(%g, step=%g, n=%d)" % (self.start, self.step, self.n)


def axis_names(ndim):
    return "zyx" if ndim == 3 else "zx"


def face_mask(faces):
    m = 0
    for f in faces:
        m |= FACE_BITS.get(str(f).lstrip(":"), 0)
    return m


def padgrid(grid, npml, mask):
    """padmgrid (src/media/media.jl:298-316)."""
    out = []
    for g, d in zip(grid, axis_names(len(grid))):
        lo = npml if mask & FACE_BITS[d + "min"] else 0
        hi = npml if mask & FACE_BITS[d + "max"] else 0
        out.append(Grid(g.start - lo * g.step, g.step, g.n + lo + hi))
    return out


def padarray(m, npml, mask):
    """Replicate-pad on PML faces only (padarray!, src/media/media.jl:280-296)."""
    pads = []
    for d in axis_names(m.ndim):
        pads.append((npml if mask & FACE_BITS[d + "min"] else 0, npml if mask & FACE_BITS[d + "max"] else 0))
    return np.pad(np.asarray(m, np.float32), pads, mode="edge")


def ref_bounds(m, frac=0.1):
    """Medium parameter reference value and bounds (src/media/media.jl:24-33)."""
    m = np.asarray(m, np.float32)
    ref = np.float32(m.mean(dtype=np.float32))
    f = np.float32(frac)
    lo = max(np.float32(0.0), np.float32(m.min() - f * ref))
    return ref, (np.float32(lo), np.float32(m.max() + f * ref))


def invK(vp, rho):
    vp = np.asarray(vp, np.float32)
    return (np.float32(1.0) / ((vp * vp) * np.asarray(rho, np.float32))).astype(np.float32)


def invlambda(vp, vs, rho):
    vp, vs = np.asarray(vp, np.float32), np.asarray(vs, np.float32)
    return (np.float32(1.0) / (((vp * vp) - np.float32(2.0) * (vs * vs)) * np.asarray(rho, np.float32))).astype(np.float32)


def invmu(vs, rho):
    vs = np.asarray(vs, np.float32)
    return (np.float32(1.0) / ((vs * vs) * np.asarray(rho, np.float32))).astype(np.float32)


def field_axis(g, kind, h):
    """Positions of a staggered field along one axis (get_mgrid)."""
    if kind == KV:
        return g.start - 0.5 * g.step * h + g.step * np.arange(g.n + h)
    if kind == KH:
        return g.start + 0.5 * g.step * h + g.step * np.arange(g.n - h)
    if kind == KI:
        return g.start + g.step * h + g.step * np.arange(g.n - 2 * h)
    return g.values()


def cpml_profile(x, g, flags, dt32, velavg32, fpeak32, npml):
    """a, b, kI on the first/last npml points of axis x (update_pml!,
    src/fdtd/cpml.jl:8-103); Float64 arithmetic, Float32 result."""
    xl = g.first - 2 * g.step
    xr = g.last + 2 * g.step
    thick = (npml - 1) * g.step
    amax = math.pi * float(fpeak32)
    d0 = -(2.0 + 1) * float(velavg32) * math.log(0.001) / (2.0 * thick)
    d = np.zeros(len(x))
    alpha = np.zeros(len(x))
    for on, ab in ((flags[0], xl - x), (flags[1], x - xr)):
        if not on:
            continue
        sel = ab >= 0.0
        an = ab[sel] / thick
        d[sel] = d0 * an ** 2.0
        alpha[sel] = amax * (1.0 - an) + 0.01 * amax
    alpha[alpha < 0.0] = 0.0
    k = np.ones(len(x))
    b = np.exp(-(d / k + alpha) * float(dt32))
    a = np.zeros(len(x))
    nzd = np.abs(d) > 1e-6
    a[nzd] = d[nzd] * (b[nzd] - 1.0) / (k[nzd] * (d[nzd] + k[nzd] * alpha[nzd]))
    sel = np.r_[0:npml, len(x) - npml:len(x)]
    return a[sel].astype(np.float32), b[sel].astype(np.float32), (1.0 / k[sel]).astype(np.float32)


def cpml_all(physics, ndim, order, grid, mask, dt32, velavg32, fpeak32, npml):
    """update_pml! for every derivative field (src/fdtd/cpml.jl:125-155).
    `npml` is the plan's PML width: it sets the padding of the extended
    grid, the damping thickness (npml - 1) * step and the strips kept (the
    reference uses its constant _fd_npml = 40 + order - 1 for all three,
    src/fdtd/cpml.jl:29,88-99)."""
    h = order - 1
    npml = int(npml)
    if npml < 1:
        raise ValueError("npml must be positive")
    ex = padgrid(grid, npml, mask)
    names = axis_names(ndim)
    out = []
    for _, axis, kinds in DERIV[(physics, ndim)]:
        ia = axis if ndim == 3 else (0 if axis == 0 else 1)
        x = field_axis(ex[ia], kinds[axis], h)
        d = names[ia]
        flags = (bool(mask & FACE_BITS[d + "min"]), bool(mask & FACE_BITS[d + "max"]))
        out.append(cpml_profile(x, grid[ia], flags, dt32, velavg32, fpeak32, npml))
    return out


def _bracket(x, v):
    """get_neighbour_indices (src/proj_mat.jl:69-79), vectorised, 0-based."""
    n = len(x)
    idx = np.searchsorted(x, v, side="left") + 1
    i1 = np.where(idx == 1, 0, np.where(idx >= n, n - 2, idx - 2))
    f = np.where(v < x.min(), 0.0, np.where(v > x.max(), 1.0, (v - x[i1]) / (x[i1 + 1] - x[i1])))
    return i1, f


def projection(field, exgrid, points, order, ref_compat=True):
    """Sparse CSC (colptr, rowval, nzval) from the field grid to `points`
    (get_proj_matrix + bilinear_interp, src/proj_mat.jl:85-247).  points:
    array (npts, ndim) of (z, [y,] x).  In 3-D the reference pairs the z grid
    with the x coordinate and vice versa (bilinear_interp(x, y, z, zi, yi,
    xi) called with (mz, my, mx, pz, py, px)); ref_compat keeps that."""
    ndim = len(exgrid)
    h = order - 1
    kinds = FIELD_KINDS[field]
    kinds = (kinds[0], kinds[2]) if ndim == 2 else kinds
    axes = [field_axis(g, k, h) for g, k in zip(exgrid, kinds)]
    P = np.asarray(points, dtype=np.float64).reshape(-1, ndim)
    npts = len(P)
    if ndim == 3 and ref_compat:
        P = P[:, [2, 1, 0]]
    idx, fr = zip(*[_bracket(ax, P[:, i]) for i, ax in enumerate(axes)])
    dims = [len(ax) for ax in axes]
    rows, vals = [], []
    corners = [(0, 0), (0, 1), (1, 0), (1, 1)] if ndim == 2 else \
        [(a, b, c) for a in (0, 1) for b in (0, 1) for c in (0, 1)]
    for cor in corners:
        lin = np.zeros(npts, np.int64)
        w = np.ones(npts)
        stride = 1
        for ax in range(ndim):
            lin += (idx[ax] + cor[ax]) * stride
            stride *= dims[ax]
        # weight product in the reference's order ((1-dz)(1-dy))(1-dx)
        for ax in range(ndim):
            w = w * (fr[ax] if cor[ax] else (1.0 - fr[ax]))
        rows.append(lin)
        vals.append(w.astype(np.float32))
    rows = np.stack(rows, 1)
    vals = np.stack(vals, 1)
    order_ = np.argsort(rows, axis=1, kind="stable")
    rows = np.take_along_axis(rows, order_, 1)
    vals = np.take_along_axis(vals, order_, 1)
    colptr = np.arange(npts + 1, dtype=np.int64) * rows.shape[1]
    return colptr, rows.reshape(-1).astype(np.int64), vals.reshape(-1).astype(np.float32)


def ricker(fqdom, tgrid, tpeak=None, maxamp=1.0):
    """Ricker wavelet (src/srcwav/wavelets.jl:14-72)."""
    if tpeak is None:
        tpeak = tgrid.first + 1.5 / fqdom
    pf = (math.pi * math.pi) * fqdom ** 2.0
    t = tgrid.values()
    ts = (t - tpeak) * (t - tpeak)
    return (1.0 - 2.0 * pf * ts) * np.exp(-1.0 * pf * ts) * maxamp


def taper(x, perc=0.0, bperc=None, eperc=None):
    """taper! along the first axis (src/Utils/taper.jl:20-36): the first
    round(nt perc / 100) samples times sin((i - 1) pi / (2 n - 1)), the last
    ones times sin((nt - i) pi / (2 n - 1)) (1-based i; ties of the rounding
    to even, as Julia's round)."""
    x = np.array(x, np.float64, copy=True)
    nt = x.shape[0]
    bperc = perc if bperc is None else bperc
    eperc = perc if eperc is None else eperc
    nb, ne = int(round(nt * bperc * 0.01)), int(round(nt * eperc * 0.01))
    ntb, nte = min(nb, nt), min(ne, nt)
    kb, ke = math.pi / (2.0 * nb - 1), math.pi / (2.0 * ne - 1)
    i = np.arange(1, nt + 1, dtype=np.float64)
    shape = (nt,) + (1,) * (x.ndim - 1)
    if ntb > 0:
        w = np.where(i <= ntb, np.sin((i - 1) * kb), 1.0)
        x *= w.reshape(shape)
    if nte > 0:
        w = np.where(i >= nt - nte + 1, np.sin((-i + nt) * ke), 1.0)
        x *= w.reshape(shape)
    return x


def ormsby(fqdom, tgrid, fracbandwidth=1.2, f1=None, f4=None, f2=None, f3=None, tpeak=None, trim_tol=0.0,
           tperc=0.0, maxamp_rand_flag=False, rng=None):
    """Ormsby wavelet (src/srcwav/wavelets.jl:75-142): corner frequencies
    f1 < f2 < f3 < f4 around fqdom (fracbandwidth 1.2 as for the Ricker),
    w(t) = (A43 S4 - A34 S3) - (A21 S2 - A12 S1) with Sk = sinc(pi fk t)^2,
    t = tgrid - tpeak, normalised to a maximum |w| of 1, then tapered by
    tperc percent at both ends.  sinc is the normalised sinc (Julia's and
    numpy's: sin(pi x) / (pi x)), so the reference's argument pi fk t puts
    the pass band at pi [f1, f4]; kept as the reference computes it."""
    f1 = fqdom - fracbandwidth * 0.5 * fqdom if f1 is None else f1
    f4 = fqdom + fracbandwidth * 0.5 * fqdom if f4 is None else f4
    f2 = 0.25 * f4 + 0.75 * f1 if f2 is None else f2
    f3 = 0.25 * f1 + 0.75 * f4 if f3 is None else f3
    if tpeak is None:
        tpeak = tgrid.first + 1.5 / (0.25 * (f1 + f4))
    pi = math.pi
    A43 = (pi * f4) ** 2 / (pi * f4 - pi * f3)
    A34 = (pi * f3) ** 2 / (pi * f4 - pi * f3)
    A21 = (pi * f2) ** 2 / (pi * f2 - pi * f1)
    A12 = (pi * f1) ** 2 / (pi * f2 - pi * f1)
    t = tgrid.values() - tpeak
    S4 = np.sinc(pi * f4 * t) ** 2
    S3 = np.sinc(pi * f3 * t) ** 2
    S2 = np.sinc(pi * f2 * t) ** 2
    S1 = np.sinc(pi * f1 * t) ** 2
    wav = (A43 * S4 - A34 * S3) - (A21 * S2 - A12 * S1)
    wav = wav / np.max(np.abs(wav))
    if maxamp_rand_flag:
        wav = wav * (rng or np.random.default_rng()).uniform(-1.0, 1.0)
    if trim_tol != 0.0:
        wav = wav[np.abs(wav) >= trim_tol]
    return taper(wav, tperc)


def findfreq_peak(w, dt):
    """Peak frequency of |rfft|^2 over all columns (findfreq, src/Utils/freq.jl:28-57)."""
    w = np.asarray(w, np.float32)
    w = w[:, None] if w.ndim == 1 else w
    ax = np.abs(np.fft.rfft(w, axis=0)) ** 2
    i = int(np.argmax(ax.T.reshape(-1)))
    return np.fft.rfftfreq(w.shape[0], dt)[i % ax.shape[0]]


def findfreq(w, dt, attrib="peak", threshold=-50.0):
    """findfreq (src/Utils/freq.jl:28-57): on the power spectrum of all
    columns, normalised to its maximum in dB, the frequency of the maximum
    ("peak"), of the last ("max") or first ("min") sample at or above
    `threshold`, in the column-major order of the spectra."""
    w = np.asarray(w, np.float64)
    w = w[:, None] if w.ndim == 1 else w
    ax = np.abs(np.fft.rfft(w, axis=0)) ** 2
    f = np.fft.rfftfreq(w.shape[0], dt)
    if ax.max() == 0.0:
        return 0.0
    db = 10.0 * np.log10(np.maximum(ax / ax.max(), 1e-300))
    flat = db.T.reshape(-1)  # column-major order of (frequency, column)
    if attrib == "peak":
        i = int(np.argmax(flat))
    elif attrib == "max":
        i = int(np.nonzero(flat >= threshold)[0][-1])
    else:
        i = int(np.nonzero(flat >= threshold)[0][0])
    return float(f[i % ax.shape[0]])


def reverse_source(w):
    """Source of the time-reversed wavefield (get_source(..., Val{-1}),
    src/fdtd/source.jl:8-19): -w shifted by one sample, reversed, row 1 zero."""
    ww = np.roll(-np.asarray(w, np.float32), -1, axis=0)[::-1].copy()
    ww[0] = 0
    return ww
