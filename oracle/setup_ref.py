"""Setup half of the CPU ORACLE (test infrastructure only).

numpy restatements of the host-side functions that prepare the inputs of the
GeoPhyInv FDTD time loop.  Each function cites the reference it follows.  The
product computes the same quantities in its own C++ code; tests compare the
two.  Nothing in the product imports this module.

Floating-point types follow the reference: media and derived parameters are
Float32 (`Data.Number`), the PML profile is computed in Float64 from Float32
inputs (`pac.fc` is Float32) and stored as Float32, projection weights are
computed in Float64 and stored as Float32.
"""
import math

import numpy as np

ZMIN, ZMAX, YMIN, YMAX, XMIN, XMAX = 1, 2, 4, 8, 16, 32
FACE_BITS = {"zmin": ZMIN, "zmax": ZMAX, "ymin": YMIN, "ymax": YMAX, "xmin": XMIN, "xmax": XMAX}

# field shape kinds per axis (z, y, x): 0 n, 1 n+h, 2 n-h, 3 n-2h
# (get_mgrid, src/fields.jl:92-671)
KF, KV, KH, KI = 0, 1, 2, 3
FIELD_KINDS = {
    "p": (KF, KF, KF), "vx": (KF, KF, KV), "vy": (KF, KV, KF), "vz": (KV, KF, KF),
    "tauxx": (KF, KF, KF), "tauyy": (KF, KF, KF), "tauzz": (KF, KF, KF),
    "tauxy": (KI, KH, KH), "tauxz": (KH, KI, KH), "tauyz": (KH, KH, KI),
}
FIELD_ID = {"p": 0, "vx": 1, "vy": 2, "vz": 3, "tauxx": 4, "tauyy": 5, "tauzz": 6,
            "tauxy": 7, "tauxz": 8, "tauyz": 9}

# canonical derivative-field order (oracle/gpo.h) with (axis, kinds)
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


def npml_of(order):
    """_fd_npml = 40 + (order - 1) (src/GeoPhyInv.jl:90-91)."""
    return 40 + order - 1


def axis_grid(start, step, n, kind, h):
    """Positions of a field grid along one axis (get_mgrid, src/fields.jl:92-671)."""
    if kind == KV:
        return start - 0.5 * step * h + step * np.arange(n + h)
    if kind == KH:
        return start + 0.5 * step * h + step * np.arange(n - h)
    if kind == KI:
        return start + step * h + step * np.arange(n - 2 * h)
    return start + step * np.arange(n)


def padmgrid(grid, npml, faces):
    """padmgrid (src/media/media.jl:298-316): list of (start, step, n)."""
    names = "zyx" if len(grid) == 3 else "zx"
    out = []
    for (start, step, n), d in zip(grid, names):
        lo = npml if (faces & FACE_BITS[d + "min"]) else 0
        hi = npml if (faces & FACE_BITS[d + "max"]) else 0
        out.append((start - lo * step, step, n + lo + hi))
    return out


def padarray(m, npml, faces):
    """Replicate padding on PML faces only (padarray!, src/media/media.jl:280-296)."""
    names = "zyx" if m.ndim == 3 else "zx"
    pads = []
    for d in names:
        pads.append((npml if faces & FACE_BITS[d + "min"] else 0, npml if faces & FACE_BITS[d + "max"] else 0))
    return np.pad(m, pads, mode="edge")


def bounds(m, frac=0.1):
    """ref = mean(m); bounds = [max(0, min - frac ref), max + frac ref] in eltype
    (src/media/media.jl:24-33)."""
    m = np.asarray(m, dtype=np.float32)
    ref = np.float32(np.mean(m, dtype=np.float32))
    f = np.float32(frac)
    return ref, np.array([max(np.float32(0), m.min() - f * ref), m.max() + f * ref], dtype=np.float32)


def derived_acoustic(vp, rho):
    """mod = [invK, rho] (src/media/media.jl:111-130, src/fdtd/medium.jl:81-95)."""
    vp = np.asarray(vp, np.float32)
    rho = np.asarray(rho, np.float32)
    invK = np.float32(1) / ((vp * vp) * rho)
    return [invK.astype(np.float32), rho.copy()]


def derived_elastic(vp, vs, rho):
    """mod = [invlambda, invmu, rho] (src/media/media.jl:119-126)."""
    vp = np.asarray(vp, np.float32)
    vs = np.asarray(vs, np.float32)
    rho = np.asarray(rho, np.float32)
    invl = np.float32(1) / (((vp * vp) - np.float32(2) * (vs * vs)) * rho)
    invm = np.float32(1) / ((vs * vs) * rho)
    return [invl.astype(np.float32), invm.astype(np.float32), rho.copy()]


def pml_profile(exgrid_f, mgrid_start, mgrid_step, mgrid_n, flags, dt32, velavg32, fpeak32, npml):
    """update_pml! (src/fdtd/cpml.jl:8-103): a, b, kI of length 2*npml (Float32)."""
    nx = len(exgrid_f)
    xl = mgrid_start - 2 * mgrid_step
    xr = (mgrid_start + (mgrid_n - 1) * mgrid_step) + 2 * mgrid_step
    NPOWER = 2.0
    alpha_max = math.pi * float(fpeak32)
    thick = (npml - 1) * mgrid_step
    d0 = -(NPOWER + 1) * float(velavg32) * math.log(0.001) / (2.0 * thick)
    dt = float(dt32)
    k = np.ones(nx)
    d = np.zeros(nx)
    alpha = np.zeros(nx)
    a = np.zeros(nx)
    b = np.zeros(nx)
    for ix in range(nx):
        if flags[0]:
            ab = xl - exgrid_f[ix]
            if ab >= 0.0:
                an = ab / thick
                d[ix] = d0 * an ** NPOWER
                k[ix] = 1.0
                alpha[ix] = alpha_max * (1.0 - an) + 0.01 * alpha_max
        if flags[1]:
            ab = exgrid_f[ix] - xr
            if ab >= 0.0:
                an = ab / thick
                d[ix] = d0 * an ** NPOWER
                k[ix] = 1.0
                alpha[ix] = alpha_max * (1.0 - an) + 0.01 * alpha_max
        if alpha[ix] < 0.0:
            alpha[ix] = 0.0
        b[ix] = math.exp(-(d[ix] / k[ix] + alpha[ix]) * dt)
        if abs(d[ix]) > 1e-6:
            a[ix] = d[ix] * (b[ix] - 1.0) / (k[ix] * (d[ix] + k[ix] * alpha[ix]))
    sel = np.r_[0:npml, nx - npml:nx]
    return (a[sel].astype(np.float32), b[sel].astype(np.float32), (1.0 / k[sel]).astype(np.float32))


def pml_all(physics, ndim, order, mgrid, faces, dt32, velavg32, fpeak32, npml=None):
    """update_pml! over all derivative fields (src/fdtd/cpml.jl:125-155).
    mgrid: physical (start, step, n) per axis (z, [y,] x).  npml: the PML
    width that replaces the reference's constant _fd_npml in the padding,
    the thickness (npml - 1) * step and the kept strips (cpml.jl:29,88-99);
    default _fd_npml."""
    h = order - 1
    npml = npml_of(order) if npml is None else int(npml)
    ex = padmgrid(mgrid, npml, faces)
    out = []
    names = "zyx" if ndim == 3 else "zx"
    for name, axis, kinds in DERIV[(physics, ndim)]:
        ia = axis if ndim == 3 else (0 if axis == 0 else 1)
        s, st, n = ex[ia]
        g = axis_grid(s, st, n, kinds[axis], h)
        d = names[ia]
        flags = (bool(faces & FACE_BITS[d + "min"]), bool(faces & FACE_BITS[d + "max"]))
        ms, mst, mn = mgrid[ia]
        out.append(pml_profile(g, ms, mst, mn, flags, dt32, velavg32, fpeak32, npml))
    return out


def _neighbours(arr, val):
    """get_neighbour_indices (src/proj_mat.jl:69-79), returned 0-based."""
    n = len(arr)
    idx = int(np.searchsorted(arr, val, side="left")) + 1
    if idx == 1:
        return 0, 1
    if idx >= n:
        return n - 2, n - 1
    return idx - 2, idx - 1


def _frac(arr, val, i1, i2):
    if val < arr.min():
        return 0.0
    if val > arr.max():
        return 1.0
    return (val - arr[i1]) / (arr[i2] - arr[i1])


def proj_matrix(field, grids, points, ndim, order, ref_compat=True):
    """get_proj_matrix / bilinear_interp (src/proj_mat.jl:85-247): CSC arrays
    (colptr, rowval, nzval) mapping the field's grid to the points.

    grids: extended (start, step, n) per axis; points: list of coordinate
    tuples (z, x) or (z, y, x).  In 3-D the reference passes (z, y, x)
    coordinates into bilinear_interp(x, y, z, zi, yi, xi), which pairs the z
    grid with the x coordinate and the x grid with the z coordinate
    (src/proj_mat.jl:85-90, :240); ref_compat=True keeps that pairing."""
    h = order - 1
    kinds = FIELD_KINDS[field]
    if ndim == 2:
        kinds = (kinds[0], kinds[2])
    ax = [axis_grid(s, st, n, k, h) for (s, st, n), k in zip(grids, kinds)]
    colptr = [0]
    rows = []
    vals = []
    for P in points:
        if ndim == 2:
            gz, gx = ax
            z1, z2 = _neighbours(gz, P[0])
            x1, x2 = _neighbours(gx, P[1])
            fz = _frac(gz, P[0], z1, z2)
            fx = _frac(gx, P[1], x1, x2)
            n1 = len(gz)
            ent = {
                z1 + n1 * x1: (1 - fz) * (1 - fx),
                z1 + n1 * x2: (1 - fz) * fx,
                z2 + n1 * x1: fz * (1 - fx),
                z2 + n1 * x2: fz * fx,
            }
        else:
            gz, gy, gx = ax
            pz, py, px = P
            if ref_compat:
                pz, px = px, pz
            z1, z2 = _neighbours(gz, pz)
            y1, y2 = _neighbours(gy, py)
            x1, x2 = _neighbours(gx, px)
            fz = _frac(gz, pz, z1, z2)
            fy = _frac(gy, py, y1, y2)
            fx = _frac(gx, px, x1, x2)
            n1, n2 = len(gz), len(gy)
            ent = {}
            for zi, wz in ((z1, 1 - fz), (z2, fz)):
                for yi, wy in ((y1, 1 - fy), (y2, fy)):
                    for xi, wx in ((x1, 1 - fx), (x2, fx)):
                        ent[zi + n1 * (yi + n2 * xi)] = wz * wy * wx
        for r in sorted(ent):
            rows.append(r)
            vals.append(np.float32(ent[r]))
        colptr.append(len(rows))
    return (np.array(colptr, np.int64), np.array(rows, np.int64), np.array(vals, np.float32))


def ricker(fqdom, nt, dt, t0=0.0, tpeak=None, maxamp=1.0):
    """ricker (src/srcwav/wavelets.jl:14-72), Float64."""
    if tpeak is None:
        tpeak = t0 + 1.5 / fqdom
    pf = (math.pi * math.pi) * fqdom ** 2.0
    t = t0 + dt * np.arange(nt)
    ts = (t - tpeak) * (t - tpeak)
    return (1.0 - 2.0 * pf * ts) * np.exp(-1.0 * pf * ts) * maxamp


def findfreq_peak(w, dt):
    """findfreq(..., attrib=:peak) (src/Utils/freq.jl:28-57): w is nt x ns."""
    w = np.asarray(w, dtype=np.float32)
    if w.ndim == 1:
        w = w[:, None]
    nt = w.shape[0]
    cx = np.fft.rfft(w, axis=0)
    ax = np.abs(cx) ** 2
    i = int(np.argmax(ax.T.reshape(-1)))  # column-major first maximum
    fi = i % ax.shape[0]
    return np.fft.rfftfreq(nt, dt)[fi]


def source_reverse(w):
    """get_source(w, ::Union{vz,vx,vy}, ::Val{-1}) (src/fdtd/source.jl:8-19)."""
    ww = -np.asarray(w, np.float32)
    ww = np.roll(ww, -1, axis=0)
    ww = ww[::-1].copy()
    ww[0] = 0
    return ww


def l2_value(dobs, dcal):
    """L2DistLoss value (LossFunctions 0.11.2): (output - target)^2 summed,
    called as loss(dobs, dcal) (src/database/database.jl:355-366)."""
    return float(np.sum((np.asarray(dobs, np.float64) - np.asarray(dcal, np.float64)) ** 2))


def l2_deriv(dobs, dcal):
    """deriv(L2DistLoss(), dobs, dcal) = 2 (dobs - dcal) (LossFunctions 0.11.2,
    called at src/database/database.jl:369-373)."""
    return (np.float32(2) * (np.asarray(dobs, np.float32) - np.asarray(dcal, np.float32))).astype(np.float32)
